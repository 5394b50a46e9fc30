"""Pin the CPU oracle against fixtures produced by the reference's own code.

The fixtures come from ``tests/golden/make_golden.py`` (reference Python run
in the build container); these tests need neither the reference nor a GPU.
"""
import os

import numpy as np
import pytest

from oracle import sdbe_oracle as O


def _load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def test_dbe_frame_header_fields(golden_dir):
    g = _load(golden_dir, "dbe_frame_decode.npz")
    invalid, c, f, b = O.decode_beng_headers(g["packets"])
    assert (invalid == 0).all()
    np.testing.assert_array_equal(c, g["c"])
    np.testing.assert_array_equal(f, g["f"])
    np.testing.assert_array_equal(b, g["b"])


def test_dbe_frame_unpack_bit_layout(golden_dir):
    """vdif_to_beng places every 2-bit sample where DBEFrame.from_bin says."""
    g = _load(golden_dir, "dbe_frame_decode.npz")
    for i, pkt in enumerate(g["packets"]):
        beng0, beng1 = O.vdif_to_beng(pkt[None], b_zero=int(g["b"][i]), n_frames=1)
        base = int(O.channel_base_aphids(int(g["c"][i]), int(g["f"][i])))
        for k in range(8):
            got0 = beng0[0, :, base + k, 1] + 1j * beng0[0, :, base + k, 0]
            got1 = beng1[0, :, base + k, 1] + 1j * beng1[0, :, base + k, 0]
            np.testing.assert_array_equal(got0, g["p0"][i, k])
            np.testing.assert_array_equal(got1, g["p1"][i, k])
        # nothing else written: 8 channels x 128 snapshots per pol
        assert np.count_nonzero(np.abs(beng0[0]).sum(-1).sum(0)) <= 8


def test_mar2015_channel_map_matches_reader(golden_dir):
    """read_sdbe_vdif.py:193 map covers all 16384 channels exactly once."""
    c, f = np.meshgrid(np.arange(256), np.arange(8), indexing="ij")
    ch = (O.channel_base_mar2015(c, f)[..., None] + np.arange(8)).ravel()
    assert np.array_equal(np.sort(ch), np.arange(16384))
    ch = (O.channel_base_aphids(c, f)[..., None] + np.arange(8)).ravel()
    assert np.array_equal(np.sort(ch), np.arange(16384))


def test_quantize_rule_matches_reference(golden_dir):
    g = _load(golden_dir, "quantize_pack.npz")
    xs, th = g["xs"], float(g["th"])
    ref_codes = g["codes"].astype(np.int16) + 2
    ours = O.quantize2bit_codes(xs, th, 0.0).astype(np.int16)
    exact_neg_th = xs == -th
    # the GPU kernel (.cu:577) puts v == -th in code 0, the numpy path in code 1
    np.testing.assert_array_equal(ours[~exact_neg_th], ref_codes[~exact_neg_th])
    assert (ours[exact_neg_th] == 0).all() and (ref_codes[exact_neg_th] == 1).all()


def test_pack_and_header_match_vdif_to_bin(golden_dir):
    g = _load(golden_dir, "quantize_pack.npz")
    codes = (g["codes"].astype(np.int16) + 2).astype(np.uint8)
    payload = O.pack2bit(codes).view(np.uint8)
    for k in range(len(g["frames"])):
        frame = g["frames"][k]
        assert frame.size == O.OUT_PKT_BYTES
        np.testing.assert_array_equal(payload, frame[32:])
        words = O.vdif_out_header_words(
            1, pol=int(g["hdr_pol"][k]), secs=int(g["hdr_secs"][k]), df=int(g["hdr_df"][k]),
            psn=int(g["hdr_psn"][k]), ref_epoch=int(g["ref_epoch"]),
            bdc_sideband=int(g["bdc_sideband"]), rx_sideband=int(g["rx_sideband"]))
        np.testing.assert_array_equal(words[0].view(np.uint8), frame[:32])
    np.testing.assert_array_equal(O.unpack2bit(payload.view("<u4")), codes)


def test_header_df_wrap_and_psn():
    w = O.vdif_out_header_words(4, pol=1, secs=10, df=124998, psn=2**32 - 2)
    assert list(w[:, 1] & 0xFFFFFF) == [124998, 124999, 0, 1]
    assert list(w[:, 0]) == [10, 10, 11, 11]
    psn = w[:, 6].astype(np.uint64) | (w[:, 7].astype(np.uint64) << np.uint64(32))
    assert list(psn) == [2**32 - 2, 2**32 - 1, 2**32, 2**32 + 1]


def test_mar2015_reorder_matches_reference(golden_dir):
    g = _load(golden_dir, "reorder_mar2015.npz")
    data = g["data"]                        # [channel][frame][snapshot]
    ours = O.reorder_mar2015(np.transpose(data, (1, 2, 0)))
    np.testing.assert_array_equal(np.transpose(ours, (2, 0, 1)), g["result"])


def test_fft_chain_scale_matches_reference_check(golden_dir):
    """Oracle FFT A/B/C with cuFFT scaling == the reference's numpy check x scale."""
    g = _load(golden_dir, "fft_resample_2496.npz")
    rng = np.random.default_rng(int(g["seed"]))
    cpu_in = (rng.integers(-2, 2, (39, O.BENG_CHANNELS))
              + 1j * rng.integers(-2, 2, (39, O.BENG_CHANNELS))).astype(np.complex64)
    cpu_in[:, -1] = 0
    n_out = int(g["n_out"])
    a = O.swarm_c2r(cpu_in.astype(np.complex128))
    b = O.swarm_r2c(a.reshape(-1), n_fft=39 * O.N_A)
    c = O.r2dbe_c2r(b, skip_chan=0, n_out=n_out).ravel()
    scaled = c / (n_out * 2 * O.BENG_CHANNELS_)      # resample.py:138
    ref = g["sample"]
    err = np.abs(scaled[::int(g["stride"])] - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err                             # reference check ran in FP32
    assert abs(scaled.sum() - float(g["sum"])) <= 1e-4 * np.sqrt(float(g["sumsq"]))


def test_skip_chan_from_trim():
    assert O.skip_chan_from_mhz(150) == 1200
    assert O.skip_chan_from_mhz(102) == 816
    assert O.skip_chan_from_mhz(0) == 0
    assert O.skip_chan_from_mhz(240) == 1920
    with pytest.raises(ValueError):
        O.skip_chan_from_mhz(241)
