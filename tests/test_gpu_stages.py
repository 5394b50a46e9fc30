"""Per-stage parity of the CUDA kernels against the CPU oracle, through the C ABI.

Integer stages (unpack, fill, complex conversion, quantize, VDIF headers,
reorder) must match bit for bit.  FFT stages are FP32 against the FP64 oracle
with the relative-RMS tolerance stated per test.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import crel_rms, dev, empty, host, packed_to_complex, ptr, rel_rms, zeros
from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu

FFT_REL_RMS_TOL = 2e-6   # FP32 radix FFT vs FP64, per transform stage


@pytest.fixture(scope="module")
def N():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import _native

    return _native


@pytest.fixture(scope="module")
def rs(N):
    from sdbe_gb300 import Resampler

    r = Resampler(trim_mhz=150, max_frames=16)
    yield r
    r.close()


def _impaired_packets(synth_mod, n_frames=2, seed_stream=0):
    spec = synth_mod.config1(stream=seed_stream)
    spec.n_frames = n_frames
    p = synth_mod.generate(spec).copy()
    rng = np.random.default_rng(5)
    keep = np.ones(p.shape[0], bool)
    keep[rng.choice(p.shape[0], 40, replace=False)] = False      # drops
    p = p[keep]
    p = p[rng.permutation(p.shape[0])]                            # arbitrary order
    w = p.view("<u4").reshape(p.shape[0], -1)
    w[0, 0] |= np.uint32(1 << 31)                                 # invalid flag
    w[1, 5] = (w[1, 5] & np.uint32(0xFF00FFFF)) | np.uint32(9 << 16)  # f = 9
    b_bad = spec.b_start + n_frames + 3                           # beyond the window
    w[2, 4] = np.uint32(b_bad >> 8)
    w[2, 5] = (w[2, 5] & np.uint32(0x00FFFFFF)) | np.uint32((b_bad & 0xFF) << 24)
    return p, spec.b_start


@pytest.fixture(scope="module")
def synth_mod(N):
    from sdbe_gb300 import synth

    return synth


def test_vdif_to_beng_bit_exact(N, synth_mod):
    p, b0 = _impaired_packets(synth_mod)
    nf = 2
    d = dev(p)
    nbytes = nf * 128 * 16384 * 2
    e0, e1 = empty(nbytes, "int8"), empty(nbytes, "int8")
    N.check(N.lib().sdbe_vdif_to_beng(ptr(d), p.shape[0], b0, nf, 0, ptr(e0), ptr(e1), None))
    r0, r1 = O.vdif_to_beng(p, b0, nf)
    np.testing.assert_array_equal(host(e0).reshape(r0.shape), r0)
    np.testing.assert_array_equal(host(e1).reshape(r1.shape), r1)


def test_unpack_packed_fill_and_completion(N, synth_mod):
    p, b0 = _impaired_packets(synth_mod, seed_stream=1)
    nf, snap0 = 2, 5
    snaps = snap0 + nf * 128
    pol_stride = snaps * 2048
    spec = empty(2 * pol_stride * 4, "int32")
    bitmap = zeros(nf * 256)
    counts = zeros(nf * 4, "int32")
    rej = zeros(4, "int32")
    lib = N.lib()
    d = dev(p)
    N.check(lib.sdbe_unpack(ptr(d), p.shape[0], b0, nf, 0, ptr(spec), pol_stride, snap0, ptr(bitmap),
                            ptr(counts), ptr(rej), None))
    N.check(lib.sdbe_fill_missing(ptr(bitmap), nf, 0, ptr(spec), pol_stride, snap0, None))
    words = host(spec).view(np.uint32).reshape(2, snaps, 2048)[:, snap0:]
    r = O.vdif_to_beng(p, b0, nf)
    for pol in range(2):
        ref = O.beng_to_complex(r[pol].reshape(-1, 16384, 2))
        np.testing.assert_array_equal(packed_to_complex(words[pol]), ref)
    cc, cnt = O.completion_bitmap(p, b0, nf)
    np.testing.assert_array_equal(host(bitmap).reshape(nf, 256), cc)
    np.testing.assert_array_equal(host(counts), cnt)
    assert host(rej)[0] == 3


def test_beng_to_complex_exact(N):
    rng = np.random.default_rng(3)
    beng = rng.integers(-2, 2, size=(3, 16384, 2)).astype(np.int8)
    out = empty(3 * 16385 * 8, "float32")
    N.check(N.lib().sdbe_beng_to_complex(ptr(dev(beng)), 3, ptr(out), None))
    got = host(out).view(np.complex64).reshape(3, 16385)
    np.testing.assert_array_equal(got, O.beng_to_complex(beng).astype(np.complex64))


def _packed_spectra(N, synth_mod, n_frames=2):
    spec = synth_mod.config1(stream=2)
    spec.n_frames = n_frames
    p = synth_mod.generate(spec)
    snaps = n_frames * 128
    words = empty(2 * snaps * 2048 * 4, "int32")
    bitmap = zeros(n_frames * 256)
    counts = zeros(n_frames * 4, "int32")
    rej = zeros(4, "int32")
    lib = N.lib()
    N.check(lib.sdbe_unpack(ptr(dev(p)), p.shape[0], spec.b_start, n_frames, 0, ptr(words), snaps * 2048, 0,
                            ptr(bitmap), ptr(counts), ptr(rej), None))
    return words, snaps


def test_swarm_c2r_vs_oracle(N, rs, synth_mod):
    words, snaps = _packed_spectra(N, synth_mod)
    out = empty(snaps * 32768 * 4, "float32")
    N.check(N.lib().sdbe_swarm_c2r(rs.handle, ptr(words), snaps, ptr(out), None), rs.handle)
    got = host(out).reshape(snaps, 32768)
    ref = O.swarm_c2r(packed_to_complex(host(words).view(np.uint32).reshape(2, snaps, 2048)[0]))
    err = rel_rms(got, ref)
    assert err < FFT_REL_RMS_TOL, err


def test_swarm_r2c_vs_oracle(N, rs):
    rng = np.random.default_rng(11)
    x = (rng.standard_normal((4, 36608)) * 180).astype(np.float32)
    out = empty(4 * 18305 * 8, "float32")
    N.check(N.lib().sdbe_swarm_r2c(rs.handle, ptr(dev(x)), 4, ptr(out), None), rs.handle)
    got = host(out).view(np.complex64).reshape(4, 18305)
    ref = O.swarm_r2c(x.astype(np.float64).reshape(-1))
    err = crel_rms(got, ref)
    assert err < FFT_REL_RMS_TOL, err


@pytest.mark.parametrize("skip", [0, 816, 1200, 1920])
def test_r2dbe_c2r_vs_oracle(N, rs, skip):
    rng = np.random.default_rng(12 + skip)
    y = (rng.standard_normal((3, 18305)) + 1j * rng.standard_normal((3, 18305))).astype(np.complex64)
    out = empty(3 * 32768 * 4, "float32")
    N.check(N.lib().sdbe_r2dbe_c2r(rs.handle, ptr(dev(y.view(np.float32))), 3, skip, ptr(out), None), rs.handle)
    got = host(out).reshape(3, 32768)
    ref = O.r2dbe_c2r(y.astype(np.complex128), skip)
    err = rel_rms(got, ref)
    assert err < FFT_REL_RMS_TOL, err


def test_resample_chunks_fused_vs_oracle(N, rs):
    rng = np.random.default_rng(13)
    x = (rng.standard_normal((5, 36608)) * 180).astype(np.float32)
    d = dev(x)
    out = empty(5 * 32768 * 4, "float32")
    N.check(N.lib().sdbe_resample_chunks(rs.handle, ptr(d), 5, ptr(out), None), rs.handle)
    got = host(out).reshape(5, 32768)
    ref = O.r2dbe_c2r(O.swarm_r2c(x.astype(np.float64).reshape(-1)), rs.skip_chan)
    err = rel_rms(got, ref)
    assert err < 2 * FFT_REL_RMS_TOL, err
    # fused == the two stage kernels composed, to FP32 rounding
    mid = empty(5 * 18305 * 8, "float32")
    out2 = empty(5 * 32768 * 4, "float32")
    lib = N.lib()
    N.check(lib.sdbe_swarm_r2c(rs.handle, ptr(d), 5, ptr(mid), None), rs.handle)
    N.check(lib.sdbe_r2dbe_c2r(rs.handle, ptr(mid), 5, rs.skip_chan, ptr(out2), None), rs.handle)
    assert rel_rms(got, host(out2).reshape(5, 32768)) < 1e-6


def test_summary_stats_fp64(N):
    rng = np.random.default_rng(14)
    y = (rng.standard_normal(1_000_003) * 7.0e6 + 3.0e4).astype(np.float32)
    out = (C.c_double * 2)()
    N.check(N.lib().sdbe_summary_stats(ptr(dev(y)), y.size, out, None))
    mean, std = O.summary_stats(y)
    assert abs(out[0] - mean) <= 1e-9 * abs(std)
    assert abs(out[1] - std) <= 1e-9 * std


def test_quantize2bit_bit_exact(N):
    rng = np.random.default_rng(15)
    th, off = np.float32(1.25), np.float32(0.125)
    y = (rng.standard_normal(4096 * 16) * 1.3).astype(np.float32)
    y[:6] = [off - th, off + th, off, off - 0.0, -np.inf, np.inf]
    out = empty(y.size // 16 * 4, "int32")
    N.check(N.lib().sdbe_quantize2bit(ptr(dev(y)), ptr(out), y.size, float(th), float(off), None))
    ref = O.pack2bit(O.quantize2bit_codes(y, th, off, np.float32))
    np.testing.assert_array_equal(host(out).view(np.uint32), ref)


def test_vdif_headers_exact(N):
    n = 7
    frames = zeros(2 * n * 8224)
    N.check(N.lib().sdbe_vdif_headers(ptr(frames), n, n * 8224, 77, 124997, 2**32 - 3, 30,
                                      (ord("S") << 8) | ord("m"), 1, 0, None))
    got = host(frames).reshape(2, n, 8224)
    for pol in range(2):
        ref = O.vdif_out_header_words(n, pol, secs=77, df=124997, psn=2**32 - 3, ref_epoch=30,
                                      bdc_sideband=1, rx_sideband=0)
        np.testing.assert_array_equal(got[pol, :, :32].view("<u4"), ref)
        assert not got[pol, :, 32:].any()


def test_reorder_mar2015_exact(N):
    rng = np.random.default_rng(16)
    nf = 3
    words = rng.integers(0, 2**32, size=(nf, 128, 2048), dtype=np.uint64).astype(np.uint32)
    out = empty((nf - 1) * 128 * 2048 * 4, "int32")
    N.check(N.lib().sdbe_reorder_mar2015(ptr(dev(words)), nf, ptr(out), None))
    got = host(out).view(np.uint32).reshape(nf - 1, 128, 2048)
    nib = (words[..., None] >> (4 * np.arange(8, dtype=np.uint32))) & 0xF      # [f][s][g][k]
    chan = nib.reshape(nf, 128, 16384)
    ref = O.reorder_mar2015(chan).reshape(nf - 1, 128, 2048, 8).astype(np.uint32)
    ref_words = np.bitwise_or.reduce(ref << (4 * np.arange(8, dtype=np.uint32)), axis=-1)
    np.testing.assert_array_equal(got, ref_words)


def test_misaligned_pointers_refused(N, rs):
    """The stage entry points refuse device pointers that their kernels'
    vector accesses cannot take, with SDBE_ERR_ARG and no launch."""
    lib = N.lib()
    buf = zeros(4 * 36608 * 4 + 64)
    out = zeros(4 * 32768 * 4 + 64)
    base, obase = ptr(buf), ptr(out)
    assert lib.sdbe_resample_chunks(rs.handle, base + 4, 1, obase, None) == N.ERR_ARG
    assert lib.sdbe_resample_chunks(rs.handle, base, 1, obase + 8, None) == N.ERR_ARG
    assert lib.sdbe_swarm_c2r(rs.handle, base + 4, 1, obase, None) == N.ERR_ARG
    assert lib.sdbe_swarm_r2c(rs.handle, base + 4, 1, obase, None) == N.ERR_ARG
    assert lib.sdbe_r2dbe_c2r(rs.handle, base + 4, 1, 1200, obase, None) == N.ERR_ARG
    assert lib.sdbe_quantize2bit(base + 4, obase, 16, 1.0, 0.0, None) == N.ERR_ARG
    assert lib.sdbe_beng_to_complex(base + 1, 1, obase, None) == N.ERR_ARG
    assert lib.sdbe_unpack(base + 8, 1, 0, 1, 0, obase, 0, 0, obase, obase, obase, None) == N.ERR_ARG
    # the aligned call still works afterwards (nothing was launched or left pending)
    N.check(lib.sdbe_resample_chunks(rs.handle, base, 1, obase, None), rs.handle)
    N.check(lib.sdbe_sync(rs.handle), rs.handle)
