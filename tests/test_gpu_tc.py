"""The tensor-core precision form (SDBE_PRECISION_TC16) against the FP64 oracle
and against the FP32 path.

Bar: 2-bit code agreement >= 99.9% against the FP64 oracle, the same bar as
the FP32 path; thresholds within 1e-5 (relative) of the oracle's for
SDBE_PRECISION_TC16 and 2e-4 for SDBE_PRECISION_TC16_FAST (data rounded to FP16).  The
error of the series before requantization is measured in test_gpu_precision.
"""
import numpy as np
import pytest

from gpu_util import codes_of
from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu

AGREE_MIN = 0.999
THR_TOL = 1e-5


@pytest.fixture(scope="module")
def S():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth

    return synth


def _agree(a, b):
    return float(np.mean(codes_of(a) == codes_of(b)))


@pytest.mark.parametrize("fast", [False, True])
def test_tc_process_vs_oracle_and_fp32(S, fast):
    """8 frames (7 batches) in waves of 2: first batch, two full waves and a
    short one; codes against the oracle and against the FP32 path."""
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    spec = S.config1()
    p = S.generate(spec)
    prec = N.PRECISION_TC16_FAST if fast else N.PRECISION_TC16
    thr_tol = 2e-4 if fast else THR_TOL
    with Resampler(trim_mhz=150, max_frames=8, wave_batches=2, precision=prec) as tc, \
            Resampler(trim_mhz=150, max_frames=8, wave_batches=2) as f32:
        out, res = tc.process(p, 8, spec.b_start)
        (th0, th1), (off0, off1), ok = tc.thresholds
        out32, _ = f32.process(p, 8, spec.b_start)
    assert ok and res.n_batches == 7 and out.shape == out32.shape
    st = O.StreamState()
    ref = O.process_group(p, spec.b_start, 8, 150, state=st)
    rows = []
    for pol in range(2):
        for b in range(7):
            sl = slice(b * 128, (b + 1) * 128)
            rows.append({"pol": pol, "batch": b, "agree_oracle": _agree(out[pol, sl], ref[pol, sl]),
                         "agree_fp32": _agree(out[pol, sl], out32[pol, sl])})
    for r in rows:
        assert r["agree_oracle"] >= AGREE_MIN, r
    for pol, th, off in ((0, th0, off0), (1, th1, off1)):
        assert abs(th - st.threshold[pol]) <= thr_tol * st.threshold[pol]
        assert abs(off - st.offset[pol]) <= thr_tol * st.threshold[pol]


def test_tc_carry_and_framed_match_single_call(S):
    """Two calls (3 + 5 frames, snapshot carry between them) equal one call of 8
    frames bit for bit, framed headers included."""
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    spec = S.config1()
    p = S.generate(spec)
    cut = 3 * 2048
    with Resampler(trim_mhz=150, max_frames=8, precision=N.PRECISION_TC16) as a, \
            Resampler(trim_mhz=150, max_frames=8, precision=N.PRECISION_TC16) as b:
        whole, _ = a.process(p, 8, spec.b_start, framed=True)
        o1, r1 = b.process(p[:cut], 3, spec.b_start, framed=True)
        o2, r2 = b.process(p[cut:], 5, spec.b_start + 3, framed=True)
    assert r1.n_batches + r2.n_batches == 7
    assert np.array_equal(np.concatenate([o1, o2], axis=1), whole)


def test_tc_config_errors(S):
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    with pytest.raises(N.SdbeError) as e:
        Resampler(precision=7)
    assert e.value.code == N.ERR_ARG
    spec = S.config1()
    p = S.generate(spec, n_frames=1)
    from sdbe_gb300 import process_multi

    with Resampler(max_frames=2, precision=N.PRECISION_TC16) as a, Resampler(max_frames=2) as b:
        with pytest.raises(N.SdbeError) as e:
            process_multi([a, b], [(p, 1, spec.b_start, None), (p, 1, spec.b_start, None)])
        assert e.value.code == N.ERR_ARG


def _rebase(p, b_from, b_to):
    """The same packets with B-counters shifted from b_from to b_to."""
    q = p.copy()
    w = q.view("<u4").reshape(q.shape[0], -1)
    b = ((w[:, 4].astype(np.int64) << 8) | (w[:, 5].astype(np.int64) >> 24)) - b_from + b_to
    w[:, 4] = (b >> 8).astype(np.uint32)
    w[:, 5] = (w[:, 5] & np.uint32(0x00FFFFFF)) | ((b & 0xFF).astype(np.uint32) << 24)
    return q


@pytest.mark.parametrize("fast", [False, True])
def test_tc_multi_equals_one_by_one(S, fast):
    """sdbe_process_multi over three tensor-core handles (uneven lengths,
    trims 150 / 0 / 240 MHz, waves 4 / 8 / 16) equals sdbe_process one handle
    at a time, bit for bit, over two calls: first batches, then carried
    snapshots with the thresholds set."""
    from sdbe_gb300 import Resampler, process_multi
    from sdbe_gb300 import _native as N

    prec = N.PRECISION_TC16_FAST if fast else N.PRECISION_TC16
    cfg = [dict(trim_mhz=150, wave_batches=4), dict(trim_mhz=0, wave_batches=8), dict(trim_mhz=240, wave_batches=16)]
    frames = [5, 2, 9]
    st = []
    for f, seed in zip(frames, [0, 1, 2]):
        spec = S.config1(stream=seed)
        spec.b_start = 1_000_000 + 5000 * seed
        st.append((spec, S.generate(spec, frame_offset=0, n_frames=f)))
    ms = [Resampler(max_frames=10, precision=prec, **c) for c in cfg]
    ss = [Resampler(max_frames=10, precision=prec, **c) for c in cfg]
    try:
        for call in range(2):
            items = [(p if call == 0 else _rebase(p, spec.b_start, spec.b_start + f), f, spec.b_start + call * f, None)
                     for (spec, p), f in zip(st, frames)]
            got, res = process_multi(ms, items, want_results=True)
            for i, (r, it) in enumerate(zip(ss, items)):
                want, wres = r.process(it[0], it[1], it[2])
                assert np.array_equal(got[i], want), (call, i)
                assert res[i] == wres, (call, i)
        for a, b in zip(ms, ss):
            assert a.thresholds == b.thresholds
    finally:
        for r in ms + ss:
            r.close()


def test_tc_aligned_and_mar2015_match_fp32(S):
    """Time-aligned output and the Mar-2015 channel map run the tensor-core
    chain too: headers equal to the FP32 path's, payload codes >= 99.9% equal."""
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    spec = S.config1()
    p = S.generate(spec, frame_offset=0, n_frames=4)
    for kw in (dict(), dict(channel_map=N.MAP_MAR2015)):
        outs = []
        for prec in (N.PRECISION_FP32, N.PRECISION_TC16):
            with Resampler(trim_mhz=150, max_frames=4, precision=prec, **kw) as rs:
                if not kw:
                    rs.align_start(1_234_567, 285_800_000, ref_epoch=30)
                    o, _ = rs.process(p, 4, spec.b_start, aligned=True)
                else:
                    o, _ = rs.process(p, 4, spec.b_start, framed=True)
                outs.append(o)
        f32, tc = outs
        assert f32.shape == tc.shape and f32.shape[1] > 0, kw
        assert np.array_equal(f32[:, :, :32], tc[:, :, :32]), kw  # VDIF headers
        agree = float(np.mean(codes_of(f32[:, :, 32:]) == codes_of(tc[:, :, 32:])))
        assert agree >= AGREE_MIN, (kw, agree)


def test_tc_ingest_group_equals_process(S):
    """Group assembly (sdbe_ingest) on a tensor-core handle resamples in the
    handle's precision: the shipped group equals sdbe_process of the same
    packets on another tensor-core handle, bit for bit."""
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    G = 143
    spec = S.config1()
    batch = S.generate(spec, frame_offset=0, n_frames=1 + G)
    with Resampler(max_frames=G, precision=N.PRECISION_TC16_FAST) as rs, \
            Resampler(max_frames=G, precision=N.PRECISION_TC16_FAST) as ref, \
            Resampler(max_frames=G) as f32:
        groups, n = rs.ingest(batch)
        assert n == 1
        pk = S.generate(spec, frame_offset=1, n_frames=G)
        want, _ = ref.process(pk, G, spec.b_start + 1)
        assert np.array_equal(groups[0], want)
        got32, _ = f32.process(pk, G, spec.b_start + 1)
        assert float(np.mean(codes_of(groups[0]) == codes_of(got32))) >= AGREE_MIN


@pytest.mark.parametrize("fill", [0x00, 0xFF])
def test_tc_fast_saturated_spectra_stay_finite(S, fill):
    """The fast form keeps its FP16 operands in range with fixed power-of-two
    scales; the largest spectra stress them: every payload byte set to one
    value (0x00: every channel -2 - 2i, 0xFF: +1 + 1i), so that each
    snapshot's time series is one large impulse.  Stage A (float output) and
    stages B + C (sdbe_resample_chunks, through the FP16 time series) against
    the FP64 oracle: finite, relative RMS below the fast form's bound."""
    import torch

    from gpu_util import dev, empty, host, ptr, rel_rms, zeros
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    spec = S.config1()
    nf = 2
    p = S.generate(spec, frame_offset=0, n_frames=nf).copy()
    p[:, 32:] = fill
    snaps = nf * 128
    words = empty(2 * snaps * 2048 * 4, "int32")
    bitmap, counts, rej = zeros(nf * 256), zeros(nf * 4, "int32"), zeros(4, "int32")
    lib = N.lib()
    N.check(lib.sdbe_unpack(ptr(dev(p)), p.shape[0], spec.b_start, nf, 0, ptr(words), snaps * 2048, 0, ptr(bitmap),
                            ptr(counts), ptr(rej), None))
    beng = O.vdif_to_beng(p, spec.b_start, nf)
    sp = O.beng_to_complex(beng[0].reshape(-1, 16384, 2))[:143]
    ts_ref = O.swarm_c2r(sp).reshape(-1)
    with Resampler(trim_mhz=150, max_frames=nf, precision=N.PRECISION_TC16_FAST) as rs:
        ts = empty(143 * 32768 * 4, "float32")
        y = empty(128 * 32768 * 4, "float32")
        N.check(lib.sdbe_swarm_c2r(rs.handle, ptr(words), 143, ptr(ts), None), rs.handle)
        N.check(lib.sdbe_resample_chunks(rs.handle, ptr(dev(ts_ref.astype(np.float32))), 128, ptr(y), None),
                rs.handle)
        ref = O.r2dbe_c2r(O.swarm_r2c(ts_ref), rs.skip_chan)
        got_ts, got_y = host(ts).astype(np.float64), host(y).reshape(128, 32768).astype(np.float64)
    torch.cuda.synchronize()
    assert np.isfinite(got_ts).all() and np.isfinite(got_y).all()
    assert rel_rms(got_ts, ts_ref) < 2e-3
    assert rel_rms(got_y, ref) < 2e-3
