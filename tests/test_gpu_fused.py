"""One persistent launch per wave (SDBE_STAGES_FUSED, ``k_tcf_chain``) against
three launches per wave (SDBE_STAGES_SPLIT) in the fast tensor-core form.

The fused launch runs the same per-item code on tickets from a device work
queue, so its payloads, thresholds and window state equal the three-launch
path's bit for bit: one stream in waves smaller and larger than the grid,
several handles in one sdbe_process_multi pass, and windowed thresholds
(the stage-C variant that also sums each chunk).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth

    return synth


def _pair(N, **kw):
    from sdbe_gb300 import Resampler

    return (Resampler(precision=N.PRECISION_TC16_FAST, stage_launches=N.STAGES_FUSED, **kw),
            Resampler(precision=N.PRECISION_TC16_FAST, stage_launches=N.STAGES_SPLIT, **kw))


@pytest.mark.parametrize("frames,wave", [(8, 2), (40, 16)])
def test_fused_equals_split_one_stream(S, frames, wave):
    from sdbe_gb300 import _native as N

    spec = S.config2(n_frames=frames)
    p = S.generate(spec)
    fu, sp = _pair(N, trim_mhz=150, max_frames=frames, wave_batches=wave)
    try:
        for r in (fu, sp):
            r.profile(True)
        a, ra = fu.process(p, frames, spec.b_start)
        b, rb = sp.process(p, frames, spec.b_start)
        pa, pb = fu.read_profile(), sp.read_profile()
        assert ra == rb and ra.n_batches > 1
        assert np.array_equal(a, b)
        assert fu.thresholds == sp.thresholds
        waves = -(-(ra.n_batches - 1) // wave)  # after the first-batch wave
        assert pa.fused_launches == waves and pa.stage_a_launches == 0 and pa.stage_bc_launches == 0
        assert pb.fused_launches == 0 and pb.stage_a_launches == waves
        assert pa.fused_chunks == pb.stage_bc_chunks
        assert pa.launches == pb.launches - 2 * waves
    finally:
        fu.close()
        sp.close()


def test_fused_equals_split_multi(S):
    """Three handles (uneven lengths, trims 150 / 0 / 240 MHz) in one
    sdbe_process_multi pass per call, two calls (thresholds set in the
    first, carried snapshots in the second)."""
    from sdbe_gb300 import Resampler, process_multi
    from sdbe_gb300 import _native as N

    cfg = [dict(trim_mhz=150), dict(trim_mhz=0), dict(trim_mhz=240)]
    frames = [6, 3, 11]
    streams = []
    for f, seed in zip(frames, [3, 4, 5]):
        spec = S.config1(stream=seed)
        spec.b_start = 2_000_000 + 7000 * seed
        streams.append((spec, S.generate(spec, frame_offset=0, n_frames=2 * f)))
    fu = [Resampler(max_frames=12, wave_batches=4, precision=N.PRECISION_TC16_FAST, stage_launches=N.STAGES_FUSED, **c)
          for c in cfg]
    sp = [Resampler(max_frames=12, wave_batches=4, precision=N.PRECISION_TC16_FAST, stage_launches=N.STAGES_SPLIT, **c)
          for c in cfg]
    try:
        for call in range(2):
            items = [(p[call * f * 2048:(call + 1) * f * 2048], f, spec.b_start + call * f, None)
                     for (spec, p), f in zip(streams, frames)]
            got_f, res_f = process_multi(fu, items, want_results=True)
            got_s, res_s = process_multi(sp, items, want_results=True)
            for i in range(3):
                assert res_f[i] == res_s[i], (call, i)
                assert np.array_equal(got_f[i], got_s[i]), (call, i)
        for a, b in zip(fu, sp):
            assert a.thresholds == b.thresholds
    finally:
        for r in fu + sp:
            r.close()


def test_fused_equals_split_windowed(S):
    """Windowed thresholds: stage C also sums each chunk; the thresholds
    adapt over the run and both paths follow the same sequence."""
    from sdbe_gb300 import _native as N

    frames = 24
    spec = S.config2(n_frames=frames)
    p = S.generate(spec)
    fu, sp = _pair(N, trim_mhz=150, max_frames=frames, wave_batches=4, threshold_mode=N.THRESH_WINDOW,
                   threshold_window=4)
    try:
        for call in range(2):
            sl = p[call * 12 * 2048:(call + 1) * 12 * 2048]
            a, ra = fu.process(sl, 12, spec.b_start + 12 * call)
            b, rb = sp.process(sl, 12, spec.b_start + 12 * call)
            assert ra == rb
            assert np.array_equal(a, b), call
            assert fu.thresholds == sp.thresholds, call
    finally:
        fu.close()
        sp.close()
