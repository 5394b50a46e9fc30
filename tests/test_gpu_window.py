"""Windowed thresholds (SDBE_THRESH_WINDOW) against the oracle's restatement,
on a stream whose noise power steps up: the first-batch thresholds of the
reference stay where the first batch put them, the windowed ones follow.

Bar: >= 99.9% 2-bit code agreement with the oracle, thresholds within 1e-5
relative (FP32 path; 3e-5 for the tensor-core paths), outputs independent of
the wave size."""
import os

import numpy as np
import pytest

from gpu_util import codes_of
from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def step_stream():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth as S

    lo = S.config1(stream=7)
    lo.b_start = 3_000_000
    hi = S.config1(stream=7)
    hi.b_start = lo.b_start
    hi.sigma = 4.0   # the 2-bit input saturates: about 1.45x the output rms
    p = np.concatenate([S.generate(lo, frame_offset=0, n_frames=10), S.generate(hi, frame_offset=10, n_frames=30)])
    return lo.b_start, p


def _outer(codes):
    return float(np.mean((codes == 0) | (codes == 3)))


def test_window_thresholds_match_oracle_and_adapt(step_stream):
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    b0, p = step_stream
    W = 16
    with Resampler(max_frames=40, threshold_mode=N.THRESH_WINDOW, threshold_window=W, wave_batches=4) as a, \
            Resampler(max_frames=40, threshold_mode=N.THRESH_WINDOW, threshold_window=W, wave_batches=16) as b, \
            Resampler(max_frames=40) as ref_mode:
        out_a, res = a.process(p, 40, b0)
        out_b, _ = b.process(p, 40, b0)
        out_r, _ = ref_mode.process(p, 40, b0)
        (th0, th1), (off0, off1), _ = a.thresholds
    assert res.n_batches == 35
    assert np.array_equal(out_a, out_b)                      # wave size does not matter
    st = O.StreamState()
    ref = O.process_group(p, b0, 40, 150, state=st, precision="f32", workers=os.cpu_count() or 1,
                          threshold_window=W)
    for pol in range(2):
        agree = float(np.mean(codes_of(out_a[pol]) == codes_of(ref[pol])))
        assert agree >= 0.999, (pol, agree)
    assert abs(th0 - st.threshold[0]) <= 1e-5 * st.threshold[0]
    assert abs(th1 - st.threshold[1]) <= 1e-5 * st.threshold[1]
    assert abs(off0 - st.offset[0]) <= 1e-5 * st.threshold[0]
    # after the step, the last block (batches 32-34) is quantized with thresholds
    # from batches 16-31, all at the new power: the fraction of outer codes
    # returns to that of the first batches (threshold = own rms); the
    # reference's once-set thresholds give many more
    first = slice(0, 8 * 128)
    last = slice(32 * 128, 35 * 128)
    for pol in range(2):
        f_first = _outer(codes_of(out_a[pol, first]))
        f_win = _outer(codes_of(out_a[pol, last]))
        f_ref = _outer(codes_of(out_r[pol, last]))
        assert abs(f_win - f_first) < 0.04, (f_first, f_win)
        assert f_ref > f_win + 0.1, (f_ref, f_win)


@pytest.mark.parametrize("fast", [False, True])
def test_window_thresholds_tensor_core_paths(step_stream, fast):
    """The tensor-core chains with windowed thresholds, against the oracle."""
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    b0, p = step_stream
    W = 16
    prec = N.PRECISION_TC16_FAST if fast else N.PRECISION_TC16
    kw = dict(max_frames=40, threshold_mode=N.THRESH_WINDOW, threshold_window=W, precision=prec)
    with Resampler(wave_batches=4, **kw) as a, Resampler(wave_batches=16, **kw) as b:
        out_a, res = a.process(p, 40, b0)
        out_b, _ = b.process(p, 40, b0)
        (th0, th1), _, _ = a.thresholds
    assert res.n_batches == 35
    assert np.array_equal(out_a, out_b)
    st = O.StreamState()
    ref = O.process_group(p, b0, 40, 150, state=st, precision="f32", workers=os.cpu_count() or 1,
                          threshold_window=W)
    for pol in range(2):
        agree = float(np.mean(codes_of(out_a[pol]) == codes_of(ref[pol])))
        assert agree >= 0.999, (pol, agree)
    assert abs(th0 - st.threshold[0]) <= 3e-5 * st.threshold[0]
    assert abs(th1 - st.threshold[1]) <= 3e-5 * st.threshold[1]
