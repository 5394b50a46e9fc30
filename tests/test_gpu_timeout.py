"""Bounded mbarrier waits of the tensor-core kernels (failure detection
without a GPU fault).

``sdbe_test_tc_timeout`` arms a handle so that its next fast tensor-core
launch withholds one MMA completion signal and bounds every mbarrier wait by
a short limit.  The wait on the withheld signal runs out; the kernel records
the time-out, frees its tensor memory and returns.  The call after it fails
with SDBE_ERR_CUDA, and a fresh handle on the same device then processes the
stream correctly (the context stayed usable)."""
import time

import numpy as np
import pytest

from gpu_util import codes_of
from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu


def test_tc_wait_timeout_is_reported_and_context_survives():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import Resampler, synth
    from sdbe_gb300 import _native as N

    spec = synth.config1()
    spec.n_frames = 4
    p = synth.generate(spec)
    lib = N.lib()
    with Resampler(trim_mhz=150, max_frames=4, precision=N.PRECISION_TC16_FAST) as rs:
        # the hook refuses out-of-range limits
        assert lib.sdbe_test_tc_timeout(rs.handle, 10) == N.ERR_ARG
        N.check(lib.sdbe_test_tc_timeout(rs.handle, 2_000_000), rs.handle)  # 2 ms
        t0 = time.perf_counter()
        try:
            rs.process(p, 4, spec.b_start)
        except N.SdbeError as e:  # the flag may already be seen by a later wave of the same call
            assert e.code == N.ERR_CUDA, e
        rs.sync()
        elapsed = time.perf_counter() - t0
        with pytest.raises(N.SdbeError) as ei:
            rs.process(p, 4, spec.b_start)
        assert ei.value.code == N.ERR_CUDA and "timed out" in str(ei.value), ei.value
    assert elapsed < 5.0, elapsed  # bounded: no wait ran to its 1 s default
    # a fresh handle on the same context processes the stream correctly
    with Resampler(trim_mhz=150, max_frames=4, precision=N.PRECISION_TC16_FAST) as rs:
        out, res = rs.process(p, 4, spec.b_start)
    ref = O.process_group(p, spec.b_start, 4, 150)
    nb = res.n_batches
    assert nb == 3
    agree = float(np.mean(codes_of(out[:, :nb * 128]) == codes_of(ref[:, :nb * 128])))
    print(f"after the time-out, fresh handle: agreement {agree:.6f}")
    assert agree >= 0.999
