"""GPU test of sdbe_summary_stats_noalloc, the entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (threads sharing the device with
asynchronous copies that an allocation would stall, or processes held to a
fixed amount of device memory), so its scratch is a fixed device array inside the
library.  Its results must match the allocating sdbe_summary_stats within the
tolerance of the other statistics test (1e-9 relative, FP64), on two calls in
a row with different data (the array keeps the previous call's contents).
Named so that pytest collects it last.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-9


@pytest.fixture(scope="module")
def N():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import _native

    return _native


def _stats(N, fn, t):
    out = (C.c_double * 2)()
    rc = getattr(N.lib(), fn)(C.c_void_p(t.data_ptr()), t.numel(), out, None)
    N.check(rc)
    return out[0], out[1]


def test_noalloc_matches_allocating_entry_point_twice(N):
    import torch

    g = torch.Generator(device="cuda").manual_seed(2024)
    first = torch.randn(4_194_304, device="cuda", generator=g) * 6.3e6 + 2.5e4
    second = torch.randn(1_000_003, device="cuda", generator=g) * 0.7 - 3.0
    for t in (first, second):
        mean_ref, std_ref = _stats(N, "sdbe_summary_stats", t)
        mean, std = _stats(N, "sdbe_summary_stats_noalloc", t)
        assert abs(mean - mean_ref) <= REL_TOL * std_ref
        assert abs(std - std_ref) <= REL_TOL * std_ref


def test_noalloc_largest_size_and_rejects_larger(N):
    import torch

    n = N.NOALLOC_MAX_SAMPLES
    t = torch.empty(n + 1, device="cuda", dtype=torch.float32)
    t.uniform_(-1.0, 1.0, generator=torch.Generator(device="cuda").manual_seed(7))
    mean_ref, std_ref = _stats(N, "sdbe_summary_stats", t[:n])
    mean, std = _stats(N, "sdbe_summary_stats_noalloc", t[:n])
    assert abs(mean - mean_ref) <= REL_TOL * std_ref and abs(std - std_ref) <= REL_TOL * std_ref
    out = (C.c_double * 2)()
    rc = N.lib().sdbe_summary_stats_noalloc(C.c_void_p(t.data_ptr()), n + 1, out, None)
    assert rc == N.ERR_CAPACITY
    assert "exceeds the maximum" in N.last_error()


def test_large_offset_against_oracle(N):
    """A common offset 1e4 times the spread: both entry points sum the samples
    minus the first one, so the variance keeps its digits (FP64 oracle)."""
    import torch

    from oracle import sdbe_oracle as O

    g = torch.Generator(device="cuda").manual_seed(99)
    t = torch.randn(2_000_000, device="cuda", generator=g) * 0.5 + 5.0e3
    x = t.cpu().numpy()
    mean_o, std_o = O.summary_stats(x)
    for fn in ("sdbe_summary_stats", "sdbe_summary_stats_noalloc"):
        mean, std = _stats(N, fn, t)
        assert abs(mean - mean_o) <= REL_TOL * std_o * 1e3, fn
        assert abs(std - std_o) <= 1e-9 * std_o, fn
