"""Several packet streams in shared FFT launches (sdbe_process_multi) against
the same streams through sdbe_process one by one; and the multi-stream pass
captured into a CUDA graph and replayed.

Bar: bit-exact outputs and identical per-stream results."""
import numpy as np
import pytest

from gpu_util import dev, host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth

    return synth


def _streams(S, frames, seeds):
    out = []
    for f, s in zip(frames, seeds):
        spec = S.config1(stream=s)
        spec.b_start = 1_000_000 + 5000 * s
        p = S.generate(spec, frame_offset=0, n_frames=f)
        out.append((spec, p))
    return out


CFG = [dict(trim_mhz=150, wave_batches=4), dict(trim_mhz=0, wave_batches=8), dict(trim_mhz=240, wave_batches=16)]


@pytest.mark.parametrize("framed", [False, True])
def test_multi_equals_one_by_one_host_buffers(S, framed):
    from sdbe_gb300 import Resampler, process_multi

    frames = [5, 2, 9]
    st = _streams(S, frames, [0, 1, 2])
    ms = [Resampler(max_frames=10, **c) for c in CFG]
    ss = [Resampler(max_frames=10, **c) for c in CFG]
    try:
        for call in range(2):  # second call: carried snapshots, thresholds already set
            items = [(p, f, spec.b_start + call * f, None) for (spec, p), f in zip(st, frames)]
            if call:
                items = [(_rebase(p, spec.b_start, spec.b_start + f), f, spec.b_start + f, None)
                         for (spec, p), f in zip(st, frames)]
            got, res = process_multi(ms, items, framed=framed, want_results=True)
            for i, (r, it) in enumerate(zip(ss, items)):
                want, wres = r.process(it[0], it[1], it[2], framed=framed)
                assert np.array_equal(got[i], want), (call, i)
                assert res[i] == wres, (call, i)
        for a, b in zip(ms, ss):
            assert a.thresholds == b.thresholds
    finally:
        for r in ms + ss:
            r.close()


def _rebase(p, b_from, b_to):
    """The same packets with B-counters shifted from b_from to b_to."""
    q = p.copy()
    w = q.view("<u4").reshape(q.shape[0], -1)
    b = ((w[:, 4].astype(np.int64) << 8) | (w[:, 5].astype(np.int64) >> 24)) - b_from + b_to
    w[:, 4] = (b >> 8).astype(np.uint32)
    w[:, 5] = (w[:, 5] & np.uint32(0x00FFFFFF)) | ((b & 0xFF).astype(np.uint32) << 24)
    return q


def test_multi_graph_capture_replays_the_pass(S):
    """Device buffers: the multi pass captured once and replayed twice equals
    a direct pass of freshly reset handles."""
    import torch

    from sdbe_gb300 import Resampler, process_multi

    frames = [3, 6]
    st = _streams(S, frames, [3, 4])
    ms = [Resampler(max_frames=6, wave_batches=4), Resampler(max_frames=6, wave_batches=4)]
    ds = [Resampler(max_frames=6, wave_batches=4), Resampler(max_frames=6, wave_batches=4)]
    try:
        dpk = [dev(p) for _, p in st]
        outs = [torch.zeros(r.output_bytes(f), dtype=torch.uint8, device="cuda") for r, f in zip(ms, frames)]
        items = [(d, f, spec.b_start, o) for d, f, (spec, _), o in zip(dpk, frames, st, outs)]
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            process_multi(ms, items, stream=torch.cuda.current_stream().cuda_stream)
        for rep in range(2):
            for o in outs:
                o.zero_()
            g.replay()
            torch.cuda.synchronize()
            for r in ds:
                r.reset()
            d_outs = [torch.zeros_like(o) for o in outs]
            d_items = [(d, f, spec.b_start, o) for d, f, (spec, _), o in zip(dpk, frames, st, d_outs)]
            process_multi(ds, d_items)
            for r in ds:
                r.sync()
            for a, b in zip(outs, d_outs):
                assert torch.equal(a, b), rep
                assert int(a.count_nonzero()) > 0
    finally:
        for r in ms + ds:
            r.close()
