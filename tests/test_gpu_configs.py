"""Parity at the shapes of the multi-stream and stress workloads, for the FP32
path and both tensor-core precisions.

* Uneven streams (8 phased sums = 4 packet streams x 2): seeded lengths of
  64-512 B-frames and per-stream noise sigma in [0.5, 2] (the 2-bit input
  levels are fixed, so sigma changes the code statistics), all four streams
  in one ``sdbe_process_multi`` pass.  The first batch (which sets the
  thresholds), the middle and the last batch of every stream are checked
  against the FP64 oracle's series and FP64 thresholds.
* Impaired streams with windowed thresholds (2 packet streams x 286
  B-frames of the stress generator: 1% of packets dropped, 0.5% displaced by
  up to 64 places, sigma x4 bursts on 1% of snapshots; 64-batch window):
  every output code against the oracle (FP32 transforms; their own code
  disagreement with FP64 is far below the bar).

Bar: >= 99.9% 2-bit code agreement per stream and pol; thresholds within
1e-5 relative of the oracle's (FP32), 3e-5 (SDBE_PRECISION_TC16), 2e-4
(SDBE_PRECISION_TC16_FAST).  Agreements are printed (``pytest -s``).
"""
import os

import numpy as np
import pytest

from gpu_util import codes_of
from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu

AGREE_MIN = 0.999
THR_TOL = {"fp32": 1e-5, "tc16": 3e-5, "tc16fast": 2e-4}
TRIM = 150


def _prec(N, name):
    return {"fp32": N.PRECISION_FP32, "tc16": N.PRECISION_TC16, "tc16fast": N.PRECISION_TC16_FAST}[name]


def _oracle_batch(p, b_start, b, skip):
    """FP64 series of batch b (both pols) from frame-ordered packets."""
    s0, s1 = b * 143, (b + 1) * 143
    f0, f1 = s0 // 128, (s1 - 1) // 128 + 1
    beng = O.vdif_to_beng(p[f0 * 2048:f1 * 2048], b_start + f0, f1 - f0)
    ys = []
    for pol in range(2):
        spec = O.beng_to_complex(beng[pol].reshape(-1, 16384, 2))[s0 - f0 * 128:s1 - f0 * 128]
        ts = O.swarm_c2r(spec, workers=os.cpu_count() or 1).reshape(-1)
        ys.append(O.r2dbe_c2r(O.swarm_r2c(ts, workers=os.cpu_count() or 1), skip, workers=os.cpu_count() or 1))
    return ys


@pytest.fixture(scope="module")
def uneven():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth as S

    specs = S.config4(n_packet_streams=4)
    pk = [S.generate(sp) for sp in specs]
    skip = O.skip_chan_from_mhz(TRIM)
    refs = []
    for sp, p in zip(specs, pk):
        nb = sp.n_frames * 128 // 143
        picks = sorted({0, nb // 2, nb - 1})
        ys = {b: _oracle_batch(p, sp.b_start, b, skip) for b in picks}
        stats = [O.summary_stats(ys[0][pol]) for pol in range(2)]
        refs.append((nb, picks, ys, stats))
    return specs, pk, refs


@pytest.mark.parametrize("path", ["fp32", "tc16", "tc16fast"])
def test_uneven_streams_multi_vs_oracle(uneven, path):
    from sdbe_gb300 import Resampler, process_multi
    from sdbe_gb300 import _native as N

    specs, pk, refs = uneven
    hs = [Resampler(trim_mhz=TRIM, max_frames=sp.n_frames, precision=_prec(N, path)) for sp in specs]
    try:
        outs, res = process_multi(hs, [(p, sp.n_frames, sp.b_start, None) for sp, p in zip(specs, pk)],
                                  want_results=True)
        thr = [h.thresholds for h in hs]
    finally:
        for h in hs:
            h.close()
    for i, (sp, p, (nb, picks, ys, stats)) in enumerate(zip(specs, pk, refs)):
        assert res[i].n_batches == nb and res[i].packets_accepted == p.shape[0], (i, res[i])
        (th0, th1), (off0, off1), _ = thr[i]
        for pol, (th, off) in enumerate(((th0, off0), (th1, off1))):
            off_o, th_o = stats[pol]
            assert abs(th - th_o) <= THR_TOL[path] * th_o, (i, pol, th, th_o)
            assert abs(off - off_o) <= THR_TOL[path] * th_o, (i, pol, off, off_o)
            for b in picks:
                ref = O.quantize2bit_codes(ys[b][pol], th_o, off_o)
                got = codes_of(outs[i][pol, b * 128:(b + 1) * 128]).reshape(ref.shape)
                agree = float(np.mean(got == ref))
                print(f"{path} stream {i} (sigma {sp.sigma:.2f}, {sp.n_frames} frames) pol {pol} batch {b}: "
                      f"agreement {agree:.6f}")
                assert agree >= AGREE_MIN, (path, i, pol, b, agree)


@pytest.fixture(scope="module")
def impaired():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth as S

    frames = 286
    specs = S.config5(n_packet_streams=2, n_frames=2048)
    pk = [S.generate(sp, frame_offset=0, n_frames=frames) for sp in specs]
    # one oracle process per stream, started with spawn (CUDA may already be
    # initialised in this process)
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    workers = max(1, (os.cpu_count() or 2) // len(specs))
    with ProcessPoolExecutor(len(specs), mp_context=mp.get_context("spawn")) as ex:
        refs = list(ex.map(_oracle_windowed, pk, [sp.b_start for sp in specs], [frames] * len(specs),
                           [workers] * len(specs)))
    return frames, specs, pk, refs


def _oracle_windowed(p, b_start, frames, workers):
    """The oracle's output and final state with 64-batch windowed thresholds."""
    st = O.StreamState()
    out = O.process_group(p, b_start, frames, TRIM, state=st, precision="f32", workers=workers,
                          threshold_window=64)
    return out, st


@pytest.mark.parametrize("path", ["fp32", "tc16fast"])
def test_impaired_windowed_streams_vs_oracle(impaired, path):
    from sdbe_gb300 import Resampler, process_multi
    from sdbe_gb300 import _native as N

    frames, specs, pk, refs = impaired
    hs = [Resampler(trim_mhz=TRIM, max_frames=frames, precision=_prec(N, path), threshold_mode=N.THRESH_WINDOW,
                    threshold_window=64) for _ in specs]
    try:
        outs, res = process_multi(hs, [(p, frames, sp.b_start, None) for sp, p in zip(specs, pk)],
                                  want_results=True)
        thr = [h.thresholds for h in hs]
    finally:
        for h in hs:
            h.close()
    for i, (p, (ref, st)) in enumerate(zip(pk, refs)):
        assert res[i].n_batches == 256 and res[i].packets_accepted == p.shape[0] < frames * 2048, res[i]
        assert res[i].frames_incomplete > 0
        (th0, th1), _, _ = thr[i]
        for pol, th in enumerate((th0, th1)):
            # 256 batches end on a block boundary: the handle already holds the
            # thresholds of the next block, from batches [192, 256)
            _, th_next = O.window_thresholds(st, pol, 256, 64)
            assert abs(th - th_next) <= THR_TOL[path] * th_next, (i, pol, th, th_next)
            agree = float(np.mean(codes_of(outs[i][pol]) == codes_of(ref[pol])))
            print(f"{path} impaired stream {i} pol {pol}: agreement {agree:.6f} over 256 batches")
            assert agree >= AGREE_MIN, (path, i, pol, agree)
