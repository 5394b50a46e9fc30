"""8pac unpack and B-engine header reform on the device, against the
reference's own C code (the committed fixture) and the oracle; and group
assembly fed 8pac units (sdbe_ingest with SDBE_IN_8PAC).

Bar: bit-exact packets and identical reform state (T0, TPREV, BPREV)."""
import os

import numpy as np
import pytest

from conftest import ROOT
from gpu_util import dev, empty, host
from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden", "pac8_reform.npz")
CASES = ["regular", "jitter", "jumps", "corrupt", "random"]
G = O.BENG_FRAMES_PER_GROUP


@pytest.fixture(scope="module")
def P():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import pac8

    return pac8


def _device_transform(P, src, batches):
    st = P.new_state()
    outs, lo = [], 0
    for n in batches:
        d_src = dev(src[lo:lo + n])
        d_dst = empty(8 * n * O.IN_PKT_BYTES)
        P.unpack_8pac(d_src, n, d_dst)
        P.beng_reform(st, d_dst, 8 * n)
        outs.append(host(d_dst).reshape(8 * n, O.IN_PKT_BYTES))
        lo += n
    return np.concatenate(outs), st


def _state_list(st):
    t0 = O.beng_timestamp_decrement(st.t0_sec, st.t0_clk)
    return [t0[0], t0[1], st.tprev_sec, st.tprev_clk, st.bprev]


@pytest.mark.parametrize("case", CASES)
def test_device_matches_reference_fixture(P, case):
    g = np.load(GOLDEN)
    out, st = _device_transform(P, g[f"{case}_in"], g[f"{case}_batches"].tolist())
    ref = g[f"{case}_out"]
    bad = np.nonzero((out != ref).any(axis=1))[0]
    assert bad.size == 0, (case, bad[:5])
    assert _state_list(st) == g[f"{case}_state"].tolist()
    if case == "regular":
        assert st.slow_tiles == 0          # on-grid: the block-scan path
    if case in ("jitter", "jumps", "corrupt"):
        assert st.slow_tiles > 0           # irregular tiles walked one packet at a time
    if case == "jumps":
        assert st.marked_invalid > 0


def test_multi_tile_stream_fast_path_equals_oracle(P):
    """Several 1024-packet tiles with a second boundary, invalid units and
    batch cuts inside tiles: the scan path only, equal to the oracle."""
    from sdbe_gb300 import synth as S

    spec = S.config1()
    p = S.generate(spec, frame_offset=0, n_frames=3)
    units = S.to_8pac(p, 1234, 286000000 - 2 * 262144 + 17, spec.b_start, seed=4)
    w = units.view("<u4").reshape(units.shape[0], -1)
    w[[3, 100, 500], 0] |= np.uint32(1 << 31)                  # invalid units (all 8 packets)
    cuts = [1, 200, 311, units.shape[0] - 512]
    out, st = _device_transform(P, units, cuts)
    ost = O.ReformState()
    ref, lo = [], 0
    for n in cuts:
        ref.append(O.beng_reform_headers(O.unpack_8pac(units[lo:lo + n]), ost))
        lo += n
    assert np.array_equal(out, np.concatenate(ref))
    assert st.slow_tiles == 0 and st.marked_invalid == 0
    assert (st.t0_sec, st.t0_clk, st.tprev_sec, st.tprev_clk, st.bprev) == (*ost.t0, *ost.tprev, ost.bprev)
    inv, c, f, b = O.decode_beng_headers(out)
    assert b[inv == 0].max() == 2 and inv.sum() == 24


def _old_format(p, b_new):
    q = p.copy()
    w = q.view("<u4").reshape(q.shape[0], -1)
    w[:, 4] = (b_new >> 8).astype(np.uint32)
    w[:, 5] = (w[:, 5] & np.uint32(0x00FFFFFF)) | ((b_new & 0xFF).astype(np.uint32) << 24)
    return q


def test_ingest_8pac_equals_ingest_of_reformed_packets(P):
    """A clean stream as 8pac units: groups and statistics equal those of the
    same packets with old-format headers counting from the first frame."""
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import synth as S

    spec = S.config1()
    n_frames = 1 + G + 6
    p = S.generate(spec, frame_offset=0, n_frames=n_frames)
    units = S.to_8pac(p, 88, 285000000, spec.b_start, seed=9)
    inv, c, f, b = O.decode_beng_headers(p)
    plain = _old_format(p, b - spec.b_start)
    per = 4000
    with Resampler(max_frames=G) as a, Resampler(max_frames=G) as r:
        shipped = 0
        for lo in range(0, units.shape[0], per):
            ga, na = a.ingest(units[lo:lo + per], pac8=True)
            gr, nr = r.ingest(plain[8 * lo:8 * (lo + per)])
            assert na == nr
            for i in range(na):
                assert np.array_equal(ga[i], gr[i]), shipped
                shipped += 1
        assert shipped == 1
        sa, sr = a.ingest_stats(), r.ingest_stats()
        assert sa == sr and sa["b_first"] == 0
        rf = a.ingest_reform_state()
        assert (rf.t0_sec, rf.t0_clk, rf.bprev, rf.slow_tiles) == (88, 285000000, n_frames - 1, 0)


def test_ingest_device_packets_equal_host_packets(P):
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import synth as S

    spec = S.config1()
    p = S.generate(spec, frame_offset=0, n_frames=1 + G)
    with Resampler(max_frames=G) as a, Resampler(max_frames=G) as r:
        ga, na = a.ingest(dev(p), n_packets=p.shape[0])
        gr, nr = r.ingest(p)
        assert na == nr == 1 and np.array_equal(ga, gr)
        assert a.ingest_stats() == r.ingest_stats()
