"""Group assembly on the device (sdbe_ingest) against the ingest policy of the
oracle and against sdbe_process on the packets each group accepted.

Bar: per-batch ship counts, the accept decisions (through the statistics) and
every shipped group bit-exact: a group assembled from received packets equals
sdbe_process over the packets the oracle policy let into that group.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu

G = O.BENG_FRAMES_PER_GROUP


@pytest.fixture(scope="module")
def S():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth

    return synth


def _b_of(rows):
    w = np.ascontiguousarray(rows[:, :24]).view("<u4")
    return ((w[:, 4].astype(np.int64) << 8) | (w[:, 5].astype(np.int64) >> 24))


def _with_b(rows, b):
    r = np.ascontiguousarray(rows).copy()
    w = r.view("<u4")
    w[:, 4] = np.uint32(b >> 8)
    w[:, 5] = (w[:, 5] & np.uint32(0x00FFFFFF)) | np.uint32((b & 0xFF) << 24)
    return r


def _stats_equal(rs, st):
    got = rs.ingest_stats()
    want = dict(st.stats, b_first=st.b_first)
    assert got == want


def test_complete_groups_framed_equal_process(S):
    """A clean stream: each group ships in the batch that completes it, framed
    output (headers continue the handle counters) equal to sdbe_process."""
    from sdbe_gb300 import Resampler

    spec = S.config1()
    n_frames = 1 + 2 * G
    per = 13
    with Resampler(max_frames=G) as rs, Resampler(max_frames=G) as ref:
        ships = []
        for k, lo in enumerate(range(0, n_frames, per)):
            batch = S.generate(spec, frame_offset=lo, n_frames=min(per, n_frames - lo))
            groups, n = rs.ingest(batch, framed=True)
            for i in range(n):
                g = len(ships)
                ships.append(k)
                want, _ = ref.process(S.generate(spec, frame_offset=1 + G * g, n_frames=G), G,
                                      spec.b_start + 1 + G * g, framed=True)
                assert np.array_equal(groups[i], want), g
        assert ships == [G // per, (2 * G) // per]
        s = rs.ingest_stats()
        assert s["b_first"] == spec.b_start and s["before_start"] == 2048
        assert s["used"] == 2 * G * 2048 and s["groups_shipped"] == 2 and s["groups_incomplete"] == 0
        _, n = rs.ingest_flush()
        assert n == 0


def _impaired_stream(S, rng):
    """Frame 0, then 5 frames of each of groups 0-4 with 1% drops (one frame
    complete plus 4 duplicate packets), shuffled in windows of 3000 packets,
    then a late, a far-ahead and an invalid packet."""
    spec = S.config1()
    drop = S.config1()
    drop.drop_frac = 0.01
    parts = [S.generate(spec, frame_offset=0, n_frames=1)]
    for g in range(5):
        for j, k in enumerate(sorted(rng.choice(G, 5, replace=False))):
            fo = 1 + G * g + int(k)
            if g == 1 and j == 2:
                full = S.generate(spec, frame_offset=fo, n_frames=1)
                parts += [full, full[:4]]
            else:
                parts.append(S.generate(drop, frame_offset=fo, n_frames=1))
    rows = np.concatenate(parts)
    for lo in range(0, rows.shape[0], 3000):
        seg = rows[lo:lo + 3000]
        rows[lo:lo + 3000] = seg[rng.permutation(seg.shape[0])]
    b0 = spec.b_start
    late = _with_b(rows[:1], b0 + 3)
    far = _with_b(rows[:1], b0 + 1 + G * 20)
    bad = rows[5:6].copy()
    bad.view("<u4")[:, 0] |= np.uint32(1 << 31)
    tail = np.concatenate([late, far, bad])
    cuts = np.sort(rng.choice(np.arange(4000, rows.shape[0]), 6, replace=False))
    batches = np.split(rows, cuts) + [tail]
    return spec, batches


def test_impaired_stream_matches_oracle_policy_and_process(S):
    from sdbe_gb300 import Resampler

    rng = np.random.default_rng(21)
    spec, batches = _impaired_stream(S, rng)
    st = O.IngestState()
    accepted = {}
    n_shipped = 0
    with Resampler(max_frames=G) as rs, Resampler(max_frames=G) as ref:

        def check(groups, n, ships):
            nonlocal n_shipped
            assert n == len(ships)
            for i, g in enumerate(ships):
                assert g == n_shipped
                n_shipped += 1
                pk = accepted.pop(g, np.zeros((0, O.IN_PKT_BYTES), np.uint8))
                want, _ = ref.process(pk, G, st.start(g))
                assert np.array_equal(groups[i], want), g

        for batch in batches:
            acc, ships = O.ingest_policy(batch, st)
            got = batch[acc]
            gid = (_b_of(got) - st.b_first - 1) // G
            for g in np.unique(gid):
                prev = accepted.get(int(g))
                new = got[gid == g]
                accepted[int(g)] = new if prev is None else np.concatenate([prev, new])
            groups, n = rs.ingest(batch)
            check(groups, n, ships)
            _stats_equal(rs, st)
        _, ships = O.ingest_policy(np.zeros((0, O.IN_PKT_BYTES), np.uint8), st, flush=True)
        groups, n = rs.ingest_flush(out_groups=4)
        check(groups, n, ships)
        _stats_equal(rs, st)
    s = st.stats
    assert s["groups_incomplete"] == s["groups_shipped"] == 5
    assert s["overflow"] == 4 and s["too_far_ahead"] == 1 and s["invalid"] == 1 and s["before_start"] >= 2049


def test_capacity_error_reports_groups_and_keeps_state(S):
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    spec = S.config1()
    a = S.generate(spec, frame_offset=0, n_frames=2)
    ahead = S.generate(spec, frame_offset=1 + 3 * G, n_frames=1)[:8]
    with Resampler(max_frames=G) as rs:
        rs.ingest(a)
        before = rs.ingest_stats()
        n = C.c_int32(-1)
        rc = rs._lib.sdbe_ingest(rs.handle, ahead.ctypes.data, ahead.shape[0], None, 0, N.OUT_HOST, C.byref(n))
        assert rc == N.ERR_CAPACITY and n.value == 1
        assert rs.ingest_stats() == before
        groups, n = rs.ingest(ahead)
        assert n == 1 and groups.shape == (1, 2, 16384, 8192)
        s = rs.ingest_stats()
        assert s["groups_shipped"] == 1 and s["groups_incomplete"] == 1 and s["used"] == 2048 + 8


def test_ingest_rejects_mar2015_map(S):
    from sdbe_gb300 import Resampler
    from sdbe_gb300 import _native as N

    spec = S.config1()
    p = S.generate(spec, frame_offset=0, n_frames=1)
    with Resampler(max_frames=G, channel_map=N.MAP_MAR2015) as rs:
        with pytest.raises(N.SdbeError) as e:
            rs.ingest(p)
        assert e.value.code == N.ERR_STATE


@pytest.mark.parametrize("case", ["sparse", "overflow", "boundary", "far", "complete"])
def test_device_policy_on_reference_scenarios(S, case):
    """The group assembly decisions, made on the device, over the seeded
    ingest scenarios whose per-packet outcomes and ships the reference's own
    C code recorded (tests/golden/hostlogic.npz, through the oracle it pins):
    invalid, early, late and too-far packets, frames over 2048 packets (the
    first ones in arrival order kept), look-ahead and completion ships.  After
    every batch the device's accept flag of every packet, the statistics and
    the shipped groups equal the oracle's, and each shipped group equals
    sdbe_process over the packets the oracle let into it.  A packet's payload
    is a function of its (b, c, f) slot, so duplicates carry the same data
    and the groups do not depend on which duplicate a frame keeps."""
    import os
    import sys

    from sdbe_gb300 import Resampler

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_hostlogic_golden as HG

    hdr, cuts = HG.scenario(case)
    w = np.ascontiguousarray(hdr).view("<u4")
    slot = (_b_of(hdr) * 2048 + (w[:, 5] & 0xFF) * 8 + ((w[:, 5] >> 16) & 7)).astype(np.int64)
    payload = ((slot[:, None] * 2654435761 + np.arange(O.IN_PKT_BYTES - 32)[None, :] * 40503) >> 7) & 0xFF
    pk = np.concatenate([hdr, payload.astype(np.uint8)], axis=1)
    st = O.IngestState()
    accepted = {}
    with Resampler(max_frames=G) as rs, Resampler(max_frames=G) as ref:
        pos = 0
        for m in cuts:
            batch = pk[pos:pos + m]
            pos += m
            acc, ships = O.ingest_policy(batch, st)
            got = batch[acc]
            gid = (_b_of(got) - st.b_first - 1) // G
            for g in np.unique(gid):
                prev = accepted.get(int(g))
                new = got[gid == g]
                accepted[int(g)] = new if prev is None else np.concatenate([prev, new])
            groups, n = rs.ingest(batch)
            mask = np.zeros(m, np.uint8)
            assert rs._lib.sdbe_test_ingest_accept(rs.handle, mask.ctypes.data, m) == 0
            bad = np.flatnonzero(mask.astype(bool) != acc)
            assert bad.size == 0, (case, pos, bad[:10])
            assert n == len(ships), (case, pos)
            for i, g in enumerate(ships):
                want, _ = ref.process(accepted.pop(g, np.zeros((0, O.IN_PKT_BYTES), np.uint8)), G, st.start(g))
                assert np.array_equal(groups[i], want), (case, g)
            _stats_equal(rs, st)
