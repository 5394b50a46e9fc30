"""CPU checks of the ingest policy restated in the oracle (group windowing,
look-ahead shipping, limits), on header rows built here."""
import numpy as np

from oracle import sdbe_oracle as O

G = O.BENG_FRAMES_PER_GROUP


def headers(b, c=None, f=None, invalid=None):
    """[n, 24] header rows for B-counters b (c, f default to packet order)."""
    b = np.asarray(b, np.int64)
    n = b.size
    c = np.arange(n) % 256 if c is None else np.asarray(c)
    f = (np.arange(n) // 256) % 8 if f is None else np.asarray(f)
    w = np.zeros((n, 6), "<u4")
    w[:, 0] = (np.zeros(n, np.int64) if invalid is None else np.asarray(invalid)).astype(np.uint32) << 31
    w[:, 4] = (b >> 8).astype(np.uint32)
    w[:, 5] = (((b & 0xFF) << 24) | (f << 16) | c).astype(np.uint32)
    return w.view(np.uint8).reshape(n, 24)


def frame_rows(b):
    """All 2048 packets of B-frame b, in (c, f) order."""
    i = np.arange(O.VDIF_PER_BENG)
    return headers(np.full(i.size, b), c=i // 8, f=i % 8)


def test_complete_groups_ship_as_they_complete():
    b0 = 5000
    rows = np.concatenate([frame_rows(b0 + k) for k in range(1 + 2 * G)])
    st = O.IngestState()
    shipped_at = []
    for lo in range(0, rows.shape[0], 7000):
        acc, ships = O.ingest_policy(rows[lo:lo + 7000], st)
        shipped_at += [(g, lo) for g in ships]
    assert st.b_first == b0
    assert [g for g, _ in shipped_at] == [0, 1]
    # each group ships in the batch holding its last packet
    for g, lo in shipped_at:
        last = (1 + (g + 1) * G) * 2048 - 1
        assert lo <= last < lo + 7000
    s = st.stats
    assert s["before_start"] == 2048 and s["used"] == 2 * G * 2048
    assert s["groups_shipped"] == 2 and s["groups_incomplete"] == 0 and s["overflow"] == 0


def test_look_ahead_ships_oldest_incomplete_and_retries():
    b0 = 100
    st = O.IngestState()
    acc, ships = O.ingest_policy(headers([b0, b0 + 1, b0 + 2]), st)
    assert ships == [] and acc.tolist() == [False, True, True]
    start = st.start
    # a packet 3 groups ahead: group 0 ships incomplete, the packet joins group 3
    acc, ships = O.ingest_policy(headers([start(3) + 5]), st)
    assert ships == [0] and acc.tolist() == [True] and st.ref == 1
    # 5 groups ahead of ref=1: groups 1, 2 (empty) and 3 ship until it is 2 ahead
    acc, ships = O.ingest_policy(headers([start(6)]), st)
    assert ships == [1, 2, 3] and acc.tolist() == [True] and st.ref == 4
    # late packet, packet too far ahead, invalid packet
    far = start(st.ref + 5) - 1 + 4 * G + 1  # past the group after the four searched, by 4 groups
    acc, ships = O.ingest_policy(headers([start(0) + 3, far, start(3)], invalid=[0, 0, 1]), st)
    assert ships == [] and not acc.any()
    s = st.stats
    assert (s["before_start"], s["too_far_ahead"], s["invalid"]) == (2, 1, 1)
    assert s["groups_shipped"] == 4 and s["groups_incomplete"] == 4
    # flush ships the groups up to the newest holding packets
    _, ships = O.ingest_policy(headers([]), st, flush=True)
    assert ships == [4, 5, 6] and not st.count


def test_frame_and_group_limits():
    b0 = 7
    st = O.IngestState()
    rows = np.concatenate([frame_rows(b0), frame_rows(b0 + 1), frame_rows(b0 + 1)[:5]])
    acc, ships = O.ingest_policy(rows, st)
    assert acc[:2048].sum() == 0 and acc[2048:4096].all() and not acc[4096:].any()
    assert st.stats["overflow"] == 5 and st.stats["used"] == 2048 + 5


def test_invalid_first_and_sort_within_batch():
    """The first valid b of a batch (after sorting) fixes the groups; invalid
    packets sort first and never start the stream."""
    st = O.IngestState()
    acc, ships = O.ingest_policy(headers([50, 40, 45], invalid=[0, 1, 0]), st)
    assert st.b_first == 45 and acc.tolist() == [True, False, False]
    st2 = O.IngestState()
    acc, _ = O.ingest_policy(headers([9], invalid=[1]), st2)
    assert st2.b_first == -1 and st2.stats["invalid"] == 1


def test_counts_add_up_on_a_random_stream():
    rng = np.random.default_rng(3)
    b = 1000 + np.cumsum(rng.integers(0, 3, 20000))      # slowly advancing b
    stray = rng.random(b.size) < 0.01
    b[stray] += rng.integers(-800, 3000, int(stray.sum()))   # strays both ways
    inval = (rng.random(b.size) < 0.005).astype(np.int64)
    st = O.IngestState()
    rows = headers(b, invalid=inval)
    n_acc = 0
    for lo in range(0, b.size, 1500):
        acc, _ = O.ingest_policy(rows[lo:lo + 1500], st)
        n_acc += int(acc.sum())
    s = st.stats
    assert s["packets"] == s["invalid"] + s["before_start"] + s["too_far_ahead"] + s["used"]
    assert n_acc == s["used"] - s["overflow"]
    assert s["groups_shipped"] == st.ref and s["before_start"] > 0 and s["too_far_ahead"] > 0
