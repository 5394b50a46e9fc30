"""The oracle's restated host logic against the reference's own C code
(``tests/golden/hostlogic.npz``, made by ``tests/golden/make_hostlogic_golden.py``
with ``oracle/_ref/ref_hostlogic`` built from ``software/aphids/vdif_in_databuf.c``,
``vdif_out_databuf.c`` and ``beng_reform.c``).

* group assembly: per packet, whether it is inserted and into which group
  (``get_beng_group_index_offset`` / ``insert_vdif_in_beng_group_buffer`` /
  ``check_beng_group_complete`` under the ingest loop), and the shipped
  groups with their packet counts, for four seeded streams;
* the output timestamp template (``fill_vdif_header_template``);
* the output header fields ``init_vdif_out`` sets once.
"""
import os
import sys

import numpy as np
import pytest

from oracle import sdbe_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_hostlogic_golden as G  # noqa: E402

FX = np.load(os.path.join(HERE, "golden", "hostlogic.npz"))


@pytest.mark.parametrize("case", G.CASES)
def test_ingest_policy_matches_reference(case):
    hdr, batches = G.scenario(case)
    want = FX[f"{case}_outcome"]
    st = O.IngestState()
    got_accept = []
    pos = 0
    for m in batches:
        acc, _ = O.ingest_policy(hdr[pos:pos + m], st)
        got_accept.append(acc)
        pos += m
    acc = np.concatenate(got_accept)
    w = np.ascontiguousarray(hdr[:, :24]).view("<u4")
    b = ((w[:, 4].astype(np.int64) << 8) | (w[:, 5].astype(np.int64) >> 24))
    group = np.where(acc, (b - st.b_first - 1) // O.BENG_FRAMES_PER_GROUP, -1)
    ref_group = np.where(want >= 0, want, -1)
    bad = np.flatnonzero(group != ref_group)
    assert bad.size == 0, (case, bad[:10], group[bad[:10]], want[bad[:10]], b[bad[:10]] - st.b_first)
    np.testing.assert_array_equal(np.array(st.shipped, np.int64).reshape(-1, 2), FX[f"{case}_ships"])


def test_header_template_matches_reference():
    for sec, clk, res in zip(FX["tmpl_sec"], FX["tmpl_clk"], FX["tmpl_result"]):
        s, df, ps, _ = O.header_template(int(sec), int(clk))
        assert (s & 0x3FFFFFFF, df & 0xFFFFFF, ps) == tuple(int(v) for v in res), (sec, clk, res)


def test_output_header_constants_match_reference():
    # fields init_vdif_out sets once and the output thread leaves alone
    keep = np.array([0xC0000000, 0xC0000000, 0xFFFFFFFF, 0x80000000, 0xFFFFFFF8, 0xFFFFFFFF, 0, 0], np.uint32)
    ref = FX["outhdr"]
    for pol in (0, 1):
        w = O.vdif_out_header_words(3, pol, secs=123, df=45, psn=6)
        for row in ref:
            np.testing.assert_array_equal(w[0] & keep, row & keep)
        # the station the output thread writes is init_vdif_out's 'Sm'
        assert (w[0, 3] & 0xFFFF) == (ref[0, 3] & 0xFFFF)
