"""The oracle's 8pac unpack and header reform against the reference's own C
code: the committed fixture (tests/golden/make_8pac_golden.py) and, where the
reference binary was built here, fresh seeded streams."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import sdbe_oracle as O

GOLDEN = os.path.join(ROOT, "tests", "golden", "pac8_reform.npz")
CASES = ["regular", "jitter", "jumps", "corrupt", "random"]


def run_oracle(src, batches):
    st = O.ReformState()
    outs, lo = [], 0
    for n in batches:
        pk = O.unpack_8pac(src[lo:lo + n])
        outs.append(O.beng_reform_headers(pk, st))
        lo += n
    t0 = O.reform_t0(st)
    return np.concatenate(outs), [t0[0], t0[1], st.tprev[0], st.tprev[1], st.bprev]


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_fixture(case):
    g = np.load(GOLDEN)
    out, state = run_oracle(g[f"{case}_in"], g[f"{case}_batches"].tolist())
    ref = g[f"{case}_out"]
    assert out.shape == ref.shape
    bad = np.nonzero((out != ref).any(axis=1))[0]
    assert bad.size == 0, (case, bad[:5])
    assert state == g[f"{case}_state"].tolist()


def test_fixture_exercises_every_branch():
    g = np.load(GOLDEN)
    jumps = O.decode_beng_headers(g["jumps_out"])
    assert jumps[0].sum() > 0                                   # marked invalid by the reform
    w = g["jumps_out"].view("<u4").reshape(-1, 264)
    assert ((w[:, 0] >> 31) == 0).any() and (w[:, 4] == 0x7FFFFF).any()   # count -1 written
    reg = O.decode_beng_headers(g["regular_out"])
    assert reg[3].max() > 4                                     # crossed the second boundary


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "ref_8pac")),
                    reason="reference binary not built here")
def test_oracle_matches_reference_binary_on_fresh_streams(tmp_path):
    import sys

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_8pac_golden as M

    rng = np.random.default_rng(77)
    for trial in range(4):
        n = 40 * 8
        sec = 100 + rng.integers(0, 2, n)
        t = sec * M.C + rng.integers(0, M.C, n)
        t = np.sort(t) if trial % 2 == 0 else t
        src = M.units(t // M.C, t % M.C, rng.integers(0, 256, n), rng.integers(0, 8, n),
                      (rng.random(40) < 0.1).astype(int), rng)
        cuts = [13, 27]
        ref, state = M.run_reference(src, cuts)
        out, st = run_oracle(src, cuts)
        assert np.array_equal(out, ref), trial
        assert st == state.tolist(), trial
