"""Layout invariants the FP32 FFT kernels rely on, checked on the CPU.

The constant tables and index maps live in ``sdbe_gb300/csrc/k_fft.cu``;
these tests read them from the source (so they check the shipped values,
not a copy) and verify the properties the kernels assume:

* ``kFirstPassGroups``: the first pass of the 18304-point transform gives
  half-warp h the groups of 8 inputs g0 = table[2h], g1 = table[2h + 1].
  Every group 0..142 appears once (plus one empty slot, 255), and
  rho(8 g1) - rho(8 g0) = 8 (mod 16) with rho(8g) = g/11 + 13 (g % 11), so
  the 16 lanes' digit-reversed stores hit 16 distinct bank pairs.
* ``c2r_col``: the inverse's first-pass column map of stage A is a
  permutation of 0..511 whose 16 values per half-warp are distinct mod 16
  (conflict-free stores), and lanes l and l ^ 16 hold mirror columns
  b + b' = 512, except warp 0's self-mirrored columns 0 and 256.
* the 2-bit pack's 8 x 8 nibble transpose (three xor-shuffle steps over 8
  lanes) is a transpose, modelled here step by step.
"""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sdbe_gb300", "csrc", "k_fft.cu")


def _source():
    with open(SRC) as f:
        return f.read()


def _first_pass_table():
    m = re.search(r"kFirstPassGroups\[144\]\s*=\s*\{([^}]*)\}", _source())
    assert m, "kFirstPassGroups not found"
    return [int(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]


def _rho(g):
    return g // 11 + 13 * (g % 11)


def test_first_pass_table_is_a_permutation():
    t = _first_pass_table()
    assert len(t) == 144
    assert t.count(255) == 1
    assert sorted(x for x in t if x != 255) == list(range(143))


def test_first_pass_stores_are_conflict_free():
    t = _first_pass_table()
    for h in range(72):
        g0, g1 = t[2 * h], t[2 * h + 1]
        if 255 in (g0, g1):
            continue
        assert (_rho(g1) - _rho(g0)) % 16 == 8, (h, g0, g1)
        # the slots 17 rho(8g + c) + r of the 16 lanes at fixed r fall in 16
        # distinct bank pairs (float2 slot s -> bank pair s mod 16)
        for r in range(16):
            slots = {(17 * (_rho(g) + 143 * c) + r) % 16 for g in (g0, g1) for c in range(8)}
            assert len(slots) == 16, (h, r)


def _c2r_col(t):
    # the same expression as c2r_col() in k_fft.cu
    w, l = t >> 5, t & 31
    if l < 16:
        return 16 * w + l
    return 256 if (w == 0 and l == 16) else 512 - 16 * w - (l - 16)


def test_c2r_col_matches_source():
    src = _source()
    assert "if (l < 16) return 16 * w + l;" in src
    assert "return (w == 0 && l == 16) ? 256 : 512 - 16 * w - (l - 16);" in src


def test_c2r_col_properties():
    cols = [_c2r_col(t) for t in range(512)]
    assert sorted(cols) == list(range(512))
    for h in range(32):
        assert len({c % 16 for c in cols[16 * h:16 * h + 16]}) == 16, h
    for t in range(512):
        p = t ^ 16
        if t in (0, 16):
            assert {cols[t], cols[p]} == {0, 256}
        else:
            assert cols[t] + cols[p] == 512, t


def test_c2r_pairing_model_matches_direct_formula():
    """The pair-and-swap of stage A's C2R input, modelled on the CPU with
    the column map: every thread ends with Z[col + 512 r], r < 32."""
    M = 16384
    rng = np.random.default_rng(5)
    Y = rng.standard_normal(M + 1) + 1j * rng.standard_normal(M + 1)
    Y[M] = 0.0  # the Nyquist bin of stage A's packed spectra
    Yd = Y.copy()
    Yd[0] = Yd[0].real
    k = np.arange(M)
    Zref = (Yd[k] + np.conj(Yd[M - k])) + 1j * np.exp(2j * np.pi * k / 32768) * (Yd[k] - np.conj(Yd[M - k]))

    def pair(y, ym, kk):
        w = np.exp(2j * np.pi * kk / 32768)
        e = (y.real + ym.real) + 1j * (y.imag - ym.imag)
        tt = ((y.real - ym.real) + 1j * (y.imag + ym.imag)) * w
        return (e.real - tt.imag) + 1j * (e.imag + tt.real), (e.real + tt.imag) + 1j * (tt.real - e.imag)

    cols = [_c2r_col(t) for t in range(512)]
    V = np.zeros((512, 32), complex)
    for w in range(16):
        zmk = {}
        for l in range(32):
            t = 32 * w + l
            c = cols[t]
            for p in range(16):
                y, ym = Y[c + 512 * p], Y[M - c - 512 * p]
                if c == 0 and p == 0:
                    y, ym = y.real + 0j, 0j
                V[t, p], zmk[(l, p)] = pair(y, ym, c + 512 * p)
        for l in range(32):
            t = 32 * w + l
            for p in range(16):
                if w == 0 and l == 16:
                    V[t, 31 - p] = zmk[(l, p)]
                elif w == 0 and l == 0:
                    if p >= 1:
                        V[t, 32 - p] = zmk[(l, p)]
                else:
                    V[t, 31 - p] = zmk[(l ^ 16, p)]
        if w == 0:
            y = Y[8192]
            V[0, 16] = (y + np.conj(y)) + 1j * 1j * (y - np.conj(y))
    for t in range(512):
        np.testing.assert_allclose(V[t], Zref[cols[t] + 512 * np.arange(32)], rtol=0, atol=1e-9)


def test_nibble_transpose_model():
    """nib_transpose8: step m (1, 2, 4) swaps between lanes c and c ^ m the
    nibbles whose index bit m differs from the lane's bit m; the result is
    the transpose of the 8 x 8 nibble matrix."""
    with open(os.path.join(os.path.dirname(SRC), "fft_core.cuh")) as f:
        src = f.read()
    assert "kKeep[3] = {0x0F0F0F0Fu, 0x00FF00FFu, 0x0000FFFFu}" in src
    keep = [0x0F0F0F0F, 0x00FF00FF, 0x0000FFFF]
    rng = np.random.default_rng(9)
    for _ in range(50):
        n = rng.integers(0, 16, size=(8, 8))
        x = [int(sum(int(n[c, r]) << (4 * r) for r in range(8))) for c in range(8)]
        for s in range(3):
            m, sh = 1 << s, 4 << s
            y = [x[c ^ m] for c in range(8)]
            x = [((x[c] & ~keep[s]) | ((y[c] >> sh) & keep[s])) & 0xFFFFFFFF if c & m
                 else ((x[c] & keep[s]) | ((y[c] << sh) & ~keep[s])) & 0xFFFFFFFF for c in range(8)]
        for c in range(8):
            assert x[c] == sum(int(n[r, c]) << (4 * r) for r in range(8))
