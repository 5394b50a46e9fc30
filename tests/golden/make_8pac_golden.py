"""Golden vectors for the ingest transforms, made by the reference's own C code.

Builds ``oracle/_ref/ref_8pac`` from ``software/aphids/vdif_8pac.c`` and
``software/aphids/beng_reform.c`` (``oracle/Makefile``), feeds it seeded 8pac
streams cut into receive batches, and stores inputs, batch cuts, the unpacked
and reformed packets and the final reform state (T0 as ``get_beng_t0``
returns it, TPREV, BPREV) in ``pac8_reform.npz``.  Run where the reference
checkout exists, with ``SDBE_REFERENCE`` set to it; the fixture is committed.

Cases: ``regular`` (on-grid timestamps across a second boundary, random
payloads in the first units), ``jitter`` (off-grid by up to 1500 clocks),
``jumps`` (steps of 1000/1001/1200 frames and backwards, invalid first
packets), ``corrupt`` (clk at and above 286e6, seconds two apart, values at
the 1024-clock tolerance), ``random`` (random timestamps and flags).  Every
case also carries odd df_len / df_num / psn values in the first packet of its
units.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

REF = os.environ.get("SDBE_REFERENCE", "")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BIN = os.path.join(ROOT, "oracle", "_ref", "ref_8pac")

C, F = 286000000, 262144
PAC8 = 1056 + 7 * 1064


def units(sec, clk, c, f, inv1, rng, n_random_payload=0):
    """8pac units whose packet i carries timestamp (sec[i], clk[i]), c[i],
    f[i]; inv1[u] is the invalid flag of unit u's first packet."""
    n = len(sec)
    assert n % 8 == 0
    w = np.zeros((n, 264), np.uint32)
    w[:, 0] = rng.integers(0, 2**30, n).astype(np.uint32) | (rng.integers(0, 2, n).astype(np.uint32) << 30)
    w[:, 0] |= rng.integers(0, 2, n).astype(np.uint32) << 31          # garbage flags on packets 2..8
    w[:, 1] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    w[:, 2] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    w[:, 3] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    ts = (np.asarray(sec, np.int64) << 29) | np.asarray(clk, np.int64)
    w[:, 4] = (ts >> 21).astype(np.uint32)
    w[:, 5] = (np.asarray(c, np.int64) | (np.asarray(f, np.int64) << 8) | ((ts & 0x1FFFFF) << 11)).astype(np.uint32)
    w[:, 6] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    w[:, 7] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    u = n // 8
    w = w.reshape(u, 8, 264)
    w[:, 0, 0] = (w[:, 0, 0] & np.uint32(0x7FFFFFFF)) | (np.asarray(inv1, np.uint32) << 31)
    dfl = np.full(u, PAC8 // 8, np.int64)
    dfl[rng.random(u) < 0.1] = rng.integers(0, 7, 1)[0]          # below 7: negative before the divide
    dfl[rng.random(u) < 0.05] = 0xFFFFFF
    w[:, 0, 2] = (w[:, 0, 2] & np.uint32(0xFF000000)) | dfl.astype(np.uint32)
    if n_random_payload:
        k = min(n_random_payload, u)
        w[:k, :, 8:] = rng.integers(0, 2**32, (k, 8, 256), dtype=np.uint64).astype(np.uint32)
    pk = w.view(np.uint8).reshape(u, 8, 1056)
    out = np.empty((u, PAC8), np.uint8)
    out[:, :1056] = pk[:, 0]
    vtp = rng.integers(0, 256, (u, 7, 8), dtype=np.uint8)
    for j in range(7):
        o = 1056 + j * 1064
        out[:, o:o + 8] = vtp[:, j]
        out[:, o + 8:o + 1064] = pk[:, j + 1]
    return out


def grid(n, t0_sec, t0_clk, per_frame, start_frame=0):
    k = start_frame + np.arange(n) // per_frame
    t = t0_sec * C + t0_clk + k * F
    return t // C, t % C


def cases():
    rng = np.random.default_rng(8504)
    out = {}
    # regular: 96 units, a new frame every 64 packets, crossing a second
    n = 96 * 8
    s, k = grid(n, 4000, C - 5 * F + 100, 64)
    cf = np.arange(n) % 2048
    out["regular"] = (units(s, k, cf // 8, cf % 8, np.zeros(96, int), rng, 16), [10, 30, 56])
    # jitter
    n = 96 * 8
    s, k = grid(n, 77, 1000, 48)
    t = s * C + k
    j = rng.random(n) < 0.1
    t[j] += rng.integers(-1500, 1501, int(j.sum()))
    t[0] += 700
    out["jitter"] = (units(t // C, t % C, cf[:n] // 8, cf[:n] % 8, np.zeros(96, int), rng), [48, 48])
    # jumps
    n = 48 * 8
    s, k = grid(n, 9, 5000, 32)
    t = s * C + k
    t[100:104] += 1200 * F
    t[150:152] += 1000 * F
    t[152:154] += 1001 * F
    t[200:230] -= 3 * F
    t[300:] += 999 * F
    inv1 = np.zeros(48, int)
    inv1[[0, 5, 6, 40]] = 1
    out["jumps"] = (units(t // C, t % C, cf[:n] // 8, cf[:n] % 8, inv1, rng), [1, 7, 40])
    # corrupt / tolerance edges
    n = 64 * 8
    choices_clk = np.array([C - 1024, C - 1023, C - 1025, C, C + 5, 2**29 - 1, 0, 1023, 1024, 1025, F, C - F])
    s = 500 + rng.integers(0, 3, n)
    k = choices_clk[rng.integers(0, choices_clk.size, n)]
    out["corrupt"] = (units(s, k, rng.integers(0, 256, n), rng.integers(0, 8, n),
                            (rng.random(64) < 0.1).astype(int), rng), [64])
    # random
    n = 32 * 8
    s = 1234 + rng.integers(0, 2, n)
    k = rng.integers(0, 2**29, n)
    out["random"] = (units(s, k, rng.integers(0, 256, n), rng.integers(0, 8, n),
                           (rng.random(32) < 0.2).astype(int), rng), [5, 11, 16])
    return out


def run_reference(src: np.ndarray, batches):
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        src.tofile(fi)
        r = subprocess.run([BIN, fi, fo] + [str(b) for b in batches], capture_output=True, text=True, check=True)
        out = np.fromfile(fo, np.uint8).reshape(-1, 1056)
    t0s, t0c, tps, tpc, bp, size = (int(v) for v in r.stdout.split())
    assert size == PAC8
    return out, np.array([t0s, t0c, tps, tpc, bp], np.int64)


def main():
    if not REF:
        sys.exit("set SDBE_REFERENCE to the Smithsonian/sdbe checkout")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), f"REF={os.path.join(REF, 'software', 'aphids')}"],
                   check=True)
    arrays = {}
    for name, (src, batches) in cases().items():
        assert sum(batches) == src.shape[0]
        out, state = run_reference(src, batches)
        arrays[f"{name}_in"] = src
        arrays[f"{name}_batches"] = np.array(batches, np.int64)
        arrays[f"{name}_out"] = out
        arrays[f"{name}_state"] = state
        print(name, src.shape, out.shape, state.tolist(), file=sys.stderr)
    np.savez_compressed(os.path.join(HERE, "pac8_reform.npz"), **arrays)


if __name__ == "__main__":
    main()
