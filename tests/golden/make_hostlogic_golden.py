"""Golden vectors for the host-side group assembly and output headers, made
by the reference's own C code.

Builds ``oracle/_ref/ref_hostlogic`` from ``software/aphids/vdif_in_databuf.c``,
``vdif_out_databuf.c`` and ``beng_reform.c`` (``oracle/Makefile``) and stores
in ``hostlogic.npz``:

* ``tmpl_*``: ``fill_vdif_header_template`` for seeded and edge T0 values
  (clk 0, one frame before the second boundary, the boundary itself, ...):
  secs_inre, df_num_insec and the picoseconds hidden in edh_psn.
* ``outhdr``: the eight header words ``init_vdif_out`` writes (channels 0
  and 1, first and last packet of a block).
* ``<case>_outcome`` / ``<case>_ships`` (cases sparse, overflow, boundary,
  far, complete): per packet the absolute group it
  was inserted into (or -1 invalid, -2 before the start, -3 too far ahead,
  -4 not inserted) and the shipped groups with their packet counts, from the
  reference's ``get_beng_group_index_offset`` / ``insert_vdif_in_beng_group_buffer``
  / ``check_beng_group_complete`` run by the ingest loop of
  ``vdif_in_net_thread.c:340-500``.  The packets themselves are not stored:
  ``scenario(name)`` below regenerates them from a seed (the tests import it).

Run where the reference checkout exists (``make -C oracle`` builds the driver
from it; ``SDBE_REFERENCE`` names the checkout); the fixture is committed.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BIN = os.path.join(ROOT, "oracle", "_ref", "ref_hostlogic")
OUT = os.path.join(HERE, "hostlogic.npz")

GF = 143                     # B-frames per group
GP = GF * 2048               # packets per complete group
CASES = ("sparse", "overflow", "boundary", "far", "complete")


def headers(b, c, f, invalid, rng):
    """32-byte input headers (vdif_in_header_t) for packets (b, c, f, invalid)."""
    n = len(b)
    b = np.asarray(b, np.int64)
    w = np.zeros((n, 8), np.uint32)
    w[:, 0] = rng.integers(0, 2**30, n).astype(np.uint32) | (np.asarray(invalid, np.uint32) << 31)
    w[:, 1] = rng.integers(0, 2**24, n).astype(np.uint32)
    w[:, 2] = 132
    w[:, 4] = (b >> 8).astype(np.uint32)
    w[:, 5] = (np.asarray(c, np.int64) | (np.asarray(f, np.int64) << 16) | ((b & 0xFF) << 24)).astype(np.uint32)
    return w.view(np.uint8).reshape(n, 32)


def _cut(n, rng, lo, hi):
    out, left = [], n
    while left > 0:
        m = int(min(left, rng.integers(lo, hi)))
        out.append(m)
        left -= m
    return out


def scenario(name):
    """(headers uint8 [n, 32], batch sizes) of a seeded ingest case."""
    b0 = 1_000_000
    if name == "sparse":  # jittered, mostly increasing b over 9 groups; invalid, early and late packets
        rng = np.random.default_rng(71)
        n = 5000
        b = b0 + np.sort(rng.integers(-30, 9 * GF, n) + rng.integers(-200, 200, n))
        b[:3] = b0  # the first batch starts the stream at b0
        b[rng.random(n) < 0.01] += 12 * GF  # a few far ahead
        inv = rng.random(n) < 0.04
        inv[:3] = False
        c, f = rng.integers(0, 256, n), rng.integers(0, 8, n)
        return headers(b, c, f, inv, rng), _cut(n, rng, 40, 600)
    if name == "overflow":  # more than 2048 packets for some frames
        rng = np.random.default_rng(72)
        b = np.concatenate([[b0], np.full(2100, b0 + 3), np.full(2060, b0 + 150), b0 + 1 + rng.integers(0, 4 * GF, 800)])
        n = b.size
        c, f = rng.integers(0, 256, n), rng.integers(0, 8, n)
        return headers(b, c, f, np.zeros(n, bool), rng), _cut(n, rng, 500, 3000)
    if name == "boundary":  # b at the too-far-ahead and look-ahead limits, in one batch and across ships
        rng = np.random.default_rng(73)
        s = b0 + 1
        edge = [s - 1, s, s + 3 * GF - 1, s + 3 * GF, s + 4 * GF - 1, s + 4 * GF, s + 5 * GF - 1 + 4 * GF,
                s + 5 * GF + 4 * GF, s + 4 * GF - 1 + 4 * GF, s + 4 * GF + 4 * GF, s + 9 * GF]
        b = np.concatenate([[b0], np.repeat(edge, 3), s + rng.integers(0, 6 * GF, 300), np.repeat(edge, 2) + 2 * GF])
        n = b.size
        c, f = rng.integers(0, 256, n), rng.integers(0, 8, n)
        return headers(b, c, f, np.zeros(n, bool), rng), [1 + 3 * len(edge), 300, n - 1 - 3 * len(edge) - 300]
    if name == "far":  # lone packets just inside and just past the too-far-ahead limit of a fresh ring
        rng = np.random.default_rng(75)
        s = b0 + 1
        lim = s + 5 * GF - 1 + 4 * GF  # last b that is not too far ahead while the ring starts at s
        b = np.array([b0, lim, lim + 1, lim + 1 + 8 * GF, lim + 2 + 8 * GF, s + 2])
        n = b.size
        c, f = rng.integers(0, 256, n), rng.integers(0, 8, n)
        return headers(b, c, f, np.zeros(n, bool), rng), [1, 1, 1, 1, 1, 1]
    if name == "complete":  # one complete group (every c, f of every frame), then 1% dropped of the next
        rng = np.random.default_rng(74)
        fr = np.repeat(np.arange(GF), 2048)
        cf = np.tile(np.arange(2048), GF)
        keep = rng.random(GF * 2048) >= 0.01
        b = np.concatenate([[b0], b0 + 1 + fr, b0 + 1 + GF + fr[keep]])
        c = np.concatenate([[0], cf >> 3, (cf >> 3)[keep]])
        f = np.concatenate([[0], cf & 7, (cf & 7)[keep]])
        n = b.size
        perm = np.concatenate([[0], 1 + rng.permutation(n - 1)])  # shuffled after the first packet
        order = np.argsort(b[perm] // 300 * 10**7 + rng.integers(0, 10**7, n), kind="stable")  # loosely by b
        idx = perm[order]
        idx = np.concatenate([[0], idx[idx != 0]])
        return headers(b[idx], c[idx], f[idx], np.zeros(n, bool), rng), _cut(n, rng, 20000, 60000)
    raise ValueError(name)


def run_ingest(name):
    hdr, batches = scenario(name)
    with tempfile.TemporaryDirectory() as d:
        hp, op = os.path.join(d, "h.bin"), os.path.join(d, "o.bin")
        hdr.tofile(hp)
        subprocess.run([BIN, "ingest", hp, op] + [str(m) for m in batches], check=True, stdout=subprocess.DEVNULL)
        raw = np.fromfile(op, dtype="<i8")
    n = int(raw[0])
    outcome = raw[1:1 + n]
    ns = int(raw[1 + n])
    ships = raw[2 + n:2 + n + 2 * ns].reshape(ns, 2)
    assert outcome.size == hdr.shape[0]
    return outcome.astype(np.int32), ships.astype(np.int64)


def run_template(sec, clk, nskip):
    out = subprocess.run([BIN, "template", str(sec), str(clk), str(nskip)], check=True, capture_output=True, text=True)
    line = [x for x in out.stdout.splitlines() if x.startswith("RESULT ")][-1]
    return [int(v) for v in line.split()[1:]]


def main():
    if not os.path.exists(BIN):
        sys.exit(f"{BIN} missing: build it with `make -C oracle` where the reference checkout exists")
    rng = np.random.default_rng(70)
    C, F = 286000000, 262144
    clks = [0, 1, F - 1, F, C - F - 1, C - F, C - F + 1, C - 2, C - 1, 143000000] + list(rng.integers(0, C, 22))
    secs = list(rng.integers(0, 2**30 - 10, len(clks)))
    nskip = list(rng.integers(0, 2048, len(clks)))
    res = np.array([run_template(s, c, k) for s, c, k in zip(secs, clks, nskip)], np.int64)
    out = subprocess.run([BIN, "outhdr"], check=True, capture_output=True, text=True).stdout
    words = np.array([[int(x, 16) for x in ln.split()[3:]] for ln in out.splitlines() if ln.startswith("WORDS ")],
                     np.uint32)
    fx = dict(tmpl_sec=np.array(secs, np.int64), tmpl_clk=np.array(clks, np.int64), tmpl_nskip=np.array(nskip, np.int64),
              tmpl_result=res, outhdr=words)
    for name in CASES:
        o, s = run_ingest(name)
        fx[f"{name}_outcome"] = o
        fx[f"{name}_ships"] = s
        print(name, "packets", o.size, "accepted", int((o >= 0).sum()), "ships", s.tolist()[:8])
    np.savez_compressed(OUT, **fx)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
