"""Seeded synthetic SWARM B-engine VDIF streams (wraps ``libsdbe_synth.so``).

Recorded SDBE scans are not available, so every workload is generated:
per channel and snapshot a complex Gaussian sample (sigma per component) plus
optional CW tones and broadband bursts, quantized to 2-bit offset-binary codes
at the fixed levels {-0.98, 0, +0.98}, packed into 1056-B packets in the
APHIDS 11/11 layout.  Seeds are ``1000 + stream`` by convention.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as N


@dataclass
class StreamSpec:
    """One packet stream (carries two phased sums, p0 and p1)."""
    n_frames: int
    seed: int = 1000
    sigma: float = 1.0
    level: float = 0.98
    tones: list = field(default_factory=list)   # [(channel, amplitude, phase)]
    burst_frac: float = 0.0
    burst_gain: float = 4.0
    drop_frac: float = 0.0
    reorder_frac: float = 0.0
    reorder_max: int = 64
    b_start: int = 1_000_000
    channel_map: int = N.MAP_APHIDS


def tone_10db(channel=5000, sigma=1.0):
    """CW tone at 10 dB SNR per channel: |A|^2 = 10 * (2 sigma^2)."""
    return (channel, math.sqrt(20.0) * sigma, 0.3)


def seeded_tones(seed, n=3, lo=0.1, hi=0.5, sigma=1.0):
    rng = np.random.default_rng(seed + 77)
    ch = rng.choice(np.arange(64, 16320), size=n, replace=False)
    amp = rng.uniform(lo, hi, size=n) * sigma
    ph = rng.uniform(0, 2 * np.pi, size=n)
    return [(int(c), float(a), float(p)) for c, a, p in zip(ch, amp, ph)]


def config1(stream=0):
    """1 stream x 8 B-frames, sigma 1, one CW tone at channel 5000 (10 dB)."""
    return StreamSpec(n_frames=8, seed=1000 + stream, tones=[tone_10db()])


def config2(stream=0, n_frames=512):
    """1 stream x 512 B-frames, 3 tones at seeded channels, 0.1-0.5 sigma."""
    return StreamSpec(n_frames=n_frames, seed=1000 + stream, tones=seeded_tones(1000 + stream))


def config4(n_packet_streams=4):
    """Uneven streams: lengths U{64..512} B-frames, per-stream sigma U[0.5, 2]."""
    rng = np.random.default_rng(4000)
    out = []
    for s in range(n_packet_streams):
        sig = float(rng.uniform(0.5, 2.0))
        out.append(StreamSpec(n_frames=int(rng.integers(64, 513)), seed=1000 + s, sigma=sig,
                              tones=seeded_tones(1000 + s, sigma=sig), b_start=1_000_000 + 10_000 * s))
    return out


def config5(n_packet_streams=16, n_frames=2048):
    """Stress: drops 1%, displaced 0.5% (<= 64 places), bursts sigma x4 on 1% of snapshots."""
    return [StreamSpec(n_frames=n_frames, seed=1000 + s, tones=seeded_tones(1000 + s), burst_frac=0.01,
                       burst_gain=4.0, drop_frac=0.01, reorder_frac=0.005, reorder_max=64,
                       b_start=2_000_000 + 100_000 * s) for s in range(n_packet_streams)]


def _cfg(spec: StreamSpec) -> N.SynthConfig:
    c = N.SynthConfig()
    c.sigma = spec.sigma
    c.level = spec.level
    if len(spec.tones) > 8:
        raise ValueError("at most 8 tones")
    c.n_tones = len(spec.tones)
    for i, (ch, a, p) in enumerate(spec.tones):
        c.tone_channel[i] = int(ch)
        c.tone_amp[i] = float(a)
        c.tone_phase[i] = float(p)
    c.burst_frac = spec.burst_frac
    c.burst_gain = spec.burst_gain
    c.channel_map = spec.channel_map
    c.secs0 = 12345
    c.ref_epoch = 30
    c.station = (ord("S") << 8) | ord("m")
    return c


def generate(spec: StreamSpec, out: np.ndarray | None = None, n_threads: int = 0,
             frame_offset: int = 0, n_frames: int | None = None) -> np.ndarray:
    """Packets of ``spec`` (or of frames [frame_offset, frame_offset+n_frames)).

    Returns uint8 ``[n_packets, 1056]``; impairments (drops, displacement)
    applied when the spec asks for them.
    """
    nf = spec.n_frames if n_frames is None else n_frames
    n = nf * N.PKTS_PER_FRAME
    lib = N.synth_lib()
    cfg = _cfg(spec)
    impaired = spec.drop_frac > 0 or spec.reorder_frac > 0
    raw = np.empty((n, N.IN_PKT_BYTES), np.uint8) if (out is None or impaired) else out
    got = lib.sdbe_synth_packets(raw.ctypes.data, nf, spec.b_start + frame_offset, spec.seed, C.byref(cfg),
                                 n_threads)
    if got != n:
        raise RuntimeError("synthetic generator failed")
    if not impaired:
        return raw
    dst = np.empty_like(raw) if out is None else out
    m = lib.sdbe_synth_impair(raw.ctypes.data, n, dst.ctypes.data, spec.seed + frame_offset,
                              spec.drop_frac, spec.reorder_frac, spec.reorder_max)
    return dst[:m]


# -- 8pac input format ------------------------------------------------------
PAC8_BYTES = 1056 + 7 * (8 + 1056)   # one 8pac unit: packet, then 7 x (8-B VTP + packet)
CLK_PER_SEC = 286000000              # SWARM FPGA clock
BFRAME_CLK = 262144                  # clocks per B-frame


def new_format_words(c, f, sec, clk):
    """(w4, w5) of the new-format B-engine header: a 53-bit timestamp
    (sec << 29 | clk) split as b_upper (w4) and b_lower (w5 bits 11-31), with
    c in w5 bits 0-7 and f in bits 8-10."""
    ts = (np.asarray(sec, np.int64) << 29) | np.asarray(clk, np.int64)
    w4 = (ts >> 21).astype(np.uint32)
    w5 = (np.asarray(c, np.int64) | (np.asarray(f, np.int64) << 8) | ((ts & 0x1FFFFF) << 11)).astype(np.uint32)
    return w4, w5


def to_8pac(packets, t0_sec: int, t0_clk: int, b_ref: int, seed: int = 0, psn0: int = 0, df0: int = 0):
    """Packets with old-format headers (b in w4/w5) -> 8pac units whose
    headers carry the timestamp of frame b (t0 + (b - b_ref) B-frames) in the
    new format.  The first packet of each unit has df_len = 8504/8, the
    unit's data-frame number and psn; the other 7 and the VTP prefixes carry
    seeded garbage in the fields the unpack rewrites.  ``len(packets)`` must
    be a multiple of 8."""
    p = np.ascontiguousarray(packets, dtype=np.uint8).reshape(-1, 1056)
    n = p.shape[0]
    if n % 8:
        raise ValueError("packet count must be a multiple of 8")
    rng = np.random.default_rng(seed)
    w = p.view("<u4").reshape(n, 264).copy()
    c = w[:, 5] & 0xFF
    f = (w[:, 5] >> 16) & 0xFF
    b = ((w[:, 4].astype(np.int64) << 8) | (w[:, 5].astype(np.int64) >> 24))
    t = t0_sec * np.int64(CLK_PER_SEC) + t0_clk + (b - b_ref) * BFRAME_CLK
    w[:, 4], w[:, 5] = new_format_words(c, f & 7, t // CLK_PER_SEC, t % CLK_PER_SEC)
    units = n // 8
    w = w.reshape(units, 8, 264)
    garbage = rng.integers(0, 2**32, (units, 8, 4), dtype=np.uint64).astype(np.uint32)
    w[:, 1:, 1] = (w[:, 1:, 1] & np.uint32(0xFF000000)) | (garbage[:, 1:, 0] & np.uint32(0xFFFFFF))
    w[:, 1:, 2] = (w[:, 1:, 2] & np.uint32(0xFF000000)) | (garbage[:, 1:, 1] & np.uint32(0xFFFFFF))
    w[:, 1:, 6] = garbage[:, 1:, 2]
    w[:, 1:, 7] = garbage[:, 1:, 3]
    w[:, 1:, 0] ^= (garbage[:, 1:, 0] & np.uint32(1 << 31))
    k = np.arange(units, dtype=np.int64)
    w[:, 0, 1] = (w[:, 0, 1] & np.uint32(0xFF000000)) | ((df0 + k) & 0xFFFFFF).astype(np.uint32)
    w[:, 0, 2] = (w[:, 0, 2] & np.uint32(0xFF000000)) | np.uint32(PAC8_BYTES // 8)
    psn = (psn0 + k).astype(np.uint64)
    w[:, 0, 6] = (psn & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    w[:, 0, 7] = (psn >> np.uint64(32)).astype(np.uint32)
    out = np.empty((units, PAC8_BYTES), np.uint8)
    pk = w.view(np.uint8).reshape(units, 8, 1056)
    out[:, :1056] = pk[:, 0]
    vtp = rng.integers(0, 256, (units, 7, 8), dtype=np.uint8)
    for j in range(7):
        o = 1056 + j * 1064
        out[:, o:o + 8] = vtp[:, j]
        out[:, o + 8:o + 1064] = pk[:, j + 1]
    return out
