"""CPU oracle for the APHIDS GPU stage (SWARM B-engine VDIF -> R2DBE 2-bit VDIF).

TEST INFRASTRUCTURE ONLY.  This module is the oracle: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import it.  The product path (``sdbe_gb300``) never calls it.

It restates, in numpy, the algorithm of the reference's GPU stage
``software/aphids/vdif_inout_gpu_thread.cu`` (Smithsonian/sdbe) for the
SWARM 11/11 rate build, with every function citing the reference lines it
follows.  FFT arithmetic in the reference is cuFFT (closed); here it is
numpy/pocketfft in FP64 (``precision="f64"``, the oracle of record) or
scipy.fft in FP32 (``precision="f32"``, the timed CPU path).  Scaling follows
cuFFT's unnormalised convention so that intermediate values equal the
reference's device buffers.

Pinned against reference code run in this container on seeded inputs: see
``tests/golden/make_golden.py`` (bit layout of ``swarm.DBEFrame.from_bin``,
``sdbe_preprocess.quantize_to_2bit`` + ``vdif.VDIFFrame.to_bin`` packing and
header words, the Mar-2015 reorder check of ``prototyping/cuda/reorder.py`` and
the cuFFT scale convention of the FFT-resample check in
``prototyping/cuda/resample.py``).  The 8pac unpack and header reform are
pinned against the reference's own C (``software/aphids/vdif_8pac.c``,
``beng_reform.c``) compiled by ``oracle/Makefile``: see
``tests/golden/make_8pac_golden.py``.  The ingest policy
(``ingest_policy``) is a restatement checked by properties only.
"""
from __future__ import annotations

import numpy as np

try:  # scipy gives multi-threaded FP32 FFTs for the timed CPU path
    import scipy.fft as _sfft
except Exception:  # pragma: no cover - numpy fallback for the oracle itself
    _sfft = None

# --- constants: software/aphids/sample_rates.h:17-20,52-53,59,70,74 and
#     software/aphids/vdif_inout_gpu_thread.h:10-53 (SWARM_RATE_FRAC 11/11) ---
SWARM_RATE = 4576e6                  # sample_rates.h:17,20 (FRAC 11 of 11)
R2DBE_RATE = 4096e6                  # sample_rates.h:18
DECIMATION_FACTOR = 143              # sample_rates.h:52
EXPANSION_FACTOR = 128               # sample_rates.h:53
BENG_FRAMES_PER_GROUP = 143          # sample_rates.h:70
VDIF_OUT_PKTS_PER_BLOCK = 16384      # sample_rates.h:59
VDIF_OUT_FRAMES_PER_SECOND = 125000  # sample_rates.h:74
BENG_CHANNELS_ = 16384               # vdif_inout_gpu_thread.h:20
BENG_CHANNELS = BENG_CHANNELS_ + 1   # vdif_inout_gpu_thread.h:21
BENG_SNAPSHOTS = 128                 # vdif_inout_gpu_thread.h:22
VDIF_PER_BENG = 2048                 # vdif_inout_gpu_thread.h:17
IN_PKT_BYTES = 1056                  # vdif_inout_gpu_thread.h:10
IN_HDR_BYTES = 32                    # vdif_inout_gpu_thread.h:11
OUT_PKT_DATA_BYTES = 8192            # vdif_out_databuf.h:61
OUT_PKT_BYTES = 8224                 # sizeof(vdif_out_packet_t), vdif_out_databuf.h:66-69
BATCH_SNAPSHOTS = DECIMATION_FACTOR  # RESAMPLE_BATCH_SNAPSHOTS, vdif_inout_gpu_thread.h:31
N_A = 2 * BENG_CHANNELS_             # FFT_SIZE_SWARM_C2R = 32768, .h:35
N_B = DECIMATION_FACTOR * 256        # FFT_SIZE_SWARM_R2C = 36608, .h:45-47
N_C = EXPANSION_FACTOR * 256         # FFT_SIZE_R2DBE_C2R = 32768, .h:51
CHUNKS_PER_BATCH = BATCH_SNAPSHOTS * N_A // N_B   # FFT_BATCHES_SWARM_R2C = 128, .h:49
OUT_SAMPLES_PER_BATCH = CHUNKS_PER_BATCH * N_C    # 4,194,304
MAX_SKIP_CHAN = N_B // 2 - BENG_CHANNELS_         # 1920: bins left after 16385 kept


def skip_chan_from_mhz(trim_mhz: int) -> int:
    """Bins trimmed from DC: ``(int)(skip_mhz*1e6/(SWARM_RATE/FFT_SIZE_SWARM_R2C))``.

    Follows ``vdif_inout_gpu_thread.cu:269``.  Bin width is 125 kHz, so this is
    ``8*trim_mhz``.  Raises if the trimmed window would run past the 18305 bins
    the R2C produces (the reference would read past its buffer).
    """
    skip = int(trim_mhz * 1e6 / (SWARM_RATE / N_B))
    if skip < 0 or skip > MAX_SKIP_CHAN:
        raise ValueError(f"trim {trim_mhz} MHz -> skip {skip} outside [0, {MAX_SKIP_CHAN}]")
    return skip


# ---------------------------------------------------------------- headers ---
def decode_beng_headers(packets: np.ndarray):
    """Per-packet (invalid, c, f, b) from the B-engine VDIF header.

    c = w5 & 0xFF, f = (w5 >> 16) & 0xFF (``vdif_inout_gpu_thread.cu:353-362``);
    b is the 40-bit counter ``(w4 << 8) | (w5 >> 24)`` of
    ``vdif_in_databuf.c:66-74`` (``get_packet_b_count``; the GPU kernel keeps
    only its low 32 bits, ``.cu:367-369``, which changes nothing for packets
    inside one group); invalid = w0 bit 31 (``vdif_in_databuf.h:30-34``).
    """
    words = np.ascontiguousarray(packets).reshape(-1, IN_PKT_BYTES).view("<u4")
    w0, w4, w5 = words[:, 0], words[:, 4].astype(np.uint64), words[:, 5].astype(np.uint64)
    invalid = (w0 >> 31) & 1
    c = (w5 & 0xFF).astype(np.int64)
    f = ((w5 >> 16) & 0xFF).astype(np.int64)
    b = ((w4 << np.uint64(8)) | (w5 >> np.uint64(24))).astype(np.int64)
    return invalid.astype(np.int64), c, f, b


def channel_base_aphids(c, f):
    """First of the 8 channels a packet carries, APHIDS 11/11 map.

    ``((c>>1)*16 + (c&1) + 2*f) * 8`` from ``vdif_inout_gpu_thread.cu:442``.
    """
    return ((c >> 1) * 16 + (c & 1) + 2 * f) * 8


def channel_base_mar2015(c, f):
    """First channel of a packet in the Mar-2015 SDBE format.

    ``SWARM_XENG_PARALLEL_CHAN*(chan_id*SWARM_N_FIDS + fid)`` from
    ``prototyping/read_sdbe_vdif.py:193``.
    """
    return 8 * (c * 8 + f)


def packet_frame_index(packets, b_zero: int, n_frames: int):
    """Frame slot of each packet and whether it is scattered at all.

    The reference writes frame ``(b - b_zero) % 143`` (``.cu:437,443``) for
    packets its ingest already placed in the group window
    (``vdif_in_databuf.c:96-156``).  Here a packet is kept iff it is not flagged
    invalid, f < 8 and 0 <= b - b_zero < n_frames; anything else would land
    outside the reference's buffers, so it is dropped instead.
    """
    invalid, c, f, b = decode_beng_headers(packets)
    frame = b - int(b_zero)
    ok = (invalid == 0) & (f < 8) & (frame >= 0) & (frame < n_frames)
    return frame, c, f, ok


# --------------------------------------------------------------- unpack ----
def vdif_to_beng(packets, b_zero: int, n_frames: int = BENG_FRAMES_PER_GROUP,
                 channel_map: str = "aphids"):
    """Unpack + channel scatter into the reference's int8 B-engine buffers.

    Follows ``vdif_to_beng`` (``vdif_inout_gpu_thread.cu:404-507``) including
    the pre-zeroing memset (``.cu:897-898``): returns ``beng0, beng1`` of shape
    ``[n_frames, 128, 16384, 2]`` int8 holding (imag, real) = 2-bit code - 2
    (``.cu:387-392``).  Per snapshot the packet holds two 32-bit words; bytes
    0..3 of word 0 carry channels 3,2,1,0 and of word 1 channels 7,6,5,4
    (``.cu:464-495``); within a byte, bits 0-1/2-3 are pol-1 imag/real and
    bits 4-5/6-7 pol-0 imag/real (``.cu:482-485``).
    """
    pk = np.ascontiguousarray(packets, dtype=np.uint8).reshape(-1, IN_PKT_BYTES)
    frame, c, f, ok = packet_frame_index(pk, b_zero, n_frames)
    base = channel_base_aphids(c, f) if channel_map == "aphids" else channel_base_mar2015(c, f)
    beng = np.zeros((2, n_frames, BENG_SNAPSHOTS, BENG_CHANNELS_, 2), dtype=np.int8)
    sel = np.nonzero(ok)[0]
    if sel.size == 0:
        return beng[0], beng[1]
    # per packet and snapshot the two little-endian words as 8 bytes; byte j of
    # word h carries channel 4h + 3 - j, so reversing each word's bytes puts
    # channel k of the packet at position k
    raw = pk[sel, IN_HDR_BYTES:].reshape(sel.size, BENG_SNAPSHOTS, 2, 4)
    b8 = raw[..., ::-1].reshape(sel.size, BENG_SNAPSHOTS, 8).astype(np.int16)
    # bit pairs of a byte, LSB first: pol1 im, pol1 re, pol0 im, pol0 re
    vals = [((b8 >> (2 * q)) & 3) - 2 for q in range(4)]
    fr = frame[sel]
    grp = base[sel] // 8                       # packets carry 8 consecutive channels
    view = beng.reshape(2, n_frames, BENG_SNAPSHOTS, BENG_CHANNELS_ // 8, 8, 2)
    view[1][fr, :, grp] = np.stack([vals[0], vals[1]], axis=-1).astype(np.int8)   # (imag, real)
    view[0][fr, :, grp] = np.stack([vals[2], vals[3]], axis=-1).astype(np.int8)
    return beng[0], beng[1]


def completion_bitmap(packets, b_zero: int, n_frames: int):
    """Per-frame channel completion bytes: bit f of byte c set per packet seen.

    Same layout as ``beng_frame_completion_t.cc[256]`` set by
    ``insert_vdif_in_beng_group_buffer`` (``vdif_in_databuf.c:141-144``), plus
    the per-frame packet count (``:143``).
    """
    frame, c, f, ok = packet_frame_index(packets, b_zero, n_frames)
    cc = np.zeros((n_frames, 256), dtype=np.uint8)
    np.bitwise_or.at(cc, (frame[ok], c[ok]), (1 << f[ok]).astype(np.uint8))
    counts = np.bincount(frame[ok], minlength=n_frames).astype(np.int64)
    return cc, counts


def reorder_mar2015(spec):
    """Mar-2015 SDBE snapshot fix on ``[n_frames, 128, channels]`` spectra.

    Channels with ``(cid/4)`` even are rolled by -2 snapshots inside each
    128-snapshot B-frame, then snapshots >= 69 are taken from the next B-frame;
    the last frame is dropped.  Restates the numpy check of
    ``prototyping/cuda/reorder.py:284-293`` (kernel ``reorder``, ``:13-43``) on
    a snapshot-major layout.  Returns ``[n_frames-1, 128, channels]``.
    """
    spec = np.asarray(spec)
    out = spec.copy()
    ch = np.arange(spec.shape[2])
    shifted = ((ch // 4) & 1) == 0
    out[:, :, shifted] = np.roll(spec[:, :, shifted], -2, axis=1)
    res = out.copy()
    res[:-1, 69:, :] = out[1:, 69:, :]
    return res[:-1]


# ----------------------------------------------------------- spectra -------
def beng_to_complex(beng, dtype=np.complex128):
    """int8 (imag, real) pairs -> complex spectra with a zero Nyquist bin.

    ``beng_int8_to_cufftComplex`` (``vdif_inout_gpu_thread.cu:532-556``) plus
    the memset that zeroes channel 16384 (``.cu:925-926``).  Input
    ``[..., 16384, 2]``, output ``[..., 16385]``.
    """
    beng = np.asarray(beng)
    out = np.zeros(beng.shape[:-2] + (BENG_CHANNELS,), dtype=dtype)
    out[..., :BENG_CHANNELS_] = beng[..., 1].astype(np.float64) + 1j * beng[..., 0].astype(np.float64)
    return out


def _irfft(x, n, precision, workers):
    if precision == "f32":
        if _sfft is not None:
            return _sfft.irfft(x.astype(np.complex64), n=n, axis=-1, workers=workers)
        return np.fft.irfft(x, n=n, axis=-1).astype(np.float32)
    return np.fft.irfft(x, n=n, axis=-1)


def _rfft(x, precision, workers):
    if precision == "f32":
        if _sfft is not None:
            return _sfft.rfft(x.astype(np.float32), axis=-1, workers=workers)
        return np.fft.rfft(x, axis=-1).astype(np.complex64)
    return np.fft.rfft(x, axis=-1)


def swarm_c2r(spectra, precision="f64", workers=1):
    """FFT A, ``SwarmC2R``: per snapshot, C2R 32768, unnormalised.

    Plan ``vdif_inout_gpu_thread.cu:271-286``, exec ``:589-625``.  cuFFT's C2R
    is ``N * numpy.irfft`` (the scale the reference's own numpy check divides
    out, ``prototyping/cuda/resample.py:138``); imaginary parts of the DC and
    Nyquist bins do not contribute.  ``[n, 16385] -> [n, 32768]``.
    """
    y = _irfft(spectra, N_A, precision, workers)
    return y * (np.float32(N_A) if precision == "f32" else float(N_A))


def swarm_r2c(timeseries, n_fft=N_B, precision="f64", workers=1):
    """FFT B, ``SwarmR2C``: R2C over consecutive 36608-sample chunks.

    Plan ``vdif_inout_gpu_thread.cu:294-309`` (batch 128, contiguous input),
    exec ``:631-667``.  Each chunk is transformed on its own (no overlap), so
    chunks span snapshot boundaries exactly as the reference's flat buffer does.
    ``[..., n_chunks*36608] -> [..., n_chunks, 18305]``.
    """
    x = np.asarray(timeseries)
    n_chunks = x.shape[-1] // n_fft
    x = x[..., : n_chunks * n_fft].reshape(x.shape[:-1] + (n_chunks, n_fft))
    return _rfft(x, precision, workers)


def r2dbe_c2r(spectra, skip_chan: int, n_out=N_C, precision="f64", workers=1):
    """FFT C, ``R2dbeC2R``: C2R 32768 of bins ``[skip, skip+16385)``.

    Plan ``vdif_inout_gpu_thread.cu:317-333`` (input batch stride 18305 = the
    R2C output stride), exec ``:673-709`` with input pointer ``+skip_chan``.
    Unnormalised (cuFFT), DC/Nyquist imaginary parts ignored.  Bins the window
    asks for beyond the spectrum read as zero (the zero-padded upsampling of
    ``prototyping/cuda/resample.py:132-134`` is the same call with skip 0).
    """
    spec = np.asarray(spectra)
    need = n_out // 2 + 1
    win = spec[..., skip_chan: skip_chan + need]
    if win.shape[-1] < need:
        pad = np.zeros(win.shape[:-1] + (need - win.shape[-1],), dtype=win.dtype)
        win = np.concatenate([win, pad], axis=-1)
    y = _irfft(win, n_out, precision, workers)
    return y * (np.float32(n_out) if precision == "f32" else float(n_out))


# ------------------------------------------------------------ statistics ---
def summary_stats(y):
    """Offset and threshold: mean and sqrt(sample variance), in FP64.

    The reference merges (n, mean, M2) with Chan's formula in float through
    ``thrust::transform_reduce`` (``vdif_inout_gpu_thread.cu:66-137``) and sets
    ``quantizeThreshold = sqrt(M2/(n-1))``, ``quantizeOffset = mean``
    (``.cu:953-977``).  Returns ``(offset, threshold)``.
    """
    y = np.asarray(y, dtype=np.float64).ravel()
    return float(y.mean()), float(np.sqrt(y.var(ddof=1)))


def quantize2bit_codes(y, threshold, offset, compute_dtype=np.float64):
    """2-bit offset-binary codes per ``quantize2bit`` (``.cu:565-583``).

    ``code = ((|v| >= th) | 2) ^ (3*(v < 0))`` with ``v = x - offset``:
    0 for v <= -th, 1 for -th < v < 0, 2 for 0 <= v < th, 3 for v >= th
    (00=-2, 01=-1, 10=0, 11=+1).  ``sdbe_preprocess.quantize_to_2bit``
    (``prototyping/sdbe_preprocess.py:668-692``) differs only at v == -th
    exactly.  ``compute_dtype=np.float32`` reproduces the device's FP32 compare.
    """
    cd = compute_dtype
    v = np.asarray(y).astype(cd) - cd(offset)
    th = cd(threshold)
    above = (np.abs(v) >= th).astype(np.uint8)
    neg = (v < 0).astype(np.uint8)
    return ((above | 2) ^ (3 * neg)) & 3


def pack2bit(codes):
    """Pack 2-bit codes 16 per little-endian uint32, sample i at bits 2i..2i+1.

    ``quantize2bit`` shifts by ``threadIdx.x*2`` and ORs into one word
    (``.cu:578-580``); ``vdif.VDIFFrame.to_bin`` packs offset-binary samples
    LSB-first the same way (``prototyping/vdif.py:224-240``).
    """
    c = np.asarray(codes, dtype=np.uint32).reshape(-1, 16)
    shifts = (2 * np.arange(16, dtype=np.uint32))[None, :]
    return np.bitwise_or.reduce(c << shifts, axis=1).astype("<u4")


def unpack2bit(words):
    """Inverse of :func:`pack2bit`: uint32 words -> codes."""
    w = np.asarray(words, dtype=np.uint32).reshape(-1, 1)
    return ((w >> (2 * np.arange(16, dtype=np.uint32))[None, :]) & 3).astype(np.uint8).ravel()


# ------------------------------------------------------------- pipeline ----
class StreamState:
    """Per-stream state the reference keeps between groups.

    Thresholds/offsets (set once, ``.cu:151-152,954``) and the snapshots left
    over when the snapshot count is not a multiple of 143 (carried, not
    emitted; the reference's 143-frame groups never leave any).
    """

    def __init__(self):
        self.threshold = [0.0, 0.0]
        self.offset = [0.0, 0.0]
        self.carry = [np.zeros((0, BENG_CHANNELS), np.complex128) for _ in range(2)]
        self.raw = [None, None]   # Mar-2015 format: last unpacked B-frame, held for the next call
        # windowed thresholds: per pol the (n, mean, M2) of every batch so far and
        # the (offset, threshold) each batch was quantized with
        self.batch_stats = [[], []]
        self.used = [[], []]


THRESH_BLOCK = 16   # windowed thresholds move every 16 batches


def merge_stats(stats):
    """(n, mean, M2) of the union of batches given their (n, mean, M2)."""
    st = np.asarray(stats, np.float64).reshape(-1, 3)
    n = st[:, 0].sum()
    mean = (st[:, 0] * st[:, 1]).sum() / n
    m2 = st[:, 2].sum() + (st[:, 0] * (st[:, 1] - mean) ** 2).sum()
    return n, mean, m2


def window_thresholds(state: StreamState, pol: int, t: int, window: int):
    """(offset, threshold) for stream batch t in windowed mode (a
    restatement of this library's SDBE_THRESH_WINDOW; the reference sets the
    thresholds once): batch 0's own statistics for the first block, then at
    every block boundary T the statistics of batches [max(0, T - window), T)."""
    T = (t // THRESH_BLOCK) * THRESH_BLOCK
    if T == 0:
        n, mean, m2 = state.batch_stats[pol][0]
    else:
        n, mean, m2 = merge_stats(state.batch_stats[pol][max(0, T - window):T])
    return float(mean), float(np.sqrt(m2 / (n - 1.0)))


def process_group(packets, b_zero: int, n_frames: int, trim_mhz: int,
                  state: StreamState | None = None, precision="f64", workers=1,
                  pol1_uses_pol0_threshold=False, channel_map="aphids",
                  return_float=False, threshold_window=None):
    """One call of the GPU stage on ``n_frames`` B-frames of packets.

    Follows the body of ``run_method`` (``vdif_inout_gpu_thread.cu:894-1017``):
    unpack (K1), then for every 143-snapshot batch FFT A, FFT B, FFT C, the
    one-off threshold from the first batch ever seen, and quantize2bit.  Output
    is ``uint8 [2, n_batches*128, 8192]`` = ``vdif_out_data_group_t`` payloads
    (``vdif_out_databuf.h:110-116``), packet ``iter*128 + k`` holding chunk k
    of batch iter (``.cu:994``).  The reference applies pol 0's threshold to
    pol 1 (``.cu:1004-1005``); ``pol1_uses_pol0_threshold`` reproduces that,
    the default uses each pol's own.  ``threshold_window`` (batches) switches
    to windowed thresholds (``window_thresholds``).
    """
    if state is None:
        state = StreamState()
    skip = skip_chan_from_mhz(trim_mhz)
    beng0, beng1 = vdif_to_beng(packets, b_zero, n_frames, channel_map)
    spec_dtype = np.complex64 if precision == "f32" else np.complex128
    outs, floats = [], []
    for pol, beng in enumerate((beng0, beng1)):
        if channel_map == "mar2015":
            # Mar-2015 SDBE: output frame f needs input frames f and f+1
            # (reorder.py:284-293), so the last input frame waits for the next call.
            if state.raw[pol] is not None:
                beng = np.concatenate([state.raw[pol], beng], axis=0)
            state.raw[pol] = beng[-1:].copy() if beng.shape[0] else state.raw[pol]
            beng = reorder_mar2015(beng) if beng.shape[0] >= 2 else beng[:0]
        spec = beng_to_complex(beng.reshape(-1, BENG_CHANNELS_, 2), spec_dtype)
        spec = np.concatenate([state.carry[pol].astype(spec_dtype), spec], axis=0)
        n_batches = spec.shape[0] // BATCH_SNAPSHOTS
        state.carry[pol] = spec[n_batches * BATCH_SNAPSHOTS:].copy()
        words = np.zeros((n_batches * CHUNKS_PER_BATCH, OUT_PKT_DATA_BYTES // 4), np.uint32)
        fl = []
        for it in range(n_batches):
            block = spec[it * BATCH_SNAPSHOTS:(it + 1) * BATCH_SNAPSHOTS]
            ts = swarm_c2r(block, precision, workers).reshape(-1)
            y = r2dbe_c2r(swarm_r2c(ts, N_B, precision, workers), skip, N_C, precision, workers)
            cd = np.float32 if precision == "f32" else np.float64
            if threshold_window:
                y64 = np.asarray(y, np.float64).ravel()
                mu = y64.mean()
                state.batch_stats[pol].append((float(y64.size), float(mu), float(((y64 - mu) ** 2).sum())))
                t = len(state.batch_stats[pol]) - 1
                state.offset[pol], state.threshold[pol] = window_thresholds(state, pol, t, threshold_window)
                state.used[pol].append((state.offset[pol], state.threshold[pol]))
                off, th = state.used[0][t] if pol1_uses_pol0_threshold else state.used[pol][t]
                codes = quantize2bit_codes(y, th, off, cd)
            else:
                if state.threshold[pol] == 0.0:
                    state.offset[pol], state.threshold[pol] = summary_stats(y)
                th_pol = 0 if pol1_uses_pol0_threshold else pol
                if pol1_uses_pol0_threshold and state.threshold[0] == 0.0:
                    raise RuntimeError("pol 0 threshold unset")
                codes = quantize2bit_codes(y, state.threshold[th_pol], state.offset[th_pol], cd)
            words[it * CHUNKS_PER_BATCH:(it + 1) * CHUNKS_PER_BATCH] = pack2bit(codes).reshape(CHUNKS_PER_BATCH, -1)
            if return_float:
                fl.append(y)
        outs.append(words.view(np.uint8).reshape(n_batches * CHUNKS_PER_BATCH, OUT_PKT_DATA_BYTES))
        if return_float:
            floats.append(np.concatenate(fl, axis=0) if fl else np.zeros((0, N_C)))
    out = np.stack(outs, axis=0)
    if return_float:
        return out, floats
    return out


# ------------------------------------------------------------ output VDIF --
def vdif_out_header_words(n_pkts: int, pol: int, secs: int, df: int, psn: int,
                          ref_epoch: int = 0, station: int = (ord("S") << 8) | ord("m"),
                          bdc_sideband: int = 0, rx_sideband: int = 0, bit_depth: int = 2):
    """Eight header words per output frame, per the reference's output thread.

    Field layout ``vdif_out_header_t`` (``vdif_out_databuf.h:19-52``); constant
    fields from ``init_vdif_out`` (``vdif_out_databuf.c:35-64``: df_len =
    8224/8, edv5 = 2, real data); per-packet fields from
    ``vdif_out_net_thread.c:295-317``: secs/df advance per packet with df
    wrapping at 125000, threadID 0, bps = bit_depth-1, pol, sidebands, psn
    incrementing per packet.  Returns ``uint32 [n_pkts, 8]``.
    """
    ii = np.arange(n_pkts, dtype=np.int64)
    dfs = df + ii
    secs_ii = secs + dfs // VDIF_OUT_FRAMES_PER_SECOND
    df_ii = dfs % VDIF_OUT_FRAMES_PER_SECOND
    psn_ii = (psn + ii).astype(np.uint64)
    w = np.zeros((n_pkts, 8), dtype=np.uint32)
    w[:, 0] = (secs_ii & 0x3FFFFFFF).astype(np.uint32)
    w[:, 1] = ((df_ii & 0xFFFFFF) | ((ref_epoch & 0x3F) << 24)).astype(np.uint32)
    w[:, 2] = (OUT_PKT_BYTES // 8) & 0xFFFFFF
    w[:, 3] = (station & 0xFFFF) | (0 << 16) | (((bit_depth - 1) & 0x1F) << 26)
    w[:, 4] = (pol & 1) | ((bdc_sideband & 1) << 1) | ((rx_sideband & 1) << 2) | (2 << 24)
    w[:, 5] = 0
    w[:, 6] = (psn_ii & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    w[:, 7] = (psn_ii >> np.uint64(32)).astype(np.uint32)
    return w


def frame_vdif(payloads, pol: int, **hdr):
    """Prepend output headers: ``[n, 8192] -> uint8 [n, 8224]`` VDIF frames."""
    payloads = np.asarray(payloads, dtype=np.uint8).reshape(-1, OUT_PKT_DATA_BYTES)
    words = vdif_out_header_words(payloads.shape[0], pol, **hdr)
    return np.concatenate([words.view(np.uint8).reshape(-1, 32), payloads], axis=1)


# ------------------------------------------------------ time alignment ------
SWARM_CLK_PER_SEC = 286000000          # beng_reform.c:25
SWARM_BFRAME_CLK = 262144              # beng_reform.c:27
SWARM_ZERO_DELAY_OFFSET_PICOSECONDS = 3715791   # vdif_out_databuf.h:11
OUT_WORDS_PER_PKT = OUT_PKT_DATA_BYTES // 4


def beng_timestamp_increment(sec, clk):
    """One B-frame later (``beng_reform.c:192-198``; wraps only when clk > 286e6)."""
    clk += SWARM_BFRAME_CLK
    if clk > SWARM_CLK_PER_SEC:
        sec += 1
        clk = clk % SWARM_CLK_PER_SEC
    return sec, clk


def beng_timestamp_decrement(sec, clk):
    """One B-frame earlier (``beng_reform.c:200-206``)."""
    clk -= SWARM_BFRAME_CLK
    if clk < 0:
        sec -= 1
        clk = clk + SWARM_CLK_PER_SEC
    return sec, clk


def header_template(t0_sec, t0_clk, ref_epoch=0):
    """Output timestamp template from the first B-engine timestamp.

    ``get_beng_t0`` moves T0 one B-frame earlier (SWARM_TIMESTAMP_OFF_BY_BENG =
    -1, ``beng_reform.c:112-126``); ``fill_vdif_header_template`` moves it one
    frame later again and sets secs, the next whole 8-us data frame and the
    picoseconds between the two (``vdif_in_databuf.c:193-220``).  Returns
    ``(secs, df, ps_early, ref_epoch)``.
    """
    s, c = beng_timestamp_decrement(t0_sec, t0_clk)
    s, c = beng_timestamp_increment(s, c)
    frame_full = VDIF_OUT_FRAMES_PER_SECOND * 1.0 * (float(c) / float(SWARM_CLK_PER_SEC))
    frame_ceil = float(np.ceil(frame_full))
    frac = frame_ceil - frame_full
    return s, int(frame_ceil), int(np.floor(frac * (1e12 / VDIF_OUT_FRAMES_PER_SECOND))), ref_epoch


class AlignState:
    """Output-thread state (``vdif_out_net_thread.c:72-80,199-317``)."""

    def __init__(self, template=None, station=(ord("S") << 8) | ord("m"), bdc=0, rx=0):
        self.pending = template is not None
        self.template = template
        self.leftover = [np.zeros(0, np.uint32), np.zeros(0, np.uint32)]
        self.secs = self.df = self.psn = self.ref_epoch = 0
        self.station, self.bdc, self.rx = station, bdc, rx


def align_frames(payload, st: AlignState):
    """Time-aligned 8224-B frames from one block of payloads ``[2, n, 8192]``.

    On the first block after a template: start on the next second boundary
    when the block would cross one (skip frames), skip
    ``floor(floor((ps + 3715791) * 4096e6/1e12) / 16)`` 32-bit words, psn from 1
    (``:206-237``).  Every block: the aligned word stream is the previous
    block's leftover words followed by this block's words; whole 8192-B
    packets are framed with secs/df/psn advancing per packet and the rest is
    carried (``:251-317``).  The reference's first block reads its skipped
    frames past the end of the block; here the skip is taken from the front.
    """
    words = [np.ascontiguousarray(payload[p]).reshape(-1).view("<u4") for p in range(2)]
    n_words = words[0].size
    skip = 0
    if st.pending:
        secs, df, ps, ref_epoch = st.template
        skip_frames = 0
        n_usable = n_words // OUT_WORDS_PER_PKT
        if df > VDIF_OUT_FRAMES_PER_SECOND - n_usable:
            skip_frames = VDIF_OUT_FRAMES_PER_SECOND - df
            df = 0
            secs += 1
        skip_ps = ps + SWARM_ZERO_DELAY_OFFSET_PICOSECONDS
        skip_samples = int(np.floor(float(skip_ps) * R2DBE_RATE / 1e12))
        skip = int(np.floor(skip_samples / (8.0 / 2) / 4)) + skip_frames * OUT_WORDS_PER_PKT
        st.secs, st.df, st.ref_epoch, st.psn = secs, df, ref_epoch, 1
        st.pending = False
    streams = [np.concatenate([st.leftover[p], words[p][skip:]]) for p in range(2)]
    n_pkts = streams[0].size // OUT_WORDS_PER_PKT
    frames = []
    for p in range(2):
        body = streams[p][:n_pkts * OUT_WORDS_PER_PKT].view(np.uint8).reshape(n_pkts, OUT_PKT_DATA_BYTES)
        st.leftover[p] = streams[p][n_pkts * OUT_WORDS_PER_PKT:].copy()
        frames.append(frame_vdif(body, p, secs=st.secs, df=st.df, psn=st.psn, ref_epoch=st.ref_epoch,
                                 station=st.station, bdc_sideband=st.bdc, rx_sideband=st.rx))
    dfs = st.df + n_pkts
    st.secs += dfs // VDIF_OUT_FRAMES_PER_SECOND
    st.df = dfs % VDIF_OUT_FRAMES_PER_SECOND
    st.psn += n_pkts
    return np.stack(frames)


# ------------------------------------------------------- group assembly -----
BENG_GROUPS_IN_BUFFER = 4              # vdif_in_databuf.h:146
MAX_INDEX_LOOK_AHEAD = 2               # vdif_in_net_thread.c:136
GROUP_PACKETS = BENG_FRAMES_PER_GROUP * VDIF_PER_BENG   # 292864


class IngestState:
    """Ingest-thread state: b_first, the oldest open group and per-group counts."""

    def __init__(self):
        self.b_first = -1
        self.ref = 0                       # index of the oldest open group
        self.count = {}                    # group -> packets inserted
        self.fcount = {}                   # group -> per-frame packets inserted
        self.shipped = []                  # (group, packets held) of every shipped group, in order
        self.stats = dict(packets=0, invalid=0, before_start=0, too_far_ahead=0, used=0, overflow=0,
                          groups_shipped=0, groups_incomplete=0)

    def start(self, g):
        return self.b_first + 1 + BENG_FRAMES_PER_GROUP * g


def ingest_policy(packets, st: IngestState, flush=False):
    """Which packets join which group, and when groups ship.

    Restates the ingest loop of ``vdif_in_net_thread.c:255-500``: each received
    batch is sorted invalid-first then by b (``compar_beng``, ``:48-68``); the
    first valid b of the stream fixes the groups at b_first+1+143k (``:317-337``);
    per packet ``get_beng_group_index_offset`` (``vdif_in_databuf.c:96-124``)
    returns invalid / before start / too far ahead (beyond the group after the
    4th by more than 4*143 frames) or the group offset; an offset above
    MAX_INDEX_LOOK_AHEAD ships the oldest group incomplete and the packet is
    examined again (``:393-401``); otherwise it is inserted
    (``insert_vdif_in_beng_group_buffer``, ``vdif_in_databuf.c:126-156``: at most
    2048 packets per frame and 292864 per group) and a complete oldest group
    ships (``check_beng_group_complete``, ``:158-167``).  Returns the accept
    mask (original packet order) and the groups shipped, in order.  Only the
    first 24 bytes of a row are read: ``[n, 1056]`` packets or ``[n, k >= 24]``
    header rows.  ``flush`` then ships every group still holding packets.
    """
    pk = np.asarray(packets, dtype=np.uint8)
    pk = pk.reshape(-1, IN_PKT_BYTES) if pk.ndim == 1 else pk
    w = np.ascontiguousarray(pk[:, :24]).view("<u4")   # header rows suffice
    invalid = ((w[:, 0] >> 31) & 1).astype(np.int64)
    b = ((w[:, 4].astype(np.uint64) << np.uint64(8)) | (w[:, 5].astype(np.uint64) >> np.uint64(24))).astype(np.int64)
    n = pk.shape[0]
    st.stats["packets"] += n
    key = np.where(invalid != 0, -(2**62), b)
    order = np.argsort(key, kind="stable")
    accept = np.zeros(n, bool)
    ships = []

    def ship():
        g = st.ref
        ships.append(g)
        st.shipped.append((g, st.count.get(g, 0)))
        st.stats["groups_shipped"] += 1
        if st.count.get(g, 0) < GROUP_PACKETS:
            st.stats["groups_incomplete"] += 1
        st.count.pop(g, None)
        st.fcount.pop(g, None)
        st.ref += 1

    if st.b_first < 0:
        valid = order[invalid[order] == 0]
        if valid.size == 0:
            st.stats["invalid"] += n
            return accept, ships
        st.b_first = int(b[valid[0]])
        st.ref = 0
    for i in order:
        bi = int(b[i])
        while True:
            if invalid[i]:
                st.stats["invalid"] += 1
                break
            lo = st.start(st.ref)
            if bi < lo:
                st.stats["before_start"] += 1
                break
            off = (bi - lo) // BENG_FRAMES_PER_GROUP
            if off >= BENG_GROUPS_IN_BUFFER:
                # the search (:107-116) leaves its upper bound at the last
                # frame of the group after the four it checked
                lu_last = st.start(st.ref + BENG_GROUPS_IN_BUFFER + 1) - 1
                if bi > lu_last + BENG_GROUPS_IN_BUFFER * BENG_FRAMES_PER_GROUP:
                    st.stats["too_far_ahead"] += 1
                    break
                off = BENG_GROUPS_IN_BUFFER
            if off > MAX_INDEX_LOOK_AHEAD:
                ship()
                continue
            g = st.ref + off
            frame = bi - st.start(g)
            fc = st.fcount.setdefault(g, np.zeros(BENG_FRAMES_PER_GROUP, np.int64))
            st.stats["used"] += 1
            if fc[frame] < VDIF_PER_BENG and st.count.get(g, 0) < GROUP_PACKETS:
                fc[frame] += 1
                st.count[g] = st.count.get(g, 0) + 1
                accept[i] = True
            else:
                st.stats["overflow"] += 1
            if st.count.get(st.ref, 0) == GROUP_PACKETS:
                ship()
            break
    if flush:
        while st.count:
            ship()
    return accept, ships


# ---------------------------------------------------------------------------
# 8pac input format and the B-engine header reform (ingest transforms)
# ---------------------------------------------------------------------------
VTP_BYTES = 8                                       # vdif_8pac.h:6
PAC8_BYTES = IN_PKT_BYTES + 7 * (VTP_BYTES + IN_PKT_BYTES)   # sizeof(vdif_8pac_packet_t) = 8504
BFRAME_CLK_TOL = 1024                               # beng_reform.c:29
MAX_COUNTABLE_BFRAME_OFFSET = 1000                  # beng_reform.c:65


def pac8_offsets():
    """Byte offset of each of the 8 packets inside one 8pac (vdif_8pac.h:8-16)."""
    return np.array([0] + [IN_PKT_BYTES + k * (VTP_BYTES + IN_PKT_BYTES) + VTP_BYTES for k in range(7)])


def unpack_8pac(src):
    """8pac units -> plain 1056-B packets, ``unpack_8pac`` (vdif_8pac.c:47-56).

    Per unit: df_len of all 8 = ((df_len_1 - 7) / 8) & 0xFFFFFF, the 24-bit
    bit-field promoted to int and divided toward zero (``reset_8pac_size``,
    :5-13); df_num_insec = 8*df_1 (+k for packet k, 24-bit field, ``:15-23``);
    psn = 8*psn_1 (+k, ``:25-34``); the invalid bit of packet 1 copied to the
    other 7 (``:36-41``).  The 8-byte VTP prefixes are dropped.
    """
    s = np.ascontiguousarray(src, dtype=np.uint8).reshape(-1, PAC8_BYTES)
    n = s.shape[0]
    off = pac8_offsets()
    out = np.empty((n, 8, IN_PKT_BYTES), np.uint8)
    for k in range(8):
        out[:, k] = s[:, off[k]:off[k] + IN_PKT_BYTES]
    w = out.view("<u4").reshape(n, 8, IN_PKT_BYTES // 4)
    w1 = w[:, 0]
    df_len = (w1[:, 2] & 0xFFFFFF).astype(np.int64) - 7
    newsize = (np.sign(df_len) * (np.abs(df_len) // 8)).astype(np.int64) & 0xFFFFFF
    df8 = (8 * (w1[:, 1] & 0xFFFFFF).astype(np.int64))
    psn1 = w1[:, 6].astype(np.uint64) | (w1[:, 7].astype(np.uint64) << np.uint64(32))
    inv = w1[:, 0] >> 31
    for k in range(8):
        wk = w[:, k]
        wk[:, 2] = (wk[:, 2] & np.uint32(0xFF000000)) | newsize.astype(np.uint32)
        wk[:, 1] = (wk[:, 1] & np.uint32(0xFF000000)) | ((df8 + k) & 0xFFFFFF).astype(np.uint32)
        psn = psn1 * np.uint64(8) + np.uint64(k)
        wk[:, 6] = (psn & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        wk[:, 7] = (psn >> np.uint64(32)).astype(np.uint32)
        if k:
            wk[:, 0] = (wk[:, 0] & np.uint32(0x7FFFFFFF)) | (inv << np.uint32(31))
    return out.reshape(n * 8, IN_PKT_BYTES)


def read_beng_timestamp(w4, w5):
    """(sec, clk) of the new-format B-engine header (beng_reform.h:14-19,
    ``_read_beng_timestamp`` beng_reform.c:16-22): b = b_upper<<21 | b_lower
    (w5 bits 11-31); clk = b & 0x1FFFFFFF, sec = bits 29-52 of b."""
    b = (int(w4) << 21) | ((int(w5) >> 11) & 0x1FFFFF)
    return (b & 0x001FFFFFE0000000) >> 29, b & 0x1FFFFFFF


def timestamp_compare(then, now):
    """``_beng_timestamp_compare_then_now`` (beng_reform.c:34-61), as written
    (the later-second branch does not check that the seconds are adjacent)."""
    C, T = SWARM_CLK_PER_SEC, BFRAME_CLK_TOL
    if then[0] < now[0]:
        if then[0] == now[0] - 1 and then[1] + T > C and (then[1] + T) % C >= now[1]:
            return 0
        return -1
    if then[0] > now[0]:
        if now[1] + T > C and (now[1] + T) % C >= then[1]:
            return 0
        return 1
    if then[1] + T < now[1]:
        return -1
    if now[1] + T < then[1]:
        return 1
    return 0


def timestamp_offset(then, now):
    """B-frames from then to now by stepping (beng_reform.c:71-104), capped
    just beyond MAX_COUNTABLE_BFRAME_OFFSET."""
    cmp = timestamp_compare(then, now)
    if cmp == 0:
        return 0
    start, end, step = (then, now, 1) if cmp < 0 else (now, then, -1)
    off = 0
    while timestamp_compare(start, end) < 0:
        start = beng_timestamp_increment(*start)
        off += step
        if abs(off) > MAX_COUNTABLE_BFRAME_OFFSET:
            break
    return off


class ReformState:
    """The reform's stream state: T0, TPREV and BPREV (beng_reform.c:6-14)."""

    def __init__(self):
        self.t0 = (-1, -1)
        self.tprev = (-1, -1)
        self.bprev = -1


def _i32(v):
    return ((int(v) + 2**31) % 2**32) - 2**31


def beng_reform_headers(pkts, st: ReformState):
    """Rewrite new-format B-engine headers to the old format in place
    (``beng_reform_headers``, beng_reform.c:137-186).

    Invalid packets are left alone; the first valid packet fixes T0; each valid
    packet's B-count is BPREV + the frame offset from TPREV (a 32-bit int, as
    in the reference); an offset beyond +-1000 frames marks the packet invalid
    with count -1 and leaves TPREV/BPREV unchanged.  Only the c, f, b_lower
    bytes of w5 and all of w4 are written; byte 1 of w5 keeps its old bits.
    """
    w = pkts.view("<u4").reshape(-1, IN_PKT_BYTES // 4)
    for i in range(w.shape[0]):
        if w[i, 0] >> 31:
            continue
        w4, w5 = int(w[i, 4]), int(w[i, 5])
        if st.t0 == (-1, -1):
            st.t0 = read_beng_timestamp(w4, w5)
            st.tprev = st.t0
            st.bprev = 0
        now = read_beng_timestamp(w4, w5)
        off = _i32(timestamp_offset(st.tprev, now))
        if off > MAX_COUNTABLE_BFRAME_OFFSET or off < -MAX_COUNTABLE_BFRAME_OFFSET:
            w[i, 0] |= np.uint32(1 << 31)
            off = -1
        else:
            off = _i32(off + st.bprev)
            st.tprev = now
            st.bprev = off
        c, f = w5 & 0xFF, (w5 >> 8) & 0x7
        w[i, 5] = np.uint32((w5 & 0x0000FF00) | c | (f << 16) | ((off & 0xFF) << 24))
        w[i, 4] = np.uint32((off & 0x7FFFFF00) >> 8)
    return pkts


def reform_t0(st: ReformState):
    """``get_beng_t0`` (beng_reform.c:113-126): T0 one B-frame earlier
    (SWARM_TIMESTAMP_OFF_BY_BENG = -1)."""
    return beng_timestamp_decrement(*st.t0)


# ---------------------------------------------------------------------------
# Polyphase filter bank and its inverse (PFB-mode SWARM data)
# ---------------------------------------------------------------------------
def hamming_pfb(n, m):
    """``hamming`` of prototyping/cuda/pfb_inverse.cu:51-53: 0.54 - 0.46 cos(2 pi n / (m-1))."""
    return 0.54 - 0.46 * np.cos(2.0 * np.pi * np.asarray(n, np.float64) / (m - 1.0))


def forward_pfb(x, lblock, ntap=4):
    """PFB spectra of a real time stream, as ``pfb`` builds them
    (pfb_inverse.cu:173-207): block i windows samples [i*L, i*L + ntap*L)
    with hamming(n, ntap*L), takes the rFFT of length ntap*L and keeps every
    ntap-th bin (``decimate``, :57-64) -> [nblock][L/2+1] complex, nblock =
    len(x)/L - (ntap-1)."""
    x = np.asarray(x, np.float64)
    nblock = x.size // lblock - (ntap - 1)
    w = hamming_pfb(np.arange(ntap * lblock), ntap * lblock)
    idx = np.arange(nblock)[:, None] * lblock + np.arange(ntap * lblock)[None, :]
    f = np.fft.rfft(x[idx] * w, axis=1)
    return f[:, ::ntap][:, :lblock // 2 + 1]


def pfb_band(lblock, ntap=4):
    """Per phase p: the P taps w[t*L + p] (t = 0..ntap-1) and the band of
    P P^T, a[d] = sum_k w[(k+d)L + p] w[kL + p] (pfb_inverse.cu:261-300)."""
    w = hamming_pfb(np.arange(ntap * lblock), ntap * lblock).reshape(ntap, lblock)
    a = np.stack([(w[d:] * w[:ntap - d]).sum(axis=0) for d in range(ntap)])
    return w, a


def banded_ldl_solve(a, y):
    """Solve T z = y for every column p, T the symmetric banded Toeplitz
    matrix with band a[0..b] (a[:, p] per column), by LDL^T, vectorised over
    p (FP64).  y: [n][P]."""
    b = a.shape[0] - 1
    n, P = y.shape
    L = np.zeros((n, b + 1, P))          # L[m, k] = L[m][m-k], k = 1..b
    d = np.zeros((n, P))
    for m in range(n):
        for k in range(b, 0, -1):
            j = m - k
            if j < 0:
                continue
            s = a[k].copy()
            for q in range(k + 1, b + 1):     # sum over columns left of j
                if m - q >= 0 and j - (m - q) <= b and j - (m - q) > 0:
                    s -= L[m, q] * d[m - q] * L[j, j - (m - q)]
            L[m, k] = s / d[j]
        d[m] = a[0] - sum(L[m, k] ** 2 * d[m - k] for k in range(1, b + 1) if m - k >= 0)
    w = np.zeros((n, P))
    for m in range(n):
        w[m] = y[m] - sum(L[m, k] * w[m - k] for k in range(1, b + 1) if m - k >= 0)
    v = w / d
    z = np.zeros((n, P))
    for m in range(n - 1, -1, -1):
        z[m] = v[m] - sum(L[m + k, k] * z[m + k] for k in range(1, b + 1) if m + k < n)
    return z


def inverse_pfb(spec, ntap=4):
    """Time stream from PFB spectra by Shaw's least-squares inversion, the
    method of prototyping/cuda/pfb_inverse.cu:213-488: the pseudo time stream
    y = irfft(S) (the C2R then the 1/L scale, :395-418), per phase p the
    banded solve (P P^T) z = y[:, p] (:420-430) and the projection
    x[:, p] = P^T z (:432-440), with P[i][j] = w[(j-i)L + p] for
    0 <= j-i < ntap.  Output [nblock + ntap - 1][L] (FP64).  The published
    method is Shaw's pfb-inverse (github.com/jrs65/pfb-inverse, unpinned);
    the prototype compiles its solve and projection out (``#if 0``)."""
    spec = np.asarray(spec, np.complex128)
    lblock = 2 * (spec.shape[1] - 1)
    nblock = spec.shape[0]
    y = np.fft.irfft(spec, n=lblock, axis=1)
    w, a = pfb_band(lblock, ntap)
    z = banded_ldl_solve(a, y)
    x = np.zeros((nblock + ntap - 1, lblock))
    for t in range(ntap):
        x[t:t + nblock] += w[t][None, :] * z
    return x
