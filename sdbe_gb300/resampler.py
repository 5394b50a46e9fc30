"""Python host side of the GB300 resampling stage (over the C ABI).

``Resampler`` owns one ``sdbe_resampler`` handle, the GB300 counterpart of
``aphids_resampler_t`` (software/aphids/vdif_inout_gpu_thread.cu:144-180):
device buffers, twiddle tables, the one-off thresholds and the carried
snapshots of a stream.  ``process`` is one pass of the GPU stage over a group
of B-frames (``run_method``'s STATE_PROC body, .cu:874-1017).

Buffers may be numpy arrays (host memory, copied in/out by the library),
torch CUDA tensors, or raw device addresses (``int``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N


def _is_device(buf) -> bool:
    if isinstance(buf, np.ndarray):
        return False
    if isinstance(buf, int):
        return True
    return bool(getattr(buf, "is_cuda", False)) or hasattr(buf, "__cuda_array_interface__")


def _addr(buf) -> int:
    if buf is None:
        return 0
    if isinstance(buf, int):
        return buf
    if isinstance(buf, np.ndarray):
        return buf.ctypes.data
    if hasattr(buf, "data_ptr"):
        return int(buf.data_ptr())
    if hasattr(buf, "__cuda_array_interface__"):
        return int(buf.__cuda_array_interface__["data"][0])
    raise TypeError(f"unsupported buffer type {type(buf)!r}")


def _nbytes(buf) -> int:
    if isinstance(buf, np.ndarray):
        return buf.nbytes
    if hasattr(buf, "element_size"):
        return int(buf.numel() * buf.element_size())
    raise TypeError("pass out_bytes for raw device addresses")


@dataclass
class GroupResult:
    n_batches: int
    n_out_packets: int
    packets_accepted: int
    packets_rejected: int
    frames_incomplete: int
    carry_snapshots: int


class Resampler:
    """One resampling stream pair (both phased sums of a packet stream)."""

    def __init__(self, trim_mhz: int = 150, device: int = 0, max_frames: int = 143,
                 threshold_mode: int = N.THRESH_FIRST_BATCH, pol1_uses_pol0_threshold: bool = False,
                 channel_map: int = N.MAP_APHIDS, wave_batches: int = 0, threshold_window: int = 0,
                 precision: int = N.PRECISION_FP32, stage_launches: int = 0):
        self._lib = N.lib()
        cfg = N.Config()
        cfg.device = device
        cfg.trim_mhz = trim_mhz
        cfg.max_frames = max_frames
        cfg.threshold_mode = threshold_mode
        cfg.pol1_uses_pol0_threshold = int(bool(pol1_uses_pol0_threshold))
        cfg.channel_map = channel_map
        cfg.wave_batches = wave_batches
        cfg.threshold_window = threshold_window
        cfg.precision = precision
        cfg.stage_launches = stage_launches
        h = C.c_void_p()
        N.check(self._lib.sdbe_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.trim_mhz = trim_mhz
        self.device = device
        self.max_frames = max_frames
        self.skip_chan = int(trim_mhz * 1e6 / (4576e6 / 36608))

    # -- lifecycle --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.sdbe_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- processing ---------------------------------------------------------
    def output_bytes(self, n_frames: int, framed: bool = False, aligned: bool = False) -> int:
        flags = (N.OUT_FRAMED if framed else 0) | (N.OUT_ALIGNED if aligned else 0)
        return int(self._lib.sdbe_output_bytes(self._h, n_frames, flags))

    def process(self, packets, n_frames: int, b_zero: int, out=None, framed: bool = False,
                stream=None, n_packets: int | None = None, out_bytes: int | None = None,
                want_result: bool = True, asynchronous: bool = False, aligned: bool = False):
        """Run the stage on ``n_frames`` B-frames starting at counter ``b_zero``.

        Returns ``(out, GroupResult | None)``; ``out`` holds the payloads as
        ``[2, n_out_packets, 8192]`` (or 8224-B VDIF frames when ``framed``).
        With ``asynchronous`` (and no result requested) the call returns once
        the work is queued; ``sync()`` waits for it, and host buffers must stay
        alive until then.
        """
        if n_packets is None:
            n_packets = int(packets.shape[0]) if hasattr(packets, "shape") else 0
        flags = 0 if _is_device(packets) else N.IN_HOST
        framed = framed or aligned
        need = self.output_bytes(n_frames, framed, aligned)
        if out is None:
            pkt = N.OUT_PKT_BYTES if framed else N.OUT_PKT_DATA_BYTES
            out = np.empty((2, need // (2 * pkt) if need else 0, pkt), np.uint8)
        if not _is_device(out):
            flags |= N.OUT_HOST
        if framed:
            flags |= N.OUT_FRAMED
        if aligned:
            flags |= N.OUT_ALIGNED
        if asynchronous:
            flags |= N.ASYNC
        cap = _nbytes(out) if out_bytes is None else out_bytes
        res = N.Result() if want_result else None
        st = C.c_void_p(stream) if isinstance(stream, int) else (
            C.c_void_p(stream.cuda_stream) if stream is not None else None)
        rc = self._lib.sdbe_process(self._h, _addr(packets), n_packets, n_frames, b_zero, _addr(out), cap,
                                    flags, st, C.byref(res) if res is not None else None)
        N.check(rc, self._h)
        if aligned and res is not None and isinstance(out, np.ndarray):
            # packed [2][P][8224] in the first 2*P*8224 bytes
            n = res.n_out_packets
            out = out.reshape(-1)[:2 * n * N.OUT_PKT_BYTES].reshape(2, n, N.OUT_PKT_BYTES)
        if res is None:
            return out, None
        return out, GroupResult(res.n_batches, res.n_out_packets, res.packets_accepted, res.packets_rejected,
                                res.frames_incomplete, res.carry_snapshots)

    # -- state ----------------------------------------------------------------
    def get_state(self) -> N.State:
        st = N.State()
        N.check(self._lib.sdbe_get_state(self._h, C.byref(st)), self._h)
        return st

    def set_state(self, st: N.State):
        N.check(self._lib.sdbe_set_state(self._h, C.byref(st)), self._h)

    def set_thresholds(self, threshold, offset):
        st = self.get_state()
        st.threshold[0], st.threshold[1] = threshold
        st.offset[0], st.offset[1] = offset
        self.set_state(st)

    def reset(self):
        N.check(self._lib.sdbe_reset(self._h), self._h)

    def align_start(self, t0_sec: int, t0_clk: int, ref_epoch: int = 0):
        """Arm output time alignment from the first B-engine timestamp."""
        t = N.TimeTemplate()
        N.check(self._lib.sdbe_header_template(t0_sec, t0_clk, ref_epoch, C.byref(t)))
        N.check(self._lib.sdbe_align_start(self._h, C.byref(t)), self._h)
        return (t.secs_inre, t.df_num_insec, t.ps_early, t.ref_epoch)

    # -- group assembly ------------------------------------------------------
    GROUP_PACKETS_OUT = 16384  # output packets per pol of one 143-frame group

    def _group_out(self, n_groups, framed):
        pkt = N.OUT_PKT_BYTES if framed else N.OUT_PKT_DATA_BYTES
        return np.empty((n_groups, 2, self.GROUP_PACKETS_OUT, pkt), np.uint8)

    def ingest(self, packets, out=None, out_groups: int | None = None, framed: bool = False,
               pac8: bool = False, n_packets: int | None = None):
        """Offer received packets to the group ring.

        ``packets``: ``[n, 1056]`` uint8 B-engine packets, or with ``pac8``
        ``[n, 8504]`` 8pac units carrying new-format headers (unpacked and
        reformed on the device first); host (numpy) or device memory.
        Returns ``(groups, n)``: the ``n`` groups this batch shipped, as
        ``[n, 2, 16384, 8192]`` payloads (8224-B frames when ``framed``).
        Without ``out`` a host array is sized from the packet count and grown
        once if the batch ships more.
        """
        unit = N.PAC8_BYTES if pac8 else N.IN_PKT_BYTES
        flags = (N.OUT_FRAMED if framed else 0) | (N.IN_8PAC if pac8 else 0)
        if _is_device(packets):
            if n_packets is None:
                n_packets = _nbytes(packets) // unit
            src = packets
        else:
            src = np.ascontiguousarray(packets, dtype=np.uint8).reshape(-1, unit)
            n_packets = src.shape[0]
            flags |= N.IN_HOST
        auto = out is None
        if auto:
            n_pk = n_packets * (8 if pac8 else 1)
            out_groups = n_pk // 292864 + 1 if out_groups is None else out_groups
            out = self._group_out(out_groups, framed)
        elif out_groups is None:
            out_groups = int(out.shape[0])
        if not _is_device(out):
            flags |= N.OUT_HOST
        n = C.c_int32(0)
        rc = self._lib.sdbe_ingest(self._h, _addr(src), n_packets, _addr(out), out_groups, flags, C.byref(n))
        if rc == N.ERR_CAPACITY and auto:  # n holds the number of groups the batch ships
            out_groups = n.value
            out = self._group_out(out_groups, framed)
            rc = self._lib.sdbe_ingest(self._h, _addr(src), n_packets, _addr(out), out_groups, flags, C.byref(n))
        N.check(rc, self._h)
        return (out[:n.value] if isinstance(out, np.ndarray) else out), n.value

    def ingest_reform_state(self) -> N.ReformState:
        st = N.ReformState()
        N.check(self._lib.sdbe_ingest_reform_state(self._h, C.byref(st)), self._h)
        return st

    def ingest_flush(self, out=None, out_groups: int = 4, framed: bool = False):
        """Ship every open group that holds packets (end of stream)."""
        flags = N.OUT_FRAMED if framed else 0
        if out is None:
            out = self._group_out(out_groups, framed)
        if not _is_device(out):
            flags |= N.OUT_HOST
        n = C.c_int32(0)
        N.check(self._lib.sdbe_ingest_flush(self._h, _addr(out), out_groups, flags, C.byref(n)), self._h)
        return (out[:n.value] if isinstance(out, np.ndarray) else out), n.value

    def ingest_stats(self) -> dict:
        st = N.IngestStats()
        N.check(self._lib.sdbe_ingest_get_stats(self._h, C.byref(st)), self._h)
        return {k: int(getattr(st, k)) for k, _ in N.IngestStats._fields_ if k != "reserved"}

    def sync(self):
        N.check(self._lib.sdbe_sync(self._h), self._h)

    # -- profiling ------------------------------------------------------------
    def profile(self, enable: bool = True):
        N.check(self._lib.sdbe_profile_enable(self._h, int(bool(enable))), self._h)

    def read_profile(self) -> N.Profile:
        p = N.Profile()
        N.check(self._lib.sdbe_profile_read(self._h, C.byref(p)), self._h)
        return p

    @property
    def thresholds(self):
        st = self.get_state()
        return (st.threshold[0], st.threshold[1]), (st.offset[0], st.offset[1]), bool(st.thresholds_set)


def host_buffer(nbytes: int) -> np.ndarray:
    """Pinned host buffer (cudaMallocHost) as a uint8 numpy array; freed with the array's owner."""
    p = C.c_void_p()
    N.check(N.lib().sdbe_host_alloc(C.byref(p), nbytes))
    arr = np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(p.value))
    return _PinnedArray(arr, p.value)


class _PinnedArray(np.ndarray):
    def __new__(cls, arr, ptr):
        obj = arr.view(cls)
        obj._pinned_ptr = ptr
        return obj

    def __array_finalize__(self, obj):
        self._pinned_ptr = None  # views never own the allocation

    def free(self):
        if getattr(self, "_pinned_ptr", None):
            N.lib().sdbe_host_free(self._pinned_ptr)
            self._pinned_ptr = None


def process_multi(resamplers, items, framed: bool = False, stream=None, want_results: bool = False,
                  host: bool | None = None, asynchronous: bool = False):
    """One pass over several packet streams with shared FFT launches
    (``sdbe_process_multi``).

    ``items``: per resampler ``(packets, n_frames, b_zero, out)``; ``out`` may
    be None for host runs (allocated).  Buffers are all host (numpy) or all
    device (torch CUDA tensors).  Returns the outputs (and the per-stream
    ``GroupResult`` list when ``want_results``).  With ``asynchronous`` (host
    buffers, no results) the call returns once the work is queued; ``sync()``
    each resampler before reading the outputs or reusing the inputs.
    """
    n = len(resamplers)
    if n != len(items) or n == 0:
        raise ValueError("one item per resampler")
    lib = resamplers[0]._lib
    if host is None:
        host = not _is_device(items[0][0])
    flags = (N.IN_HOST | N.OUT_HOST) if host else 0
    if framed:
        flags |= N.OUT_FRAMED
    if asynchronous:
        flags |= N.ASYNC
    hs = (C.c_void_p * n)(*[r.handle.value for r in resamplers])
    descs = (N.StreamDesc * n)()
    outs = []
    keep = []
    for i, (r, (pk, n_frames, b_zero, out)) in enumerate(zip(resamplers, items)):
        need = r.output_bytes(n_frames, framed)
        if out is None:
            pkt = N.OUT_PKT_BYTES if framed else N.OUT_PKT_DATA_BYTES
            out = np.empty((2, need // (2 * pkt) if need else 0, pkt), np.uint8)
        if host:
            pk = np.ascontiguousarray(pk, dtype=np.uint8)
            keep.append(pk)
        descs[i].packets = _addr(pk)
        descs[i].n_packets = int(pk.shape[0]) if hasattr(pk, "shape") else 0
        descs[i].n_frames = n_frames
        descs[i].b_zero = b_zero
        descs[i].out = _addr(out)
        descs[i].out_bytes = _nbytes(out)
        outs.append(out)
    res = (N.Result * n)() if want_results else None
    st = C.c_void_p(stream) if isinstance(stream, int) else (
        C.c_void_p(stream.cuda_stream) if stream is not None else None)
    rc = lib.sdbe_process_multi(hs, descs, n, flags, st, res)
    N.check(rc, resamplers[0].handle)
    if not want_results:
        return outs
    return outs, [GroupResult(x.n_batches, x.n_out_packets, x.packets_accepted, x.packets_rejected,
                              x.frames_incomplete, x.carry_snapshots) for x in res]
