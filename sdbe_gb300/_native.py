"""ctypes binding of ``libsdbe.so`` (C ABI declared in ``include/sdbe.h``).

There is no fallback: if the library is missing or fails to load, importing
the product path raises, so a run without the CUDA stage cannot pass silently.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libsdbe.so")
SYNTH_PATH = os.path.join(_PKG, "libsdbe_synth.so")

# ---- constants mirrored from include/sdbe.h ----
OK, ERR_ARG, ERR_CUDA, ERR_STATE, ERR_CAPACITY, ERR_NOMEM = 0, -1, -2, -3, -4, -5
IN_PKT_BYTES = 1056
OUT_PKT_DATA_BYTES = 8192
OUT_PKT_BYTES = 8224
PKTS_PER_FRAME = 2048
SNAPSHOTS_PER_FRAME = 128
CHANNELS = 16384
BATCH_SNAPSHOTS = 143
PKTS_PER_BATCH = 128
FRAMES_PER_GROUP = 143
SAMPLES_PER_OUT_PKT = 32768
THRESH_FIRST_BATCH, THRESH_FIXED, THRESH_WINDOW = 0, 1, 2
THRESH_BLOCK = 16
MAP_APHIDS, MAP_MAR2015 = 0, 1
PRECISION_FP32, PRECISION_TC16, PRECISION_TC16_FAST = 0, 1, 2
STAGES_FUSED, STAGES_SPLIT = 1, 3
IN_HOST, OUT_HOST, OUT_FRAMED, SYNC, ASYNC, OUT_ALIGNED, IN_8PAC = 1, 2, 4, 8, 16, 32, 64
PAC8_BYTES = 8504
NOALLOC_MAX_SAMPLES = 134217728


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("trim_mhz", C.c_int32), ("max_frames", C.c_int32),
                ("threshold_mode", C.c_int32), ("pol1_uses_pol0_threshold", C.c_int32),
                ("channel_map", C.c_int32), ("wave_batches", C.c_int32), ("threshold_window", C.c_int32),
                ("precision", C.c_int32), ("stage_launches", C.c_int32), ("reserved", C.c_int32 * 6)]


class State(C.Structure):
    _fields_ = [("threshold", C.c_float * 2), ("offset", C.c_float * 2), ("thresholds_set", C.c_int32),
                ("carry_snapshots", C.c_int32), ("secs_inre", C.c_uint32), ("df_num_insec", C.c_uint32),
                ("edh_psn", C.c_uint64), ("ref_epoch", C.c_uint32), ("station_id", C.c_uint32),
                ("bdc_sideband", C.c_uint32), ("rx_sideband", C.c_uint32), ("reserved", C.c_int32 * 6)]


class Result(C.Structure):
    _fields_ = [("n_batches", C.c_int64), ("n_out_packets", C.c_int64), ("packets_accepted", C.c_int64),
                ("packets_rejected", C.c_int64), ("frames_incomplete", C.c_int64), ("carry_snapshots", C.c_int64)]


class Profile(C.Structure):
    _fields_ = [("launches", C.c_int64), ("stage_a_launches", C.c_int64), ("stage_a_snapshots", C.c_int64),
                ("stage_a_ms", C.c_double), ("stage_bc_launches", C.c_int64), ("stage_bc_chunks", C.c_int64),
                ("stage_bc_ms", C.c_double), ("fused_launches", C.c_int64), ("fused_chunks", C.c_int64),
                ("fused_ms", C.c_double), ("reserved", C.c_int64 * 1)]


class TimeTemplate(C.Structure):
    _fields_ = [("secs_inre", C.c_uint32), ("df_num_insec", C.c_uint32), ("ps_early", C.c_uint64),
                ("ref_epoch", C.c_uint32), ("reserved", C.c_uint32)]


class IngestStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("packets", "invalid", "before_start", "too_far_ahead", "used", "overflow",
                                         "groups_shipped", "groups_incomplete", "b_first")] + [
        ("reserved", C.c_int64 * 3)]


class ReformState(C.Structure):
    _fields_ = [("t0_sec", C.c_int32), ("t0_clk", C.c_int32), ("tprev_sec", C.c_int32), ("tprev_clk", C.c_int32),
                ("bprev", C.c_int64), ("marked_invalid", C.c_int64), ("slow_tiles", C.c_int64),
                ("reserved", C.c_int64)]


class StreamDesc(C.Structure):
    _fields_ = [("packets", C.c_void_p), ("n_packets", C.c_int64), ("n_frames", C.c_int32), ("reserved", C.c_int32),
                ("b_zero", C.c_uint64), ("out", C.c_void_p), ("out_bytes", C.c_int64)]


class SynthConfig(C.Structure):
    _fields_ = [("sigma", C.c_double), ("level", C.c_double), ("n_tones", C.c_int32),
                ("tone_channel", C.c_int32 * 8), ("tone_amp", C.c_double * 8), ("tone_phase", C.c_double * 8),
                ("burst_frac", C.c_double), ("burst_gain", C.c_double), ("channel_map", C.c_int32),
                ("secs0", C.c_uint32), ("ref_epoch", C.c_uint32), ("station", C.c_uint32)]


vp, i32, i64, u32, u64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_float

# name -> (restype, argtypes): every entry point of include/sdbe.h
SIGNATURES = {
    "sdbe_create": (C.c_int, [C.POINTER(Config), C.POINTER(vp)]),
    "sdbe_destroy": (C.c_int, [vp]),
    "sdbe_output_bytes": (i64, [vp, i32, u32]),
    "sdbe_process": (C.c_int, [vp, vp, i64, i32, u64, vp, i64, u32, vp, C.POINTER(Result)]),
    "sdbe_get_state": (C.c_int, [vp, C.POINTER(State)]),
    "sdbe_set_state": (C.c_int, [vp, C.POINTER(State)]),
    "sdbe_reset": (C.c_int, [vp]),
    "sdbe_sync": (C.c_int, [vp]),
    "sdbe_header_template": (C.c_int, [i32, i32, u32, C.POINTER(TimeTemplate)]),
    "sdbe_align_start": (C.c_int, [vp, C.POINTER(TimeTemplate)]),
    "sdbe_ingest": (C.c_int, [vp, vp, i64, vp, i64, u32, C.POINTER(i32)]),
    "sdbe_ingest_flush": (C.c_int, [vp, vp, i64, u32, C.POINTER(i32)]),
    "sdbe_ingest_get_stats": (C.c_int, [vp, C.POINTER(IngestStats)]),
    "sdbe_ingest_reform_state": (C.c_int, [vp, C.POINTER(ReformState)]),
    "sdbe_reform_init": (C.c_int, [C.POINTER(ReformState)]),
    "sdbe_unpack_8pac": (C.c_int, [vp, i64, vp, vp]),
    "sdbe_beng_reform": (C.c_int, [C.POINTER(ReformState), vp, i64, vp]),
    "sdbe_inverse_pfb": (C.c_int, [vp, vp, i64, i32, vp, vp]),
    "sdbe_process_multi": (C.c_int, [C.POINTER(vp), C.POINTER(StreamDesc), i32, u32, vp, C.POINTER(Result)]),
    "sdbe_profile_enable": (C.c_int, [vp, i32]),
    "sdbe_profile_read": (C.c_int, [vp, C.POINTER(Profile)]),
    "sdbe_last_error": (C.c_int, [vp, C.c_char_p, C.c_size_t]),
    "sdbe_host_alloc": (C.c_int, [C.POINTER(vp), C.c_size_t]),
    "sdbe_host_free": (C.c_int, [vp]),
    "sdbe_vdif_to_beng": (C.c_int, [vp, i64, u64, i32, i32, vp, vp, vp]),
    "sdbe_unpack": (C.c_int, [vp, i64, u64, i32, i32, vp, i64, i64, vp, vp, vp, vp]),
    "sdbe_fill_missing": (C.c_int, [vp, i32, i32, vp, i64, i64, vp]),
    "sdbe_beng_to_complex": (C.c_int, [vp, i64, vp, vp]),
    "sdbe_swarm_c2r": (C.c_int, [vp, vp, i64, vp, vp]),
    "sdbe_swarm_r2c": (C.c_int, [vp, vp, i64, vp, vp]),
    "sdbe_r2dbe_c2r": (C.c_int, [vp, vp, i64, i32, vp, vp]),
    "sdbe_resample_chunks": (C.c_int, [vp, vp, i64, vp, vp]),
    "sdbe_summary_stats": (C.c_int, [vp, i64, C.POINTER(C.c_double), vp]),
    "sdbe_summary_stats_noalloc": (C.c_int, [vp, i64, C.POINTER(C.c_double), vp]),
    "sdbe_quantize2bit": (C.c_int, [vp, vp, i64, f32, f32, vp]),
    "sdbe_vdif_headers": (C.c_int, [vp, i64, i64, u32, u32, u64, u32, u32, u32, u32, vp]),
    "sdbe_reorder_mar2015": (C.c_int, [vp, i32, vp, vp]),
    "sdbe_fp32_fma_rate": (C.c_int, [i32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "sdbe_test_tc_timeout": (C.c_int, [vp, i64]),
    "sdbe_test_ingest_accept": (C.c_int, [vp, vp, i64]),
}

SYNTH_SIGNATURES = {
    "sdbe_synth_packets": (i64, [vp, i64, u64, u64, C.POINTER(SynthConfig), C.c_int]),
    "sdbe_synth_impair": (i64, [vp, i64, vp, u64, C.c_double, C.c_double, i32]),
}


class SdbeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sdbe error {code}: {msg}")
        self.code = code


def _bind(path, sigs):
    if not os.path.exists(path):
        raise ImportError(f"{os.path.basename(path)} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = None
_synth = None


def lib():
    global _lib
    if _lib is None:
        _lib = _bind(LIB_PATH, SIGNATURES)
    return _lib


def synth_lib():
    global _synth
    if _synth is None:
        _synth = _bind(SYNTH_PATH, SYNTH_SIGNATURES)
    return _synth


def last_error(handle=None) -> str:
    buf = C.create_string_buffer(1024)
    lib().sdbe_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, handle=None):
    if rc != OK:
        raise SdbeError(rc, last_error(handle))
    return rc
