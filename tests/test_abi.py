"""CPU checks of the C ABI: the library builds, loads and exports every symbol
declared in include/sdbe.h, and the Python binding agrees with the header."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "sdbe.h")


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sdbe_[a-z0-9_]+)\s*\(", text)))


def _header_defines():
    out = {}
    for name, val in re.findall(r"#define\s+(SDBE_[A-Z0-9_]+)\s+(-?\d+)u?\b", open(HEADER).read()):
        out[name] = int(val)
    return out


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import _native

    return _native


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(built.LIB_PATH)
    names = _declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(built):
    assert set(_declared_functions()) == set(built.SIGNATURES)


def test_struct_layouts(built):
    assert C.sizeof(built.Config) == 16 * 4
    assert C.sizeof(built.State) == 4 * 2 * 2 + 4 * 4 + 8 + 4 * 4 + 6 * 4
    assert C.sizeof(built.Result) == 6 * 8
    assert C.sizeof(built.ReformState) == 48
    assert C.sizeof(built.IngestStats) == 12 * 8


def test_constants_match_header(built):
    d = _header_defines()
    assert d["SDBE_IN_PKT_BYTES"] == built.IN_PKT_BYTES
    assert d["SDBE_OUT_PKT_BYTES"] == built.OUT_PKT_BYTES
    assert d["SDBE_OUT_PKT_DATA_BYTES"] == built.OUT_PKT_DATA_BYTES
    assert d["SDBE_BATCH_SNAPSHOTS"] == built.BATCH_SNAPSHOTS
    assert d["SDBE_OK"] == built.OK and d["SDBE_ERR_CAPACITY"] == built.ERR_CAPACITY
    assert d["SDBE_IN_HOST"] == built.IN_HOST and d["SDBE_OUT_FRAMED"] == built.OUT_FRAMED
    assert d["SDBE_IN_8PAC"] == built.IN_8PAC and d["SDBE_PAC8_BYTES"] == built.PAC8_BYTES


def test_error_paths_without_gpu(built):
    """Argument checks run before any CUDA call and report through sdbe_last_error."""
    lib = built.lib()
    h = C.c_void_p()
    assert lib.sdbe_create(None, C.byref(h)) == built.ERR_ARG
    cfg = built.Config()
    cfg.max_frames = 0
    assert lib.sdbe_create(C.byref(cfg), C.byref(h)) == built.ERR_ARG
    assert "max_frames" in built.last_error()
    cfg.max_frames = 143
    cfg.trim_mhz = 241
    assert lib.sdbe_create(C.byref(cfg), C.byref(h)) == built.ERR_ARG
    assert lib.sdbe_quantize2bit(None, None, 17, 1.0, 0.0, None) == built.ERR_ARG
    assert lib.sdbe_reorder_mar2015(None, 1, None, None) == built.ERR_ARG
    assert lib.sdbe_process(None, None, 0, 0, 0, None, 0, 0, None, None) == built.ERR_ARG
    assert lib.sdbe_unpack_8pac(None, 1, None, None) == built.ERR_ARG
    assert lib.sdbe_unpack_8pac(8, 1, 12, None) == built.ERR_ARG          # misaligned
    assert "aligned" in built.last_error()
    assert lib.sdbe_beng_reform(None, None, 0, None) == built.ERR_ARG
    st = built.ReformState()
    st.bprev = 77
    assert lib.sdbe_reform_init(C.byref(st)) == built.OK
    assert (st.t0_sec, st.t0_clk, st.tprev_sec, st.tprev_clk, st.bprev, st.slow_tiles) == (-1, -1, -1, -1, -1, 0)
    assert lib.sdbe_beng_reform(C.byref(st), None, 0, None) == built.OK   # nothing to do


@pytest.mark.parametrize("field,value,word", [
    ("threshold_mode", 7, "threshold_mode"),
    ("threshold_window", -1, "threshold_window"),
    ("channel_map", 5, "channel_map"),
    ("wave_batches", 65, "wave_batches"),
    ("precision", 9, "precision"),
    ("stage_launches", 2, "stage_launches"),
    ("device", -1, "device"),
])
def test_create_rejects_each_bad_config_field(built, field, value, word):
    """sdbe_create checks every field of the configuration before it touches
    a device: one bad field gives SDBE_ERR_ARG, no handle, and a message that
    names it."""
    lib = built.lib()
    cfg = built.Config()
    cfg.max_frames = 143
    cfg.trim_mhz = 150
    setattr(cfg, field, value)
    h = C.c_void_p(12345)
    assert lib.sdbe_create(C.byref(cfg), C.byref(h)) == built.ERR_ARG
    assert h.value is None
    assert word in built.last_error() or (field == "device" and "CUDA device" in built.last_error())
    assert lib.sdbe_test_ingest_accept(None, None, 0) == built.ERR_ARG


def test_header_template_matches_oracle(built):
    """sdbe_header_template (host-only) == fill_vdif_header_template restated."""
    from oracle import sdbe_oracle as O

    lib = built.lib()
    cases = [(1000, 0), (1000, 1), (1000, 262143), (1000, 262144), (1000, 262145), (7, 285999999),
             (7, 285737856), (12345, 143000000), (12345, 2288 * 1000 + 17)]
    rng = __import__("numpy").random.default_rng(9)
    cases += [(int(s), int(c)) for s, c in zip(rng.integers(0, 2**20, 50), rng.integers(0, 286000000, 50))]
    for sec, clk in cases:
        t = built.TimeTemplate()
        assert lib.sdbe_header_template(sec, clk, 30, C.byref(t)) == built.OK
        ref = O.header_template(sec, clk, 30)
        assert (t.secs_inre, t.df_num_insec, t.ps_early, t.ref_epoch) == ref, (sec, clk)
