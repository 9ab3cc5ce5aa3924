"""The C-ABI library loads and exports every entry point its header declares
(no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = ""
    for h in (ROOT / "include").glob("*.h"):
        text += h.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "hx_level_run_f64" in syms and "hx_advance_box_hydrostatic_f64" in syms
    assert len(syms) >= 25


def test_library_exports_every_declared_symbol(hxlib):
    lib = ctypes.CDLL(str(hxlib.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(hxlib.EXPORTED) == declared_symbols()


def test_version_and_error_string(hxlib):
    assert "sm_103a" in hxlib.version()
    assert hxlib.launch_count() >= 0


def test_argument_errors_need_no_gpu(hxlib):
    """Host-side argument checks fire before any CUDA call."""
    L = hxlib.lib()
    b = hxlib.Box()
    b.lo[0], b.lo[1], b.hi[0], b.hi[1] = 0, 0, -1, 5
    rc = L.hx_dt_reduce_box_f64(None, None, b, 1.0, 1.0, None, None)
    assert rc == hxlib.HX_ERR_ARG
    assert b"empty box" in L.hx_last_error()
    lv = hxlib.LevelF64()
    rc = L.hx_level_run_f64(1, ctypes.byref(lv), None, None, None, 1, 0.5, None, None, None, 0, None, None)
    assert rc == hxlib.HX_ERR_ARG
