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
    assert L.hx_debug_fast_op_f64(7, 4, None, None, None) == hxlib.HX_ERR_ARG
    assert b"unknown fast-form operation" in L.hx_last_error()
    assert L.hx_debug_fast_op_f64(hxlib.HX_FAST_OP_SLOPE, 4, None, None, None) == hxlib.HX_ERR_ARG


def test_epilogue_arguments_checked_on_the_host(hxlib):
    """The advance epilogue needs an output, and a work buffer for the
    diagnostics; a malformed eta view is named.  Checked before any CUDA call
    (the pointers below are never dereferenced)."""
    L = hxlib.lib()
    fake = ctypes.c_void_p(0x1000)
    lv = hxlib.LevelF64()
    for f in ("h", "hu", "hv", "z", "n"):
        setattr(lv, f, ctypes.cast(fake, ctypes.POINTER(ctypes.c_double)))
    lv.pitch, lv.nx, lv.ny, lv.dx, lv.dy = 64, 64, 32, 1.0, 1.0
    out = [fake, fake, fake]
    rc = L.hx_level_advance_epilogue_f64(ctypes.byref(lv), 1e-3, *out, None, None, 0, None, None, None, None)
    assert rc == hxlib.HX_ERR_ARG and b"neither eta nor diagnostics" in L.hx_last_error()
    rc = L.hx_level_advance_epilogue_f64(ctypes.byref(lv), 1e-3, *out, None, None, 0, None, fake, None, None)
    assert rc == hxlib.HX_ERR_ARG and b"work buffer" in L.hx_last_error()
    A = hxlib.Array4F64()
    A.p = ctypes.cast(fake, ctypes.POINTER(ctypes.c_double))
    A.jstride, A.nstride, A.ncomp = 64, 64 * 32, 3
    A.lo[0], A.lo[1], A.hi[0], A.hi[1] = -2, -2, 61, 29
    vb = hxlib.Box()
    vb.lo[0], vb.lo[1], vb.hi[0], vb.hi[1] = 0, 0, 59, 27
    small = hxlib.Array4F64()
    small.p, small.jstride, small.nstride, small.ncomp = A.p, 10, 100, 1
    small.lo[0], small.lo[1], small.hi[0], small.hi[1] = 0, 0, 9, 9
    rc = L.hx_advance_box_hydrostatic_epilogue_f64(*(ctypes.byref(A),) * 5, vb, 1e-3, 1.0, 1.0, None, None, 0,
                                                   ctypes.byref(small), None, None, None)
    assert rc == hxlib.HX_ERR_ARG and b"eta_new" in L.hx_last_error()


def test_box_level_plan_checks_the_tiling(hxlib):
    """The multi-box planner (host code) accepts boxes that tile the domain and
    rejects overlaps, gaps and boxes outside it, with a message."""
    L = hxlib.lib()

    def boxes(spans):
        arr = (hxlib.LevelBoxF64 * len(spans))()
        for k, (x0, y0, x1, y1) in enumerate(spans):
            b = arr[k]
            for f in ("h", "hu", "hv", "h_alt", "hu_alt", "hv_alt", "z", "n"):
                setattr(b, f, 4096)  # never dereferenced by the planner
            b.pitch = x1 - x0 + 1
            b.lo[0], b.lo[1], b.hi[0], b.hi[1] = x0, y0, x1, y1
        return arr, len(spans)

    ok = [(0, 0, 31, 23), (32, 0, 63, 23), (0, 24, 63, 47)]
    assert L.hx_boxlevel_work_bytes(len(ok), boxes(ok)[0], 64, 48) > 0
    for bad in ([(0, 0, 40, 23), (32, 0, 63, 23), (0, 24, 63, 47)],   # overlap
                [(0, 0, 31, 23), (0, 24, 63, 47)],                    # gap
                [(0, 0, 63, 47), (64, 0, 70, 47)]):                   # outside
        arr, n = boxes(bad)
        assert L.hx_boxlevel_work_bytes(n, arr, 64, 48) == 0
        assert L.hx_last_error()


def test_adjoint_work_bytes_options(hxlib):
    """Face records add to the work buffer of checkpointed sweeps only; unknown
    option bits are refused."""
    L = hxlib.lib()
    rec = hxlib.HX_ADJ_FACE_RECORDS
    plain = L.hx_adjoint_work_bytes_f64(512, 512, 512, 2000, 45, 0)
    with_rec = L.hx_adjoint_work_bytes_f64(512, 512, 512, 2000, 45, rec)
    assert plain > 0 and with_rec - plain > 2 * 45 * 250 * 512 * 512
    assert L.hx_adjoint_work_bytes_f64(512, 512, 512, 2000, 0, rec) == L.hx_adjoint_work_bytes_f64(512, 512, 512, 2000, 0, 0)
    assert L.hx_adjoint_work_bytes_f64(512, 512, 512, 2000, -20, rec) == L.hx_adjoint_work_bytes_f64(512, 512, 512, 2000, -20, 0)
    assert L.hx_adjoint_work_bytes_f64(512, 512, 512, 2000, 45, 0x4000) == 0


def test_plotfile_arguments_checked_on_the_host(hxlib, tmp_path):
    """A box outside its level's domain is refused before any copy or file."""
    L = hxlib.lib()
    box = hxlib.PlotBoxF64()
    for f in ("h", "hu", "hv", "z", "n"):
        setattr(box, f, 4096)
    box.pitch = 16
    box.lo[0], box.lo[1], box.hi[0], box.hi[1] = 0, 0, 15, 15
    lev = hxlib.PlotLevelF64()
    lev.boxes = ctypes.pointer(box)
    lev.nboxes = 1
    lev.domain_lo[0], lev.domain_lo[1], lev.domain_hi[0], lev.domain_hi[1] = 0, 0, 14, 15
    lev.dx, lev.dy = 0.1, 0.1
    lo = (ctypes.c_double * 2)(0.0, 0.0)
    hi = (ctypes.c_double * 2)(1.0, 1.0)
    rc = L.hx_write_plotfile_f64(str(tmp_path / "plt").encode(), 3, 0.0, 1, ctypes.byref(lev), lo, hi, None)
    assert rc == hxlib.HX_ERR_ARG
    assert not (tmp_path / "plt00003").exists()


def test_host_run_row_bands(hxlib):
    """The row bands of hx_level_run_host_f64 cover every row once, in at most
    ten bands, with short first and last bands (~1/32 of the rows each) on
    tall levels; every band but the last holds at least the two rows its
    predecessor's flux differences read past their own (so a band's flux work
    waits for the rows it reads); every ny from 2 to 20000 and the bench's 8192."""
    L = hxlib.lib()
    st = (ctypes.c_int * 11)()
    assert L.hx_debug_host_bands(100, st, 9) == hxlib.HX_ERR_ARG
    assert L.hx_debug_host_bands(1, st, 10) == hxlib.HX_ERR_ARG
    for ny in list(range(2, 20001)) + [8192]:
        n = L.hx_debug_host_bands(ny, st, 10)
        assert 1 <= n <= 10, (ny, n)
        s = list(st[:n + 1])
        assert s[0] == 0 and s[-1] == ny and all(a < b for a, b in zip(s, s[1:])), (ny, s)
        assert all(b - a >= 2 for a, b in zip(s[:-2], s[1:-1])), (ny, s)
        if ny >= 1024:
            edge = -(-ny // 32)
            assert s[1] <= edge + 7 and ny - s[-2] <= edge + 7, (ny, s)
    n = L.hx_debug_host_bands(8192, st, 10)
    assert list(st[:n + 1]) == [0, 256, 1216, 2176, 3136, 4096, 5056, 6016, 6976, 7936, 8192]
