"""ctypes binding of the C ABI in ``include/hydroexa_gb300.h``.

This is the reference-facing boundary: every compute call made from Python
goes through these entry points with plain device pointers, sizes and a CUDA
stream handle.  Loading fails loudly if ``libhydroexa_gb300.so`` has not been
built (``hydroexa_gb300.build.build()``); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, Structure, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_long, c_uint32, \
    c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libhydroexa_gb300.so"

HX_OK = 0
HX_ERR_ARG = -1
HX_ERR_LAUNCH = -2
HX_ERR_CUDA = -3
HX_STATUS_DT_COLLAPSE = 1
HX_STATUS_NAN = 2
HX_STATUS_STAGING_TIMEOUT = 4
HX_ARITH_EXACT = 0
HX_ARITH_FAST = 1
HX_ADJ_FACE_RECORDS = 0x100
HX_METHOD_ROE = 0
HX_METHOD_HYDROSTATIC_ROE = 1
# boundary codes of the level calls: 0 the reference's wall, 1 open, 2 a closed wall (see the C header)
HX_BC_REFLECTIVE = 0
HX_BC_TRANSMISSIVE = 1
HX_BC_CLOSED_WALL = 2
HX_FAST_OP_RCP = 0
HX_FAST_OP_SQRT = 1
HX_FAST_OP_SLOPE = 2
HX_FAST_OP_RCP_FAITHFUL = 3
HX_FAST_OP_SQRT_FAITHFUL = 4
HX_FAST_OP_RCBRT = 5


class HxError(RuntimeError):
    pass


def _array4(real):
    class A4(Structure):
        _fields_ = [("p", POINTER(real)), ("jstride", c_int64), ("nstride", c_int64), ("lo", c_int32 * 2),
                    ("hi", c_int32 * 2), ("ncomp", c_int32)]
    return A4


Array4F64 = _array4(c_double)
Array4F32 = _array4(c_float)
Array4I8 = _array4(ctypes.c_byte)
Array4I32 = _array4(c_int32)


class Box(Structure):
    _fields_ = [("lo", c_int32 * 2), ("hi", c_int32 * 2)]


def _level(real):
    class Lv(Structure):
        _fields_ = [("h", POINTER(real)), ("hu", POINTER(real)), ("hv", POINTER(real)), ("z", POINTER(real)),
                    ("n", POINTER(real)), ("pitch", c_int64), ("nx", c_int32), ("ny", c_int32), ("dx", real),
                    ("dy", real), ("bc_lo", c_int32 * 2), ("bc_hi", c_int32 * 2)]
    return Lv


LevelF64 = _level(c_double)
LevelF32 = _level(c_float)


class LevelBoxF64(Structure):
    _fields_ = [("h", c_void_p), ("hu", c_void_p), ("hv", c_void_p), ("h_alt", c_void_p), ("hu_alt", c_void_p),
                ("hv_alt", c_void_p), ("z", c_void_p), ("n", c_void_p), ("pitch", c_int64), ("lo", c_int32 * 2),
                ("hi", c_int32 * 2)]


class PlotBoxF64(Structure):
    _fields_ = [("h", c_void_p), ("hu", c_void_p), ("hv", c_void_p), ("z", c_void_p), ("n", c_void_p),
                ("pitch", c_int64), ("lo", c_int32 * 2), ("hi", c_int32 * 2)]


class PlotLevelF64(Structure):
    _fields_ = [("boxes", POINTER(PlotBoxF64)), ("nboxes", c_int32), ("domain_lo", c_int32 * 2),
                ("domain_hi", c_int32 * 2), ("dx", c_double), ("dy", c_double), ("ref_ratio", c_int32),
                ("istep", c_int32)]


class EnsembleMemberF64(Structure):
    _fields_ = [("level", LevelF64), ("h_alt", c_void_p), ("hu_alt", c_void_p), ("hv_alt", c_void_p),
                ("tile_shape", c_int32)]


HX_TILE_32x8 = 0
HX_TILE_16x16 = 1
HX_TILE_64x4 = 2
HX_TILE_32x32 = 3

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise HxError(f"{LIB_PATH} is missing: build it with hydroexa_gb300.build.build()")
        L = ctypes.CDLL(str(LIB_PATH))
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    L.hx_version.restype = c_char_p
    L.hx_last_error.restype = c_char_p
    L.hx_launch_count.restype = c_uint64
    L.hx_dt_accum_bytes.restype = c_int64
    L.hx_level_run_work_bytes.restype = c_int64
    for sfx, real, A4, Lv in (("f64", c_double, Array4F64, LevelF64), ("f32", c_float, Array4F32, LevelF32)):
        P4 = POINTER(A4)
        getattr(L, f"hx_advance_box_hydrostatic_{sfx}").argtypes = [P4, P4, P4, P4, P4, Box, real, real, real, P4, P4,
                                                                   c_void_p, c_void_p, c_int, c_void_p]
        getattr(L, f"hx_advance_box_roe_{sfx}").argtypes = [P4, P4, P4, P4, Box, real, real, real, P4, P4, P4,
                                                           c_void_p, c_void_p, c_int, c_void_p]
        getattr(L, f"hx_advance_box_hydrostatic_reflux_{sfx}").argtypes = [P4, P4, P4, P4, P4, Box, real, real, real,
                                                                          P4, c_void_p, c_void_p, c_int, c_void_p]
        getattr(L, f"hx_advance_box_roe_reflux_{sfx}").argtypes = [P4, P4, P4, P4, Box, real, real, real,
                                                                  POINTER(Array4I32), Box, P4, P4, c_void_p, c_void_p,
                                                                  c_int, c_void_p]
        getattr(L, f"hx_dt_reduce_box_{sfx}").argtypes = [P4, P4, Box, real, real, c_void_p, c_void_p]
        getattr(L, f"hx_tag_box_{sfx}").argtypes = [c_int, P4, P4, POINTER(Array4I8), Box, real, real, real, real,
                                                   real, real, ctypes.c_byte, c_void_p]
        getattr(L, f"hx_masked_average_down_box_{sfx}").argtypes = [P4, P4, Box, c_int, c_int, c_int, c_int, c_int,
                                                                    real, real, c_void_p]
        getattr(L, f"hx_average_down_box_{sfx}").argtypes = [P4, P4, Box, c_int, c_int, c_int, c_int, c_int,
                                                             c_void_p]
        getattr(L, f"hx_level_advance_{sfx}").argtypes = [c_int, POINTER(Lv), real, c_void_p, c_void_p, c_void_p,
                                                         c_void_p, c_void_p, c_int, c_void_p]
        getattr(L, f"hx_advance_box_hydrostatic_epilogue_{sfx}").argtypes = [P4, P4, P4, P4, P4, Box, real, real,
                                                                            real, c_void_p, c_void_p, c_int, P4,
                                                                            c_void_p, c_void_p, c_void_p]
        getattr(L, f"hx_level_advance_epilogue_{sfx}").argtypes = [POINTER(Lv), real, c_void_p, c_void_p, c_void_p,
                                                                  c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                                                                  c_void_p, c_void_p]
        getattr(L, f"hx_level_dt_reduce_{sfx}").argtypes = [POINTER(Lv), c_void_p, c_void_p]
        getattr(L, f"hx_level_run_{sfx}").argtypes = [c_int, POINTER(Lv), c_void_p, c_void_p, c_void_p, c_int, real,
                                                     c_void_p, c_void_p, c_void_p, c_int, POINTER(c_int), c_void_p]
        getattr(L, f"hx_dt_accum_read_{sfx}").argtypes = [c_void_p, POINTER(real), POINTER(real), c_void_p]
        getattr(L, f"hx_debug_roe_points_{sfx}").argtypes = [c_int, c_int, c_long, c_void_p, c_void_p, c_void_p,
                                                            c_void_p]
    L.hx_debug_rcp_f64.argtypes = [c_long, c_void_p, c_void_p, c_void_p]
    L.hx_debug_sqrt_f64.argtypes = [c_long, c_void_p, c_void_p, c_void_p]
    L.hx_debug_fast_op_f64.argtypes = [c_int, c_long, c_void_p, c_void_p, c_void_p]
    L.hx_debug_staging_extra_bytes.argtypes = [ctypes.c_uint]
    L.hx_debug_host_bands.argtypes = [c_int, c_void_p, c_int]
    L.hx_debug_host_split_frac.restype = c_double
    L.hx_debug_host_split_frac.argtypes = []
    L.hx_status_clear.argtypes = [c_void_p, c_void_p]
    L.hx_status_read.argtypes = [c_void_p, c_void_p]
    L.hx_dt_accum_reset.argtypes = [c_void_p, c_void_p]
    L.hx_level_run_host_f64.argtypes = [c_int, c_int, c_int, c_double, c_double, POINTER(c_int32), POINTER(c_int32),
                                        c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_double, c_int,
                                        POINTER(c_double), c_void_p]
    L.hx_host_cache_release.restype = None
    L.hx_ensemble_work_bytes.restype = c_int64
    L.hx_ensemble_work_bytes.argtypes = [c_int]
    L.hx_ensemble_tiles.argtypes = [c_int, POINTER(EnsembleMemberF64), POINTER(c_int64)]
    L.hx_ensemble_run_f64.argtypes = [c_int, POINTER(EnsembleMemberF64), c_int, c_double, c_void_p, c_void_p,
                                      c_void_p, c_int, c_int, POINTER(c_int), c_void_p]
    L.hx_derive_eta_box_f64.argtypes = [POINTER(Array4F64), POINTER(Array4F64), POINTER(Array4F64), Box, c_void_p]
    L.hx_derive_eta_box_f32.argtypes = [POINTER(Array4F32), POINTER(Array4F32), POINTER(Array4F32), Box, c_void_p]
    L.hx_diagnostics_work_bytes.restype = c_int64
    L.hx_diagnostics_work_bytes.argtypes = [Box]
    L.hx_diagnostics_box_f64.argtypes = [POINTER(Array4F64), POINTER(Array4F64), Box, c_double, c_double, c_void_p,
                                         c_void_p, c_void_p]
    L.hx_diagnostics_box_f32.argtypes = [POINTER(Array4F32), POINTER(Array4F32), Box, c_float, c_float, c_void_p,
                                         c_void_p, c_void_p]
    L.hx_level_diagnostics_f64.argtypes = [POINTER(LevelF64), c_void_p, c_void_p, c_void_p]
    L.hx_measure_fp64_rate.argtypes = [POINTER(c_double), POINTER(c_double), c_void_p]
    L.hx_write_plotfile_f64.argtypes = [ctypes.c_char_p, c_int, c_double, c_int, POINTER(PlotLevelF64),
                                        POINTER(c_double), POINTER(c_double), c_void_p]
    L.hx_boxlevel_work_bytes.restype = c_int64
    L.hx_boxlevel_work_bytes.argtypes = [c_int, POINTER(LevelBoxF64), c_int, c_int]
    L.hx_boxlevel_run_f64.argtypes = [c_int, POINTER(LevelBoxF64), c_int, c_int, c_double, c_double,
                                      POINTER(c_int32), POINTER(c_int32), c_int, c_double, c_int, c_void_p, c_void_p,
                                      c_void_p, POINTER(c_int), c_void_p]
    L.hx_adjoint_work_bytes_f64.restype = c_int64
    L.hx_adjoint_work_bytes_f64.argtypes = [c_int, c_int, c_int64, c_int, c_int, c_int]
    L.hx_adjoint_recompute_steps.restype = c_int64
    L.hx_adjoint_recompute_steps.argtypes = [c_int, c_int]
    L.hx_adjoint_forward_f64.argtypes = [POINTER(LevelF64), c_int, c_double, c_int, c_void_p, c_void_p, c_int,
                                         c_int, c_void_p, c_void_p, c_void_p]
    L.hx_adjoint_reverse_f64.argtypes = [POINTER(LevelF64), c_int, c_double, c_int, c_void_p, c_void_p, c_double,
                                         c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
    L.hx_adjoint_step_f64.argtypes = [POINTER(LevelF64), c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p]
    L.hx_level_tangent_f64.argtypes = [POINTER(LevelF64), c_double, c_double, c_void_p, c_void_p, c_void_p,
                                       c_void_p]
    L.hx_level_run_static_f64.argtypes = [c_int, POINTER(LevelF64), c_int, c_double, c_void_p, c_void_p, c_int,
                                          c_void_p]


def check(rc: int, what: str = "") -> int:
    """Raise HxError for a negative return code, else pass it through."""
    if rc < 0:
        msg = lib().hx_last_error().decode(errors="replace")
        raise HxError(f"{what}: error {rc}: {msg}")
    return rc


def fp64_rates() -> tuple:
    """(DFMA, FFMA) thread instructions per second measured on the current GPU."""
    d, f = c_double(), c_double()
    check(lib().hx_measure_fp64_rate(ctypes.byref(d), ctypes.byref(f), None), "hx_measure_fp64_rate")
    return d.value, f.value


def version() -> str:
    return lib().hx_version().decode()


def launch_count() -> int:
    return int(lib().hx_launch_count())


# Every exported symbol the header declares (checked by the CPU test suite).
EXPORTED = [
    "hx_version", "hx_last_error", "hx_launch_count", "hx_status_clear", "hx_status_read", "hx_dt_accum_bytes",
    "hx_dt_accum_reset", "hx_dt_accum_read_f64", "hx_dt_accum_read_f32",
    "hx_advance_box_hydrostatic_f64", "hx_advance_box_hydrostatic_f32", "hx_advance_box_roe_f64",
    "hx_advance_box_roe_f32", "hx_advance_box_hydrostatic_reflux_f64", "hx_advance_box_hydrostatic_reflux_f32",
    "hx_advance_box_roe_reflux_f64", "hx_advance_box_roe_reflux_f32", "hx_dt_reduce_box_f64", "hx_dt_reduce_box_f32", "hx_tag_box_f64", "hx_tag_box_f32",
    "hx_masked_average_down_box_f64", "hx_masked_average_down_box_f32", "hx_average_down_box_f64",
    "hx_average_down_box_f32", "hx_derive_eta_box_f64",
    "hx_derive_eta_box_f32", "hx_diagnostics_work_bytes", "hx_diagnostics_box_f64", "hx_diagnostics_box_f32",
    "hx_level_diagnostics_f64", "hx_advance_box_hydrostatic_epilogue_f64", "hx_advance_box_hydrostatic_epilogue_f32",
    "hx_level_advance_epilogue_f64", "hx_level_advance_epilogue_f32", "hx_measure_fp64_rate", "hx_boxlevel_work_bytes", "hx_boxlevel_run_f64", "hx_write_plotfile_f64",
    "hx_level_advance_f64",
    "hx_level_advance_f32", "hx_level_dt_reduce_f64", "hx_level_dt_reduce_f32", "hx_level_run_work_bytes",
    "hx_level_run_f64", "hx_level_run_f32", "hx_level_run_host_f64", "hx_host_cache_release",
    "hx_debug_roe_points_f64", "hx_debug_roe_points_f32", "hx_debug_rcp_f64", "hx_debug_sqrt_f64", "hx_debug_fast_op_f64", "hx_debug_staging_extra_bytes",
    "hx_debug_host_bands", "hx_debug_host_split_frac",
    "hx_level_run_static_f64",
    "hx_ensemble_work_bytes", "hx_ensemble_tiles", "hx_ensemble_run_f64",
    "hx_adjoint_work_bytes_f64", "hx_adjoint_recompute_steps", "hx_adjoint_forward_f64", "hx_adjoint_reverse_f64", "hx_adjoint_step_f64",
    "hx_level_tangent_f64",
]
HX_STATIC_RUN_MAX_CELLS = 262144
