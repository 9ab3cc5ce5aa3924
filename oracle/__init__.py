"""CPU oracle for the HydroEXA per-level advance (TEST INFRASTRUCTURE ONLY).

This package is what the CUDA path is compared against.  Only tests/,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import it; the
product package ``hydroexa_gb300`` never does.

``build()`` compiles ``hx_oracle_capi.cpp`` (a scalar C++ restatement of the
reference's arithmetic, see ``hx_oracle.hpp`` for the file:line map) into
``oracle/_build/libhx_oracle.so`` with ``-O2 -ffp-contract=off -fopenmp``.
``build_ref()`` compiles the reference's own header-only point kernels from the
reference source tree into ``oracle/_ref/libhx_ref.so`` (only where that tree
exists; used to pin the oracle and to regenerate ``tests/golden``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "libhx_oracle.so"
REF_LIB_PATH = HERE / "_ref" / "libhx_ref.so"

METHOD_CLASSIC = 0
METHOD_HYDROSTATIC = 1
LIMITER_FLOAT_ABS = 0
LIMITER_INT_ABS = 1


def build(force: bool = False) -> Path:
    """Compile the oracle shared library (a few seconds)."""
    src = [HERE / "hx_oracle_capi.cpp", HERE / "hx_oracle.hpp"]
    if LIB_PATH.exists() and not force:
        mt = LIB_PATH.stat().st_mtime
        if all(s.stat().st_mtime <= mt for s in src):
            return LIB_PATH
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-std=c++17", str(HERE / "hx_oracle_capi.cpp"), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_root() -> Path | None:
    """The reference source tree, as the recipe ``build_ref.sh`` locates it
    ($HX_REFERENCE_ROOT or the recipe's default), or None where there is none."""
    r = subprocess.run(["sh", str(HERE / "build_ref.sh"), "--root"], capture_output=True, text=True)
    return Path(r.stdout.strip()) if r.returncode == 0 and r.stdout.strip() else None


REF_OUTPUTS = ["libhx_ref.so"] + ["libhx_ref_level_%s%s.so" % (a, p) for a in ("", "fabs_") for p in ("f64", "f32")]


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference's point kernels and per-box drivers (oracle/build_ref.sh)
    if the reference tree is present; a no-op when every output is newer than
    the recipe, the AMReX stand-in and the driver harness."""
    if reference_root() is None:
        return None
    outs = [HERE / "_ref" / n for n in REF_OUTPUTS]
    srcs = [HERE / "build_ref.sh", *HERE.glob("ref_*.cpp"), *HERE.glob("ref_*.h"), *(HERE / "ref_shim").glob("*")]
    if not force and all(o.exists() for o in outs):
        oldest = min(o.stat().st_mtime for o in outs)
        if all(p.stat().st_mtime <= oldest for p in srcs):
            return REF_LIB_PATH
    subprocess.run(["sh", str(HERE / "build_ref.sh")], check=True, stdout=subprocess.DEVNULL)
    return REF_LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        _lib = ctypes.CDLL(str(LIB_PATH))
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _suffix(dtype) -> str:
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def _real(dtype):
    return ctypes.c_double if np.dtype(dtype) == np.float64 else ctypes.c_float


def set_threads(n: int) -> None:
    lib().hxo_set_threads(ctypes.c_int(int(n)))


def max_threads() -> int:
    return int(lib().hxo_max_threads())


def _bc(lo, hi):
    return (np.ascontiguousarray(lo, dtype=np.int32), np.ascontiguousarray(hi, dtype=np.int32))


def roe_hydrostatic_points(states: np.ndarray, normals: np.ndarray) -> np.ndarray:
    """states (n, 6) = (hi, hui, hvi, hj, huj, hvj); normals (n, 2) -> F (n, 3)."""
    s = np.ascontiguousarray(states)
    nr = np.ascontiguousarray(normals, dtype=s.dtype)
    out = np.empty((s.shape[0], 3), dtype=s.dtype)
    getattr(lib(), "hxo_roe_hydrostatic_points_" + _suffix(s.dtype))(
        ctypes.c_long(s.shape[0]), _ptr(s), _ptr(nr), _ptr(out))
    return out


def roe_classic_points(states: np.ndarray, aux: np.ndarray):
    """states (n, 10); aux (n, 4) = (dt, dx, nx, ny) -> (F, S_minus, S_plus), each (n, 3)."""
    s = np.ascontiguousarray(states)
    a = np.ascontiguousarray(aux, dtype=s.dtype)
    F = np.empty((s.shape[0], 3), dtype=s.dtype)
    Sm = np.empty_like(F)
    Sp = np.empty_like(F)
    getattr(lib(), "hxo_roe_classic_points_" + _suffix(s.dtype))(
        ctypes.c_long(s.shape[0]), _ptr(s), _ptr(a), _ptr(F), _ptr(Sm), _ptr(Sp))
    return F, Sm, Sp


def van_leer_slope_points(q3: np.ndarray, mode: int = LIMITER_FLOAT_ABS) -> np.ndarray:
    q = np.ascontiguousarray(q3)
    out = np.empty(q.shape[0], dtype=q.dtype)
    getattr(lib(), "hxo_van_leer_slope_points_" + _suffix(q.dtype))(
        ctypes.c_long(q.shape[0]), _ptr(q), ctypes.c_int(mode), _ptr(out))
    return out


class Level:
    """Single-box level: planes (ny, nx), x fastest, with the inputs-file BC codes."""

    def __init__(self, nx, ny, dx, dy, bc_lo=(0, 0), bc_hi=(0, 0)):
        self.nx, self.ny, self.dx, self.dy = int(nx), int(ny), float(dx), float(dy)
        self.bc_lo, self.bc_hi = _bc(bc_lo, bc_hi)


def advance(level: Level, method: int, h, hu, hv, z, n, dt, mode=LIMITER_FLOAT_ABS, faces=False):
    """One advance by dt; returns (h, hu, hv) [, face arrays]."""
    dtype = np.asarray(h).dtype
    R = _real(dtype)
    arrs = [np.ascontiguousarray(a, dtype=dtype) for a in (h, hu, hv, z, n)]
    out = [np.empty_like(arrs[0]) for _ in range(3)]
    L = level
    sfx = _suffix(dtype)
    base = [ctypes.c_int(L.nx), ctypes.c_int(L.ny), R(L.dx), R(L.dy), _ptr(L.bc_lo), _ptr(L.bc_hi)]
    base += [_ptr(a) for a in arrs] + [R(dt)] + [_ptr(o) for o in out]
    nxf, nyf = (L.nx + 1) * L.ny, L.nx * (L.ny + 1)
    if method == METHOD_HYDROSTATIC:
        if not faces:
            getattr(lib(), "hxo_advance_hydrostatic_" + sfx)(*base, ctypes.c_int(mode))
            return tuple(out)
        fx = [np.empty((3, L.ny, L.nx + 1), dtype=dtype) for _ in range(2)]
        fy = [np.empty((3, L.ny + 1, L.nx), dtype=dtype) for _ in range(2)]
        getattr(lib(), "hxo_advance_hydrostatic_faces_" + sfx)(
            *base, ctypes.c_int(mode), _ptr(fx[0]), _ptr(fx[1]), _ptr(fy[0]), _ptr(fy[1]))
        return tuple(out), {"FLx": fx[0], "FRx": fx[1], "FLy": fy[0], "FRy": fy[1]}
    if not faces:
        getattr(lib(), "hxo_advance_classic_" + sfx)(*base)
        return tuple(out)
    fx = [np.empty((3, L.ny, L.nx + 1), dtype=dtype) for _ in range(3)]
    fy = [np.empty((3, L.ny + 1, L.nx), dtype=dtype) for _ in range(3)]
    getattr(lib(), "hxo_advance_classic_faces_" + sfx)(*base, *[_ptr(a) for a in fx + fy])
    del nxf, nyf
    return tuple(out), {"Fx": fx[0], "Smx": fx[1], "Spx": fx[2], "Fy": fy[0], "Smy": fy[1], "Spy": fy[2]}


def compute_dt(level: Level, h, hu, hv, z):
    """(min per-cell CFL bound, max(|u|,|v|)) over the level, before the CFL factor."""
    dtype = np.asarray(h).dtype
    R = _real(dtype)
    arrs = [np.ascontiguousarray(a, dtype=dtype) for a in (h, hu, hv, z)]
    mn, mx = R(), R()
    getattr(lib(), "hxo_compute_dt_" + _suffix(dtype))(
        ctypes.c_int(level.nx), ctypes.c_int(level.ny), R(level.dx), R(level.dy),
        *[_ptr(a) for a in arrs], ctypes.byref(mn), ctypes.byref(mx))
    return float(mn.value), float(mx.value)


def run(level: Level, method: int, h, hu, hv, z, n, nsteps, cfl, mode=LIMITER_FLOAT_ABS, copy=True):
    """nsteps of the single-level time loop; returns (h, hu, hv, t, dt_last, status).

    The loop runs on copies of h, hu, hv, or with ``copy=False`` in place on
    the given arrays (C-contiguous, of one floating dtype)."""
    dtype = np.asarray(h).dtype
    R = _real(dtype)
    if copy:
        st = [np.array(a, dtype=dtype, copy=True, order="C") for a in (h, hu, hv)]
    else:
        st = [h, hu, hv]
        assert all(a.dtype == dtype and a.flags.c_contiguous for a in st), "in-place run needs C-contiguous planes"
    zz = np.ascontiguousarray(z, dtype=dtype)
    nn = np.ascontiguousarray(n, dtype=dtype)
    t, dtl = R(), R()
    rc = getattr(lib(), "hxo_run_" + _suffix(dtype))(
        ctypes.c_int(method), ctypes.c_int(level.nx), ctypes.c_int(level.ny), R(level.dx), R(level.dy),
        _ptr(level.bc_lo), _ptr(level.bc_hi), *[_ptr(a) for a in st], _ptr(zz), _ptr(nn),
        ctypes.c_int(nsteps), R(cfl), ctypes.c_int(mode), ctypes.byref(t), ctypes.byref(dtl))
    return st[0], st[1], st[2], float(t.value), float(dtl.value), int(rc)


def tag_cells(variant, U, T, tags, valid_lo, valid_hi, dx, dy, time, h_th, u_th, z_th, set_value=2):
    """Tag the valid box.  U (3, ny, nx) and T (2, ny, nx) carry one ghost ring:
    array index [c, j+1, i+1] holds cell (i, j); tags (ny, nx) covers the same
    grown box and is modified in place."""
    dtype = U.dtype
    R = _real(dtype)
    U = np.ascontiguousarray(U)
    T = np.ascontiguousarray(T, dtype=dtype)
    assert tags.dtype == np.int8 and tags.flags.c_contiguous
    _, uy, ux = U.shape
    _, ty, tx = T.shape
    gy, gx = tags.shape
    getattr(lib(), "hxo_tag_cells_" + _suffix(dtype))(
        ctypes.c_int(variant),
        _ptr(U), ctypes.c_longlong(ux), ctypes.c_longlong(ux * uy), ctypes.c_int(-1), ctypes.c_int(-1),
        _ptr(T), ctypes.c_longlong(tx), ctypes.c_longlong(tx * ty), ctypes.c_int(-1), ctypes.c_int(-1),
        _ptr(tags), ctypes.c_longlong(gx), ctypes.c_int(-1), ctypes.c_int(-1),
        ctypes.c_int(valid_lo[0]), ctypes.c_int(valid_lo[1]), ctypes.c_int(valid_hi[0]), ctypes.c_int(valid_hi[1]),
        R(dx), R(dy), R(time), R(h_th), R(u_th), R(z_th), ctypes.c_byte(set_value))
    return tags


def masked_average_down(fine: np.ndarray, rx: int, ry: int, fine_volume: float, nodata: float = -9999.0):
    """fine (ncomp, nyf, nxf) -> crse (ncomp, nyf//ry, nxf//rx)."""
    f = np.ascontiguousarray(fine)
    nc, nyf, nxf = f.shape
    nxc, nyc = nxf // rx, nyf // ry
    c = np.empty((nc, nyc, nxc), dtype=f.dtype)
    R = _real(f.dtype)
    getattr(lib(), "hxo_masked_average_down_" + _suffix(f.dtype))(
        _ptr(f), ctypes.c_longlong(nxf), ctypes.c_longlong(nxf * nyf), ctypes.c_int(0), ctypes.c_int(0),
        _ptr(c), ctypes.c_longlong(nxc), ctypes.c_longlong(nxc * nyc), ctypes.c_int(0), ctypes.c_int(0),
        ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(nxc - 1), ctypes.c_int(nyc - 1),
        ctypes.c_int(nc), ctypes.c_int(rx), ctypes.c_int(ry), R(fine_volume), R(nodata))
    return c


def average_down(fine: np.ndarray, rx: int, ry: int):
    """Conservative restriction (amrex::average_down as called by
    src/state/AmrMeshState_AMR.cpp:838-844): fine (ncomp, nyf, nxf) ->
    crse (ncomp, nyf//ry, nxf//rx)."""
    f = np.ascontiguousarray(fine)
    nc, nyf, nxf = f.shape
    nxc, nyc = nxf // rx, nyf // ry
    c = np.empty((nc, nyc, nxc), dtype=f.dtype)
    getattr(lib(), "hxo_average_down_" + _suffix(f.dtype))(
        _ptr(f), ctypes.c_longlong(nxf), ctypes.c_longlong(nxf * nyf), ctypes.c_int(0), ctypes.c_int(0),
        _ptr(c), ctypes.c_longlong(nxc), ctypes.c_longlong(nxc * nyc), ctypes.c_int(0), ctypes.c_int(0),
        ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(nxc - 1), ctypes.c_int(nyc - 1),
        ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(nc), ctypes.c_int(rx), ctypes.c_int(ry))
    return c


def mass_diagnostics(h, hu, hv, n, dx: float, dy: float) -> np.ndarray:
    """{mass, x-momentum, y-momentum, kinetic energy, min h} of one box
    (src/state/AmrMeshState_Utils.cpp:267-298); planes (ny, nx) of one dtype."""
    planes = [np.ascontiguousarray(a) for a in (h, hu, hv, n)]
    ny, nx = planes[0].shape
    R = _real(planes[0].dtype)
    out = np.zeros(5, dtype=np.float64)
    getattr(lib(), "hxo_mass_diagnostics_" + _suffix(planes[0].dtype))(
        ctypes.c_int(nx), ctypes.c_int(ny), ctypes.c_longlong(nx), *(_ptr(a) for a in planes), R(dx), R(dy),
        out.ctypes.data_as(ctypes.c_void_p))
    return out


def derive_eta(h, z) -> np.ndarray:
    """eta = h + z (src/state/AmrMeshState_AMR.cpp:217-219)."""
    h = np.ascontiguousarray(h)
    z = np.ascontiguousarray(z)
    eta = np.empty_like(h)
    getattr(lib(), "hxo_derive_eta_" + _suffix(h.dtype))(ctypes.c_longlong(h.size), _ptr(h), _ptr(z), _ptr(eta))
    return eta


def reflux_mean(FL, FR):
    """The hydrostatic solver's flux-register flux, 0.5 FL + 0.5 FR
    (src/solvers/HydrostaticRoe.cpp:619-626, MultiFab::LinComb); the halves
    are exact, so the sum is rounded once in any evaluation order."""
    FL, FR = np.asarray(FL), np.asarray(FR)
    return FL.dtype.type(0.5) * FL + FR.dtype.type(0.5) * FR


def roe_reflux_select(d, F, Sm, Sp, face_lo, mask=None, mask_lo=None, grid=None):
    """Side-selected effective fluxes of the classic solver's flux registers
    (src/solvers/Roe.cpp:369-388 for D- and D+, :447-566 for the selection)
    on the nodal faces of direction d.  F, Sm, Sp: (3, nyf, nxf) with face
    (i, j) at [:, j - face_lo[1], i - face_lo[0]].  mask: (ny, nx) ints with
    cell (i, j) at [j - mask_lo[1], i - mask_lo[0]] (0 coarse, 1 covered);
    grid: ((lo_x, lo_y), (hi_x, hi_y)).  Returns (flux_crse, flux_fine)."""
    F, Sm, Sp = (np.asarray(a) for a in (F, Sm, Sp))
    one = F.dtype.type(1.0)
    Dm = one * F + F.dtype.type(-1.0) * Sm
    Dp = one * F + one * Sp
    _, nyf, nxf = F.shape
    I, J = np.meshgrid(np.arange(nxf) + face_lo[0], np.arange(nyf) + face_lo[1])
    zero = np.zeros_like(F)
    fc = ff = None
    if mask is not None:
        m = np.asarray(mask)
        li, lj = (I - 1, J) if d == 0 else (I, J - 1)
        left = m[lj - mask_lo[1], li - mask_lo[0]]
        right = m[J - mask_lo[1], I - mask_lo[0]]
        fc = np.where(((left == 0) & (right == 1))[None], Dp, np.where(((left == 1) & (right == 0))[None], Dm, zero))
    if grid is not None:
        face_idx = I if d == 0 else J
        i_low, i_high = grid[0][d], grid[1][d] + 1
        ff = np.where((face_idx == i_low)[None], Dm, np.where((face_idx == i_high)[None], Dp, zero))
    return fc, ff


# --- reference kernels compiled verbatim (only where the reference tree exists) ---

_ref = None


def ref_lib() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        if not REF_LIB_PATH.exists():
            if build_ref() is None:
                raise FileNotFoundError("reference tree not available to build oracle/_ref")
        _ref = ctypes.CDLL(str(REF_LIB_PATH))
    return _ref


def ref_roe_hydrostatic_points(states, normals):
    s = np.ascontiguousarray(states)
    nr = np.ascontiguousarray(normals, dtype=s.dtype)
    out = np.empty((s.shape[0], 3), dtype=s.dtype)
    getattr(ref_lib(), "hxref_roe_hydrostatic_" + _suffix(s.dtype))(
        ctypes.c_long(s.shape[0]), _ptr(s), _ptr(nr), _ptr(out))
    return out


def ref_roe_classic_points(states, aux):
    s = np.ascontiguousarray(states)
    a = np.ascontiguousarray(aux, dtype=s.dtype)
    F = np.empty((s.shape[0], 3), dtype=s.dtype)
    Sm = np.empty_like(F)
    Sp = np.empty_like(F)
    getattr(ref_lib(), "hxref_roe_classic_" + _suffix(s.dtype))(
        ctypes.c_long(s.shape[0]), _ptr(s), _ptr(a), _ptr(F), _ptr(Sm), _ptr(Sp))
    return F, Sm, Sp


def ref_masked_average_down(fine, rx, ry, fine_volume, nodata=-9999.0):
    f = np.ascontiguousarray(fine)
    nc, nyf, nxf = f.shape
    c = np.empty((nc, nyf // ry, nxf // rx), dtype=f.dtype)
    R = _real(f.dtype)
    getattr(ref_lib(), "hxref_masked_avgdown_" + _suffix(f.dtype))(
        ctypes.c_int(nxf), ctypes.c_int(nyf), ctypes.c_int(nc), _ptr(f), ctypes.c_int(rx), ctypes.c_int(ry),
        R(fine_volume), R(nodata), _ptr(c))
    return c


# --- the reference's per-box drivers compiled verbatim (ref_level.cpp) ---------

_ref_level = {}


def ref_level_lib(dtype=np.float64, float_abs: bool = True) -> ctypes.CDLL:
    """The reference's solver drivers at one level (oracle/_ref).  float_abs
    picks the build whose limiter abs() is the floating one; otherwise C's
    int abs(int), what the host headers alone give."""
    key = (np.dtype(dtype).name, bool(float_abs))
    if key not in _ref_level:
        name = "libhx_ref_level_%s%s.so" % ("fabs_" if float_abs else "", _suffix(dtype))
        path = HERE / "_ref" / name
        if not path.exists():
            if build_ref() is None:
                raise FileNotFoundError("reference tree not available to build oracle/_ref")
        _ref_level[key] = ctypes.CDLL(str(path))
    return _ref_level[key]


def _ref_call(fn, *args):
    err = ctypes.create_string_buffer(256)
    rc = fn(*args, err)
    if rc == 2:
        raise RuntimeError("reference driver: " + err.value.decode(errors="replace"))
    return rc


def ref_run(level: Level, method: int, h, hu, hv, z, n, nsteps, cfl, float_abs=True):
    """The reference's single-level time loop: (h, hu, hv, t, dt_last, status)."""
    dtype = np.asarray(h).dtype
    R = _real(dtype)
    st = [np.array(a, dtype=dtype, copy=True, order="C") for a in (h, hu, hv)]
    zz, nn = (np.ascontiguousarray(a, dtype=dtype) for a in (z, n))
    t, dtl = R(), R()
    lib_ = ref_level_lib(dtype, float_abs)
    rc = _ref_call(getattr(lib_, "hxref_level_run_" + _suffix(dtype)), ctypes.c_int(method), ctypes.c_int(level.nx),
                   ctypes.c_int(level.ny), R(level.dx), R(level.dy), _ptr(level.bc_lo), _ptr(level.bc_hi),
                   *[_ptr(a) for a in st], _ptr(zz), _ptr(nn), ctypes.c_int(nsteps), R(cfl), ctypes.byref(t),
                   ctypes.byref(dtl))
    return st[0], st[1], st[2], float(t.value), float(dtl.value), int(rc)


def ref_advance(level: Level, method: int, h, hu, hv, z, n, dt, float_abs=True):
    """One level advance of the reference by dt: (h, hu, hv)."""
    dtype = np.asarray(h).dtype
    R = _real(dtype)
    arrs = [np.ascontiguousarray(a, dtype=dtype) for a in (h, hu, hv, z, n)]
    out = [np.empty_like(arrs[0]) for _ in range(3)]
    lib_ = ref_level_lib(dtype, float_abs)
    _ref_call(getattr(lib_, "hxref_level_advance_" + _suffix(dtype)), ctypes.c_int(method), ctypes.c_int(level.nx),
              ctypes.c_int(level.ny), R(level.dx), R(level.dy), _ptr(level.bc_lo), _ptr(level.bc_hi),
              *[_ptr(a) for a in arrs], R(dt), *[_ptr(o) for o in out])
    return tuple(out)


def ref_compute_dt(level: Level, method: int, h, hu, hv, z, cfl=1.0, float_abs=True):
    """The reference's compute_dt_level (cfl applied); None when it aborts on a collapsed dt."""
    dtype = np.asarray(h).dtype
    R = _real(dtype)
    arrs = [np.ascontiguousarray(a, dtype=dtype) for a in (h, hu, hv, z)]
    out = R()
    lib_ = ref_level_lib(dtype, float_abs)
    rc = _ref_call(getattr(lib_, "hxref_level_dt_" + _suffix(dtype)), ctypes.c_int(method), ctypes.c_int(level.nx),
                   ctypes.c_int(level.ny), R(level.dx), R(level.dy), *[_ptr(a) for a in arrs], R(cfl),
                   ctypes.byref(out))
    return None if rc == 1 else float(out.value)


def ref_tag_cells(method: int, Ug, Tg, dx, dy, time, h_th, u_th, z_th):
    """The reference's tag_cells on a box whose state Ug (3, ny+2, nx+2) and
    terrain Tg (2, ny+2, nx+2) carry one ghost cell; returns (ny, nx) int8 tags
    (2 = TagBox::SET, else 0)."""
    U = np.ascontiguousarray(Ug)
    T = np.ascontiguousarray(Tg, dtype=U.dtype)
    ny, nx = U.shape[1] - 2, U.shape[2] - 2
    R = _real(U.dtype)
    tags = np.zeros((ny, nx), dtype=np.int8)
    lib_ = ref_level_lib(U.dtype, True)
    _ref_call(getattr(lib_, "hxref_tag_cells_" + _suffix(U.dtype)), ctypes.c_int(method), ctypes.c_int(nx),
              ctypes.c_int(ny), R(dx), R(dy), _ptr(U), _ptr(T), R(time), R(h_th), R(u_th), R(z_th), _ptr(tags))
    return tags
