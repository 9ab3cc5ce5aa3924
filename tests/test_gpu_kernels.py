"""Device point solvers against the golden vectors, tagging and the NODATA
restriction against the oracle (bit-exact), the per-box drop-in forms against
the level form, and device status reporting."""
import ctypes
from pathlib import Path

import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.level import DtAccum, Level, Status, array4, box

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
EXACT, FAST = capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST


def dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def run_points(hxlib, method, arith, states, aux, dev):
    st = torch.from_numpy(np.ascontiguousarray(states)).to(dev)
    ax = torch.from_numpy(np.ascontiguousarray(aux)).to(dev)
    n = states.shape[0]
    out = torch.empty((3 if method == 0 else 1) * n * 3, dtype=st.dtype, device=dev)
    sfx = "f64" if st.dtype == torch.float64 else "f32"
    hxlib.check(getattr(hxlib.lib(), f"hx_debug_roe_points_{sfx}")(method, arith, n, dptr(st), dptr(ax), dptr(out),
                                                                    None), "points")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def term_scale(states):
    """Magnitude of the terms a face flux is made of (h u^2 + g h^2 / 2 + |h u|
    on both sides): fluxes that cancel to ~0 are measured against it."""
    s = np.asarray(states, dtype=np.float64)
    thrust = 0.0
    if s.shape[1] == 10:  # classic states also carry the bed: add the thrust g h |dz|
        thrust = 9.81 * (s[:, 0] + s[:, 5]) * np.abs(s[:, 8] - s[:, 3])
        s = s[:, [0, 1, 2, 5, 6, 7]]
    hi, hj = s[:, 0], s[:, 3]
    qi = np.abs(s[:, 1]) + np.abs(s[:, 2])
    qj = np.abs(s[:, 4]) + np.abs(s[:, 5])
    ui = np.where(hi > 0, qi / np.where(hi > 0, hi, 1), 0)
    uj = np.where(hj > 0, qj / np.where(hj > 0, hj, 1), 0)
    return (qi * ui + qj * uj + 4.905 * (hi ** 2 + hj ** 2) + qi + qj + thrust + 1e-300)[:, None]


def test_hydrostatic_points_golden(cuda, hxlib):
    g = np.load(GOLD / "roe_hydrostatic_f64.npz")
    got = run_points(hxlib, 1, EXACT, g["states"], g["normals"], cuda).reshape(-1, 3)
    assert np.array_equal(got, g["F"])
    fast = run_points(hxlib, 1, FAST, g["states"], g["normals"], cuda).reshape(-1, 3)
    assert (np.abs(fast - g["F"]) / term_scale(g["states"])).max() <= 1e-13


def test_classic_points_golden(cuda, hxlib):
    """Bit-equal where the face has no Manning roughness; with roughness the
    friction term goes through cbrt, where CUDA and glibc may differ by an ulp."""
    g = np.load(GOLD / "roe_classic_f64.npz")
    got = run_points(hxlib, 0, EXACT, g["states"], g["aux"], cuda).reshape(3, -1, 3)
    smooth = (g["states"][:, 4] + g["states"][:, 9]) == 0
    sc = term_scale(g["states"])
    for k, name in enumerate(("F", "Sm", "Sp")):
        assert np.array_equal(got[k][smooth], g[name][smooth]), name
        assert (np.abs(got[k] - g[name]) / sc).max() <= 1e-14, name
    fast = run_points(hxlib, 0, FAST, g["states"], g["aux"], cuda).reshape(3, -1, 3)
    # friction on a nearly dry face makes the sources large next to the flux terms
    sc = sc + np.abs(np.stack([g["F"], g["Sm"], g["Sp"]])).max(axis=(0, 2))[:, None]
    for k, name in enumerate(("F", "Sm", "Sp")):
        assert (np.abs(fast[k] - g[name]) / sc).max() <= 1e-12, name


def test_points_f32_golden(cuda, hxlib):
    g = np.load(GOLD / "roe_hydrostatic_f32.npz")
    got = run_points(hxlib, 1, FAST, g["states"], g["normals"], cuda).reshape(-1, 3)
    # the reference's SINGLE build promotes double literals; the FP32 kernel stays in float
    assert (np.abs(got - g["F"]) / term_scale(g["states"])).max() <= 5e-5


def ghosted(a, g=1):
    """(c, ny, nx) -> (c, ny+2g, nx+2g) with edge-copied ghosts."""
    return np.pad(a, ((0, 0), (g, g), (g, g)), mode="edge")


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("time", [0.0, 0.5])
def test_tags_bit_exact(cuda, hxlib, oracle_lib, method, time):
    case = workloads.fractal_dam_break(70, 45, seed=31, amplitude=2.0, nodata_frac=0.15)
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    h, hu, hv, *_ = oracle_lib.run(L, 1, case.h, case.hu, case.hv, case.z, case.n, 8, case.cfl)
    U = ghosted(np.stack([h, hu, hv]))
    T = ghosted(np.stack([case.z, case.n]))
    rng = np.random.default_rng(1)
    tags0 = (rng.random(U.shape[1:]) < 0.05).astype(np.int8)  # pre-existing tags stay
    for th in ((0.5, 0.5, 2.0), (5.0, 20.0, 50.0)):
        ref = oracle_lib.tag_cells(method, U, T, tags0.copy(), (0, 0), (g.nx - 1, g.ny - 1), g.dx, g.dy, time, *th)
        Ut = torch.from_numpy(U).to(cuda)
        Tt = torch.from_numpy(T).to(cuda)
        Gt = torch.from_numpy(tags0.copy()).to(cuda)
        rc = hxlib.lib().hx_tag_box_f64(method, ctypes.byref(array4(Ut, (-1, -1))), ctypes.byref(array4(Tt, (-1, -1))),
                                        ctypes.byref(array4(Gt, (-1, -1))), box((0, 0), (g.nx - 1, g.ny - 1)), g.dx,
                                        g.dy, time, *th, 2, None)
        hxlib.check(rc, "tag")
        got = Gt.cpu().numpy()
        assert np.array_equal(got, ref)
        assert (ref == 2).sum() > 10


@pytest.mark.parametrize("r", [2, 4])
def test_masked_average_down_bit_exact(cuda, hxlib, oracle_lib, r):
    g = np.load(GOLD / "masked_avgdown_f64.npz")
    fine = torch.from_numpy(g["fine"]).to(cuda)
    nc, nyf, nxf = g["fine"].shape
    crse = torch.full((nc, nyf // r, nxf // r), 123.0, dtype=torch.float64, device=cuda)
    rc = hxlib.lib().hx_masked_average_down_box_f64(ctypes.byref(array4(fine)), ctypes.byref(array4(crse)),
                                                    box((0, 0), (nxf // r - 1, nyf // r - 1)), 0, 0, nc, r, r,
                                                    float(g["fine_volume"]), -9999.0, None)
    hxlib.check(rc, "mavg")
    got = crse.cpu().numpy()
    assert np.array_equal(got, g[f"crse_r{r}"], equal_nan=True)


@pytest.mark.parametrize("rx,ry,dtype", [(2, 2, torch.float64), (4, 4, torch.float64), (2, 4, torch.float64),
                                         (3, 3, torch.float64), (2, 2, torch.float32)])
def test_average_down_bit_exact(cuda, hxlib, oracle_lib, rx, ry, dtype):
    """The state restriction (amrex::average_down of AverageDownTo) equals the
    oracle bit for bit on a coarse sub-box of an offset view with ghosts,
    components 1..2 into 0..1; cells outside the box are left alone."""
    rng = np.random.default_rng(7 * rx + ry)
    npd = np.float64 if dtype == torch.float64 else np.float32
    nxc, nyc = 21, 17
    fine = rng.uniform(-2.0, 3.0, size=(3, nyc * ry, nxc * rx)).astype(npd)
    ref = oracle_lib.average_down(fine[1:], rx, ry)
    # fine view indexed from (0,0); coarse view with one ghost, lo = (-1,-1)
    F = torch.from_numpy(fine).to(cuda)
    C = torch.full((2, nyc + 2, nxc + 2), 123.0, dtype=dtype, device=cuda)
    sfx = "f64" if dtype == torch.float64 else "f32"
    cv = array4(C, lo=(-1, -1))
    rc = getattr(hxlib.lib(), f"hx_average_down_box_{sfx}")(ctypes.byref(array4(F)), ctypes.byref(cv),
                                                             box((2, 3), (nxc - 1, nyc - 2)), 1, 0, 2, rx, ry, None)
    hxlib.check(rc, "avgdown")
    got = C.cpu().numpy()
    assert np.array_equal(got[:, 4:nyc, 3:nxc + 1], ref[:, 3:nyc - 1, 2:nxc])
    inner = np.ones_like(got, dtype=bool)
    inner[:, 4:nyc, 3:nxc + 1] = False
    assert (got[inner] == 123.0).all()
    bad = getattr(hxlib.lib(), f"hx_average_down_box_{sfx}")(ctypes.byref(array4(F)), ctypes.byref(cv),
                                                              box((0, 0), (nxc, nyc - 1)), 1, 0, 2, rx, ry, None)
    assert bad == capi.HX_ERR_ARG


def test_box_form_matches_level_form(cuda, hxlib, oracle_lib):
    """The AMReX drop-in (ghost-filled per-box views, four boxes) equals the
    single-box level form, including the FL/FR face arrays the reflux needs."""
    case = workloads.fractal_dam_break(64, 48, seed=41, amplitude=1.5, nodata_frac=0.1)
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    h, hu, hv, *_ = oracle_lib.run(L, 1, case.h, case.hu, case.hv, case.z, case.n, 5, case.cfl)
    mn, _ = oracle_lib.compute_dt(L, h, hu, hv, case.z)
    dt = mn * case.cfl
    (rh, rhu, rhv), F = oracle_lib.advance(L, 1, h, hu, hv, case.z, case.n, dt, faces=True)
    # ghost-filled arrays (2 ghosts) exactly as FillPatch + HydroPhysBC leave them: the momenta are filled with
    # BC-record offset 0 (include/utils/FillPatchUtils.H:128-129), hu with the depth's record, hv with hu's
    G = 2
    eta = h + case.z
    ext = lambda a, mode_x, mode_y: _bc_ext(a, G, mode_x, mode_y)
    eta_e = ext(eta, "even", "even")
    hu_e = ext(hu, "even", "even")
    hv_e = ext(hv, "odd", "even")
    z_e = ext(case.z, "edge", "edge")
    n_e = ext(case.n, "edge", "edge")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    Eta = dev(eta_e[None])
    Uext = dev(np.stack([np.zeros_like(hu_e), hu_e, hv_e]))
    Text = dev(np.stack([z_e, n_e]))
    Uold = dev(np.stack([h, hu, hv]))
    Unew = torch.zeros_like(Uold)
    FLx = torch.zeros((3, g.ny, g.nx + 1), dtype=torch.float64, device=cuda)
    FRx = torch.zeros_like(FLx)
    FLy = torch.zeros((3, g.ny + 1, g.nx), dtype=torch.float64, device=cuda)
    FRy = torch.zeros_like(FLy)
    acc = DtAccum(cuda)
    for (x0, x1), (y0, y1) in [((0, 29), (0, 20)), ((30, 63), (0, 20)), ((0, 29), (21, 47)), ((30, 63), (21, 47))]:
        FLarr = (capi.Array4F64 * 2)(array4(FLx), array4(FLy))
        FRarr = (capi.Array4F64 * 2)(array4(FRx), array4(FRy))
        rc = hxlib.lib().hx_advance_box_hydrostatic_f64(
            ctypes.byref(array4(Eta, (-G, -G))), ctypes.byref(array4(Uext, (-G, -G))),
            ctypes.byref(array4(Text, (-G, -G))), ctypes.byref(array4(Uold)), ctypes.byref(array4(Unew)),
            box((x0, y0), (x1, y1)), dt, g.dx, g.dy, FLarr, FRarr, acc.ptr, None, EXACT, None)
        hxlib.check(rc, "box")
    got = Unew.cpu().numpy()
    assert np.array_equal(got[0], rh) and np.array_equal(got[1], rhu) and np.array_equal(got[2], rhv)
    for name, t in (("FLx", FLx), ("FRx", FRx), ("FLy", FLy), ("FRy", FRy)):
        assert np.array_equal(t.cpu().numpy(), F[name]), name
    mn2, mx2 = oracle_lib.compute_dt(L, rh, rhu, rhv, case.z)
    assert acc.read() == (mn2, mx2)


def _bc_ext(a, G, mx, my):
    """Ghost extension of a (ny, nx) plane: 'even' mirror, 'odd' mirror with
    sign flip, 'edge' copy -- x rule then y rule (corners unused)."""
    ny, nx = a.shape
    out = np.zeros((ny + 2 * G, nx + 2 * G))
    out[G:G + ny, G:G + nx] = a
    for k in range(1, G + 1):
        for side in (0, 1):
            src = (k - 1) if side == 0 else nx - k
            dst = G - k if side == 0 else G + nx - 1 + k
            col = a[:, 0 if side == 0 else nx - 1] if mx == "edge" else a[:, src]
            out[G:G + ny, dst] = -col if mx == "odd" else col
    for k in range(1, G + 1):
        for side in (0, 1):
            src = (k - 1) if side == 0 else ny - k
            dst = G - k if side == 0 else G + ny - 1 + k
            row = out[G if side == 0 else G + ny - 1, :] if my == "edge" else out[G + src, :]
            out[dst, :] = -row if my == "odd" else row
    return out


def test_dt_collapse_sets_status(cuda):
    """A velocity explosion collapses the CFL bound below 1e-12: the loop stops
    and reports HX_STATUS_DT_COLLAPSE (the reference aborts,
    HydrostaticRoe.cpp:77-80) -- made on the host, no GPU fault involved."""
    case = workloads.dam_break(32, 32, nsteps=3)
    case.hu[5, 5] = 1.0e15
    lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
    st = lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 3, case.cfl, arith=EXACT)
    assert st & capi.HX_STATUS_DT_COLLAPSE
    assert lev.time.item() == 0.0  # no step advanced the clock


def test_nan_input_sets_status(cuda):
    case = workloads.dam_break(32, 32)
    case.h[7, 9] = np.nan
    lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
    out = lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, 1e-4, arith=FAST)
    torch.cuda.synchronize()
    assert lev.status.read() & capi.HX_STATUS_NAN
    assert torch.isnan(out).any()


def _box_case(cuda, oracle_lib, method, seed):
    case = workloads.fractal_dam_break(64, 48, seed=seed, amplitude=1.5, nodata_frac=0.1 if method else 0.0)
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    h, hu, hv, *_ = oracle_lib.run(L, method, case.h, case.hu, case.hv, case.z, case.n, 5, case.cfl)
    mn, _ = oracle_lib.compute_dt(L, h, hu, hv, case.z)
    return case, L, (h, hu, hv), mn * case.cfl


def test_hydrostatic_reflux_flux_from_the_advance(cuda, hxlib, oracle_lib):
    """The fused reflux output equals 0.5 FL + 0.5 FR of the reference's face
    arrays, bit for bit, and the update is unchanged."""
    case, L, (h, hu, hv), dt = _box_case(cuda, oracle_lib, 1, 41)
    g = case.geom
    (rh, rhu, rhv), F = oracle_lib.advance(L, 1, h, hu, hv, case.z, case.n, dt, faces=True)
    G = 2
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    Eta = dev(_bc_ext(h + case.z, G, "even", "even")[None])
    Uext = dev(np.stack([np.zeros((g.ny + 2 * G, g.nx + 2 * G)), _bc_ext(hu, G, "even", "even"),
                         _bc_ext(hv, G, "odd", "even")]))  # the reference FillPatch's records (offset 0)
    Text = dev(np.stack([_bc_ext(case.z, G, "edge", "edge"), _bc_ext(case.n, G, "edge", "edge")]))
    Uold = dev(np.stack([h, hu, hv]))
    Unew = torch.zeros_like(Uold)
    Fx = torch.zeros((3, g.ny, g.nx + 1), dtype=torch.float64, device=cuda)
    Fy = torch.zeros((3, g.ny + 1, g.nx), dtype=torch.float64, device=cuda)
    for (x0, x1), (y0, y1) in [((0, 29), (0, 20)), ((30, 63), (0, 20)), ((0, 29), (21, 47)), ((30, 63), (21, 47))]:
        Freg = (capi.Array4F64 * 2)(array4(Fx), array4(Fy))
        rc = hxlib.lib().hx_advance_box_hydrostatic_reflux_f64(
            ctypes.byref(array4(Eta, (-G, -G))), ctypes.byref(array4(Uext, (-G, -G))),
            ctypes.byref(array4(Text, (-G, -G))), ctypes.byref(array4(Uold)), ctypes.byref(array4(Unew)),
            box((x0, y0), (x1, y1)), dt, g.dx, g.dy, Freg, None, None, EXACT, None)
        hxlib.check(rc, "reflux box")
    got = Unew.cpu().numpy()
    assert np.array_equal(got[0], rh) and np.array_equal(got[1], rhu) and np.array_equal(got[2], rhv)
    assert np.array_equal(Fx.cpu().numpy(), oracle_lib.reflux_mean(F["FLx"], F["FRx"]))
    assert np.array_equal(Fy.cpu().numpy(), oracle_lib.reflux_mean(F["FLy"], F["FRy"]))


def test_classic_box_form_and_reflux_selection(cuda, hxlib, oracle_lib):
    """Classic box form (FillPatch-style ghosts) equals the level form with its
    F / S- / S+ faces; the reflux variant writes the reference's side-selected
    D+ / D- for a coarse register (fine mask) and a fine register (grid box)."""
    case, L, (h, hu, hv), dt = _box_case(cuda, oracle_lib, 0, 43)
    g = case.geom
    (rh, rhu, rhv), F = oracle_lib.advance(L, 0, h, hu, hv, case.z, case.n, dt, faces=True)
    G = 1
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)

    def inputs():
        Eta = dev(_bc_ext(h + case.z, G, "even", "even")[None])
        Uold = dev(np.stack([np.zeros((g.ny + 2 * G, g.nx + 2 * G)), _bc_ext(hu, G, "even", "even"),
                             _bc_ext(hv, G, "odd", "even")]))  # the reference FillPatch's records (offset 0)
        T = dev(np.stack([_bc_ext(case.z, G, "edge", "edge"), _bc_ext(case.n, G, "edge", "edge")]))
        return Eta, Uold, T

    vb = box((0, 0), (g.nx - 1, g.ny - 1))
    faces = lambda: [torch.zeros((3, g.ny, g.nx + 1), dtype=torch.float64, device=cuda),
                     torch.zeros((3, g.ny + 1, g.nx), dtype=torch.float64, device=cuda)]
    Eta, Uold, T = inputs()
    Unew = torch.zeros((3, g.ny, g.nx), dtype=torch.float64, device=cuda)
    Ff, Smf, Spf = faces(), faces(), faces()
    arr = lambda fs: (capi.Array4F64 * 2)(array4(fs[0]), array4(fs[1]))
    rc = hxlib.lib().hx_advance_box_roe_f64(ctypes.byref(array4(Eta, (-G, -G))), ctypes.byref(array4(Uold, (-G, -G))),
                                            ctypes.byref(array4(T, (-G, -G))), ctypes.byref(array4(Unew)), vb, dt,
                                            g.dx, g.dy, arr(Ff), arr(Smf), arr(Spf), None, None, EXACT, None)
    hxlib.check(rc, "classic box")
    got = Unew.cpu().numpy()
    assert np.array_equal(got[0], rh) and np.array_equal(got[1], rhu) and np.array_equal(got[2], rhv)
    for d, sfx in ((0, "x"), (1, "y")):
        assert np.array_equal(Ff[d].cpu().numpy(), F["F" + sfx])
        assert np.array_equal(Smf[d].cpu().numpy(), F["Sm" + sfx])
        assert np.array_equal(Spf[d].cpu().numpy(), F["Sp" + sfx])
    # reflux: a covered rectangle (and part of the ghost ring) for the coarse register, a grid box for the fine one
    mask = np.zeros((g.ny + 2 * G, g.nx + 2 * G), dtype=np.int32)
    mask[10:25, 20:45] = 1
    mask[30:, :4] = 1
    Mk = dev(mask)
    grid = ((0, 0), (g.nx - 1, g.ny - 1))
    Eta, Uold, T = inputs()
    Unew2 = torch.zeros_like(Unew)
    fc, ff = faces(), faces()
    ma = capi.Array4I32()
    ma.p = ctypes.cast(ctypes.c_void_p(Mk.data_ptr()), ctypes.POINTER(ctypes.c_int32))
    ma.jstride, ma.nstride = g.nx + 2 * G, (g.nx + 2 * G) * (g.ny + 2 * G)
    ma.lo[0], ma.lo[1], ma.hi[0], ma.hi[1], ma.ncomp = -G, -G, g.nx - 1 + G, g.ny - 1 + G, 1
    rc = hxlib.lib().hx_advance_box_roe_reflux_f64(ctypes.byref(array4(Eta, (-G, -G))),
                                                   ctypes.byref(array4(Uold, (-G, -G))),
                                                   ctypes.byref(array4(T, (-G, -G))), ctypes.byref(array4(Unew2)),
                                                   vb, dt, g.dx, g.dy, ctypes.byref(ma), box(*grid), arr(fc), arr(ff),
                                                   None, None, EXACT, None)
    hxlib.check(rc, "classic reflux box")
    assert torch.equal(Unew2, Unew)
    for d, sfx in ((0, "x"), (1, "y")):
        ref_c, ref_f = oracle_lib.roe_reflux_select(d, F["F" + sfx], F["Sm" + sfx], F["Sp" + sfx], (0, 0), mask,
                                                    (-G, -G), grid)
        assert np.array_equal(fc[d].cpu().numpy(), ref_c), sfx
        assert np.array_equal(ff[d].cpu().numpy(), ref_f), sfx
        assert np.count_nonzero(ref_c) > 0 and np.count_nonzero(ref_f) > 0


def test_fp64_rate_probe(cuda, hxlib):
    """The FP64 roof probe measures positive rates, FP32 well above FP64."""
    d, f = capi.fp64_rates()
    assert d > 1e10 and f > d


def fast_op(hxlib, cuda, op, x, n):
    xt = torch.from_numpy(np.ascontiguousarray(x)).to(cuda)
    yt = torch.empty(n, dtype=torch.float64, device=cuda)
    hxlib.check(hxlib.lib().hx_debug_fast_op_f64(op, n, dptr(xt), dptr(yt), None), "fast op")
    return yt.cpu().numpy()


def ulps(a, b):
    return np.abs(a.view(np.int64) - b.view(np.int64))


def wide_range(rng, n, lo=1e-300, hi=1e300, signed=True):
    x = np.exp(rng.uniform(np.log(lo), np.log(hi), n))
    return x * rng.choice([-1.0, 1.0], n) if signed else x


def test_fast_reciprocal_one_step(cuda, hxlib):
    """The face flux's reciprocal (float estimate of the leading bits, exponent
    restored on the integer pipe, one Newton step) is within 2^-42 relative of
    IEEE division over 2^22 values from 1e-300 to 1e300 in magnitude, both
    signs, with no range branch; the bulk is far tighter."""
    rng = np.random.default_rng(11)
    n = 1 << 22
    x = wide_range(rng, n)
    x[:1000] = 1.0 + np.arange(1000) * 2.0 ** -52  # just above 1
    x[1000:1008] = [1.0, 2.0, 0.5, -4.0, 2.0 ** 1000, 2.0 ** -1000, 3.0, 1e-6]
    y = fast_op(hxlib, cuda, capi.HX_FAST_OP_RCP, x, n)
    rel = np.abs(y - 1.0 / x) * np.abs(x)
    assert rel.max() <= 2.0 ** -42, rel.max()
    assert np.median(rel) <= 2.0 ** -46
    assert np.signbit(y[1003]) and np.all(np.isfinite(y))


def test_faithful_reciprocal(cuda, hxlib):
    """The CFL rate's reciprocal (same seed, third-order step) is within one ulp
    of IEEE division over the whole range, correctly rounded almost always."""
    rng = np.random.default_rng(12)
    n = 1 << 22
    x = wide_range(rng, n)
    x[: n // 2] = wide_range(rng, n // 2, 1e-30, 1e30)
    u = ulps(fast_op(hxlib, cuda, capi.HX_FAST_OP_RCP_FAITHFUL, x, n), 1.0 / x)
    assert u.max() <= 1, u.max()
    assert (u == 0).mean() > 0.99


def test_fast_sqrt_one_step(cuda, hxlib):
    """The face flux's square root (float estimate of 1/sqrt, one Newton step,
    three FP64 instructions) is within 2^-42 relative of the IEEE square root
    over 2^22 values from 1e-300 to 1e300, including the depths a face sees
    (1e-6 to 1e4); +0 gives +0 without the IEEE path."""
    rng = np.random.default_rng(13)
    n = 1 << 22
    x = wide_range(rng, n, signed=False)
    x[: n // 2] = wide_range(rng, n // 2, 1e-6, 1e4, signed=False)
    x[:8] = [0.0, 1.0, 4.0, 2.0, 1e-6, 9.81e-6, 2.0 ** -60, 2.0 ** 60]
    y = fast_op(hxlib, cuda, capi.HX_FAST_OP_SQRT, x, n)
    ref = np.sqrt(x)
    rel = np.abs(y - ref) / np.where(ref > 0, ref, 1.0)
    assert rel.max() <= 2.0 ** -42, rel.max()
    assert np.median(rel) <= 2.0 ** -46
    assert y[0] == 0.0 and not np.signbit(y[0])


def test_faithful_sqrt(cuda, hxlib):
    """The CFL rate's square root (the d^2 term kept) is within 2 ulps of the
    IEEE square root, exact on exact squares, mostly correctly rounded."""
    rng = np.random.default_rng(14)
    n = 1 << 22
    x = wide_range(rng, n, signed=False)
    x[: n // 2] = wide_range(rng, n // 2, 1e-6, 1e4, signed=False)
    x[:8] = [0.0, 1.0, 4.0, 2.0, 1e-6, 9.81e-6, 2.0 ** -60, 2.0 ** 60]
    y = fast_op(hxlib, cuda, capi.HX_FAST_OP_SQRT_FAITHFUL, x, n)
    u = ulps(y, np.sqrt(x))
    assert u.max() <= 2, u.max()
    assert y[0] == 0.0 and y[1] == 1.0 and y[2] == 2.0
    assert (u == 0).mean() > 0.9


def test_fast_reciprocal_cube_root(cuda, hxlib):
    """The Manning factor's h^(-1/3) in the fast form (the float rcbrtf of the
    leading bits widened, one Newton step) is within 2^-42 relative of
    1/cbrt(h) over depths from the dry tolerance to 1e4 m, and well inside it
    for the bulk."""
    rng = np.random.default_rng(15)
    n = 1 << 22
    x = wide_range(rng, n, 1e-6, 1e4, signed=False)
    x[:6] = [1e-6, 1.0, 8.0, 0.125, 27.0, 1e4]
    y = fast_op(hxlib, cuda, capi.HX_FAST_OP_RCBRT, x, n)
    ref = 1.0 / np.cbrt(x)
    rel = np.abs(y - ref) / ref
    assert rel.max() <= 2.0 ** -42, rel.max()
    assert np.median(rel) <= 2.0 ** -46


def test_fast_van_leer_slope(cuda, hxlib):
    """The fast form's van Leer slope 2 dm dp / (dm + dp) (seeds of the quotient
    and of 2/S from float estimates, one Newton correction in FP64) against the
    quotient of the same FP64 dm dp and dm + dp taken in extended precision:
    within 2^-41 relative over differences from 1e-10 to 1e6 of both signs;
    exactly 0 where dm dp <= 0 or |dp| <= 1e-12 (the reference's branches);
    where the quotient falls below the normal range the result stays within
    2^-20 of it."""
    rng = np.random.default_rng(15)
    n = 1 << 21
    q = rng.uniform(-10.0, 10.0, n)
    dm = wide_range(rng, n, 1e-10, 1e6)
    dp = np.abs(wide_range(rng, n, 1e-10, 1e6)) * np.sign(dm) * rng.choice([1.0, 1.0, 1.0, -1.0], n)
    dm[:4], dp[:4] = [1.0, 1.0, 1e-310, 2.0], [5e-13, -1.0, 1.0, 2.0]  # tiny dm: subnormal dm dp
    q[2] = 0.0
    x = np.stack([q - dm, q, q + dp], axis=1).reshape(-1)
    y = fast_op(hxlib, cuda, capi.HX_FAST_OP_SLOPE, x, n)
    xm, x0, xp = x[0::3], x[1::3], x[2::3]
    d1, d2 = x0 - xm, xp - x0  # the device's differences, bit for bit
    p, S = d1 * d2, d1 + d2
    live = (np.abs(d2) > 1e-12) & (p > 0)
    assert np.all(y[~live] == 0.0)
    ref = 2.0 * p[live].astype(np.longdouble) / S[live].astype(np.longdouble)
    rel = np.abs((y[live] - ref) / ref).astype(np.float64)
    normal = np.abs(ref) > 1e-300
    assert rel[normal].max() <= 2.0 ** -41, rel[normal].max()
    assert np.all(rel[~normal] <= 2.0 ** -20)
    assert live[2] and not normal[np.flatnonzero(live).tolist().index(2)]
    assert abs(y[3] - 2.0) <= 2.0 ** -41 and live.mean() > 0.5
