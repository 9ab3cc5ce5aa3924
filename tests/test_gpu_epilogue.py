"""The advance epilogue: eta = h + z (AmrMeshState::DeriveEtaFrom,
src/state/AmrMeshState_AMR.cpp:203-224) and the conservation diagnostics
(AmrMeshState::ComputeMassDiagnostics, src/state/AmrMeshState_Utils.cpp:213-300)
written by the update of the step that produces the state, against the same
step without them followed by the separate passes (each of which is checked
against the oracle in test_gpu_diagnostics.py).

The state and the next-dt accumulator are bit-equal to the plain step, eta is
bit-equal to the separate pass.  Diagnostics: exact arithmetic on boxes below
2048 x 2048 cells uses the separate pass's blocks and terms, so it is
bit-equal; on the 32 x 32 tiles of larger boxes and levels only the order of
the sums differs (1e-13 relative); the FP64 fast form sums unscaled terms
through a reciprocal within 2^-44 (1e-12 relative).  min h is always exact."""
import ctypes

import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.level import DtAccum, Level, Status, array4, box

pytestmark = pytest.mark.gpu
EXACT, FAST = capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST
NODATA = -9999.0


def vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def with_currents(c, seed):
    rng = np.random.default_rng(seed)
    live = c.n != NODATA
    c.hu = np.where(live, c.h * rng.uniform(-0.5, 0.5, c.h.shape), 0.0)
    c.hv = np.where(live, c.h * rng.uniform(-0.5, 0.5, c.h.shape), 0.0)
    c.h[5:9, 10:30] = 0.0  # a dry patch
    return c


def cfl_dt(c, cfl=0.4):
    live = (c.n != NODATA) & (c.h > 1e-6)
    hh = c.h[live]
    s = np.abs(c.hu[live] / hh) + np.abs(c.hv[live] / hh) + 2 * np.sqrt(9.81 * hh)
    return cfl * c.geom.dx / s.max()


def sums_close(got, ref, rtol):
    np.testing.assert_allclose(got[:4], ref[:4], rtol=rtol, atol=0)
    assert got[4] == ref[4]


def box_case(cuda, nx, ny, dtype, seed, lo=(3, -2)):
    """Ghost-filled views (2 ghosts) of a box with lower corner lo: the ghost
    values are any values (both steps read the same ones)."""
    c = with_currents(workloads.fractal_dam_break(nx + 4, ny + 4, seed=seed, amplitude=1.0, nodata_frac=0.15), seed)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dtype))).to(cuda)
    glo = (lo[0] - 2, lo[1] - 2)
    Eta = dev((c.h + c.z)[None])
    Ue = dev(np.stack([c.h, c.hu, c.hv]))
    Te = dev(np.stack([c.z, c.n]))
    Uo = dev(np.stack([c.h, c.hu, c.hv])[:, 2:-2, 2:-2])
    vb = box(lo, (lo[0] + nx - 1, lo[1] + ny - 1))
    return dict(c=c, Eta=(Eta, glo), Ue=(Ue, glo), Te=(Te, glo), Uo=(Uo, lo), vb=vb, lo=lo, dt=cfl_dt(c),
                dx=c.geom.dx, dy=c.geom.dy)


@pytest.mark.parametrize("dtype,arith,nx,ny", [
    (np.float64, EXACT, 200, 136), (np.float64, FAST, 200, 136), (np.float32, EXACT, 200, 136),
    (np.float32, FAST, 200, 136), (np.float64, EXACT, 2048, 2048), (np.float64, FAST, 2048, 2048)])
def test_box_epilogue_equals_separate_passes(cuda, hxlib, dtype, arith, nx, ny):
    L = hxlib.lib()
    k = box_case(cuda, nx, ny, dtype, seed=nx + arith)
    sfx = "f64" if dtype == np.float64 else "f32"
    R = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    A = lambda name: ctypes.byref(array4(*k[name]))
    Uo = k["Uo"][0]
    acc1, acc2 = DtAccum(cuda), DtAccum(cuda)
    st = Status(cuda)
    st.clear()
    U1 = torch.zeros_like(Uo)
    hxlib.check(getattr(L, "hx_advance_box_hydrostatic_" + sfx)(
        A("Eta"), A("Ue"), A("Te"), A("Uo"), ctypes.byref(array4(U1, k["lo"])), k["vb"], R(k["dt"]), R(k["dx"]),
        R(k["dy"]), None, None, acc1.ptr, st.ptr, arith, None), "plain box step")
    U2 = torch.zeros_like(Uo)
    eta = torch.full_like(Uo[0], 7.0)
    diag = torch.empty(5, dtype=torch.float64, device=cuda)
    work = torch.empty(int(L.hx_diagnostics_work_bytes(k["vb"])), dtype=torch.uint8, device=cuda)
    hxlib.check(getattr(L, "hx_advance_box_hydrostatic_epilogue_" + sfx)(
        A("Eta"), A("Ue"), A("Te"), A("Uo"), ctypes.byref(array4(U2, k["lo"])), k["vb"], R(k["dt"]), R(k["dx"]),
        R(k["dy"]), acc2.ptr, st.ptr, arith, ctypes.byref(array4(eta, k["lo"])), vp(diag), vp(work), None),
        "box step with epilogue")
    assert st.read() == 0
    assert torch.equal(U1, U2)
    assert acc1.read() == acc2.read()
    # the separate passes over the plain step's result
    eta_sep = torch.zeros_like(eta)
    Te = ctypes.byref(array4(*k["Te"]))
    hxlib.check(getattr(L, "hx_derive_eta_box_" + sfx)(ctypes.byref(array4(U1, k["lo"])), Te,
                                                       ctypes.byref(array4(eta_sep, k["lo"])), k["vb"], None), "eta")
    d_sep = torch.empty(5, dtype=torch.float64, device=cuda)
    hxlib.check(getattr(L, "hx_diagnostics_box_" + sfx)(ctypes.byref(array4(U1, k["lo"])), Te, k["vb"], R(k["dx"]),
                                                        R(k["dy"]), vp(d_sep), vp(work), None), "diagnostics")
    assert torch.equal(eta, eta_sep)
    got, ref = diag.cpu().numpy(), d_sep.cpu().numpy()
    assert ref[3] > 0 and ref[0] > 0
    if arith == EXACT and nx * ny < 2048 * 2048:
        assert np.array_equal(got, ref)  # same blocks, same terms
    elif dtype == np.float32:
        sums_close(got, ref, 1e-5)  # the float terms contracted into multiply-adds
    else:
        sums_close(got, ref, 1e-13 if arith == EXACT else 1e-12)


def level_case(n, seed, dtype=torch.float64, cuda="cuda"):
    c = with_currents(workloads.fractal_dam_break(n, n, seed=seed, amplitude=1.0, nodata_frac=0.15), seed)
    return c, Level.from_numpy(c.geom, c.h, c.hu, c.hv, c.z, c.n, dtype=dtype, device=cuda)


@pytest.mark.parametrize("arith", [EXACT, FAST])
@pytest.mark.parametrize("n", [320, 2048])
def test_level_epilogue_equals_separate_passes(cuda, hxlib, arith, n):
    """At 2048 x 2048 the level runs the persistent kernel with the epilogue in
    it: per-thread sums over the block's tiles, one partial per block."""
    c, lev = level_case(n, seed=11 + n)
    dt = 0.45 * lev.compute_dt()[0]
    acc1, acc2 = DtAccum(cuda), DtAccum(cuda)
    lev.status.clear()
    out1 = lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, next_dt=acc1, arith=arith)
    out2, eta, diag = lev.advance_epilogue(dt, next_dt=acc2, arith=arith)
    assert lev.status.read() == 0
    assert torch.equal(out1, out2)
    assert acc1.read() == acc2.read()
    assert torch.equal(eta, out1[0] + lev.terrain[0])
    b = box((0, 0), (c.geom.nx - 1, c.geom.ny - 1))
    work = torch.empty(int(hxlib.lib().hx_diagnostics_work_bytes(b)), dtype=torch.uint8, device=cuda)
    d_sep = torch.empty(5, dtype=torch.float64, device=cuda)
    d = lev._desc(out1)
    hxlib.check(hxlib.lib().hx_level_diagnostics_f64(ctypes.byref(d), vp(d_sep), vp(work), None), "diagnostics")
    got, ref = diag.cpu().numpy(), d_sep.cpu().numpy()
    if arith == EXACT and n < 2048:
        assert np.array_equal(got, ref)
    else:
        sums_close(got, ref, 1e-13 if arith == EXACT else 1e-12)


def test_level_epilogue_f32_and_single_outputs(cuda, hxlib):
    """FP32 level; eta alone and diagnostics alone give the same values as both."""
    c, lev = level_case(256, seed=5, dtype=torch.float32)
    dt = 0.45 * lev.compute_dt()[0]
    out, eta, diag = lev.advance_epilogue(dt, arith=EXACT)
    assert torch.equal(out, lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, arith=EXACT))
    assert torch.equal(eta, out[0] + lev.terrain[0])
    T = ctypes.byref(array4(lev.terrain))
    b = box((0, 0), (c.geom.nx - 1, c.geom.ny - 1))
    work = torch.empty(int(hxlib.lib().hx_diagnostics_work_bytes(b)), dtype=torch.uint8, device=cuda)
    d_sep = torch.empty(5, dtype=torch.float64, device=cuda)
    hxlib.check(hxlib.lib().hx_diagnostics_box_f32(ctypes.byref(array4(out)), T, b, ctypes.c_float(c.geom.dx),
                                                   ctypes.c_float(c.geom.dy), vp(d_sep), vp(work), None), "diag")
    assert np.array_equal(diag.cpu().numpy(), d_sep.cpu().numpy())
    _, eta_only, none = lev.advance_epilogue(dt, diag=False, arith=EXACT)
    assert none is None and torch.equal(eta_only, eta)
    _, none, diag_only = lev.advance_epilogue(dt, eta=False, arith=EXACT)
    assert none is None and torch.equal(diag_only, diag)


def test_epilogue_argument_errors(cuda, hxlib):
    c, lev = level_case(64, seed=2)
    d = lev._desc(lev.state)
    out = torch.empty_like(lev.state)
    diag = torch.empty(5, dtype=torch.float64, device=cuda)
    planes = [vp(out[k]) for k in range(3)]
    L = hxlib.lib()
    rc = L.hx_level_advance_epilogue_f64(ctypes.byref(d), 1e-4, *planes, None, None, EXACT, None, None, None, None)
    assert rc == capi.HX_ERR_ARG  # neither output
    rc = L.hx_level_advance_epilogue_f64(ctypes.byref(d), 1e-4, *planes, None, None, EXACT, None, vp(diag), None,
                                         None)
    assert rc == capi.HX_ERR_ARG  # diagnostics without work


def test_persistent_epilogue_reports_a_staging_timeout(cuda, hxlib):
    """The persistent kernel's bounded staging wait, made to run out (the
    expected byte count raised by a test setting): the step sets
    HX_STATUS_STAGING_TIMEOUT and the diagnostics' sums come back NaN instead
    of a partial sum; the next step runs clean."""
    c, lev = level_case(2048, seed=9)
    dt = 0.45 * lev.compute_dt()[0]
    L = hxlib.lib()
    prev = L.hx_debug_staging_extra_bytes(16)
    try:
        lev.status.clear()
        _, _, diag = lev.advance_epilogue(dt, eta=False, arith=FAST)
        assert lev.status.read() & capi.HX_STATUS_STAGING_TIMEOUT
        assert np.isnan(diag.cpu().numpy()[:4]).all()
    finally:
        L.hx_debug_staging_extra_bytes(prev)
    lev.status.clear()
    out, eta, diag = lev.advance_epilogue(dt, arith=FAST)
    assert lev.status.read() == 0
    assert np.isfinite(diag.cpu().numpy()).all()
    assert torch.equal(out, lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, arith=FAST))
