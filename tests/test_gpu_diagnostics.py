"""Conservation diagnostics and eta (src/state/AmrMeshState_Utils.cpp:213-298,
src/state/AmrMeshState_AMR.cpp:203-224) against the oracle.

Per-cell terms are the reference's in both builds; the sums are carried in
double in a fixed order on the device and row by row in the oracle, so they
agree to summation rounding (1e-12 relative); min h is exact."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.level import Level, array4, box

pytestmark = pytest.mark.gpu


def case_with_currents(nx=200, ny=136, seed=8):
    c = workloads.fractal_dam_break(nx, ny, seed=seed, amplitude=1.0, nodata_frac=0.2)
    rng = np.random.default_rng(seed)
    c.hu = np.where(c.n == -9999.0, 0.0, c.h * rng.uniform(-0.5, 0.5, c.h.shape))
    c.hv = np.where(c.n == -9999.0, 0.0, c.h * rng.uniform(-0.5, 0.5, c.h.shape))
    c.h[5:9, 10:30] = 0.0  # a dry patch
    return c


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_diagnostics_box_matches_oracle(cuda, hxlib, oracle_lib, dtype):
    c = case_with_currents()
    ny, nx = c.h.shape
    U = torch.from_numpy(np.stack([c.h, c.hu, c.hv]).astype(dtype)).to(cuda)
    T = torch.from_numpy(np.stack([c.z, c.n]).astype(dtype)).to(cuda)
    lo = (3, -2)  # box coordinates need not start at 0
    b = box(lo, (lo[0] + nx - 1, lo[1] + ny - 1))
    work = torch.empty(int(hxlib.lib().hx_diagnostics_work_bytes(b)), dtype=torch.uint8, device=cuda)
    out = torch.empty(5, dtype=torch.float64, device=cuda)
    sfx = "f64" if dtype == np.float64 else "f32"
    R = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    rc = getattr(hxlib.lib(), "hx_diagnostics_box_" + sfx)(
        ctypes.byref(array4(U, lo)), ctypes.byref(array4(T, lo)), b, R(c.geom.dx), R(c.geom.dy),
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(work.data_ptr()), None)
    assert rc == 0
    got = out.cpu().numpy()
    ref = oracle.mass_diagnostics(*(a.astype(dtype) for a in (c.h, c.hu, c.hv, c.n)), c.geom.dx, c.geom.dy)
    np.testing.assert_allclose(got[:4], ref[:4], rtol=1e-12, atol=0)
    assert got[4] == ref[4]
    mask = (c.n != -9999.0) & (c.h > 0)
    assert got[4] == c.h[mask].astype(dtype).min()


def test_level_diagnostics_and_conservation(cuda, hxlib, oracle_lib):
    """The level form equals the box form; a flat-bed dam break with walls keeps
    its mass to round-off over 50 device steps (reference check: dMass = 0)."""
    c = workloads.dam_break(128, 96)
    lev = Level.from_numpy(c.geom, c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    b = box((0, 0), (c.geom.nx - 1, c.geom.ny - 1))
    work = torch.empty(int(hxlib.lib().hx_diagnostics_work_bytes(b)), dtype=torch.uint8, device=cuda)

    def diag():
        out = torch.empty(5, dtype=torch.float64, device=cuda)
        d = lev._desc(lev.state)
        assert hxlib.lib().hx_level_diagnostics_f64(ctypes.byref(d), ctypes.c_void_p(out.data_ptr()),
                                                    ctypes.c_void_p(work.data_ptr()), None) == 0
        return out.cpu().numpy()

    d0 = diag()
    ref = oracle.mass_diagnostics(c.h, c.hu, c.hv, c.n, c.geom.dx, c.geom.dy)
    np.testing.assert_allclose(d0[:4], ref[:4], rtol=1e-13, atol=1e-15)
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 50, 0.45, arith=capi.HX_ARITH_FAST) == 0
    d1 = diag()
    assert abs(d1[0] - d0[0]) <= 1e-13 * d0[0]
    assert d1[3] > 0  # the dam break has set the water moving


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_derive_eta_with_ghosts(cuda, hxlib, oracle_lib, dtype):
    rng = np.random.default_rng(3)
    g = 2
    h = rng.uniform(0, 2, (40 + 2 * g, 70 + 2 * g)).astype(dtype)
    z = rng.uniform(-1, 1, h.shape).astype(dtype)
    U = torch.from_numpy(np.stack([h, h, h])).to(cuda)
    T = torch.from_numpy(np.stack([z, z])).to(cuda)
    eta = torch.zeros((1,) + h.shape, dtype=U.dtype, device=cuda)
    lo = (-g, -g)
    b = box(lo, (70 + g - 1, 40 + g - 1))  # the grown box
    sfx = "f64" if dtype == np.float64 else "f32"
    assert getattr(hxlib.lib(), "hx_derive_eta_box_" + sfx)(ctypes.byref(array4(U, lo)), ctypes.byref(array4(T, lo)),
                                                             ctypes.byref(array4(eta, lo)), b, None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(eta[0].cpu().numpy(), oracle.derive_eta(h, z))
