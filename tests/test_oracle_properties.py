"""Properties the reference asserts in its documents, checked on the oracle:
lake at rest, mass conservation, y-symmetry of a planar dam break and the
exact dam-break solution (from the reference's tests/dambreak/analytical.py,
committed as tests/golden/dambreak_exact.npz)."""
from pathlib import Path

import numpy as np
import pytest

from hydroexa_gb300 import workloads

GOLD = Path(__file__).resolve().parent / "golden"


def _level(oracle, case):
    g = case.geom
    return oracle.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)


def test_lake_at_rest_hydrostatic(oracle_lib):
    case = workloads.lake_at_rest(64, 64, seed=7, nodata_frac=0.0, nsteps=60)
    L = _level(oracle_lib, case)
    h, hu, hv, t, dt, rc = oracle_lib.run(L, oracle_lib.METHOD_HYDROSTATIC, case.h, case.hu, case.hv, case.z,
                                          case.n, case.nsteps, case.cfl)
    assert rc == 0
    wet = h > 1e-6
    vel = np.sqrt(hu[wet] ** 2 + hv[wet] ** 2) / h[wet]
    assert vel.max() <= 1e-13


def test_nodata_wall_drops_pressure(oracle_lib):
    """Reference behaviour, reproduced: a face touching a NODATA cell carries no
    flux at all (HydrostaticRoe.cpp:237-245), including the hydrostatic
    pressure a wall would exert, so a lake at rest beside a NODATA block starts
    to move toward it.  The disturbance starts only at cells next to NODATA."""
    case = workloads.lake_at_rest(64, 64, seed=7, nodata_frac=0.1, nsteps=1)
    L = _level(oracle_lib, case)
    mn, _ = oracle_lib.compute_dt(L, case.h, case.hu, case.hv, case.z)
    h, hu, hv = oracle_lib.advance(L, 1, case.h, case.hu, case.hv, case.z, case.n, mn * case.cfl)
    nod = case.z == -9999.0
    near = np.zeros_like(nod)
    near[1:, :] |= nod[:-1, :]
    near[:-1, :] |= nod[1:, :]
    near[:, 1:] |= nod[:, :-1]
    near[:, :-1] |= nod[:, 1:]
    near &= ~nod
    mom = np.abs(hu) + np.abs(hv)
    assert mom[near].max() > 1e-3
    assert mom[~near & ~nod].max() < 1e-14


@pytest.mark.parametrize("method", [0, 1])
def test_mass_conservation_flat_bed(oracle_lib, method):
    """Circular dam break on a flat bed that reaches the walls within the run.
    Closed walls (code 2, each momentum with its own BC record): mass to
    round-off.  The reference's walls (code 0: the momentum ghosts take the BC
    records its per-step FillPatch applies, offset 0 -- hu as a scalar, hv as
    the x-momentum) let mass cross once the wave arrives: reference behaviour,
    reproduced."""
    case = workloads.fractal_dam_break(64, 48, seed=1, nsteps=40, amplitude=0.0, nodata_frac=0.0)
    m0 = case.h.sum()
    case.geom.bc_lo, case.geom.bc_hi = (2, 2), (2, 2)
    L = _level(oracle_lib, case)
    h, hu, hv, t, dt, rc = oracle_lib.run(L, method, case.h, case.hu, case.hv, case.z, case.n, case.nsteps, case.cfl)
    assert rc == 0
    assert abs(h.sum() - m0) / m0 < 1e-13
    # flow against every wall from the start: the closed walls hold it, the reference's walls do not
    for code in (2, 0):
        c = workloads.dam_break(48, 40, x_dam=0.2, h_left=1.5, h_right=0.3)
        c.hv = 0.4 * c.h
        c.geom.bc_lo, c.geom.bc_hi = (code, code), (code, code)
        L = _level(oracle_lib, c)
        h, *_, rc = oracle_lib.run(L, method, c.h, c.hu, c.hv, c.z, c.n, 120, c.cfl)
        assert rc == 0
        dm = abs(h.sum() - c.h.sum()) / c.h.sum()
        assert (dm < 1e-13) if code == 2 else (dm > 1e-2)


def test_wall_leaks_on_sloping_bed(oracle_lib):
    """Reference behaviour, reproduced: at a reflective wall the ghost free
    surface and momenta are mirrored but the ghost bed is copied from the edge
    cell (terrain BCs are always foextrap, AmrMeshState_Init.cpp:61-70), so the
    second ghost's velocity is not the mirror of the interior one and the
    MUSCL face velocity at the wall is not zero: mass crosses the wall on a
    sloping bed, even with closed walls (code 2).  The classic first-order
    solver reads one ghost and does not leak through them."""
    case = workloads.fractal_dam_break(64, 48, seed=1, nsteps=20, amplitude=0.2, nodata_frac=0.0)
    case.geom.bc_lo, case.geom.bc_hi = (2, 2), (2, 2)
    L = _level(oracle_lib, case)
    h, *_ = oracle_lib.run(L, 1, case.h, case.hu, case.hv, case.z, case.n, case.nsteps, case.cfl)
    assert abs(h.sum() - case.h.sum()) / case.h.sum() > 1e-7
    h, *_ = oracle_lib.run(L, 0, case.h, case.hu, case.hv, case.z, case.n, case.nsteps, case.cfl)
    assert abs(h.sum() - case.h.sum()) / case.h.sum() < 1e-13


@pytest.mark.parametrize("method", [0, 1])
def test_planar_dam_break_is_one_dimensional(oracle_lib, method):
    case = workloads.dam_break(64, 16, method=method, nsteps=30)
    L = _level(oracle_lib, case)
    h, hu, hv, *_ = oracle_lib.run(L, method, case.h, case.hu, case.hv, case.z, case.n, case.nsteps, case.cfl)
    assert np.all(h == h[0:1, :])
    assert np.all(hv == 0.0)


def test_dam_break_against_exact_solution(oracle_lib):
    """1-D dam break (hl = 1.0, hr = 0.1 on [0,1]) with the classic solver, run
    to t = 0.1 against the exact wet-bed profile of the reference's
    analytical.py: L1 error of h stays at the first-order scheme's level."""
    g = np.load(GOLD / "dambreak_exact.npz")
    nx, ny = 256, 4
    case = workloads.dam_break(nx, ny, method=0, cfl=0.45)
    L = oracle_lib.Level(nx, ny, 1.0 / nx, 1.0 / ny, (1, 0), (1, 0))
    h, hu, hv = case.h.copy(), case.hu.copy(), case.hv.copy()
    t = 0.0
    while t < 0.1 - 1e-15:
        mn, _ = oracle_lib.compute_dt(L, h, hu, hv, case.z)
        dt = min(mn * case.cfl, 0.1 - t)
        h, hu, hv = oracle_lib.advance(L, 0, h, hu, hv, case.z, case.n, dt)
        t += dt
    err = np.abs(h[0] - g["h_t0.1"]).mean()
    assert err < 1.5e-2


def test_mass_diagnostics_excludes_nodata_and_dry_cells(oracle_lib):
    """ComputeMassDiagnostics counts cells that are not NODATA (roughness
    -9999) and wet; its sums are the plain sums over those cells."""
    oracle = oracle_lib
    c = workloads.fractal_dam_break(64, 48, seed=5, amplitude=1.0, nodata_frac=0.2)
    c.hu = c.h * 0.3
    c.hv = -c.h * 0.1
    c.h[3, 3:9] = 0.0
    dA = c.geom.dx * c.geom.dy
    out = oracle.mass_diagnostics(c.h, c.hu, c.hv, c.n, c.geom.dx, c.geom.dy)
    m = (c.n != -9999.0) & (c.h > 0)
    np.testing.assert_allclose(out[:4], [(c.h[m] * dA).sum(), (c.hu[m] * dA).sum(), (c.hv[m] * dA).sum(),
                                         (0.5 * (c.hu[m] ** 2 + c.hv[m] ** 2) / c.h[m] * dA).sum()], rtol=1e-13)
    assert out[4] == c.h[m].min()
    assert np.array_equal(oracle.derive_eta(c.h, c.z), c.h + c.z)


@pytest.mark.parametrize("rx,ry,dtype", [(2, 2, np.float64), (4, 4, np.float64), (2, 4, np.float64),
                                         (3, 3, np.float64), (2, 2, np.float32)])
def test_average_down_is_the_ordered_mean(oracle_lib, rx, ry, dtype):
    """average_down: coarse = (1 / (rx ry)) * sum of the fine block, summed
    rows outer, columns inner; the mean of a constant is that constant and the
    restriction conserves the integral to round-off."""
    rng = np.random.default_rng(rx * 10 + ry)
    fine = rng.uniform(-2.0, 3.0, size=(3, 12 * ry, 10 * rx)).astype(dtype)
    got = oracle_lib.average_down(fine, rx, ry)
    acc = np.zeros((3, 12, 10), dtype=dtype)
    for jr in range(ry):
        for ir in range(rx):
            acc = acc + fine[:, jr::ry, ir::rx]
    assert np.array_equal(got, (dtype(1.0) / dtype(rx * ry)) * acc)
    const = np.full_like(fine, 0.7)
    assert np.allclose(oracle_lib.average_down(const, rx, ry), dtype(0.7), rtol=4 * np.finfo(dtype).eps)
    np.testing.assert_allclose(got.sum(axis=(1, 2)) * rx * ry, fine.sum(axis=(1, 2)),
                               rtol=50 * np.finfo(dtype).eps, atol=1e-3 if dtype == np.float32 else 1e-9)
