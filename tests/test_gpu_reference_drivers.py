"""The CUDA level path against the reference's own per-box drivers.

tests/golden/drivers_f64.npz holds the state, clock and status that the
reference's HydrostaticRoe.cpp / Roe.cpp (with SolverVariant and the BCFill.H
ghost filler) reach in their own time loop, compiled verbatim and run at one
level (oracle/ref_level.cpp, tests/golden/make_golden.py).  The device time
loop in the exact form reproduces them bit for bit from the same inputs (the
build whose limiter abs() is the floating one, as in device code); Manning
friction goes through cbrt, which may differ by an ulp between CUDA and the C
library, so friction cases hold to 1e-13.  The fast form stays within 1e-10
of them over the same steps.

Walls: code 0 is the reference's wall, whose momentum ghosts take the BC
records its per-step FillPatch applies (offset 0: hu as a scalar, hv as the
x-momentum), so flow crosses it; code 2 is the closed wall.  Both are checked
against the oracle, and mass against its conservation.
"""
from pathlib import Path

import numpy as np
import pytest

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.level import Geometry, Level

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
EXACT, FAST = capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return max(float(np.abs(a[k] - b[k]).max() / max(np.abs(b[k]).max(), 1e-300)) for k in range(a.shape[0]))


def golden_cases():
    d = np.load(GOLD / "drivers_f64.npz")
    names = sorted({k.split("/")[0] for k in d.files if not k.startswith("tags/")})
    out = []
    for name in names:
        if f"{name}/geom" not in d.files:
            continue
        for m in d[f"{name}/methods"]:
            out.append((name, int(m)))
    return out


@pytest.mark.parametrize("name,method", golden_cases(), ids=[f"{n}-m{m}" for n, m in golden_cases()])
def test_level_loop_matches_reference_drivers(cuda, name, method):
    d = np.load(GOLD / "drivers_f64.npz")
    g = d[f"{name}/geom"]
    dx, dy, cfl = (float(x) for x in d[f"{name}/dxdy_cfl"])
    geom = Geometry(int(g[0]), int(g[1]), dx, dy, (int(g[2]), int(g[3])), (int(g[4]), int(g[5])))
    planes = [d[f"{name}/{k}"] for k in ("h", "hu", "hv", "z", "n")]
    nsteps = int(d[f"{name}/nsteps"])
    want = d[f"{name}/m{method}/fabs/state"]
    t_want, status_want = (float(x) for x in d[f"{name}/m{method}/fabs/t_status"])
    friction = bool((planes[4][planes[3] > -9000] != 0).any())
    for arith in (EXACT, FAST):
        lev = Level.from_numpy(geom, *planes, device=cuda)
        st = lev.run(method, nsteps, cfl, arith=arith)
        if status_want:  # the reference's loop aborted on a collapsed dt; so does the device loop
            assert st & capi.HX_STATUS_DT_COLLAPSE
            continue
        assert st == 0
        got = lev.state.cpu().numpy()
        if arith == EXACT and not friction:
            assert np.array_equal(got, want), (name, rel_err(got, want))
            assert lev.time.item() == pytest.approx(t_want, rel=1e-15)
        else:
            assert rel_err(got, want) <= (1e-13 if arith == EXACT else 1e-10), (name, arith)
            assert lev.time.item() == pytest.approx(t_want, rel=1e-10)


def wall_case(code):
    """A dam break that reaches all four walls within the run, with both
    momentum components non-zero there."""
    c = workloads.dam_break(48, 40, x_dam=0.2, h_left=1.5, h_right=0.3)
    c.hv = 0.4 * c.h
    c.geom.bc_lo, c.geom.bc_hi = (code, code), (code, code)
    return c


@pytest.mark.parametrize("method", [capi.HX_METHOD_HYDROSTATIC_ROE, capi.HX_METHOD_ROE])
@pytest.mark.parametrize("code", [capi.HX_BC_REFLECTIVE, capi.HX_BC_CLOSED_WALL])
def test_walls_match_oracle_and_mass(cuda, oracle_lib, method, code):
    """Both wall codes against the oracle (bit for bit, exact form) over 120
    steps of flow against the walls; the closed wall conserves mass to
    round-off, the reference's wall lets mass cross (the reference's
    behaviour, reproduced)."""
    c = wall_case(code)
    g = c.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    ref = oracle_lib.run(L, method, c.h, c.hu, c.hv, c.z, c.n, 120, c.cfl)
    assert ref[5] == 0
    lev = Level.from_numpy(g, c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    assert lev.run(method, 120, c.cfl, arith=EXACT) == 0
    got = lev.state.cpu().numpy()
    assert np.array_equal(got, np.stack(ref[:3]))
    m0, m1 = c.h.sum(), got[0].sum()
    if code == capi.HX_BC_CLOSED_WALL:
        assert abs(m1 - m0) <= 1e-12 * m0
    else:
        assert abs(m1 - m0) > 1e-6 * m0
