"""The benchmark configurations themselves against the oracle, at their own sizes.

- Throughput workload: the 8192^2 level of the bench (spectral fractal bed,
  20% NODATA, circular dam), FP64 hydrostatic Roe.  The exact form equals the
  oracle bit for bit after 1 and 3 steps of the device time loop; the fast
  form stays within 1e-12 relative (max |a - b| / max |b| per component).
  FP32: one step within 1e-5 of the oracle instantiated in float.
- Plain dam break: 256^2, both solvers, 200 steps: exact bit-equal, fast
  within 1e-9.
- 1000 steps on the lake-at-rest bed (Gaussian mound + N(0, 0.02) roughness,
  512^2, no NODATA block): the lake itself and a dam break over the same bed.
  Exact bit-equal, fast within 1e-9 after 1000 steps, relative to the
  state's scale: max |h| for the depth, max |h| sqrt(g max |h|) (the momentum
  of a gravity wave) for the momenta -- the lake's momenta are rounding noise
  (~1e-16), so their own maximum is no scale.  (A 1e-15 relative perturbation
  of the initial depth grows to ~1e-12 over the 1000 steps of the dam break in
  the oracle itself, so 1e-9 leaves the fast form's ~1e-15 per step a wide
  margin.)
"""
import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.level import Level

pytestmark = pytest.mark.gpu

EXACT, FAST = capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST
HYDRO, ROE = capi.HX_METHOD_HYDROSTATIC_ROE, capi.HX_METHOD_ROE


def rel_err(a, b):
    """max |a - b| / max |b| per component, worst component."""
    worst = 0.0
    for x, y in zip(a, b):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        worst = max(worst, float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300)))
    return worst


def state_err(a, b):
    """max |a - b| per component over the state's scale: max |h| for the
    depth, max |h| sqrt(g max |h|) for the momenta."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    hs = max(float(np.abs(b[0]).max()), 1e-300)
    scale = (hs, hs * np.sqrt(9.81 * hs), hs * np.sqrt(9.81 * hs))
    return max(float(np.abs(a[k] - b[k]).max()) / scale[k] for k in range(3))


def oracle_run(oracle, case, method, nsteps):
    g = case.geom
    L = oracle.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    h, hu, hv, t, _, status = oracle.run(L, method, case.h, case.hu, case.hv, case.z, case.n, nsteps, case.cfl)
    assert status == 0
    return (h, hu, hv), t


def device_run(case, method, nsteps, arith, device):
    lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=device)
    assert lev.run(method, nsteps, case.cfl, arith=arith) == 0
    return lev.state.cpu().numpy(), lev.time.item()


@pytest.fixture(scope="module")
def throughput(oracle_lib):
    """The bench's level and the oracle's states after 1 and 3 steps."""
    case = workloads.fractal_dam_break(8192, 8192, seed=3)
    one, t1 = oracle_run(oracle_lib, case, HYDRO, 1)
    three, t3 = oracle_run(oracle_lib, case, HYDRO, 3)
    return case, {1: (one, t1), 3: (three, t3)}


@pytest.mark.parametrize("arith", [EXACT, FAST])
def test_throughput_workload_matches_oracle(cuda, throughput, arith):
    case, ref = throughput
    assert abs((case.z == -9999.0).mean() - 0.2) < 0.01
    for nsteps in (1, 3):
        got, t = device_run(case, HYDRO, nsteps, arith, cuda)
        want, tw = ref[nsteps]
        if arith == EXACT:
            for k in range(3):
                assert np.array_equal(got[k], want[k]), (nsteps, k, rel_err([got[k]], [want[k]]))
            assert t == pytest.approx(tw, rel=1e-15)
        else:
            assert rel_err(got, want) <= 1e-12, nsteps
            assert t == pytest.approx(tw, rel=1e-12)
        del got


@pytest.mark.parametrize("arith", [EXACT, FAST])
def test_throughput_workload_fp32(cuda, oracle_lib, arith):
    """The FP32 line of the throughput configuration: one step of the 8192^2
    level in float, at the oracle's float CFL step."""
    case = workloads.fractal_dam_break(8192, 8192, seed=3)
    f = [a.astype(np.float32) for a in (case.h, case.hu, case.hv, case.z, case.n)]
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    mn, _ = oracle_lib.compute_dt(L, f[0], f[1], f[2], f[3])
    dt = float(np.float32(mn * case.cfl))
    ref = oracle_lib.advance(L, HYDRO, f[0], f[1], f[2], f[3], f[4], dt)
    lev = Level.from_numpy(g, *f, dtype=torch.float32, device=cuda)
    gmn, _ = lev.compute_dt()
    assert gmn == pytest.approx(mn, rel=1e-6)
    got = lev.advance(HYDRO, dt, arith=arith).cpu().numpy()
    assert rel_err(got, ref) <= 1e-5


@pytest.mark.parametrize("method", [HYDRO, ROE])
def test_plain_dam_break_200_steps(cuda, oracle_lib, method):
    case = workloads.dam_break(256, 256)
    want, tw = oracle_run(oracle_lib, case, method, 200)
    got, t = device_run(case, method, 200, EXACT, cuda)
    for k in range(3):
        assert np.array_equal(got[k], want[k]), (k, rel_err([got[k]], [want[k]]))
    assert t == pytest.approx(tw, rel=1e-15)
    fast, tf = device_run(case, method, 200, FAST, cuda)
    assert rel_err(fast, want) <= 1e-9
    assert tf == pytest.approx(tw, rel=1e-9)


def mound_case(kind):
    case = workloads.lake_at_rest(512, 512, seed=2, nodata_frac=0.0, nsteps=1000)
    if kind == "dam":  # free surface 1.5 m left of x = 0.3, 1.0 m right of it, over the same bed
        x = (np.arange(512) + 0.5) / 512
        eta = np.where(x[None, :] < 0.3, 1.5, 1.0) * np.ones((512, 1))
        case.h = np.maximum(0.0, eta - case.z)
    return case


@pytest.mark.parametrize("kind", ["lake", "dam"])
def test_mound_bed_1000_steps(cuda, oracle_lib, kind):
    case = mound_case(kind)
    want, tw = oracle_run(oracle_lib, case, HYDRO, 1000)
    got, t = device_run(case, HYDRO, 1000, EXACT, cuda)
    for k in range(3):
        assert np.array_equal(got[k], want[k]), (k, rel_err([got[k]], [want[k]]))
    assert t == pytest.approx(tw, rel=1e-15)
    fast, tf = device_run(case, HYDRO, 1000, FAST, cuda)
    assert state_err(fast, want) <= 1e-9
    assert tf == pytest.approx(tw, rel=1e-9)
