"""Host-side logic that needs no GPU: inputs-file parameters, the multi-level
dt protocol of BaseSolver::compute_dt, solver selection errors, and the seeded
workload generators."""
import numpy as np
import pytest

from hydroexa_gb300 import params, workloads
from hydroexa_gb300.solver import BaseSolver, HydroExaAbort, HydrostaticRoe, Roe, SolverVariant, make_solver

INPUTS = """
# a two-level lake at rest
HydroEXA.max_time          = 30.0
HydroEXA.model             = "HydrostaticRoe"   # well balanced
HydroEXA.cfl               = 0.45
HydroEXA.h_grad_thresh     = 0.5 0.25
HydroEXA.umag_grad_thresh  = 1.0 1.0
HydroEXA.z_grad_thresh     = 2.0 2.0
HydroEXA.lo_bc             = 1 0
HydroEXA.hi_bc             = 0 1
amr.max_level              = 1
amr.do_subcycle            = 0
amr.blocking_factor        = 16
io.plot_freq               = -1
io.input_file              = "lake.h5"
"""


def test_parameters_keys_and_defaults():
    p = params.read_parameters(INPUTS)
    assert p.physics.model == "HydrostaticRoe" and p.physics.cfl == 0.45
    assert p.physics.h_grad_thresh == [0.5, 0.25]
    assert p.physics.bc_params.lo_bc == [1, 0] and p.physics.bc_params.hi_bc == [0, 1]
    assert p.amr.max_amr_level == 1 and p.amr.do_subcycle == 0 and p.amr.blocking_factor == 16
    assert p.amr.do_reflux == 1 and p.amr.regrid_int == 2  # Params.H defaults
    assert p.io.input_file == "lake.h5" and p.io.plot_freq == -1.0
    assert p.runtime.max_time == 30.0 and p.runtime.log_progress_every == 10
    d = params.read_parameters("HydroEXA.cfl = 0.3\n")
    assert d.physics.model == "Roe" and d.physics.bc_params.lo_bc == [0, 0]
    with pytest.raises(ValueError):
        params.read_parameters("amr.blocking_factor = 0\n")


class FakeSolver(BaseSolver):
    def __init__(self, per_level):
        self.per_level = per_level

    def compute_dt_level(self, U, terrain, geom, lev, cfl):
        return self.per_level[lev] * cfl


def test_multilevel_dt_protocol():
    """BaseSolver.H:120-165: project every level's bound to level 0 through the
    product of ratios, take the minimum, then divide down by the ratios."""
    s = FakeSolver([1.0, 0.3, 0.2])
    dt = []
    s.compute_dt(dt, None, None, None, [(2, 2), (2, 2)], 2, 0.5)
    assert dt[0] == pytest.approx(min(0.5, 0.3 * 0.5 * 2, 0.2 * 0.5 * 4))
    assert dt[1] == dt[0] / 2 and dt[2] == dt[1] / 2
    s = FakeSolver([0.1, 10.0])
    dt = [0.0, 0.0]
    s.compute_dt(dt, None, None, None, [(4, 4)], 1, 1.0)
    assert dt == [0.1, 0.025]


def test_solver_selection_and_errors():
    assert isinstance(make_solver("Roe")._s, Roe)
    assert isinstance(make_solver("HydrostaticRoe")._s, HydrostaticRoe)
    with pytest.raises(HydroExaAbort, match="Unknown solver type"):
        make_solver("RoeExnerACM")
    v = SolverVariant()
    assert not v.has_solver()
    with pytest.raises(RuntimeError, match="Solver not initialized"):
        v.compute_dt([], None, None, None, [], 0, 0.5)
    with pytest.raises(HydroExaAbort, match="dt collapsed"):
        HydrostaticRoe()._dt_collapse(0, 1e-13, 1e9)
    Roe()._dt_collapse(0, 1e-13, 1e9)  # logged, not fatal (Roe.cpp:88-92)


def test_workloads_are_seeded_and_shaped():
    a = workloads.fractal_dam_break(256, 128, seed=3)
    b = workloads.fractal_dam_break(256, 128, seed=3)
    assert np.array_equal(a.z, b.z) and np.array_equal(a.h, b.h)
    nod = a.z == workloads.NODATA
    assert 0.18 < nod.mean() < 0.22
    assert np.all(a.n[nod] == workloads.NODATA) and np.all(a.h[nod] == 0.0)
    valid = a.z[~nod]
    assert valid.min() >= 0.0 and valid.max() <= 5.0 + 1e-12
    inside = a.h[~nod]
    assert set(np.unique(inside)) <= {0.5, 2.0}
    lake = workloads.lake_at_rest(128, 128, seed=2)
    assert 0.08 < (lake.z == workloads.NODATA).mean() < 0.12
    ok = lake.z != workloads.NODATA
    assert np.allclose((lake.h + lake.z)[ok & (lake.h > 0)], 1.0)
    ens = workloads.ensemble(count=16, seed=4)
    sides = [c.geom.nx for c in ens]
    assert all(64 <= s <= 1024 and s % 16 == 0 for s in sides)
    case, gauges = workloads.adjoint_case(64, 64, ngauges=16)
    assert len(set(gauges.tolist())) == 16 and np.abs(case.z).max() == pytest.approx(0.3)


def test_binomial_schedule_recomputes_the_optimal_number_of_steps(hxlib):
    """hx_adjoint_recompute_steps under binomial checkpointing equals an
    exhaustive optimum of the recursive schedule, less the steps the forward
    sweep advances while it places the first snapshots."""
    from functools import lru_cache

    @lru_cache(None)
    def opt(n, free):  # least forward steps to reverse n steps from a stored state with `free` spare slots
        if n <= 1:
            return 0
        if free == 0:
            return n * (n - 1) // 2
        return min(m + opt(n - m, free - 1) + opt(m, free) for m in range(1, n))

    def split(n, c):  # the optimal first advance (c slots including the start state)
        return min(range(1, n), key=lambda m: (m + opt(n - m, c - 2) + opt(m, c - 1), m))

    def chain_last(n, c):
        a = 0
        while n > 1 and c > 1:
            k = split(n, c)
            a, n, c = a + k, n - k, c - 1
        return a

    L = hxlib.lib()
    for n in (1, 2, 3, 7, 20, 41, 64):
        for c in (2, 3, 4, 6, 9):
            cc = min(c, n + 1)
            got = L.hx_adjoint_recompute_steps(n, -c)
            assert got == opt(n, cc - 1) - chain_last(n, cc), (n, c, got)
    assert L.hx_adjoint_recompute_steps(30, 0) == 0
    assert L.hx_adjoint_recompute_steps(30, 7) == 30
    assert L.hx_adjoint_recompute_steps(30, 31) == 0
