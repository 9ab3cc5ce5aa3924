"""Batched ensemble (hx_ensemble_run_f64) against per-member level runs.

Per member the ensemble does exactly the arithmetic of hx_level_run_f64 with
the same arithmetic form, whatever the tile shape, so results must be equal;
a member whose CFL bound collapses stops alone."""
import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.ensemble import Ensemble, autotune
from hydroexa_gb300.level import Level

pytestmark = pytest.mark.gpu


def members():
    out = [workloads.dam_break(48, 48), workloads.fractal_dam_break(64, 32, seed=71, amplitude=1.0),
           workloads.fractal_dam_break(100, 70, seed=72, amplitude=2.0, nodata_frac=0.2),
           workloads.lake_at_rest(128, 128, seed=73, nodata_frac=0.0), workloads.dam_break(37, 53, x_dam=0.4)]
    out[4].geom.bc_lo, out[4].geom.bc_hi = (1, 0), (0, 1)
    return out


@pytest.mark.parametrize("arith", [capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST])
@pytest.mark.parametrize("shape", [capi.HX_TILE_32x8, capi.HX_TILE_16x16, capi.HX_TILE_64x4, capi.HX_TILE_32x32])
def test_ensemble_equals_member_runs(cuda, hxlib, arith, shape):
    cases = members()
    nsteps = 13  # two graph periods of six steps plus one direct launch
    ens = Ensemble(cases, device=cuda, shapes=[shape] * len(cases))
    st = ens.run(nsteps, 0.45, arith=arith, use_graph=True)
    assert st == [0] * len(cases)
    for k, c in enumerate(cases):
        lev = Level.from_numpy(c.geom, c.h, c.hu, c.hv, c.z, c.n, device=cuda)
        assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, nsteps, 0.45, arith=arith) == 0
        assert torch.equal(ens.levels[k].state, lev.state), (k, shape)
        assert ens.time[k].item() == lev.time.item()


def test_ensemble_without_graph_and_mixed_shapes(cuda, hxlib):
    """Mixed shapes, the 32 x 32 members in the step's second launch among them,
    with and without graphs: the same states."""
    cases = members()
    a = Ensemble(cases, device=cuda, shapes=[0, 1, 2, 1, 0])
    b = Ensemble(cases, device=cuda, shapes=[2, 2, 0, 0, 1])
    c = Ensemble(cases, device=cuda, shapes=[3, 1, 3, 0, 3])
    assert a.run(8, 0.45, use_graph=False) == [0] * 5
    assert b.run(8, 0.45, use_graph=True) == [0] * 5
    assert c.run(8, 0.45, use_graph=False) == [0] * 5
    for x, y, z in zip(a.states(), b.states(), c.states()):
        assert torch.equal(x, y) and torch.equal(x, z)
    d = Ensemble(cases, device=cuda, shapes=[3, 3, 0, 3, 2])
    assert d.run(13, 0.45, use_graph=True) == [0] * 5
    e = Ensemble(cases, device=cuda, shapes=[0] * 5)
    assert e.run(13, 0.45, use_graph=True) == [0] * 5
    for x, y in zip(d.states(), e.states()):
        assert torch.equal(x, y)


def test_collapse_stays_with_its_member(cuda, hxlib):
    cases = members()
    cases[1].hu[3, 4] = 1.0e15  # velocity explosion in member 1 only
    ens = Ensemble(cases, device=cuda)
    st = ens.run(7, 0.45)
    assert st[1] & capi.HX_STATUS_DT_COLLAPSE
    assert all(s == 0 for k, s in enumerate(st) if k != 1)
    c = cases[2]
    lev = Level.from_numpy(c.geom, c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 7, 0.45, arith=capi.HX_ARITH_FAST)
    assert torch.equal(ens.levels[2].state, lev.state)


def test_autotune_picks_a_shape_per_class(cuda, hxlib, tmp_path, monkeypatch):
    monkeypatch.setenv("HX_CACHE_DIR", str(tmp_path))
    cases = workloads.ensemble(count=12, seed=9, smax=512)
    per_class, report = autotune(cases, device=cuda, steps=6)
    assert len(per_class) == 3 and all(s in (0, 1, 2, 3) for s in per_class)
    again, _ = autotune(cases, device=cuda, steps=6)  # served from the cache
    assert again == per_class
    assert np.isfinite(list(report["timings_ms"].values())).all()
