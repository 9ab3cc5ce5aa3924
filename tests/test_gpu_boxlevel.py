"""Multi-box level (same-level ghosts read from the neighbouring boxes,
physical ghosts by the BCFill rules) against the single-box level run: equal
bit for bit whatever the decomposition, both arithmetic forms."""
import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.boxlevel import BoxLevel
from hydroexa_gb300.level import Level

pytestmark = pytest.mark.gpu

DECOMPOSITIONS = {
    "quarters": [((0, 0), (47, 31)), ((48, 0), (99, 31)), ((0, 32), (23, 71)), ((24, 32), (99, 71))],
    "strips": [((0, 0), (99, 3)), ((0, 4), (99, 63)), ((0, 64), (99, 71))],
    "ragged": [((0, 0), (11, 71)), ((12, 0), (59, 19)), ((12, 20), (59, 71)), ((60, 0), (99, 51)),
               ((60, 52), (99, 71))],
}


@pytest.mark.parametrize("arith", [capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST])
@pytest.mark.parametrize("name", list(DECOMPOSITIONS))
@pytest.mark.parametrize("bc", [((0, 0), (0, 0)), ((1, 0), (0, 1))])
def test_boxlevel_equals_single_box(cuda, hxlib, arith, name, bc):
    c = workloads.fractal_dam_break(100, 72, seed=77, amplitude=1.5, nodata_frac=0.15)
    c.geom.bc_lo, c.geom.bc_hi = bc
    nsteps = 9
    bl = BoxLevel(c.geom, DECOMPOSITIONS[name], c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    assert bl.run(nsteps, c.cfl, arith) == 0
    lev = Level.from_numpy(c.geom, c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, nsteps, c.cfl, arith=arith) == 0
    assert np.array_equal(bl.gather(), lev.state.cpu().numpy())
    assert bl.time.item() == lev.time.item()


BIG_DECOMPOSITIONS = {
    "quarters": [((0, 0), (1023, 1023)), ((1024, 0), (2047, 1023)), ((0, 1024), (1023, 2047)),
                 ((1024, 1024), (2047, 2047))],
    "ragged": [((0, 0), (999, 2047)), ((1000, 0), (2047, 1039)), ((1000, 1040), (1599, 2047)),
               ((1600, 1040), (2047, 2047))],
    # boxes thinner than a tile and than its halo: a 32 x 32 tile of a 3-row box reads two boxes beyond it
    "thin": [((0, 0), (2047, 2)), ((0, 3), (6, 2047)), ((7, 3), (2047, 2044)), ((7, 2045), (2047, 2047))],
}


@pytest.mark.parametrize("arith", [capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST])
@pytest.mark.parametrize("name", list(BIG_DECOMPOSITIONS))
def test_big_boxlevel_equals_single_box(cuda, hxlib, arith, name):
    """A 2048^2 level (the persistent kernels on 32 x 32 tiles, for the boxes
    and for the single box): tiles straddling box edges are staged from the
    boxes that own their cells, partial tiles at box ends included; equal bit
    for bit."""
    c = workloads.fractal_dam_break(2048, 2048, seed=78, amplitude=1.5, nodata_frac=0.15)
    c.geom.bc_lo, c.geom.bc_hi = (0, 1), (1, 0)
    nsteps = 3
    bl = BoxLevel(c.geom, BIG_DECOMPOSITIONS[name], c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    assert bl.run(nsteps, c.cfl, arith) == 0
    lev = Level.from_numpy(c.geom, c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, nsteps, c.cfl, arith=arith) == 0
    assert np.array_equal(bl.gather(), lev.state.cpu().numpy())
    assert bl.time.item() == lev.time.item()


def test_boxlevel_rejects_gaps_and_overlaps(cuda, hxlib):
    c = workloads.dam_break(64, 48)
    with pytest.raises(capi.HxError):
        BoxLevel(c.geom, [((0, 0), (31, 47)), ((33, 0), (63, 47))], c.h, c.hu, c.hv, c.z, c.n, device=cuda)
    with pytest.raises(capi.HxError):
        BoxLevel(c.geom, [((0, 0), (40, 47)), ((32, 0), (63, 47))], c.h, c.hu, c.hv, c.z, c.n, device=cuda)
