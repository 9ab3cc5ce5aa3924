"""The reference's HDF5 input schema (src/io/IOHandler.cpp:127-307,
src/state/AmrMeshState_Init.cpp:125-173, AmrMeshState_AMR.cpp:75-105) on
in-memory datasets: metadata defaults, hyperslab placement with the
out-of-file fill, and the free-surface rebuild of the state.  No HDF5 library
is needed (h5py is absent on both machines this runs on); the file reader
itself is checked only for its error when h5py is missing."""
import importlib.util

import numpy as np
import pytest

from hydroexa_gb300 import hdf5_input as hi


def test_metadata_defaults_and_attributes():
    m = hi.metadata((2, 6, 10), {})
    assert (m.global_nx, m.global_ny, m.dx, m.dy) == (10, 6, 1.0, 1.0)
    assert (m.prob_lo_x, m.prob_lo_y, m.prob_hi_x, m.prob_hi_y) == (0.0, 0.0, 10.0, 6.0)
    m = hi.metadata((2, 6, 10), {"dx": np.array([0.25])})  # dy defaults to dx
    assert (m.dx, m.dy, m.prob_hi_x, m.prob_hi_y) == (0.25, 0.25, 2.5, 1.5)
    m = hi.metadata((2, 6, 10), {"dx": 0.5, "dy": 2.0, "x_ll": -1.0, "y_ll": 3.0})
    assert (m.prob_lo_x, m.prob_lo_y, m.prob_hi_x, m.prob_hi_y) == (-1.0, 3.0, 4.0, 15.0)


def test_read_components_fills_outside_the_file():
    rng = np.random.default_rng(3)
    ds = rng.normal(size=(3, 5, 7))
    box = ((-2, -1), (8, 3))  # sticks out on the left, right and bottom
    got = hi.read_components(ds, box, 1, 2, -9999.0)
    assert got.shape == (2, 5, 11)
    for c in range(2):
        for j in range(-1, 4):
            for i in range(-2, 9):
                inside = 0 <= i < 7 and 0 <= j < 5
                want = ds[1 + c, j, i] if inside else -9999.0
                assert got[c, j + 1, i + 2] == want
    # a box wholly outside reads nothing
    assert np.all(hi.read_components(ds, ((20, 20), (22, 21)), 0, 3, 0.0) == 0.0)
    with pytest.raises(ValueError):
        hi.read_components(ds, box, 2, 2, 0.0)  # components past the end
    with pytest.raises(ValueError):
        hi.read_components(ds[0], box, 0, 1, 0.0)  # not 3-D


def test_level_from_datasets_rebuilds_the_state_through_eta():
    """A lake at rest over a Gaussian bump (as the reference's own test input
    generator builds it: h = H - z, no momentum, roughness 0) with a NODATA
    patch: the depth comes back as max(0, (h + z) - z), NODATA cells dry with
    z = n = -9999, momenta as stored, geometry from the terrain's attributes."""
    ny, nx = 16, 64
    dx = 10.0 / nx
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    X, Y = np.meshgrid(x, y)
    z = 0.002 * np.exp(-((X - 5.0) ** 2 + (Y - 0.5 * ny * dx) ** 2) / 2.0)
    terrain = np.stack([z, np.zeros_like(z)])
    fluid = np.stack([0.010 - z, np.zeros_like(z), 0.3 * np.ones_like(z)])
    terrain[:, 2:5, 10:14] = -9999.0
    fluid[0, 2:5, 10:14] = 0.0
    lv = hi.level_from_datasets(terrain, fluid, {"dx": dx, "dy": dx, "x_ll": 0.0, "y_ll": 0.0}, (2, 2), (0, 1))
    assert (lv.geom.nx, lv.geom.ny, lv.geom.dx, lv.geom.dy) == (nx, ny, dx, dx)
    assert lv.geom.bc_lo == (2, 2) and lv.geom.bc_hi == (0, 1)
    live = terrain[1] != -9999.0
    assert np.array_equal(lv.h[live], np.maximum(0.0, (fluid[0] + z) - z)[live])
    assert np.all(lv.h[~live] == 0.0) and np.all(lv.z[~live] == -9999.0) and np.all(lv.n[~live] == -9999.0)
    assert np.array_equal(lv.hu, fluid[1]) and np.array_equal(lv.hv, fluid[2])
    assert np.abs((lv.h + lv.z)[live] - 0.010).max() < 1e-15
    for a in (lv.h, lv.hu, lv.hv, lv.z, lv.n):
        assert a.shape == (ny, nx) and a.dtype == np.float64 and a.flags.c_contiguous


def test_level_from_datasets_checks_components():
    t = np.zeros((3, 4, 4))
    f = np.zeros((3, 4, 4))
    with pytest.raises(ValueError):
        hi.level_from_datasets(t, f, {})
    with pytest.raises(ValueError):
        hi.level_from_datasets(np.zeros((2, 4, 4)), np.zeros((2, 4, 4)), {})


@pytest.mark.skipif(importlib.util.find_spec("h5py") is not None, reason="h5py is installed")
def test_open_input_names_the_missing_reader(tmp_path):
    with pytest.raises(ImportError, match="h5py"):
        hi.open_input(tmp_path / "input.h5")
