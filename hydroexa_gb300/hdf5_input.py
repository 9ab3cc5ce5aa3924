"""The reference's HDF5 input schema, read into a single-box level.

The reference reads its initial condition from one HDF5 file
(src/io/IOHandler.cpp, src/state/AmrMeshState_Init.cpp:125-173):

- dataset ``terrain``, shape (2, ny, nx): bed elevation z and Manning n, with
  -9999 marking NODATA cells (IOHandler.cpp:127-228 reads it with NODATA
  -9999 outside the file);
- dataset ``fluid``, shape (3, ny, nx): depth h and momenta hu, hv (0 outside
  the file);
- attributes of ``terrain``: ``dx``, ``dy`` (defaulting to ``dx``), ``x_ll``,
  ``y_ll`` (defaulting to 0); the domain is the dataset's extent and its upper
  corner is ``x_ll + nx dx``, ``y_ll + ny dy`` (IOHandler.cpp:230-307).

The static fields become the level's state through the free surface: eta = z
on cells whose second terrain component is NODATA, h + z elsewhere, then
h = max(0, eta - z) (AmrMeshState_AMR.cpp:75-105, the level at the file's own
resolution), momenta as read.

The schema logic here (metadata, hyperslab placement with the out-of-file
fill, the free-surface rebuild) works on any array-like that numpy can slice,
so it is tested without an HDF5 library.  Opening an ``.h5`` file needs
``h5py``, which is imported on demand; without it ``open_input`` raises
ImportError naming the missing package.  A caller holding the datasets in
memory (or in another container format) passes them as a mapping.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Mapping

import numpy as np

from .level import Geometry

NODATA = -9999.0


@dataclass
class SpatialMetadata:
    """HDF5SpatialMetadata (include/io/IOHandler.H:45-55)."""
    global_nx: int = 0
    global_ny: int = 0
    dx: float = 1.0
    dy: float = 1.0
    prob_lo_x: float = 0.0
    prob_lo_y: float = 0.0
    prob_hi_x: float = 1.0
    prob_hi_y: float = 1.0


def _attr(attrs: Mapping, key: str):
    if key not in attrs:
        return None
    v = np.asarray(attrs[key], dtype=np.float64).reshape(-1)
    if v.size < 1:
        raise ValueError(f"attribute {key!r} is empty")
    return float(v[0])


def metadata(shape, attrs: Mapping) -> SpatialMetadata:
    """ReadHDF5Metadata (IOHandler.cpp:230-307) for a dataset of ``shape``
    (..., ny, nx) with attributes ``attrs``: dx defaults to 1, dy to dx, x_ll
    and y_ll to 0; the upper corner follows from the extent."""
    if len(shape) < 2:
        raise ValueError("the dataset needs at least two dimensions (ny, nx)")
    ny, nx = int(shape[-2]), int(shape[-1])
    dx = _attr(attrs, "dx")
    dx = 1.0 if dx is None else dx
    dy = _attr(attrs, "dy")
    dy = dx if dy is None else dy
    x_ll = _attr(attrs, "x_ll") or 0.0
    y_ll = _attr(attrs, "y_ll") or 0.0
    return SpatialMetadata(nx, ny, dx, dy, x_ll, y_ll, x_ll + nx * dx, y_ll + ny * dy)


def read_components(ds, box, first_comp: int, ncomp: int, nodata: float) -> np.ndarray:
    """ReadHDF5HyperslabComponents (IOHandler.cpp:127-228): components
    first_comp .. first_comp + ncomp - 1 of the 3-D dataset ``ds`` (ncomp_all,
    ny, nx) over the cell box ``box`` = ((i_lo, j_lo), (i_hi, j_hi)), as an
    array (ncomp, j_hi - j_lo + 1, i_hi - i_lo + 1).  Only the part of the box
    inside the file is read (one hyperslab); cells outside it take ``nodata``."""
    shape = tuple(int(s) for s in ds.shape)
    if len(shape) != 3:
        raise ValueError("read_components expects a 3-D dataset (ncomp, ny, nx)")
    if first_comp < 0 or ncomp < 1 or first_comp + ncomp > shape[0]:
        raise ValueError("component range outside the dataset")
    (i_lo, j_lo), (i_hi, j_hi) = box
    if i_hi < i_lo or j_hi < j_lo:
        raise ValueError("empty box")
    out = np.full((ncomp, j_hi - j_lo + 1, i_hi - i_lo + 1), nodata, dtype=np.float64)
    h5_ny, h5_nx = shape[1], shape[2]
    a0, a1 = max(i_lo, 0), min(i_hi, h5_nx - 1)
    b0, b1 = max(j_lo, 0), min(j_hi, h5_ny - 1)
    if a0 <= a1 and b0 <= b1:
        slab = np.asarray(ds[first_comp:first_comp + ncomp, b0:b1 + 1, a0:a1 + 1], dtype=np.float64)
        out[:, b0 - j_lo:b1 - j_lo + 1, a0 - i_lo:a1 - i_lo + 1] = slab
    return out


@dataclass
class LevelInput:
    geom: Geometry
    meta: SpatialMetadata
    h: np.ndarray
    hu: np.ndarray
    hv: np.ndarray
    z: np.ndarray
    n: np.ndarray


def level_from_datasets(terrain, fluid, attrs: Mapping, bc_lo=(0, 0), bc_hi=(0, 0)) -> LevelInput:
    """The single-box level of the file's own extent and resolution: terrain
    (2, ny, nx) and fluid (3, ny, nx) read over the whole domain, the state
    rebuilt through the free surface (AmrMeshState_AMR.cpp:75-105)."""
    meta = metadata(terrain.shape, attrs)
    if tuple(terrain.shape)[0] != 2:
        raise ValueError("terrain must have 2 components (z, n)")
    if tuple(fluid.shape)[0] != 3:
        raise ValueError("fluid must have 3 components (h, hu, hv)")
    dom = ((0, 0), (meta.global_nx - 1, meta.global_ny - 1))
    T = read_components(terrain, dom, 0, 2, NODATA)  # AmrMeshState_Init.cpp:167
    U = read_components(fluid, dom, 0, 3, 0.0)       # AmrMeshState_Init.cpp:168
    z, n = T[0], T[1]
    eta = np.where(n == NODATA, z, U[0] + z)
    h = np.maximum(0.0, eta - z)
    geom = Geometry(meta.global_nx, meta.global_ny, meta.dx, meta.dy, tuple(bc_lo), tuple(bc_hi))
    return LevelInput(geom, meta, h, U[1].copy(), U[2].copy(), z.copy(), n.copy())


def open_input(path, bc_lo=(0, 0), bc_hi=(0, 0)) -> LevelInput:
    """Read the reference's HDF5 input file at ``path`` (datasets ``terrain``
    and ``fluid``, attributes on ``terrain``).  Needs h5py."""
    try:
        import h5py  # noqa: PLC0415 - optional dependency
    except ImportError as e:
        raise ImportError("reading the HDF5 input needs the h5py package, which is not installed") from e
    with h5py.File(path, "r") as f:
        return level_from_datasets(f["terrain"], f["fluid"], dict(f["terrain"].attrs), bc_lo, bc_hi)
