"""Native (AMReX HyperCLaw-V1.1) plotfiles of levels held as torch CUDA tensors.

``write_plotfile`` mirrors WriteNativePlotfile (src/io/NativePlotFile.cpp:19-97):
the state (h, hu, hv) and the terrain (z, Manning n) of every box of every level
as variables h_fluid, hu_momentum, hv_momentum, z_bathymetry, extra_comp_4, in
the directory ``<prefix><iteration:05d>``.  The copies and the files are made by
the C ABI (``hx_write_plotfile_f64``).  ``read_plotfile`` parses such a
directory back into numpy arrays (one per box and level).
"""
from __future__ import annotations

import ctypes
import re
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import capi

VARIABLES = ("h_fluid", "hu_momentum", "hv_momentum", "z_bathymetry", "extra_comp_4")


@dataclass
class PlotBox:
    """One box: state (3, ny, nx) and terrain (2, ny, nx) FP64 CUDA tensors whose
    element [c, 0, 0] is cell ``lo`` of the level's index space."""
    state: torch.Tensor
    terrain: torch.Tensor
    lo: tuple = (0, 0)


@dataclass
class PlotLevel:
    boxes: list
    domain_lo: tuple
    domain_hi: tuple
    dx: float
    dy: float
    ref_ratio: int = 2
    istep: int = 0


def write_plotfile(prefix: str, iteration: int, time: float, levels: list, prob_lo=(0.0, 0.0),
                   prob_hi=(1.0, 1.0), stream=None) -> Path:
    keep = []
    lv = (capi.PlotLevelF64 * len(levels))()
    for l, L in enumerate(levels):
        arr = (capi.PlotBoxF64 * len(L.boxes))()
        for k, b in enumerate(L.boxes):
            S, T = b.state, b.terrain
            if S.dtype != torch.float64 or T.dtype != torch.float64 or not S.is_cuda or not T.is_cuda:
                raise TypeError("plotfile boxes are FP64 CUDA tensors")
            if not (S.is_contiguous() and T.is_contiguous()) or S.shape[1:] != T.shape[1:]:
                raise ValueError("state and terrain of a box must be contiguous and of one shape")
            ny, nx = S.shape[1], S.shape[2]
            a = arr[k]
            a.h, a.hu, a.hv = S[0].data_ptr(), S[1].data_ptr(), S[2].data_ptr()
            a.z, a.n = T[0].data_ptr(), T[1].data_ptr()
            a.pitch = nx
            a.lo[0], a.lo[1] = int(b.lo[0]), int(b.lo[1])
            a.hi[0], a.hi[1] = int(b.lo[0]) + nx - 1, int(b.lo[1]) + ny - 1
        keep.append(arr)
        lv[l].boxes = arr
        lv[l].nboxes = len(L.boxes)
        lv[l].domain_lo[0], lv[l].domain_lo[1] = L.domain_lo
        lv[l].domain_hi[0], lv[l].domain_hi[1] = L.domain_hi
        lv[l].dx, lv[l].dy = float(L.dx), float(L.dy)
        lv[l].ref_ratio, lv[l].istep = int(L.ref_ratio), int(L.istep)
    lo = (ctypes.c_double * 2)(*prob_lo)
    hi = (ctypes.c_double * 2)(*prob_hi)
    dev = levels[0].boxes[0].state.device
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    capi.check(capi.lib().hx_write_plotfile_f64(str(prefix).encode(), int(iteration), float(time), len(levels), lv,
                                                lo, hi, ctypes.c_void_p(s.cuda_stream)), "hx_write_plotfile_f64")
    return Path("%s%05d" % (prefix, iteration))


_BOX = re.compile(r"\(\((-?\d+),(-?\d+)\) \((-?\d+),(-?\d+)\) \((\d+),(\d+)\)\)")
_FAB = re.compile(rb"^FAB \(\(8, \(64 11 52 0 1 12 0 1023\)\),\(8, \(8 7 6 5 4 3 2 1\)\)\)"
                  rb"\(\((-?\d+),(-?\d+)\) \((-?\d+),(-?\d+)\) \(0,0\)\) (\d+)\n")


def read_plotfile(path) -> dict:
    """Header fields and, per level, the boxes [(lo, hi, array (ncomp, ny, nx))]
    of a 2-D FP64 little-endian plotfile."""
    path = Path(path)
    lines = (path / "Header").read_text().split("\n")
    it = iter(lines)
    out = {"version": next(it)}
    nvar = int(next(it))
    out["variables"] = [next(it) for _ in range(nvar)]
    out["dim"] = int(next(it))
    out["time"] = float(next(it))
    finest = int(next(it))
    out["prob_lo"] = [float(x) for x in next(it).split()]
    out["prob_hi"] = [float(x) for x in next(it).split()]
    out["ref_ratio"] = [int(x) for x in next(it).split()]
    out["domains"] = [tuple(int(g) for g in m.groups()[:4]) for m in _BOX.finditer(next(it))]
    out["steps"] = [int(x) for x in next(it).split()]
    out["cell_size"] = [[float(x) for x in next(it).split()] for _ in range(finest + 1)]
    out["coord_sys"] = int(next(it))
    out["bwidth"] = int(next(it))
    levels = []
    for _ in range(finest + 1):
        lev, nb, t = next(it).split()
        step = int(next(it))
        extents = [[[float(x) for x in next(it).split()] for _ in range(out["dim"])] for _ in range(int(nb))]
        prefix = next(it)
        cell_h = (path / (prefix + "_H")).read_text().split("\n")
        nbox = int(cell_h[4][1:].split()[0])
        boxes = [tuple(int(g) for g in _BOX.match(cell_h[5 + k]).groups()[:4]) for k in range(nbox)]
        fod = [ln.split() for ln in cell_h if ln.startswith("FabOnDisk:")]
        arrays = []
        for (lo0, lo1, hi0, hi1), (_, fname, off) in zip(boxes, fod):
            raw = (path / prefix).parent.joinpath(fname).read_bytes()
            m = _FAB.match(raw[int(off):int(off) + 200])
            if m is None:
                raise ValueError("unexpected FAB header")
            ncomp = int(m.group(5))
            nx, ny = hi0 - lo0 + 1, hi1 - lo1 + 1
            start = int(off) + m.end()
            data = np.frombuffer(raw, dtype="<f8", count=ncomp * nx * ny, offset=start).reshape(ncomp, ny, nx)
            if (int(m.group(1)), int(m.group(2)), int(m.group(3)), int(m.group(4))) != (lo0, lo1, hi0, hi1):
                raise ValueError("FAB box differs from the FabArray header")
            arrays.append(((lo0, lo1), (hi0, hi1), data.copy()))
        levels.append({"level": int(lev), "time": float(t), "step": step, "extents": extents, "boxes": arrays,
                       "cell_h": cell_h})
    out["levels"] = levels
    return out


__all__ = ["PlotBox", "PlotLevel", "write_plotfile", "read_plotfile", "VARIABLES"]
