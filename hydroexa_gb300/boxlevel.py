"""A level given as several boxes (a same-level BoxArray), advanced without
ghost filling: hx_boxlevel_run_f64 reads every ghost from the box that owns
the cell (or from the physical-boundary rule), one launch per step over the
tiles of all boxes."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi
from .level import Geometry


class BoxLevel:
    """boxes: list of ((x0, y0), (x1, y1)) inclusive cell boxes that tile the domain."""

    def __init__(self, geom: Geometry, boxes, h, hu, hv, z, n, device="cuda"):
        self.geom = geom
        self.boxes = [tuple(map(tuple, b)) for b in boxes]
        self.device = torch.device(device)
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(self.device)
        self.state, self.alt, self.terrain = [], [], []
        for (x0, y0), (x1, y1) in self.boxes:
            sl = (slice(y0, y1 + 1), slice(x0, x1 + 1))
            self.state.append(T(np.stack([h[sl], hu[sl], hv[sl]])))
            self.alt.append(torch.empty_like(self.state[-1]))
            self.terrain.append(T(np.stack([z[sl], n[sl]])))
        self.desc = (capi.LevelBoxF64 * len(self.boxes))()
        for k, ((x0, y0), (x1, y1)) in enumerate(self.boxes):
            d = self.desc[k]
            s, a, t = self.state[k], self.alt[k], self.terrain[k]
            d.h, d.hu, d.hv = (s[c].data_ptr() for c in range(3))
            d.h_alt, d.hu_alt, d.hv_alt = (a[c].data_ptr() for c in range(3))
            d.z, d.n = t[0].data_ptr(), t[1].data_ptr()
            d.pitch = x1 - x0 + 1
            d.lo[0], d.lo[1], d.hi[0], d.hi[1] = x0, y0, x1, y1
        L = capi.lib()
        nbytes = L.hx_boxlevel_work_bytes(len(self.boxes), self.desc, geom.nx, geom.ny)
        if nbytes <= 0:
            raise capi.HxError("boxlevel: " + capi.lib().hx_last_error().decode())
        self.work = torch.empty(int(nbytes), dtype=torch.uint8, device=self.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.time = torch.zeros(1, dtype=torch.float64, device=self.device)

    def run(self, nsteps: int, cfl: float, arith: int = capi.HX_ARITH_EXACT) -> int:
        g = self.geom
        lo = (ctypes.c_int32 * 2)(*g.bc_lo)
        hi = (ctypes.c_int32 * 2)(*g.bc_hi)
        fin = ctypes.c_int(0)
        self.status.zero_()
        capi.check(capi.lib().hx_boxlevel_run_f64(
            len(self.boxes), self.desc, g.nx, g.ny, g.dx, g.dy, lo, hi, nsteps, cfl, arith,
            ctypes.c_void_p(self.work.data_ptr()), ctypes.c_void_p(self.status.data_ptr()),
            ctypes.c_void_p(self.time.data_ptr()), ctypes.byref(fin),
            ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)), "hx_boxlevel_run_f64")
        if fin.value:  # the result is in the second state: swap the roles (descriptors included)
            self.state, self.alt = self.alt, self.state
            for k in range(len(self.boxes)):
                d = self.desc[k]
                d.h, d.h_alt = d.h_alt, d.h
                d.hu, d.hu_alt = d.hu_alt, d.hu
                d.hv, d.hv_alt = d.hv_alt, d.hv
        return int(self.status.item())

    def gather(self) -> np.ndarray:
        """The current state as one (3, ny, nx) array."""
        out = np.zeros((3, self.geom.ny, self.geom.nx))
        for ((x0, y0), (x1, y1)), s in zip(self.boxes, self.state):
            out[:, y0:y1 + 1, x0:x1 + 1] = s.cpu().numpy()
        return out
