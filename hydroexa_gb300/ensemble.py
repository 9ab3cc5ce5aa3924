"""Batched ensemble of independent scenarios on one GPU.

``Ensemble`` holds many single-box levels (any sizes) in HBM and advances them
all with ``hx_ensemble_run_f64``: one persistent launch per step over a tile
queue spanning every member, each member with its own dt chain, steps replayed
from a CUDA graph.  ``plain_loop`` is the comparison: the same members advanced
one after another by the per-level path, with the host reading each member's
CFL bound every step (the reference's ``compute_dt`` + ``compute_fluxes``
pattern).  ``autotune`` picks the tile shape per size class by timing (256-cell tiles on
256-thread blocks, or 32 x 32 tiles on 1024-thread blocks, which the large
members run in a second launch of the step).
"""
from __future__ import annotations

import ctypes
import json
import os
from pathlib import Path

import torch

from . import capi
from .level import Level

SHAPES = (capi.HX_TILE_32x8, capi.HX_TILE_16x16, capi.HX_TILE_64x4, capi.HX_TILE_32x32)
SHAPE_NAMES = {capi.HX_TILE_32x8: "32x8", capi.HX_TILE_16x16: "16x16", capi.HX_TILE_64x4: "64x4",
               capi.HX_TILE_32x32: "32x32"}
# size classes by level side: small, medium, large
CLASS_EDGES = (128, 384)


def size_class(side: int) -> int:
    return 0 if side <= CLASS_EDGES[0] else (1 if side <= CLASS_EDGES[1] else 2)


class Ensemble:
    """Members: workloads.Case objects (FP64), resident on one device."""

    def __init__(self, cases, device="cuda", shapes=None):
        self.device = torch.device(device)
        self.cases = list(cases)
        self.levels = [Level.from_numpy(c.geom, c.h, c.hu, c.hv, c.z, c.n, device=self.device) for c in self.cases]
        n = len(self.levels)
        self.status = torch.zeros(n, dtype=torch.int32, device=self.device)
        self.time = torch.zeros(n, dtype=torch.float64, device=self.device)
        self.work = torch.zeros(int(capi.lib().hx_ensemble_work_bytes(n)), dtype=torch.uint8, device=self.device)
        self.shapes = list(shapes) if shapes is not None else [capi.HX_TILE_32x8] * n

    @property
    def cells(self) -> int:
        return sum(c.cells for c in self.cases)

    def set_shapes_by_class(self, per_class):
        self.shapes = [per_class[size_class(c.geom.nx)] for c in self.cases]

    def _members(self):
        arr = (capi.EnsembleMemberF64 * len(self.levels))()
        for k, lev in enumerate(self.levels):
            arr[k].level = lev._desc(lev.state)
            arr[k].h_alt = lev.alt[0].data_ptr()
            arr[k].hu_alt = lev.alt[1].data_ptr()
            arr[k].hv_alt = lev.alt[2].data_ptr()
            arr[k].tile_shape = self.shapes[k]
        return arr

    def tiles(self) -> int:
        t = ctypes.c_int64()
        capi.check(capi.lib().hx_ensemble_tiles(len(self.levels), self._members(), ctypes.byref(t)), "tiles")
        return int(t.value)

    def run(self, nsteps: int, cfl: float, arith=capi.HX_ARITH_FAST, use_graph=True, stream=None,
            check_status=True):
        """Advance every member nsteps; returns the per-member status bits (if checked)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        self.status.zero_()
        fin = ctypes.c_int(0)
        capi.check(capi.lib().hx_ensemble_run_f64(
            len(self.levels), self._members(), nsteps, cfl, ctypes.c_void_p(self.work.data_ptr()),
            ctypes.c_void_p(self.status.data_ptr()), ctypes.c_void_p(self.time.data_ptr()), arith,
            1 if use_graph else 0, ctypes.byref(fin), ctypes.c_void_p(s.cuda_stream)), "hx_ensemble_run_f64")
        if fin.value:
            for lev in self.levels:
                lev.state, lev.alt = lev.alt, lev.state
        if check_status:
            return self.status.cpu().tolist()
        return None

    def plain_loop(self, nsteps: int, cfl: float, arith=capi.HX_ARITH_FAST, stream=None):
        """The comparison path: members one after another, each step = host
        read of the member's CFL bound (compute_dt) + one advance."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        for lev in self.levels:
            for _ in range(nsteps):
                mn, _ = lev.compute_dt(stream=s)
                out = lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, mn * cfl, out=lev.alt, arith=arith, stream=s)
                lev.state, lev.alt = out, lev.state

    def member_loop(self, nsteps: int, cfl: float, arith=capi.HX_ARITH_FAST, stream=None):
        """The members one after another, each with the per-level device time
        loop hx_level_run_f64 (no host round trip inside a member's run)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        for lev in self.levels:
            lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, nsteps, cfl, arith=arith, stream=s, check_status=False)

    def states(self):
        return [lev.state for lev in self.levels]


def _cache_path() -> Path:
    root = Path(os.environ.get("HX_CACHE_DIR", Path.home() / ".cache" / "hydroexa_gb300"))
    return root / "ensemble_tiles.json"


def autotune(cases, device="cuda", steps=6, cfl=0.45, use_cache=True, verbose=False):
    """Tile shape per size class (small/medium/large side), chosen by timing the
    ensemble kernel on the members of each class with every candidate shape.
    Results are cached per GPU name."""
    dev = torch.device(device)
    # the candidate set is part of the key: a cache written for other shapes is not reused
    key = "%s|%s" % (torch.cuda.get_device_name(dev), ",".join(SHAPE_NAMES[x] for x in SHAPES))
    path = _cache_path()
    if use_cache and path.exists():
        try:
            cached = json.loads(path.read_text()).get(key)
            if cached:
                return [int(x) for x in cached["per_class"]], cached
        except (ValueError, KeyError):
            pass
    per_class = []
    report = {"per_class": [], "timings_ms": {}}
    for cls in range(3):
        members = [c for c in cases if size_class(c.geom.nx) == cls]
        if not members:
            per_class.append(capi.HX_TILE_32x8)
            continue
        best, best_ms = None, None
        for shape in SHAPES:
            ens = Ensemble(members, device=dev, shapes=[shape] * len(members))
            ens.run(steps, cfl)  # warm-up (also compiles the graph path)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s = torch.cuda.current_stream(dev)
            e0.record(s)
            ens.run(steps, cfl, check_status=False)
            e1.record(s)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            report["timings_ms"]["%d:%s" % (cls, SHAPE_NAMES[shape])] = ms
            if verbose:
                print("class", cls, SHAPE_NAMES[shape], ms)
            if best_ms is None or ms < best_ms:
                best, best_ms = shape, ms
            del ens
        per_class.append(best)
    report["per_class"] = per_class
    if use_cache:
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            data = json.loads(path.read_text()) if path.exists() else {}
            data[key] = report
            path.write_text(json.dumps(data, indent=1))
        except OSError:
            pass
    return per_class, report
