"""The reference solver's operator surface over the GB300 kernels.

Mirrors include/solvers/BaseSolver.H:41-193 and SolverVariant.H:45-192: the
same names, argument meaning and error behaviour, on single-box levels held as
torch CUDA tensors.  Every computation goes through the C ABI
(``hydroexa_gb300.capi``); the ghost fill of a single-box level (the physical
boundary, BCFill.H) happens inside the tile loader.  Coarse-fine ghost filling,
flux registers and regridding stay with the AMR framework (AMReX in the
reference) and are not reproduced here.

Layout: state tensors are (3, ny, nx) = (h, hu, hv), terrain (2, ny, nx) =
(z, Manning n), tags (ny, nx) int8.
"""
from __future__ import annotations

import ctypes
import logging
from dataclasses import dataclass, field

import torch

from . import capi, ranks
from .level import DtAccum, Geometry, Level, array4, box
from .params import PhysicsParameters

log = logging.getLogger("hydroexa_gb300")


class HydroExaAbort(RuntimeError):
    """Raised where the reference calls amrex::Abort."""


@dataclass
class SolverContext:
    """Per-level views the solver advances (SolverContext.H:43-118, single-box levels)."""
    U_new: list
    U_old: list
    Terrain: list
    geom: list
    t_new: list = field(default_factory=list)
    t_old: list = field(default_factory=list)
    finest_level: int = 0
    do_reflux: bool = False


def _level_view(U: torch.Tensor, T: torch.Tensor, g: Geometry) -> Level:
    lev = Level.__new__(Level)
    lev.geom, lev.state, lev.terrain = g, U, T
    lev.dtype, lev.pitch = U.dtype, U.shape[2]
    from .level import Status
    lev.status = Status(U.device)
    return lev


class BaseSolver:
    """CRTP base of the reference, as a Python base class."""

    method: int = -1
    arith: int = capi.HX_ARITH_FAST

    def __init__(self, arith: int = capi.HX_ARITH_FAST):
        self.arith = arith

    # BaseSolver.H:57-61 -- swap U_new/U_old, then advance into U_new
    def compute_fluxes(self, ctx: SolverContext, lev: int, dt: float, time: float) -> None:
        ctx.U_new[lev], ctx.U_old[lev] = ctx.U_old[lev], ctx.U_new[lev]
        U_o, U_n = ctx.U_old[lev], ctx.U_new[lev]
        lv = _level_view(U_o, ctx.Terrain[lev], ctx.geom[lev])
        lv.advance(self.method, dt, out=U_n, arith=self.arith)
        st = lv.status.read()
        if st & capi.HX_STATUS_NAN:
            raise HydroExaAbort(f"compute_fluxes: non-finite state on level {lev}")

    # BaseSolver.H:77-83 and compute_dt_Impl
    def compute_dt_level(self, U, terrain, geom, lev: int, cfl: float) -> float:
        lv = _level_view(U[lev], terrain[lev], geom[lev])
        dt_est, max_vel = lv.compute_dt()
        log.debug("[compute_dt] lev=%d dt=%g max|vel|=%g", lev, dt_est, max_vel)
        if dt_est < 1.e-12:
            self._dt_collapse(lev, dt_est, max_vel)
        return dt_est * cfl

    def _dt_collapse(self, lev, dt_est, max_vel):
        raise NotImplementedError

    # BaseSolver.H:120-165
    def compute_dt(self, dt: list, U, terrain, geom, ref_ratio, finest_level: int, cfl: float) -> None:
        dt_tmp = [self.compute_dt_level(U, terrain, geom, lev, cfl) for lev in range(finest_level + 1)]
        # 1. minimum over the ranks first (ParallelDescriptor::ReduceRealMin, BaseSolver.H:133)
        dt_tmp = ranks.reduce_real_min(dt_tmp)
        dt_0 = dt_tmp[0]
        factor = 1.0
        for lev in range(1, finest_level + 1):
            factor *= float(ref_ratio[lev - 1][0])
            dt_0 = min(dt_0, dt_tmp[lev] * factor)
        while len(dt) < finest_level + 1:
            dt.append(0.0)
        dt[0] = dt_0
        for lev in range(1, finest_level + 1):
            dt[lev] = dt[lev - 1] / float(ref_ratio[lev - 1][0])

    # BaseSolver.H:185-191 and tag_cells_Impl
    def tag_cells(self, tags: torch.Tensor, U: torch.Tensor, terrain: torch.Tensor, geom: Geometry, lev: int,
                  time: float, phys_params: PhysicsParameters, set_value: int = 2) -> None:
        """Tag the valid cells of a single-box level.  The one-cell ghost ring the
        stencil reads is generated with the level's boundary rules (the
        reference reads whatever its MultiFab ghosts hold)."""
        Ug = _pad_state(U, geom)
        Tg = _pad_terrain(terrain)
        tg = torch.zeros((geom.ny + 2, geom.nx + 2), dtype=torch.int8, device=U.device)
        tg[1:-1, 1:-1] = tags
        R = ctypes.c_double if U.dtype == torch.float64 else ctypes.c_float
        sfx = "f64" if U.dtype == torch.float64 else "f32"
        th = (phys_params.h_grad_thresh[lev], phys_params.umag_grad_thresh[lev], phys_params.z_grad_thresh[lev])
        rc = getattr(capi.lib(), f"hx_tag_box_{sfx}")(
            self.method, ctypes.byref(array4(Ug, (-1, -1))), ctypes.byref(array4(Tg, (-1, -1))),
            ctypes.byref(array4(tg, (-1, -1))), box((0, 0), (geom.nx - 1, geom.ny - 1)), R(geom.dx), R(geom.dy),
            R(time), *(R(x) for x in th), set_value, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        capi.check(rc, "hx_tag_box")
        tags.copy_(tg[1:-1, 1:-1])


def _mirror(a: torch.Tensor, dim: int, lo_rule: str, hi_rule: str) -> torch.Tensor:
    def ghost(edge_idx, mirror_idx, rule):
        if rule == "edge":
            return a.narrow(dim, edge_idx, 1)
        g = a.narrow(dim, mirror_idx, 1)
        return -g if rule == "odd" else g
    n = a.shape[dim]
    return torch.cat([ghost(0, 0, lo_rule), a, ghost(n - 1, n - 1, hi_rule)], dim=dim)


def _rule(code: int, kind: str) -> str:
    if code != 0:
        return "edge"
    return "odd" if kind == "normal" else "even"


def _pad_state(U, g: Geometry):
    out = []
    for c, (kx, ky) in enumerate((("scalar", "scalar"), ("normal", "tangential"), ("tangential", "normal"))):
        p = _mirror(U[c], 1, _rule(g.bc_lo[0], kx), _rule(g.bc_hi[0], kx))
        p = _mirror(p, 0, _rule(g.bc_lo[1], ky), _rule(g.bc_hi[1], ky))
        out.append(p)
    return torch.stack(out).contiguous()


def _pad_terrain(T):
    out = [_mirror(_mirror(T[c], 1, "edge", "edge"), 0, "edge", "edge") for c in range(T.shape[0])]
    return torch.stack(out).contiguous()


class Roe(BaseSolver):
    """Classic Roe (src/solvers/Roe.cpp); dt collapse is logged, not fatal (Roe.cpp:88-92)."""
    method = capi.HX_METHOD_ROE

    def _dt_collapse(self, lev, dt_est, max_vel):
        log.error("compute_dt: dt collapsed on lev %d (dt=%g, max|vel|=%g)", lev, dt_est, max_vel)


class HydrostaticRoe(BaseSolver):
    """Well-balanced hydrostatic Roe (src/solvers/HydrostaticRoe.cpp); dt collapse aborts (:77-80)."""
    method = capi.HX_METHOD_HYDROSTATIC_ROE

    def _dt_collapse(self, lev, dt_est, max_vel):
        raise HydroExaAbort("compute_dt: dt collapsed (velocity explosion). "
                            "Use dipole_probe.py on the latest plotfile to locate the offending cell.")


class SolverVariant:
    """std::variant<monostate, Roe, HydrostaticRoe> with forwarding (SolverVariant.H:45-192)."""

    def __init__(self, solver: BaseSolver | None = None):
        self._s = solver

    def has_solver(self) -> bool:
        return self._s is not None

    def _get(self):
        if self._s is None:
            raise RuntimeError("[SolverVariant Error] Solver not initialized.")
        return self._s

    def compute_fluxes(self, ctx, lev, dt, time):
        self._get().compute_fluxes(ctx, lev, dt, time)

    def compute_dt(self, dt, U, terrain, geom, ref_ratio, finest_level, cfl):
        self._get().compute_dt(dt, U, terrain, geom, ref_ratio, finest_level, cfl)

    def compute_dt_level(self, U, terrain, geom, lev, cfl):
        return self._get().compute_dt_level(U, terrain, geom, lev, cfl)

    def tag_cells(self, tags, U, terrain, geom, lev, time, phys_params):
        self._get().tag_cells(tags, U, terrain, geom, lev, time, phys_params)


def make_solver(model: str, arith: int = capi.HX_ARITH_FAST) -> SolverVariant:
    """AmrMeshState::InitializeSolver (AmrMeshState_Init.cpp:175-184)."""
    if model == "Roe":
        return SolverVariant(Roe(arith))
    if model == "HydrostaticRoe":
        return SolverVariant(HydrostaticRoe(arith))
    raise HydroExaAbort("Unknown solver type: " + model)


def masked_average_down(S_fine: torch.Tensor, S_crse: torch.Tensor, fgeom: Geometry, cgeom: Geometry, scomp: int,
                        ncomp: int, ratio, nodata_val: float = -9999.0) -> None:
    """amrex::masked_average_down (src/utils/MaskedAverageDown.cpp:12-63) for
    single-box levels: components scomp.. of S_fine restricted into S_crse."""
    del cgeom
    rx, ry = int(ratio[0]), int(ratio[1])
    nc, nyc, nxc = S_crse.shape
    if S_fine.shape[1] != nyc * ry or S_fine.shape[2] != nxc * rx:
        raise ValueError("fine and coarse boxes do not match the ratio")
    R = ctypes.c_double if S_fine.dtype == torch.float64 else ctypes.c_float
    sfx = "f64" if S_fine.dtype == torch.float64 else "f32"
    fv = fgeom.dx * fgeom.dy
    rc = getattr(capi.lib(), f"hx_masked_average_down_box_{sfx}")(
        ctypes.byref(array4(S_fine)), ctypes.byref(array4(S_crse)), box((0, 0), (nxc - 1, nyc - 1)), scomp, scomp,
        ncomp, rx, ry, R(fv), R(nodata_val), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    capi.check(rc, "hx_masked_average_down_box")


def average_down(S_fine: torch.Tensor, S_crse: torch.Tensor, scomp: int, ncomp: int, ratio) -> None:
    """amrex::average_down of the state as AmrMeshState::AverageDownTo calls it
    (src/state/AmrMeshState_AMR.cpp:838-844), for single-box levels:
    components scomp.. of S_fine (ncomp, ny, nx) restricted into S_crse."""
    rx, ry = int(ratio[0]), int(ratio[1])
    nc, nyc, nxc = S_crse.shape
    if S_fine.shape[1] != nyc * ry or S_fine.shape[2] != nxc * rx:
        raise ValueError("fine and coarse boxes do not match the ratio")
    sfx = "f64" if S_fine.dtype == torch.float64 else "f32"
    rc = getattr(capi.lib(), f"hx_average_down_box_{sfx}")(
        ctypes.byref(array4(S_fine)), ctypes.byref(array4(S_crse)), box((0, 0), (nxc - 1, nyc - 1)), scomp, scomp,
        ncomp, rx, ry, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    capi.check(rc, "hx_average_down_box")


__all__ = ["BaseSolver", "Roe", "HydrostaticRoe", "SolverVariant", "SolverContext", "HydroExaAbort", "make_solver",
           "masked_average_down", "average_down", "DtAccum"]
