"""Gradients of a gauge-misfit loss through the hydrostatic-Roe time loop.

``gauge_misfit(z, h0, hu0, hv0, problem, href)`` is a differentiable torch
function: its forward runs the N-step forward sweep on the GPU
(``hx_adjoint_forward_f64``: device CFL chain, states or checkpoints kept in
HBM), its backward the hand-written reverse sweep
(``hx_adjoint_reverse_f64``).  The loss is
J = sum over steps n = 1..N and gauge cells g of (h^n_g - href[n-1, g])^2.

``tangent_step`` and ``adjoint_step`` expose one step at a fixed dt in forward
mode (dual numbers through the exact arithmetic form) and in reverse mode, for
the dot-product test <J v, w> = <v, J^T w>; ``tangent_misfit`` chains the
tangent step over the whole run (the forward-mode derivative of the misfit,
the exact counterpart of the reverse sweep).
"""
from __future__ import annotations

import ctypes

import torch

from . import capi
from .level import Geometry


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _level(geom: Geometry, h, hu, hv, z, n, pitch=None):
    d = capi.LevelF64()
    P = lambda t: ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctypes.c_double))
    d.h, d.hu, d.hv, d.z, d.n = P(h), P(hu), P(hv), P(z), P(n)
    d.pitch = pitch if pitch is not None else geom.nx
    d.nx, d.ny = geom.nx, geom.ny
    d.dx, d.dy = geom.dx, geom.dy
    d.bc_lo[0], d.bc_lo[1] = geom.bc_lo
    d.bc_hi[0], d.bc_hi[1] = geom.bc_hi
    return d


def _plane(t: torch.Tensor, geom: Geometry):
    assert t.is_cuda and t.dtype == torch.float64 and t.shape == (geom.ny, geom.nx)
    return t.contiguous()


# Face records are kept when they take at most this much device memory.
RECORD_BUDGET = 16 << 30


class GaugeProblem:
    """Geometry, roughness, gauges and step count of a misfit problem.
    gauges: (G,) flat cell indices i + j * nx.  checkpoint_every: 0 keeps every
    state; k > 0 keeps every k-th and recomputes segments in the reverse sweep;
    k < 0 binomial checkpointing with -k slots.  records (fast form, k > 0):
    the segment recompute records each face's Roe intermediates for the
    reverse sweep; None keeps them when they fit RECORD_BUDGET."""

    def __init__(self, geom: Geometry, n: torch.Tensor, gauges, nsteps: int, cfl: float, checkpoint_every: int = 0,
                 arith: int = capi.HX_ARITH_FAST, records=None):
        self.geom = geom
        self.arith = int(arith)
        self.n = _plane(n, geom)
        dev = self.n.device
        self.gauges = torch.as_tensor(gauges, dtype=torch.int64, device=dev).contiguous()
        self.nsteps, self.cfl, self.every = int(nsteps), float(cfl), int(checkpoint_every)
        L = capi.lib()
        plain = L.hx_adjoint_work_bytes_f64(geom.nx, geom.ny, geom.nx, self.nsteps, self.every, 0)
        if plain <= 0:
            raise capi.HxError("bad adjoint problem size")
        self.options = 0
        if self.arith == capi.HX_ARITH_FAST and self.every > 0 and records is not False:
            with_rec = L.hx_adjoint_work_bytes_f64(geom.nx, geom.ny, geom.nx, self.nsteps, self.every,
                                                   capi.HX_ADJ_FACE_RECORDS)
            if records or with_rec - plain <= RECORD_BUDGET:
                self.options = capi.HX_ADJ_FACE_RECORDS
        nbytes = L.hx_adjoint_work_bytes_f64(geom.nx, geom.ny, geom.nx, self.nsteps, self.every, self.options)
        self.work = torch.empty(int(nbytes), dtype=torch.uint8, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._inputs = None

    @property
    def work_bytes(self) -> int:
        return self.work.numel()

    def forward(self, z, h0, hu0, hv0, stream=None):
        """Forward sweep; returns the gauge series (N, G)."""
        g = self.geom
        z, h0, hu0, hv0 = (_plane(t, g) for t in (z, h0, hu0, hv0))
        self._inputs = (z, h0, hu0, hv0)
        series = torch.empty((self.nsteps, self.gauges.numel()), dtype=torch.float64, device=z.device)
        s = stream if stream is not None else torch.cuda.current_stream(z.device)
        self.status.zero_()
        d = _level(g, h0, hu0, hv0, z, self.n)
        capi.check(capi.lib().hx_adjoint_forward_f64(
            ctypes.byref(d), self.nsteps, self.cfl, self.gauges.numel(), _vp(self.gauges), _vp(series), self.every,
            self.arith, _vp(self.work), _vp(self.status), ctypes.c_void_p(s.cuda_stream)), "hx_adjoint_forward_f64")
        st = int(self.status.item())
        if st & capi.HX_STATUS_DT_COLLAPSE:
            raise capi.HxError(f"adjoint forward sweep: the CFL bound collapsed (status {st})")
        return series

    def reverse(self, href: torch.Tensor, seed: float = 1.0, stream=None):
        """Reverse sweep after forward(): seed * dJ/d(z, h0, hu0, hv0)."""
        z, h0, hu0, hv0 = self._inputs
        g = self.geom
        href = href.to(torch.float64).contiguous()
        gz, gh, ghu, ghv = (torch.empty_like(z) for _ in range(4))
        s = stream if stream is not None else torch.cuda.current_stream(z.device)
        d = _level(g, h0, hu0, hv0, z, self.n)
        capi.check(capi.lib().hx_adjoint_reverse_f64(
            ctypes.byref(d), self.nsteps, self.cfl, self.gauges.numel(), _vp(self.gauges), _vp(href), float(seed),
            self.every, self.arith | self.options, _vp(self.work), _vp(gh), _vp(ghu), _vp(ghv), _vp(gz),
            ctypes.c_void_p(s.cuda_stream)),
            "hx_adjoint_reverse_f64")
        return gz, gh, ghu, ghv


class GaugeMisfit(torch.autograd.Function):
    """J(z, h0, hu0, hv0) = sum (h^n_g - href)^2 with a hand-written backward."""

    @staticmethod
    def forward(ctx, z, h0, hu0, hv0, problem: GaugeProblem, href: torch.Tensor):
        series = problem.forward(z.detach(), h0.detach(), hu0.detach(), hv0.detach())
        ctx.problem = problem
        ctx.save_for_backward(href)
        return ((series - href) ** 2).sum()

    @staticmethod
    def backward(ctx, gloss):
        (href,) = ctx.saved_tensors
        gz, gh, ghu, ghv = ctx.problem.reverse(href, seed=float(gloss))
        return gz, gh, ghu, ghv, None, None


def gauge_misfit(z, h0, hu0, hv0, problem: GaugeProblem, href: torch.Tensor):
    return GaugeMisfit.apply(z, h0, hu0, hv0, problem, href)


def run_series(problem: GaugeProblem, z, h0, hu0, hv0):
    """The gauge series of a forward run (no gradient)."""
    return problem.forward(z, h0, hu0, hv0)


def tangent_misfit(problem: GaugeProblem, base, direction, href: torch.Tensor) -> float:
    """dJ/d(z, h0, hu0, hv0) . direction by the N-step tangent-linear model.

    Each step carries (value, derivative) pairs through the exact arithmetic
    form (hx_level_tangent_f64) at the step's dt, whose derivative comes from
    the cell that sets the CFL bound: dt = cfl / max_c rate_c with
    rate = (|u| + c) / dx + (|v| + c) / dy (HydrostaticRoe.cpp:41-61), the
    arg max taken at the lowest flat index on ties as in the reverse sweep.
    The trajectory is that of an HX_ARITH_EXACT forward sweep bit for bit, so
    the result is the exact directional derivative that the adjoint of an
    HX_ARITH_EXACT problem must reproduce.  Levels without dry or NODATA
    cells only (their CFL clamps are not differentiated here).
    """
    g = problem.geom
    z, h0, hu0, hv0 = base
    dz, dh0, dhu0, dhv0 = direction
    state = torch.stack([h0, hu0, hv0])
    dstate = torch.stack([dh0, dhu0, dhv0])
    gauges = problem.gauges
    href = href.to(torch.float64)
    G = 9.81
    dJ = torch.zeros((), dtype=torch.float64, device=z.device)
    for n in range(problem.nsteps):
        h, hu, hv = state
        if not bool((h > 1e-12).all()):
            raise ValueError("tangent_misfit: a cell is dry")
        u, v = hu / h, hv / h
        c = torch.sqrt(G * h)
        rate = (u.abs() + c) / g.dx + (v.abs() + c) / g.dy
        k = int(torch.argmax(rate.reshape(-1)))
        j, i = divmod(k, g.nx)
        R = float(rate[j, i])
        dt = (1.0 / R) * problem.cfl
        hk, uk, vk, ck = (float(t[j, i]) for t in (h, u, v, c))
        dhk, dhuk, dhvk = (float(t[j, i]) for t in dstate)
        sgn = lambda x: (x > 0) - (x < 0)
        dc = G / (2.0 * ck) * dhk
        drate = (sgn(uk) * (dhuk - uk * dhk) / hk + dc) / g.dx + (sgn(vk) * (dhvk - vk * dhk) / hk + dc) / g.dy
        ddt = -problem.cfl * drate / (R * R)
        state, dstate = tangent_step(g, state, dstate, z, dz, problem.n, dt, ddt)
        hn, dhn = state[0].reshape(-1), dstate[0].reshape(-1)
        dJ += (2.0 * (hn[gauges] - href[n]) * dhn[gauges]).sum()
    return float(dJ)


# ----------------------------------------------------------------- one step
def tangent_step(geom: Geometry, state, dstate, z, dz, n, dt, ddt=0.0):
    """(U^{n+1}, dU^{n+1}) for state (3, ny, nx) and tangents, fixed dt."""
    pair = lambda v, d: torch.stack([v, d], dim=-1).contiguous()
    zeros = torch.zeros_like(z)
    P = [pair(state[k], dstate[k]) for k in range(3)] + [pair(z, dz), pair(n, zeros)]
    out = [torch.empty_like(P[0]) for _ in range(3)]
    d = _level(geom, P[0], P[1], P[2], P[3], P[4], pitch=geom.nx)
    capi.check(capi.lib().hx_level_tangent_f64(ctypes.byref(d), float(dt), float(ddt), _vp(out[0]), _vp(out[1]),
                                               _vp(out[2]), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "hx_level_tangent_f64")
    torch.cuda.synchronize()
    return torch.stack([o[..., 0] for o in out]), torch.stack([o[..., 1] for o in out])


def adjoint_step(geom: Geometry, state, z, n, dt, lam, arith: int = capi.HX_ARITH_EXACT):
    """(lambda^n, zbar, dtbar) for lambda^{n+1} = lam at fixed dt."""
    st = [state[k].contiguous() for k in range(3)]
    lm = [lam[k].contiguous() for k in range(3)]
    out = [torch.empty_like(st[0]) for _ in range(3)]
    zbar = torch.zeros_like(z)
    dtbar = torch.zeros(1, dtype=torch.float64, device=z.device)
    nbytes = capi.lib().hx_adjoint_work_bytes_f64(geom.nx, geom.ny, geom.nx, 1, 0, 0)
    work = torch.empty(int(nbytes), dtype=torch.uint8, device=z.device)
    d = _level(geom, st[0], st[1], st[2], z.contiguous(), n.contiguous())
    capi.check(capi.lib().hx_adjoint_step_f64(ctypes.byref(d), float(dt), *(_vp(t) for t in lm),
                                              *(_vp(t) for t in out), _vp(zbar), _vp(dtbar), int(arith), _vp(work),
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "hx_adjoint_step_f64")
    torch.cuda.synchronize()
    return torch.stack(out), zbar, float(dtbar.item())
