"""The hand-written adjoint against two independent derivatives:

* the tangent-linear step (dual numbers through the exact arithmetic form):
  <J v, w> == <v, J^T w> for one step at fixed dt, with friction, dry cells,
  NODATA walls, open and reflective boundaries;
* central finite differences of the gauge misfit of a multi-step run
  (including the dependence of every dt on the CFL-limiting cell): directional
  derivatives agree to 1e-6 relative, on a smooth state over a short
  horizon (the exact linearisation of single-stage MUSCL with forward Euler
  amplifies grid-scale modes by up to ~1.06 per step at CFL 0.45, so long
  horizons leave the linear regime of a 1e-6 step).
Also: checkpointed and store-all reverse sweeps agree exactly, and the
torch.autograd.Function returns the same gradients.
"""
import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.adjoint import (GaugeProblem, adjoint_step, gauge_misfit, run_series, tangent_misfit,
                                    tangent_step)
from hydroexa_gb300.level import Geometry, Level

pytestmark = pytest.mark.gpu


def smooth_field(nx, ny, seed, amp, n=6):
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid((np.arange(nx) + 0.5) / nx, (np.arange(ny) + 0.5) / ny)
    f = np.zeros((ny, nx))
    for _ in range(n):
        cx, cy = rng.uniform(0, 1, 2)
        s = rng.uniform(0.08, 0.25)
        f += rng.uniform(-1, 1) * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    return amp * f / max(np.abs(f).max(), 1e-300)


def dot_case(kind):
    nx, ny = 48, 40
    z = smooth_field(nx, ny, 1, 0.3)
    X, Y = np.meshgrid((np.arange(nx) + 0.5) / nx, (np.arange(ny) + 0.5) / ny)
    eta = 1.0 + 0.2 * np.exp(-((X - 0.4) ** 2 + (Y - 0.6) ** 2) / 0.02)
    h = np.maximum(0.0, eta - z)
    rng = np.random.default_rng(2)
    hu = h * 0.3 * smooth_field(nx, ny, 3, 1.0)
    hv = h * 0.3 * smooth_field(nx, ny, 4, 1.0)
    n = np.zeros_like(h)
    geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (0, 0), (0, 0))
    if kind == "friction":
        n[:, : nx // 2] = 0.03
    if kind == "dry":  # an island; currents vary in space (a uniform velocity puts every u-limiter on a rounding-level kink)
        z = z + 0.9 * np.exp(-((X - 0.7) ** 2 + (Y - 0.3) ** 2) / 0.01)
        h = np.maximum(0.0, eta - z)
        hu = h * 0.2 * smooth_field(nx, ny, 5, 1.0)
        hv = h * 0.1 * smooth_field(nx, ny, 6, 1.0)
    if kind == "nodata":
        z[10:16, 20:30] = -9999.0
        n[10:16, 20:30] = -9999.0
        h[10:16, 20:30] = 0.0
        hu[10:16, 20:30] = 0.0
        hv[10:16, 20:30] = 0.0
    if kind == "open":
        geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (1, 0), (0, 1))
    del rng
    return geom, h, hu, hv, z, n


@pytest.mark.parametrize("kind", ["smooth", "friction", "dry", "nodata", "open"])
def test_dot_product_one_step(cuda, hxlib, kind):
    geom, h, hu, hv, z, n = dot_case(kind)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    lev = Level.from_numpy(geom, h, hu, hv, z, n, device=cuda)
    dt = 0.4 * lev.compute_dt()[0]
    state = torch.stack([T(h), T(hu), T(hv)])
    rng = np.random.default_rng(7)
    wet = torch.from_numpy((h > 1e-3).astype(np.float64)).to(cuda)
    dstate = T(rng.standard_normal((3, geom.ny, geom.nx))) * 1e-3 * wet
    dz = T(rng.standard_normal((geom.ny, geom.nx))) * 1e-3 * wet
    ddt = 0.1 * dt
    w = T(rng.standard_normal((3, geom.ny, geom.nx)))
    out, dout = tangent_step(geom, state, dstate, T(z), dz, T(n), dt, ddt)
    lam0, zbar, dtbar = adjoint_step(geom, state, T(z), T(n), dt, w)
    lhs = float((w * dout).sum())
    rhs = float((dstate * lam0).sum() + (dz * zbar).sum()) + ddt * dtbar
    assert abs(lhs - rhs) <= 1e-9 * (abs(lhs) + abs(rhs)), (kind, lhs, rhs)
    # the tangent step's value part is the forward step itself
    ref = lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, arith=capi.HX_ARITH_EXACT)
    assert torch.allclose(out, ref, rtol=0, atol=0)


def misfit_problem(every=0, nsteps=30, nx=64, ny=48):
    """A smooth state with no quiescent region: undulating free surface, a hump
    off the cell boundaries and smooth currents, so that no limiter sits on its
    flat-data branch (|dp| <= 1e-12) and the map is differentiable over the
    finite-difference step."""
    z = smooth_field(nx, ny, 11, 0.3, n=8)
    X, Y = np.meshgrid((np.arange(nx) + 0.5) / nx, (np.arange(ny) + 0.5) / ny)
    eta = 1.0 + 0.05 * smooth_field(nx, ny, 14, 1.0) + 0.2 * np.exp(-((X - 0.43) ** 2 + (Y - 0.57) ** 2) / (2 * 0.08 ** 2))
    h0 = eta - z
    hu0 = h0 * 0.2 * smooth_field(nx, ny, 15, 1.0)
    hv0 = h0 * 0.2 * smooth_field(nx, ny, 16, 1.0)
    rng = np.random.default_rng(12)
    gauges = rng.choice(nx * ny, size=16, replace=False)
    geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (0, 0), (0, 0))
    return geom, z, h0, hu0, hv0, gauges, nsteps, every


@pytest.mark.parametrize("every", [0, 7])
def test_gradient_matches_central_differences(cuda, hxlib, every):
    """Directional derivatives of the misfit along smooth directions in z, h0
    and hu0 agree with central differences to 1e-6 relative.

    The misfit is piecewise smooth: the van Leer limiter has kinks at r = 0,
    the face bed is max(zL, zR) and dt follows the arg max of the CFL rate.  A
    central difference whose interval straddles a kink is no derivative, so
    each direction is differenced with steps 1e-6 and 1e-7 and the closer one
    is held to the tolerance (on this problem the bed direction straddles a
    limiter kink at 1e-6 after ten steps; at 1e-7 it agrees to ~1e-8)."""
    geom, z, h0, hu0, hv0, gauges, nsteps, _ = misfit_problem()
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    zt, ht, ut, vt = T(z), T(h0), T(hu0), T(hv0)
    prob = GaugeProblem(geom, torch.zeros_like(ht), gauges, nsteps, 0.45, checkpoint_every=every)
    # reference data: the same run on a perturbed bed
    href = run_series(prob, zt + T(smooth_field(geom.nx, geom.ny, 13, 0.02)), ht, ut, vt).clone()
    series = prob.forward(zt, ht, ut, vt)
    assert float(((series - href) ** 2).sum()) > 0
    grads = prob.reverse(href)  # (z, h, hu, hv)
    base = [zt, ht, ut, vt]

    def J(args):
        return float(((run_series(prob, *args) - href) ** 2).sum())

    for k, name, seed in ((0, "z", 21), (1, "h0", 22), (2, "hu0", 23)):
        d = T(smooth_field(geom.nx, geom.ny, seed, 1.0))
        ad = float((grads[k] * d).sum())
        errs = {}
        for eps in (1e-6, 1e-7):
            plus = list(base)
            minus = list(base)
            plus[k] = base[k] + eps * d
            minus[k] = base[k] - eps * d
            fd = (J(plus) - J(minus)) / (2 * eps)
            errs[eps] = abs(ad - fd) / abs(fd)
        assert min(errs.values()) <= 1e-6, (name, ad, errs)


@pytest.mark.parametrize("every", [0, 7])
def test_gradient_matches_multistep_tangent(cuda, hxlib, every):
    """The whole reverse sweep (CFL arg max, gauge injection, checkpoint
    recompute) against the N-step tangent-linear model on the same exact
    trajectory: no finite-difference step, so agreement is to rounding."""
    geom, z, h0, hu0, hv0, gauges, nsteps, _ = misfit_problem()
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    base = [T(z), T(h0), T(hu0), T(hv0)]
    prob = GaugeProblem(geom, torch.zeros_like(base[0]), gauges, nsteps, 0.45, checkpoint_every=every,
                        arith=capi.HX_ARITH_EXACT)
    href = run_series(prob, base[0] + T(smooth_field(geom.nx, geom.ny, 13, 0.02)), *base[1:]).clone()
    prob.forward(*base)
    grads = prob.reverse(href)
    dirs = [T(smooth_field(geom.nx, geom.ny, s_, 1.0)) for s_ in (31, 32, 33, 34)]
    tan = tangent_misfit(prob, base, dirs, href)
    ad = sum(float((gk * dk).sum()) for gk, dk in zip(grads, dirs))
    assert abs(tan - ad) <= 1e-10 * abs(tan), (tan, ad)


def test_checkpointed_reverse_equals_store_all(cuda, hxlib):
    geom, z, h0, _, _, gauges, nsteps, _ = misfit_problem(nsteps=23)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    zt, ht = T(z), T(h0)
    zero = torch.zeros_like(ht)
    href = torch.zeros((nsteps, len(gauges)), dtype=torch.float64, device=cuda)
    grads = []
    for every in (0, 5):
        prob = GaugeProblem(geom, torch.zeros_like(ht), gauges, nsteps, 0.45, checkpoint_every=every, records=False)
        prob.forward(zt, ht, zero, zero)
        grads.append(prob.reverse(href))
    for a, b in zip(*grads):
        assert torch.equal(a, b)


@pytest.mark.parametrize("every", [1, 5, 11])
def test_face_records_reverse_matches(cuda, hxlib, every):
    """Uniform checkpoints with face records (the reverse reads the Roe
    intermediates the segment recompute wrote, Manning and dry-clamp steps
    included) against the same sweep evaluating them again: equal to rounding.
    The two differ in the last bits only: the forward forms 1/den, 1/cm and
    1/sden from one reciprocal and the sonic-fixed speeds by division, the
    recomputation from a reciprocal of a longer product."""
    geom, z, h0, hu0, hv0, gauges, _, _ = misfit_problem(nsteps=23)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    base = [T(z), T(h0), T(hu0), T(hv0)]
    nman = torch.zeros_like(base[0])
    nman[:, : geom.nx // 2] = 0.03
    href = torch.full((23, len(gauges)), 1.0, dtype=torch.float64, device=cuda)
    grads = []
    for rec in (False, True):
        prob = GaugeProblem(geom, nman, gauges, 23, 0.45, checkpoint_every=every, records=rec)
        assert (prob.options == capi.HX_ADJ_FACE_RECORDS) == rec
        prob.forward(*base)
        grads.append(prob.reverse(href))
    for a, b in zip(*grads):
        scale = float(b.abs().max())
        assert scale > 0
        assert float((a - b).abs().max()) <= 1e-12 * scale


@pytest.mark.parametrize("slots", [2, 3, 5, 9])
def test_binomial_reverse_equals_store_all(cuda, hxlib, slots):
    """Binomial checkpointing with few slots (2: no spare slot after the
    first snapshot) recomputes states bit for bit and reverses the same
    steps: gradients equal to the store-all sweep, Manning factor included."""
    geom, z, h0, hu0, hv0, gauges, _, _ = misfit_problem(nsteps=23)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    base = [T(z), T(h0), T(hu0), T(hv0)]
    nman = torch.zeros_like(base[0])
    nman[:, : geom.nx // 2] = 0.03
    href = torch.full((23, len(gauges)), 1.0, dtype=torch.float64, device=cuda)
    grads, series = [], []
    for every in (0, -slots):
        prob = GaugeProblem(geom, nman, gauges, 23, 0.45, checkpoint_every=every)
        series.append(prob.forward(*base))
        grads.append(prob.reverse(href))
    assert torch.equal(series[0], series[1])
    for a, b in zip(*grads):
        assert torch.equal(a, b)


def test_autograd_function(cuda, hxlib):
    geom, z, h0, _, _, gauges, nsteps, _ = misfit_problem(nsteps=12)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    zt = T(z).requires_grad_(True)
    ht = T(h0).requires_grad_(True)
    zero = torch.zeros_like(ht)
    href = torch.full((nsteps, len(gauges)), 1.0, dtype=torch.float64, device=cuda)
    prob = GaugeProblem(geom, torch.zeros_like(ht), gauges, nsteps, 0.45)
    loss = 3.0 * gauge_misfit(zt, ht, zero, zero, prob, href)
    gz, gh = torch.autograd.grad(loss, [zt, ht])
    prob2 = GaugeProblem(geom, torch.zeros_like(ht), gauges, nsteps, 0.45)
    prob2.forward(zt.detach(), ht.detach(), zero, zero)
    rz, rh, _, _ = prob2.reverse(href, seed=3.0)
    assert torch.equal(gz, rz) and torch.equal(gh, rh)


@pytest.mark.parametrize("every", [0, 5])
def test_gradient_matches_fd_without_kinks(cuda, hxlib, every):
    """On a state whose step map has no kink near the gauges (planar bed,
    strictly increasing free surface and currents, open boundaries, gauges in
    the centre: see workloads.adjoint_monotone_case) the misfit is smooth, and
    central differences with the configured step 1e-6 agree with the adjoint
    to 1e-6 relative in z, h0 and hu0."""
    case, gauges = workloads.adjoint_monotone_case(64, 48, nsteps=20, ngauges=12)
    g = case.geom
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    base = [T(case.z), T(case.h), T(case.hu), T(case.hv)]
    prob = GaugeProblem(g, torch.zeros_like(base[0]), gauges, 20, case.cfl, checkpoint_every=every)
    href = run_series(prob, base[0] + T(smooth_field(g.nx, g.ny, 13, 0.002)), *base[1:]).clone()
    prob.forward(*base)
    grads = prob.reverse(href)

    def J(args):
        return float(((run_series(prob, *args) - href) ** 2).sum())

    eps = 1e-6
    for k, name, seed in ((0, "z", 21), (1, "h0", 22), (2, "hu0", 23)):
        d = T(smooth_field(g.nx, g.ny, seed, 1.0))
        ad = float((grads[k] * d).sum())
        plus, minus = list(base), list(base)
        plus[k] = base[k] + eps * d
        minus[k] = base[k] - eps * d
        fd = (J(plus) - J(minus)) / (2 * eps)
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)
