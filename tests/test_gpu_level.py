"""CUDA level advance, dt reduction and time loop against the oracle.

Tolerances: conserved state within 1e-12 relative per step.  The
exact arithmetic form is held to equality with the oracle (no friction) or
1e-14 (friction: cbrt may differ by an ulp); the fast form to 1e-12 per step.
FP32 is compared with the oracle instantiated in float at 1e-5.
"""
import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.level import DtAccum, Level

pytestmark = pytest.mark.gpu

EXACT, FAST = capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST


def rel_err(a, b):
    """max |a - b| / max |b| per component, worst component."""
    worst = 0.0
    for x, y in zip(a, b):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        scale = max(np.abs(y).max(), 1e-300)
        worst = max(worst, np.abs(x - y).max() / scale)
    return worst


def cases():
    out = []
    out.append(("dam_break", workloads.dam_break(64, 64)))
    out.append(("lake_nodata", workloads.lake_at_rest(64, 64, seed=3, nodata_frac=0.1)))
    out.append(("fractal", workloads.fractal_dam_break(96, 80, seed=5)))
    c = workloads.fractal_dam_break(96, 80, seed=6, amplitude=1.0)
    c.n[c.z > -9000] = 0.03
    out.append(("friction", c))
    c = workloads.fractal_dam_break(64, 64, seed=8, amplitude=1.0, nodata_frac=0.0)
    c.geom.bc_lo, c.geom.bc_hi = (1, 0), (0, 1)
    out.append(("mixed_bc", c))
    c = workloads.fractal_dam_break(37, 23, seed=9, amplitude=0.5)
    c.geom.bc_lo, c.geom.bc_hi = (1, 1), (1, 1)
    out.append(("ragged_open", c))
    return out


def evolve(oracle, case, method, steps):
    """A non-trivial state: the case advanced `steps` steps by the oracle."""
    g = case.geom
    L = oracle.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    h, hu, hv, *_ = oracle.run(L, method, case.h, case.hu, case.hv, case.z, case.n, steps, case.cfl)
    return L, h, hu, hv


def to_level(case, h, hu, hv, device, dtype=torch.float64):
    return Level.from_numpy(case.geom, h, hu, hv, case.z, case.n, dtype=dtype, device=device)


@pytest.mark.parametrize("method", [capi.HX_METHOD_HYDROSTATIC_ROE, capi.HX_METHOD_ROE])
@pytest.mark.parametrize("name,case", cases(), ids=[c[0] for c in cases()])
def test_advance_matches_oracle(cuda, oracle_lib, method, name, case):
    if method == capi.HX_METHOD_ROE and (case.z == -9999.0).any():
        pytest.skip("classic Roe has no NODATA wall: see test_classic_roe_nodata_collapses")
    L, h, hu, hv = evolve(oracle_lib, case, method, 6)
    mn, _ = oracle_lib.compute_dt(L, h, hu, hv, case.z)
    dt = mn * case.cfl
    ref = oracle_lib.advance(L, method, h, hu, hv, case.z, case.n, dt)
    lev = to_level(case, h, hu, hv, cuda)
    got = lev.advance(method, dt, arith=EXACT).cpu().numpy()
    friction = (case.n[case.z > -9000] != 0).any()
    if friction:
        assert rel_err(got, ref) <= 1e-14
    else:
        for k in range(3):
            assert np.array_equal(got[k], ref[k]), (name, k, rel_err([got[k]], [ref[k]]))
    fast = lev.advance(method, dt, arith=FAST).cpu().numpy()
    assert rel_err(fast, ref) <= 1e-12
    assert lev.status.read() == 0


@pytest.mark.parametrize("name,case", cases(), ids=[c[0] for c in cases()])
def test_dt_reduce_matches_oracle(cuda, oracle_lib, name, case):
    L, h, hu, hv = evolve(oracle_lib, case, 1, 4)
    mn, mx = oracle_lib.compute_dt(L, h, hu, hv, case.z)
    lev = to_level(case, h, hu, hv, cuda)
    gmn, gmx = lev.compute_dt()
    assert gmn == mn and gmx == mx


@pytest.mark.parametrize("method", [capi.HX_METHOD_HYDROSTATIC_ROE, capi.HX_METHOD_ROE])
def test_time_loop_matches_oracle(cuda, oracle_lib, method):
    """hx_level_run: device-resident dt chain (fused next-step bound) over 25
    steps equals the oracle's host time loop."""
    nod = 0.2 if method == capi.HX_METHOD_HYDROSTATIC_ROE else 0.0
    case = workloads.fractal_dam_break(80, 72, seed=12, amplitude=2.0, nodata_frac=nod)
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    ref = oracle_lib.run(L, method, case.h, case.hu, case.hv, case.z, case.n, 25, case.cfl)
    assert ref[5] == 0
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    st = lev.run(method, 25, case.cfl, arith=EXACT)
    assert st == 0
    got = lev.state.cpu().numpy()
    assert rel_err(got, ref[:3]) == 0.0
    assert lev.time.item() == pytest.approx(ref[3], rel=1e-15)
    lev2 = to_level(case, case.h, case.hu, case.hv, cuda)
    lev2.run(method, 25, case.cfl, arith=FAST)
    assert rel_err(lev2.state.cpu().numpy(), ref[:3]) <= 1e-10


def test_classic_roe_nodata_collapses(cuda, oracle_lib):
    """Reference behaviour, reproduced: the classic solver has no NODATA wall, so
    a wet cell next to a NODATA cell (bed -9999 m, roughness -9999) drains into
    it, velocities explode and the CFL bound collapses; the oracle's time loop
    stops (status 1) and the device loop reports HX_STATUS_DT_COLLAPSE."""
    case = workloads.fractal_dam_break(80, 72, seed=12, amplitude=2.0, nodata_frac=0.2)
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    ref = oracle_lib.run(L, capi.HX_METHOD_ROE, case.h, case.hu, case.hv, case.z, case.n, 60, case.cfl)
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    st = lev.run(capi.HX_METHOD_ROE, 60, case.cfl, arith=EXACT)
    assert ref[5] == 1 and (st & capi.HX_STATUS_DT_COLLAPSE)


@pytest.mark.parametrize("arith", [EXACT, FAST])
def test_lake_at_rest_1000_steps(cuda, arith):
    """C-property over 1000 steps on the 512^2 Gaussian mound with roughness
    (no NODATA block: see test_nodata_wall_drops_pressure)."""
    case = workloads.lake_at_rest(512, 512, seed=2, nodata_frac=0.0, nsteps=1000)
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 1000, case.cfl, arith=arith) == 0
    s = lev.state
    wet = s[0] > 1e-6
    vel = torch.sqrt(s[1] ** 2 + s[2] ** 2)[wet] / s[0][wet]
    assert vel.max().item() <= 1e-13


@pytest.mark.parametrize("method", [capi.HX_METHOD_HYDROSTATIC_ROE, capi.HX_METHOD_ROE])
def test_mass_conservation_flat_bed_gpu(cuda, method):
    case = workloads.fractal_dam_break(256, 256, seed=1, amplitude=0.0, nodata_frac=0.0)
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    m0 = lev.state[0].sum().item()
    assert lev.run(method, 300, case.cfl, arith=FAST) == 0
    m1 = lev.state[0].sum().item()
    assert abs(m1 - m0) / m0 < 1e-12


def test_fp32_advance(cuda, oracle_lib):
    case = workloads.fractal_dam_break(64, 64, seed=21, amplitude=1.0)
    L, h, hu, hv = evolve(oracle_lib, case, 1, 5)
    f = [a.astype(np.float32) for a in (h, hu, hv, case.z, case.n)]
    mn, _ = oracle_lib.compute_dt(L, f[0], f[1], f[2], f[3])
    dt = np.float32(mn * case.cfl)
    ref = oracle_lib.advance(L, 1, f[0], f[1], f[2], f[3], f[4], float(dt))
    lev = Level.from_numpy(case.geom, *f, dtype=torch.float32, device=cuda)
    got = lev.advance(1, float(dt), arith=FAST).cpu().numpy()
    assert rel_err(got, ref) <= 1e-5


@pytest.mark.parametrize("method,nx,ny,nsteps,arith", [(1, 64, 48, 10, EXACT), (1, 64, 48, 1, EXACT),
                                                      (1, 70, 45, 3, EXACT), (0, 53, 61, 1, EXACT),
                                                      (1, 96, 130, 2, FAST), (1, 40, 65, 1, EXACT),
                                                      (1, 40, 66, 2, FAST), (1, 64, 2053, 1, EXACT)])
def test_host_buffer_run(cuda, oracle_lib, hxlib, method, nx, ny, nsteps, arith):
    """hx_level_run_host_f64 (host buffers in, host buffers out: the upload in
    row bands with the CFL reduction and, for the hydrostatic solver, the first
    step's flux differences running under it; the last step in row bands
    downloaded as they finish) equals the device-resident run: bit for bit in
    the exact form, to 1e-13 in the fast form (multiply-add contraction may
    differ between the split and the fused kernels); partial bands included,
    down to bands of one and two rows (the head rows a band's flux
    differences wait for), with short first and last bands."""
    import ctypes
    case = workloads.fractal_dam_break(nx, ny, seed=4, amplitude=1.0, nodata_frac=0.2 if method else 0.0)
    h, hu, hv = case.h.copy(), case.hu.copy(), case.hv.copy()
    t = ctypes.c_double()
    lo = (ctypes.c_int32 * 2)(*case.geom.bc_lo)
    hi = (ctypes.c_int32 * 2)(*case.geom.bc_hi)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = hxlib.lib().hx_level_run_host_f64(method, nx, ny, case.geom.dx, case.geom.dy, lo, hi, P(h), P(hu), P(hv),
                                           P(case.z), P(case.n), nsteps, case.cfl, arith, ctypes.byref(t), None)
    assert rc == 0
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    lev.run(method, nsteps, case.cfl, arith=arith)
    got = lev.state.cpu().numpy()
    if arith == EXACT:
        assert np.array_equal(got[0], h) and np.array_equal(got[1], hu) and np.array_equal(got[2], hv)
        assert t.value == lev.time.item()
    else:
        for k, a in enumerate((h, hu, hv)):
            assert rel_err(a, got[k]) <= 1e-13
        assert abs(t.value - lev.time.item()) <= 1e-13 * lev.time.item()


@pytest.mark.parametrize("nx,ny,nsteps,arith", [(40, 65, 1, EXACT), (96, 65, 2, FAST), (64, 17, 1, EXACT),
                                                (48, 313, 1, EXACT)])
def test_host_buffer_run_pinned(cuda, hxlib, nx, ny, nsteps, arith):
    """The same call from page-locked host buffers, where the copies run
    asynchronously and a band's flux differences must wait for every row they
    read: heights whose band layout once held a one-row band before the last
    (65, 17, 313 rows).  Equal to the device-resident run (bit for bit in the
    exact form, 1e-13 in the fast form)."""
    import ctypes
    case = workloads.fractal_dam_break(nx, ny, seed=5, amplitude=1.0, nodata_frac=0.2)
    pinned = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
              for a in (case.h, case.hu, case.hv, case.z, case.n)]
    t = ctypes.c_double()
    lo = (ctypes.c_int32 * 2)(*case.geom.bc_lo)
    hi = (ctypes.c_int32 * 2)(*case.geom.bc_hi)
    P = [ctypes.c_void_p(a.data_ptr()) for a in pinned]
    rc = hxlib.lib().hx_level_run_host_f64(1, nx, ny, case.geom.dx, case.geom.dy, lo, hi, *P, nsteps, case.cfl,
                                           arith, ctypes.byref(t), None)
    assert rc == 0
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    lev.run(1, nsteps, case.cfl, arith=arith)
    got = lev.state.cpu().numpy()
    for k in range(3):
        res = pinned[k].numpy()
        if arith == EXACT:
            assert np.array_equal(got[k], res), k
        else:
            assert rel_err([res], [got[k]]) <= 1e-13, k


def test_host_buffer_run_repeated_calls(cuda, hxlib):
    """The split share of the first step follows each call's measured upload
    and compute times, so successive calls split different bands; the result
    does not depend on it: five calls on the same page-locked inputs, each bit
    for bit the device-resident run (exact form)."""
    import ctypes
    nx, ny = 256, 1536
    case = workloads.fractal_dam_break(nx, ny, seed=6, amplitude=1.0, nodata_frac=0.2)
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    lev.run(1, 1, case.cfl, arith=EXACT)
    want = lev.state.cpu().numpy()
    lo = (ctypes.c_int32 * 2)(*case.geom.bc_lo)
    hi = (ctypes.c_int32 * 2)(*case.geom.bc_hi)
    t = ctypes.c_double()
    terrain = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (case.z, case.n)]
    for _ in range(5):
        state = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (case.h, case.hu, case.hv)]
        P = [ctypes.c_void_p(a.data_ptr()) for a in state + terrain]
        assert hxlib.lib().hx_level_run_host_f64(1, nx, ny, case.geom.dx, case.geom.dy, lo, hi, *P, 1, case.cfl,
                                                 EXACT, ctypes.byref(t), None) == 0
        for k in range(3):
            assert np.array_equal(state[k].numpy(), want[k]), k
        assert 0.15 <= hxlib.lib().hx_debug_host_split_frac() <= 0.85


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_nodata_predicate_at_its_edges(cuda, oracle_lib, dtype):
    """The NODATA test |z + 9999| < 1e-10 at the edge of its interval: beds a
    few representable steps either side of -9999 (double: |k| <= 54 steps of
    2^-39 qualify; float: -9999 alone) give the oracle's walls, dt and state."""
    rng = np.random.default_rng(17)
    case = workloads.fractal_dam_break(64, 48, seed=23, amplitude=1.0, nodata_frac=0.0)
    z = case.z.astype(dtype)
    sel = rng.random(z.shape) < 0.08
    k = rng.integers(-60, 61, size=z.shape)
    if dtype == np.float64:
        b = np.array(-9999.0).view(np.int64) + k
        edge = b.view(np.float64)
    else:
        b = np.array(-9999.0, dtype=np.float32).view(np.int32) + (k % 3 - 1)
        edge = b.astype(np.int32).view(np.float32)
    z[sel] = edge[sel]
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    f = [a.astype(dtype) for a in (case.h, case.hu, case.hv, z, case.n)]
    mn, mx = oracle_lib.compute_dt(L, f[0], f[1], f[2], f[3])
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    lev = Level.from_numpy(g, *f, dtype=tdt, device=cuda)
    gmn, gmx = lev.compute_dt()
    dt = float(dtype(mn * case.cfl))
    ref = oracle_lib.advance(L, 1, f[0], f[1], f[2], f[3], f[4], dt)
    got = lev.advance(1, dt, arith=EXACT).cpu().numpy()
    if dtype == np.float64:
        assert gmn == mn and gmx == mx
        for c in range(3):
            assert np.array_equal(got[c], ref[c]), c
    else:  # a misplaced wall changes the state by O(1) next to it
        assert gmn == pytest.approx(mn, rel=1e-6) and gmx == pytest.approx(mx, rel=1e-6)
        assert rel_err(got, ref) <= 1e-5


def test_big_tile_levels_match_oracle(cuda, oracle_lib, hxlib):
    """Boxes of 2048 x 2048 cells and more take the 32 x 32 tile kernels (level
    step, split first step of the host-buffer call): the exact form stays
    bit-equal to the oracle and to the device loop, the fast form within 1e-12."""
    import ctypes
    n = 2048
    case = workloads.fractal_dam_break(n, n, seed=31, amplitude=2.0, nodata_frac=0.2)
    g = case.geom
    L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
    ref = oracle_lib.run(L, capi.HX_METHOD_HYDROSTATIC_ROE, case.h, case.hu, case.hv, case.z, case.n, 2, case.cfl)
    assert ref[5] == 0
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 2, case.cfl, arith=EXACT) == 0
    got = lev.state.cpu().numpy()
    for k in range(3):
        assert np.array_equal(got[k], ref[k]), k
    fast = to_level(case, case.h, case.hu, case.hv, cuda)
    assert fast.run(capi.HX_METHOD_HYDROSTATIC_ROE, 2, case.cfl, arith=FAST) == 0
    assert rel_err(fast.state.cpu().numpy(), ref[:3]) <= 1e-12
    # the host-buffer call on 8192 x 4096 cells: its row bands (512 x 8192) take the big tile too, in the split
    # first step and in the banded last step; bit-equal to the device loop
    case = workloads.fractal_dam_break(8192, 4096, seed=32, amplitude=2.0, nodata_frac=0.2)
    g = case.geom
    h, hu, hv = case.h.copy(), case.hu.copy(), case.hv.copy()
    t = ctypes.c_double()
    lo = (ctypes.c_int32 * 2)(*g.bc_lo)
    hi = (ctypes.c_int32 * 2)(*g.bc_hi)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = hxlib.lib().hx_level_run_host_f64(capi.HX_METHOD_HYDROSTATIC_ROE, g.nx, g.ny, g.dx, g.dy, lo, hi, P(h),
                                           P(hu), P(hv), P(case.z), P(case.n), 2, case.cfl, EXACT, ctypes.byref(t),
                                           None)
    assert rc == 0
    lev = to_level(case, case.h, case.hu, case.hv, cuda)
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 2, case.cfl, arith=EXACT) == 0
    got = lev.state.cpu().numpy()
    assert np.array_equal(h, got[0]) and np.array_equal(hu, got[1]) and np.array_equal(hv, got[2])


@pytest.mark.parametrize("arith", [EXACT, FAST])
def test_full_size_properties(cuda, arith):
    """The throughput size, 8192^2 FP64, through size-independent properties:
    a lake at rest over the 5 m fractal bed (free surface at 6 m, every cell wet,
    no NODATA) stays at rest (|u| <= 1e-13) and a dam break on a flat bed between
    reflective walls conserves mass to round-off, over 10 steps of the device
    loop (32 x 32 tiles).  (With emerged bed, cells a few millimetres deep turn
    the rounding-level momentum of the pressure balance into |u| ~ 1e-10: the
    reference's own lake check keeps every cell wet.)"""
    n = 8192
    case = workloads.fractal_dam_break(n, n, seed=3, nodata_frac=0.0)
    h = 6.0 - case.z
    lev = Level.from_numpy(case.geom, h, np.zeros_like(h), np.zeros_like(h), case.z, case.n, device=cuda)
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 10, case.cfl, arith=arith) == 0
    s = lev.state
    wet = s[0] > 1e-6
    vel = torch.sqrt(s[1] ** 2 + s[2] ** 2)[wet] / s[0][wet]
    assert vel.max().item() <= 1e-13
    del lev, s, wet, vel
    flat = workloads.dam_break(n, n)
    lev = Level.from_numpy(flat.geom, flat.h, flat.hu, flat.hv, flat.z, flat.n, device=cuda)
    m0 = lev.state[0].sum(dtype=torch.float64).item()
    assert lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 10, flat.cfl, arith=arith) == 0
    m1 = lev.state[0].sum(dtype=torch.float64).item()
    assert abs(m1 - m0) <= 1e-12 * m0


def _fold_reference(state, z, dx, dy):
    """(1 / max rate, max speed) of a state over its wet, non-NODATA cells,
    evaluated in numpy: the bound every cell's contribution gives."""
    h, hu, hv = (np.asarray(a, dtype=np.float64) for a in state)
    live = (np.abs(z + 9999.0) >= 1e-10) & (h > 1e-12)
    u, v = np.abs(hu[live] / h[live]), np.abs(hv[live] / h[live])
    c = np.sqrt(9.81 * h[live])
    rate = (u + c) / dx + (v + c) / dy
    return 1.0 / rate.max(), max(u.max(), v.max())


@pytest.mark.parametrize("n,kind", [(64, "varied"), (96, "uniform"), (2048, "varied"), (2048, "uniform")])
def test_screened_cfl_fold_is_the_maximum(cuda, oracle_lib, n, kind):
    """The fast form folds the next CFL bound through a float screen (FP64 only
    for the cells that can hold the block maximum, and once per block for
    bit-identical candidates).  The folded bound and speed equal those of every
    cell (to the last few ulps of the fast form's own rate arithmetic), on an
    evolved state with NODATA and dry cells and on a uniform lake (all ties);
    2048^2 runs the 32 x 32 tile."""
    if kind == "varied":
        case = workloads.fractal_dam_break(n, n, seed=41, amplitude=1.0, nodata_frac=0.15)
        g = case.geom
        L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
        h, hu, hv, *_ = oracle_lib.run(L, 1, case.h, case.hu, case.hv, case.z, case.n, 4, case.cfl)
        h[5, 5:9] = 0.0  # dry cells
    else:
        case = workloads.fractal_dam_break(n, n, seed=42, amplitude=1.0, nodata_frac=0.0)
        g = case.geom
        h = np.full_like(case.h, 2.0)
        case.z = np.zeros_like(case.z)
        hu = np.zeros_like(h)
        hv = np.zeros_like(h)
    lev = to_level(case, h, hu, hv, cuda)
    dt = 0.2 * lev.compute_dt()[0]
    acc = DtAccum(cuda)
    out = lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, next_dt=acc, arith=FAST)
    got_dt, got_v = acc.read()
    ref_dt, ref_v = _fold_reference(out.cpu().numpy(), case.z, g.dx, g.dy)
    assert got_dt == pytest.approx(ref_dt, rel=4e-16 * 8) and got_v == pytest.approx(ref_v, rel=4e-16 * 8)


@pytest.mark.parametrize("n,kind", [(70, "varied"), (96, "uniform"), (2048, "varied")])
def test_screened_dt_reduce_equals_the_fused_fold(cuda, oracle_lib, n, kind):
    """The fast FP64 CFL reduction of a level (hx_level_run_f64 with no steps:
    the bound of the state into the first work slot; 4 rows per thread) goes
    through the same float screen as the fold fused into the advance.  Over the
    state that advance wrote, both give the same bits: bound, speed and the
    dry / NODATA flags, on an evolved state and on a uniform lake (all ties)."""
    if kind == "varied":
        case = workloads.fractal_dam_break(n, n + 3, seed=43, amplitude=1.0, nodata_frac=0.15)
        g = case.geom
        L = oracle_lib.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
        h, hu, hv, *_ = oracle_lib.run(L, 1, case.h, case.hu, case.hv, case.z, case.n, 3, case.cfl)
        h[7, 3:11] = 0.0  # dry cells
    else:
        case = workloads.fractal_dam_break(n, n, seed=44, amplitude=1.0, nodata_frac=0.0)
        h = np.full_like(case.h, 1.5)
        case.z = np.zeros_like(case.z)
        hu = np.zeros_like(h)
        hv = np.zeros_like(h)
    lev = to_level(case, h, hu, hv, cuda)
    dt = 0.2 * lev.compute_dt()[0]
    acc = DtAccum(cuda)
    out = lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, next_dt=acc, arith=FAST).cpu().numpy()
    nxt = to_level(case, out[0], out[1], out[2], cuda)
    assert nxt.run(capi.HX_METHOD_HYDROSTATIC_ROE, 0, case.cfl, arith=FAST) == 0
    torch.cuda.synchronize()
    got, ref = nxt.work[:20].cpu(), acc.buf[:20].cpu()
    assert torch.equal(got, ref), (got.tolist(), ref.tolist())
    flags = int(ref[16])
    assert (flags & 2) == (2 if kind == "varied" else 0) and (kind == "varied" or flags == 0)


def test_host_buffer_run_on_two_devices(cuda, hxlib):
    """hx_level_run_host_f64 keeps its device buffers, streams and events per
    device: one thread calling it on device 0, then device 1, then device 0
    again gets each device's own resources (the results equal the device
    loop on each).  Needs two GPUs; skipped on one."""
    import ctypes
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    case = workloads.fractal_dam_break(64, 48, seed=7, amplitude=1.0, nodata_frac=0.1)
    lo = (ctypes.c_int32 * 2)(*case.geom.bc_lo)
    hi = (ctypes.c_int32 * 2)(*case.geom.bc_hi)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    ref = to_level(case, case.h, case.hu, case.hv, cuda)
    ref.run(1, 3, case.cfl, arith=EXACT)
    want = ref.state.cpu().numpy()
    for dev in (0, 1, 0):
        with torch.cuda.device(dev):
            h, hu, hv = case.h.copy(), case.hu.copy(), case.hv.copy()
            t = ctypes.c_double()
            rc = hxlib.lib().hx_level_run_host_f64(1, 64, 48, case.geom.dx, case.geom.dy, lo, hi, P(h), P(hu), P(hv),
                                                   P(case.z), P(case.n), 3, case.cfl, EXACT, ctypes.byref(t), None)
            assert rc == 0, hxlib.lib().hx_last_error()
            assert np.array_equal(h, want[0]) and np.array_equal(hu, want[1]) and np.array_equal(hv, want[2])
    hxlib.lib().hx_host_cache_release()


@pytest.mark.parametrize("arith", [EXACT, FAST])
def test_persistent_staging_tma_equals_cp_async(cuda, arith):
    """The persistent level kernel stages each tile by TMA when the planes' rows
    are whole 16-byte units, else by cp.async: a 2048^2 level stored with row
    pitch 2048 and 2050 (TMA) and 2049 (cp.async) gives the same state, bit for
    bit, after three steps of the device loop, with a clean status."""
    case = workloads.fractal_dam_break(2048, 2048, seed=5)
    out = []
    for pitch in (2048, 2049, 2050):
        st = torch.zeros((3, 2048, pitch), dtype=torch.float64)
        tr = torch.zeros((2, 2048, pitch), dtype=torch.float64)
        for k, a in enumerate((case.h, case.hu, case.hv)):
            st[k, :, :2048] = torch.from_numpy(a)
        tr[0, :, :2048] = torch.from_numpy(case.z)
        tr[1, :, :2048] = torch.from_numpy(case.n)
        lev = Level(case.geom, st.to(cuda), tr.to(cuda))
        assert lev.run(1, 3, case.cfl, arith=arith) == 0
        out.append((lev.state[:, :, :2048].cpu().numpy(), lev.time.item()))
    for s, t in out[1:]:
        assert np.array_equal(s, out[0][0]) and t == out[0][1]


def test_persistent_staging_wait_is_bounded(cuda, hxlib):
    """The persistent kernel's TMA staging wait is bounded: with the test
    setting that makes every tile wait for 16 bytes more than it brings, the
    wait runs out after about a second, the step ends with
    HX_STATUS_STAGING_TIMEOUT instead of hanging, and the context stays usable:
    the same step with the normal setting runs clean afterwards."""
    case = workloads.fractal_dam_break(2048, 2048, seed=5)
    L = hxlib.lib()
    lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
    assert L.hx_debug_staging_extra_bytes(16) == 0
    try:
        st = lev.run(1, 1, case.cfl, arith=FAST)
    finally:
        L.hx_debug_staging_extra_bytes(0)
    assert st & capi.HX_STATUS_STAGING_TIMEOUT
    lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
    assert lev.run(1, 1, case.cfl, arith=FAST) == 0
