"""Regenerate the golden vectors in this folder from the reference itself.

Run from the repository root, in a checkout that has the reference source tree
(where oracle/build_ref.sh finds it, or $HX_REFERENCE_ROOT):

    python tests/golden/make_golden.py

What it writes (all seeded, all small):

* ``roe_hydrostatic_{f64,f32}.npz`` -- inputs and outputs of the reference's
  homogeneous Roe point kernel (include/solvers/kernels/HydrostaticRoe.H:44-159)
  compiled verbatim from the reference tree (oracle/build_ref.sh).
* ``roe_classic_{f64,f32}.npz`` -- the same for the classic Roe kernel with bed
  slope, friction and positivity guard (include/solvers/kernels/Roe.H:51-309).
* ``masked_avgdown_f64.npz`` -- the reference's NODATA-aware restriction
  (include/utils/MaskedAverageDown.H:64-104) on fields with NaN and sentinels.
* ``dambreak_exact.npz`` -- the exact dam-break-on-wet-bed profiles of the
  reference's tests/dambreak/analytical.py, imported from the reference tree.
* ``drivers_{f64,f32}.npz`` -- the reference's per-box solver drivers
  (src/solvers/HydrostaticRoe.cpp, src/solvers/Roe.cpp with SolverVariant and
  the BCFill.H ghost filler) compiled verbatim and run at one level by
  oracle/ref_level.cpp: for each case the inputs, the state, clock and status
  after the reference's own time loop, with the limiter's abs() bound both
  ways (``fabs``: the floating abs; ``iabs``: C's int abs), the first CFL
  bound, and tag flags (``python tests/golden/make_golden.py drivers``
  rewrites these two files alone).

The families of inputs are chosen to drive every branch of the kernels: dry
clamps, both sonic entropy fixes, both positivity guards, both thrust forms,
friction on and off, and x and y normals.
"""
from __future__ import annotations

import importlib.util
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
REF = oracle.reference_root()


def hydro_states(rng, n):
    """(n, 6) face states and (n, 2) normals covering the kernel's branches."""
    q = n // 4
    fam = []
    # smooth wet states
    h = rng.uniform(0.05, 3.0, (q, 2))
    u = rng.normal(0.0, 1.0, (q, 4))
    fam.append(np.column_stack([h[:, 0], h[:, 0] * u[:, 0], h[:, 0] * u[:, 1], h[:, 1], h[:, 1] * u[:, 2], h[:, 1] * u[:, 3]]))
    # transonic (sonic entropy fix): fast flow of the same sign as a wave
    h = rng.uniform(0.01, 1.0, (q, 2))
    c = np.sqrt(9.81 * h)
    un = np.column_stack([c[:, 0] * rng.uniform(-1.5, 1.5, q), c[:, 1] * rng.uniform(-1.5, 1.5, q)])
    fam.append(np.column_stack([h[:, 0], h[:, 0] * un[:, 0], h[:, 0] * rng.normal(0, 0.5, q),
                                h[:, 1], h[:, 1] * un[:, 1], h[:, 1] * rng.normal(0, 0.5, q)]))
    # dry and nearly dry sides
    h = rng.uniform(0.0, 1.0, (q, 2))
    mask = rng.random((q, 2))
    h[mask < 0.2] = 0.0
    h[(mask >= 0.2) & (mask < 0.35)] = rng.choice([1e-9, 5e-7, 1e-6, 1.5e-6, 1e-5], int(((mask >= 0.2) & (mask < 0.35)).sum()))
    u = rng.normal(0.0, 2.0, (q, 4))
    fam.append(np.column_stack([h[:, 0], h[:, 0] * u[:, 0], h[:, 0] * u[:, 1], h[:, 1], h[:, 1] * u[:, 2], h[:, 1] * u[:, 3]]))
    # equal states (lake at rest) and exact zeros
    m = n - 3 * q
    h = rng.uniform(0.0, 2.0, m)
    z = np.zeros(m)
    fam.append(np.column_stack([h, z, z, h, z, z]))
    states = np.concatenate(fam)
    normals = np.zeros((n, 2))
    normals[0::2, 0] = 1.0
    normals[1::2, 1] = 1.0
    return states, normals


def classic_states(rng, n):
    """(n, 10) = (hi hui hvi zi ni hj huj hvj zj nj), (n, 4) = (dt dx nx ny)."""
    s6, nr = hydro_states(rng, n)
    zi = rng.normal(0.0, 0.3, n)
    zj = zi + rng.normal(0.0, 0.3, n)
    # steps high enough to dry one side, and NODATA-like cliffs
    cliff = rng.random(n) < 0.1
    zj[cliff] = zi[cliff] + rng.choice([-1.0, 1.0], int(cliff.sum())) * rng.uniform(0.5, 5.0, int(cliff.sum()))
    ni = np.where(rng.random(n) < 0.5, 0.0, rng.uniform(0.01, 0.06, n))
    nj = np.where(rng.random(n) < 0.5, ni, rng.uniform(0.0, 0.06, n))
    states = np.column_stack([s6[:, 0:3], zi, ni, s6[:, 3:6], zj, nj])
    dt = rng.uniform(1e-4, 5e-2, n)
    dx = rng.choice([0.01, 0.1, 1.0], n)
    aux = np.column_stack([dt, dx, nr[:, 0], nr[:, 1]])
    return states, aux


def driver_cases():
    """Small single-level cases that reach every branch of the drivers: walls
    with flow against them (both momentum components), mixed and open
    boundaries, NODATA walls, Manning friction, wet/dry fronts, the lake at
    rest, and the classic solver's collapse next to NODATA."""
    from hydroexa_gb300 import workloads
    out = []
    c = workloads.dam_break(40, 32, x_dam=0.25)
    c.hv = 0.3 * c.h
    out.append(("walls_flow", c, (1, 0), 30))
    c = workloads.fractal_dam_break(40, 32, seed=5, amplitude=1.0, nodata_frac=0.15)
    out.append(("fractal_nodata", c, (1,), 12))
    c = workloads.fractal_dam_break(40, 32, seed=6, amplitude=1.0, nodata_frac=0.0)
    c.n[:] = 0.03
    c.geom.bc_lo, c.geom.bc_hi = (1, 0), (0, 1)
    out.append(("friction_mixed_bc", c, (1, 0), 15))
    c = workloads.fractal_dam_break(37, 23, seed=9, amplitude=0.5, nodata_frac=0.1)
    c.geom.bc_lo, c.geom.bc_hi = (1, 1), (1, 1)
    out.append(("open_ragged", c, (1,), 15))
    c = workloads.fractal_dam_break(37, 23, seed=9, amplitude=0.5, nodata_frac=0.0)
    c.geom.bc_lo, c.geom.bc_hi = (1, 1), (1, 1)
    out.append(("open_ragged_classic", c, (0,), 15))
    c = workloads.lake_at_rest(40, 40, seed=2, nodata_frac=0.1)
    out.append(("lake_nodata", c, (1,), 25))
    c = workloads.fractal_dam_break(40, 32, seed=12, amplitude=2.0, nodata_frac=0.2)
    out.append(("classic_nodata_collapse", c, (0,), 60))
    return out


def driver_goldens():
    """drivers_{f64,f32}.npz from the reference's own drivers (oracle/ref_level.cpp)."""
    for dtype, sfx in ((np.float64, "f64"), (np.float32, "f32")):
        rec = {}
        for name, c, methods, nsteps in driver_cases():
            g = c.geom
            L = oracle.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
            planes = [a.astype(dtype) for a in (c.h, c.hu, c.hv, c.z, c.n)]
            for k, key in enumerate(("h", "hu", "hv", "z", "n")):
                rec[f"{name}/{key}"] = planes[k]
            rec[f"{name}/geom"] = np.array([g.nx, g.ny, g.bc_lo[0], g.bc_lo[1], g.bc_hi[0], g.bc_hi[1]], np.int32)
            rec[f"{name}/dxdy_cfl"] = np.array([g.dx, g.dy, c.cfl], np.float64)
            rec[f"{name}/nsteps"] = np.int32(nsteps)
            rec[f"{name}/methods"] = np.array(methods, np.int32)
            for m in methods:
                rec[f"{name}/m{m}/dt0"] = np.float64(oracle.ref_compute_dt(L, m, *planes[:4], cfl=1.0))
                for fa, tag in ((True, "fabs"), (False, "iabs")):
                    h, hu, hv, t, dtl, st = oracle.ref_run(L, m, *planes, nsteps, c.cfl, float_abs=fa)
                    rec[f"{name}/m{m}/{tag}/state"] = np.stack([h, hu, hv])
                    rec[f"{name}/m{m}/{tag}/t_status"] = np.array([t, st], np.float64)
        # tags: an evolved state with one ghost ring copied from the edge, two threshold sets, t = 0 and t > 0
        c = workloads_fractal(48, 36)
        g = c.geom
        L = oracle.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
        h, hu, hv, *_ = oracle.ref_run(L, 1, *[a.astype(dtype) for a in (c.h, c.hu, c.hv, c.z, c.n)], 8, c.cfl)
        U = np.pad(np.stack([h, hu, hv]), ((0, 0), (1, 1), (1, 1)), mode="edge")
        T = np.pad(np.stack([c.z, c.n]).astype(dtype), ((0, 0), (1, 1), (1, 1)), mode="edge")
        rec["tags/U"], rec["tags/T"] = U, T
        rec["tags/dxdy"] = np.array([g.dx, g.dy], np.float64)
        for m in (0, 1):
            for ti, time in enumerate((0.0, 0.5)):
                for si, th in enumerate(((0.5, 0.5, 2.0), (5.0, 20.0, 50.0), (1e9, 1e9, 20.0))):
                    rec[f"tags/m{m}/t{ti}/s{si}"] = oracle.ref_tag_cells(m, U, T, g.dx, g.dy, time, *th)
        np.savez_compressed(OUT / f"drivers_{sfx}.npz", **rec)


def workloads_fractal(nx, ny):
    from hydroexa_gb300 import workloads
    return workloads.fractal_dam_break(nx, ny, seed=31, amplitude=2.0, nodata_frac=0.15)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "drivers":
        if oracle.build_ref() is None:
            raise SystemExit("reference tree not found (oracle/build_ref.sh --root names none)")
        driver_goldens()
        print("driver golden vectors written to", OUT)
        return
    if oracle.build_ref() is None:
        raise SystemExit("reference tree not found (oracle/build_ref.sh --root names none)")
    rng = np.random.default_rng(20261203)

    s, nr = hydro_states(rng, 4096)
    for dt, sfx in ((np.float64, "f64"), (np.float32, "f32")):
        si, ni = s.astype(dt), nr.astype(dt)
        F = oracle.ref_roe_hydrostatic_points(si, ni)
        np.savez_compressed(OUT / f"roe_hydrostatic_{sfx}.npz", states=si, normals=ni, F=F)

    s10, aux = classic_states(rng, 4096)
    for dt, sfx in ((np.float64, "f64"), (np.float32, "f32")):
        si, ai = s10.astype(dt), aux.astype(dt)
        F, Sm, Sp = oracle.ref_roe_classic_points(si, ai)
        np.savez_compressed(OUT / f"roe_classic_{sfx}.npz", states=si, aux=ai, F=F, Sm=Sm, Sp=Sp)

    fine = rng.normal(0.0, 2.0, (2, 48, 64))
    fine[:, rng.random((48, 64)) < 0.35] = -9999.0
    fine[:, 10:18, 20:28] = -9999.0
    fine[0, 5, 7] = np.nan
    fine[1, 30, 33] = -9999.0004  # within the 1e-3 sentinel tolerance
    fv = 0.25 * 0.25
    out = {}
    for r in (2, 4):
        out[f"crse_r{r}"] = oracle.ref_masked_average_down(fine, r, r, fv)
    np.savez_compressed(OUT / "masked_avgdown_f64.npz", fine=fine, fine_volume=np.float64(fv), **out)

    spec = importlib.util.spec_from_file_location("hx_ref_analytical", REF / "tests" / "dambreak" / "analytical.py")
    mod = importlib.util.module_from_spec(spec)
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        spec.loader.exec_module(mod)
        x = (np.arange(256) + 0.5) / 256.0
        prof = {}
        for t in (0.05, 0.1, 0.15):
            h, u = mod.dambreak_on_wet_no_friction_analytical(t, x, L=1.0, hl=1.0, hr=0.1, x0=0.5)[:2]
            prof[f"h_t{t}"] = np.asarray(h, dtype=np.float64)
            prof[f"u_t{t}"] = np.asarray(u, dtype=np.float64)
    np.savez_compressed(OUT / "dambreak_exact.npz", x=x, hl=1.0, hr=0.1, x0=0.5, **prof)
    driver_goldens()
    print("golden vectors written to", OUT)


if __name__ == "__main__":
    main()
