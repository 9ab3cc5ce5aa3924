"""Regenerate the golden vectors in this folder from the reference itself.

Run from the repository root, in a checkout that has the reference source tree
(default /root/reference, or $HX_REFERENCE_ROOT):

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
REF = Path(os.environ.get("HX_REFERENCE_ROOT", "/root/reference"))


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


def main():
    if oracle.build_ref() is None:
        raise SystemExit(f"reference tree not found at {REF}")
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
    print("golden vectors written to", OUT)


if __name__ == "__main__":
    main()
