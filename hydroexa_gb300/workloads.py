"""Seeded synthetic inputs with the shapes of the benchmark configurations.

Every generator returns numpy float64 planes ``(h, hu, hv, z, n)`` of shape
(ny, nx) plus the level geometry.  NODATA cells carry z = n = -9999 (both
terrain components, as the reference's HDF5 reader and static database do,
src/io/IOHandler.cpp:212-216) and a dry, still fluid state: the reference
builds eta = z there (src/state/AmrMeshState_AMR.cpp:80-86), so h = 0.

Random numbers come from ``numpy.random.Generator(PCG64(seed))``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .level import Geometry

NODATA = -9999.0


@dataclass
class Case:
    name: str
    geom: Geometry
    h: np.ndarray
    hu: np.ndarray
    hv: np.ndarray
    z: np.ndarray
    n: np.ndarray
    cfl: float
    nsteps: int
    method: int  # capi.HX_METHOD_*

    @property
    def cells(self) -> int:
        return self.geom.nx * self.geom.ny


def _centres(nx, ny, lx=1.0, ly=1.0):
    x = (np.arange(nx) + 0.5) * (lx / nx)
    y = (np.arange(ny) + 0.5) * (ly / ny)
    return np.meshgrid(x, y)


def _apply_nodata(mask, h, hu, hv, z, n):
    z[mask] = NODATA
    n[mask] = NODATA
    h[mask] = 0.0
    hu[mask] = 0.0
    hv[mask] = 0.0


def dam_break(nx=256, ny=256, method=1, cfl=0.45, nsteps=200, h_left=1.0, h_right=0.1, x_dam=0.5):
    """Plain dam break on [0,1]^2: flat bed, h = 1.0 for x < 0.5 else 0.1, walls."""
    X, _ = _centres(nx, ny)
    h = np.where(X < x_dam, h_left, h_right).astype(np.float64)
    z = np.zeros_like(h)
    geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (0, 0), (0, 0))
    return Case("dam_break_%dx%d" % (nx, ny), geom, h, np.zeros_like(h), np.zeros_like(h), z, np.zeros_like(h), cfl,
                nsteps, method)


def lake_at_rest(nx=512, ny=512, seed=2, nodata_frac=0.10, cfl=0.5, nsteps=1000, method=1):
    """Lake at rest over a Gaussian mound with seeded N(0, 0.02) roughness and a
    seeded axis-aligned NODATA rectangle covering ~10% of the cells."""
    rng = np.random.default_rng(seed)
    X, Y = _centres(nx, ny)
    z = 0.8 * np.exp(-((X - 0.5) ** 2 + (Y - 0.5) ** 2) / 0.01) + rng.normal(0.0, 0.02, (ny, nx))
    h = np.maximum(0.0, 1.0 - z)
    hu = np.zeros_like(h)
    hv = np.zeros_like(h)
    n = np.zeros_like(h)
    if nodata_frac > 0:
        area = nodata_frac * nx * ny
        w = int(round(math.sqrt(area * rng.uniform(0.5, 2.0))))
        w = max(1, min(nx - 2, w))
        hgt = max(1, min(ny - 2, int(round(area / w))))
        i0 = int(rng.integers(0, nx - w + 1))
        j0 = int(rng.integers(0, ny - hgt + 1))
        mask = np.zeros((ny, nx), dtype=bool)
        mask[j0:j0 + hgt, i0:i0 + w] = True
        _apply_nodata(mask, h, hu, hv, z, n)
    geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (0, 0), (0, 0))
    return Case("lake_at_rest_%dx%d" % (nx, ny), geom, h, hu, hv, z, n, cfl, nsteps, method)


def spectral_field(nx, ny, exponent, rng):
    """Gaussian random field with power spectrum ~ |k|^exponent, zero mean, unit std."""
    kx = np.fft.rfftfreq(nx) * nx
    ky = np.fft.fftfreq(ny) * ny
    KX, KY = np.meshgrid(kx, ky)
    k2 = KX ** 2 + KY ** 2
    k2[0, 0] = 1.0
    amp = k2 ** (exponent / 4.0)  # |F| ~ |k|^(exponent/2)
    amp[0, 0] = 0.0
    coef = (rng.standard_normal(amp.shape) + 1j * rng.standard_normal(amp.shape)) * amp
    f = np.fft.irfft2(coef, s=(ny, nx))
    f -= f.mean()
    s = f.std()
    return f / s if s > 0 else f


def fractal_dam_break(nx=8192, ny=8192, seed=3, nodata_frac=0.20, amplitude=5.0, cfl=0.45, nsteps=100, method=1):
    """Throughput case: spectral fractal terrain (power law k^-2) scaled to a
    5 m range, NODATA where a smoother seeded noise exceeds its 80th percentile,
    circular dam of radius 0.1 at the centre: depth 2.0 m inside, 0.5 m outside."""
    rng = np.random.default_rng(seed)
    z = spectral_field(nx, ny, -2.0, rng)
    z = (z - z.min()) / max(z.max() - z.min(), 1e-300) * amplitude
    mask_noise = spectral_field(nx, ny, -3.0, rng)
    thr = np.quantile(mask_noise, 1.0 - nodata_frac)
    mask = mask_noise > thr
    X, Y = _centres(nx, ny)
    h = np.where((X - 0.5) ** 2 + (Y - 0.5) ** 2 < 0.1 ** 2, 2.0, 0.5)
    hu = np.zeros_like(h)
    hv = np.zeros_like(h)
    n = np.zeros_like(h)
    _apply_nodata(mask, h, hu, hv, z, n)
    geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (0, 0), (0, 0))
    return Case("fractal_dam_break_%dx%d" % (nx, ny), geom, h, hu, hv, z, n, cfl, nsteps, method)


def ensemble(count=256, seed=4, smin=64, smax=1024, nsteps=500, cfl=0.45, method=1):
    """Independent dam breaks of uneven size: side ~ logUniform[64, 1024]
    rounded to a multiple of 16, dam position U(0.3, 0.7), upstream depth
    U(0.5, 3.0), downstream U(0.05, 0.5), Gaussian bump bed of amplitude
    U(0, 0.5) at a random centre (sigma 0.1 of the domain)."""
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(count):
        side = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax))) / 16.0)) * 16
        side = max(smin, min(smax, side))
        xd = rng.uniform(0.3, 0.7)
        hl = rng.uniform(0.5, 3.0)
        hr = rng.uniform(0.05, 0.5)
        amp = rng.uniform(0.0, 0.5)
        cx, cy = rng.uniform(0.2, 0.8, 2)
        X, Y = _centres(side, side)
        z = amp * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * 0.1 ** 2))
        eta = np.where(X < xd, hl, hr)
        h = np.maximum(0.0, eta - z)
        geom = Geometry(side, side, 1.0 / side, 1.0 / side, (0, 0), (0, 0))
        cases.append(Case("ens%03d_%d" % (k, side), geom, h, np.zeros_like(h), np.zeros_like(h), z,
                          np.zeros_like(h), cfl, nsteps, method))
    return cases


def smooth_field(nx, ny, seed, amplitude, ngauss=8):
    """Sum of seeded Gaussians scaled to a maximum magnitude of ``amplitude``."""
    rng = np.random.default_rng(seed)
    X, Y = _centres(nx, ny)
    f = np.zeros((ny, nx))
    for _ in range(ngauss):
        cx, cy = rng.uniform(0.0, 1.0, 2)
        s = rng.uniform(0.05, 0.2)
        f += rng.uniform(-1.0, 1.0) * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    return amplitude * f / max(np.abs(f).max(), 1e-300)


def adjoint_case(nx=512, ny=512, seed=5, ngauss=32, amplitude=0.3, hump=0.2, ngauges=64, nsteps=2000, cfl=0.45):
    """Smooth bed (sum of 32 seeded Gaussians scaled to 0.3 m), free surface
    1.0 plus a 0.2 m Gaussian hump, and 64 seeded gauge cells."""
    rng = np.random.default_rng(seed)
    X, Y = _centres(nx, ny)
    z = np.zeros((ny, nx))
    for _ in range(ngauss):
        cx, cy = rng.uniform(0.0, 1.0, 2)
        s = rng.uniform(0.03, 0.12)
        a = rng.uniform(-1.0, 1.0)
        z += a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    z *= amplitude / max(np.abs(z).max(), 1e-300)
    eta = 1.0 + hump * np.exp(-((X - 0.5) ** 2 + (Y - 0.5) ** 2) / (2 * 0.05 ** 2))
    h = np.maximum(0.0, eta - z)
    gauges = rng.choice(nx * ny, size=ngauges, replace=False)
    geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (0, 0), (0, 0))
    case = Case("adjoint_%dx%d" % (nx, ny), geom, h, np.zeros_like(h), np.zeros_like(h), z, np.zeros_like(h), cfl,
                nsteps, 1)
    return case, gauges


def adjoint_monotone_case(nx=512, ny=512, seed=5, ngauges=64, nsteps=100, cfl=0.45):
    """A state on which the step map has no kink near the gauges' domain of
    dependence: a planar bed (0.2 x + 0.1 y, so the face bed max(zL, zR) never
    switches side), a free surface and currents increasing strictly in x and y
    (every van Leer ratio positive, no limiter at r <= 0 or on the flat-data
    branch), open boundaries (the edge copies hold the edge slopes at exactly
    zero whatever the perturbation) and gauges in the central [0.3, 0.7]^2,
    farther from the boundaries than any wave travels in nsteps."""
    rng = np.random.default_rng(seed)
    X, Y = _centres(nx, ny)
    z = 0.2 * X + 0.1 * Y
    eta = 1.0 + 0.03 * X + 0.02 * Y + 0.01 * X * Y
    h = eta - z
    u = 0.10 + 0.05 * X + 0.02 * Y
    v = 0.05 + 0.03 * Y + 0.01 * X
    gi = rng.integers(int(0.3 * nx), int(0.7 * nx), size=ngauges)
    gj = rng.integers(int(0.3 * ny), int(0.7 * ny), size=ngauges)
    gauges = np.unique(gi + gj * nx)
    geom = Geometry(nx, ny, 1.0 / nx, 1.0 / ny, (1, 1), (1, 1))
    case = Case("adjoint_monotone_%dx%d" % (nx, ny), geom, h, h * u, h * v, z, np.zeros_like(h), cfl, nsteps, 1)
    return case, gauges


def adjoint_smooth_case(nx=512, ny=512, seed=5, ngauges=64, nsteps=100, cfl=0.45):
    """The adjoint bed and gauges with a state that has no quiescent region:
    free surface 1.0 + 0.05 m undulation + 0.2 m hump (centre off the cell
    boundaries) and smooth currents of up to 0.2 m/s, so the limiters stay off
    their flat-data branch and the misfit is differentiable."""
    case, gauges = adjoint_case(nx, ny, seed=seed, ngauges=ngauges, nsteps=nsteps, cfl=cfl)
    X, Y = _centres(nx, ny)
    eta = (1.0 + 0.05 * smooth_field(nx, ny, seed + 100, 1.0)
           + 0.2 * np.exp(-((X - 0.4637) ** 2 + (Y - 0.5311) ** 2) / (2 * 0.05 ** 2)))
    case.h = np.maximum(0.0, eta - case.z)
    case.hu = case.h * 0.2 * smooth_field(nx, ny, seed + 101, 1.0)
    case.hv = case.h * 0.2 * smooth_field(nx, ny, seed + 102, 1.0)
    case.name = "adjoint_smooth_%dx%d" % (nx, ny)
    return case, gauges
