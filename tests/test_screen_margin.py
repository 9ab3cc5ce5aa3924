"""The float screen of the FP64 CFL fold, checked on the CPU.

The fast form folds the CFL bound through a float screen (screened_fold in
hydroexa_gb300/csrc/hx_kernels.cuh): every wet cell's rate
(|u| + c) / dx + (|v| + c) / dy and speed max(|u|, |v|) are estimated in float
from the leading 24 bits of h, hu, hv (f32_lead, a truncation), and only the
cells whose estimate is within 2^-12 of the block's largest estimate are
evaluated in FP64.  The result equals the fold over every cell as long as each
estimate is within a relative error e of its FP64 value with
(1 + e) / (1 - e) < 1 / (1 - 2^-12): then the cell holding the true maximum
always passes.  This test emulates the estimate in numpy float32 with the
hardware approximations (rcp.approx, sqrt.approx) replaced by correctly
rounded results pushed 2 ulps the wrong way, over states from dry-edge depths
to fast flows, and bounds e (measured: 2^-20.7 for the rate, 2^-21.0 for the
speed, against the 2^-12 of the screen).
"""
import numpy as np

MARGIN = 2.0 ** -12
WORST_ULPS = 2.0 * 2.0 ** -23  # a generous bound for rcp.approx.ftz.f32 and sqrt.approx.ftz.f32


def f32_lead(x):
    """The leading 24 significand bits of doubles as floats (truncated toward
    zero), for zeros and doubles inside the float normal range."""
    b = np.atleast_1d(np.asarray(x, dtype=np.float64)).view(np.uint64)
    sign = (b >> np.uint64(32)) & np.uint64(0x80000000)
    de = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    mant = (b >> np.uint64(29)) & np.uint64(0x7FFFFF)
    fe = de - 1023 + 127
    zero = (b << np.uint64(1)) == 0
    assert ((fe > 0) & (fe < 255) | zero).all(), "inputs must be zero or inside the float normal range"
    f = np.where(zero, sign, sign | (np.maximum(fe, 0).astype(np.uint64) << np.uint64(23)) | mant)
    return f.astype(np.uint32).view(np.float32)


def push(x, sgn):
    """x moved 2 ulps (relative) up (sgn = 1) or down (sgn = -1), in float."""
    return (x.astype(np.float64) * (1.0 + sgn * WORST_ULPS)).astype(np.float32)


def estimate(h, hu, hv, idx, idy, sgn):
    """The screen's float rate and speed, approximations pushed by sgn."""
    hf = f32_lead(h)
    qx = np.abs(f32_lead(hu))
    qy = np.abs(f32_lead(hv))
    rh = push(np.float32(1.0) / hf, sgn)
    u = qx * rh
    v = qy * rh
    cc = push(np.sqrt(np.float32(9.81) * hf), sgn)
    r = (u + cc) * f32_lead(idx) + (v + cc) * f32_lead(idy)
    return r, np.maximum(u, v)


def exact(h, hu, hv, idx, idy):
    u, v = np.abs(hu / h), np.abs(hv / h)
    c = np.sqrt(9.81 * h)
    return (u + c) * idx + (v + c) * idy, np.maximum(u, v)


def states(n, seed):
    rng = np.random.default_rng(seed)
    h = 10.0 ** rng.uniform(-12, 4, n)                    # dry edge (1e-12 m) to 10 km of water
    speed = 10.0 ** rng.uniform(-30, 3, n)                # still water to 1 km/s
    ang = rng.uniform(0, 2 * np.pi, n)
    hu, hv = h * speed * np.cos(ang), h * speed * np.sin(ang)
    hu[rng.random(n) < 0.05] = 0.0
    keep = (np.abs(hu) > 2e-38) | (hu == 0)
    keep &= (np.abs(hv) > 2e-38) | (hv == 0)
    return h[keep], hu[keep], hv[keep]


def test_estimate_error_is_far_inside_the_margin():
    worst_r = worst_m = 0.0
    for seed in range(4):
        h, hu, hv = states(200_000, seed)
        for dx in (1e-3, 0.37, 25.0, 1e4):
            idx, idy = np.float64(1.0) / dx, np.float64(1.0) / (1.7 * dx)
            r64, m64 = exact(h, hu, hv, idx, idy)
            for sgn in (-1, 1):
                r32, m32 = estimate(h, hu.copy(), hv.copy(), idx, idy, sgn)
                assert np.isfinite(r32).all()
                worst_r = max(worst_r, float(np.max(np.abs(r32 / r64 - 1.0))))
                moving = m64 > 2e-37  # the speed is estimated relatively where it is a float normal
                worst_m = max(worst_m, float(np.max(np.abs(m32[moving] / m64[moving] - 1.0))))
    e = max(worst_r, worst_m)
    assert e < 2.0 ** -19, (worst_r, worst_m)
    assert (1 + e) / (1 - e) < 1 / (1 - MARGIN)


def test_the_true_maximum_is_always_a_candidate():
    """Blocks of 256 cells with near-ties: the cell of the exact maximum rate
    and the cell of the exact maximum speed both pass the screen."""
    rng = np.random.default_rng(11)
    for trial in range(400):
        h, hu, hv = states(4096, 100 + trial)
        h, hu, hv = h[:256], hu[:256], hv[:256]
        # near-ties: copies of one cell nudged by a few ulps of double
        k = rng.integers(0, h.size, 16)
        h[k[8:]] = h[k[0]] * (1 + rng.integers(-4, 5, 8) * 2.0 ** -52)
        hu[k[8:]] = hu[k[0]]
        hv[k[8:]] = hv[k[0]]
        idx, idy = 1.0 / 3.3, 1.0 / 2.9
        r64, m64 = exact(h, hu, hv, idx, idy)
        for sgn in (-1, 1):
            r32, m32 = estimate(h, hu, hv, idx, idy, sgn)
            kr, km = r32.max() * np.float32(1 - MARGIN), m32.max() * np.float32(1 - MARGIN)
            assert r32[np.argmax(r64)] >= kr
            assert m32[np.argmax(m64)] >= km


SQRT_G = 3.1320919526731650  # sqrt(9.81) correctly rounded, the FP64 constant of the Roe flux


def sonic_rules(ui, si, uj, sj):
    """The float rules of the hydrostatic Roe flux (roe_hydrostatic_fast in
    hydroexa_gb300/csrc/hx_device.cuh): rule0 (rule2) true means the entropy
    fix of the slow (fast) wave is ruled out without FP64 work."""
    ui32, uj32 = f32_lead(ui), f32_lead(uj)
    ci32 = np.float32(3.13209195) * f32_lead(si)
    cj32 = np.float32(3.13209195) * f32_lead(sj)
    mi = np.float32(2.0 ** -16) * (np.abs(ui32) + ci32)
    mj = np.float32(2.0 ** -16) * (np.abs(uj32) + cj32)
    rule0 = (ui32 - ci32 >= mi) | (uj32 - cj32 <= -mj)
    rule2 = (ui32 + ci32 >= mi) | (uj32 + cj32 <= -mj)
    return rule0, rule2


def test_sonic_screen_rules_out_only_impossible_fixes():
    """Each entropy fix needs e_i < 0 < e_j (e = u -+ sqrt(g) s, s = sqrt(h)).
    Where a float rule rules a fix out, the exact signs agree: e_i >= 0 or
    e_j <= 0.  Wet sides (h >= 1e-6, so |u| + c >= 3e-3) and dry sides
    (h = u = 0), velocities at, near (to 2^-50) and away from the sonic point;
    the rules decide most subsonic faces."""
    rng = np.random.default_rng(5)
    n = 400_000
    wet_i, wet_j = rng.random(n) > 0.05, rng.random(n) > 0.05
    si = np.where(wet_i, np.sqrt(10.0 ** rng.uniform(-6, 4, n)), 0.0)
    sj = np.where(wet_j, np.sqrt(10.0 ** rng.uniform(-6, 4, n)), 0.0)

    def speeds(s, wet):
        c = SQRT_G * s
        kind = rng.integers(0, 4, n)
        near = c * (1 + rng.choice([-1.0, 1.0], n) * 2.0 ** rng.uniform(-50, -8, n))
        u = np.select([kind == 0, kind == 1, kind == 2], [c, near, rng.uniform(-5, 5, n) * c],
                      rng.uniform(-1e-3, 1e-3, n))
        u = u * rng.choice([-1.0, 1.0], n)
        return np.where(wet, u, 0.0)

    ui, uj = speeds(si, wet_i), speeds(sj, wet_j)
    rule0, rule2 = sonic_rules(ui, si, uj, sj)
    L = np.longdouble
    ci, cj = L(SQRT_G) * si.astype(L), L(SQRT_G) * sj.astype(L)
    for rule, ei, ej in ((rule0, ui.astype(L) - ci, uj.astype(L) - cj), (rule2, ui.astype(L) + ci, uj.astype(L) + cj)):
        possible = (ei < 0) & (ej > 0)
        assert not (rule & possible).any()
    subsonic = wet_i & wet_j & (np.abs(ui) < 0.9 * SQRT_G * si) & (np.abs(uj) < 0.9 * SQRT_G * sj)
    assert (rule0 & rule2)[subsonic].mean() > 0.99
