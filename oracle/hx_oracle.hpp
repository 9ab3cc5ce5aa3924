// CPU oracle for the HydroEXA per-level advance.
//
// TEST INFRASTRUCTURE ONLY.  This header is the checker that the CUDA kernels of
// hydroexa_gb300 are compared against; nothing in the product library includes,
// links or calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load the shared library built from it.
//
// It restates, in plain scalar C++, the arithmetic of the reference solver
// (jkhansell/HydroEXA) for one AMR level, one box covering the whole domain:
//
//   roe_hydrostatic ....... include/solvers/kernels/HydrostaticRoe.H:44-159
//   roe_classic ........... include/solvers/kernels/Roe.H:51-309
//   van_leer_limiter/slope  src/solvers/HydrostaticRoe.cpp:173-195
//   hydrostatic face flux . src/solvers/HydrostaticRoe.cpp:197-398
//   hydrostatic advance ... src/solvers/HydrostaticRoe.cpp:400-606 (h rebuild :490-500,
//                           update :551-604)
//   classic advance ....... src/solvers/Roe.cpp:184-248 (faces, h rebuild),
//                           :250-434 (fill, faces, update)
//   compute_dt ............ src/solvers/HydrostaticRoe.cpp:7-86, src/solvers/Roe.cpp:8-98
//   tag_cells ............. src/solvers/HydrostaticRoe.cpp:88-171, src/solvers/Roe.cpp:100-181
//   masked average-down ... include/utils/MaskedAverageDown.H:64-104,
//                           src/utils/MaskedAverageDown.cpp:12-63
//   ghost rules ........... include/boundaries/BCFill.H:35-86,159-181 (AMReX FilccCell
//                           foextrap / reflect_even / reflect_odd), terrain always
//                           foextrap (src/state/AmrMeshState_Init.cpp:61-70)
//   eta derivation ........ src/state/AmrMeshState_AMR.cpp:203-224 (eta = h + z)
//
// Every expression keeps the reference's operation order and literal types
// (double literals promote float operands exactly as the reference's SINGLE
// build does), so oracle<double> reproduces the reference DOUBLE build bit for
// bit where the reference kernels were compiled here (tests/golden), and the
// passes are kept separate (ghost fill, h rebuild, face arrays, update) as in
// the reference rather than fused.
//
// Built with -ffp-contract=off: no multiply-add contraction on x86 or Arm.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <limits>
#include <vector>

namespace hxo {

// include/utils/Constants.H:25-78.  Each is a function returning Real in the
// reference, so in a float instantiation the constant is rounded to float.
template <class R> struct K {
    static R grav() { return R(9.81); }
    static R toldry() { return R(1e-6); }
    static R tol12() { return R(1e-12); }
    static R tol10() { return R(1e-10); }
};

// std::max / std::min semantics (first argument wins ties and NaN compares).
template <class R> inline R smax(R a, R b) { return (a < b) ? b : a; }
template <class R> inline R smin(R a, R b) { return (b < a) ? b : a; }

// The reference's vanLeerLimiter calls an unqualified abs(r).  Whether that
// resolves to the floating std::abs or to C's int abs(int) depends on which
// headers the translation unit pulled in (it is <cmath>-only in some builds).
// LIMITER_FLOAT_ABS is the intended behaviour and the default everywhere;
// LIMITER_INT_ABS reproduces the int-abs resolution for comparison.
enum LimiterAbs { LIMITER_FLOAT_ABS = 0, LIMITER_INT_ABS = 1 };

template <class R> inline R limiter_abs(R r, int mode) {
    if (mode == LIMITER_INT_ABS) {
        // abs((int)r): truncation toward zero, then converted back in the
        // expression.  A value outside the int range (or NaN) has no defined
        // conversion in C; this follows what the x86-64 build of the
        // reference does (cvttsd2si / cvttss2si give INT_MIN, and abs(INT_MIN)
        // wraps to INT_MIN), the machine the golden vectors come from.
        const double t = (double)r;
        long long v;
        if (!(t == t) || t >= 2147483648.0 || t <= -2147483649.0) v = -2147483648ll;
        else v = (long long)(int)t;
        const long long a = (v == -2147483648ll) ? v : (v < 0 ? -v : v);
        return (R)a;
    }
    return std::abs(r);
}

// src/solvers/HydrostaticRoe.cpp:173-177
template <class R> inline R van_leer_limiter(R r, int mode) {
    return (r + limiter_abs(r, mode)) / (R(1) + limiter_abs(r, mode));
}

// src/solvers/HydrostaticRoe.cpp:179-195
template <class R> inline R van_leer_slope(R qim1, R qi, R qip1, int mode) {
    const R dm = qi - qim1;
    const R dp = qip1 - qi;
    if (std::abs(dp) <= K<R>::tol12()) return R(0.0);
    const R r = dm / dp;
    return van_leer_limiter(r, mode) * dp;
}

// Homogeneous Roe flux of two reconstructed face states,
// include/solvers/kernels/HydrostaticRoe.H:44-159.
template <class R>
inline void roe_hydrostatic(R hi, R hui, R hvi, R hj, R huj, R hvj, R F[3], R nx, R ny) {
    const R g = K<R>::grav();
    hi = (hi >= K<R>::toldry()) ? hi : 0.0;
    hj = (hj >= K<R>::toldry()) ? hj : 0.0;

    R si = (hi > 0.0) ? std::sqrt(hi) : 0.0;
    R sj = (hj > 0.0) ? std::sqrt(hj) : 0.0;

    R ui = (hi > 0.0) ? hui / hi : 0.0;
    R vi = (hi > 0.0) ? hvi / hi : 0.0;
    R uj = (hj > 0.0) ? huj / hj : 0.0;
    R vj = (hj > 0.0) ? hvj / hj : 0.0;

    R uni = ui * nx + vi * ny;
    R uti = -ui * ny + vi * nx;
    R unj = uj * nx + vj * ny;
    R utj = -uj * ny + vj * nx;

    R hm = (0.5 * (hi + hj) > K<R>::toldry()) ? 0.5 * (hi + hj) : K<R>::toldry();
    R cm = std::sqrt(g * hm);
    R sden = si + sj + K<R>::tol12();
    R um = (uni * si + unj * sj) / sden;
    R vm = (uti * si + utj * sj) / sden;

    R l0 = um - cm;
    R l1 = um;
    R l2 = um + cm;
    {
        R ei = uni - std::sqrt(g * hi);
        R ej = unj - std::sqrt(g * hj);
        if (ei < 0.0 && ej > 0.0) l0 = ei * (ej - l0) / (ej - ei);
        ei = uni + std::sqrt(g * hi);
        ej = unj + std::sqrt(g * hj);
        if (ei < 0.0 && ej > 0.0) l2 = ej * (l2 - ei) / (ej - ei);
    }
    R den = 2.0 * cm + K<R>::tol12();
    R dh = hj - hi;
    R dhu = hj * unj - hi * uni;
    R dhv = hj * utj - hi * uti;
    R a0 = (l2 * dh - dhu) / den;
    R a1 = (-vm * dh + dhv) / cm;
    R a2 = (-l0 * dh + dhu) / den;

    F[0] = 0.5 * (hi * uni + hj * unj);
    F[1] = 0.5 * (hi * uni * uni + 0.5 * g * hi * hi + hj * unj * unj + 0.5 * g * hj * hj);
    F[2] = 0.5 * (hi * uni * uti + hj * unj * utj);

    for (int k = 0; k < 3; ++k) {
        R lk = (k == 0) ? l0 : ((k == 1) ? l1 : l2);
        R ak = (k == 0) ? a0 : ((k == 1) ? a1 : a2);
        R e0 = (k == 1) ? 0.0 : 1.0;
        R e1 = (k == 0) ? l0 : (k == 1 ? 0.0 : l2);
        R e2 = (k == 0) ? vm : (k == 1 ? cm : vm);
        R w = 0.5 * std::abs(lk) * ak;
        F[0] -= w * e0;
        F[1] -= w * e1;
        F[2] -= w * e2;
    }
    R t1 = F[1], t2 = F[2];
    F[1] = t1 * nx - t2 * ny;
    F[2] = t1 * ny + t2 * nx;
}

// Classic Roe flux with upwinded bed-slope thrust and Manning friction,
// include/solvers/kernels/Roe.H:51-309.
template <class R>
inline void roe_classic(R hi, R hui, R hvi, R zi, R ni, R hj, R huj, R hvj, R zj, R nj,
                        R F[3], R Sm[3], R Sp[3], R dt, R dx, R nx, R ny) {
    (void)dt;
    const R g = K<R>::grav();
    const R T12 = K<R>::tol12();
    const R TD = K<R>::toldry();
    hi = (hi >= TD) ? hi : 0.0;
    hj = (hj >= TD) ? hj : 0.0;

    R si = (hi > 0.0) ? std::sqrt(hi) : 0.0;
    R sj = (hj > 0.0) ? std::sqrt(hj) : 0.0;
    R ui = (hi > 0.0) ? hui / hi : 0.0;
    R vi = (hi > 0.0) ? hvi / hi : 0.0;
    R uj = (hj > 0.0) ? huj / hj : 0.0;
    R vj = (hj > 0.0) ? hvj / hj : 0.0;

    R uni = ui * nx + vi * ny;
    R uti = -ui * ny + vi * nx;
    R unj = uj * nx + vj * ny;
    R utj = -uj * ny + vj * nx;

    R hm = (0.5 * (hi + hj) > TD) ? 0.5 * (hi + hj) : TD;
    R cm = std::sqrt(g * hm);
    R sden = si + sj + T12;
    R um = (uni * si + unj * sj) / sden;
    R vm = (uti * si + utj * sj) / sden;

    R l0 = um - cm;
    R l1 = um;
    R l2 = um + cm;
    {
        R ei = uni - std::sqrt(g * hi);
        R ej = unj - std::sqrt(g * hj);
        if (ei < 0.0 && ej > 0.0) l0 = ei * (ej - l0) / (ej - ei);
        ei = uni + std::sqrt(g * hi);
        ej = unj + std::sqrt(g * hj);
        if (ei < 0.0 && ej > 0.0) l2 = ej * (l2 - ei) / (ej - ei);
    }
    R den = 2.0 * cm + T12;
    R dh = hj - hi;
    R dhu = hj * unj - hi * uni;
    R dhv = hj * utj - hi * uti;
    R a0 = (l2 * dh - dhu) / den;
    R a1 = (-vm * dh + dhv) / cm;
    R a2 = (-l0 * dh + dhu) / den;

    // bed-slope thrust, Roe.H:151-176
    R dz = zj - zi;
    R di = hi + zi;
    R dj = hj + zj;
    R dd = dj - di;
    R thrust, tau;
    {
        R ta = -g * hm * dz;
        R dzt;
        if ((dz >= 0.0) && (di < zj)) dzt = hi;
        else if ((dz < 0.0) && (dj < zi)) dzt = hj;
        else dzt = dz;
        R hr = (dz >= 0.0) ? hi : hj;
        R tb = -g * (hr - 0.5 * std::abs(dzt)) * dzt;
        thrust = ((dz * dd >= 0.0) && (um * dz > 0.0)) ? smax(ta, tb) : tb;
        // Manning friction, Roe.H:182-188
        R nm = 0.5 * (ni + nj);
        R sf = (nm * nm * std::sqrt(um * um + vm * vm) * um) / smax(TD, hm * std::cbrt(hm));
        tau = g * hm * sf * dx;
    }

    R b0 = (thrust - tau) / den;
    R b1 = 0.0;
    R b2 = -b0;
    {
        // positivity guard, Roe.H:200-247
        const R l0s = (std::abs(l0) > T12) ? l0 : (l0 >= 0.0 ? T12 : -T12);
        const R l2s = (std::abs(l2) > T12) ? l2 : (l2 >= 0.0 ? T12 : -T12);
        const R hi1 = hi + a0 - (b0 / l0s);
        const R hj3 = hj - a2 + (b2 / l2s);
        R ml = std::abs(l0);
        ml = smax(ml, std::abs(l1));
        ml = smax(ml, std::abs(l2));
        const R ldt = dx / (ml + T12);
        const R d1 = hi - hi1;
        const R d1s = (std::abs(d1) > T12) ? d1 : (d1 >= 0.0 ? T12 : -T12);
        const R d3 = hj - hj3;
        const R d3s = (std::abs(d3) > T12) ? d3 : (d3 >= 0.0 ? T12 : -T12);
        const R dt1 = (dx * 0.5 / l0s) * (hi / d1s);
        const R dt3 = (dx * 0.5 / l2s) * (hj / d3s);
        if ((hi1 < -TD) && (hj3 > TD) && (dt1 < ldt)) {
            const R b1min = -(hi + a0) * std::abs(l0);
            const R b3min = -(hj - a2) * l2;
            if (-b1min >= b3min) b0 = b1min;
            b2 = -b0;
        }
        if ((hi1 > TD) && (hj3 < -TD) && (dt3 < ldt)) {
            const R b1min = -(hi + a0) * std::abs(l0);
            const R b3min = -(hj - a2) * l2;
            if (-b3min >= b1min) b2 = b3min;
            b0 = -b2;
        }
    }
    for (int k = 0; k < 3; ++k) { Sm[k] = 0.0; Sp[k] = 0.0; }
    F[0] = 0.5 * (hi * uni + hj * unj);
    F[1] = 0.5 * (hi * uni * uni + 0.5 * g * hi * hi + hj * unj * unj + 0.5 * g * hj * hj);
    F[2] = 0.5 * (hi * uni * uti + hj * unj * utj);
    for (int k = 0; k < 3; ++k) {
        R lk = (k == 0) ? l0 : ((k == 1) ? l1 : l2);
        R ak = (k == 0) ? a0 : ((k == 1) ? a1 : a2);
        R bk = (k == 0) ? b0 : ((k == 1) ? b1 : b2);
        R e0 = (k == 1) ? 0.0 : 1.0;
        R e1 = (k == 0) ? l0 : (k == 1 ? 0.0 : l2);
        R e2 = (k == 0) ? vm : (k == 1 ? cm : vm);
        R w = 0.5 * std::abs(lk) * ak;
        F[0] -= w * e0;
        F[1] -= w * e1;
        F[2] -= w * e2;
        if (lk > 0.0) {
            Sm[0] += bk * e0; Sm[1] += bk * e1; Sm[2] += bk * e2;
        } else if (lk < 0.0) {
            Sp[0] += bk * e0; Sp[1] += bk * e1; Sp[2] += bk * e2;
        }
    }
    R t1 = F[1], t2 = F[2];
    F[1] = t1 * nx - t2 * ny;
    F[2] = t1 * ny + t2 * nx;
    t1 = Sm[1]; t2 = Sm[2];
    Sm[1] = t1 * nx - t2 * ny;
    Sm[2] = t1 * ny + t2 * nx;
    t1 = Sp[1]; t2 = Sp[2];
    Sp[1] = t1 * nx - t2 * ny;
    Sp[2] = t1 * ny + t2 * nx;
}

// ---------------------------------------------------------------------------
// Ghost-extended single-box level.
// ---------------------------------------------------------------------------

// Physical boundary kinds of the inputs file (include/boundaries/BCFill.H:35-138):
// code 0 is a reflective wall, any other code is transmissive (foextrap) --
// except 2, a closed wall of this library (below), which the reference's
// inputs do not have.
//
// Code 0, the reference's wall, as its time loop fills the ghosts: the state
// ghosts come from FillPatch(lev, time, U_ext, UBCs, 1, 2) (HydrostaticRoe.cpp
// :477, Roe.cpp:337), which reaches the BC functor through FillPatchFrom ->
// FillPatchSingleLevel(..., fphysbc, 0) (include/utils/FillPatchUtils.H
// :128-129); HydroPhysBC starts at BC record 0 for the first filled component
// (BCFill.H:244-264), so hu (component 1) takes record 0 -- the scalar rule,
// reflect_even on every wall -- and hv (component 2) takes record 1, the
// x-momentum rules: reflect_odd across x walls, reflect_even across y walls.
// Code 2 gives each momentum its own record: hu reflect_odd across x walls,
// hv reflect_odd across y walls, even across the others.
enum GhostRule { FOEXTRAP = 0, REFLECT_EVEN = 1, REFLECT_ODD = 2 };
constexpr int BC_WALL = 0, BC_CLOSED_WALL = 2;

inline bool is_wall(int code) { return code == BC_WALL || code == BC_CLOSED_WALL; }
inline int scalar_rule(int code) { return is_wall(code) ? REFLECT_EVEN : FOEXTRAP; }
// hu at an x side (xdir) or a y side
inline int hu_rule(int code, bool xdir) {
    if (!is_wall(code)) return FOEXTRAP;
    return (code == BC_CLOSED_WALL && xdir) ? REFLECT_ODD : REFLECT_EVEN;
}
// hv at an x side (xdir) or a y side
inline int hv_rule(int code, bool xdir) {
    if (!is_wall(code)) return FOEXTRAP;
    if (code == BC_WALL) return xdir ? REFLECT_ODD : REFLECT_EVEN;
    return xdir ? REFLECT_EVEN : REFLECT_ODD;
}

// A plane of (nx + 2G) x (ny + 2G) values, x fastest, cell (i, j) of the valid
// box at offset (i + G) + (j + G) * (nx + 2G).
template <class R> struct Ext {
    int nx = 0, ny = 0, G = 0;
    std::vector<R> v;
    Ext() = default;
    Ext(int nx_, int ny_, int G_) : nx(nx_), ny(ny_), G(G_), v((size_t)(nx_ + 2 * G_) * (ny_ + 2 * G_), R(0)) {}
    R& at(int i, int j) { return v[(size_t)(i + G) + (size_t)(j + G) * (nx + 2 * G)]; }
    R at(int i, int j) const { return v[(size_t)(i + G) + (size_t)(j + G) * (nx + 2 * G)]; }
};

// Copy the valid plane q (pitch nx) into e and fill its ghosts with the
// per-side rules (rule[0]=x-lo, rule[1]=x-hi, rule[2]=y-lo, rule[3]=y-hi), in
// the order BCFill.H:159-181 uses: cells outside in one direction first, then
// corners (which read the already filled edge ghosts).
template <class R> void fill_ext(Ext<R>& e, const R* q, const int rule[4]) {
    const int nx = e.nx, ny = e.ny, G = e.G;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) e.at(i, j) = q[(size_t)i + (size_t)j * nx];
    auto xsrc = [&](int i, int j, int r, bool lo) -> R {
        if (r == FOEXTRAP) return e.at(lo ? 0 : nx - 1, j);
        int m = lo ? (-1 - i) : (2 * nx - 1 - i);
        R val = e.at(m, j);
        return r == REFLECT_ODD ? -val : val;
    };
    auto ysrc = [&](int i, int j, int r, bool lo) -> R {
        if (r == FOEXTRAP) return e.at(i, lo ? 0 : ny - 1);
        int m = lo ? (-1 - j) : (2 * ny - 1 - j);
        R val = e.at(i, m);
        return r == REFLECT_ODD ? -val : val;
    };
    for (int pass = 1; pass <= 2; ++pass) {
        for (int j = -G; j < ny + G; ++j)
            for (int i = -G; i < nx + G; ++i) {
                const bool ox = (i < 0 || i >= nx), oy = (j < 0 || j >= ny);
                if ((int)ox + (int)oy != pass) continue;
                if (ox) e.at(i, j) = xsrc(i, j, rule[i < 0 ? 0 : 1], i < 0);
                if (oy) e.at(i, j) = ysrc(i, j, rule[j < 0 ? 2 : 3], j < 0);
            }
    }
}

template <class R> struct Level {
    int nx, ny;
    R dx, dy;
    int bc_lo[2], bc_hi[2];
};

inline void rules_scalar(const int lo[2], const int hi[2], int out[4]) {
    out[0] = scalar_rule(lo[0]); out[1] = scalar_rule(hi[0]);
    out[2] = scalar_rule(lo[1]); out[3] = scalar_rule(hi[1]);
}
inline void rules_xmom(const int lo[2], const int hi[2], int out[4]) {
    out[0] = hu_rule(lo[0], true); out[1] = hu_rule(hi[0], true);
    out[2] = hu_rule(lo[1], false); out[3] = hu_rule(hi[1], false);
}
inline void rules_ymom(const int lo[2], const int hi[2], int out[4]) {
    out[0] = hv_rule(lo[0], true); out[1] = hv_rule(hi[0], true);
    out[2] = hv_rule(lo[1], false); out[3] = hv_rule(hi[1], false);
}
inline void rules_terrain(int out[4]) { out[0] = out[1] = out[2] = out[3] = FOEXTRAP; }

// Ghost-extended inputs of one advance: h rebuilt from eta, momenta, terrain.
template <class R> struct ExtState {
    Ext<R> h, hu, hv, z, n;
};

// Build the G-ghost extended state the reference's FillPatch calls produce for
// a single-level domain: eta = h + z on valid cells (AmrMeshState_AMR.cpp:218),
// eta/momenta/terrain ghosts by their BC rules, then h = max(0, eta - z) over
// the grown region (HydrostaticRoe.cpp:490-500; Roe.cpp:237-248).
template <class R>
void build_ext(const Level<R>& L, int G, const R* h, const R* hu, const R* hv, const R* z, const R* n,
               ExtState<R>& X) {
    const int nx = L.nx, ny = L.ny;
    const size_t N = (size_t)nx * ny;
    std::vector<R> eta(N);
    for (size_t c = 0; c < N; ++c) eta[c] = h[c] + z[c];
    int rs[4], rx[4], ry[4], rt[4];
    rules_scalar(L.bc_lo, L.bc_hi, rs);
    rules_xmom(L.bc_lo, L.bc_hi, rx);
    rules_ymom(L.bc_lo, L.bc_hi, ry);
    rules_terrain(rt);
    Ext<R> e(nx, ny, G);
    X.h = Ext<R>(nx, ny, G);
    X.hu = Ext<R>(nx, ny, G);
    X.hv = Ext<R>(nx, ny, G);
    X.z = Ext<R>(nx, ny, G);
    X.n = Ext<R>(nx, ny, G);
    fill_ext(e, eta.data(), rs);
    fill_ext(X.hu, hu, rx);
    fill_ext(X.hv, hv, ry);
    fill_ext(X.z, z, rt);
    fill_ext(X.n, n, rt);
    for (size_t c = 0; c < e.v.size(); ++c) X.h.v[c] = smax(R(0.0), e.v[c] - X.z.v[c]);
}

// One hydrostatic face (HydrostaticRoe.cpp:218-396).  (lm, l, r, rp) are the
// four cells along the face normal; FL/FR receive the two effective fluxes.
template <class R>
inline void hydrostatic_face(const ExtState<R>& X, int ilm, int jlm, int il, int jl, int ir, int jr, int irp,
                             int jrp, R nx, R ny, int mode, R FL[3], R FR[3]) {
    const R zL = X.z.at(il, jl);
    const R zR = X.z.at(ir, jr);
    if (std::abs(zL + 9999.0) < K<R>::tol10() || std::abs(zR + 9999.0) < K<R>::tol10()) {
        for (int c = 0; c < 3; ++c) { FL[c] = 0.0; FR[c] = 0.0; }
        return;
    }
    const R zf = smax(zL, zR);
    R etaLf, etaRf;
    {
        const R eLm = X.h.at(ilm, jlm) + X.z.at(ilm, jlm);
        const R eL = X.h.at(il, jl) + zL;
        const R eR = X.h.at(ir, jr) + zR;
        const R eRp = X.h.at(irp, jrp) + X.z.at(irp, jrp);
        const R sL = van_leer_slope(eLm, eL, eR, mode);
        const R sR = van_leer_slope(eL, eR, eRp, mode);
        etaLf = eL + 0.5 * sL;
        etaRf = eR - 0.5 * sR;
    }
    const R hLm = X.h.at(ilm, jlm), hL = X.h.at(il, jl), hR = X.h.at(ir, jr), hRp = X.h.at(irp, jrp);
    const R T12 = K<R>::tol12();
    R uLf, uRf, vLf, vRf;
    {
        const R a = (hLm > T12) ? X.hu.at(ilm, jlm) / hLm : 0.0;
        const R b = (hL > T12) ? X.hu.at(il, jl) / hL : 0.0;
        const R c = (hR > T12) ? X.hu.at(ir, jr) / hR : 0.0;
        const R d = (hRp > T12) ? X.hu.at(irp, jrp) / hRp : 0.0;
        uLf = b + 0.5 * van_leer_slope(a, b, c, mode);
        uRf = c - 0.5 * van_leer_slope(b, c, d, mode);
    }
    {
        const R a = (hLm > T12) ? X.hv.at(ilm, jlm) / hLm : 0.0;
        const R b = (hL > T12) ? X.hv.at(il, jl) / hL : 0.0;
        const R c = (hR > T12) ? X.hv.at(ir, jr) / hR : 0.0;
        const R d = (hRp > T12) ? X.hv.at(irp, jrp) / hRp : 0.0;
        vLf = b + 0.5 * van_leer_slope(a, b, c, mode);
        vRf = c - 0.5 * van_leer_slope(b, c, d, mode);
    }
    const R hLu = smax(R(0.0), etaLf - zL);
    const R hRu = smax(R(0.0), etaRf - zR);
    const R hLs = smax(R(0.0), etaLf - zf);
    const R hRs = smax(R(0.0), etaRf - zf);
    const R huL = (hLs > 0.0) ? hLs * uLf : 0.0;
    const R hvL = (hLs > 0.0) ? hLs * vLf : 0.0;
    const R huR = (hRs > 0.0) ? hRs * uRf : 0.0;
    const R hvR = (hRs > 0.0) ? hRs * vRf : 0.0;
    R f[3] = {R(0), R(0), R(0)};
    roe_hydrostatic(hLs, huL, hvL, hRs, huR, hvR, f, nx, ny);
    const R pL = 0.5 * K<R>::grav() * (hLu * hLu - hLs * hLs);
    const R pR = 0.5 * K<R>::grav() * (hRu * hRu - hRs * hRs);
    FL[0] = f[0];
    FL[1] = f[1] + pL * nx;
    FL[2] = f[2] + pL * ny;
    FR[0] = f[0];
    FR[1] = f[1] + pR * nx;
    FR[2] = f[2] + pR * ny;
}

// Face arrays, component-major: comp c of x-face (i, j) at c*(nx+1)*ny + i + j*(nx+1);
// y-face (i, j) at c*nx*(ny+1) + i + j*nx.
template <class R> struct Faces {
    int nx, ny;
    std::vector<R> xa, xb, xc, ya, yb, yc;  // hydrostatic: FL, FR (c unused); classic: F, S-, S+
    size_t xi(int i, int j, int c) const { return (size_t)c * (nx + 1) * ny + (size_t)i + (size_t)j * (nx + 1); }
    size_t yi(int i, int j, int c) const { return (size_t)c * nx * (ny + 1) + (size_t)i + (size_t)j * nx; }
};

#define HXO_PARFOR_ROWS _Pragma("omp parallel for schedule(static)")

// Hydrostatic advance of a single-box level by dt (HydrostaticRoe.cpp:400-606,
// reflux excluded).  (h, hu, hv) is the state at the start of the step, also
// the u_o of the update (the STORED depth, not the rebuilt one, :559).
template <class R>
void advance_hydrostatic(const Level<R>& L, const R* h, const R* hu, const R* hv, const R* z, const R* n, R dt,
                         R* ho, R* huo, R* hvo, int mode, Faces<R>* keep = nullptr) {
    const int nx = L.nx, ny = L.ny;
    ExtState<R> X;
    build_ext(L, 2, h, hu, hv, z, n, X);
    Faces<R> Fc;
    Fc.nx = nx; Fc.ny = ny;
    Fc.xa.assign((size_t)3 * (nx + 1) * ny, R(0));
    Fc.xb.assign((size_t)3 * (nx + 1) * ny, R(0));
    Fc.ya.assign((size_t)3 * nx * (ny + 1), R(0));
    Fc.yb.assign((size_t)3 * nx * (ny + 1), R(0));
    HXO_PARFOR_ROWS
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            R FL[3], FR[3];
            hydrostatic_face(X, i - 2, j, i - 1, j, i, j, i + 1, j, R(1.0), R(0.0), mode, FL, FR);
            for (int c = 0; c < 3; ++c) { Fc.xa[Fc.xi(i, j, c)] = FL[c]; Fc.xb[Fc.xi(i, j, c)] = FR[c]; }
        }
    HXO_PARFOR_ROWS
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i < nx; ++i) {
            R FL[3], FR[3];
            hydrostatic_face(X, i, j - 2, i, j - 1, i, j, i, j + 1, R(0.0), R(1.0), mode, FL, FR);
            for (int c = 0; c < 3; ++c) { Fc.ya[Fc.yi(i, j, c)] = FL[c]; Fc.yb[Fc.yi(i, j, c)] = FR[c]; }
        }
    const R g = K<R>::grav();
    HXO_PARFOR_ROWS
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t p = (size_t)i + (size_t)j * nx;
            const R uo[3] = {h[p], hu[p], hv[p]};
            R un[3];
            for (int c = 0; c < 3; ++c)
                un[c] = uo[c] - (dt / L.dx) * (Fc.xa[Fc.xi(i + 1, j, c)] - Fc.xb[Fc.xi(i, j, c)]) -
                        (dt / L.dy) * (Fc.ya[Fc.yi(i, j + 1, c)] - Fc.yb[Fc.yi(i, j, c)]);
            const R hh = un[0];
            if (hh >= K<R>::toldry()) {
                const R qx = un[1], qy = un[2];
                const R nsq = n[p] * n[p];
                const R inv_h = 1.0 / hh;
                const R u = qx * inv_h, v = qy * inv_h;
                const R modM = std::sqrt(u * u + v * v);
                if (nsq > K<R>::tol12() && modM > K<R>::tol12()) {
                    const R h43 = hh * std::cbrt(hh);
                    const R tt = dt * g * nsq * modM / h43;
                    const R ff = std::sqrt(1.0 + 4.0 * tt);
                    const R fac = 2.0 / (1.0 + ff);
                    un[1] = qx * fac;
                    un[2] = qy * fac;
                }
            } else {
                un[0] = smax(hh, R(0.0));
                un[1] = 0.0;
                un[2] = 0.0;
            }
            ho[p] = un[0]; huo[p] = un[1]; hvo[p] = un[2];
        }
    if (keep) *keep = std::move(Fc);
}

// Classic Roe advance of a single-box level by dt (Roe.cpp:250-434, reflux
// excluded).  h is rebuilt in place from eta = h + z on the grown box (one
// ghost) before the faces and the rebuilt depth is the u_o of the update.
template <class R>
void advance_classic(const Level<R>& L, const R* h, const R* hu, const R* hv, const R* z, const R* n, R dt, R* ho,
                     R* huo, R* hvo, Faces<R>* keep = nullptr) {
    const int nx = L.nx, ny = L.ny;
    ExtState<R> X;
    build_ext(L, 1, h, hu, hv, z, n, X);
    Faces<R> Fc;
    Fc.nx = nx; Fc.ny = ny;
    Fc.xa.assign((size_t)3 * (nx + 1) * ny, R(0));
    Fc.xb.assign((size_t)3 * (nx + 1) * ny, R(0));
    Fc.xc.assign((size_t)3 * (nx + 1) * ny, R(0));
    Fc.ya.assign((size_t)3 * nx * (ny + 1), R(0));
    Fc.yb.assign((size_t)3 * nx * (ny + 1), R(0));
    Fc.yc.assign((size_t)3 * nx * (ny + 1), R(0));
    HXO_PARFOR_ROWS
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            R F[3], Sm[3], Sp[3];
            roe_classic(X.h.at(i - 1, j), X.hu.at(i - 1, j), X.hv.at(i - 1, j), X.z.at(i - 1, j), X.n.at(i - 1, j),
                        X.h.at(i, j), X.hu.at(i, j), X.hv.at(i, j), X.z.at(i, j), X.n.at(i, j), F, Sm, Sp, dt, L.dx,
                        R(1.0), R(0.0));
            for (int c = 0; c < 3; ++c) {
                Fc.xa[Fc.xi(i, j, c)] = F[c]; Fc.xb[Fc.xi(i, j, c)] = Sm[c]; Fc.xc[Fc.xi(i, j, c)] = Sp[c];
            }
        }
    HXO_PARFOR_ROWS
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i < nx; ++i) {
            R F[3], Sm[3], Sp[3];
            roe_classic(X.h.at(i, j - 1), X.hu.at(i, j - 1), X.hv.at(i, j - 1), X.z.at(i, j - 1), X.n.at(i, j - 1),
                        X.h.at(i, j), X.hu.at(i, j), X.hv.at(i, j), X.z.at(i, j), X.n.at(i, j), F, Sm, Sp, dt, L.dy,
                        R(0.0), R(1.0));
            for (int c = 0; c < 3; ++c) {
                Fc.ya[Fc.yi(i, j, c)] = F[c]; Fc.yb[Fc.yi(i, j, c)] = Sm[c]; Fc.yc[Fc.yi(i, j, c)] = Sp[c];
            }
        }
    HXO_PARFOR_ROWS
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t p = (size_t)i + (size_t)j * nx;
            const R uo[3] = {X.h.at(i, j), hu[p], hv[p]};
            R un[3];
            for (int c = 0; c < 3; ++c)
                un[c] = uo[c] - (dt / L.dx) * (Fc.xa[Fc.xi(i + 1, j, c)] - Fc.xa[Fc.xi(i, j, c)]) -
                        (dt / L.dy) * (Fc.ya[Fc.yi(i, j + 1, c)] - Fc.ya[Fc.yi(i, j, c)]) -
                        (dt / L.dx) * (Fc.xc[Fc.xi(i + 1, j, c)] + Fc.xb[Fc.xi(i, j, c)]) -
                        (dt / L.dy) * (Fc.yc[Fc.yi(i, j + 1, c)] + Fc.yb[Fc.yi(i, j, c)]);
            ho[p] = un[0]; huo[p] = un[1]; hvo[p] = un[2];
        }
    if (keep) *keep = std::move(Fc);
}

// Per-cell CFL bound, HydrostaticRoe.cpp:37-62 and Roe.cpp:38-73 (identical
// arithmetic; both depth thresholds are 1e-12).
template <class R>
inline void dt_cell(R h, R hu, R hv, R z, R dx, R dy, R& dtc, R& mu) {
    if (std::abs(z - (-9999.0)) < K<R>::tol10()) { dtc = 1.e30; mu = 0.0; return; }
    dtc = 1.e6;
    mu = 0.0;
    if (h > K<R>::tol12()) {
        R u = hu / h;
        R v = hv / h;
        R c = std::sqrt(K<R>::grav() * h);
        const R sx = std::abs(u) + c;
        const R sy = std::abs(v) + c;
        dtc = 1.0 / (sx / dx + sy / dy);
        mu = smax(std::abs(u), std::abs(v));
    }
}

// Minimum of the per-cell bound and maximum of max(|u|,|v|) over the valid
// cells.  Both reductions are exact, so the result is order-independent.
template <class R>
void compute_dt(const Level<R>& L, const R* h, const R* hu, const R* hv, const R* z, R& dtmin, R& maxvel) {
    const size_t N = (size_t)L.nx * L.ny;
    R mn = std::numeric_limits<R>::max();
    R mx = std::numeric_limits<R>::lowest();
#pragma omp parallel for reduction(min : mn) reduction(max : mx) schedule(static)
    for (long long p = 0; p < (long long)N; ++p) {
        R dtc, mu;
        dt_cell(h[p], hu[p], hv[p], z[p], L.dx, L.dy, dtc, mu);
        mn = std::min(mn, dtc);
        mx = std::max(mx, mu);
    }
    dtmin = mn;
    maxvel = mx;
}

// Array4-like strided view used by the tag and restriction restatements:
// element (i, j, c) at p[(i - lo0) + (j - lo1) * js + c * ns].
template <class R> struct View {
    R* p;
    long long js, ns;
    int lo0, lo1;
    R& operator()(int i, int j, int c) const { return p[(i - lo0) + (long long)(j - lo1) * js + c * ns]; }
};

// Gradient tagging of the valid box [vlo, vhi] (HydrostaticRoe.cpp:109-169 for
// variant 1, Roe.cpp:121-179 for variant 0).  U and T must cover one ghost.
// Only tagged cells are written, with set_value; the rest are left untouched.
template <class R>
void tag_cells(int variant, View<const R> U, View<const R> T, View<signed char> tags, int vlo0, int vlo1, int vhi0,
               int vhi1, R dx, R dy, R time, R h_th, R u_th, R z_th, signed char set_value) {
    for (int j = vlo1; j <= vhi1; ++j)
        for (int i = vlo0; i <= vhi0; ++i) {
            if (variant == 1) {
                const R nod = K<R>::tol10();
                if (std::abs(T(i + 1, j, 0) + 9999.0) < nod || std::abs(T(i - 1, j, 0) + 9999.0) < nod ||
                    std::abs(T(i, j + 1, 0) + 9999.0) < nod || std::abs(T(i, j - 1, 0) + 9999.0) < nod)
                    continue;
            } else {
                if (T(i + 1, j, 0) == -9999.0 || T(i - 1, j, 0) == -9999.0 || T(i, j + 1, 0) == -9999.0 ||
                    T(i, j - 1, 0) == -9999.0)
                    continue;
            }
            bool tag = false;
            R dhdx = (U(i + 1, j, 0) - U(i - 1, j, 0)) / (2.0 * dx);
            R dhdy = (U(i, j + 1, 0) - U(i, j - 1, 0)) / (2.0 * dy);
            if (std::sqrt(dhdx * dhdx + dhdy * dhdy) > h_th) tag = true;
            auto zgrad = [&]() {
                R dzdx = (T(i + 1, j, 0) - T(i - 1, j, 0)) / (2.0 * dx);
                R dzdy = (T(i, j + 1, 0) - T(i, j - 1, 0)) / (2.0 * dy);
                return std::sqrt(dzdx * dzdx + dzdy * dzdy) > z_th;
            };
            auto umag = [&](int ii, int jj) -> R {
                R hh = U(ii, jj, 0), qx = U(ii, jj, 1), qy = U(ii, jj, 2);
                if (hh < R(1.0e-6)) return R(0.0);
                R u = qx / hh, v = qy / hh;
                return std::sqrt(u * u + v * v);
            };
            auto ugrad = [&]() {
                R uE = umag(i + 1, j), uW = umag(i - 1, j), uN = umag(i, j + 1), uS = umag(i, j - 1);
                R dudx = (uE - uW) / (2.0 * dx);
                R dudy = (uN - uS) / (2.0 * dy);
                return std::sqrt(dudx * dudx + dudy * dudy) > u_th;
            };
            if (variant == 1) {
                if (!tag) {
                    if (ugrad()) tag = true;
                    if (time <= 1.0e-8 && zgrad()) tag = true;
                }
            } else {
                if (time <= 1.0e-8 && zgrad()) tag = true;
                if (!tag && ugrad()) tag = true;
            }
            if (tag) tags(i, j, 0) = set_value;
        }
}

// NODATA-aware volume-weighted restriction of one coarse box [clo, chi]
// (MaskedAverageDown.H:64-104), components 0..ncomp-1 of fine into crse.
// fv is the (constant, Cartesian) fine-cell volume.
template <class R>
void masked_average_down(View<const R> fine, View<R> crse, int clo0, int clo1, int chi0, int chi1, int ncomp, int rx,
                         int ry, R fv, R nodata) {
    for (int n = 0; n < ncomp; ++n)
        for (int j = clo1; j <= chi1; ++j)
            for (int i = clo0; i <= chi0; ++i) {
                R cd = 0.0, cv = 0.0;
                int nvalid = 0;
                const int total = rx * ry;
                for (int jr = 0; jr < ry; ++jr)
                    for (int ir = 0; ir < rx; ++ir) {
                        R val = fine(i * rx + ir, j * ry + jr, n);
                        if (!std::isnan(val) && std::abs(val - nodata) > 1e-3) {
                            ++nvalid;
                            cv += fv;
                            cd += val * fv;
                        }
                    }
                if (nvalid * 2 >= total && cv > 0.0) crse(i, j, n) = cd / cv;
                else crse(i, j, n) = nodata;
            }
}

// Conservative restriction of the state, amrex::average_down as
// AmrMeshState::AverageDownTo calls it (src/state/AmrMeshState_AMR.cpp:838-844)
// on a Cartesian geometry.  The kernel is AMReX's amrex_avgdown
// (AMReX_MultiFabUtil_2D_C.H; AMReX is an un-vendored submodule with no pinned
// version): the rx*ry fine values are summed, rows outer and columns inner,
// starting from 0, and the sum is multiplied by volfrac = 1/(rx*ry).
template <class R>
void average_down(View<const R> fine, View<R> crse, int clo0, int clo1, int chi0, int chi1, int scomp, int ccomp,
                  int ncomp, int rx, int ry) {
    const R volfrac = R(1.0) / R(rx * ry);
    for (int n = 0; n < ncomp; ++n)
        for (int j = clo1; j <= chi1; ++j)
            for (int i = clo0; i <= chi0; ++i) {
                R c = R(0);
                for (int jr = 0; jr < ry; ++jr)
                    for (int ir = 0; ir < rx; ++ir) c += fine(i * rx + ir, j * ry + jr, scomp + n);
                crse(i, j, ccomp + n) = volfrac * c;
            }
}

// Per-box reduction of AmrMeshState::ComputeMassDiagnostics,
// src/state/AmrMeshState_Utils.cpp:267-298, over the valid cells of one box:
// out = {mass, x-momentum, y-momentum, kinetic energy, min h}.  A cell counts
// when its roughness (terrain comp 1) is not -9999 and h > 0 (:273, :281); its
// terms keep the reference's expressions and types (:282-286; the 0.5 literal
// is double).  The reference's ReduceOps fixes no summation order; here the
// terms are summed in double, row by row.
template <class R>
void mass_diagnostics(int nx, int ny, long long pitch, const R* h, const R* hu, const R* hv, const R* n, R dx, R dy,
                      double out[5]) {
    const R dA = dx * dy;                // :239
    const R nodata_val = R(-9999.0);     // :217
    double m = 0.0, px = 0.0, py = 0.0, ke = 0.0;
    R min_h = std::numeric_limits<R>::max();
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const long long o = (long long)i + (long long)j * pitch;
            const R hh = h[o], a = hu[o], c = hv[o];
            const int is_nodata = (n[o] == nodata_val) ? 1 : 0;
            if (is_nodata == 0 && hh > 0.0) {
                const R s_mass = hh * dA;
                const R s_mx = a * dA;
                const R s_my = c * dA;
                const R s_ke = 0.5 * (a * a + c * c) / hh * dA;
                m += s_mass;
                px += s_mx;
                py += s_my;
                ke += s_ke;
                min_h = smin(min_h, hh);
            }
        }
    out[0] = m; out[1] = px; out[2] = py; out[3] = ke; out[4] = (double)min_h;
}

// eta = h + z, the kernel of DeriveEtaFrom, src/state/AmrMeshState_AMR.cpp:217-219.
template <class R> void derive_eta(long long count, const R* h, const R* z, R* eta) {
    for (long long k = 0; k < count; ++k) eta[k] = h[k] + z[k];
}

}  // namespace hxo
