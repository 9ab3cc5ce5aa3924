// Hand-written adjoint (reverse mode) of the hydrostatic-Roe time loop.
//
// The loss is J = sum over steps n = 1..N and gauge cells g of
// (h^n_g - href^n_g)^2.  Its gradient with respect to the initial state
// (h, hu, hv) and the bed z is obtained by one forward sweep (states kept in
// HBM, all of them or every L-th with the segments recomputed) and one reverse
// sweep of three kernels per step:
//
//   A  post-map reverse: lambda_lin = J_post^T lambda^{n+1}, where post is the
//      Manning factor and the dry clamp (src/solvers/HydrostaticRoe.cpp:566-603),
//      skipped for steps where no cell took either branch;
//   B  face reverse: per 32x16 tile, the forward values with a 3-cell halo are
//      recomputed, every face flux (HydrostaticRoe.cpp:218-396 with the
//      homogeneous Roe flux of include/solvers/kernels/HydrostaticRoe.H:44-159)
//      is differentiated in reverse taking the forward's branches (dry clamps,
//      entropy fixes, hydrostatic caps, NODATA walls), the van Leer slopes are
//      reversed, per-cell adjoints are gathered in a fixed order (no atomics,
//      reproducible), boundary-ghost adjoints are folded into the cells their
//      values came from, and the h rebuild is reversed;
//   C  one block: the dt of step n is cfl / max rate(U^n), so its adjoint
//      flows into the cell that set the CFL bound; then the gauge misfit of
//      state n is injected.
#include <cstdio>
#include <functional>
#include <vector>

#include "hx_kernels.cuh"

namespace hx {
void note_launches(int n);
int set_error(int code, const char* msg);
// Instantiated in hx_exact.cu (--fmad=false) and hx_fast.cu: never here, so the
// exact form's forward sweep stays bit-identical to the exact level advance.
extern template cudaError_t launch_adj_forward<false>(const LevelSrc<double>&, const Cells3<double>&,
                                                      const Plane<double>&, const Cells3W<double>&, const IBox&,
                                                      const StepCtl<double>&, const double*, unsigned*,
                                                      const AdjRecord&, cudaStream_t);
extern template cudaError_t launch_adj_forward<true>(const LevelSrc<double>&, const Cells3<double>&,
                                                     const Plane<double>&, const Cells3W<double>&, const IBox&,
                                                     const StepCtl<double>&, const double*, unsigned*,
                                                     const AdjRecord&, cudaStream_t);
extern template cudaError_t launch_adj_forward_rec<true>(const LevelSrc<double>&, const Cells3<double>&,
                                                         const Plane<double>&, const Cells3W<double>&, const IBox&,
                                                         double, double, const double*, unsigned*, const FaceRec&,
                                                         cudaStream_t);
extern template cudaError_t launch_adj_forward_linear<false>(const LevelSrc<double>&, const Cells3<double>&,
                                                             const Plane<double>&, const Cells3W<double>&,
                                                             const IBox&, double, double, const double*, cudaStream_t);
extern template cudaError_t launch_adj_forward_linear<true>(const LevelSrc<double>&, const Cells3<double>&,
                                                            const Plane<double>&, const Cells3W<double>&, const IBox&,
                                                            double, double, const double*, cudaStream_t);
extern template cudaError_t launch_dt_reduce<double, false>(const Cells3<double>&, const Plane<double>&, const IBox&,
                                                            double, double, DtAccum*, cudaStream_t);
extern template cudaError_t launch_dt_reduce<double, true>(const Cells3<double>&, const Plane<double>&, const IBox&,
                                                           double, double, DtAccum*, cudaStream_t);
}  // namespace hx

using namespace hx;

namespace {

constexpr double G = 9.81, HG = 0.5 * 9.81, TD = 1e-6, T12 = 1e-12;
constexpr int ATX = 32, ATY = 16, ANT = 512;
constexpr int H3 = 3;  // forward halo of the reverse tile

// sign with sgn(+-0) = 0, decided on the integer pipe
__device__ __forceinline__ double sgn(double x) { return pos_i(x) ? 1.0 : (neg_i(x) ? -1.0 : 0.0); }
// sgn(x) a, all on the integer pipe (a sign flip or a zero instead of a multiply)
__device__ __forceinline__ double sgn_mul(double x, double a) {
    const double na = __longlong_as_double(__double_as_longlong(a) ^ (long long)0x8000000000000000ull);
    return pos_i(x) ? a : (neg_i(x) ? na : 0.0);
}

// ---------------------------------------------------------------------------
// Reverse of the homogeneous Roe flux in the face-normal frame.  (hi, ui, vi)
// and (hj, uj, vj) are the face depths and the normal / tangential face
// velocities; b0..b2 the adjoints of the normal-frame flux.  Adjoints of the
// inputs are added to g*.
// ---------------------------------------------------------------------------
__device__ void roe_rev(double hi, double ui, double vi, double hj, double uj, double vj, double b0, double b1,
                        double b2, double& ghi, double& gui, double& gvi, double& ghj, double& guj, double& gvj) {
    const bool wi = hi >= TD, wj = hj >= TD;
    const double Hi = wi ? hi : 0.0, Hj = wj ? hj : 0.0;
    const double Ui = wi ? ui : 0.0, Vi = wi ? vi : 0.0, Uj = wj ? uj : 0.0, Vj = wj ? vj : 0.0;
    const double si = sqrt(Hi), sj = sqrt(Hj);
    const double hh = 0.5 * (Hi + Hj);
    const bool hmb = hh > TD;
    const double hm = hmb ? hh : TD;
    const double cm = sqrt(G * hm);
    const double sden = si + sj + T12;
    const double um = (Ui * si + Uj * sj) / sden;
    const double vm = (Vi * si + Vj * sj) / sden;
    const double l0a = um - cm, l2a = um + cm;
    const double ci = sqrt(G * Hi), cj = sqrt(G * Hj);
    const double e0i = Ui - ci, e0j = Uj - cj;
    const bool fix0 = e0i < 0.0 && e0j > 0.0;
    const double l0 = fix0 ? e0i * (e0j - l0a) / (e0j - e0i) : l0a;
    const double e2i = Ui + ci, e2j = Uj + cj;
    const bool fix2 = e2i < 0.0 && e2j > 0.0;
    const double l2 = fix2 ? e2j * (l2a - e2i) / (e2j - e2i) : l2a;
    const double l1 = um;
    const double den = 2.0 * cm + T12;
    const double dh = Hj - Hi;
    const double dhu = Hj * Uj - Hi * Ui;
    const double dhv = Hj * Vj - Hi * Vi;
    const double a0 = (l2 * dh - dhu) / den, a1 = (dhv - vm * dh) / cm, a2 = (dhu - l0 * dh) / den;
    const double w0 = 0.5 * fabs(l0) * a0, w1 = 0.5 * fabs(l1) * a1, w2 = 0.5 * fabs(l2) * a2;

    double gHi = 0, gHj = 0, gUi = 0, gUj = 0, gVi = 0, gVj = 0;
    // F0 = (Hi Ui + Hj Uj)/2 - w0 - w2
    gHi += 0.5 * b0 * Ui; gUi += 0.5 * b0 * Hi; gHj += 0.5 * b0 * Uj; gUj += 0.5 * b0 * Hj;
    // F1 = (Hi Ui^2 + HG Hi^2 + Hj Uj^2 + HG Hj^2)/2 - w0 l0 - w2 l2
    gHi += 0.5 * b1 * (Ui * Ui + 2.0 * HG * Hi); gUi += b1 * Hi * Ui;
    gHj += 0.5 * b1 * (Uj * Uj + 2.0 * HG * Hj); gUj += b1 * Hj * Uj;
    // F2 = (Hi Ui Vi + Hj Uj Vj)/2 - w0 vm - w1 cm - w2 vm
    gHi += 0.5 * b2 * Ui * Vi; gUi += 0.5 * b2 * Hi * Vi; gVi += 0.5 * b2 * Hi * Ui;
    gHj += 0.5 * b2 * Uj * Vj; gUj += 0.5 * b2 * Hj * Vj; gVj += 0.5 * b2 * Hj * Uj;
    const double gw0 = -b0 - b1 * l0 - b2 * vm;
    const double gw1 = -b2 * cm;
    const double gw2 = -b0 - b1 * l2 - b2 * vm;
    double gl0 = -b1 * w0, gl2 = -b1 * w2, gvm = -b2 * (w0 + w2), gcm = -b2 * w1;
    const double ga0 = gw0 * 0.5 * fabs(l0);
    gl0 += gw0 * 0.5 * sgn(l0) * a0;
    const double ga1 = gw1 * 0.5 * fabs(l1);
    const double gl1 = gw1 * 0.5 * sgn(l1) * a1;
    const double ga2 = gw2 * 0.5 * fabs(l2);
    gl2 += gw2 * 0.5 * sgn(l2) * a2;
    // wave strengths
    gl2 += ga0 * dh / den;
    double gdh = ga0 * l2 / den, gdhu = -ga0 / den, gden = -ga0 * a0 / den;
    const double gdhv = ga1 / cm;
    gvm += -ga1 * dh / cm;
    gdh += -ga1 * vm / cm;
    gcm += -ga1 * a1 / cm;
    gdhu += ga2 / den;
    gl0 += -ga2 * dh / den;
    gdh += -ga2 * l0 / den;
    gden += -ga2 * a2 / den;
    gcm += 2.0 * gden;
    gHj += gdh; gHi -= gdh;
    gHj += gdhu * Uj; gUj += gdhu * Hj; gHi -= gdhu * Ui; gUi -= gdhu * Hi;
    gHj += gdhv * Vj; gVj += gdhv * Hj; gHi -= gdhv * Vi; gVi -= gdhv * Hi;
    // eigenvalues and the sonic fixes (the forward's branches)
    double gum = gl1, gci = 0.0, gcj = 0.0;
    if (fix2) {
        const double D = e2j - e2i;
        const double gl2a = gl2 * e2j / D;
        const double ge2i = gl2 * e2j * (l2a - e2j) / (D * D);
        const double ge2j = -gl2 * (l2a - e2i) * e2i / (D * D);
        gUi += ge2i; gci += ge2i; gUj += ge2j; gcj += ge2j;
        gum += gl2a; gcm += gl2a;
    } else {
        gum += gl2; gcm += gl2;
    }
    if (fix0) {
        const double D = e0j - e0i;
        const double gl0a = -gl0 * e0i / D;
        const double ge0i = gl0 * (e0j - l0a) * e0j / (D * D);
        const double ge0j = gl0 * e0i * (l0a - e0i) / (D * D);
        gUi += ge0i; gci -= ge0i; gUj += ge0j; gcj -= ge0j;
        gum += gl0a; gcm -= gl0a;
    } else {
        gum += gl0; gcm -= gl0;
    }
    if (ci > 0.0) gHi += gci * G / (2.0 * ci);
    if (cj > 0.0) gHj += gcj * G / (2.0 * cj);
    // Roe averages
    const double gnu = gum / sden, gnv = gvm / sden, gsden = -(gum * um + gvm * vm) / sden;
    gUi += gnu * si; gUj += gnu * sj; gVi += gnv * si; gVj += gnv * sj;
    const double gsi = gnu * Ui + gnv * Vi + gsden, gsj = gnu * Uj + gnv * Vj + gsden;
    const double ghm = gcm * G / (2.0 * cm);
    if (hmb) { gHi += 0.5 * ghm; gHj += 0.5 * ghm; }
    if (si > 0.0) gHi += gsi / (2.0 * si);
    if (sj > 0.0) gHj += gsj / (2.0 * sj);
    if (wi) { ghi += gHi; gui += gUi; gvi += gVi; }
    if (wj) { ghj += gHj; guj += gUj; gvj += gVj; }
}

// Fast form of roe_rev, in two parts.  The forward section gives the
// quantities the reverse needs: either recomputed (roe_fwd_fast, taking the
// branches roe_hydrostatic_fast takes, every division of the reverse turned
// into a product with one of five reciprocals 1/sden, 1/den, 1/cm, 1/si, 1/sj
// from a single rcp_nr of their product), or read from the record the segment
// recompute wrote for the face (roe_fwd_rec: square roots, Roe averages,
// entropy-fixed speeds and wave strengths as the forward step computed them;
// only 1/si and 1/sj are formed).  roe_rev_core then runs the reverse.
struct RoeFwd {
    double Hi, Hj, Ui, Uj, Vi, Vj, si, sj, hrsi, hrsj, cm, rs, rden, rcm, um, vm, l0, l2, dh;  // hrs = 1/(2 s)
    double a0h, a1h, a2h, w0, w1, w2, hrden, hrcm;  // half wave strengths, w = |l| ah, halves of 1/den, 1/cm
    double e0i, e0j, e2i, e2j, l0a, l2a, rD0, rD2;
    bool wi, wj, hmb, fix0, fix2;
};


__device__ __forceinline__ void roe_fwd_fast(double hi, double ui, double vi, double hj, double uj, double vj,
                                             RoeFwd& F) {
    using C = Cst<double>;
    const bool wi = ge_bits(hi, C::toldry_bits), wj = ge_bits(hj, C::toldry_bits);
    F.wi = wi; F.wj = wj;
    const double Hi = wi ? hi : 0.0, Hj = wj ? hj : 0.0;
    const double Ui = wi ? ui : 0.0, Vi = wi ? vi : 0.0, Uj = wj ? uj : 0.0, Vj = wj ? vj : 0.0;
    F.Hi = Hi; F.Hj = Hj; F.Ui = Ui; F.Uj = Uj; F.Vi = Vi; F.Vj = Vj;
    // the forward's own square roots (fast_sqrt, fast_sqrt_hrsqrt of g hm = (g/2)(Hi + Hj)), bit for bit
    const double si = fast_sqrt(Hi), sj = fast_sqrt(Hj);
    F.si = si; F.sj = sj;
    const double hh = 0.5 * (Hi + Hj);
    F.hmb = gt_bits(hh, C::toldry_bits);
    const double hm = F.hmb ? hh : TD;
    double hrcm_unused;
    const double cm = fast_sqrt_hrsqrt(G * hm, hrcm_unused);
    F.cm = cm;
    const double den = 2.0 * cm + T12;
    const double sden = si + sj + T12;
    const double cd = cm * den, S3 = sden * cd;
    double q3;
    F.hrsi = 0.0; F.hrsj = 0.0;
    if (wi && wj) {
        const double pij = si * sj;
        const double q = rcp_nr(S3 * pij);
        q3 = pij * q;
        F.hrsi = (sj * (0.5 * S3)) * q;
        F.hrsj = (si * (0.5 * S3)) * q;
    } else {
        q3 = rcp_nr(S3);
        if (wi) F.hrsi = rcp_nr(si + si);
        if (wj) F.hrsj = rcp_nr(sj + sj);
    }
    F.rs = cd * q3; F.rden = (sden * cm) * q3; F.rcm = (sden * den) * q3;
    const double um = (Ui * si + Uj * sj) * F.rs;
    const double vm = (Vi * si + Vj * sj) * F.rs;
    F.um = um; F.vm = vm;
    F.l0a = um - cm; F.l2a = um + cm;
    const double ci = C::sqrt_g * si, cj = C::sqrt_g * sj;
    F.e0i = Ui - ci; F.e0j = Uj - cj;
    F.fix0 = neg_i(F.e0i) && pos_i(F.e0j);
    F.e2i = Ui + ci; F.e2j = Uj + cj;
    F.fix2 = neg_i(F.e2i) && pos_i(F.e2j);
    F.l0 = F.l0a; F.l2 = F.l2a; F.rD0 = 0.0; F.rD2 = 0.0;
    if (F.fix0) { F.rD0 = rcp_nr(F.e0j - F.e0i); F.l0 = F.e0i * (F.e0j - F.l0a) * F.rD0; }
    if (F.fix2) { F.rD2 = rcp_nr(F.e2j - F.e2i); F.l2 = F.e2j * (F.l2a - F.e2i) * F.rD2; }
    const double dh = Hj - Hi;
    F.dh = dh;
    const double dhu = Hj * Uj - Hi * Ui;
    const double dhv = Hj * Vj - Hi * Vi;
    F.a0h = 0.5 * ((F.l2 * dh - dhu) * F.rden);
    F.a1h = 0.5 * ((dhv - vm * dh) * F.rcm);
    F.a2h = 0.5 * ((dhu - F.l0 * dh) * F.rden);
    F.w0 = fabs(F.l0) * F.a0h; F.w1 = fabs(um) * F.a1h; F.w2 = fabs(F.l2) * F.a2h;
    F.hrden = 0.5 * F.rden; F.hrcm = 0.5 * F.rcm;
}

__device__ __forceinline__ void roe_fwd_rec(double hi, double ui, double vi, double hj, double uj, double vj,
                                            const RoeRecVals& R, RoeFwd& F) {
    using C = Cst<double>;
    const bool wi = (R.fl & RR_WI) != 0, wj = (R.fl & RR_WJ) != 0;
    F.wi = wi; F.wj = wj;
    const double Hi = wi ? hi : 0.0, Hj = wj ? hj : 0.0;
    const double Ui = wi ? ui : 0.0, Vi = wi ? vi : 0.0, Uj = wj ? uj : 0.0, Vj = wj ? vj : 0.0;
    F.Hi = Hi; F.Hj = Hj; F.Ui = Ui; F.Uj = Uj; F.Vi = Vi; F.Vj = Vj;
    const double si = R.si, sj = R.sj, cm = R.cm;
    F.si = si; F.sj = sj; F.cm = cm;
    F.hmb = (R.fl & RR_HM) != 0;
    F.rs = R.rs; F.hrden = R.hrden; F.hrcm = R.hrcm;  // as the forward computed them
    F.hrsi = 0.0; F.hrsj = 0.0;
    if (wi && wj) {
        const double r = rcp_nr((si + si) * sj);
        F.hrsi = sj * r;
        F.hrsj = si * r;
    } else {
        if (wi) F.hrsi = rcp_nr(si + si);
        if (wj) F.hrsj = rcp_nr(sj + sj);
    }
    F.um = R.um; F.vm = R.vm; F.l0 = R.l0; F.l2 = R.l2;
    F.fix0 = (R.fl & RR_FIX0) != 0;
    F.fix2 = (R.fl & RR_FIX2) != 0;
    if (F.fix0 | F.fix2) {  // the sonic-fix derivatives need the one-sided speeds
        const double ci = C::sqrt_g * si, cj = C::sqrt_g * sj;
        F.l0a = R.um - cm; F.l2a = R.um + cm;
        F.e0i = Ui - ci; F.e0j = Uj - cj; F.e2i = Ui + ci; F.e2j = Uj + cj;
        F.rD0 = F.fix0 ? rcp_nr(F.e0j - F.e0i) : 0.0;
        F.rD2 = F.fix2 ? rcp_nr(F.e2j - F.e2i) : 0.0;
    }
    F.dh = Hj - Hi;
    F.a0h = R.a0h; F.a1h = R.a1h; F.a2h = R.a2h;
    F.w0 = fabs(R.l0) * R.a0h; F.w1 = fabs(R.um) * R.a1h; F.w2 = fabs(R.l2) * R.a2h;
}

__device__ __forceinline__ void roe_rev_core(const RoeFwd& F, double b0, double b1, double b2, double& ghi,
                                             double& gui, double& gvi, double& ghj, double& guj, double& gvj) {
    using C = Cst<double>;
    const double Hi = F.Hi, Hj = F.Hj, Ui = F.Ui, Uj = F.Uj, Vi = F.Vi, Vj = F.Vj;
    const double l0 = F.l0, l1 = F.um, l2 = F.l2, vm = F.vm, cm = F.cm, dh = F.dh;
    const double w0 = F.w0, w1 = F.w1, w2 = F.w2;
    // central flux (F(U_i) + F(U_j)) / 2 with F = (H U, H U^2 + HG H^2, H U V):
    // dF/dH = (U, U^2 + G H, U V), dF/dU = (H, 2 H U, H V), dF/dV = (0, 0, H U)
    const double hb0 = 0.5 * b0, hb1 = 0.5 * b1, hb2 = 0.5 * b2;
    double gHi = fma(hb0, Ui, fma(hb1, fma(Ui, Ui, G * Hi), hb2 * Ui * Vi));
    double gHj = fma(hb0, Uj, fma(hb1, fma(Uj, Uj, G * Hj), hb2 * Uj * Vj));
    double gUi = Hi * fma(hb2, Vi, fma(b1, Ui, hb0));
    double gUj = Hj * fma(hb2, Vj, fma(b1, Uj, hb0));
    double gVi = hb2 * Hi * Ui, gVj = hb2 * Hj * Uj;
    const double gw0 = -b0 - b1 * l0 - b2 * vm;
    const double gw1 = -b2 * cm;
    const double gw2 = -b0 - b1 * l2 - b2 * vm;
    // w_k = |l_k| ah_k, ah_k = alpha_k / 2
    double gl0 = fma(gw0, sgn_mul(l0, F.a0h), -b1 * w0);
    double gl2 = fma(gw2, sgn_mul(l2, F.a2h), -b1 * w2);
    double gvm = -b2 * (w0 + w2), gcm = -b2 * w1;
    const double gl1 = gw1 * sgn_mul(l1, F.a1h);
    const double ga0 = gw0 * fabs(l0) * F.hrden;  // d/d alpha0, already divided by den
    const double ga1 = gw1 * fabs(l1) * F.hrcm;   // d/d alpha1, already divided by cm
    const double ga2 = gw2 * fabs(l2) * F.hrden;
    gl2 += ga0 * dh;
    double gdh = ga0 * l2 - ga1 * vm - ga2 * l0;
    double gdhu = ga2 - ga0;
    const double gdhv = ga1;
    gvm -= ga1 * dh;
    gcm -= 2.0 * fma(ga1, F.a1h, 2.0 * fma(ga0, F.a0h, ga2 * F.a2h));  // ga1 a1 + 2 (ga0 a0 + ga2 a2)
    gl0 -= ga2 * dh;
    gHj += gdh + gdhu * Uj + gdhv * Vj;
    gHi -= gdh + gdhu * Ui + gdhv * Vi;
    gUj += gdhu * Hj; gUi -= gdhu * Hi;
    gVj += gdhv * Hj; gVi -= gdhv * Hi;
    double gum = gl1, gci = 0.0, gcj = 0.0;
    if (F.fix2) {
        const double t = gl2 * F.rD2;
        const double gl2a = t * F.e2j;
        const double ge2i = t * F.e2j * (F.l2a - F.e2j) * F.rD2;
        const double ge2j = -t * (F.l2a - F.e2i) * F.e2i * F.rD2;
        gUi += ge2i; gci += ge2i; gUj += ge2j; gcj += ge2j;
        gum += gl2a; gcm += gl2a;
    } else {
        gum += gl2; gcm += gl2;
    }
    if (F.fix0) {
        const double t = gl0 * F.rD0;
        const double gl0a = -t * F.e0i;
        const double ge0i = t * (F.e0j - F.l0a) * F.e0j * F.rD0;
        const double ge0j = t * F.e0i * (F.l0a - F.e0i) * F.rD0;
        gUi += ge0i; gci -= ge0i; gUj += ge0j; gcj -= ge0j;
        gum += gl0a; gcm -= gl0a;
    } else {
        gum += gl0; gcm -= gl0;
    }
    const double gnu = gum * F.rs, gnv = gvm * F.rs, gsden = -(gnu * F.um + gnv * vm);
    gUi += gnu * F.si; gUj += gnu * F.sj; gVi += gnv * F.si; gVj += gnv * F.sj;
    // s = sqrt(H) and c = sqrt(g) s: d/dH = (gs + sqrt(g) gc) / (2 s)
    const double gsi = gnu * Ui + gnv * Vi + gsden + C::sqrt_g * gci;
    const double gsj = gnu * Uj + gnv * Vj + gsden + C::sqrt_g * gcj;
    if (F.hmb) {
        const double hghm = gcm * (0.5 * G) * F.hrcm;
        gHi += hghm; gHj += hghm;
    }
    gHi = fma(gsi, F.hrsi, gHi);
    gHj = fma(gsj, F.hrsj, gHj);
    // written, not added: the caller's outputs hold nothing before (a dry side's are 0)
    ghi = F.wi ? gHi : 0.0; gui = F.wi ? gUi : 0.0; gvi = F.wi ? gVi : 0.0;
    ghj = F.wj ? gHj : 0.0; guj = F.wj ? gUj : 0.0; gvj = F.wj ? gVj : 0.0;
}

// Inputs and adjoints of one hydrostatic face: eta, z, u, v of the two cells
// and the cells' slopes along the normal.
struct FaceVals {
    double eL, eR, zL, zR, uL, uR, vL, vR, seL, seR, suL, suR, svL, svR;
};

// Reverse of the hydrostatic face (HydrostaticRoe.cpp:247-396) for direction
// DIR, given the adjoints of FL and FR (global frame).  Writes g.
template <int DIR, bool FAST, bool REC = false>
__device__ void face_rev(const FaceVals& f, const double gFL[3], const double gFR[3], FaceVals& g,
                         const RoeRecVals* rec = nullptr) {
    const bool zLmax = okey(f.zL) >= okey(f.zR);  // std::max(zL, zR) keeps zL on ties
    const double zf = zLmax ? f.zL : f.zR;
    const double etaLf = f.eL + 0.5 * f.seL, etaRf = f.eR - 0.5 * f.seR;
    const double uLf = f.uL + 0.5 * f.suL, uRf = f.uR - 0.5 * f.suR;
    const double vLf = f.vL + 0.5 * f.svL, vRf = f.vR - 0.5 * f.svR;
    const double dLu = etaLf - f.zL, dRu = etaRf - f.zR, dLs = etaLf - zf, dRs = etaRf - zf;
    const double hLu = max0_i(dLu), hRu = max0_i(dRu);
    const double hLs = max0_i(dLs), hRs = max0_i(dRs);
    // normal frame
    const double unL = DIR == 0 ? uLf : vLf, utL = DIR == 0 ? vLf : -uLf;
    const double unR = DIR == 0 ? uRf : vRf, utR = DIR == 0 ? vRf : -uRf;
    double gf0 = gFL[0] + gFR[0], gf1 = gFL[1] + gFR[1], gf2 = gFL[2] + gFR[2];
    double gpL, gpR, b1, b2;
    if (DIR == 0) { gpL = gFL[1]; gpR = gFR[1]; b1 = gf1; b2 = gf2; }
    else { gpL = gFL[2]; gpR = gFR[2]; b1 = gf2; b2 = -gf1; }
    double ghLs = 0, gunL = 0, gutL = 0, ghRs = 0, gunR = 0, gutR = 0;
    if constexpr (FAST) {
        RoeFwd F;
        if constexpr (REC) roe_fwd_rec(hLs, unL, utL, hRs, unR, utR, *rec, F);
        else roe_fwd_fast(hLs, unL, utL, hRs, unR, utR, F);
        roe_rev_core(F, gf0, b1, b2, ghLs, gunL, gutL, ghRs, gunR, gutR);
    } else {
        static_assert(!REC, "face records are kept for the fast form");
        roe_rev(hLs, unL, utL, hRs, unR, utR, gf0, b1, b2, ghLs, gunL, gutL, ghRs, gunR, gutR);
    }
    // pressure correction p = HG (hu^2 - hs^2)
    double getaL, getaR, gzL, gzR;
    if constexpr (FAST) {
        // the face-bed side's capped and uncapped depths are one value, so its two pressure terms cancel:
        // only the lower side's are formed (as in the fast forward); the depth caps max(0, .) pass the
        // adjoints where their argument is positive
        if (zLmax) {  // left: the face-bed side
            ghRs = fma(-gpR, G * hRs, ghRs);
            const double ghRu = gpR * (G * hRu);
            const double sL = pos_i(dLs) ? ghLs : 0.0, sR = pos_i(dRs) ? ghRs : 0.0;
            const double uR = pos_i(dRu) ? ghRu : 0.0;
            getaL = sL; getaR = sR + uR;
            gzL = -(sL + sR); gzR = -uR;
        } else {
            ghLs = fma(-gpL, G * hLs, ghLs);
            const double ghLu = gpL * (G * hLu);
            const double sL = pos_i(dLs) ? ghLs : 0.0, sR = pos_i(dRs) ? ghRs : 0.0;
            const double uL = pos_i(dLu) ? ghLu : 0.0;
            getaL = sL + uL; getaR = sR;
            gzL = -uL; gzR = -(sL + sR);
        }
    } else {
        getaL = 0; getaR = 0; gzL = 0; gzR = 0;
        double gzf = 0;
        const double ghLu = gpL * (G * hLu), ghRu = gpR * (G * hRu);
        ghLs = fma(-gpL, G * hLs, ghLs);
        ghRs = fma(-gpR, G * hRs, ghRs);
        if (pos_i(dLu)) { getaL += ghLu; gzL -= ghLu; }
        if (pos_i(dRu)) { getaR += ghRu; gzR -= ghRu; }
        if (pos_i(dLs)) { getaL += ghLs; gzf -= ghLs; }
        if (pos_i(dRs)) { getaR += ghRs; gzf -= ghRs; }
        if (zLmax) gzL += gzf; else gzR += gzf;
    }
    double guL, gvL, guR, gvR;
    if (DIR == 0) { guL = gunL; gvL = gutL; guR = gunR; gvR = gutR; }
    else { gvL = gunL; guL = -gutL; gvR = gunR; guR = -gutR; }
    // the adjoints of the face states (written: the caller's g holds nothing else).  Those of the cells'
    // slopes follow from them (+1/2 on the left, -1/2 on the right), and the slope reverse forms them there.
    g.eL = getaL; g.eR = getaR;
    g.uL = guL; g.uR = guR;
    g.vL = gvL; g.vR = gvR;
    g.zL = gzL; g.zR = gzR;
}

// Reverse of van_leer_slope(qm, q, qp) (HydrostaticRoe.cpp:179-195).
__device__ __forceinline__ void slope_rev(double qm, double q, double qp, double gs, double& gqm, double& gq,
                                          double& gqp) {
    gqm = gq = gqp = 0.0;
    const double dm = q - qm, dp = qp - q;
    if (abs_le_bits(dp, Cst<double>::tol12_bits) || (sbits(gs) << 1) == 0) return;
    if ((sbits(dm) << 1) == 0) {  // r = 0: the mean of the one-sided derivatives (0 and 2), d s / d dm = 1
        gq = gs;
        gqm = -gs;
        return;
    }
    if (!pos_i(dm * dp)) return;  // phi = 0 for r < 0
    const double rS = rcp_nr(dm + dp);
    const double t = 2.0 * gs * rS * rS;
    const double gdm = t * dp * dp, gdp = t * dm * dm;
    gq = gdm - gdp;
    gqm = -gdm;
    gqp = gdp;
}

// slope_rev with the reciprocal from van_leer_slope_rs (rS == 0: the slope was 0 by a branch), given
// gs2 = twice the slope's adjoint (what the faces hand over: the slope enters each face state with 1/2).
__device__ __forceinline__ void slope_rev_rs(double qm, double q, double qp, double rS, double gs2, double& gqm,
                                             double& gq, double& gqp) {
    gqm = gq = gqp = 0.0;
    if ((sbits(gs2) << 1) == 0) return;
    const double dm = q - qm, dp = qp - q;
    if ((sbits(rS) << 1) == 0) {
        if (!abs_le_bits(dp, Cst<double>::tol12_bits) && (sbits(dm) << 1) == 0) {  // r = 0: d s / d dm = 1
            gq = 0.5 * gs2;
            gqm = -gq;
        }
        return;
    }
    const double t = gs2 * rS * rS;  // 2 gs / S^2
    const double gdm = t * dp * dp, gdp = t * dm * dm;
    gq = gdm - gdp;
    gqm = -gdm;
    gqp = gdp;
}

// ---------------------------------------------------------------------------
// Kernel B: face reverse of one tile.
// ---------------------------------------------------------------------------
struct AdjSmem {
    static constexpr int GX = ATX + 2 * H3, GY = ATY + 2 * H3;
    double hp[GY][GX], eta[GY][GX], u[GY][GX], v[GY][GX], z[GY][GX], lam[3][GY][GX];
    unsigned char nod[GY][GX];
    union {
        struct {  // x pass
            double s[3][ATY][ATX + 4];      // slopes of columns x0-2 .. x0+TX+1
            double rs[3][ATY][ATX + 4];     // their 1 / (dm + dp) (fast form; 0 where the slope is 0 by a branch)
            double fa[8][ATY][ATX + 3];     // face adjoints of eta, z, u, v on either side, faces x0-1 .. x0+TX+1
            double sp[9][ATY][ATX + 2];     // slope-reverse partials, columns x0-1 .. x0+TX
        } x;
        struct {  // y pass
            double s[3][ATY + 4][ATX];
            double rs[3][ATY + 4][ATX];
            double fa[8][ATY + 3][ATX];
            double sp[9][ATY + 2][ATX];
        } y;
    } p;
    double fold[4][ATY][ATX];  // ghost adjoints folded into own cells (h, hu, hv, z)
};

struct AdjArgs {
    LevelSrc<double> src;  // U^n, z, n with the level's BCs
    const double* lam[3];  // lambda_lin
    double* out[3];        // lambda^n
    double* zbar;          // accumulated gradient w.r.t. z
    long long pitch;
    int nx, ny;
    double cx, cy;         // dt/dx, dt/dy
    double dx, dy, idx, idy, idt;
    // per block: CFL rate arg max of U^n (rate, cell, flags) and, when un1 is set
    // (a step without friction or clamp, lambda_lin = lambda^{n+1}), the dt partial
    // sum_c lambda^{n+1} . (U^{n+1} - U^n) / dt
    const double* un1[3];
    double *p_dt, *p_rate;
    long long* p_idx;
    unsigned* p_fl;
    FaceRec rec;  // the step's face records (k_adj_faces<true, true>)
    // the step's finish, run by the last block to finish (done != null): block counter (zero between
    // launches), CFL number, gauges and the reference series of step n
    unsigned* done = nullptr;
    double cfl = 0.0, seed = 0.0;
    int ngauges = 0;
    const long long* gauges = nullptr;
    const double* href = nullptr;
};

// The record of x face (f, j) (d = 0) or y face (i, f) (d = 1).
__device__ __forceinline__ RoeRecVals load_rec(const FaceRec& R, int d, long long o) {
    const double* b = R.f[d] + o;
    const long long ps = R.plane[d];
    RoeRecVals r;
    r.si = b[0]; r.sj = b[ps]; r.cm = b[2 * ps]; r.rs = b[3 * ps]; r.hrden = b[4 * ps]; r.hrcm = b[5 * ps];
    r.um = b[6 * ps]; r.vm = b[7 * ps]; r.l0 = b[8 * ps]; r.l2 = b[9 * ps]; r.a0h = b[10 * ps];
    r.a1h = b[11 * ps]; r.a2h = b[12 * ps];
    r.fl = R.fl[d][o];
    return r;
}

__device__ __forceinline__ double fget(const FaceVals& f, int k) { return (&f.eL)[k]; }

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
    return s;
}

// The end of a reverse step: the CFL arg max and dt adjoint over the blocks' partials, the dt term
// folded into lambda at the arg-max cell, and the gauge misfit of step n.  One block.
__device__ __forceinline__ void adj_finish_body(int nblocks, const double* dtbar_p, const double* prate,
                                                     const long long* pidx, const unsigned* pflags, double cfl,
                                                     double dx, double dy, const double* h, const double* hu,
                                                     const double* hv, double* lam_h, double* lam_hu, double* lam_hv,
                                                     int with_dt, int ngauges, const long long* gauges,
                                                     const double* href, double seed) {
    __shared__ double sh[ANT / 32];
    __shared__ double s_rate[ANT / 32];
    __shared__ long long s_idx[ANT / 32];
    __shared__ unsigned s_fl[ANT / 32];
    double d = 0, rate = 0;
    long long idx = 0x7fffffffffffffffll;
    unsigned fl = 0;
    if (with_dt) {
        for (int k = threadIdx.x; k < nblocks; k += ANT) {
            d += __ldcg(dtbar_p + k);
            const double pr = __ldcg(prate + k);
            const long long pi = __ldcg(pidx + k);
            if (pr > rate || (pr == rate && pi < idx)) { rate = pr; idx = pi; }
            fl |= __ldcg(pflags + k);
        }
    }
    const double dtbar = block_sum(d, sh);
    for (int o = 16; o > 0; o >>= 1) {  // arg max: the larger rate, then the lower cell offset
        const double r2 = __shfl_xor_sync(0xffffffffu, rate, o);
        const long long i2 = __shfl_xor_sync(0xffffffffu, idx, o);
        if (r2 > rate || (r2 == rate && i2 < idx)) { rate = r2; idx = i2; }
    }
    fl = __reduce_or_sync(0xffffffffu, fl);
    if ((threadIdx.x & 31) == 0) {
        s_rate[threadIdx.x >> 5] = rate;
        s_idx[threadIdx.x >> 5] = idx;
        s_fl[threadIdx.x >> 5] = fl;
    }
    __syncthreads();
    if (threadIdx.x == 0 && with_dt) {
        for (int k = 1; k < ANT / 32; ++k) {
            if (s_rate[k] > rate || (s_rate[k] == rate && s_idx[k] < idx)) { rate = s_rate[k]; idx = s_idx[k]; }
            fl |= s_fl[k];
        }
        // dt = cfl * min(1/rate, 1e6 if a dry cell, 1e30 if NODATA): differentiable through the rate only
        const double m = accum_dt_min<double>(to_bits<double>(rate), fl);
        if (rate > 0 && m == 1.0 / rate) {
            const double hh = h[idx], u = hu[idx] / hh, v = hv[idx] / hh, c = sqrt(G * hh);
            const double gr = dtbar * (-cfl / (rate * rate));  // d dt / d rate
            const double su = sgn(u), sv = sgn(v), dc = G / (2.0 * c);
            lam_h[idx] = __ldcg(lam_h + idx) + gr * ((su * (-u / hh) + dc) / dx + (sv * (-v / hh) + dc) / dy);
            lam_hu[idx] = __ldcg(lam_hu + idx) + gr * su / (hh * dx);
            lam_hv[idx] = __ldcg(lam_hv + idx) + gr * sv / (hh * dy);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < ngauges; k += ANT) {  // atomic: a cell may be listed twice
        const long long gcell = gauges[k];
        atomicAdd(&lam_h[gcell], seed * 2.0 * (h[gcell] - href[k]));
    }
}


template <bool FAST, bool REC = false>
__global__ void __launch_bounds__(ANT) k_adj_faces(AdjArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    AdjSmem& S = *reinterpret_cast<AdjSmem*>(smem_raw);
    constexpr int GX = AdjSmem::GX, GY = AdjSmem::GY;
    const int t = threadIdx.x;
    const int x0 = blockIdx.x * ATX, y0 = blockIdx.y * ATY;
    const int nx = A.nx, ny = A.ny;

    // forward values on the grown tile (halo 3) and lambda_lin (0 outside the domain)
    for (int idx = t; idx < GX * GY; idx += ANT) {
        const int r = idx / GX, c = idx - r * GX;
        const int gi = x0 + c - H3, gj = y0 + r - H3;
        double e = 0, zz = 0, qx = 0, qy = 0, nn = 0;
        const bool in_grown = gi >= -2 && gi <= nx + 1 && gj >= -2 && gj <= ny + 1;
        // the forward's own depth: in the fast form a cell of the level takes its stored depth (a ghost the
        // rebuild from its rule's eta and z); both have dh'/dh = 1, dh'/dz = 0 where h' > 0
        const bool stored = FAST && gi >= 0 && gi < nx && gj >= 0 && gj < ny;
        if (stored) A.src.fetch_in(gi, gj, e, zz, qx, qy);  // e: h
        else if (in_grown) A.src.fetch(gi, gj, e, zz, qx, qy, nn);
        const double hp = stored ? max0_i(e) : max0_i(e - zz);
        S.hp[r][c] = hp;
        S.eta[r][c] = hp + zz;
        if constexpr (FAST) {  // the forward's own velocity arithmetic, so the limiters take its branches
            const double rh = gt_bits(hp, Cst<double>::tol12_bits) ? rcp_nr(hp) : 0.0;
            S.u[r][c] = qx * rh;
            S.v[r][c] = qy * rh;
        } else {
            S.u[r][c] = gt_bits(hp, Cst<double>::tol12_bits) ? qx / hp : 0.0;
            S.v[r][c] = gt_bits(hp, Cst<double>::tol12_bits) ? qy / hp : 0.0;
        }
        S.z[r][c] = zz;
        S.nod[r][c] = (in_grown && is_nodata(zz)) ? 1 : 0;
        const bool inside = gi >= 0 && gi < nx && gj >= 0 && gj < ny;
        const long long o = (long long)gi + (long long)gj * A.pitch;
        for (int k = 0; k < 3; ++k) S.lam[k][r][c] = inside ? A.lam[k][o] : 0.0;
    }
    for (int idx = t; idx < 4 * ATX * ATY; idx += ANT) (&S.fold[0][0][0])[idx] = 0.0;
    __syncthreads();

    const int tx = t % ATX, ty = t / ATX;
    double ae = 0, au = 0, av = 0, az = 0;  // gathered adjoints of this thread's cell

    // ===================== x pass =====================
    {
        auto& P = S.p.x;
        for (int k = t; k < ATY * (ATX + 4); k += ANT) {  // slopes, columns x0-2 .. x0+TX+1
            const int row = k / (ATX + 4), col = k % (ATX + 4) - 2;
            const int r = row + H3, c = col + H3;
            if constexpr (REC) {  // recorded for cells -1..nx; others feed no face of the domain
                const int gi = x0 + col, gj = y0 + row;
                const bool in = gi >= -1 && gi <= nx && gj < ny;
                const long long o = (long long)(gi + 1) + (long long)gj * (nx + 2), ps = A.rec.slplane[0];
                for (int q = 0; q < 3; ++q) {
                    P.s[q][row][col + 2] = in ? A.rec.sl[0][q * ps + o] : 0.0;
                    P.rs[q][row][col + 2] = in ? A.rec.sl[0][(3 + q) * ps + o] : 0.0;
                }
            } else if constexpr (FAST) {
                P.s[0][row][col + 2] = van_leer_slope_rs(S.eta[r][c - 1], S.eta[r][c], S.eta[r][c + 1], P.rs[0][row][col + 2]);
                P.s[1][row][col + 2] = van_leer_slope_rs(S.u[r][c - 1], S.u[r][c], S.u[r][c + 1], P.rs[1][row][col + 2]);
                P.s[2][row][col + 2] = van_leer_slope_rs(S.v[r][c - 1], S.v[r][c], S.v[r][c + 1], P.rs[2][row][col + 2]);
            } else {
                P.s[0][row][col + 2] = van_leer_slope<double, false>(S.eta[r][c - 1], S.eta[r][c], S.eta[r][c + 1]);
                P.s[1][row][col + 2] = van_leer_slope<double, false>(S.u[r][c - 1], S.u[r][c], S.u[r][c + 1]);
                P.s[2][row][col + 2] = van_leer_slope<double, false>(S.v[r][c - 1], S.v[r][c], S.v[r][c + 1]);
            }
        }
        __syncthreads();
        for (int k = t; k < ATY * (ATX + 3); k += ANT) {  // faces x0-1 .. x0+TX+1
            const int row = k / (ATX + 3), fcol = k % (ATX + 3) - 1;  // face at the left of column fcol
            const int f = x0 + fcol, gj = y0 + row;
            const int r = row + H3, cl = fcol - 1 + H3, cr = fcol + H3;
            FaceVals g{};
            if (f >= 0 && f <= nx && gj < ny && !(S.nod[r][cl] | S.nod[r][cr])) {
                FaceVals fv;
                fv.eL = S.eta[r][cl]; fv.eR = S.eta[r][cr]; fv.zL = S.z[r][cl]; fv.zR = S.z[r][cr];
                fv.uL = S.u[r][cl]; fv.uR = S.u[r][cr]; fv.vL = S.v[r][cl]; fv.vR = S.v[r][cr];
                fv.seL = P.s[0][row][fcol - 1 + 2]; fv.seR = P.s[0][row][fcol + 2];
                fv.suL = P.s[1][row][fcol - 1 + 2]; fv.suR = P.s[1][row][fcol + 2];
                fv.svL = P.s[2][row][fcol - 1 + 2]; fv.svR = P.s[2][row][fcol + 2];
                // FL(f) enters cell f-1 with -cx, FR(f) enters cell f with +cx; the face reverse is linear in
                // these, so it runs on -lambda, +lambda and the gathers below apply cx once per cell
                double gFL[3], gFR[3];
                for (int c = 0; c < 3; ++c) {
                    gFL[c] = -S.lam[c][r][cl];
                    gFR[c] = S.lam[c][r][cr];
                }
                if constexpr (REC) {
                    const RoeRecVals rv = load_rec(A.rec, 0, (long long)f + (long long)gj * (nx + 1));
                    face_rev<0, FAST, true>(fv, gFL, gFR, g, &rv);
                } else {
                    face_rev<0, FAST>(fv, gFL, gFR, g);
                }
            }
            for (int q = 0; q < 8; ++q) P.fa[q][row][fcol + 1] = fget(g, q);
        }
        __syncthreads();
        for (int k = t; k < ATY * (ATX + 2); k += ANT) {  // slope reverse, columns x0-1 .. x0+TX
            const int row = k / (ATX + 2), col = k % (ATX + 2) - 1;
            const int r = row + H3, c = col + H3;
            // slope of this column: read as the R slope by face col (index col+1), where the face state is
            // q - s/2, and as the L slope by face col+1, where it is q + s/2; twice its adjoint is the
            // difference of the two face states' adjoints
            for (int qi = 0; qi < 3; ++qi) {
                const int qL = qi == 0 ? 0 : 2 + 2 * qi, qR = qL + 1;  // eta: 0, 1; u: 4, 5; v: 6, 7
                const double gs2 = P.fa[qL][row][col + 2] - P.fa[qR][row][col + 1];
                const double(*Q)[GX] = qi == 0 ? S.eta : (qi == 1 ? S.u : S.v);
                double gm, g0, gp;
                if constexpr (FAST) slope_rev_rs(Q[r][c - 1], Q[r][c], Q[r][c + 1], P.rs[qi][row][col + 2], gs2, gm, g0, gp);
                else slope_rev(Q[r][c - 1], Q[r][c], Q[r][c + 1], 0.5 * gs2, gm, g0, gp);
                P.sp[3 * qi + 0][row][col + 1] = gm;  // to column col-1
                P.sp[3 * qi + 1][row][col + 1] = g0;  // to column col
                P.sp[3 * qi + 2][row][col + 1] = gp;  // to column col+1
            }
        }
        __syncthreads();
        // gather for column c: faces c (R side) and c+1 (L side), slopes c-1 (to right), c (self), c+1 (to left)
        auto gather_x = [&](int row, int col, double& ge, double& gu, double& gv, double& gz) {
            auto F = [&](int q, int fcol) { return (fcol >= -1 && fcol <= ATX + 1) ? P.fa[q][row][fcol + 1] : 0.0; };
            auto SP = [&](int q, int scol) { return (scol >= -1 && scol <= ATX) ? P.sp[q][row][scol + 1] : 0.0; };
            ge = A.cx * (F(1, col) + F(0, col + 1) + SP(2, col - 1) + SP(1, col) + SP(0, col + 1));
            gu = A.cx * (F(5, col) + F(4, col + 1) + SP(5, col - 1) + SP(4, col) + SP(3, col + 1));
            gv = A.cx * (F(7, col) + F(6, col + 1) + SP(8, col - 1) + SP(7, col) + SP(6, col + 1));
            gz = A.cx * (F(3, col) + F(2, col + 1));
        };
        gather_x(ty, tx, ae, au, av, az);  // the x pass starts the cell's sums
        // x-boundary ghosts: one thread per row folds both sides
        if (t < ATY && y0 + t < ny) {
            const int row = t, gj = y0 + row, r = row + H3;
            for (int side = 0; side < 2; ++side) {
                const bool lo = side == 0;
                if (lo ? (x0 != 0) : (x0 + ATX - 1 < nx - 1)) continue;
                const int code = lo ? A.src.bc_xlo : A.src.bc_xhi;
                for (int k = 1; k <= 2; ++k) {
                    const int gi = lo ? -k : nx - 1 + k;  // ghost column
                    const int col = gi - x0, c = col + H3;
                    double ge, gu, gv, gz;
                    gather_x(row, col, ge, gu, gv, gz);
                    const double hp = S.hp[r][c];
                    double gzt = gz + ge, ghp = ge, ghu = 0, ghv = 0;
                    if (gt_bits(hp, Cst<double>::tol12_bits)) {
                        ghu = gu / hp;
                        ghv = gv / hp;
                        ghp -= (gu * S.u[r][c] + gv * S.v[r][c]) / hp;
                    }
                    double geta = 0;
                    if (pos_i(hp)) { geta = ghp; gzt -= ghp; }
                    const int edge = lo ? 0 : nx - 1;
                    const bool wall = bc_is_wall(code);
                    const int src = wall ? (lo ? -1 - gi : 2 * nx - 1 - gi) : edge;
                    bool neg_u, neg_v;  // the forward's sign flips of this ghost's momenta (ghost_source)
                    ghost_momentum_signs(wall, code, false, -1, neg_u, neg_v);
                    const int sc = src - x0, ec = edge - x0;
                    if (sc >= 0 && sc < ATX) {
                        S.fold[0][row][sc] += geta;
                        S.fold[3][row][sc] += geta;
                        S.fold[1][row][sc] += neg_u ? -ghu : ghu;
                        S.fold[2][row][sc] += neg_v ? -ghv : ghv;
                    }
                    if (ec >= 0 && ec < ATX) S.fold[3][row][ec] += gzt;
                    (void)gj;
                }
            }
        }
        __syncthreads();
    }

    // ===================== y pass =====================
    {
        auto& P = S.p.y;
        for (int k = t; k < (ATY + 4) * ATX; k += ANT) {  // slopes, rows y0-2 .. y0+TY+1
            const int row = k / ATX - 2, col = k % ATX;
            const int r = row + H3, c = col + H3;
            if constexpr (REC) {
                const int gi = x0 + col, gj = y0 + row;
                const bool in = gj >= -1 && gj <= ny && gi < nx;
                const long long o = (long long)gi + (long long)(gj + 1) * nx, ps = A.rec.slplane[1];
                for (int q = 0; q < 3; ++q) {
                    P.s[q][row + 2][col] = in ? A.rec.sl[1][q * ps + o] : 0.0;
                    P.rs[q][row + 2][col] = in ? A.rec.sl[1][(3 + q) * ps + o] : 0.0;
                }
            } else if constexpr (FAST) {
                P.s[0][row + 2][col] = van_leer_slope_rs(S.eta[r - 1][c], S.eta[r][c], S.eta[r + 1][c], P.rs[0][row + 2][col]);
                P.s[1][row + 2][col] = van_leer_slope_rs(S.u[r - 1][c], S.u[r][c], S.u[r + 1][c], P.rs[1][row + 2][col]);
                P.s[2][row + 2][col] = van_leer_slope_rs(S.v[r - 1][c], S.v[r][c], S.v[r + 1][c], P.rs[2][row + 2][col]);
            } else {
                P.s[0][row + 2][col] = van_leer_slope<double, false>(S.eta[r - 1][c], S.eta[r][c], S.eta[r + 1][c]);
                P.s[1][row + 2][col] = van_leer_slope<double, false>(S.u[r - 1][c], S.u[r][c], S.u[r + 1][c]);
                P.s[2][row + 2][col] = van_leer_slope<double, false>(S.v[r - 1][c], S.v[r][c], S.v[r + 1][c]);
            }
        }
        __syncthreads();
        for (int k = t; k < (ATY + 3) * ATX; k += ANT) {  // faces y0-1 .. y0+TY+1
            const int frow = k / ATX - 1, col = k % ATX;
            const int f = y0 + frow, gi = x0 + col;
            const int c = col + H3, rl = frow - 1 + H3, rr = frow + H3;
            FaceVals g{};
            if (f >= 0 && f <= ny && gi < nx && !(S.nod[rl][c] | S.nod[rr][c])) {
                FaceVals fv;
                fv.eL = S.eta[rl][c]; fv.eR = S.eta[rr][c]; fv.zL = S.z[rl][c]; fv.zR = S.z[rr][c];
                fv.uL = S.u[rl][c]; fv.uR = S.u[rr][c]; fv.vL = S.v[rl][c]; fv.vR = S.v[rr][c];
                fv.seL = P.s[0][frow - 1 + 2][col]; fv.seR = P.s[0][frow + 2][col];
                fv.suL = P.s[1][frow - 1 + 2][col]; fv.suR = P.s[1][frow + 2][col];
                fv.svL = P.s[2][frow - 1 + 2][col]; fv.svR = P.s[2][frow + 2][col];
                double gFL[3], gFR[3];  // unscaled, as in the x pass; cy in the gathers
                for (int q = 0; q < 3; ++q) {
                    gFL[q] = -S.lam[q][rl][c];
                    gFR[q] = S.lam[q][rr][c];
                }
                if constexpr (REC) {
                    const RoeRecVals rv = load_rec(A.rec, 1, (long long)gi + (long long)f * nx);
                    face_rev<1, FAST, true>(fv, gFL, gFR, g, &rv);
                } else {
                    face_rev<1, FAST>(fv, gFL, gFR, g);
                }
            }
            for (int q = 0; q < 8; ++q) P.fa[q][frow + 1][col] = fget(g, q);
        }
        __syncthreads();
        for (int k = t; k < (ATY + 2) * ATX; k += ANT) {  // slope reverse, rows y0-1 .. y0+TY
            const int row = k / ATX - 1, col = k % ATX;
            const int r = row + H3, c = col + H3;
            for (int qi = 0; qi < 3; ++qi) {  // as in the x pass: faces row (R side) and row+1 (L side)
                const int qL = qi == 0 ? 0 : 2 + 2 * qi, qR = qL + 1;
                const double gs2 = P.fa[qL][row + 2][col] - P.fa[qR][row + 1][col];
                const double(*Q)[GX] = qi == 0 ? S.eta : (qi == 1 ? S.u : S.v);
                double gm, g0, gp;
                if constexpr (FAST) slope_rev_rs(Q[r - 1][c], Q[r][c], Q[r + 1][c], P.rs[qi][row + 2][col], gs2, gm, g0, gp);
                else slope_rev(Q[r - 1][c], Q[r][c], Q[r + 1][c], 0.5 * gs2, gm, g0, gp);
                P.sp[3 * qi + 0][row + 1][col] = gm;
                P.sp[3 * qi + 1][row + 1][col] = g0;
                P.sp[3 * qi + 2][row + 1][col] = gp;
            }
        }
        __syncthreads();
        auto gather_y = [&](int row, int col, double& ge, double& gu, double& gv, double& gz) {
            auto F = [&](int q, int frow) { return (frow >= -1 && frow <= ATY + 1) ? P.fa[q][frow + 1][col] : 0.0; };
            auto SP = [&](int q, int srow) { return (srow >= -1 && srow <= ATY) ? P.sp[q][srow + 1][col] : 0.0; };
            ge = A.cy * (F(1, row) + F(0, row + 1) + SP(2, row - 1) + SP(1, row) + SP(0, row + 1));
            gu = A.cy * (F(5, row) + F(4, row + 1) + SP(5, row - 1) + SP(4, row) + SP(3, row + 1));
            gv = A.cy * (F(7, row) + F(6, row + 1) + SP(8, row - 1) + SP(7, row) + SP(6, row + 1));
            gz = A.cy * (F(3, row) + F(2, row + 1));
        };
        {
            double ge, gu, gv, gz;
            gather_y(ty, tx, ge, gu, gv, gz);
            ae += ge; au += gu; av += gv; az += gz;
        }
        if (t < ATX && x0 + t < nx) {
            const int col = t, c = col + H3;
            for (int side = 0; side < 2; ++side) {
                const bool lo = side == 0;
                if (lo ? (y0 != 0) : (y0 + ATY - 1 < ny - 1)) continue;
                const int code = lo ? A.src.bc_ylo : A.src.bc_yhi;
                for (int k = 1; k <= 2; ++k) {
                    const int gj = lo ? -k : ny - 1 + k;
                    const int row = gj - y0, r = row + H3;
                    double ge, gu, gv, gz;
                    gather_y(row, col, ge, gu, gv, gz);
                    const double hp = S.hp[r][c];
                    double gzt = gz + ge, ghp = ge, ghu = 0, ghv = 0;
                    if (gt_bits(hp, Cst<double>::tol12_bits)) {
                        ghu = gu / hp;
                        ghv = gv / hp;
                        ghp -= (gu * S.u[r][c] + gv * S.v[r][c]) / hp;
                    }
                    double geta = 0;
                    if (pos_i(hp)) { geta = ghp; gzt -= ghp; }
                    const int edge = lo ? 0 : ny - 1;
                    const bool wall = bc_is_wall(code);
                    const int src = wall ? (lo ? -1 - gj : 2 * ny - 1 - gj) : edge;
                    bool neg_u, neg_v;
                    ghost_momentum_signs(false, -1, wall, code, neg_u, neg_v);
                    const int sr = src - y0, er = edge - y0;
                    if (sr >= 0 && sr < ATY) {
                        S.fold[0][sr][col] += geta;
                        S.fold[3][sr][col] += geta;
                        S.fold[1][sr][col] += neg_u ? -ghu : ghu;
                        S.fold[2][sr][col] += neg_v ? -ghv : ghv;
                    }
                    if (er >= 0 && er < ATY) S.fold[3][er][col] += gzt;
                }
            }
        }
        __syncthreads();
    }

    // ===================== own cell: rebuild reverse, outputs, CFL rate, dt partial =====================
    const int gi = x0 + tx, gj = y0 + ty;
    const bool own = gi < nx && gj < ny;
    double rate = 0.0, dtb = 0.0;
    long long ridx = 0x7fffffffffffffffll;
    unsigned rfl = 0;
    if (own) {
        const int r = ty + H3, c = tx + H3;
        const double hp = S.hp[r][c];
        double gz = az + ae, ghp = ae, ghu = 0, ghv = 0;
        if (gt_bits(hp, Cst<double>::tol12_bits)) {
            const double rh = FAST ? rcp_nr(hp) : 1.0 / hp;
            ghu = au * rh;
            ghv = av * rh;
            ghp -= (au * S.u[r][c] + av * S.v[r][c]) * rh;
        }
        double gh = 0;
        if (pos_i(hp)) gh = ghp;  // h' = max(0, (h + z) - z): dh'/dh = 1, dh'/dz = 0
        const long long o = (long long)gi + (long long)gj * A.pitch;
        // lambda^n = lambda_lin (the stored state passes through the update) + the flux part + ghost folds
        A.out[0][o] = S.lam[0][r][c] + gh + S.fold[0][ty][tx];
        A.out[1][o] = S.lam[1][r][c] + ghu + S.fold[1][ty][tx];
        A.out[2][o] = S.lam[2][r][c] + ghv + S.fold[2][ty][tx];
        A.zbar[o] += gz + S.fold[3][ty][tx];
        if (A.un1[0])
            dtb = (S.lam[0][r][c] * (A.un1[0][o] - A.src.h[o]) + S.lam[1][r][c] * (A.un1[1][o] - A.src.hu[o]) +
                   S.lam[2][r][c] * (A.un1[2][o] - A.src.hv[o])) * A.idt;
    }
    // The block's CFL arg max.  The fast form screens it in float first (as the forward's fold does): only
    // the cells within 2^-12 of the block's largest float estimate, or with a non-finite one, take the FP64
    // rate; the cell holding the true maximum is always among them, ties included.
    __shared__ double s_sum[ANT / 32], s_rate[ANT / 32];
    __shared__ long long s_idx[ANT / 32];
    __shared__ unsigned s_fl[ANT / 32];
    __shared__ float s_r32[ANT / 32];
    {
        const int r = ty + H3, c = tx + H3;
        const long long o = (long long)gi + (long long)gj * A.pitch;
        double h = 0.0, hu = 0.0, hv = 0.0;
        bool wet = false, bad = false;
        float r32 = 0.f;
        if (own) {
            h = A.src.h[o]; hu = A.src.hu[o]; hv = A.src.hv[o];
            if (S.nod[r][c]) rfl |= DTF_NODATA;
            else if (!gt_bits(h, Cst<double>::tol12_bits)) rfl |= DTF_DRY;
            else wet = true;
        }
        if constexpr (FAST) {
            if (wet) {
                const float hf = f32_lead(h), qx = fabsf(f32_lead(hu)), qy = fabsf(f32_lead(hv));
                const float rh = rcp_nr(hf);
                const float u = qx * rh, v = qy * rh;
                const float cc = fast_sqrt(9.81f * hf);
                r32 = (u + cc) * f32_lead(A.idx) + (v + cc) * f32_lead(A.idy);
                bad = !(r32 <= 3.0e38f);
            }
            float wr = (wet && !bad) ? r32 : 0.f;
            for (int off = 16; off > 0; off >>= 1) wr = fmaxf(wr, __shfl_xor_sync(0xffffffffu, wr, off));
            if ((t & 31) == 0) s_r32[t >> 5] = wr;
            __syncthreads();
            float br = 0.f;
#pragma unroll
            for (int k = 0; k < ANT / 32; ++k) br = fmaxf(br, s_r32[k]);
            wet = bad || (wet && r32 >= br * (1.f - 0x1p-12f));
        }
        if (wet) {
            double mv;
            unsigned f = 0;
            dt_cell_contrib<double, FAST>(h, hu, hv, false, A.dx, A.dy, A.idx, A.idy, rate, mv, f);
            rfl |= f;
            if (pos_i(rate)) ridx = o;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        dtb += __shfl_xor_sync(0xffffffffu, dtb, off);
        const double r2 = __shfl_xor_sync(0xffffffffu, rate, off);
        const long long i2 = __shfl_xor_sync(0xffffffffu, ridx, off);
        if (r2 > rate || (r2 == rate && i2 < ridx)) { rate = r2; ridx = i2; }
    }
    rfl = __reduce_or_sync(0xffffffffu, rfl);
    const int w = t >> 5;
    if ((t & 31) == 0) { s_sum[w] = dtb; s_rate[w] = rate; s_idx[w] = ridx; s_fl[w] = rfl; }
    __syncthreads();
    if (t == 0) {
        double sum = s_sum[0];
        for (int k = 1; k < ANT / 32; ++k) {
            sum += s_sum[k];
            if (s_rate[k] > rate || (s_rate[k] == rate && s_idx[k] < ridx)) { rate = s_rate[k]; ridx = s_idx[k]; }
            rfl |= s_fl[k];
        }
        const long long b = blockIdx.x + (long long)blockIdx.y * gridDim.x;
        A.p_rate[b] = rate;
        A.p_idx[b] = ridx;
        A.p_fl[b] = rfl;
        if (A.un1[0]) A.p_dt[b] = sum;
    }
    if (A.done) {  // the last block to get here runs the step's finish (k_adj_finish's work, no launch)
        __shared__ bool s_last;
        const unsigned nb = gridDim.x * gridDim.y;
        if (t == 0) {
            __threadfence();  // this block's partials and lambda before its count
            s_last = atomicAdd(A.done, 1u) == nb - 1u;
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            adj_finish_body((int)nb, A.p_dt, A.p_rate, A.p_idx, A.p_fl, A.cfl, A.dx, A.dy, A.src.h, A.src.hu,
                            A.src.hv, A.out[0], A.out[1], A.out[2], 1, A.ngauges, A.gauges, A.href, A.seed);
            if (t == 0) *A.done = 0u;  // for the next step's launch (stream-ordered)
        }
    }
}

// ---------------------------------------------------------------------------
// Kernel A (general steps): lambda_lin = J_post^T lambda^{n+1} from the linear
// (pre-clamp) state, and the dt adjoint partials of the update.
// ---------------------------------------------------------------------------
struct PostArgs {
    const double* lin[3];   // state after the flux update, before friction / clamp
    const double* un[3];    // U^n
    const double* lam[3];   // lambda^{n+1}
    const double* nman;     // Manning n
    double* out[3];         // lambda_lin
    double* dtbar;          // one partial per block
    long long pitch;
    int nx, ny;
    double dt;
};


__global__ void __launch_bounds__(ANT) k_adj_post(PostArgs P) {
    __shared__ double sh[ANT / 32];
    const int i = blockIdx.x * ATX + (threadIdx.x % ATX), j = blockIdx.y * ATY + threadIdx.x / ATX;
    double dtb = 0;
    if (i < P.nx && j < P.ny) {
        const long long o = (long long)i + (long long)j * P.pitch;
        const double h = P.lin[0][o], qx = P.lin[1][o], qy = P.lin[2][o];
        const double lh = P.lam[0][o], lqx = P.lam[1][o], lqy = P.lam[2][o];
        double gh = 0, gqx = 0, gqy = 0, gdt = 0;
        if (h >= TD) {
            gh = lh;
            gqx = lqx;
            gqy = lqy;
            const double nv = P.nman[o], nsq = nv * nv;
            if (nsq > T12) {
                const double u = qx / h, vv = qy / h;
                const double modM = sqrt(u * u + vv * vv);
                if (modM > T12) {
                    const double h43 = h * cbrt(h);
                    const double tt = P.dt * G * nsq * modM / h43;
                    const double ff = sqrt(1.0 + 4.0 * tt);
                    const double fac = 2.0 / (1.0 + ff);
                    gqx = lqx * fac;
                    gqy = lqy * fac;
                    const double gfac = lqx * qx + lqy * qy;
                    const double gff = -gfac * fac * fac / 2.0;
                    const double gtt = gff * 2.0 / ff;
                    gdt += gtt * tt / P.dt;
                    const double gmod = gtt * tt / modM;
                    const double gh43 = -gtt * tt / h43;
                    gh += gh43 * (4.0 / 3.0) * h43 / h;
                    const double gu = gmod * u / modM, gv = gmod * vv / modM;
                    gqx += gu / h;
                    gqy += gv / h;
                    gh += -(gu * u + gv * vv) / h;
                }
            }
        } else {
            gh = h < 0.0 ? 0.0 : lh;  // max(h, 0) keeps h at h == 0 (a dry cell stays at its value); momenta are zeroed
        }
        P.out[0][o] = gh;
        P.out[1][o] = gqx;
        P.out[2][o] = gqy;
        // the flux update is linear in dt: d(lin)/d dt = (lin - U^n) / dt
        dtb = gdt + (gh * (h - P.un[0][o]) + gqx * (qx - P.un[1][o]) + gqy * (qy - P.un[2][o])) / P.dt;
    }
    const double s = block_sum(dtb, sh);
    if (threadIdx.x == 0) P.dtbar[blockIdx.x + (long long)blockIdx.y * gridDim.x] = s;
}

// Kernel C: dt adjoint into the cell that set the CFL bound, then the gauge
// misfit of state n (seed * 2 (h - href)).  One block.
__global__ void __launch_bounds__(ANT) k_adj_finish(int nblocks, const double* dtbar_p, const double* prate,
                                                     const long long* pidx, const unsigned* pflags, double cfl,
                                                     double dx, double dy, const double* h, const double* hu,
                                                     const double* hv, double* lam_h, double* lam_hu, double* lam_hv,
                                                     int with_dt, int ngauges, const long long* gauges,
                                                     const double* href, double seed) {
    adj_finish_body(nblocks, dtbar_p, prate, pidx, pflags, cfl, dx, dy, h, hu, hv, lam_h, lam_hu, lam_hv,
                    with_dt, ngauges, gauges, href, seed);
}

// h of the final state at the gauge cells.
__global__ void k_adj_series(const double* h, int ngauges, const long long* gauges, double* series) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ngauges; k += gridDim.x * blockDim.x)
        series[k] = h[gauges[k]];
}

}  // namespace

// ===========================================================================
// Drivers
// ===========================================================================
namespace {

struct AdjLayout {
    size_t plane;                 // doubles per plane (ny * pitch)
    int nslots, seg, binom;       // stored states; segment length (uniform); snapshot slots (binomial)
    size_t states, segbuf, segbuf_stride, lam, lamlin, lin, tmp, nxt, dthist, pflags, slots, status, done, part,
        total;
    int nblocks;
    // face records (uniform checkpoints, fast form, on request): one set per step of the two segments in
    // flight, after everything else so the layout is otherwise the same with and without them
    size_t rec, rec_step, rec_plane[2], rec_slplane[2];
};

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// ---------------------------------------------------------------------------
// Binomial checkpointing (Griewank's revolve schedule).  With c snapshot slots
// (one of them holding the state the reversal starts from) and r repetitions,
// beta(c, r) = C(c + r, c) steps can be reversed; the least number of forward
// steps to reverse n steps, the first sweep included, is
// t(n, c) = r n - beta(c + 1, r - 1) with r the least repetition number such
// that beta(c, r) >= n (Griewank and Walther, ACM TOMS 26(1), 2000).  Each
// split is chosen among the break points of the piecewise-linear cost
// k + t(n - k, c - 1) + t(k, c), which attains that optimum.
// ---------------------------------------------------------------------------
long long binom_beta(int c, int r) {
    if (c < 0 || r < 0) return 0;
    unsigned long long v = 1;  // C(c + r, r) built as prod (c + i) / i, integral at every step
    for (int i = 1; i <= r; ++i) {
        const unsigned long long f = (unsigned long long)(c + i);
        if (v > (1ull << 62) / f) return 1ll << 62;
        v = v * f / (unsigned long long)i;
    }
    return (long long)v;
}

int binom_reps(long long n, int c) {
    int r = 0;
    while (binom_beta(c, r) < n) ++r;
    return r;
}

long long binom_cost(long long n, int c) {
    if (n <= 1) return 0;
    if (c <= 1) return n * (n - 1) / 2;
    const int r = binom_reps(n, c);
    return (long long)r * n - binom_beta(c + 1, r - 1);
}

// Steps to advance before the next snapshot, reversing n >= 2 steps with c >= 2 slots.
long long binom_split(long long n, int c) {
    const int r = binom_reps(n, c);
    long long lo = n - binom_beta(c - 1, r), hi = binom_beta(c, r - 1);
    if (lo < 1) lo = 1;
    if (hi > n - 1) hi = n - 1;
    long long best_k = lo, best = -1;
    auto consider = [&](long long k) {
        if (k < lo || k > hi) return;
        const long long v = k + binom_cost(n - k, c - 1) + binom_cost(k, c);
        if (best < 0 || v < best || (v == best && k < best_k)) { best = v; best_k = k; }
    };
    consider(lo);
    consider(hi);
    for (int j = 0; j <= r + 1; ++j) {
        const long long b1 = binom_beta(c, j), b2 = binom_beta(c - 1, j);
        consider(b1); consider(b1 + 1); consider(n - b2); consider(n - b2 - 1);
    }
    return best_k;
}

// Snapshot positions the forward sweep stores (the schedule's first descent),
// in the order the slots 1, 2, ... are taken.
std::vector<long long> binom_chain(long long n, int c) {
    std::vector<long long> pos;
    long long a = 0;
    while (n > 1 && c > 1) {
        const long long k = binom_split(n, c);
        a += k;
        pos.push_back(a);
        n -= k;
        --c;
    }
    return pos;
}

AdjLayout adj_layout(int nx, int ny, long long pitch, int nsteps, int every, bool records = false) {
    AdjLayout L{};
    L.plane = (size_t)ny * (size_t)pitch;
    const size_t st = 3 * L.plane * sizeof(double);
    L.binom = every < 0 ? (-every < nsteps + 1 ? -every : nsteps + 1) : 0;
    if (L.binom == 1) L.binom = 2;  // the state the reversal starts from plus at least one snapshot
    L.seg = (every > 0 && every < nsteps) ? every : 0;
    L.nslots = L.binom ? L.binom : (L.seg ? (nsteps / L.seg + 1) : (nsteps + 1));
    size_t o = 0;
    L.states = o; o += al256((size_t)L.nslots * st);
    L.segbuf_stride = L.seg ? al256((size_t)(L.seg + 1) * st) : 0;
    L.segbuf = o; o += L.seg ? 2 * al256((size_t)(L.seg + 1) * st) : 0;  // two segments in flight
    L.tmp = o; o += L.seg ? al256(2 * st) : (L.binom ? al256(3 * st) : 0);
    L.nxt = o; o += L.binom ? al256(st) : 0;
    L.lam = o; o += al256(2 * st);
    L.lamlin = o; o += al256(st);
    L.lin = o; o += al256(st);
    L.dthist = o; o += al256((size_t)nsteps * sizeof(double));
    L.pflags = o; o += al256((size_t)nsteps * sizeof(unsigned));
    L.slots = o; o += 256;
    L.status = o; o += 256;
    L.done = o; o += 256;  // the reverse kernel's block counter (its fused finish)
    L.nblocks = ((nx + ATX - 1) / ATX) * ((ny + ATY - 1) / ATY);
    L.part = o; o += al256((size_t)L.nblocks * (2 * sizeof(double) + sizeof(long long) + sizeof(unsigned)));
    if (records && L.seg) {
        L.rec_plane[0] = al256((size_t)(nx + 1) * ny * sizeof(double)) / sizeof(double);
        L.rec_plane[1] = al256((size_t)nx * (ny + 1) * sizeof(double)) / sizeof(double);
        L.rec_slplane[0] = al256((size_t)(nx + 2) * ny * sizeof(double)) / sizeof(double);
        L.rec_slplane[1] = al256((size_t)nx * (ny + 2) * sizeof(double)) / sizeof(double);
        L.rec_step = (NREC * (L.rec_plane[0] + L.rec_plane[1]) + 6 * (L.rec_slplane[0] + L.rec_slplane[1])) *
                         sizeof(double) +
                     al256((size_t)(nx + 1) * ny) + al256((size_t)nx * (ny + 1));
        L.rec = o; o += 2 * (size_t)L.seg * L.rec_step;
    }
    L.total = o;
    return L;
}

// The face records of step slot k (0 .. 2 seg - 1) of the layout.
FaceRec rec_at(const AdjLayout& A, char* base, int k, int nx, int ny) {
    FaceRec R;
    char* p = base + A.rec + (size_t)k * A.rec_step;
    R.f[0] = reinterpret_cast<double*>(p);
    R.f[1] = R.f[0] + NREC * A.rec_plane[0];
    R.sl[0] = R.f[1] + NREC * A.rec_plane[1];
    R.sl[1] = R.sl[0] + 6 * A.rec_slplane[0];
    R.slplane[0] = (long long)A.rec_slplane[0];
    R.slplane[1] = (long long)A.rec_slplane[1];
    R.fl[0] = reinterpret_cast<unsigned char*>(R.sl[1] + 6 * A.rec_slplane[1]);
    R.fl[1] = R.fl[0] + al256((size_t)(nx + 1) * ny);
    R.plane[0] = (long long)A.rec_plane[0];
    R.plane[1] = (long long)A.rec_plane[1];
    R.nx = nx;
    R.ny = ny;
    return R;
}

struct Views {
    double* base;
    size_t plane;
    double* state(size_t off, int k) const { return base + off / sizeof(double) + (size_t)k * 3 * plane; }
};

int adj_check(const hx_level_f64* L, int nsteps, int ngauges, const int64_t* gauges) {
    if (!L || !L->h || !L->hu || !L->hv || !L->z || !L->n) return set_error(HX_ERR_ARG, "adjoint: null level plane");
    if (L->nx < 2 || L->ny < 2 || L->pitch < L->nx || !(L->dx > 0) || !(L->dy > 0))
        return set_error(HX_ERR_ARG, "adjoint: bad level geometry");
    if (L->nx % ATX == 1 || L->ny % ATY == 1)
        return set_error(HX_ERR_ARG, "adjoint: nx % 32 == 1 or ny % 16 == 1 is not supported (a one-cell edge tile)");
    if (nsteps < 1) return set_error(HX_ERR_ARG, "adjoint: nsteps < 1");
    if (ngauges < 0 || (ngauges > 0 && !gauges)) return set_error(HX_ERR_ARG, "adjoint: bad gauges");
    if (ngauges > 0) {  // gauge offsets i + j * pitch must name cells of the level
        std::vector<int64_t> g((size_t)ngauges);
        if (cudaMemcpy(g.data(), gauges, g.size() * sizeof(int64_t), cudaMemcpyDeviceToHost) != cudaSuccess)
            return set_error(HX_ERR_CUDA, "adjoint: gauges are not readable device memory");
        for (int64_t o : g)
            if (o < 0 || o % L->pitch >= L->nx || o / L->pitch >= L->ny)
                return set_error(HX_ERR_ARG, "adjoint: gauge offset outside the level");
    }
    return HX_OK;
}

LevelSrc<double> make_src(const hx_level_f64* L, const double* const* st, int g) {
    LevelSrc<double> s;
    s.h = st[0]; s.hu = st[1]; s.hv = st[2]; s.z = L->z; s.n = L->n;
    s.pitch = L->pitch;
    s.nx = L->nx; s.ny = L->ny;
    s.bc_xlo = L->bc_lo[0]; s.bc_ylo = L->bc_lo[1]; s.bc_xhi = L->bc_hi[0]; s.bc_yhi = L->bc_hi[1];
    s.glo0 = -g; s.glo1 = -g; s.ghi0 = L->nx - 1 + g; s.ghi1 = L->ny - 1 + g;
    return s;
}

template <bool FAST>
cudaError_t forward_step(const hx_level_f64* L, double* const* in, double* const* out, StepCtl<double> ctl,
                         const double* dt_fixed, unsigned* pflags, const AdjRecord& rec, cudaStream_t st) {
    const IBox vb{0, 0, L->nx - 1, L->ny - 1};
    const double* cin[3] = {in[0], in[1], in[2]};
    LevelSrc<double> src = make_src(L, cin, 2);
    Cells3<double> uo;
    for (int k = 0; k < 3; ++k) uo.p[k] = in[k];
    uo.js = L->pitch; uo.lo0 = 0; uo.lo1 = 0;
    Cells3W<double> o;
    for (int k = 0; k < 3; ++k) o.p[k] = out[k];
    o.js = L->pitch; o.lo0 = 0; o.lo1 = 0;
    Plane<double> np{L->n, L->pitch, 0, 0};
    return launch_adj_forward<FAST>(src, uo, np, o, vb, ctl, dt_fixed, pflags, rec, st);
}

// A recompute step at the recorded dt that also writes the step's face records.
cudaError_t forward_step_rec(const hx_level_f64* L, double* const* in, double* const* out, const double* dt_fixed,
                             const FaceRec& rec, cudaStream_t st) {
    const double* cin[3] = {in[0], in[1], in[2]};
    LevelSrc<double> src = make_src(L, cin, 2);
    Cells3<double> uo;
    for (int k = 0; k < 3; ++k) uo.p[k] = in[k];
    uo.js = L->pitch; uo.lo0 = 0; uo.lo1 = 0;
    Cells3W<double> o;
    for (int k = 0; k < 3; ++k) o.p[k] = out[k];
    o.js = L->pitch; o.lo0 = 0; o.lo1 = 0;
    Plane<double> np{L->n, L->pitch, 0, 0};
    return launch_adj_forward_rec<true>(src, uo, np, o, IBox{0, 0, L->nx - 1, L->ny - 1}, L->dx, L->dy, dt_fixed,
                                        nullptr, rec, st);
}

// The flux update of U^n alone (before friction and clamp) into lin.
template <bool FAST>
cudaError_t linear_step(const hx_level_f64* L, const double* Un, size_t plane, double* lin, const double* dt_dev,
                        cudaStream_t st) {
    const double* cin[3] = {Un, Un + plane, Un + 2 * plane};
    LevelSrc<double> src = make_src(L, cin, 2);
    Cells3<double> uo;
    for (int k = 0; k < 3; ++k) uo.p[k] = cin[k];
    uo.js = L->pitch; uo.lo0 = 0; uo.lo1 = 0;
    Cells3W<double> o;
    for (int k = 0; k < 3; ++k) o.p[k] = lin + k * plane;
    o.js = L->pitch; o.lo0 = 0; o.lo1 = 0;
    Plane<double> np{L->n, L->pitch, 0, 0};
    return launch_adj_forward_linear<FAST>(src, uo, np, o, IBox{0, 0, L->nx - 1, L->ny - 1}, L->dx, L->dy, dt_dev, st);
}

template <bool FAST>
int adjoint_forward(const hx_level_f64* L, int nsteps, double cfl, int ngauges, const int64_t* gauges, double* series,
                    int checkpoint_every, void* work, uint32_t* status, cudaStream_t st) {
    const AdjLayout A = adj_layout(L->nx, L->ny, L->pitch, nsteps, checkpoint_every);
    Views V{static_cast<double*>(work), A.plane};
    char* base = static_cast<char*>(work);
    DtAccum* slot = reinterpret_cast<DtAccum*>(base + A.slots);
    unsigned* pfl = reinterpret_cast<unsigned*>(base + A.pflags);
    double* dth = reinterpret_cast<double*>(base + A.dthist);
    unsigned* stw = status ? status : reinterpret_cast<unsigned*>(base + A.status);
    const size_t pb = A.plane * sizeof(double);
    cudaError_t e = cudaMemsetAsync(base + A.slots, 0, 512, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(pfl, 0, (size_t)nsteps * sizeof(unsigned), st);
    // state 0 into its slot
    double* s0 = V.state(A.states, 0);
    const double* src0[3] = {L->h, L->hu, L->hv};
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemcpy2DAsync(s0 + k * A.plane, L->pitch * sizeof(double), src0[k], L->pitch * sizeof(double),
                              L->nx * sizeof(double), L->ny, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    {
        Cells3<double> U;
        U.p[0] = s0; U.p[1] = s0 + A.plane; U.p[2] = s0 + 2 * A.plane;
        U.js = L->pitch; U.lo0 = 0; U.lo1 = 0;
        Plane<double> Z{L->z, L->pitch, 0, 0};
        e = launch_dt_reduce<double, FAST>(U, Z, IBox{0, 0, L->nx - 1, L->ny - 1}, L->dx, L->dy, &slot[0], st);
        if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    }
    int launches = 1;
    // binomial: the schedule's first snapshots, taken as the sweep passes them (slot k + 1 for chain[k])
    const std::vector<long long> chain = A.binom ? binom_chain(nsteps, A.binom) : std::vector<long long>();
    size_t next_snap = 0;
    for (int n = 0; n < nsteps; ++n) {
        double *in[3], *out[3];
        double* a;
        double* b;
        if (!A.seg && !A.binom) {
            a = V.state(A.states, n);
            b = V.state(A.states, n + 1);
        } else {
            a = n == 0 ? s0 : V.state(A.tmp, n % 2);
            b = V.state(A.tmp, (n + 1) % 2);
        }
        for (int k = 0; k < 3; ++k) { in[k] = a + k * A.plane; out[k] = b + k * A.plane; }
        StepCtl<double> ctl;
        ctl.dt_host = 0.0; ctl.cfl = cfl;
        ctl.dt_in = &slot[n % 3]; ctl.dt_out = n + 1 < nsteps ? &slot[(n + 1) % 3] : nullptr;
        ctl.dt_reset = &slot[(n + 2) % 3];
        ctl.status = stw; ctl.time = nullptr; ctl.dx = L->dx; ctl.dy = L->dy;
        AdjRecord rec{&dth[n], (series && n >= 1) ? series + (size_t)(n - 1) * ngauges : nullptr,
                      (const long long*)gauges, ngauges};
        e = forward_step<FAST>(L, in, out, ctl, nullptr, &pfl[n], rec, st);
        if (e == cudaSuccess && n == nsteps - 1 && series && ngauges > 0) {  // gauges of the final state
            k_adj_series<<<1, 64, 0, st>>>(out[0], ngauges, (const long long*)gauges,
                                           series + (size_t)n * ngauges);
            e = cudaGetLastError();
            ++launches;
        }
        ++launches;
        if (e == cudaSuccess && A.seg && (n + 1) % A.seg == 0) {
            double* ck = V.state(A.states, (n + 1) / A.seg);
            e = cudaMemcpyAsync(ck, b, 3 * pb, cudaMemcpyDeviceToDevice, st);
        }
        if (e == cudaSuccess && A.binom) {
            if (next_snap < chain.size() && chain[next_snap] == n + 1) {
                e = cudaMemcpyAsync(V.state(A.states, (int)next_snap + 1), b, 3 * pb, cudaMemcpyDeviceToDevice, st);
                ++next_snap;
            }
            if (e == cudaSuccess && n == nsteps - 1)  // U^N: the reverse sweep starts from it
                e = cudaMemcpyAsync(V.state(A.nxt, 0), b, 3 * pb, cudaMemcpyDeviceToDevice, st);
        }
        if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    }
    note_launches(launches);
    return HX_OK;
}

// Faces-kernel arguments for the reverse of step n (U^n at Un; un1 = U^{n+1}
// when lambda_lin = lambda^{n+1}, else null).
AdjArgs faces_args(const hx_level_f64* L, const AdjLayout& A, char* base, const double* Un, const double* un1,
                   const double* lam, double* out, double* zbar, double dt) {
    AdjArgs B;
    const double* cin[3] = {Un, Un + A.plane, Un + 2 * A.plane};
    B.src = make_src(L, cin, 2);
    for (int k = 0; k < 3; ++k) {
        B.lam[k] = lam + k * A.plane;
        B.out[k] = out + k * A.plane;
        B.un1[k] = un1 ? un1 + k * A.plane : nullptr;
    }
    B.zbar = zbar; B.pitch = L->pitch; B.nx = L->nx; B.ny = L->ny;
    B.cx = dt / L->dx; B.cy = dt / L->dy;
    B.dx = L->dx; B.dy = L->dy; B.idx = 1.0 / L->dx; B.idy = 1.0 / L->dy; B.idt = 1.0 / dt;
    B.p_dt = reinterpret_cast<double*>(base + A.part);
    B.p_rate = B.p_dt + A.nblocks;
    B.p_idx = reinterpret_cast<long long*>(B.p_rate + A.nblocks);
    B.p_fl = reinterpret_cast<unsigned*>(B.p_idx + A.nblocks);
    return B;
}

// A second stream and its events, released when the reverse sweep returns
// (destruction is deferred by the runtime until queued work completes).
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t rec[2] = {nullptr, nullptr}, freed[2] = {nullptr, nullptr}, start = nullptr;
    cudaError_t init() {
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&rec[k], cudaEventDisableTiming);
        for (int k = 0; k < 2 && e == cudaSuccess; ++k)
            e = cudaEventCreateWithFlags(&freed[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&start, cudaEventDisableTiming);
        return e;
    }
    ~SideStream() {
        for (int k = 0; k < 2; ++k) {
            if (rec[k]) cudaEventDestroy(rec[k]);
            if (freed[k]) cudaEventDestroy(freed[k]);
        }
        if (start) cudaEventDestroy(start);
        if (s) cudaStreamDestroy(s);
    }
};

// Reverse sweep under the binomial schedule.  Snapshot slots hold states;
// U^{n+1} of the step being reversed is kept in the nxt buffer (it was the
// state of the step reversed just before), so every reverse step uses the
// same kernels as with all states stored.
template <bool FAST>
int adjoint_reverse_binomial(const hx_level_f64* L, int nsteps, double cfl, int ngauges, const int64_t* gauges,
                             const double* href, double seed, void* work, const AdjLayout& A, double* const* grad,
                             double* grad_z, cudaStream_t st) {
    Views V{static_cast<double*>(work), A.plane};
    char* base = static_cast<char*>(work);
    const size_t pb = A.plane * sizeof(double);
    double* dth = reinterpret_cast<double*>(base + A.dthist);
    unsigned* pfl = reinterpret_cast<unsigned*>(base + A.pflags);
    const AdjArgs P0 = faces_args(L, A, base, V.state(A.states, 0), nullptr, grad_z, grad_z, grad_z, 1.0);
    const long long* gcells = reinterpret_cast<const long long*>(gauges);
    std::vector<unsigned> pf_host((size_t)nsteps);
    std::vector<double> dt_host((size_t)nsteps);
    cudaError_t e = cudaMemcpyAsync(dt_host.data(), dth, nsteps * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pf_host.data(), pfl, nsteps * sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_z, 0, pb, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + A.done, 0, sizeof(unsigned), st);
    double* lamb[2] = {V.state(A.lam, 0), V.state(A.lam, 1)};
    if (e == cudaSuccess) e = cudaMemsetAsync(lamb[0], 0, 3 * pb, st);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_adj_faces<FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(AdjSmem));
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    const IBox vb{0, 0, L->nx - 1, L->ny - 1};
    const dim3 grid = tile_grid(vb, ATX, ATY);
    double* nxt = V.state(A.nxt, 0);
    double* tmp[3] = {V.state(A.tmp, 0), V.state(A.tmp, 1), V.state(A.tmp, 2)};
    int cur = 0, launches = 0;

    auto finish = [&](int n, const double* Un, double* lam, int with_dt) {
        const double* series_ref = n >= 1 ? href + (size_t)(n - 1) * ngauges : nullptr;
        k_adj_finish<<<1, ANT, 0, st>>>(A.nblocks, P0.p_dt, P0.p_rate, P0.p_idx, P0.p_fl, cfl, L->dx, L->dy, Un,
                                        Un + A.plane, Un + 2 * A.plane, lam, lam + A.plane, lam + 2 * A.plane, with_dt,
                                        n >= 1 ? ngauges : 0, gcells, series_ref, seed);
        ++launches;
        return cudaGetLastError();
    };
    // the reverse kernel's own finish of step n (with the dt term)
    auto fused_finish = [&](AdjArgs& B, int n) {
        B.done = reinterpret_cast<unsigned*>(base + A.done);
        B.cfl = cfl; B.seed = seed;
        B.ngauges = n >= 1 ? ngauges : 0;
        B.gauges = gcells;
        B.href = n >= 1 ? href + (size_t)(n - 1) * ngauges : nullptr;
    };
    // forward from state a (in src) to state m into dst, with the recorded dt
    auto advance = [&](long long a, const double* src, long long m, double* dst) -> cudaError_t {
        cudaError_t r = cudaSuccess;
        const double* from = src;
        for (long long n = a; n < m && r == cudaSuccess; ++n) {
            double* to = (n == m - 1) ? dst : tmp[(n - a) & 1];
            double *in[3], *out[3];
            for (int k = 0; k < 3; ++k) {
                in[k] = const_cast<double*>(from) + k * A.plane;
                out[k] = to + k * A.plane;
            }
            StepCtl<double> ctl{};
            ctl.dx = L->dx; ctl.dy = L->dy;
            r = forward_step<FAST>(L, in, out, ctl, &dth[n], nullptr, AdjRecord{}, st);
            ++launches;
            from = to;
        }
        return r;
    };
    // reverse step j from U^j (in Uj) and U^{j+1} (in nxt); then U^j becomes the next step's U^{j+1}
    auto leaf = [&](long long j, const double* Uj) -> cudaError_t {
        const double dt = dt_host[(size_t)j];
        double* lam1 = lamb[cur];
        double* lam0 = lamb[cur ^ 1];
        const double* lam_for_faces = lam1;
        const double* un1 = nxt;
        cudaError_t r = cudaSuccess;
        if (pf_host[(size_t)j]) {
            double* lin = V.state(A.lin, 0);
            double* ll = V.state(A.lamlin, 0);
            r = linear_step<FAST>(L, Uj, A.plane, lin, &dth[j], st);
            PostArgs P;
            for (int k = 0; k < 3; ++k) {
                P.lin[k] = lin + k * A.plane; P.un[k] = Uj + k * A.plane; P.lam[k] = lam1 + k * A.plane;
                P.out[k] = ll + k * A.plane;
            }
            P.nman = L->n; P.dtbar = P0.p_dt; P.pitch = L->pitch; P.nx = L->nx; P.ny = L->ny; P.dt = dt;
            k_adj_post<<<grid, ANT, 0, st>>>(P);
            launches += 2;
            lam_for_faces = ll;
            un1 = nullptr;
        }
        AdjArgs B = faces_args(L, A, base, Uj, un1, lam_for_faces, lam0, grad_z, dt);
        fused_finish(B, (int)j);
        k_adj_faces<FAST><<<grid, ANT, sizeof(AdjSmem), st>>>(B);
        ++launches;
        if (r == cudaSuccess) r = cudaGetLastError();
        if (r == cudaSuccess && j > 0) r = cudaMemcpyAsync(nxt, Uj, 3 * pb, cudaMemcpyDeviceToDevice, st);
        cur ^= 1;
        return r;
    };
    // slots: 0 holds U^0; the forward sweep left chain[k] in slot k + 1
    std::vector<long long> slot_pos((size_t)A.binom, -1);
    slot_pos[0] = 0;
    const std::vector<long long> chain = binom_chain(nsteps, A.binom);
    for (size_t k = 0; k < chain.size(); ++k) slot_pos[k + 1] = chain[k];
    std::vector<int> pool;  // free slots, taken from the back
    for (int k = A.binom - 1; k >= 1; --k) pool.push_back(k);
    std::function<cudaError_t(long long, long long, int)> rev = [&](long long a, long long b, int slot_a) {
        const double* Ua = V.state(A.states, slot_a);
        if (b - a == 1) return leaf(a, Ua);
        if (pool.empty()) {  // no free slot: recompute each state from U^a
            for (long long j = b - 1; j >= a; --j) {
                cudaError_t r = j == a ? cudaSuccess : advance(a, Ua, j, tmp[2]);
                if (r == cudaSuccess) r = leaf(j, j == a ? Ua : tmp[2]);
                if (r != cudaSuccess) return r;
            }
            return cudaSuccess;
        }
        const long long m = a + binom_split(b - a, (int)pool.size() + 1);
        const int slot_m = pool.back();
        pool.pop_back();
        cudaError_t r = cudaSuccess;
        if (slot_pos[(size_t)slot_m] != m) {
            r = advance(a, Ua, m, V.state(A.states, slot_m));
            slot_pos[(size_t)slot_m] = m;
        }
        if (r == cudaSuccess) r = rev(m, b, slot_m);
        pool.push_back(slot_m);
        if (r == cudaSuccess) r = rev(a, m, slot_a);
        return r;
    };
    e = finish(nsteps, nxt, lamb[cur], 0);  // lambda^N: the misfit of the final state
    if (e == cudaSuccess) e = rev(0, nsteps, 0);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemcpyAsync(grad[k], lamb[cur] + k * A.plane, pb, cudaMemcpyDeviceToDevice, st);
    note_launches(launches);
    if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    return HX_OK;
}

template <bool FAST>
int adjoint_reverse(const hx_level_f64* L, int nsteps, double cfl, int ngauges, const int64_t* gauges,
                    const double* href, double seed, int checkpoint_every, bool records, void* work, double* grad_h,
                    double* grad_hu, double* grad_hv, double* grad_z, cudaStream_t st) {
    const AdjLayout A = adj_layout(L->nx, L->ny, L->pitch, nsteps, checkpoint_every, FAST && records);
    const bool use_rec = A.rec_step != 0;  // uniform checkpoints, fast form, records requested
    if (A.binom) {
        double* grad[3] = {grad_h, grad_hu, grad_hv};
        return adjoint_reverse_binomial<FAST>(L, nsteps, cfl, ngauges, gauges, href, seed, work, A, grad, grad_z, st);
    }
    Views V{static_cast<double*>(work), A.plane};
    char* base = static_cast<char*>(work);
    const size_t pb = A.plane * sizeof(double);
    double* dth = reinterpret_cast<double*>(base + A.dthist);
    unsigned* pfl = reinterpret_cast<unsigned*>(base + A.pflags);
    const AdjArgs P0 = faces_args(L, A, base, V.state(A.states, 0), nullptr, grad_h, grad_h, grad_z, 1.0);
    const long long* gcells = reinterpret_cast<const long long*>(gauges);

    std::vector<double> dt_host((size_t)nsteps);
    std::vector<unsigned> pf_host((size_t)nsteps);
    cudaError_t e = cudaMemcpyAsync(dt_host.data(), dth, nsteps * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pf_host.data(), pfl, nsteps * sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_z, 0, pb, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + A.done, 0, sizeof(unsigned), st);
    double* lamb[2] = {V.state(A.lam, 0), V.state(A.lam, 1)};
    if (e == cudaSuccess) e = cudaMemsetAsync(lamb[0], 0, 3 * pb, st);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_adj_faces<FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(AdjSmem));
    if constexpr (FAST) {
        if (e == cudaSuccess && use_rec)
            e = cudaFuncSetAttribute(k_adj_faces<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(AdjSmem));
    }
    SideStream side;
    if (e == cudaSuccess && A.seg) e = side.init();
    if (e == cudaSuccess && A.seg) e = cudaEventRecord(side.start, st);
    if (e == cudaSuccess && A.seg) e = cudaStreamWaitEvent(side.s, side.start, 0);
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    int cur = 0;  // lamb[cur] holds lambda^{n+1}
    const IBox vb{0, 0, L->nx - 1, L->ny - 1};
    const dim3 grid = tile_grid(vb, ATX, ATY);
    int launches = 0;

    auto finish = [&](int n, const double* Un, double* lam, int with_dt) {
        const double* series_ref = n >= 1 ? href + (size_t)(n - 1) * ngauges : nullptr;
        k_adj_finish<<<1, ANT, 0, st>>>(A.nblocks, P0.p_dt, P0.p_rate, P0.p_idx, P0.p_fl, cfl, L->dx, L->dy, Un,
                                        Un + A.plane, Un + 2 * A.plane, lam, lam + A.plane, lam + 2 * A.plane, with_dt,
                                        n >= 1 ? ngauges : 0, gcells, series_ref, seed);
        ++launches;
        return cudaGetLastError();
    };
    // the reverse kernel's own finish of step n (with the dt term)
    auto fused_finish = [&](AdjArgs& B, int n) {
        B.done = reinterpret_cast<unsigned*>(base + A.done);
        B.cfl = cfl; B.seed = seed;
        B.ngauges = n >= 1 ? ngauges : 0;
        B.gauges = gcells;
        B.href = n >= 1 ? href + (size_t)(n - 1) * ngauges : nullptr;
    };
    const int L_seg = A.seg ? A.seg : nsteps;
    const int nseg = (nsteps + L_seg - 1) / L_seg;
    auto segstate = [&](int sg, int k) { return V.state(A.segbuf + (size_t)(sg & 1) * A.segbuf_stride, k); };
    auto state_at = [&](int sg, int n) -> double* {
        if (!A.seg) return V.state(A.states, n);
        return segstate(sg, n - sg * L_seg);
    };
    // Recompute segment sg's states from its checkpoint with the recorded dt, on the side stream, into the
    // segment buffer of its parity; the reverse of segment sg + 1 runs meanwhile on st.
    auto recompute = [&](int sg) -> cudaError_t {
        const int n0 = sg * L_seg, n1 = (n0 + L_seg < nsteps) ? n0 + L_seg : nsteps;
        cudaError_t r = cudaMemcpyAsync(segstate(sg, 0), V.state(A.states, sg), 3 * pb, cudaMemcpyDeviceToDevice,
                                        side.s);
        for (int n = n0; n < n1 && r == cudaSuccess; ++n) {
            double* a = segstate(sg, n - n0);
            double* b = segstate(sg, n - n0 + 1);
            double *in[3], *out[3];
            for (int k = 0; k < 3; ++k) { in[k] = a + k * A.plane; out[k] = b + k * A.plane; }
            if (use_rec) {
                r = forward_step_rec(L, in, out, &dth[n], rec_at(A, base, (sg & 1) * L_seg + (n - n0), L->nx, L->ny),
                                     side.s);
            } else {
                StepCtl<double> ctl{};
                ctl.dx = L->dx; ctl.dy = L->dy;
                r = forward_step<FAST>(L, in, out, ctl, &dth[n], nullptr, AdjRecord{}, side.s);
            }
            ++launches;
        }
        if (r == cudaSuccess) r = cudaEventRecord(side.rec[sg & 1], side.s);
        return r;
    };
    if (A.seg) e = recompute(nseg - 1);
    bool first = true;
    for (int sg = nseg - 1; sg >= 0 && e == cudaSuccess; --sg) {
        const int n0 = sg * L_seg, n1 = (n0 + L_seg < nsteps) ? n0 + L_seg : nsteps;
        if (A.seg) {
            e = cudaStreamWaitEvent(st, side.rec[sg & 1], 0);
            if (e == cudaSuccess && sg >= 1) {  // the buffer of segment sg - 1 was last read by segment sg + 1
                if (sg + 1 < nseg) e = cudaStreamWaitEvent(side.s, side.freed[(sg + 1) & 1], 0);
                if (e == cudaSuccess) e = recompute(sg - 1);
            }
            if (e != cudaSuccess) break;
        }
        if (first) {  // lambda^N: the misfit of the final state
            e = finish(nsteps, state_at(sg, nsteps), lamb[cur], 0);
            first = false;
        }
        for (int n = n1 - 1; n >= n0 && e == cudaSuccess; --n) {
            double* Un = state_at(sg, n);
            double* Un1 = state_at(sg, n + 1);
            const double dt = dt_host[(size_t)n];
            double* lam1 = lamb[cur];
            double* lam0 = lamb[cur ^ 1];
            const double* lam_for_faces = lam1;
            const double* un1 = Un1;
            if (pf_host[(size_t)n]) {  // friction or dry clamp in this step: reverse the post map
                double* lin = V.state(A.lin, 0);
                double* ll = V.state(A.lamlin, 0);
                e = linear_step<FAST>(L, Un, A.plane, lin, &dth[n], st);
                PostArgs P;
                for (int k = 0; k < 3; ++k) {
                    P.lin[k] = lin + k * A.plane; P.un[k] = Un + k * A.plane; P.lam[k] = lam1 + k * A.plane;
                    P.out[k] = ll + k * A.plane;
                }
                P.nman = L->n; P.dtbar = P0.p_dt; P.pitch = L->pitch; P.nx = L->nx; P.ny = L->ny; P.dt = dt;
                k_adj_post<<<grid, ANT, 0, st>>>(P);
                launches += 2;
                lam_for_faces = ll;
                un1 = nullptr;  // the post kernel wrote the dt partials
            }
            AdjArgs B = faces_args(L, A, base, Un, un1, lam_for_faces, lam0, grad_z, dt);
            fused_finish(B, n);
            if constexpr (FAST) {
                if (use_rec) {
                    B.rec = rec_at(A, base, (sg & 1) * L_seg + (n - n0), L->nx, L->ny);
                    k_adj_faces<true, true><<<grid, ANT, sizeof(AdjSmem), st>>>(B);
                } else {
                    k_adj_faces<FAST><<<grid, ANT, sizeof(AdjSmem), st>>>(B);
                }
            } else {
                k_adj_faces<FAST><<<grid, ANT, sizeof(AdjSmem), st>>>(B);
            }
            ++launches;
            if (e == cudaSuccess) e = cudaGetLastError();
            cur ^= 1;
        }
        if (A.seg && e == cudaSuccess) e = cudaEventRecord(side.freed[sg & 1], st);
    }
    if (e == cudaSuccess) {
        double* g[3] = {grad_h, grad_hu, grad_hv};
        for (int k = 0; k < 3 && e == cudaSuccess; ++k)
            e = cudaMemcpyAsync(g[k], lamb[cur] + k * A.plane, pb, cudaMemcpyDeviceToDevice, st);
    }
    if (e != cudaSuccess && A.seg) {  // nothing may still run on the side stream when the buffers go back
        cudaStreamSynchronize(side.s);
        cudaStreamSynchronize(st);
    }
    note_launches(launches);
    if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    return HX_OK;
}

template <bool FAST>
int adjoint_step(const hx_level_f64* L, double dt, const double* const* lam, double* const* outs, double* zbar,
                 double* dtbar, void* work, cudaStream_t st) {
    const AdjLayout A = adj_layout(L->nx, L->ny, L->pitch, 1, 0);
    char* base = static_cast<char*>(work);
    Views V{static_cast<double*>(work), A.plane};
    double* p_dt = reinterpret_cast<double*>(base + A.part);
    double* dth = reinterpret_cast<double*>(base + A.dthist);
    double* lin = V.state(A.lin, 0);
    double* ll = V.state(A.lamlin, 0);
    double* un = V.state(A.states, 0);  // U^n copied to the work layout (pitch of the level)
    const IBox vb{0, 0, L->nx - 1, L->ny - 1};
    const dim3 grid = tile_grid(vb, ATX, ATY);
    const double* src0[3] = {L->h, L->hu, L->hv};
    cudaError_t e = cudaMemcpyAsync(dth, &dt, sizeof(double), cudaMemcpyHostToDevice, st);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemcpy2DAsync(un + k * A.plane, L->pitch * sizeof(double), src0[k], L->pitch * sizeof(double),
                              L->nx * sizeof(double), L->ny, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_adj_faces<FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(AdjSmem));
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    e = linear_step<FAST>(L, un, A.plane, lin, dth, st);
    if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    PostArgs P;
    for (int k = 0; k < 3; ++k) {
        P.lin[k] = lin + k * A.plane; P.un[k] = un + k * A.plane; P.lam[k] = lam[k]; P.out[k] = ll + k * A.plane;
    }
    P.nman = L->n; P.dtbar = p_dt; P.pitch = L->pitch; P.nx = L->nx; P.ny = L->ny; P.dt = dt;
    k_adj_post<<<grid, ANT, 0, st>>>(P);
    AdjArgs B = faces_args(L, A, base, un, nullptr, ll, ll, zbar, dt);  // outputs replaced below
    for (int k = 0; k < 3; ++k) B.out[k] = outs[k];
    k_adj_faces<FAST><<<grid, ANT, sizeof(AdjSmem), st>>>(B);
    e = cudaGetLastError();
    if (e == cudaSuccess) {  // dtbar = sum of the per-block partials
        std::vector<double> parts((size_t)A.nblocks);
        e = cudaMemcpyAsync(parts.data(), p_dt, parts.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        double sum = 0;
        for (double x : parts) sum += x;
        if (e == cudaSuccess) e = cudaMemcpyAsync(dtbar, &sum, sizeof(double), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    note_launches(3);
    if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    return HX_OK;
}

bool arith_ok(int arith) { return arith == HX_ARITH_EXACT || arith == HX_ARITH_FAST; }

}  // namespace

extern "C" int64_t hx_adjoint_recompute_steps(int nsteps, int checkpoint_every) {
    if (nsteps < 1) return -1;
    if (checkpoint_every > 0) return checkpoint_every < nsteps ? nsteps : 0;
    if (checkpoint_every == 0) return 0;
    int c = -checkpoint_every < nsteps + 1 ? -checkpoint_every : nsteps + 1;
    if (c < 2) c = 2;
    const std::vector<long long> chain = binom_chain(nsteps, c);  // advanced by the forward sweep already
    return binom_cost(nsteps, c) - (chain.empty() ? 0 : chain.back());
}

extern "C" int64_t hx_adjoint_work_bytes_f64(int nx, int ny, int64_t pitch, int nsteps, int checkpoint_every,
                                             int options) {
    if (nx < 2 || ny < 2 || pitch < nx || nsteps < 1 || (options & ~HX_ADJ_FACE_RECORDS)) return 0;
    return (int64_t)adj_layout(nx, ny, pitch, nsteps, checkpoint_every, (options & HX_ADJ_FACE_RECORDS) != 0).total;
}

extern "C" int hx_adjoint_forward_f64(const hx_level_f64* L, int nsteps, double cfl, int ngauges,
                                      const int64_t* gauges, double* series, int checkpoint_every, int arith,
                                      void* work, uint32_t* status, hx_stream_t stream) {
    int rc = adj_check(L, nsteps, ngauges, gauges);
    if (rc) return rc;
    arith &= ~HX_ADJ_FACE_RECORDS;  // the forward sweep writes no records
    if (!work || !(cfl > 0) || (ngauges > 0 && !series) || !arith_ok(arith))
        return set_error(HX_ERR_ARG, "adjoint forward: bad arguments");
    return arith == HX_ARITH_FAST
               ? adjoint_forward<true>(L, nsteps, cfl, ngauges, gauges, series, checkpoint_every, work, status,
                                       (cudaStream_t)stream)
               : adjoint_forward<false>(L, nsteps, cfl, ngauges, gauges, series, checkpoint_every, work, status,
                                        (cudaStream_t)stream);
}

extern "C" int hx_adjoint_reverse_f64(const hx_level_f64* L, int nsteps, double cfl, int ngauges,
                                      const int64_t* gauges, const double* href, double seed, int checkpoint_every,
                                      int arith, void* work, double* grad_h, double* grad_hu, double* grad_hv,
                                      double* grad_z, hx_stream_t stream) {
    int rc = adj_check(L, nsteps, ngauges, gauges);
    if (rc) return rc;
    const bool records = (arith & HX_ADJ_FACE_RECORDS) != 0;
    arith &= ~HX_ADJ_FACE_RECORDS;
    if (!work || !grad_h || !grad_hu || !grad_hv || !grad_z || (ngauges > 0 && !href) || !arith_ok(arith))
        return set_error(HX_ERR_ARG, "adjoint reverse: bad arguments");
    return arith == HX_ARITH_FAST
               ? adjoint_reverse<true>(L, nsteps, cfl, ngauges, gauges, href, seed, checkpoint_every, records, work,
                                       grad_h, grad_hu, grad_hv, grad_z, (cudaStream_t)stream)
               : adjoint_reverse<false>(L, nsteps, cfl, ngauges, gauges, href, seed, checkpoint_every, records, work,
                                        grad_h, grad_hu, grad_hv, grad_z, (cudaStream_t)stream);
}

// One reverse step with a given dt (no CFL dependence, no gauges): the
// transpose of the step map (U^n, z) -> U^{n+1} at fixed dt, plus d/d dt.
extern "C" int hx_adjoint_step_f64(const hx_level_f64* L, double dt, const double* lam_h, const double* lam_hu,
                                   const double* lam_hv, double* out_h, double* out_hu, double* out_hv,
                                   double* zbar, double* dtbar, int arith, void* work, hx_stream_t stream) {
    int rc = adj_check(L, 1, 0, nullptr);
    if (rc) return rc;
    if (!lam_h || !lam_hu || !lam_hv || !out_h || !out_hu || !out_hv || !zbar || !dtbar || !work || !(dt > 0) ||
        !arith_ok(arith))
        return set_error(HX_ERR_ARG, "hx_adjoint_step_f64: bad arguments");
    const double* lam[3] = {lam_h, lam_hu, lam_hv};
    double* outs[3] = {out_h, out_hu, out_hv};
    return arith == HX_ARITH_FAST ? adjoint_step<true>(L, dt, lam, outs, zbar, dtbar, work, (cudaStream_t)stream)
                                  : adjoint_step<false>(L, dt, lam, outs, zbar, dtbar, work, (cudaStream_t)stream);
}
