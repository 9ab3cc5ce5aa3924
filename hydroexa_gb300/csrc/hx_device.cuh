// Device building blocks of the GB300 per-level advance: constants, point
// Riemann solvers, limiter, ghost rules and the dt accumulator.
//
// Two arithmetic forms of every formula:
//   FAST == false  repeats the reference's operation order term by term; the
//                  translation unit that instantiates it is compiled with
//                  --fmad=false, so results equal the reference's host
//                  arithmetic bit for bit (sqrt and division are IEEE in both;
//                  only cbrt in the Manning factor may differ by an ulp).
//   FAST == true   same mathematics with shared reciprocals and square roots
//                  and contracted multiply-adds: ~1e-15 relative per step.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/hydroexa_gb300.h"
#include "hx_dual.cuh"

namespace hx {

template <class R> struct Cst;
template <> struct Cst<double> {
    // include/utils/Constants.H:25-78
    static constexpr double g = 9.81;
    static constexpr double half_g = 0.5 * 9.81;
    static constexpr double sqrt_g = 3.1320919526731650;  // sqrt(9.81), correctly rounded
    static constexpr double toldry = 1e-6;
    static constexpr double tol12 = 1e-12;
    static constexpr double tol10 = 1e-10;
    // IEEE bit patterns of the positive tolerances (for integer comparisons)
    static constexpr long long toldry_bits = 0x3eb0c6f7a0b5ed8dll;
    static constexpr long long tol12_bits = 0x3d719799812dea11ll;
    static constexpr long long toldry2_bits = 0x3ec0c6f7a0b5ed8dll;  // 2 toldry
    static constexpr double g_toldry = 9.81 * 1e-6;                  // g toldry, rounded once
    static constexpr double max_value = 1.7976931348623157e308;  // std::numeric_limits<double>::max()
};
template <> struct Cst<float> {
    static constexpr float g = 9.81f;
    static constexpr float half_g = 0.5f * 9.81f;
    static constexpr float sqrt_g = 3.13209195f;
    static constexpr float toldry = 1e-6f;
    static constexpr float tol12 = 1e-12f;
    static constexpr float tol10 = 1e-10f;
    static constexpr int toldry_bits = 0x358637bd;
    static constexpr int tol12_bits = 0x2b8cbccc;
    static constexpr int toldry2_bits = 0x360637bd;
    static constexpr float g_toldry = 9.81f * 1e-6f;
    static constexpr float max_value = 3.40282347e38f;  // std::numeric_limits<float>::max()
};

template <> struct Cst<Dual> {
    static constexpr Dual g = Dual(9.81);
    static constexpr Dual half_g = Dual(0.5 * 9.81);
    static constexpr Dual sqrt_g = Dual(3.1320919526731650);
    static constexpr Dual toldry = Dual(1e-6);
    static constexpr Dual tol12 = Dual(1e-12);
    static constexpr Dual tol10 = Dual(1e-10);
};

// std::max(0, x) of the reference: (0 < x) ? x : 0 (NaN -> 0).
template <class R> __host__ __device__ __forceinline__ R max0(R x) { return (R(0) < x) ? x : R(0); }
template <class R> __host__ __device__ __forceinline__ R smax(R a, R b) { return (a < b) ? b : a; }

// NODATA predicate of the hydrostatic face kernel and compute_dt_Impl
// (HydrostaticRoe.cpp:41,238): |z + 9999| < 1e-10, evaluated in double as the
// reference's literal -9999.0 forces.  Generic form (dual numbers); double and
// float have integer forms below.
template <class R> __host__ __device__ __forceinline__ bool is_nodata(R z) {
    return fabs((double)z + 9999.0) < 1e-10;
}

template <class R> __device__ __forceinline__ bool bits_nonfinite(R x);
template <> __device__ __forceinline__ bool bits_nonfinite<double>(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7FF0000000000000ull) == 0x7FF0000000000000ull;
}
template <> __device__ __forceinline__ bool bits_nonfinite<float>(float x) {
    return ((unsigned)__float_as_uint(x) & 0x7F800000u) == 0x7F800000u;
}
template <> __device__ __forceinline__ bool bits_nonfinite<Dual>(Dual x) {
    return bits_nonfinite<double>(x.v) || bits_nonfinite<double>(x.d);
}

// ----------------------------------------------------------------------------
// Comparisons on IEEE bit patterns.  On GB300 a double-precision compare,
// min or max issues on the scarce FP64 pipe; the same decision taken on the
// integer pipe is free by comparison.  For non-NaN x:
//   x > c  (c > 0)   <=>  bits(x) > bits(c) as signed integers
//   x > 0            <=>  bits(x) > 0           (+0 and -0 are not > 0)
//   x < 0            <=>  bits(x) > sign bit as unsigned (-0 is not < 0)
// and okey() maps doubles to integers with the same order (for max of signed
// values).  Used by the fast form only; NaN inputs are flagged separately.
// ----------------------------------------------------------------------------
__host__ __device__ __forceinline__ long long sbits(double x) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    long long b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}
__host__ __device__ __forceinline__ int sbits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_int(x);
#else
    int b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}
// is_nodata on the bit pattern.  A double z with |z + 9999| < 1e-10 lies in
// [-19998, -4999.5], where z + 9999 is exact (Sterbenz), and there the doubles
// are spaced 2^-39 apart; 1e-10 / 2^-39 = 54.98, so the predicate holds exactly
// for the 109 doubles -9999 + k 2^-39, |k| <= 54, whose patterns are
// bits(-9999.0) + k.  One integer range check replaces an FP64 add and compare.
// A float converted to double and added to 9999 is exact too, and the float
// spacing near 9999 (2^-10) leaves -9999.0f as the only float that qualifies.
__host__ __device__ __forceinline__ bool is_nodata(double z) {
    return (unsigned long long)sbits(z) - (0xC0C3878000000000ull - 54ull) <= 108ull;
}
__host__ __device__ __forceinline__ bool is_nodata(float z) { return sbits(z) == (int)0xC61C3C00u; }

// The leading 24 significand bits of a double as a float (truncated, so within
// 2^-23 relative; 0 below the float range, inf above, NaN kept as NaN or inf),
// made on the integer pipe: for decisions whose outcome is certain at that
// precision, taken without FP64 instructions.
__host__ __device__ __forceinline__ float f32_lead(double x) {
    const unsigned long long b = (unsigned long long)sbits(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int de = (int)((hi >> 20) & 0x7FF);
    const unsigned sign = hi & 0x80000000u, mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const int fe = de - 1023 + 127;
    unsigned f;
    if (de == 0x7FF) f = sign | 0x7F800000u | mant;
    else if (fe >= 255) f = sign | 0x7F800000u;
    else if (fe <= 0) f = sign;
    else f = sign | ((unsigned)fe << 23) | mant;
    float y;
    memcpy(&y, &f, sizeof y);
    return y;
}

template <class R> __host__ __device__ __forceinline__ bool gt_bits(R x, decltype(sbits(R(0))) cb) {
    return sbits(x) > cb;
}
template <class R> __host__ __device__ __forceinline__ bool ge_bits(R x, decltype(sbits(R(0))) cb) {
    return sbits(x) >= cb;
}
template <class R> __host__ __device__ __forceinline__ bool pos_i(R x) { return sbits(x) > 0; }
__host__ __device__ __forceinline__ bool neg_i(double x) {
    return (unsigned long long)sbits(x) > 0x8000000000000000ull;
}
__host__ __device__ __forceinline__ bool neg_i(float x) { return (unsigned)sbits(x) > 0x80000000u; }
template <class R> __host__ __device__ __forceinline__ R max0_i(R x) { return pos_i(x) ? x : R(0); }
__host__ __device__ __forceinline__ bool abs_le_bits(double x, long long cb) {
    return (sbits(x) & 0x7FFFFFFFFFFFFFFFll) <= cb;
}
__host__ __device__ __forceinline__ bool abs_le_bits(float x, int cb) { return (sbits(x) & 0x7FFFFFFF) <= cb; }
__host__ __device__ __forceinline__ long long okey(double x) {
    const long long b = sbits(x);
    return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFll);
}
__host__ __device__ __forceinline__ int okey(float x) {
    const int b = sbits(x);
    return b >= 0 ? b : (b ^ 0x7FFFFFFF);
}
// std::max(a, b) = (a < b) ? b : a
template <class R> __host__ __device__ __forceinline__ R smax_i(R a, R b) { return okey(a) < okey(b) ? b : a; }
// max of two non-negative values
template <class R> __host__ __device__ __forceinline__ R nnmax_i(R a, R b) { return sbits(a) < sbits(b) ? b : a; }

// The double holding a normal float exactly, built on the integer pipe.
__host__ __device__ __forceinline__ double f64_widen(float f) {
    const unsigned b = (unsigned)sbits(f);
    const unsigned long long d = ((unsigned long long)(b & 0x80000000u) << 32) |
                                 ((unsigned long long)(((b >> 23) & 0xFFu) + (1023u - 127u)) << 52) |
                                 ((unsigned long long)(b & 0x7FFFFFu) << 29);
    double y;
    memcpy(&y, &d, sizeof y);
    return y;
}
// True when |x| has an exponent well inside the normal float range, so that
// f32_lead(x) is a normal float and its reciprocal / reciprocal square root
// are normal too.
__host__ __device__ __forceinline__ bool in_f32_range(double x) {
    const int e = (int)(((unsigned long long)sbits(x) >> 52) & 0x7FFu) - 1023;
    return e > -120 && e < 120;
}

// FP64 reciprocal and square root of the fast form.  Each starts from a float
// estimate (rcp.approx.ftz.f32 / rsqrt.approx.ftz.f32) of the leading 24
// significand bits, widened to a double on the integer pipe, so only the
// correction steps issue on the FP64 pipe (GB300 issues FP64 at 1/64 of its
// FP32 rate).  The seeds carry a relative error delta below 2^-21.5.
//
// The flux arithmetic takes ONE Newton step, whose error is of order delta^2
// (below 2^-42 relative, typically ~2^-46): two FMAs for 1/x, three FP64
// instructions for sqrt(x).  A face flux built from them differs from the
// IEEE-rounded one by a few parts in 1e14 of its terms, inside the fast form's
// 1e-12-per-step bound with two orders of magnitude to spare, and the rounding
// of the exact form is not what the fast form reproduces anyway.
//
// The CFL rate takes the third-order step (Householder's method of order 3;
// Markstein, IBM J. Res. Dev. 34, 1990, gives the FMA formulation), within an
// ulp: the time step stays that of the exact form to the last few ulps.  It
// runs once per candidate cell of the screened fold, not per face.

// The double of a positive normal float f times 2^k with the sign bit sg, assembled on the integer pipe (the
// exponent field must stay within 1..2046: the callers select another value where it would not).
__device__ __forceinline__ double f64_of_f32_scaled(float f, int k, unsigned sg) {
    const unsigned fb = (unsigned)__float_as_int(f);
    const unsigned hi = sg | ((fb >> 3) + ((unsigned)(896 + k) << 20));
    return __hiloint2double((int)hi, (int)(fb << 29));
}
// Float seed of 1/x for any normal double x below 2^1021 in magnitude: the
// reciprocal of the significand's leading bits (a float in [1, 2)), with the
// exponent and sign put back on the integer pipe.  No branch on the range.
__device__ __forceinline__ double rcp_seed(double x) {
    const unsigned hx = (unsigned)__double2hiint(x), lx = (unsigned)__double2loint(x);
    const int ex = (int)((hx >> 20) & 0x7FFu);
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;"
        : "=f"(rf)
        : "f"(__int_as_float((int)(0x3F800000u | ((hx & 0xFFFFFu) << 3) | (lx >> 29)))));
    return f64_of_f32_scaled(rf, 1023 - ex, hx & 0x80000000u);  // rf in (0.5, 1]
}
// 1/x, one Newton step: y0 (1 + e) with e = 1 - x y0.  Callers pass finite
// normal arguments below 2^1021 in magnitude (depths, wave-speed sums).
__host__ __device__ __forceinline__ double rcp_nr(double x) {
#ifdef __CUDA_ARCH__
    const double y = rcp_seed(x);
    return fma(y, fma(-x, y, 1.0), y);
#else
    return 1.0 / x;
#endif
}
// 1/x within an ulp (the CFL rate): y0 + y0 (e + e^2).
__host__ __device__ __forceinline__ double rcp_fa(double x) {
#ifdef __CUDA_ARCH__
    const double y = rcp_seed(x);
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
#else
    return 1.0 / x;
#endif
}
// Float: the hardware approximation alone (rcp.approx.ftz.f32, within an ulp);
// the FP32 fast form is held to 1e-5 of the oracle in float, and is bound by
// instruction issue, where the IEEE reciprocal's correction steps cost.
__host__ __device__ __forceinline__ float rcp_nr(float x) {
#ifdef __CUDA_ARCH__
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return 1.0f / x;
#endif
}

// sqrt(x) from the estimate r0 of 1/sqrt(x): with t = x r0 and d = 1 - t r0,
// sqrt(x) = t (1 - d)^(-1/2) = t (1 + d/2 + 3 d^2/8 + ...).  One step keeps
// t (1 + d/2) = t (1.5 - t r0/2), the halved seed being exact: three FP64
// instructions, error ~1.5 delta^2.  +0 gives +0 through the same steps (its
// seed is 2^128, finite, from the infinite float estimate), so dry sides do
// not branch off; negative, non-finite and out-of-float-range arguments take
// the IEEE square root.  Float: sqrt.approx.ftz.f32.
__host__ __device__ __forceinline__ double fast_sqrt(double x) {
#ifdef __CUDA_ARCH__
    if (sbits(x) != 0 && (!pos_i(x) || !in_f32_range(x))) return sqrt(x);
    float rf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(f32_lead(x)));
    const double r0 = f64_widen(rf), r0h = f64_widen(rf * 0.5f);
    const double t = x * r0;
    return t * fma(-t, r0h, 1.5);
#else
    return sqrt(x);
#endif
}
// sqrt(x) within about an ulp (the CFL rate): the d^2 term kept, five FP64
// instructions, error ~2.5 delta^3.
__host__ __device__ __forceinline__ double fast_sqrt_fa(double x) {
#ifdef __CUDA_ARCH__
    if (sbits(x) != 0 && (!pos_i(x) || !in_f32_range(x))) return sqrt(x);
    float rf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(f32_lead(x)));
    const double r0 = f64_widen(rf);
    const double t = x * r0;
    const double d = fma(-t, r0, 1.0);
    return fma(t, d * fma(0.375, d, 0.5), t);
#else
    return sqrt(x);
#endif
}
// sqrt(x) as fast_sqrt (same bits) and, for one more multiply, half the
// reciprocal square root 1/(2 sqrt(x)) = (r0/2) (1.5 - t r0/2) from the same
// step.  x must be a positive normal double (a depth above the dry tolerance,
// times g).
__device__ __forceinline__ double fast_sqrt_hrsqrt(double x, double& hrsq) {
    if (!in_f32_range(x)) {
        const double s = sqrt(x);
        hrsq = 0.5 / s;
        return s;
    }
    float rf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(f32_lead(x)));
    const double r0 = f64_widen(rf), r0h = f64_widen(rf * 0.5f);
    const double t = x * r0;
    const double e = fma(-t, r0h, 1.5);
    hrsq = r0h * e;
    return t * e;
}
__host__ __device__ __forceinline__ float fast_sqrt(float x) {
#ifdef __CUDA_ARCH__
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return sqrtf(x);
#endif
}

// h^(-1/3) for a wet depth (a positive normal double within the float range) in the fast form's Manning
// factor: the float seed rcbrtf of its leading 24 bits (within ~2^-22.5 with the truncation), widened on the
// integer pipe, then one Newton step for f(r) = r^-3 - h, r + r (1 - h r^3) / 3, whose error is twice the
// seed's squared (~2^-44): five FP64 instructions where cbrt and a division take several times that.
// Float: rcbrtf alone.
__host__ __device__ __forceinline__ double rcbrt_nr(double h) {
#ifdef __CUDA_ARCH__
    const double r = f64_widen(rcbrtf(f32_lead(h)));
    const double e = fma(-h, r * r * r, 1.0);
    return fma(r * e, 1.0 / 3.0, r);
#else
    return 1.0 / cbrt(h);
#endif
}
__host__ __device__ __forceinline__ float rcbrt_nr(float h) {
#ifdef __CUDA_ARCH__
    return rcbrtf(h);
#else
    return 1.0f / cbrtf(h);
#endif
}

// 2 p / S for p = dm dp > 0 and S = dm + dp (the van Leer slope 2 dm dp / (dm + dp)), S a normal double of
// magnitude below 2^1000.  The seeds come from the leading 24 bits of the two significands, taken as floats
// in [1, 2): rf ~ 1 / mS by rcp.approx.ftz.f32 and hf = mp rf; the exponents are added back on the integer
// pipe, giving s0h ~ p / S, s0 = 2 s0h and r2 ~ 2 / S without FP64 instructions (and without a branch on
// the range of S).  One Newton correction in FP64, s0 + r2 (p - s0h S), leaves the product of the two
// seed errors (each below 2^-21): the slope is within ~2^-42 relative.  Where p / S is below the normal
// range the seed is 0 and r2 p is the result.
__device__ __forceinline__ double van_leer_div2(double p, double S) {
    const unsigned hp = (unsigned)__double2hiint(p), lp = (unsigned)__double2loint(p);
    const unsigned hS = (unsigned)__double2hiint(S), lS = (unsigned)__double2loint(S);
    const int ep = (int)((hp >> 20) & 0x7FFu), eS = (int)((hS >> 20) & 0x7FFu);
    const float mp = __int_as_float((int)(0x3F800000u | ((hp & 0xFFFFFu) << 3) | (lp >> 29)));
    const float mS = __int_as_float((int)(0x3F800000u | ((hS & 0xFFFFFu) << 3) | (lS >> 29)));
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(mS));  // (0.5, 1]
    const float hf = mp * rf;                                 // [0.5, 2]
    const unsigned sg = hS & 0x80000000u;                    // p / S has the sign of S
    const double r2 = f64_of_f32_scaled(rf, 1024 - eS, sg);
    const int ks = ep - eS;
    const bool ok = ep != 0 && (int)((unsigned)__float_as_int(hf) >> 23) + 896 + ks >= 1;
    const double s0h = ok ? f64_of_f32_scaled(hf, ks, sg) : 0.0;
    const double s0 = ok ? f64_of_f32_scaled(hf, ks + 1, sg) : 0.0;
    const double t = fma(-s0h, S, p);  // p - s0h S
    return fma(r2, t, s0);
}

// ----------------------------------------------------------------------------
// MUSCL van Leer slope (src/solvers/HydrostaticRoe.cpp:173-195), floating abs.
// ----------------------------------------------------------------------------
template <class R, bool FAST> __host__ __device__ __forceinline__ R van_leer_slope(R qm, R q, R qp) {
    const R dm = q - qm;
    const R dp = qp - q;
    if constexpr (FAST) {
        if (abs_le_bits(dp, Cst<R>::tol12_bits)) return R(0);
    } else {
        if (fabs(dp) <= Cst<R>::tol12) return R(0);
    }
    if constexpr (!FAST) {
        const R r = dm / dp;
        return (r + fabs(r)) / (R(1) + fabs(r)) * dp;
    } else {
        // phi(r) dp with r = dm/dp is 0 for r <= 0 and 2 dm dp / (dm + dp) otherwise.
        const R p = dm * dp;
#ifdef __CUDA_ARCH__
        if constexpr (sizeof(R) == 8) return pos_i(p) ? van_leer_div2(p, dm + dp) : R(0);
#else
        if constexpr (sizeof(R) == 8) return pos_i(p) ? p * (R(2) / (dm + dp)) : R(0);
#endif
        else return pos_i(p) ? (p + p) * rcp_nr(dm + dp) : R(0);
    }
}

// The fast van Leer slope (van_leer_slope<double, true>, same operations) that
// also hands back the reciprocal 1 / (dm + dp) its reverse needs (0 where the
// slope is 0 by a branch).
__host__ __device__ __forceinline__ double van_leer_slope_rs(double qm, double q, double qp, double& rS) {
    const double dm = q - qm, dp = qp - q;
    rS = 0.0;
    if (abs_le_bits(dp, Cst<double>::tol12_bits)) return 0.0;
    const double p = dm * dp;
    if (!pos_i(p)) return 0.0;
    const double S = dm + dp;
    rS = rcp_nr(S);
#ifdef __CUDA_ARCH__
    return van_leer_div2(p, S);
#else
    return (p + p) * rS;
#endif
}

// ----------------------------------------------------------------------------
// Homogeneous Roe flux (include/solvers/kernels/HydrostaticRoe.H:44-159) for a
// face of direction DIR (0: normal +x, 1: normal +y).  The normal is fixed at
// compile time, so the rotation by (nx, ny) becomes a relabelling, which is
// value-exact.  Exact form: inputs are the face depths and global momenta.
// ----------------------------------------------------------------------------
template <int DIR, class R>
__host__ __device__ __forceinline__ void roe_hydrostatic_exact(R hi, R hui, R hvi, R hj, R huj, R hvj, R& F0, R& F1,
                                                      R& F2) {
    using C = Cst<R>;
    hi = (hi >= C::toldry) ? hi : R(0);
    hj = (hj >= C::toldry) ? hj : R(0);
    const R si = (hi > R(0)) ? sqrt(hi) : R(0);
    const R sj = (hj > R(0)) ? sqrt(hj) : R(0);
    const R ui = (hi > R(0)) ? hui / hi : R(0);
    const R vi = (hi > R(0)) ? hvi / hi : R(0);
    const R uj = (hj > R(0)) ? huj / hj : R(0);
    const R vj = (hj > R(0)) ? hvj / hj : R(0);
    R uni, uti, unj, utj;
    if (DIR == 0) { uni = ui; uti = vi; unj = uj; utj = vj; }
    else { uni = vi; uti = -ui; unj = vj; utj = -uj; }
    const R hsum = hi + hj;
    const R hm = (0.5 * hsum > C::toldry) ? R(0.5) * hsum : C::toldry;
    const R cm = sqrt(C::g * hm);
    const R sden = si + sj + C::tol12;
    const R um = (uni * si + unj * sj) / sden;
    const R vm = (uti * si + utj * sj) / sden;
    R l0 = um - cm;
    const R l1 = um;
    R l2 = um + cm;
    {
        const R ci = sqrt(C::g * hi), cj = sqrt(C::g * hj);
        R ei = uni - ci, ej = unj - cj;
        if (ei < R(0) && ej > R(0)) l0 = ei * (ej - l0) / (ej - ei);
        ei = uni + ci;
        ej = unj + cj;
        if (ei < R(0) && ej > R(0)) l2 = ej * (l2 - ei) / (ej - ei);
    }
    const R den = R(2) * cm + C::tol12;
    const R dh = hj - hi;
    const R dhu = hj * unj - hi * uni;
    const R dhv = hj * utj - hi * uti;
    const R a0 = (l2 * dh - dhu) / den;
    const R a1 = (-vm * dh + dhv) / cm;
    const R a2 = (-l0 * dh + dhu) / den;
    R f0 = R(0.5) * (hi * uni + hj * unj);
    R f1 = R(0.5) * (hi * uni * uni + C::half_g * hi * hi + hj * unj * unj + C::half_g * hj * hj);
    R f2 = R(0.5) * (hi * uni * uti + hj * unj * utj);
    const R w0 = R(0.5) * fabs(l0) * a0;
    f0 -= w0;
    f1 -= w0 * l0;
    f2 -= w0 * vm;
    const R w1 = R(0.5) * fabs(l1) * a1;  // contact wave: eigenvector (0, 0, c)
    f2 -= w1 * cm;
    const R w2 = R(0.5) * fabs(l2) * a2;
    f0 -= w2;
    f1 -= w2 * l2;
    f2 -= w2 * vm;
    F0 = f0;
    if (DIR == 0) { F1 = f1; F2 = f2; }
    else { F1 = -f2; F2 = f1; }
}

// Intermediates of one fast-form face flux that its reverse needs: square
// roots, the shared reciprocal, Roe averages, the entropy-fixed speeds and the
// half wave strengths, with the branch flags.  Recorded by the adjoint's
// segment recompute so the reverse sweep does not evaluate them again.
struct RoeRecVals {
    double si, sj, cm, rs, hrden, hrcm, um, vm, l0, l2, a0h, a1h, a2h;  // 1/sden, 1/(2 den), 1/(2 cm)
    unsigned fl;  // RR_WI | RR_WJ | RR_HM | RR_FIX0 | RR_FIX2
};
constexpr int NREC = 13;  // doubles of a RoeRecVals
constexpr unsigned RR_WI = 1u, RR_WJ = 2u, RR_HM = 4u, RR_FIX0 = 8u, RR_FIX2 = 16u;

// Fast form: inputs are the face depths and face velocities (the reference
// rebuilds the velocity as (h u)/h, which equals u to an ulp).  In FP64 one
// reciprocal 1/(sden den) gives both 1/sden (the Roe averages) and 1/den (two
// wave strengths), and 1/cm (the contact wave) comes from the correction step
// of cm's own square root; the wave speeds sqrt(g h) reuse sqrt(h).  With REC
// the intermediates go to *rv (values only stored: the arithmetic is the same
// instruction for instruction).
template <class R, int DIR, bool REC = false>
__host__ __device__ __forceinline__ void roe_hydrostatic_fast(R hi, R ui, R vi, R hj, R uj, R vj, R& F0, R& F1,
                                                             R& F2, RoeRecVals* rv = nullptr) {
    using C = Cst<R>;
    // depths arrive non-negative (capped with max(0, .)), so bit comparisons apply
    const bool wi = ge_bits(hi, C::toldry_bits), wj = ge_bits(hj, C::toldry_bits);
    hi = wi ? hi : R(0);
    hj = wj ? hj : R(0);
    ui = wi ? ui : R(0);
    vi = wi ? vi : R(0);
    uj = wj ? uj : R(0);
    vj = wj ? vj : R(0);
    const R si = fast_sqrt(hi), sj = fast_sqrt(hj);
    R uni, uti, unj, utj;
    if (DIR == 0) { uni = ui; uti = vi; unj = uj; utj = vj; }
    else { uni = vi; uti = -ui; unj = vj; utj = -uj; }
    // hm = max(0.5 (hi + hj), toldry) enters only as g hm: 0.5 hs > toldry exactly when hs > 2 toldry, and
    // g (0.5 hs) and (g / 2) hs are one rounding of the same product, so the halving goes
    const R hs = hi + hj;
    const bool hmb = gt_bits(hs, C::toldry2_bits);
    const R ghm = hmb ? C::half_g * hs : C::g_toldry;
    R cm, hrcm;  // hrcm = 1 / (2 cm)
    const R sden = si + sj + C::tol12;
    // FP64: one reciprocal 1 / (2 sden den) = q/2 for 1/sden and 1/(2 den), 1/(2 cm) from cm's square root
    // (den = 2 cm + tol12 and 2 den = 4 cm + 2 tol12 exactly, so every value is that of q = 1/(sden den));
    // float: one reciprocal for all three
    R rs, hrden;
    if constexpr (sizeof(R) == 8) {
        cm = fast_sqrt_hrsqrt(ghm, hrcm);
        const R den2 = R(4) * cm + R(2) * C::tol12;
        const R hq = rcp_nr(sden * den2);
        rs = den2 * hq;
        hrden = sden * hq;
    } else {
        cm = fast_sqrt(ghm);
        const R den = R(2) * cm + C::tol12;
        const R cd = cm * den;
        const R q = rcp_nr(sden * cd);
        rs = cd * q;
        hrden = R(0.5) * ((sden * cm) * q);
        hrcm = R(0.5) * ((sden * den) * q);
    }
    const R um = (uni * si + unj * sj) * rs;
    const R vm = (uti * si + utj * sj) * rs;
    R l0 = um - cm;
    const R l1 = um;
    R l2 = um + cm;
    bool fix0 = false, fix2 = false;
    // Entropy fixes need e_i < 0 < e_j for e = u -+ c.  In FP64 the tests are
    // first taken in float from the leading bits (error below 2^-20 of
    // |u| + c, against a margin of 2^-16 of it): where a sign is certain the
    // fix is ruled out without FP64 work (subsonic faces); otherwise the FP64
    // tests decide, so the outcome is that of the FP64 tests everywhere.
    bool rule0 = false, rule2 = false;
    if constexpr (sizeof(R) == 8) {
        const float ui32 = f32_lead(uni), uj32 = f32_lead(unj);
        const float ci32 = 3.13209195f * f32_lead(si), cj32 = 3.13209195f * f32_lead(sj);
        const float mi = 0x1p-16f * (fabsf(ui32) + ci32), mj = 0x1p-16f * (fabsf(uj32) + cj32);
        rule0 = (ui32 - ci32 >= mi) || (uj32 - cj32 <= -mj);
        rule2 = (ui32 + ci32 >= mi) || (uj32 + cj32 <= -mj);
    }
    if (!(rule0 && rule2)) {
        const R ci = C::sqrt_g * si, cj = C::sqrt_g * sj;
        R ei = uni - ci, ej = unj - cj;
        fix0 = !rule0 && neg_i(ei) && pos_i(ej);
        if (fix0) l0 = ei * (ej - l0) / (ej - ei);
        ei = uni + ci;
        ej = unj + cj;
        fix2 = !rule2 && neg_i(ei) && pos_i(ej);
        if (fix2) l2 = ej * (l2 - ei) / (ej - ei);
    }
    const R dh = hj - hi;
    const R qi = hi * uni, qj = hj * unj;
    const R dhu = qj - qi;
    const R dhv = hj * utj - hi * uti;
    const R a0h = (l2 * dh - dhu) * hrden;  // alpha0 / 2
    const R a1h = (dhv - vm * dh) * hrcm;
    const R a2h = (dhu - l0 * dh) * hrden;
    const R w0 = fabs(l0) * a0h;
    const R w1 = fabs(l1) * a1h;
    const R w2 = fabs(l2) * a2h;
    const R f0 = R(0.5) * (qi + qj) - (w0 + w2);
    const R f1 = R(0.5) * (qi * uni + qj * unj + C::half_g * (hi * hi + hj * hj)) - (w0 * l0 + w2 * l2);
    const R f2 = R(0.5) * (qi * uti + qj * utj) - ((w0 + w2) * vm + w1 * cm);
    F0 = f0;
    if (DIR == 0) { F1 = f1; F2 = f2; }
    else { F1 = -f2; F2 = f1; }
    if constexpr (REC) {
        rv->si = si; rv->sj = sj; rv->cm = cm; rv->rs = rs; rv->hrden = hrden; rv->hrcm = hrcm;
        rv->um = um; rv->vm = vm; rv->l0 = l0; rv->l2 = l2;
        rv->a0h = a0h; rv->a1h = a1h; rv->a2h = a2h;
        rv->fl = (wi ? RR_WI : 0u) | (wj ? RR_WJ : 0u) | (hmb ? RR_HM : 0u) | (fix0 ? RR_FIX0 : 0u) |
                 (fix2 ? RR_FIX2 : 0u);
    }
}

// ----------------------------------------------------------------------------
// Classic Roe flux with bed-slope thrust, Manning friction and positivity
// guard (include/solvers/kernels/Roe.H:51-309), direction fixed at compile
// time.  Outputs F, S-, S+ in global coordinates.
// ----------------------------------------------------------------------------
template <class R, bool FAST, int DIR>
__host__ __device__ __forceinline__ void roe_classic(R hi, R hui, R hvi, R zi, R ni, R hj, R huj, R hvj, R zj, R nj, R dx,
                                            R F[3], R Sm[3], R Sp[3]) {
    using C = Cst<R>;
    const R T12 = C::tol12, TD = C::toldry;
    hi = (hi >= TD) ? hi : R(0);
    hj = (hj >= TD) ? hj : R(0);
    R si, sj, ui, vi, uj, vj;
    if constexpr (!FAST) {
        si = (hi > R(0)) ? sqrt(hi) : R(0);
        sj = (hj > R(0)) ? sqrt(hj) : R(0);
        ui = (hi > R(0)) ? hui / hi : R(0);
        vi = (hi > R(0)) ? hvi / hi : R(0);
        uj = (hj > R(0)) ? huj / hj : R(0);
        vj = (hj > R(0)) ? hvj / hj : R(0);
    } else {
        si = fast_sqrt(hi);
        sj = fast_sqrt(hj);
        const R ri = (hi > R(0)) ? R(1) / hi : R(0);
        const R rj = (hj > R(0)) ? R(1) / hj : R(0);
        ui = hui * ri; vi = hvi * ri; uj = huj * rj; vj = hvj * rj;
    }
    R uni, uti, unj, utj;
    if (DIR == 0) { uni = ui; uti = vi; unj = uj; utj = vj; }
    else { uni = vi; uti = -ui; unj = vj; utj = -uj; }
    const R hsum = hi + hj;
    const R hm = (R(0.5) * hsum > TD) ? R(0.5) * hsum : TD;
    const R cm = FAST ? fast_sqrt(C::g * hm) : sqrt(C::g * hm);
    const R sden = si + sj + T12;
    const R um = (uni * si + unj * sj) / sden;
    const R vm = (uti * si + utj * sj) / sden;
    R l0 = um - cm;
    const R l1 = um;
    R l2 = um + cm;
    {
        R ci, cj;
        if constexpr (!FAST) { ci = sqrt(C::g * hi); cj = sqrt(C::g * hj); }
        else { ci = C::sqrt_g * si; cj = C::sqrt_g * sj; }
        R ei = uni - ci, ej = unj - cj;
        if (ei < R(0) && ej > R(0)) l0 = ei * (ej - l0) / (ej - ei);
        ei = uni + ci;
        ej = unj + cj;
        if (ei < R(0) && ej > R(0)) l2 = ej * (l2 - ei) / (ej - ei);
    }
    const R den = R(2) * cm + T12;
    const R dh = hj - hi;
    const R dhu = hj * unj - hi * uni;
    const R dhv = hj * utj - hi * uti;
    const R a0 = (l2 * dh - dhu) / den;
    const R a1 = (-vm * dh + dhv) / cm;
    const R a2 = (-l0 * dh + dhu) / den;

    const R dz = zj - zi;
    const R di = hi + zi;
    const R dj = hj + zj;
    const R dd = dj - di;
    R thrust, tau;
    {
        const R ta = -C::g * hm * dz;
        R dzt;
        if ((dz >= R(0)) && (di < zj)) dzt = hi;
        else if ((dz < R(0)) && (dj < zi)) dzt = hj;
        else dzt = dz;
        const R hr = (dz >= R(0)) ? hi : hj;
        const R tb = -C::g * (hr - R(0.5) * fabs(dzt)) * dzt;
        thrust = ((dz * dd >= R(0)) && (um * dz > R(0))) ? smax(ta, tb) : tb;
        const R nm = R(0.5) * (ni + nj);
        if constexpr (!FAST) {
            const R sf = (nm * nm * sqrt(um * um + vm * vm) * um) / smax(TD, hm * cbrt(hm));
            tau = C::g * hm * sf * dx;
        } else {
            // the friction term vanishes identically when the face roughness is zero
            if (nm != R(0)) {
                const R sf = (nm * nm * sqrt(um * um + vm * vm) * um) / smax(TD, hm * cbrt(hm));
                tau = C::g * hm * sf * dx;
            } else {
                tau = R(0);
            }
        }
    }
    R b0 = (thrust - tau) / den;
    const R b1 = R(0);
    R b2 = -b0;
    {
        const R l0s = (fabs(l0) > T12) ? l0 : (l0 >= R(0) ? T12 : -T12);
        const R l2s = (fabs(l2) > T12) ? l2 : (l2 >= R(0) ? T12 : -T12);
        const R hi1 = hi + a0 - (b0 / l0s);
        const R hj3 = hj - a2 + (b2 / l2s);
        R ml = fabs(l0);
        ml = smax(ml, fabs(l1));
        ml = smax(ml, fabs(l2));
        const R ldt = dx / (ml + T12);
        const R d1 = hi - hi1;
        const R d1s = (fabs(d1) > T12) ? d1 : (d1 >= R(0) ? T12 : -T12);
        const R d3 = hj - hj3;
        const R d3s = (fabs(d3) > T12) ? d3 : (d3 >= R(0) ? T12 : -T12);
        const bool g1 = (hi1 < -TD) && (hj3 > TD);
        const bool g3 = (hi1 > TD) && (hj3 < -TD);
        if (g1 || g3) {
            const R dt1 = (dx * R(0.5) / l0s) * (hi / d1s);
            const R dt3 = (dx * R(0.5) / l2s) * (hj / d3s);
            if (g1 && (dt1 < ldt)) {
                const R b1min = -(hi + a0) * fabs(l0);
                const R b3min = -(hj - a2) * l2;
                if (-b1min >= b3min) b0 = b1min;
                b2 = -b0;
            }
            if (g3 && (dt3 < ldt)) {
                const R b1min = -(hi + a0) * fabs(l0);
                const R b3min = -(hj - a2) * l2;
                if (-b3min >= b1min) b2 = b3min;
                b0 = -b2;
            }
        }
    }
    R f0 = R(0.5) * (hi * uni + hj * unj);
    R f1 = R(0.5) * (hi * uni * uni + C::half_g * hi * hi + hj * unj * unj + C::half_g * hj * hj);
    R f2 = R(0.5) * (hi * uni * uti + hj * unj * utj);
    R m0 = 0, m1 = 0, m2 = 0, p0 = 0, p1 = 0, p2 = 0;
    {
        const R w = R(0.5) * fabs(l0) * a0;
        f0 -= w; f1 -= w * l0; f2 -= w * vm;
        if (l0 > R(0)) { m0 += b0; m1 += b0 * l0; m2 += b0 * vm; }
        else if (l0 < R(0)) { p0 += b0; p1 += b0 * l0; p2 += b0 * vm; }
    }
    {
        const R w = R(0.5) * fabs(l1) * a1;
        f2 -= w * cm;
        if (l1 > R(0)) { m2 += b1 * cm; }
        else if (l1 < R(0)) { p2 += b1 * cm; }
    }
    {
        const R w = R(0.5) * fabs(l2) * a2;
        f0 -= w; f1 -= w * l2; f2 -= w * vm;
        if (l2 > R(0)) { m0 += b2; m1 += b2 * l2; m2 += b2 * vm; }
        else if (l2 < R(0)) { p0 += b2; p1 += b2 * l2; p2 += b2 * vm; }
    }
    F[0] = f0; Sm[0] = m0; Sp[0] = p0;
    if (DIR == 0) {
        F[1] = f1; F[2] = f2; Sm[1] = m1; Sm[2] = m2; Sp[1] = p1; Sp[2] = p2;
    } else {
        F[1] = -f2; F[2] = f1; Sm[1] = -m2; Sm[2] = m1; Sp[1] = -p2; Sp[2] = p1;
    }
}

// ----------------------------------------------------------------------------
// dt accumulator (hx_dt_accum).  min over cells of fl(1/x_c) equals
// fl(1/max x_c) because rounded division is monotone, so the device keeps the
// largest wave-speed rate x_c = (|u|+c)/dx + (|v|+c)/dy of the wet cells and
// flags for the constant bounds of dry (1e6) and NODATA (1e30) cells.  All
// values are non-negative, so their IEEE bit patterns order as integers.
// ----------------------------------------------------------------------------
struct DtAccum {
    unsigned long long rate_bits;    // max rate over wet cells (R's bit pattern)
    unsigned long long maxvel_bits;  // max of max(|u|,|v|)
    unsigned int flags;              // 1: a dry cell, 2: a NODATA cell, 4: NaN seen
    unsigned int pad[11];
};
static_assert(sizeof(DtAccum) == 64, "hx_dt_accum is 64 bytes");

enum { DTF_DRY = 1, DTF_NODATA = 2, DTF_NAN = 4, DTF_COLLAPSED = 8 };

template <class R> __device__ __forceinline__ unsigned long long to_bits(R x);
template <> __device__ __forceinline__ unsigned long long to_bits<double>(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
template <> __device__ __forceinline__ unsigned long long to_bits<float>(float x) {
    return (unsigned long long)__float_as_uint(x);
}
template <> __device__ __forceinline__ unsigned long long to_bits<Dual>(Dual x) { return to_bits<double>(x.v); }
template <class R> __host__ __device__ __forceinline__ R from_bits(unsigned long long b);
template <> __host__ __device__ __forceinline__ double from_bits<double>(unsigned long long b) {
    union { unsigned long long u; double d; } c;
    c.u = b;
    return c.d;
}
template <> __host__ __device__ __forceinline__ float from_bits<float>(unsigned long long b) {
    union { unsigned u; float f; } c;
    c.u = (unsigned)b;
    return c.f;
}

// min CFL bound (before the CFL factor) of an accumulator: the reference's
// 1.0 / rate evaluated in double and stored in R.
template <class R> __host__ __device__ __forceinline__ R accum_dt_min(unsigned long long rate_bits, unsigned flags) {
    const R rate = from_bits<R>(rate_bits);
    R m = R(3.4e38);
    if (sizeof(R) == 8) m = (R)1.7976931348623157e308;
    if (rate > R(0)) m = (R)(1.0 / (double)rate);
    if (flags & DTF_DRY) m = (m < R(1.e6)) ? m : R(1.e6);
    if (flags & DTF_NODATA) m = (m < R(1.e30)) ? m : R(1.e30);
    return m;
}

// Per-cell contribution of compute_dt_Impl (HydrostaticRoe.cpp:41-61).  nod is
// the cell's NODATA predicate |z + 9999| < 1e-10.
template <class R, bool FAST>
__device__ __forceinline__ void dt_cell_contrib(R h, R hu, R hv, bool nod, R dx, R dy, R idx, R idy, R& rate, R& mv,
                                                unsigned& flags) {
    rate = R(0);
    mv = R(0);
    if (nod) { flags |= DTF_NODATA; return; }
    if constexpr (!FAST) {
        if (!(h > Cst<R>::tol12)) { flags |= DTF_DRY; return; }
        const R u = hu / h, v = hv / h;
        const R c = sqrt(Cst<R>::g * h);
        const R sx = fabs(u) + c;
        const R sy = fabs(v) + c;
        rate = sx / dx + sy / dy;
        mv = smax(fabs(u), fabs(v));
    } else {
        if (!gt_bits(h, Cst<R>::tol12_bits)) { flags |= DTF_DRY; return; }
        R r, c;
        if constexpr (sizeof(R) == 8) {  // within an ulp: dt follows the exact form's to the last few ulps
            r = rcp_fa(h);
            c = fast_sqrt_fa(Cst<R>::g * h);
        } else {
            r = rcp_nr(h);
            c = fast_sqrt(Cst<R>::g * h);
        }
        const R u = hu * r, v = hv * r;
        rate = (fabs(u) + c) * idx + (fabs(v) + c) * idy;
        mv = nnmax_i(fabs(u), fabs(v));
    }
    if (bits_nonfinite(rate)) { flags |= DTF_NAN; rate = R(0); mv = R(0); }
}

// Block-wide reduction of (rate, maxvel, flags) into acc.  All threads of the
// block must call it.  Integer max on the non-negative bit patterns.
template <class R, int NT>
__device__ __forceinline__ void block_fold_dt(R rate, R mv, unsigned flags, DtAccum* acc) {
    unsigned long long rb = to_bits(rate), vb = to_bits(mv);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long r2 = __shfl_xor_sync(0xffffffffu, rb, o);
        const unsigned long long v2 = __shfl_xor_sync(0xffffffffu, vb, o);
        rb = r2 > rb ? r2 : rb;
        vb = v2 > vb ? v2 : vb;
    }
    flags = __reduce_or_sync(0xffffffffu, flags);
    __shared__ unsigned long long s_r[NT / 32], s_v[NT / 32];
    __shared__ unsigned s_f[NT / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { s_r[w] = rb; s_v[w] = vb; s_f[w] = flags; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < NT / 32; ++k) {
            rb = s_r[k] > rb ? s_r[k] : rb;
            vb = s_v[k] > vb ? s_v[k] : vb;
            flags |= s_f[k];
        }
        if (rb) atomicMax(&acc->rate_bits, rb);
        if (vb) atomicMax(&acc->maxvel_bits, vb);
        if (flags) atomicOr(&acc->flags, flags);
    }
}

}  // namespace hx
