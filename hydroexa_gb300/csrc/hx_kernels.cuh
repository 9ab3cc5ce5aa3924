// Tile kernels of the per-level advance.  Included by hx_exact.cu (compiled
// with --fmad=false) and hx_fast.cu; each instantiates its arithmetic form.
//
// One CTA advances a TX x TY tile of cells.  It stages the tile and its MUSCL
// halo in shared memory (h rebuilt from eta and z on load, velocities and eta
// derived once per cell), computes each cell's van Leer slopes once per
// direction, each face flux once, then the update of its own cell, and folds
// the next step's CFL bound of the updated cell into the dt accumulator.  The
// reference runs these as separate passes over separate arrays
// (src/solvers/HydrostaticRoe.cpp:490-606): here each cell is read once and
// written once per step.
#pragma once

#include <cuda.h>  // CUtensorMap (the type only; its encoder is reached through the runtime)

#include <cstdint>
#include <cstring>
#include <type_traits>

#include "hx_device.cuh"
#include "hx_internal.h"

namespace hx {

// ---------------------------------------------------------------------------
// Hydrostatic-Roe tile kernel.
// ---------------------------------------------------------------------------
// Sources with an interior fetch (kInterior): the fast form's phase A reads the stored depth directly on
// tiles whose grown region lies in the level.
template <class T, class = void> struct InteriorFetch : std::false_type {};
template <class T> struct InteriorFetch<T, std::void_t<decltype(T::kInterior)>> : std::bool_constant<T::kInterior> {};

template <class R, int TXv = TX, int TYv = TY> struct HydroSmem {
    static constexpr int GX = TXv + 4, GY = TYv + 4;
    R z[GY][GX], eta[GY][GX], u[GY][GX], v[GY][GX];
    R sxe[TYv][TXv + 2], sxu[TYv][TXv + 2], sxv[TYv][TXv + 2];  // x-slopes of tile columns -1..TX
    R sye[TYv + 2][TXv], syu[TYv + 2][TXv], syv[TYv + 2][TXv];  // y-slopes of tile rows -1..TY
    R fx[4][TYv][TXv + 1];                                      // x faces: F0, FL1, FR1, F2
    R fy[4][TYv + 1][TXv];                                      // y faces: F0, F1, FL2, FR2
    unsigned char nod[GY][GX];                                  // NODATA predicate of each grown-tile cell
    R kc[4];  // dt/dx, dt/dy, 1/dx, 1/dy: computed once per tile, not once per cell
};

// One hydrostatic face (src/solvers/HydrostaticRoe.cpp:218-396).  L and R are
// the cells on either side; sX are the cells' slopes along the face normal.
template <class R, bool FAST, int DIR, bool REC = false>
__device__ __forceinline__ void hydro_face(bool wall, R zL, R zR, R eL, R eR, R seL, R seR, R uL, R uR, R suL, R suR,
                                           R vL, R vR, R svL, R svR, R& F0, R& Fa, R& Fb, R& Fc,
                                           RoeRecVals* rv = nullptr) {
    // wall: either side is NODATA (HydrostaticRoe.cpp:237-245)
    if (wall) {
        F0 = R(0); Fa = R(0); Fb = R(0); Fc = R(0);
        return;
    }
    R zf;
    if constexpr (FAST) zf = smax_i(zL, zR);
    else zf = smax(zL, zR);
    const R etaLf = eL + R(0.5) * seL;
    const R etaRf = eR - R(0.5) * seR;
    const R uLf = uL + R(0.5) * suL;
    const R uRf = uR - R(0.5) * suR;
    const R vLf = vL + R(0.5) * svL;
    const R vRf = vR - R(0.5) * svR;
    R hLu, hRu, hLs, hRs;
    R pW = R(0);       // fast form: the pressure correction of the lower-bed side (the other side's is 0)
    bool lhigh = false;  // fast form: the left bed is the face bed
    if constexpr (FAST) {
        // The side whose bed is the face bed zf has its capped depth equal to its own (uncapped) one, so its
        // pressure correction is exactly +0: only the lower side's depths and correction are computed (the
        // face-bed side's flux is then the Roe flux itself, which differs from adding +0 only for a -0 flux).
        lhigh = !(okey(zL) < okey(zR));  // zf == zL
        const R eH = lhigh ? etaLf : etaRf, zH = lhigh ? zL : zR;
        const R eW = lhigh ? etaRf : etaLf, zW = lhigh ? zR : zL;
        const R hH = max0_i(eH - zH);
        const R hWu = max0_i(eW - zW), hWs = max0_i(eW - zf);
        // (a^2 - b^2) = (a - b)(a + b) is exactly zero whenever a == b (lake at rest)
        pW = (hWu - hWs) * (hWu + hWs);  // times g/2 in the flux's multiply-add below
        hLu = lhigh ? hH : hWu;
        hLs = lhigh ? hH : hWs;
        hRu = lhigh ? hWu : hH;
        hRs = lhigh ? hWs : hH;
    } else {
        hLu = max0(etaLf - zL);
        hRu = max0(etaRf - zR);
        hLs = max0(etaLf - zf);
        hRs = max0(etaRf - zf);
    }
    R f0, f1, f2;
    if constexpr (!FAST) {
        const R huL = (hLs > R(0)) ? hLs * uLf : R(0);
        const R hvL = (hLs > R(0)) ? hLs * vLf : R(0);
        const R huR = (hRs > R(0)) ? hRs * uRf : R(0);
        const R hvR = (hRs > R(0)) ? hRs * vRf : R(0);
        roe_hydrostatic_exact<DIR>(hLs, huL, hvL, hRs, huR, hvR, f0, f1, f2);
    } else {
        roe_hydrostatic_fast<R, DIR, REC>(hLs, uLf, vLf, hRs, uRf, vRf, f0, f1, f2, rv);
    }
    // hydrostatic pressure correction, rotated with the normal
    F0 = f0;
    if constexpr (!FAST) {
        const R pL = Cst<R>::half_g * (hLu * hLu - hLs * hLs);
        const R pR = Cst<R>::half_g * (hRu * hRu - hRs * hRs);
        if (DIR == 0) { Fa = f1 + pL; Fb = f1 + pR; Fc = f2; }
        else { Fa = f1; Fb = f2 + pL; Fc = f2 + pR; }
    } else {
        // one add: the face-bed side's flux is the normal-momentum flux itself (adding its +0 correction
        // would change only a -0 flux into +0)
        (void)hLu;
        (void)hRu;
        const R fn = (DIR == 0) ? f1 : f2, fw = fma(Cst<R>::half_g, pW, fn);
        if (DIR == 0) { Fa = lhigh ? fn : fw; Fb = lhigh ? fw : fn; Fc = f2; }
        else { Fa = f1; Fb = lhigh ? fn : fw; Fc = lhigh ? fw : fn; }
    }
}

// dt of a step of the device time loop.  A collapse (min CFL bound < 1e-12,
// HydrostaticRoe.cpp:77-80) is carried forward as a flag in the next
// accumulator, so every later step sees it in launch-constant data and every
// thread of every block takes the same early exit.
template <class R> __device__ __forceinline__ bool resolve_dt(const StepCtl<R>& c, R& dt) {
    if (c.dt_in == nullptr) { dt = c.dt_host; return true; }
    const unsigned fl = c.dt_in->flags;
    const R m = accum_dt_min<R>(c.dt_in->rate_bits, fl);
    if ((fl & DTF_COLLAPSED) || m < R(1.e-12)) {
        if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
            if (c.status) atomicOr(c.status, (unsigned)HX_STATUS_DT_COLLAPSE);
            if (c.dt_out) atomicOr(&c.dt_out->flags, (unsigned)DTF_COLLAPSED);
        }
        return false;
    }
    dt = m * c.cfl;
    return true;
}

template <class R> __device__ __forceinline__ void step_bookkeeping(const StepCtl<R>& c, R dt) {
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
        if (c.dt_reset) {
            c.dt_reset->rate_bits = 0ull;
            c.dt_reset->maxvel_bits = 0ull;
            c.dt_reset->flags = 0u;
        }
        if (c.time) *c.time += dt;
    }
}

// The advance of one TXv x TYv tile with origin (x0, y0) by NTv threads (any
// NTv; each thread takes cells t, t+NTv, ...).  Shared by the plain per-level
// kernel and the ensemble kernel.  The caller has resolved dt.  Every thread
// of the block must call it (it synchronises).
// LINEAR: store the state after the flux update but before friction and the
// dry clamp (used by the adjoint).  post_flags (optional): OR-ed with 1 when a
// cell of the tile took the friction branch and 2 when one took the dry clamp.
// The per-cell end of a step: the update of the stored state by the flux
// differences (HydrostaticRoe.cpp:554-564), Manning friction and the dry clamp
// (:566-603), the store, and the cell's share of the next CFL bound.  One
// function for the fused tile kernel and the split update kernel, so both do
// the same arithmetic.  LINEAR stores the updated state before friction and
// clamp.  pflags: 1 if the Manning factor applied, 2 if the clamp did.
// A cell's updated state kept for the screened CFL fold (screened_fold).
template <class R> struct ScreenCell {
    R h = R(0), hu = R(0), hv = R(0);
    bool nod = false, live = false;
};

template <class R, bool FAST, bool LINEAR, class NP = Plane<R>>
__device__ __forceinline__ void step_cell(R o0, R o1, R o2, R dx0, R dx1, R dx2, R dy0, R dy1, R dy2, R cx, R cy,
                                          R dt, const NP& nplane, const Cells3W<R>& out, int gi, int gj,
                                          bool nod, R dx, R dy, R idx, R idy, bool fold_dt, R& rate, R& mv,
                                          unsigned& flags, unsigned& pflags, ScreenCell<R>* sc = nullptr) {
    R un[3];
    un[0] = (o0 - cx * dx0) - cy * dy0;
    un[1] = (o1 - cx * dx1) - cy * dy1;
    un[2] = (o2 - cx * dx2) - cy * dy2;
    if constexpr (LINEAR) {
        out.st(gi, gj, un[0], un[1], un[2]);
        return;
    }
    const R hh = un[0];
    bool wet, rough;
    if constexpr (FAST) wet = ge_bits(hh, Cst<R>::toldry_bits);
    else wet = hh >= Cst<R>::toldry;
    if (wet) {
        const R nv = nplane.ld(gi, gj);
        const R nsq = nv * nv;
        if constexpr (FAST) rough = gt_bits(nsq, Cst<R>::tol12_bits);
        else rough = nsq > Cst<R>::tol12;
        if (rough) {  // the friction factor needs a rough bed
            const R qx = un[1], qy = un[2];
            if constexpr (!FAST) {
                const R inv_h = R(1.0) / hh;
                const R uu = qx * inv_h, vv = qy * inv_h;
                const R modM = sqrt(uu * uu + vv * vv);
                if (modM > Cst<R>::tol12) {
                    pflags |= 1u;
                    const R h43 = hh * cbrt(hh);
                    const R tt = dt * Cst<R>::g * nsq * modM / h43;
                    const R ff = sqrt(R(1.0) + R(4.0) * tt);
                    const R fac = R(2.0) / (R(1.0) + ff);
                    un[1] = qx * fac;
                    un[2] = qy * fac;
                }
            } else {
                // the same factor with h^(4/3) as h / h^(-1/3) sharing 1/h with |u|, and the square root and
                // reciprocals of the fast form: 2 / (1 + ff) = 1 / (0.5 + 0.5 ff)
                const R rh = rcp_nr(hh);
                const R modM = fast_sqrt(qx * qx + qy * qy) * rh;
                if (gt_bits(modM, Cst<R>::tol12_bits)) {
                    pflags |= 1u;
                    const R tt = dt * Cst<R>::g * nsq * modM * (rcbrt_nr(hh) * rh);
                    const R ff = fast_sqrt(fma(R(4.0), tt, R(1.0)));
                    const R fac = rcp_nr(fma(R(0.5), ff, R(0.5)));
                    un[1] = qx * fac;
                    un[2] = qy * fac;
                }
            }
        }
    } else {
        pflags |= 2u;
        if constexpr (FAST) un[0] = neg_i(hh) ? R(0) : hh;
        else un[0] = smax(hh, R(0));
        un[1] = R(0);
        un[2] = R(0);
    }
    out.st(gi, gj, un[0], un[1], un[2]);
    if (bits_nonfinite(un[0]) || bits_nonfinite(un[1]) || bits_nonfinite(un[2])) flags |= DTF_NAN;
    if (sc) {
        sc->h = un[0]; sc->hu = un[1]; sc->hv = un[2]; sc->nod = nod; sc->live = true;
    }
    if (fold_dt) {
        R rc, mc;
        dt_cell_contrib<R, FAST>(un[0], un[1], un[2], nod, dx, dy, idx, idy, rc, mc, flags);
        if constexpr (FAST) {
            rate = nnmax_i(rate, rc);
            mv = nnmax_i(mv, mc);
        } else {
            rate = smax(rate, rc);
            mv = smax(mv, mc);
        }
    }
}

// No face records (every step but the adjoint's segment recompute).
struct NoRec {
    static constexpr bool on = false;
};
// Face records of one step of the adjoint's segment recompute (fast form,
// FP64): NREC field planes and one flag plane per direction.  x face (i, j),
// i in 0..nx, j in 0..ny-1, at i + j (nx + 1); y face (i, j), i in 0..nx-1,
// j in 0..ny, at i + j nx.  Each face is written once, by the tile of the cell
// on its high side (the domain's last face by the last tile); wall faces are
// not written (the reverse skips them).  Slope records: per direction the
// three van Leer slopes (eta, u, v) and their reciprocals 1 / (dm + dp), six
// planes, of the cells the faces use: x slopes of cells i in -1..nx at
// (i + 1) + j (nx + 2), y slopes of cells j in -1..ny at i + (j + 1) nx; each
// written by the tile that owns the cell (ghost cells by the edge tiles).
struct FaceRec {
    static constexpr bool on = true;
    double* f[2];
    unsigned char* fl[2];
    long long plane[2];  // doubles per field plane
    double* sl[2];
    long long slplane[2];
    int nx, ny;
    __device__ __forceinline__ void put_sx(int col, int TXv, int gi, int gj, int k, double s, double rS) const {
        if (gj < 0 || gj >= ny) return;
        const bool own = (col >= 0 && col < TXv) ? (gi <= nx) : (col < 0 ? gi == -1 : gi == nx);
        if (!own) return;
        const long long o = (long long)(gi + 1) + (long long)gj * (nx + 2);
        sl[0][k * slplane[0] + o] = s;
        sl[0][(3 + k) * slplane[0] + o] = rS;
    }
    __device__ __forceinline__ void put_sy(int row, int TYv, int gi, int gj, int k, double s, double rS) const {
        if (gi < 0 || gi >= nx) return;
        const bool own = (row >= 0 && row < TYv) ? (gj <= ny) : (row < 0 ? gj == -1 : gj == ny);
        if (!own) return;
        const long long o = (long long)gi + (long long)(gj + 1) * nx;
        sl[1][k * slplane[1] + o] = s;
        sl[1][(3 + k) * slplane[1] + o] = rS;
    }
    __device__ __forceinline__ void put(int d, long long o, const RoeRecVals& r) const {
        double* b = f[d] + o;
        const long long ps = plane[d];
        b[0] = r.si; b[ps] = r.sj; b[2 * ps] = r.cm; b[3 * ps] = r.rs; b[4 * ps] = r.hrden; b[5 * ps] = r.hrcm;
        b[6 * ps] = r.um; b[7 * ps] = r.vm; b[8 * ps] = r.l0; b[9 * ps] = r.l2; b[10 * ps] = r.a0h;
        b[11 * ps] = r.a1h; b[12 * ps] = r.a2h;
        fl[d][o] = (unsigned char)r.fl;
    }
    __device__ __forceinline__ void put_x(int gi, int gj, const RoeRecVals& r, bool extra) const {
        if (gi < 0 || gi > nx || gj < 0 || gj >= ny || (extra && gi != nx)) return;
        put(0, (long long)gi + (long long)gj * (nx + 1), r);
    }
    __device__ __forceinline__ void put_y(int gi, int gj, const RoeRecVals& r, bool extra) const {
        if (gi < 0 || gi >= nx || gj < 0 || gj > ny || (extra && gj != ny)) return;
        put(1, (long long)gi + (long long)gj * nx, r);
    }
};

// The CFL bound of a block's cells (K cells per thread) with FP64 work only
// where it can decide the maximum.  Each wet cell's rate
// (|u| + c)/dx + (|v| + c)/dy and speed max(|u|, |v|) are first estimated in
// float from the leading bits of h, hu, hv (error below 2^-19 relative); the
// cells within 2^-12 of the block's float maxima, and any whose estimate is not
// finite, are the candidates.  A candidate whose state is bit-identical to the
// first candidate's has that cell's exact contribution, so only the first
// candidate and the candidates that differ from it compute the exact FP64
// contribution (dt_cell_contrib).  The block maxima, flags and the fold are then
// exactly those of computing every cell: the cell holding the true maximum is
// always a candidate.  Warps without such a cell skip the FP64 work, which in
// regions of uniform state (a lake at rest, the still water ahead of a wave)
// is all warps but one.  Cell k of thread t is candidate number k * NTv + t.
// Every thread of the block must call it.
// The threads that run one tile body together (a policy of the body and the
// fold: the whole block, barrier 0).
struct BlockSync {
    __device__ __forceinline__ int tid() const { return threadIdx.x; }
    __device__ __forceinline__ void bar() const { __syncthreads(); }
    __device__ __forceinline__ int slot() const { return 0; }
};

template <int NTv, int K = 1, class Sync = BlockSync, bool FAST = true>
__device__ __forceinline__ void screened_fold(const ScreenCell<double>* c, double dx, double dy, double idx,
                                              double idy, double& rate, double& mv, unsigned& flags,
                                              const Sync& sy = Sync{}) {
    __shared__ float s_r_all[2][NTv / 32], s_m_all[2][NTv / 32];
    __shared__ int s_rep_all[2];
    __shared__ long long s_bits_all[2][3];
    float* s_r = s_r_all[sy.slot()];
    float* s_m = s_m_all[sy.slot()];
    int& s_rep = s_rep_all[sy.slot()];
    long long* s_bits = s_bits_all[sy.slot()];
    const int t = sy.tid();
    bool wet[K], bad[K];
    float r32[K], m32[K], wr = 0.f, wm = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        wet[k] = false;
        r32[k] = 0.f;
        m32[k] = 0.f;
        if (c[k].live) {
            if (c[k].nod) flags |= DTF_NODATA;
            else if (!gt_bits(c[k].h, Cst<double>::tol12_bits)) flags |= DTF_DRY;
            else {
                wet[k] = true;
                const float h = f32_lead(c[k].h), qx = fabsf(f32_lead(c[k].hu)), qy = fabsf(f32_lead(c[k].hv));
                const float rh = rcp_nr(h);
                const float u = qx * rh, v = qy * rh;
                const float cc = fast_sqrt(9.81f * h);
                r32[k] = (u + cc) * f32_lead(idx) + (v + cc) * f32_lead(idy);
                m32[k] = fmaxf(u, v);
            }
        }
        bad[k] = wet[k] && !(r32[k] <= 3.0e38f && m32[k] <= 3.0e38f);  // inf or NaN: decided in FP64
        const float ar = (wet[k] && !bad[k]) ? r32[k] : 0.f, am = (wet[k] && !bad[k]) ? m32[k] : 0.f;
        wr = k ? fmaxf(wr, ar) : ar;
        wm = k ? fmaxf(wm, am) : am;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        wr = fmaxf(wr, __shfl_xor_sync(0xffffffffu, wr, o));
        wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, o));
    }
    if (t == 0) s_rep = K * NTv;
    if ((t & 31) == 0) { s_r[t >> 5] = wr; s_m[t >> 5] = wm; }
    sy.bar();
    float br = 0.f, bm = 0.f;
#pragma unroll
    for (int k = 0; k < NTv / 32; ++k) { br = fmaxf(br, s_r[k]); bm = fmaxf(bm, s_m[k]); }
    const float kr = br * (1.f - 0x1p-12f), km = bm * (1.f - 0x1p-12f);
    bool cand[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        cand[k] = bad[k] || (wet[k] && (r32[k] >= kr || m32[k] >= km));
        if (cand[k]) atomicMin(&s_rep, k * NTv + t);
    }
    sy.bar();
    const int rep = s_rep;
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (k * NTv + t == rep) { s_bits[0] = sbits(c[k].h); s_bits[1] = sbits(c[k].hu); s_bits[2] = sbits(c[k].hv); }
    sy.bar();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const bool same = k * NTv + t != rep && sbits(c[k].h) == s_bits[0] && sbits(c[k].hu) == s_bits[1] &&
                          sbits(c[k].hv) == s_bits[2];
        if (cand[k] && !same) {
            double rc, mc;
            unsigned f = 0;
            dt_cell_contrib<double, FAST>(c[k].h, c[k].hu, c[k].hv, false, dx, dy, idx, idy, rc, mc, f);
            flags |= f;
            rate = nnmax_i(rate, rc);  // non-negative: the integer max is the max either form takes
            mv = nnmax_i(mv, mc);
        }
    }
}

// A thread's share of the next CFL bound, kept across the tiles of a
// persistent block and folded into the accumulator once at the end.
template <class R> struct ThreadFold {
    R rate = R(0), mv = R(0);
    unsigned flags = 0;
};
// ---------------------------------------------------------------------------
// The advance epilogue (EpiOut): eta and the conservation diagnostics of the
// updated state, taken from the values the update stores, so neither needs
// another pass over the level.
// ---------------------------------------------------------------------------
constexpr long long kNodataRoughBits = (long long)0xC0C3878000000000ull;  // -9999.0, the NODATA roughness

// One updated cell.  eta = h + z (AmrMeshState_AMR.cpp:219).  The cell counts
// when its roughness is not NODATA (== -9999) and h > 0
// (AmrMeshState_Utils.cpp:270-283).  Exact form: the reference's terms,
// s_mass = h dA, s_mx = hu dA, s_my = hv dA, s_ke = 0.5 (hu^2 + hv^2) / h dA
// in its types and order (the 0.5 literal is double), as k_diag_partial takes
// them.  FP64 fast form: h, hu, hv and (hu^2 + hv^2) / h through the
// float-seeded reciprocal (2^-44 relative) summed unscaled, dA and 0.5 dA
// applied once per block; the predicates on the integer pipe (a NaN h is not
// counted, as h > 0 is false for it).
template <class R, bool FAST>
__device__ __forceinline__ void epi_cell(const EpiOut<R>& e, int i, int j, R h, R a, R c, R z, R n, DiagAcc& acc) {
    if (e.eta) e.eta[(long long)(i - e.elo0) + (long long)(j - e.elo1) * e.ejs] = h + z;
    if (!e.part) return;
    if constexpr (FAST && sizeof(R) == 8) {
        const long long hb = sbits(h);
        if (sbits(n) != kNodataRoughBits && hb > 0 && hb <= 0x7ff0000000000000ll) {
            acc.m += h;
            acc.px += a;
            acc.py += c;
            acc.ke += fma(a, a, c * c) * rcp_nr(h);
            if ((unsigned long long)hb < acc.mn) acc.mn = (unsigned long long)hb;
        }
    } else {
        if (!(n == R(-9999.0)) && h > R(0)) {
            const R s_mass = h * e.dA, s_mx = a * e.dA, s_my = c * e.dA;
            const R s_ke = 0.5 * (a * a + c * c) / h * e.dA;
            acc.m += s_mass;
            acc.px += s_mx;
            acc.py += s_my;
            acc.ke += s_ke;
            const unsigned long long hb = (unsigned long long)sbits((double)h);
            if (hb < acc.mn) acc.mn = hb;
        }
    }
}

// The block's sums and min of the diagnostics into q[0..4] by a fixed tree.
// The four sums go through scr (4 NTv doubles of shared memory, free when
// called): halved in place, row n + k into row k, while more than a warp's
// worth is left, then one warp's shuffles; each level is full-width warp
// instructions on the FP64 pipe, about 4 NTv / 32 of them in all instead of
// five shuffle levels in every warp.  min h is taken on the bits (the values
// are positive doubles, ordered as integers) on the integer pipe.  The sums
// are scaled by sm (mass, momenta) and sk (kinetic energy) at the end.  Every
// thread of the block calls it.
template <int NTv>
__device__ __forceinline__ void diag_block_store(double m, double px, double py, double ke, double mn, double* q,
                                                 double* scr, double sm = 1.0, double sk = 1.0) {
    static_assert(NTv % 32 == 0 && (NTv & (NTv - 1)) == 0, "a power-of-two block of whole warps");
    __shared__ long long s_mn[NTv / 32];
    const int t = threadIdx.x;
    scr[t] = m;
    scr[NTv + t] = px;
    scr[2 * NTv + t] = py;
    scr[3 * NTv + t] = ke;
    long long mb = sbits(mn);
    for (int o = 16; o > 0; o >>= 1) {
        const long long x = __shfl_xor_sync(0xffffffffu, mb, o);
        mb = x < mb ? x : mb;
    }
    if ((t & 31) == 0) s_mn[t >> 5] = mb;
    __syncthreads();
#pragma unroll
    for (int n = NTv / 2; n >= 32; n >>= 1) {
        if (t < n)
            for (int c = 0; c < 4; ++c) scr[c * NTv + t] += scr[c * NTv + t + n];
        __syncthreads();
    }
    if (t < 32) {
        double v[4];
        for (int c = 0; c < 4; ++c) v[c] = scr[c * NTv + t];
        long long mm = t < NTv / 32 ? s_mn[t] : 0x7fffffffffffffffll;
        for (int o = 16; o > 0; o >>= 1) {
            for (int c = 0; c < 4; ++c) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
            const long long x = __shfl_xor_sync(0xffffffffu, mm, o);
            mm = x < mm ? x : mm;
        }
        if (t == 0) {
            q[0] = v[0] * sm; q[1] = v[1] * sm; q[2] = v[2] * sm; q[3] = v[3] * sk;
            q[4] = __longlong_as_double(mm);
        }
    }
}
// scr: shared memory the caller no longer reads (the tile kernels pass their
// tile arrays; the call starts with a barrier so no thread still reads them).
template <class R, bool FAST, int NTv>
__device__ __forceinline__ void epi_block_store(const EpiOut<R>& e, const DiagAcc& acc, long long slot, double* scr) {
    constexpr bool SCALED = FAST && sizeof(R) == 8;
    const double dA = (double)e.dA;
    // no cell counted: the reference's initial min, std::numeric_limits<R>::max()
    const double mn = acc.mn == DiagAcc{}.mn ? (double)Cst<R>::max_value : __longlong_as_double((long long)acc.mn);
    __syncthreads();
    diag_block_store<NTv>(acc.m, acc.px, acc.py, acc.ke, mn, e.part + 5 * slot, scr, SCALED ? dA : 1.0,
                          SCALED ? 0.5 * dA : 1.0);
}

// Points in the tile body where a persistent kernel does its own work: after
// the grown tile is loaded (every thread, before the barrier that ends phase A)
// and after the faces are computed (every thread, after the barrier that ends
// phase C, when the grown-tile and slope arrays are dead).
struct NoHooks {
    __device__ __forceinline__ void after_load() const {}
    __device__ __forceinline__ void faces_done() const {}
    __device__ __forceinline__ void after_faces() const {}
};

template <class R, bool FAST, int TXv, int TYv, int NTv, class Src, bool LINEAR = false, class Div = NoDiv,
          class Rec = NoRec, class UO = Cells3<R>, class NP = Plane<R>, class Hooks = NoHooks, class Sync = BlockSync,
          bool EPI = false>
__device__ __forceinline__ void hydro_tile_body(HydroSmem<R, TXv, TYv>& S, const Src& src, const UO& uo,
                                                const NP& nplane, const Cells3W<R>& out, const FaceOut<R>& fo,
                                                const IBox& vb, int x0, int y0, R dt, R dx, R dy, DtAccum* dt_out,
                                                unsigned* status, unsigned* post_flags = nullptr,
                                                const Div& div = Div{}, const Rec& rec = Rec{},
                                                const Hooks& hooks = Hooks{}, ThreadFold<R>* defer = nullptr,
                                                const Sync& sy = Sync{}, bool start_barrier = true,
                                                const EpiOut<R>* epi = nullptr, DiagAcc* eacc = nullptr,
                                                bool set_kc = true) {
    static_assert(!Rec::on || (FAST && sizeof(R) == 8), "face records are kept for the FP64 fast form");
    static_assert(!EPI || (!LINEAR && !Div::on), "the epilogue follows a whole update");
    constexpr int GX = HydroSmem<R, TXv, TYv>::GX, GY = HydroSmem<R, TXv, TYv>::GY;
    constexpr int CELLS = TXv * TYv;
    const int t = sy.tid();
    if (start_barrier) sy.bar();  // the previous tile of this block is done with S (else the caller synced)
    if (set_kc && t == 0) {  // read after the barriers below (a persistent caller sets them once)
        S.kc[0] = dt / dx;
        S.kc[1] = dt / dy;
        S.kc[2] = R(1) / dx;
        S.kc[3] = R(1) / dy;
    }

    // --- A: grown tile -> h rebuilt, eta = h + z, velocities -----------------
    // The fast form takes the stored depth of a cell of the level as it is (sources with an interior fetch):
    // the reference's rebuild max(0, (h + z) - z) differs from it by rounding only.  Tiles whose grown region
    // lies inside the level skip the ghost rules altogether.
    bool interior = false;
    if constexpr (FAST && InteriorFetch<Src>::value)
        interior = src.interior(x0 - 2, y0 - 2, x0 + TXv + 1, y0 + TYv + 1);
    if constexpr (FAST && InteriorFetch<Src>::value) {
        if (interior) {
            for (int idx = t; idx < GX * GY; idx += NTv) {
                const int r = idx / GX, c = idx - r * GX;
                R hh, zz, qx, qy;
                src.fetch_in(x0 + c - 2, y0 + r - 2, hh, zz, qx, qy);
                const R hp = max0_i(hh);
                const R rh = gt_bits(hp, Cst<R>::tol12_bits) ? rcp_nr(hp) : R(0);
                S.nod[r][c] = is_nodata(zz) ? 1 : 0;
                S.z[r][c] = zz;
                S.eta[r][c] = hp + zz;
                S.u[r][c] = qx * rh;
                S.v[r][c] = qy * rh;
            }
        }
    }
    for (int idx = interior ? GX * GY : t; idx < GX * GY; idx += NTv) {
        const int r = idx / GX, c = idx - r * GX;
        const int gi = x0 + c - 2, gj = y0 + r - 2;
        R e = R(0), zz = R(0), qx = R(0), qy = R(0), nn = R(0);
        // the same rule per cell on tiles at the level's edge: a cell of the level takes its stored depth, so
        // the result does not depend on where the tiles lie (a multi-box level tiles each box from its corner)
        bool stored = false;
        if constexpr (FAST && InteriorFetch<Src>::value) stored = src.interior(gi, gj, gi, gj);
        if (stored) {
            if constexpr (FAST && InteriorFetch<Src>::value) src.fetch_in(gi, gj, e, zz, qx, qy);  // e: h
        } else if (src.inside(gi, gj)) {
            src.fetch(gi, gj, e, zz, qx, qy, nn);
        }
        R hp, uu, vv;
        if constexpr (!FAST) {
            hp = max0(e - zz);  // HydrostaticRoe.cpp:498
            uu = (hp > Cst<R>::tol12) ? qx / hp : R(0);
            vv = (hp > Cst<R>::tol12) ? qy / hp : R(0);
        } else {
            hp = stored ? max0_i(e) : max0_i(e - zz);
            const R rh = gt_bits(hp, Cst<R>::tol12_bits) ? rcp_nr(hp) : R(0);
            uu = qx * rh;
            vv = qy * rh;
        }
        S.nod[r][c] = is_nodata(zz) ? 1 : 0;
        S.z[r][c] = zz;
        S.eta[r][c] = hp + zz;  // HydrostaticRoe.cpp:257-260
        S.u[r][c] = uu;
        S.v[r][c] = vv;
    }
    hooks.after_load();
    sy.bar();

    // --- B: van Leer slopes, once per cell and direction ---------------------
    auto xslopes = [&](int row, int col) {  // tile cell (col, row), col in -1..TXv
        const int r = row + 2, c = col + 2;
        if constexpr (Rec::on) {
            double rs0, rs1, rs2;
            const double s0 = van_leer_slope_rs(S.eta[r][c - 1], S.eta[r][c], S.eta[r][c + 1], rs0);
            const double s1 = van_leer_slope_rs(S.u[r][c - 1], S.u[r][c], S.u[r][c + 1], rs1);
            const double s2 = van_leer_slope_rs(S.v[r][c - 1], S.v[r][c], S.v[r][c + 1], rs2);
            S.sxe[row][col + 1] = s0; S.sxu[row][col + 1] = s1; S.sxv[row][col + 1] = s2;
            const int gi = x0 + col, gj = y0 + row;
            rec.put_sx(col, TXv, gi, gj, 0, s0, rs0);
            rec.put_sx(col, TXv, gi, gj, 1, s1, rs1);
            rec.put_sx(col, TXv, gi, gj, 2, s2, rs2);
        } else {
            S.sxe[row][col + 1] = van_leer_slope<R, FAST>(S.eta[r][c - 1], S.eta[r][c], S.eta[r][c + 1]);
            S.sxu[row][col + 1] = van_leer_slope<R, FAST>(S.u[r][c - 1], S.u[r][c], S.u[r][c + 1]);
            S.sxv[row][col + 1] = van_leer_slope<R, FAST>(S.v[r][c - 1], S.v[r][c], S.v[r][c + 1]);
        }
    };
    auto yslopes = [&](int row, int col) {  // row in -1..TYv
        const int r = row + 2, c = col + 2;
        if constexpr (Rec::on) {
            double rs0, rs1, rs2;
            const double s0 = van_leer_slope_rs(S.eta[r - 1][c], S.eta[r][c], S.eta[r + 1][c], rs0);
            const double s1 = van_leer_slope_rs(S.u[r - 1][c], S.u[r][c], S.u[r + 1][c], rs1);
            const double s2 = van_leer_slope_rs(S.v[r - 1][c], S.v[r][c], S.v[r + 1][c], rs2);
            S.sye[row + 1][col] = s0; S.syu[row + 1][col] = s1; S.syv[row + 1][col] = s2;
            const int gi = x0 + col, gj = y0 + row;
            rec.put_sy(row, TYv, gi, gj, 0, s0, rs0);
            rec.put_sy(row, TYv, gi, gj, 1, s1, rs1);
            rec.put_sy(row, TYv, gi, gj, 2, s2, rs2);
        } else {
            S.sye[row + 1][col] = van_leer_slope<R, FAST>(S.eta[r - 1][c], S.eta[r][c], S.eta[r + 1][c]);
            S.syu[row + 1][col] = van_leer_slope<R, FAST>(S.u[r - 1][c], S.u[r][c], S.u[r + 1][c]);
            S.syv[row + 1][col] = van_leer_slope<R, FAST>(S.v[r - 1][c], S.v[r][c], S.v[r + 1][c]);
        }
    };
    for (int k = t; k < CELLS; k += NTv) {
        xslopes(k / TXv, k % TXv);
        yslopes(k / TXv, k % TXv);
    }
    for (int k = t; k < 2 * TYv + 2 * TXv; k += NTv) {
        if (k < 2 * TYv) xslopes(k % TYv, (k < TYv) ? -1 : TXv);  // columns -1 and TX
        else {
            const int m = k - 2 * TYv;
            yslopes((m < TXv) ? -1 : TYv, m % TXv);                // rows -1 and TY
        }
    }
    sy.bar();

    // --- C: faces.  The x face at the left of each cell and the y face below
    // it, then the right column and the top row. ------------------------------
    auto xface = [&](int fi, int fj) {
        const int r = fj + 2, cl = fi + 1, cr = fi + 2;
        R F0, Fa, Fb, Fc;
        const bool wall = S.nod[r][cl] | S.nod[r][cr];
        if constexpr (Rec::on) {
            RoeRecVals rv;
            hydro_face<R, FAST, 0, true>(wall, S.z[r][cl], S.z[r][cr], S.eta[r][cl], S.eta[r][cr], S.sxe[fj][fi],
                                         S.sxe[fj][fi + 1], S.u[r][cl], S.u[r][cr], S.sxu[fj][fi], S.sxu[fj][fi + 1],
                                         S.v[r][cl], S.v[r][cr], S.sxv[fj][fi], S.sxv[fj][fi + 1], F0, Fa, Fb, Fc,
                                         &rv);
            if (!wall) rec.put_x(x0 + fi, y0 + fj, rv, fi == TXv);
        } else {
            hydro_face<R, FAST, 0>(wall, S.z[r][cl], S.z[r][cr], S.eta[r][cl], S.eta[r][cr], S.sxe[fj][fi],
                                   S.sxe[fj][fi + 1], S.u[r][cl], S.u[r][cr], S.sxu[fj][fi], S.sxu[fj][fi + 1],
                                   S.v[r][cl], S.v[r][cr], S.sxv[fj][fi], S.sxv[fj][fi + 1], F0, Fa, Fb, Fc);
        }
        S.fx[0][fj][fi] = F0; S.fx[1][fj][fi] = Fa; S.fx[2][fj][fi] = Fb; S.fx[3][fj][fi] = Fc;
        fo.store_x(x0 + fi, y0 + fj, vb, F0, Fa, Fb, Fc, fi == TXv);
    };
    auto yface = [&](int fi, int fj) {
        const int c = fi + 2, rl = fj + 1, rr = fj + 2;
        R F0, Fa, Fb, Fc;
        const bool wall = S.nod[rl][c] | S.nod[rr][c];
        if constexpr (Rec::on) {
            RoeRecVals rv;
            hydro_face<R, FAST, 1, true>(wall, S.z[rl][c], S.z[rr][c], S.eta[rl][c], S.eta[rr][c], S.sye[fj][fi],
                                         S.sye[fj + 1][fi], S.u[rl][c], S.u[rr][c], S.syu[fj][fi], S.syu[fj + 1][fi],
                                         S.v[rl][c], S.v[rr][c], S.syv[fj][fi], S.syv[fj + 1][fi], F0, Fa, Fb, Fc,
                                         &rv);
            if (!wall) rec.put_y(x0 + fi, y0 + fj, rv, fj == TYv);
        } else {
            hydro_face<R, FAST, 1>(wall, S.z[rl][c], S.z[rr][c], S.eta[rl][c], S.eta[rr][c], S.sye[fj][fi],
                                   S.sye[fj + 1][fi], S.u[rl][c], S.u[rr][c], S.syu[fj][fi], S.syu[fj + 1][fi],
                                   S.v[rl][c], S.v[rr][c], S.syv[fj][fi], S.syv[fj + 1][fi], F0, Fa, Fb, Fc);
        }
        S.fy[0][fj][fi] = F0; S.fy[1][fj][fi] = Fa; S.fy[2][fj][fi] = Fb; S.fy[3][fj][fi] = Fc;
        fo.store_y(x0 + fi, y0 + fj, vb, F0, Fa, Fb, Fc, fj == TYv);
    };
    for (int k = t; k < CELLS; k += NTv) {
        const int tx = k % TXv, ty = k / TXv;
        const int gi = x0 + tx, gj = y0 + ty;
        // a face is needed if it bounds a valid cell
        if (gi <= vb.hi0 + 1 && gj <= vb.hi1) xface(tx, ty);
        if (gi <= vb.hi0 && gj <= vb.hi1 + 1) yface(tx, ty);
    }
    // the right column and the top row: where the tile leaves enough threads without a cell, those take them
    // (two faces at most, as every other thread), so that no thread computes a third face while the rest wait
    constexpr int SPARE = NTv - CELLS;
    if constexpr (SPARE >= TXv && SPARE >= TYv) {
        const int e = t - CELLS;
        if (e >= 0) {
            if (e < TYv && x0 + TXv <= vb.hi0 + 1 && y0 + e <= vb.hi1) xface(TXv, e);
            if (e < TXv && x0 + e <= vb.hi0 && y0 + TYv <= vb.hi1 + 1) yface(e, TYv);
        }
    } else {
        for (int k = t; k < TYv + TXv; k += NTv) {
            if (k < TYv) {
                if (x0 + TXv <= vb.hi0 + 1 && y0 + k <= vb.hi1) xface(TXv, k);
            } else {
                const int m = k - TYv;
                if (x0 + m <= vb.hi0 && y0 + TYv <= vb.hi1 + 1) yface(m, TYv);
            }
        }
    }
    hooks.faces_done();
    sy.bar();
    hooks.after_faces();

    // --- D: update, Manning friction, dry clamp (HydrostaticRoe.cpp:551-604) --
    R rate = R(0), mv = R(0);
    unsigned flags = 0, pflags = 0;
    const R cx = S.kc[0], cy = S.kc[1], idx = S.kc[2], idy = S.kc[3];
    // FP64 folds the next CFL bound through the float screen (the candidates in the form's own arithmetic)
    constexpr bool SCREEN = sizeof(R) == 8 && CELLS <= NTv && !LINEAR && !Div::on;  // at most a cell a thread
    const bool fold = dt_out != nullptr || defer != nullptr;
    ScreenCell<R> sc;
    for (int k = t; k < CELLS; k += NTv) {
        const int tx = k % TXv, ty = k / TXv;
        const int gi = x0 + tx, gj = y0 + ty;
        if (gi > vb.hi0 || gj > vb.hi1) continue;
        const R dx0 = S.fx[0][ty][tx + 1] - S.fx[0][ty][tx];
        const R dx1 = S.fx[1][ty][tx + 1] - S.fx[2][ty][tx];
        const R dx2 = S.fx[3][ty][tx + 1] - S.fx[3][ty][tx];
        const R dy0 = S.fy[0][ty + 1][tx] - S.fy[0][ty][tx];
        const R dy1 = S.fy[1][ty + 1][tx] - S.fy[1][ty][tx];
        const R dy2 = S.fy[2][ty + 1][tx] - S.fy[3][ty][tx];
        if constexpr (Div::on) {  // the flux differences only: the update waits for dt
            div.st(gi, gj, dx0, dx1, dx2, dy0, dy1, dy2);
            continue;
        }
        const R o0 = uo.ld(0, gi, gj), o1 = uo.ld(1, gi, gj), o2 = uo.ld(2, gi, gj);
        step_cell<R, FAST, LINEAR, NP>(o0, o1, o2, dx0, dx1, dx2, dy0, dy1, dy2, cx, cy, dt, nplane, out, gi, gj,
                                   S.nod[ty + 2][tx + 2] != 0, dx, dy, idx, idy, fold && !SCREEN, rate, mv, flags,
                                   pflags, ((SCREEN && fold) || EPI) ? &sc : nullptr);
        if constexpr (EPI) epi_cell<R, FAST>(*epi, gi, gj, sc.h, sc.hu, sc.hv, S.z[ty + 2][tx + 2], nplane.ld(gi, gj), *eacc);
    }
    if constexpr (SCREEN) {
        if (fold) screened_fold<NTv, 1, Sync, FAST>(&sc, dx, dy, idx, idy, rate, mv, flags, sy);
    }
    if (defer) {
        if constexpr (FAST) {
            defer->rate = nnmax_i(defer->rate, rate);
            defer->mv = nnmax_i(defer->mv, mv);
        } else {
            defer->rate = smax(defer->rate, rate);
            defer->mv = smax(defer->mv, mv);
        }
        defer->flags |= flags;
    } else if (dt_out) {
        block_fold_dt<R, NTv>(rate, mv, flags, dt_out);
    }
    if ((flags & DTF_NAN) && status) atomicOr(status, (unsigned)HX_STATUS_NAN);
    if (post_flags) {
        pflags = __reduce_or_sync(0xffffffffu, pflags);
        if (pflags && (threadIdx.x & 31) == 0) atomicOr(post_flags, pflags);
    }
}

// Tile shapes of the level kernels, one cell per thread.  FP64 is bound by
// FP64 issue: a 32 x 32 tile loads 1.27 cells, computes 6.4 slopes and 2.06
// faces per cell (32 x 8: 1.69, 6.9, 2.16) and runs ~9% faster on large boxes
// (one CTA of 1024 threads per SM).  On boxes of a few waves the four 32 x 8
// CTAs per SM overlap each other's barriers and win, and FP32 (bound by issue
// of every kind) always prefers them.
template <class R> struct BigTile {
    static constexpr int X = 32, Y = 32;
};
template <> struct BigTile<float> {
    static constexpr int X = 32, Y = 8;
};
// Resident CTAs per SM the tile kernels are compiled for: 1024-thread tiles
// one, 512-thread tiles two, 256-thread tiles three (85 registers; four, at
// 64, spill in the exact form and moved the fast form's small levels by 1%).
constexpr int min_ctas(int threads) { return threads >= 1024 ? 1 : (threads >= 512 ? 2 : 3); }
struct SmallTile {
    static constexpr int X = TX, Y = TY;
};
template <class R> inline bool big_tile(const IBox& vb) {
    return BigTile<R>::Y != TY &&
           (long long)(vb.hi0 - vb.lo0 + 1) * (long long)(vb.hi1 - vb.lo1 + 1) >= kBigTileCells;
}

// EPI: the advance epilogue (eta and this tile's diagnostics partial, slot =
// the block's linear index).
template <class R, bool FAST, class Src, int TXH = TX, int TYH = TY, bool EPI = false>
__global__ void __launch_bounds__(TXH * TYH, min_ctas(TXH * TYH))
    k_hydro_tile(Src src, Cells3<R> uo, Plane<R> nplane, Cells3W<R> out, FaceOut<R> fo, IBox vb, StepCtl<R> ctl,
                 EpiOut<R> epi) {
    static_assert(!EPI || sizeof(HydroSmem<R, TXH, TYH>) >= 4 * TXH * TYH * sizeof(double),
                  "the epilogue's block sums reuse the tile arrays");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HydroSmem<R, TXH, TYH>& S = *reinterpret_cast<HydroSmem<R, TXH, TYH>*>(smem_raw);
    R dt;
    if (!resolve_dt(ctl, dt)) return;
    step_bookkeeping(ctl, dt);
    DiagAcc acc;
    hydro_tile_body<R, FAST, TXH, TYH, TXH * TYH, Src, false, NoDiv, NoRec, Cells3<R>, Plane<R>, NoHooks, BlockSync,
                    EPI>(S, src, uo, nplane, out, fo, vb, vb.lo0 + (int)blockIdx.x * TXH,
                         vb.lo1 + (int)blockIdx.y * TYH, dt, ctl.dx, ctl.dy, ctl.dt_out, ctl.status, nullptr,
                         NoDiv{}, NoRec{}, NoHooks{}, nullptr, BlockSync{}, true, &epi, &acc);
    if constexpr (EPI) {
        if (epi.part)
            epi_block_store<R, FAST, TXH * TYH>(epi, acc, blockIdx.x + (long long)blockIdx.y * gridDim.x,
                                                reinterpret_cast<double*>(smem_raw));
    }
}

// ---------------------------------------------------------------------------
// The persistent FP64 level step on 32 x 32 tiles.  One block of 1024 threads
// per SM walks its tiles (k = blockIdx.x, blockIdx.x + gridDim.x, ...; row-major
// over the box, so the blocks in flight share halo rows in L2).  The grown tile
// of the next tile -- h, hu, hv, z of its in-level cells and the roughness of
// its own cells -- is copied into shared memory by cp.async while the current
// tile is updated, so phase A reads shared memory and the global-load latency
// is hidden under the update's FP64 work.  The staging buffer lies on the slope
// arrays, which are dead from the end of phase C of one tile to phase B of the
// next; the own cells' stored state and roughness, which the update reads, are
// copied out of it during phase A.  Ghosts outside the level are resolved from
// staged in-level cells by the rules of ghost_source (a tile touching a
// boundary holds the cells its ghosts mirror or copy), so every value is the
// one LevelSrc::fetch reads and the arithmetic is k_hydro_tile's, bit for bit.
// The next CFL bound is folded per thread across the block's tiles and into
// the accumulator once.
// ---------------------------------------------------------------------------
constexpr int kPX = 32, kPY = 32;              // tile
constexpr int kPGX = kPX + 4, kPGY = kPY + 4;  // grown tile (2-cell MUSCL halo)
constexpr int kPN = 1024;                      // threads of the block, one cell each at most
struct PersistStaging {
    double h[kPGY][kPGX], hu[kPGY][kPGX], hv[kPGY][kPGX], z[kPGY][kPGX];
    double n[kPY][kPX];
};
struct PersistOwn {
    double h[kPX * kPY], hu[kPX * kPY], hv[kPX * kPY], n[kPX * kPY];
    ThreadFold<double> fold[kPN];  // each thread's share of the next CFL bound (kept out of registers)
    unsigned long long mbar;       // completion barrier of the TMA staging
};
static_assert(kPX * kPY <= kPN, "one cell per thread at most");
static_assert(sizeof(HydroSmem<double, kPX, kPY>) >= 4 * kPN * sizeof(double),
              "the epilogue's block sums reuse the tile arrays");
static_assert(sizeof(PersistStaging) <= sizeof(double) * 3 * (kPY * (kPX + 2) + (kPY + 2) * kPX),
              "the staging buffer must fit in the slope arrays it lies on");
// (+128: the staging arrays start on a 128-byte boundary, which the kernel rounds its shared base up to)
constexpr size_t persist_smem_bytes() { return sizeof(HydroSmem<double, kPX, kPY>) + sizeof(PersistOwn) + 128; }
static_assert(sizeof(double) * 4 * kPGX * kPGY % 128 == 0, "the staging buffer starts 128-byte aligned");
static_assert(sizeof(double) * kPGX * kPGY % 128 == 0 && sizeof(double) * kPGX % 16 == 0,
              "each staged plane starts 128-byte aligned; a staged row is a whole number of 16-byte units");

// Tensor maps of the level's planes for the TMA staging: h, hu, hv, z in 36 x 36 boxes (the grown tile),
// n in 32 x 32 boxes (the own cells).  valid = 0: the planes do not meet TMA's alignment (16-byte base
// and row pitch); the kernel stages by cp.async instead.
struct PersistMaps {
    CUtensorMap h, hu, hv, z, n;
    int valid;
    unsigned extra_tx;  // added to the expected bytes: nonzero only to test the bounded wait (it then runs out)
};
constexpr unsigned kStageBytes = (unsigned)(sizeof(double) * (4 * kPGX * kPGY + kPX * kPY));

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Waits for the phase of the given parity to complete, for one second at most by the global timer (each
// try_wait suspends for a bounded, hardware-chosen time, and at most 2^24 of them are tried); false when
// it did not.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
    const unsigned long long t0 = global_ns();
    for (int k = 0; k < (1 << 24); ++k) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > 1000000000ull) break;
    }
    return false;
}
// One 2D tile of a tensor map into shared memory; its bytes complete the barrier's transaction count.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
// Thread 0: the five planes of tile (x0, y0).  x0 is a multiple of 32, so the grown box's x = x0 - 2 is
// even: 16-byte aligned in doubles, as TMA requires of the innermost coordinate.  Boxes reaching past the
// level are filled with zeros there; nothing reads those cells (ghosts are resolved to level cells).
__device__ __forceinline__ void persist_stage_tma(PersistStaging* st, const PersistMaps& m, int x0, int y0,
                                                  unsigned long long* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(kStageBytes + m.extra_tx)
                 : "memory");
    tma_load_2d(&st->h[0][0], &m.h, x0 - 2, y0 - 2, bar);
    tma_load_2d(&st->hu[0][0], &m.hu, x0 - 2, y0 - 2, bar);
    tma_load_2d(&st->hv[0][0], &m.hv, x0 - 2, y0 - 2, bar);
    tma_load_2d(&st->z[0][0], &m.z, x0 - 2, y0 - 2, bar);
    tma_load_2d(&st->n[0][0], &m.n, x0, y0, bar);
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Issue the copies of tile (x0, y0) into st (every thread of the block).
__device__ __forceinline__ void persist_stage(PersistStaging* st, const LevelSrc<double>& src, int x0, int y0) {
    const int t = threadIdx.x;
    for (int idx = t; idx < kPGX * kPGY; idx += kPN) {
        const int r = idx / kPGX, c = idx - r * kPGX;
        const int gi = x0 - 2 + c, gj = y0 - 2 + r;
        if (gi < 0 || gi >= src.nx || gj < 0 || gj >= src.ny) continue;
        const long long o = (long long)gi + (long long)gj * src.pitch;
        cp_async8(&st->h[r][c], src.h + o);
        cp_async8(&st->hu[r][c], src.hu + o);
        cp_async8(&st->hv[r][c], src.hv + o);
        cp_async8(&st->z[r][c], src.z + o);
    }
    const int r = t / kPX, c = t % kPX, gi = x0 + c, gj = y0 + r;
    if (t < kPX * kPY && gi < src.nx && gj < src.ny)
        cp_async8(&st->n[r][c], src.n + (long long)gi + (long long)gj * src.pitch);
    cp_async_commit();
}

// Phase A's source: the staged grown tile, ghosts resolved as LevelSrc does.
struct StagedSrc {
    static constexpr bool kInterior = true;  // has interior() / fetch_in()
    const PersistStaging* st;
    int x0, y0, nx, ny;
    int bc_xlo, bc_xhi, bc_ylo, bc_yhi;
    int glo0, glo1, ghi0, ghi1;
    __device__ __forceinline__ bool inside(int i, int j) const {
        return i >= glo0 && i <= ghi0 && j >= glo1 && j <= ghi1;
    }
    // true when cells (i0, j0) .. (i1, j1) all lie in the level
    __device__ __forceinline__ bool interior(int i0, int j0, int i1, int j1) const {
        return i0 >= 0 && j0 >= 0 && i1 < nx && j1 < ny;
    }
    // (h, z, hu, hv) of a cell of the level, as stored
    __device__ __forceinline__ void fetch_in(int i, int j, double& h, double& zz, double& qx, double& qy) const {
        const int r = j - y0 + 2, c = i - x0 + 2;
        h = st->h[r][c];
        zz = st->z[r][c];
        qx = st->hu[r][c];
        qy = st->hv[r][c];
    }
    __device__ __forceinline__ void fetch(int i, int j, double& eta, double& zz, double& qx, double& qy,
                                          double& nn) const {
        int mi, mj, ei, ej;
        bool neg_u, neg_v;
        ghost_source(i, j, nx, ny, bc_xlo, bc_xhi, bc_ylo, bc_yhi, mi, mj, ei, ej, neg_u, neg_v);
        const int mr = mj - y0 + 2, mc = mi - x0 + 2, er = ej - y0 + 2, ec = ei - x0 + 2;
        eta = st->h[mr][mc] + st->z[mr][mc];
        zz = st->z[er][ec];
        nn = 0.0;
        const double a = st->hu[mr][mc], b = st->hv[mr][mc];
        qx = neg_u ? -a : a;
        qy = neg_v ? -b : b;
    }
};
// The update's stored state and roughness of the tile's own cells.
struct OwnState {
    const PersistOwn* o;
    int x0, y0;
    __device__ __forceinline__ double ld(int c, int i, int j) const {
        const int k = (j - y0) * kPX + (i - x0);
        return c == 0 ? o->h[k] : (c == 1 ? o->hu[k] : o->hv[k]);
    }
};
struct OwnRough {
    const PersistOwn* o;
    int x0, y0;
    __device__ __forceinline__ double ld(int i, int j) const { return o->n[(j - y0) * kPX + (i - x0)]; }
};
// The own cells' stored state and roughness, out of the staging buffer (phase A, each thread its own cell).
__device__ __forceinline__ void persist_own_copy(const PersistStaging* st, PersistOwn* own) {
    const int t = threadIdx.x, r = t / kPX + 2, c = t % kPX + 2;
    if (t >= kPX * kPY) return;
    own->h[t] = st->h[r][c];
    own->hu[t] = st->hu[r][c];
    own->hv[t] = st->hv[r][c];
    own->n[t] = st->n[r - 2][c - 2];
}
struct PersistHooks {
    PersistStaging* st;
    PersistOwn* own;
    const LevelSrc<double>* src;
    const PersistMaps* maps;  // null: cp.async staging
    int nx0, ny0;  // origin of the next tile
    bool next;
    __device__ __forceinline__ void after_load() const { persist_own_copy(st, own); }
    // the staging buffer lies on the slope arrays: order this thread's accesses to them (generic proxy)
    // before the TMA writes (async proxy) that the next tile's staging issues after the barrier
    __device__ __forceinline__ void faces_done() const {
        if (maps) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __device__ __forceinline__ void after_faces() const {
        if (!next) return;
        if (maps) {
            if (threadIdx.x == 0) persist_stage_tma(st, *maps, nx0, ny0, &own->mbar);
        } else {
            persist_stage(st, *src, nx0, ny0);
        }
    }
};

// With Div = DivOut<double> the kernel writes the flux differences of every
// cell instead of the update (the first step of the host-buffer call, whose
// update waits for the level's dt): no dt, no CFL fold.
// The next tile is staged by TMA (five 2D tensor-map loads issued by one thread, completing on an mbarrier)
// when the planes allow it (maps.valid), else by cp.async from every thread.  A TMA wait that runs out
// (about a second) sets HX_STATUS_STAGING_TIMEOUT and ends the block's work after a second bounded wait for
// the copies in flight.
// EPI: the advance epilogue, each thread's diagnostics summed over its cells of
// every tile of the block and the block's partial stored at slot blockIdx.x
// (NaN when the block gave up on a staging wait).
template <bool FAST, class Div = NoDiv, bool EPI = false>
__global__ void __launch_bounds__(kPN, 1)
    k_hydro_persist(LevelSrc<double> src, Cells3W<double> out, IBox vb, int tiles_x, int ntiles,
                    StepCtl<double> ctl, Div div, const __grid_constant__ PersistMaps maps, unsigned* err,
                    EpiOut<double> epi) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // 128-byte aligned
    HydroSmem<double, kPX, kPY>& S = *reinterpret_cast<HydroSmem<double, kPX, kPY>*>(base);
    PersistOwn* own = reinterpret_cast<PersistOwn*>(base + sizeof(HydroSmem<double, kPX, kPY>));
    PersistStaging* st = reinterpret_cast<PersistStaging*>(&S.sxe[0][0]);
    double dt = 0.0;
    if constexpr (!Div::on) {
        if (!resolve_dt(ctl, dt)) return;
        step_bookkeeping(ctl, dt);
    }
    const bool fold = !Div::on && ctl.dt_out != nullptr;
    int k = (int)blockIdx.x;
    if (k >= ntiles) return;
    const bool tma = maps.valid != 0;
    if (tma) {
        if (threadIdx.x == 0) {
            mbar_init(&own->mbar);
            persist_stage_tma(st, maps, vb.lo0 + (k % tiles_x) * kPX, vb.lo1 + (k / tiles_x) * kPY, &own->mbar);
        }
        __syncthreads();  // the barrier is initialised before any thread waits on it
    } else {
        persist_stage(st, src, vb.lo0 + (k % tiles_x) * kPX, vb.lo1 + (k / tiles_x) * kPY);
    }
    ThreadFold<double>* tf = &own->fold[threadIdx.x];
    *tf = ThreadFold<double>{};
    if (threadIdx.x == 0) {  // the tile body's per-tile constants, the same for every tile of the launch
        S.kc[0] = dt / ctl.dx;
        S.kc[1] = dt / ctl.dy;
        S.kc[2] = 1.0 / ctl.dx;
        S.kc[3] = 1.0 / ctl.dy;
    }
    const FaceOut<double> fo{};
    unsigned parity = 0;
    DiagAcc acc;
    for (; k < ntiles; k += (int)gridDim.x) {
        const int x0 = vb.lo0 + (k % tiles_x) * kPX, y0 = vb.lo1 + (k / tiles_x) * kPY;
        const int kn = k + (int)gridDim.x;
        const PersistHooks hooks{st, own, &src, tma ? &maps : nullptr, vb.lo0 + (kn % tiles_x) * kPX,
                                 vb.lo1 + (kn / tiles_x) * kPY, kn < ntiles};
        const StagedSrc ss{st, x0, y0, src.nx, src.ny, src.bc_xlo, src.bc_xhi, src.bc_ylo, src.bc_yhi,
                           src.glo0, src.glo1, src.ghi0, src.ghi1};
        if (tma) {
            // tile k's planes have landed (the barrier below also ends the previous tile's use of S)
            const bool late = !mbar_wait_bounded(&own->mbar, parity);
            parity ^= 1u;
            if (__syncthreads_or(late)) {
                if (threadIdx.x == 0) {
                    if (err) atomicOr(err, (unsigned)HX_STATUS_STAGING_TIMEOUT);
                    mbar_wait_bounded(&own->mbar, parity ^ 1u);  // the copies in flight, once more
                    if constexpr (EPI) {
                        if (epi.part)
                            for (int c = 0; c < 5; ++c) epi.part[5ll * blockIdx.x + c] = __longlong_as_double(-1ll);
                    }
                }
                __syncthreads();
                return;
            }
        } else {
            cp_async_wait_all();  // this thread's copies of tile k; the body's first barrier publishes everyone's
        }
        hydro_tile_body<double, FAST, kPX, kPY, kPN, StagedSrc, false, Div, NoRec, OwnState, OwnRough,
                        PersistHooks, BlockSync, EPI>(S, ss, OwnState{own, x0, y0}, OwnRough{own, x0, y0}, out, fo,
                                                      vb, x0, y0, dt, ctl.dx, ctl.dy, nullptr,
                                                      Div::on ? nullptr : ctl.status, nullptr, div, NoRec{}, hooks,
                                                      fold ? tf : nullptr, BlockSync{}, !tma, &epi, &acc, false);
    }
    if (fold) block_fold_dt<double, kPN>(tf->rate, tf->mv, tf->flags, ctl.dt_out);
    if constexpr (EPI) {
        if (epi.part) epi_block_store<double, FAST, kPN>(epi, acc, blockIdx.x, reinterpret_cast<double*>(base));
    }
}

// ---------------------------------------------------------------------------
// The persistent step of a multi-box level of 2048^2 cells and more: the tile
// loop of k_hydro_persist over a table of the 32 x 32 tiles of every box.  A
// tile's grown region is staged by cp.async from the boxes that own its cells
// (the map of the domain), its ghosts outside the level are resolved from the
// staged cells, and its update goes to its own box.  The staged values are
// the ones the single-box level stages, and the tile arithmetic is the same,
// so the two give the same state bit for bit.
// ---------------------------------------------------------------------------
// Issue the copies of tile (x0, y0) of box b into st (every thread of the block).
__device__ __forceinline__ void boxset_stage(PersistStaging* st, const BoxSetSrc& s, int b, int x0, int y0) {
    const int t = threadIdx.x;
    const DevBox& B = s.boxes[b];
    for (int idx = t; idx < kPGX * kPGY; idx += kPN) {
        const int r = idx / kPGX, c = idx - r * kPGX;
        const int gi = x0 - 2 + c, gj = y0 - 2 + r;
        if (gi < 0 || gi >= s.nx || gj < 0 || gj >= s.ny) continue;  // a ghost: resolved from staged cells
        const bool mine = gi >= B.lo0 && gi <= B.hi0 && gj >= B.lo1 && gj <= B.hi1;
        const DevBox& O = mine ? B : s.boxes[ld_ro(s.map + (long long)(gj / s.g) * s.mnx + gi / s.g)];
        const long long o = (long long)(gi - O.lo0) + (long long)(gj - O.lo1) * O.pitch;
        cp_async8(&st->h[r][c], O.h[s.phase] + o);
        cp_async8(&st->hu[r][c], O.hu[s.phase] + o);
        cp_async8(&st->hv[r][c], O.hv[s.phase] + o);
        cp_async8(&st->z[r][c], O.z + o);
    }
    const int r = t / kPX, c = t % kPX, gi = x0 + c, gj = y0 + r;
    if (t < kPX * kPY && gi <= B.hi0 && gj <= B.hi1)
        cp_async8(&st->n[r][c], B.n + (long long)(gi - B.lo0) + (long long)(gj - B.lo1) * B.pitch);
    cp_async_commit();
}
struct BoxPersistHooks {
    PersistStaging* st;
    PersistOwn* own;
    const BoxSetSrc* src;
    int nb, nx0, ny0;  // the next tile: its box and origin
    bool next;
    __device__ __forceinline__ void after_load() const { persist_own_copy(st, own); }
    __device__ __forceinline__ void faces_done() const {}
    __device__ __forceinline__ void after_faces() const {
        if (next) boxset_stage(st, *src, nb, nx0, ny0);
    }
};
template <bool FAST>
__global__ void __launch_bounds__(kPN, 1)
    k_boxlevel_persist(BoxSetSrc src, const int* __restrict__ tiles, int ntiles, StepCtl<double> ctl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // 128-byte aligned
    HydroSmem<double, kPX, kPY>& S = *reinterpret_cast<HydroSmem<double, kPX, kPY>*>(base);
    PersistOwn* own = reinterpret_cast<PersistOwn*>(base + sizeof(HydroSmem<double, kPX, kPY>));
    PersistStaging* st = reinterpret_cast<PersistStaging*>(&S.sxe[0][0]);
    double dt;
    if (!resolve_dt(ctl, dt)) return;
    step_bookkeeping(ctl, dt);
    const bool fold = ctl.dt_out != nullptr;
    int k = (int)blockIdx.x;
    if (k >= ntiles) return;
    boxset_stage(st, src, tiles[3 * k], tiles[3 * k + 1], tiles[3 * k + 2]);
    ThreadFold<double>* tf = &own->fold[threadIdx.x];
    *tf = ThreadFold<double>{};
    if (threadIdx.x == 0) {  // the tile body's per-tile constants, the same for every tile of the launch
        S.kc[0] = dt / ctl.dx;
        S.kc[1] = dt / ctl.dy;
        S.kc[2] = 1.0 / ctl.dx;
        S.kc[3] = 1.0 / ctl.dy;
    }
    const FaceOut<double> fo{};
    const int nxt = 1 - src.phase;
    for (; k < ntiles; k += (int)gridDim.x) {
        const int b = tiles[3 * k], x0 = tiles[3 * k + 1], y0 = tiles[3 * k + 2];
        const int kn = k + (int)gridDim.x;
        const bool next = kn < ntiles;
        const BoxPersistHooks hooks{st, own, &src, next ? tiles[3 * kn] : 0, next ? tiles[3 * kn + 1] : 0,
                                    next ? tiles[3 * kn + 2] : 0, next};
        const StagedSrc ss{st, x0, y0, src.nx, src.ny, src.bc_xlo, src.bc_xhi, src.bc_ylo, src.bc_yhi,
                           src.glo0, src.glo1, src.ghi0, src.ghi1};
        const DevBox& B = src.boxes[b];
        Cells3W<double> out;
        out.p[0] = const_cast<double*>(B.h[nxt]);
        out.p[1] = const_cast<double*>(B.hu[nxt]);
        out.p[2] = const_cast<double*>(B.hv[nxt]);
        out.js = B.pitch;
        out.lo0 = B.lo0;
        out.lo1 = B.lo1;
        const IBox vb{B.lo0, B.lo1, B.hi0, B.hi1};
        cp_async_wait_all();  // this thread's copies of tile k; the body's first barrier publishes everyone's
        hydro_tile_body<double, FAST, kPX, kPY, kPN, StagedSrc, false, NoDiv, NoRec, OwnState, OwnRough,
                        BoxPersistHooks>(S, ss, OwnState{own, x0, y0}, OwnRough{own, x0, y0}, out, fo, vb, x0, y0,
                                         dt, ctl.dx, ctl.dy, nullptr, ctl.status, nullptr, NoDiv{}, NoRec{}, hooks,
                                         fold ? tf : nullptr, BlockSync{}, true, nullptr, nullptr, false);
    }
    if (fold) block_fold_dt<double, kPN>(tf->rate, tf->mv, tf->flags, ctl.dt_out);
}

// Extra bytes the next launches' staging waits for (a test setting; 0 in use).
unsigned& staging_test_extra_bytes();

// Tensor maps of the level's planes for k_hydro_persist's TMA staging (host side; valid = 0 where the
// planes do not meet TMA's alignment, or the encoder is unavailable).
inline PersistMaps persist_maps(const LevelSrc<double>& src) {
    PersistMaps m;
    std::memset(&m, 0, sizeof m);
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static const Encode enc = [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        return reinterpret_cast<Encode>(fn);
    }();
    const unsigned long long row = (unsigned long long)src.pitch * sizeof(double);
    const double* planes[5] = {src.h, src.hu, src.hv, src.z, src.n};
    if (!enc || row % 16 != 0) return m;
    for (const double* p : planes)
        if (reinterpret_cast<uintptr_t>(p) % 16 != 0) return m;
    const cuuint64_t dims[2] = {(cuuint64_t)src.nx, (cuuint64_t)src.ny};
    const cuuint64_t strides[1] = {(cuuint64_t)row};
    const cuuint32_t grown[2] = {(cuuint32_t)kPGX, (cuuint32_t)kPGY}, own[2] = {(cuuint32_t)kPX, (cuuint32_t)kPY};
    const cuuint32_t unit[2] = {1, 1};
    CUtensorMap* maps[5] = {&m.h, &m.hu, &m.hv, &m.z, &m.n};
    for (int k = 0; k < 5; ++k) {
        if (enc(maps[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(planes[k]), dims, strides,
                k < 4 ? grown : own, unit, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
            std::memset(&m, 0, sizeof m);
            return m;
        }
    }
    m.valid = 1;
    m.extra_tx = staging_test_extra_bytes();
    return m;
}

// ---------------------------------------------------------------------------
// A hydrostatic step split in two, for a caller that receives its level while
// the step starts (the host-buffer entry): the flux differences of every cell
// need no dt and run band by band as the rows arrive; the update applies dt
// once the CFL bound of the whole level is known.  Together they do exactly
// the fused kernel's arithmetic.
// ---------------------------------------------------------------------------
template <class R, bool FAST, int TXH = TX, int TYH = TY>
__global__ void __launch_bounds__(TXH * TYH, min_ctas(TXH * TYH))
    k_hydro_div(LevelSrc<R> src, Cells3<R> uo, Plane<R> nplane, DivOut<R> div, IBox vb, R dx, R dy) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HydroSmem<R, TXH, TYH>& S = *reinterpret_cast<HydroSmem<R, TXH, TYH>*>(smem_raw);
    FaceOut<R> fo{};
    Cells3W<R> none{};
    hydro_tile_body<R, FAST, TXH, TYH, TXH * TYH, LevelSrc<R>, false, DivOut<R>>(
        S, src, uo, nplane, none, fo, vb, vb.lo0 + (int)blockIdx.x * TXH, vb.lo1 + (int)blockIdx.y * TYH, R(0), dx,
        dy, nullptr, nullptr, nullptr, div);
}

template <class R, bool FAST>
__global__ void __launch_bounds__(NT) k_hydro_update(Cells3<R> uo, DivOut<R> div, Plane<R> nplane, Plane<R> zplane,
                                                     Cells3W<R> out, IBox vb, StepCtl<R> ctl) {
    __shared__ R kc[4];
    R dt;
    if (!resolve_dt(ctl, dt)) return;
    step_bookkeeping(ctl, dt);
    if (threadIdx.x == 0) { kc[0] = dt / ctl.dx; kc[1] = dt / ctl.dy; kc[2] = R(1) / ctl.dx; kc[3] = R(1) / ctl.dy; }
    __syncthreads();
    R rate = R(0), mv = R(0);
    unsigned flags = 0, pflags = 0;
    const int gi = vb.lo0 + (int)blockIdx.x * TX + (threadIdx.x % TX);
    for (int r = 0; r < ROWS_PER_THREAD; ++r) {  // a 32 x (8 ROWS) block: fewer blocks, fewer dt atomics
        const int gj = vb.lo1 + ((int)blockIdx.y * ROWS_PER_THREAD + r) * TY + (threadIdx.x / TX);
        if (gi > vb.hi0 || gj > vb.hi1) continue;
        const long long o = (long long)(gi - div.lo0) + (long long)(gj - div.lo1) * div.js;
        step_cell<R, FAST, false>(uo.ld(0, gi, gj), uo.ld(1, gi, gj), uo.ld(2, gi, gj), div.p[0][o], div.p[1][o],
                                  div.p[2][o], div.p[3][o], div.p[4][o], div.p[5][o], kc[0], kc[1], dt, nplane, out,
                                  gi, gj, is_nodata(zplane.ld(gi, gj)), ctl.dx, ctl.dy, kc[2], kc[3],
                                  ctl.dt_out != nullptr, rate, mv, flags, pflags);
    }
    if (ctl.dt_out) block_fold_dt<R, NT>(rate, mv, flags, ctl.dt_out);
    if ((flags & DTF_NAN) && ctl.status) atomicOr(ctl.status, (unsigned)HX_STATUS_NAN);
}

// ---------------------------------------------------------------------------
// One step of a multi-box level: one block per tile of any box (tiles[k] =
// box, x0, y0), ghosts from the neighbouring boxes (BoxSetSrc), one dt chain.
// ---------------------------------------------------------------------------
template <bool FAST>
__global__ void __launch_bounds__(NT) k_boxlevel_hydro(BoxSetSrc base, const int* tiles, StepCtl<double> ctl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HydroSmem<double>& S = *reinterpret_cast<HydroSmem<double>*>(smem_raw);
    double dt;
    if (!resolve_dt(ctl, dt)) return;
    step_bookkeeping(ctl, dt);
    const int b = tiles[3 * blockIdx.x], x0 = tiles[3 * blockIdx.x + 1], y0 = tiles[3 * blockIdx.x + 2];
    const DevBox& B = base.boxes[b];
    BoxSetSrc src = base;
    src.self = b;
    const int cur = base.phase, nxt = 1 - base.phase;
    Cells3<double> uo;
    uo.p[0] = B.h[cur]; uo.p[1] = B.hu[cur]; uo.p[2] = B.hv[cur];
    uo.js = B.pitch; uo.lo0 = B.lo0; uo.lo1 = B.lo1;
    Cells3W<double> out;
    out.p[0] = const_cast<double*>(B.h[nxt]); out.p[1] = const_cast<double*>(B.hu[nxt]);
    out.p[2] = const_cast<double*>(B.hv[nxt]);
    out.js = B.pitch; out.lo0 = B.lo0; out.lo1 = B.lo1;
    const Plane<double> np{B.n, B.pitch, B.lo0, B.lo1};
    const IBox vb{B.lo0, B.lo1, B.hi0, B.hi1};
    FaceOut<double> fo{};
    hydro_tile_body<double, FAST, TX, TY, NT>(S, src, uo, np, out, fo, vb, x0, y0, dt, ctl.dx, ctl.dy, ctl.dt_out,
                                              ctl.status);
}

// ---------------------------------------------------------------------------
// Batched ensemble: many independent single-box levels advanced by one
// persistent launch per step.  The launch drains a queue of tiles that spans
// every instance; each instance keeps its own dt chain (three rotating
// accumulators), status word and clock, so instances of any size run side by
// side and small ones no longer leave the GPU idle.
// ---------------------------------------------------------------------------
template <class R> constexpr size_t ens_smem_bytes() {
    size_t a = sizeof(HydroSmem<R, 32, 8>), b = sizeof(HydroSmem<R, 16, 16>), c = sizeof(HydroSmem<R, 64, 4>);
    return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

// The member owning queue tile `tile` and that member's dt for this step; false
// when the member's CFL chain has collapsed (block-uniform: the member's slot is
// launch-constant).  Resets the slot of the step after next and advances the
// member's clock on the member's first tile.
template <class R>
__device__ __forceinline__ bool ens_member(const EnsInstance<R>* __restrict__ inst, int ninst, long long tile, int step,
                                           R cfl, const EnsInstance<R>*& Ip, long long& local, R& dt) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].tile_base <= tile) lo = mid;
        else hi = mid - 1;
    }
    const EnsInstance<R>& I = inst[lo];
    Ip = &I;
    const DtAccum* din = &I.slots[step % 3];
    const unsigned fl = din->flags;
    const R m = accum_dt_min<R>(din->rate_bits, fl);
    local = tile - I.tile_base;
    if ((fl & DTF_COLLAPSED) || m < R(1.e-12)) {
        if (local == 0 && threadIdx.x == 0) {
            atomicOr(I.status, (unsigned)HX_STATUS_DT_COLLAPSE);
            atomicOr(&I.slots[(step + 1) % 3].flags, (unsigned)DTF_COLLAPSED);
        }
        return false;
    }
    dt = m * cfl;
    if (local == 0 && threadIdx.x == 0) {
        DtAccum* r = &I.slots[(step + 2) % 3];
        r->rate_bits = 0ull;
        r->maxvel_bits = 0ull;
        r->flags = 0u;
        *I.time += dt;
    }
    return true;
}

template <class R>
__device__ __forceinline__ void ens_views(const EnsInstance<R>& I, int par, LevelSrc<R>& src, Cells3<R>& uo,
                                          Cells3W<R>& out) {
    src.h = I.st[par][0]; src.hu = I.st[par][1]; src.hv = I.st[par][2]; src.z = I.z; src.n = I.n;
    src.pitch = I.pitch;
    src.nx = I.nx; src.ny = I.ny;
    src.bc_xlo = I.bc[0]; src.bc_xhi = I.bc[1]; src.bc_ylo = I.bc[2]; src.bc_yhi = I.bc[3];
    src.glo0 = -2; src.glo1 = -2; src.ghi0 = I.nx + 1; src.ghi1 = I.ny + 1;
    uo.p[0] = I.st[par][0]; uo.p[1] = I.st[par][1]; uo.p[2] = I.st[par][2];
    uo.js = I.pitch; uo.lo0 = 0; uo.lo1 = 0;
    out.p[0] = I.st[par ^ 1][0]; out.p[1] = I.st[par ^ 1][1]; out.p[2] = I.st[par ^ 1][2];
    out.js = I.pitch; out.lo0 = 0; out.lo1 = 0;
}

// Four blocks of 256 threads per SM (64 registers, ~100 B spilled in the fast form): the barrier waits of
// one tile's phases overlap the other blocks' FP64 work; measured against two blocks (128 registers) and
// three (80): 2070, 2236 and 2281 Mcell-updates/s on 256 members with 16 x 16 tiles (five: 48 registers,
// 552 B spilled).
template <class R, bool FAST>
__global__ void __launch_bounds__(NT, 4) k_ensemble_hydro(const EnsInstance<R>* __restrict__ inst, int ninst,
                                                       long long total_tiles, int step, R cfl,
                                                       unsigned long long* queue) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_tile;
    // the other queue counter was drained by the previous launch: clear it for the next one
    if (blockIdx.x == 0 && threadIdx.x == 0) queue[(step + 1) & 1] = 0ull;
    const int par = step & 1;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(&queue[par], 1ull);
        __syncthreads();
        const long long tile = s_tile;
        __syncthreads();
        if (tile >= total_tiles) break;
        const EnsInstance<R>* Ip;
        long long local;
        R dt;
        if (!ens_member(inst, ninst, tile, step, cfl, Ip, local, dt)) continue;
        const EnsInstance<R>& I = *Ip;
        const int bx = (int)(local % I.tiles_x), by = (int)(local / I.tiles_x);
        LevelSrc<R> src;
        Cells3<R> uo;
        Cells3W<R> out;
        ens_views(I, par, src, uo, out);
        const Plane<R> np{I.n, I.pitch, 0, 0};
        FaceOut<R> fo{};
        fo.on = 0;
        const IBox vb{0, 0, I.nx - 1, I.ny - 1};
        DtAccum* dout = &I.slots[(step + 1) % 3];
        switch (I.shape) {
            case HX_TILE_16x16:
                hydro_tile_body<R, FAST, 16, 16, NT>(*reinterpret_cast<HydroSmem<R, 16, 16>*>(smem_raw), src, uo, np,
                                                     out, fo, vb, bx * 16, by * 16, dt, I.dx, I.dy, dout, I.status);
                break;
            case HX_TILE_64x4:
                hydro_tile_body<R, FAST, 64, 4, NT>(*reinterpret_cast<HydroSmem<R, 64, 4>*>(smem_raw), src, uo, np,
                                                    out, fo, vb, bx * 64, by * 4, dt, I.dx, I.dy, dout, I.status);
                break;
            default:
                hydro_tile_body<R, FAST, 32, 8, NT>(*reinterpret_cast<HydroSmem<R, 32, 8>*>(smem_raw), src, uo, np,
                                                    out, fo, vb, bx * 32, by * 8, dt, I.dx, I.dy, dout, I.status);
        }
    }
}

// The ensemble's large members on 32 x 32 tiles: the same queue discipline
// (counters queue[2 + parity]) with one CTA of 1024 threads per SM, so that
// members of many tiles run with the level kernel's halo economy (1.27 loaded
// cells, 6.4 slopes and 2.06 faces per cell against 1.56, 6.75 and 2.13 on
// 16 x 16 tiles).
template <class R, bool FAST>
__global__ void __launch_bounds__(32 * 32, 1) k_ensemble_big(const EnsInstance<R>* __restrict__ inst, int ninst,
                                                            long long total_tiles, int step, R cfl,
                                                            unsigned long long* queue) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_tile;
    if (blockIdx.x == 0 && threadIdx.x == 0) queue[2 + ((step + 1) & 1)] = 0ull;
    const int par = step & 1;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(&queue[2 + par], 1ull);
        __syncthreads();
        const long long tile = s_tile;
        __syncthreads();
        if (tile >= total_tiles) break;
        const EnsInstance<R>* Ip;
        long long local;
        R dt;
        if (!ens_member(inst, ninst, tile, step, cfl, Ip, local, dt)) continue;
        const EnsInstance<R>& I = *Ip;
        const int bx = (int)(local % I.tiles_x), by = (int)(local / I.tiles_x);
        LevelSrc<R> src;
        Cells3<R> uo;
        Cells3W<R> out;
        ens_views(I, par, src, uo, out);
        const Plane<R> np{I.n, I.pitch, 0, 0};
        FaceOut<R> fo{};
        fo.on = 0;
        const IBox vb{0, 0, I.nx - 1, I.ny - 1};
        hydro_tile_body<R, FAST, 32, 32, 32 * 32>(*reinterpret_cast<HydroSmem<R, 32, 32>*>(smem_raw), src, uo, np,
                                                   out, fo, vb, bx * 32, by * 32, dt, I.dx, I.dy,
                                                   &I.slots[(step + 1) % 3], I.status);
    }
}

// ---------------------------------------------------------------------------
// Classic Roe tile kernel (src/solvers/Roe.cpp:184-248, 327-434).
// ---------------------------------------------------------------------------
template <class R> struct ClassicSmem {
    static constexpr int GX = TX + 2, GY = TY + 2;
    R h[GY][GX], hu[GY][GX], hv[GY][GX], z[GY][GX], n[GY][GX];
    R fx[9][TY][TX + 1];  // F0..2, S-0..2, S+0..2
    R fy[9][TY + 1][TX];
    R kc[4];  // dt/dx, dt/dy, 1/dx, 1/dy: computed once per tile
};

template <class R, bool FAST, class Src>
__global__ void __launch_bounds__(NT) k_classic_tile(Src src, Cells3W<R> out, FaceOut9<R> fo, RebuildOut<R> hb,
                                                     IBox vb, StepCtl<R> ctl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ClassicSmem<R>& S = *reinterpret_cast<ClassicSmem<R>*>(smem_raw);
    constexpr int GX = ClassicSmem<R>::GX, GY = ClassicSmem<R>::GY;

    R dt;
    if (!resolve_dt(ctl, dt)) return;
    step_bookkeeping(ctl, dt);

    const int t = threadIdx.x;
    if (t == 0) {  // read after the loader's barrier
        S.kc[0] = dt / ctl.dx;
        S.kc[1] = dt / ctl.dy;
        S.kc[2] = R(1) / ctl.dx;
        S.kc[3] = R(1) / ctl.dy;
    }
    const int tx = t & (TX - 1), ty = t / TX;
    const int x0 = vb.lo0 + blockIdx.x * TX;
    const int y0 = vb.lo1 + blockIdx.y * TY;

    for (int idx = t; idx < GX * GY; idx += NT) {
        const int r = idx / GX, c = idx - r * GX;
        const int gi = x0 + c - 1, gj = y0 + r - 1;
        R e = R(0), zz = R(0), qx = R(0), qy = R(0), nn = R(0);
        if (src.inside(gi, gj)) src.fetch(gi, gj, e, zz, qx, qy, nn);
        const R hp = max0(e - zz);  // Roe.cpp:246, in place on the grown tile
        S.h[r][c] = hp;
        S.hu[r][c] = qx;
        S.hv[r][c] = qy;
        S.z[r][c] = zz;
        S.n[r][c] = nn;
        hb.store(gi, gj, vb, hp);
    }
    __syncthreads();

    auto xface = [&](int fi, int fj) {
        const int r = fj + 1, cl = fi, cr = fi + 1;
        R F[3], Sm[3], Sp[3];
        roe_classic<R, FAST, 0>(S.h[r][cl], S.hu[r][cl], S.hv[r][cl], S.z[r][cl], S.n[r][cl], S.h[r][cr],
                                S.hu[r][cr], S.hv[r][cr], S.z[r][cr], S.n[r][cr], ctl.dx, F, Sm, Sp);
        for (int k = 0; k < 3; ++k) { S.fx[k][fj][fi] = F[k]; S.fx[3 + k][fj][fi] = Sm[k]; S.fx[6 + k][fj][fi] = Sp[k]; }
        fo.store_x(x0 + fi, y0 + fj, vb, F, Sm, Sp, fi == TX);
    };
    auto yface = [&](int fi, int fj) {
        const int c = fi + 1, rl = fj, rr = fj + 1;
        R F[3], Sm[3], Sp[3];
        roe_classic<R, FAST, 1>(S.h[rl][c], S.hu[rl][c], S.hv[rl][c], S.z[rl][c], S.n[rl][c], S.h[rr][c],
                                S.hu[rr][c], S.hv[rr][c], S.z[rr][c], S.n[rr][c], ctl.dy, F, Sm, Sp);
        for (int k = 0; k < 3; ++k) { S.fy[k][fj][fi] = F[k]; S.fy[3 + k][fj][fi] = Sm[k]; S.fy[6 + k][fj][fi] = Sp[k]; }
        fo.store_y(x0 + fi, y0 + fj, vb, F, Sm, Sp, fj == TY);
    };
    {
        const int gi = x0 + tx, gj = y0 + ty;
        if (gi <= vb.hi0 + 1 && gj <= vb.hi1) xface(tx, ty);
        if (gi <= vb.hi0 && gj <= vb.hi1 + 1) yface(tx, ty);
        if (t < TY) {
            if (x0 + TX <= vb.hi0 + 1 && y0 + t <= vb.hi1) xface(TX, t);
        } else if (t >= 32 && t < 32 + TX) {
            const int m = t - 32;
            if (x0 + m <= vb.hi0 && y0 + TY <= vb.hi1 + 1) yface(m, TY);
        }
    }
    __syncthreads();

    const int gi = x0 + tx, gj = y0 + ty;
    const bool valid = gi <= vb.hi0 && gj <= vb.hi1;
    R rate = R(0), mv = R(0);
    unsigned flags = 0;
    if (valid) {
        const R cx = S.kc[0], cy = S.kc[1];
        const R uo[3] = {S.h[ty + 1][tx + 1], S.hu[ty + 1][tx + 1], S.hv[ty + 1][tx + 1]};
        R un[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            // Roe.cpp:426-430, in this order
            un[k] = uo[k] - cx * (S.fx[k][ty][tx + 1] - S.fx[k][ty][tx]) - cy * (S.fy[k][ty + 1][tx] - S.fy[k][ty][tx]) -
                    cx * (S.fx[6 + k][ty][tx + 1] + S.fx[3 + k][ty][tx]) -
                    cy * (S.fy[6 + k][ty + 1][tx] + S.fy[3 + k][ty][tx]);
        }
        out.st(gi, gj, un[0], un[1], un[2]);
        if (bits_nonfinite(un[0]) || bits_nonfinite(un[1]) || bits_nonfinite(un[2])) flags |= DTF_NAN;
        if (ctl.dt_out) {
            dt_cell_contrib<R, FAST>(un[0], un[1], un[2], is_nodata(S.z[ty + 1][tx + 1]), ctl.dx, ctl.dy,
                                     S.kc[2], S.kc[3], rate, mv, flags);
        }
    }
    if (ctl.dt_out) block_fold_dt<R, NT>(rate, mv, flags, ctl.dt_out);
    if ((flags & DTF_NAN) && ctl.status) atomicOr(ctl.status, (unsigned)HX_STATUS_NAN);
}

// ---------------------------------------------------------------------------
// compute_dt_Impl over a box (HydrostaticRoe.cpp:19-65, Roe.cpp:20-76).
// ---------------------------------------------------------------------------
template <class R, bool FAST>
__global__ void __launch_bounds__(NT) k_dt_reduce(Cells3<R> U, Plane<R> Z, IBox vb, R dx, R dy, R idx, R idy,
                                                  DtAccum* acc) {
    const int i = vb.lo0 + blockIdx.x * TX + (threadIdx.x & (TX - 1));
    R rate = R(0), mv = R(0);
    unsigned flags = 0;
    if constexpr (sizeof(R) == 8) {  // through the float screen: FP64 for the candidates only
        ScreenCell<double> c[ROWS_PER_THREAD];
#pragma unroll
        for (int r = 0; r < ROWS_PER_THREAD; ++r) {
            const int j = vb.lo1 + ((int)blockIdx.y * ROWS_PER_THREAD + r) * TY + threadIdx.x / TX;
            if (i > vb.hi0 || j > vb.hi1) continue;
            c[r].h = U.ld(0, i, j);
            c[r].hu = U.ld(1, i, j);
            c[r].hv = U.ld(2, i, j);
            c[r].nod = is_nodata(Z.ld(i, j));
            c[r].live = true;
        }
        screened_fold<NT, ROWS_PER_THREAD, BlockSync, FAST>(c, dx, dy, idx, idy, rate, mv, flags);
    } else {
        for (int r = 0; r < ROWS_PER_THREAD; ++r) {  // a 32 x (8 ROWS) block: fewer blocks, fewer atomics
            const int j = vb.lo1 + ((int)blockIdx.y * ROWS_PER_THREAD + r) * TY + threadIdx.x / TX;
            if (i > vb.hi0 || j > vb.hi1) continue;
            R rc, mc;
            dt_cell_contrib<R, FAST>(U.ld(0, i, j), U.ld(1, i, j), U.ld(2, i, j), is_nodata(Z.ld(i, j)), dx, dy,
                                     idx, idy, rc, mc, flags);
            if constexpr (FAST) {
                rate = nnmax_i(rate, rc);
                mv = nnmax_i(mv, mc);
            } else {
                rate = smax(rate, rc);
                mv = smax(mv, mc);
            }
        }
    }
    block_fold_dt<R, NT>(rate, mv, flags, acc);
}

// ---------------------------------------------------------------------------
// tag_cells_Impl (HydrostaticRoe.cpp:109-169 method 1; Roe.cpp:121-179 method 0).
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(NT) k_tag(int method, V4<R> U, V4<R> T, V4<signed char> tags, IBox vb, R dx, R dy,
                                            R time, R h_th, R u_th, R z_th, signed char set_value) {
    const int i = vb.lo0 + blockIdx.x * TX + (threadIdx.x & (TX - 1));
    const int j = vb.lo1 + blockIdx.y * TY + threadIdx.x / TX;
    if (i > vb.hi0 || j > vb.hi1) return;
    const R zE = T.ld(i + 1, j, 0), zW = T.ld(i - 1, j, 0), zN = T.ld(i, j + 1, 0), zS = T.ld(i, j - 1, 0);
    if (method == HX_METHOD_HYDROSTATIC_ROE) {
        if (is_nodata(zE) || is_nodata(zW) || is_nodata(zN) || is_nodata(zS)) return;
    } else {
        if ((double)zE == -9999.0 || (double)zW == -9999.0 || (double)zN == -9999.0 || (double)zS == -9999.0) return;
    }
    bool tag = false;
    {
        // the reference divides by the double 2.0 * dx and stores the quotient in Real
        const R dhdx = (R)((double)(U.ld(i + 1, j, 0) - U.ld(i - 1, j, 0)) / (2.0 * (double)dx));
        const R dhdy = (R)((double)(U.ld(i, j + 1, 0) - U.ld(i, j - 1, 0)) / (2.0 * (double)dy));
        if (sqrt(dhdx * dhdx + dhdy * dhdy) > h_th) tag = true;
    }
    auto umag = [&](int ii, int jj) -> R {
        const R hh = U.ld(ii, jj, 0);
        if (hh < R(1.0e-6)) return R(0);
        const R uu = U.ld(ii, jj, 1) / hh, vv = U.ld(ii, jj, 2) / hh;
        return sqrt(uu * uu + vv * vv);
    };
    if (!tag && (double)time <= 1.0e-8) {
        const R dzdx = (R)((double)(zE - zW) / (2.0 * (double)dx));
        const R dzdy = (R)((double)(zN - zS) / (2.0 * (double)dy));
        if (sqrt(dzdx * dzdx + dzdy * dzdy) > z_th) tag = true;
    }
    if (!tag) {
        const R uE = umag(i + 1, j), uW = umag(i - 1, j), uN = umag(i, j + 1), uS = umag(i, j - 1);
        const R dudx = (R)((double)(uE - uW) / (2.0 * (double)dx));
        const R dudy = (R)((double)(uN - uS) / (2.0 * (double)dy));
        if (sqrt(dudx * dudx + dudy * dudy) > u_th) tag = true;
    }
    if (tag) tags.ref(i, j, 0) = set_value;
}

// ---------------------------------------------------------------------------
// masked_avgdown_with_vol over a coarse box (MaskedAverageDown.H:64-104).
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(NT) k_masked_avgdown(V4<R> fine, V4<R> crse, IBox cb, int scomp, int ccomp,
                                                       int ncomp, int rx, int ry, R fv, R nodata) {
    const int i = cb.lo0 + blockIdx.x * TX + (threadIdx.x & (TX - 1));
    const int j = cb.lo1 + blockIdx.y * TY + threadIdx.x / TX;
    if (i > cb.hi0 || j > cb.hi1) return;
    for (int n = 0; n < ncomp; ++n) {
        R cd = R(0), cv = R(0);
        int nvalid = 0;
        for (int jr = 0; jr < ry; ++jr)
            for (int ir = 0; ir < rx; ++ir) {
                const R val = fine.ld(i * rx + ir, j * ry + jr, scomp + n);
                if (!isnan(val) && (double)fabs(val - nodata) > 1e-3) {
                    ++nvalid;
                    cv += fv;
                    cd += val * fv;
                }
            }
        crse.ref(i, j, ccomp + n) = (nvalid * 2 >= rx * ry && cv > R(0)) ? cd / cv : nodata;
    }
}

// ---------------------------------------------------------------------------
// Conservative restriction of the state over a coarse box: amrex::average_down
// as AmrMeshState::AverageDownTo calls it (src/state/AmrMeshState_AMR.cpp:
// 838-844), Cartesian.  AMReX's amrex_avgdown sums the rx*ry fine values rows
// outer, columns inner, from 0, and multiplies by 1/(rx*ry); the same order
// here keeps the result bit-equal.  One thread per coarse cell and component
// loop inside, so a warp reads rx*32 consecutive fine values per fine row.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(NT) k_average_down(V4<R> fine, V4<R> crse, IBox cb, int scomp, int ccomp,
                                                     int ncomp, int rx, int ry, R volfrac) {
    const int i = cb.lo0 + blockIdx.x * TX + (threadIdx.x & (TX - 1));
    const int j = cb.lo1 + blockIdx.y * TY + threadIdx.x / TX;
    if (i > cb.hi0 || j > cb.hi1) return;
    for (int n = 0; n < ncomp; ++n) {
        R c = R(0);
        for (int jr = 0; jr < ry; ++jr)
            for (int ir = 0; ir < rx; ++ir) c += fine.ld(i * rx + ir, j * ry + jr, scomp + n);
        crse.ref(i, j, ccomp + n) = volfrac * c;
    }
}

// ---------------------------------------------------------------------------
// Level diagnostics and eta (src/state/AmrMeshState_Utils.cpp:213-298,
// src/state/AmrMeshState_AMR.cpp:203-224).
// ---------------------------------------------------------------------------
// eta = h + z on any box of the views (ghosts included).
template <class R>
__global__ void __launch_bounds__(NT) k_derive_eta(V4<R> U, V4<R> T, V4<R> eta, IBox b) {
    const int i = b.lo0 + blockIdx.x * TX + (threadIdx.x & (TX - 1));
    const int j = b.lo1 + blockIdx.y * TY + threadIdx.x / TX;
    if (i > b.hi0 || j > b.hi1) return;
    eta.ref(i, j, 0) = U.ld(i, j, 0) + T.ld(i, j, 0);
}

// Per-block sums of the conservation diagnostics over the valid cells that are
// not NODATA (roughness == -9999) and wet (h > 0): mass = h dA, momenta hu dA,
// hv dA, kinetic energy 0.5 (hu^2 + hv^2) / h dA, and min h.  Each cell's terms
// take the reference's types and order (the 0.5 literal is double, so a float
// build evaluates the kinetic term in double and rounds it to float); sums are
// carried in double.  part: 5 doubles per block.
template <class R>
__global__ void __launch_bounds__(NT) k_diag_partial(Plane<R> h, Plane<R> hu, Plane<R> hv, Plane<R> nr, IBox b, R dA,
                                                     double* part) {
    const int i = b.lo0 + blockIdx.x * TX + (threadIdx.x & (TX - 1));
    const int j = b.lo1 + blockIdx.y * TY + threadIdx.x / TX;
    double m = 0.0, px = 0.0, py = 0.0, ke = 0.0, mn = (double)Cst<R>::max_value;
    if (i <= b.hi0 && j <= b.hi1) {
        const R hh = h.ld(i, j), a = hu.ld(i, j), c = hv.ld(i, j);
        const R nodata_val = R(-9999.0);
        if (!(nr.ld(i, j) == nodata_val) && hh > R(0)) {
            const R s_mass = hh * dA, s_mx = a * dA, s_my = c * dA;
            const R s_ke = 0.5 * (a * a + c * c) / hh * dA;
            m = s_mass; px = s_mx; py = s_my; ke = s_ke; mn = hh;
        }
    }
    __shared__ double scr[4 * NT];
    diag_block_store<NT>(m, px, py, ke, mn, part + 5 * (blockIdx.x + (long long)blockIdx.y * gridDim.x), scr);
}

// The block partials folded in a fixed order into out[5] (one block; R only
// ties the instance to the unit that instantiates launch_diagnostics<R>).
template <class R>
__global__ void __launch_bounds__(NT) k_diag_final(const double* part, long long nblocks, double* out) {
    __shared__ double sh[5][NT / 32];
    double v[5] = {0.0, 0.0, 0.0, 0.0, 1.7976931348623157e308};
    for (long long k = threadIdx.x; k < nblocks; k += NT) {
        for (int c = 0; c < 4; ++c) v[c] += part[5 * k + c];
        v[4] = fmin(v[4], part[5 * k + 4]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int c = 0; c < 4; ++c) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
        v[4] = fmin(v[4], __shfl_xor_sync(0xffffffffu, v[4], o));
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 5; ++c) sh[c][w] = v[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < NT / 32; ++k) {
            for (int c = 0; c < 4; ++c) v[c] += sh[c][k];
            v[4] = fmin(v[4], sh[4][k]);
        }
        for (int c = 0; c < 5; ++c) out[c] = v[c];
    }
}

// ---------------------------------------------------------------------------
// Point evaluation of the Riemann solvers (diagnostic entry, golden vectors).
// method 1: states (n, 6) = (hi hui hvi hj huj hvj), aux (n, 2) = normal;
// method 0: states (n, 10), aux (n, 4) = (dt dx nx ny).  out: (n, 3) F then,
// for method 0, (n, 3) S- and (n, 3) S+.
// ---------------------------------------------------------------------------
template <class R, bool FAST>
__global__ void k_points(int method, long n, const R* __restrict__ st, const R* __restrict__ aux, R* __restrict__ out) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    if (method == HX_METHOD_HYDROSTATIC_ROE) {
        const R* q = st + 6 * p;
        const bool ydir = aux[2 * p + 1] != R(0);
        R f0, f1, f2;
        if constexpr (!FAST) {
            if (ydir) roe_hydrostatic_exact<1>(q[0], q[1], q[2], q[3], q[4], q[5], f0, f1, f2);
            else roe_hydrostatic_exact<0>(q[0], q[1], q[2], q[3], q[4], q[5], f0, f1, f2);
        } else {
            const R ui = q[0] > R(0) ? q[1] / q[0] : R(0), vi = q[0] > R(0) ? q[2] / q[0] : R(0);
            const R uj = q[3] > R(0) ? q[4] / q[3] : R(0), vj = q[3] > R(0) ? q[5] / q[3] : R(0);
            if (ydir) roe_hydrostatic_fast<R, 1>(q[0], ui, vi, q[3], uj, vj, f0, f1, f2);
            else roe_hydrostatic_fast<R, 0>(q[0], ui, vi, q[3], uj, vj, f0, f1, f2);
        }
        out[3 * p] = f0; out[3 * p + 1] = f1; out[3 * p + 2] = f2;
    } else {
        const R* q = st + 10 * p;
        const R* a = aux + 4 * p;
        R F[3], Sm[3], Sp[3];
        if (a[3] != R(0)) roe_classic<R, FAST, 1>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], a[1], F, Sm, Sp);
        else roe_classic<R, FAST, 0>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], a[1], F, Sm, Sp);
        for (int k = 0; k < 3; ++k) { out[3 * p + k] = F[k]; out[3 * n + 3 * p + k] = Sm[k]; out[6 * n + 3 * p + k] = Sp[k]; }
    }
}

}  // namespace hx

// ---------------------------------------------------------------------------
// Forward steps of the adjoint's sweeps (see launch_adj_forward), on the level
// kernel's tile for the box's size.
// ---------------------------------------------------------------------------
namespace hx {
template <bool FAST, int AX = TX, int AY = TY>
__global__ void __launch_bounds__(AX * AY, min_ctas(AX * AY)) k_adj_forward(LevelSrc<double> src, Cells3<double> uo, Plane<double> np,
                                                     Cells3W<double> out, IBox vb, StepCtl<double> ctl,
                                                     const double* dt_fixed, unsigned* post_flags, AdjRecord rec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HydroSmem<double, AX, AY>& S = *reinterpret_cast<HydroSmem<double, AX, AY>*>(smem_raw);
    double dt;
    if (dt_fixed) {
        dt = *dt_fixed;
    } else {
        if (!resolve_dt(ctl, dt)) return;
        step_bookkeeping(ctl, dt);
    }
    if (blockIdx.x == 0 && blockIdx.y == 0) {  // the step's dt and the gauges of its input state
        if (rec.dt && threadIdx.x == 0) *rec.dt = dt;
        if (rec.series)
            for (int k = threadIdx.x; k < rec.ngauges; k += blockDim.x) rec.series[k] = uo.p[0][rec.gauges[k]];
    }
    FaceOut<double> fo{};
    fo.on = 0;
    hydro_tile_body<double, FAST, AX, AY, AX * AY>(S, src, uo, np, out, fo, vb, vb.lo0 + (int)blockIdx.x * AX,
                                                   vb.lo1 + (int)blockIdx.y * AY, dt, ctl.dx, ctl.dy,
                                                   dt_fixed ? nullptr : ctl.dt_out, ctl.status, post_flags);
}

// A recompute step (dt given) that also records every face's intermediates
// (FAST must be true: records exist for the fast form only).
template <bool FAST, int AX = TX, int AY = TY>
__global__ void __launch_bounds__(AX * AY, min_ctas(AX * AY)) k_adj_forward_rec(LevelSrc<double> src, Cells3<double> uo, Plane<double> np,
                                                         Cells3W<double> out, IBox vb, double dx, double dy,
                                                         const double* dt_fixed, unsigned* post_flags, FaceRec rec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HydroSmem<double, AX, AY>& S = *reinterpret_cast<HydroSmem<double, AX, AY>*>(smem_raw);
    FaceOut<double> fo{};
    fo.on = 0;
    static_assert(FAST, "face records are kept for the fast form");
    hydro_tile_body<double, FAST, AX, AY, AX * AY, LevelSrc<double>, false, NoDiv, FaceRec>(
        S, src, uo, np, out, fo, vb, vb.lo0 + (int)blockIdx.x * AX, vb.lo1 + (int)blockIdx.y * AY, *dt_fixed, dx, dy,
        nullptr, nullptr, post_flags, NoDiv{}, rec);
}

template <bool FAST, int AX = TX, int AY = TY>
__global__ void __launch_bounds__(AX * AY, min_ctas(AX * AY)) k_adj_forward_linear(LevelSrc<double> src, Cells3<double> uo, Plane<double> np,
                                                            Cells3W<double> out, IBox vb, double dx, double dy,
                                                            const double* dt_fixed) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HydroSmem<double, AX, AY>& S = *reinterpret_cast<HydroSmem<double, AX, AY>*>(smem_raw);
    FaceOut<double> fo{};
    fo.on = 0;
    hydro_tile_body<double, FAST, AX, AY, AX * AY, LevelSrc<double>, true>(
        S, src, uo, np, out, fo, vb, vb.lo0 + (int)blockIdx.x * AX, vb.lo1 + (int)blockIdx.y * AY, *dt_fixed, dx, dy,
        nullptr, nullptr);
}
}  // namespace hx

// ---------------------------------------------------------------------------
// Launchers (explicitly instantiated per arithmetic form).
// ---------------------------------------------------------------------------
#include "hx_launch.h"

namespace hx {

template <class K> inline cudaError_t ensure_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// The step's kernel; nblocks receives its block count (the epilogue's partials).
template <class R, bool FAST, class Src, bool EPI>
cudaError_t launch_hydro_k(const Src& src, const Cells3<R>& uo, const Plane<R>& np, const Cells3W<R>& out,
                           const FaceOut<R>& fo, const IBox& vb, const StepCtl<R>& ctl, cudaStream_t st,
                           const EpiOut<R>& epi, long long& nblocks) {
    if constexpr (std::is_same_v<Src, LevelSrc<double>>) {
        // a whole level (or a band of its rows) on the big tile: the persistent kernel, when the stored state
        // and roughness are the level's own planes and no face arrays are asked for
        if (big_tile<R>(vb) && !fo.on && !fo.mean && uo.p[0] == src.h && uo.p[1] == src.hu && uo.p[2] == src.hv &&
            uo.js == src.pitch && uo.lo0 == 0 && uo.lo1 == 0 && np.p == src.n && np.js == src.pitch &&
            np.lo0 == 0 && np.lo1 == 0) {
            const dim3 tg = tile_grid(vb, kPX, kPY);
            const int ntiles = (int)(tg.x * tg.y);
            int dev = 0, sms = 0;
            cudaError_t e = cudaGetDevice(&dev);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            auto k = k_hydro_persist<FAST, NoDiv, EPI>;
            e = ensure_smem(k, persist_smem_bytes());
            if (e != cudaSuccess) return e;
            const PersistMaps maps = persist_maps(src);
            const int grid = ntiles < sms ? ntiles : sms;
            k<<<(unsigned)grid, kPN, persist_smem_bytes(), st>>>(src, out, vb, (int)tg.x, ntiles, ctl, NoDiv{}, maps,
                                                                 ctl.status, epi);
            nblocks = grid;
            return cudaGetLastError();
        }
    }
    if (big_tile<R>(vb)) {
        constexpr int BX = BigTile<R>::X, BY = BigTile<R>::Y;
        const size_t sm = sizeof(HydroSmem<R, BX, BY>);
        auto k = k_hydro_tile<R, FAST, Src, BX, BY, EPI>;
        cudaError_t e = ensure_smem(k, sm);
        if (e != cudaSuccess) return e;
        const dim3 g = tile_grid(vb, BX, BY);
        k<<<g, BX * BY, sm, st>>>(src, uo, np, out, fo, vb, ctl, epi);
        nblocks = (long long)g.x * g.y;
        return cudaGetLastError();
    }
    const size_t sm = sizeof(HydroSmem<R>);
    auto k = k_hydro_tile<R, FAST, Src, TX, TY, EPI>;
    cudaError_t e = ensure_smem(k, sm);
    if (e != cudaSuccess) return e;
    const dim3 g = tile_grid(vb, TX, TY);
    k<<<g, NT, sm, st>>>(src, uo, np, out, fo, vb, ctl, epi);
    nblocks = (long long)g.x * g.y;
    return cudaGetLastError();
}

// The hydrostatic step; with an epilogue (epi not null) the update also writes
// eta and the diagnostics' block partials, which k_diag_final then folds into
// epi->out.  The partials are at most one per TX x TY tile of vb.
template <class R, bool FAST, class Src>
cudaError_t launch_hydro(const Src& src, const Cells3<R>& uo, const Plane<R>& np, const Cells3W<R>& out,
                         const FaceOut<R>& fo, const IBox& vb, const StepCtl<R>& ctl, cudaStream_t st,
                         const EpiOut<R>* epi) {
    long long nblocks = 0;
    if (!epi) return launch_hydro_k<R, FAST, Src, false>(src, uo, np, out, fo, vb, ctl, st, EpiOut<R>{}, nblocks);
    cudaError_t e = launch_hydro_k<R, FAST, Src, true>(src, uo, np, out, fo, vb, ctl, st, *epi, nblocks);
    if (e != cudaSuccess || !epi->part) return e;
    k_diag_final<R><<<1, NT, 0, st>>>(epi->part, nblocks, epi->out);
    return cudaGetLastError();
}

template <class R, bool FAST, class Src>
cudaError_t launch_classic(const Src& src, const Cells3W<R>& out, const FaceOut9<R>& fo, const RebuildOut<R>& hb,
                           const IBox& vb, const StepCtl<R>& ctl, cudaStream_t st) {
    const size_t sm = sizeof(ClassicSmem<R>);
    auto k = k_classic_tile<R, FAST, Src>;
    cudaError_t e = ensure_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<tile_grid(vb, TX, TY), NT, sm, st>>>(src, out, fo, hb, vb, ctl);
    return cudaGetLastError();
}

template <class R, bool FAST>
cudaError_t launch_ensemble(const EnsInstance<R>* inst, int ninst, long long total_tiles, int step, R cfl,
                           unsigned long long* queue, int grid, cudaStream_t st) {
    const size_t sm = ens_smem_bytes<R>();
    auto k = k_ensemble_hydro<R, FAST>;
    cudaError_t e = ensure_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<grid, NT, sm, st>>>(inst, ninst, total_tiles, step, cfl, queue);
    return cudaGetLastError();
}

template <class R, bool FAST>
cudaError_t launch_ensemble_big(const EnsInstance<R>* inst, int ninst, long long total_tiles, int step, R cfl,
                               unsigned long long* queue, int grid, cudaStream_t st) {
    const size_t sm = sizeof(HydroSmem<R, 32, 32>);
    auto k = k_ensemble_big<R, FAST>;
    cudaError_t e = ensure_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<grid, 32 * 32, sm, st>>>(inst, ninst, total_tiles, step, cfl, queue);
    return cudaGetLastError();
}

template <class R, bool FAST>
int ensemble_blocks_per_sm() {
    int n = 0;
    if (ensure_smem(k_ensemble_hydro<R, FAST>, ens_smem_bytes<R>()) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_ensemble_hydro<R, FAST>, NT, ens_smem_bytes<R>()) !=
        cudaSuccess)
        return 0;
    return n;
}

template <bool FAST>
cudaError_t launch_boxlevel(const BoxSetSrc& src, const int* tiles, int ntiles, const StepCtl<double>& ctl,
                            cudaStream_t st, bool big) {
    if (ntiles <= 0) return cudaSuccess;
    if (big) {  // 32 x 32 tiles: the persistent kernel, one block per SM
        int dev = 0, sms = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        auto k = k_boxlevel_persist<FAST>;
        e = ensure_smem(k, persist_smem_bytes());
        if (e != cudaSuccess) return e;
        k<<<(unsigned)(ntiles < sms ? ntiles : sms), kPN, persist_smem_bytes(), st>>>(src, tiles, ntiles, ctl);
        return cudaGetLastError();
    }
    const size_t sm = sizeof(HydroSmem<double>);
    cudaError_t e = ensure_smem(k_boxlevel_hydro<FAST>, sm);
    if (e != cudaSuccess) return e;
    k_boxlevel_hydro<FAST><<<ntiles, NT, sm, st>>>(src, tiles, ctl);
    return cudaGetLastError();
}

template <class R, bool FAST>
cudaError_t launch_hydro_split(const LevelSrc<R>& src, const Cells3<R>& uo, const Plane<R>& np, const DivOut<R>& div,
                               const IBox& vb, R dx, R dy, cudaStream_t st) {
    if constexpr (std::is_same_v<R, double>) {
        if (big_tile<R>(vb) && uo.p[0] == src.h && uo.p[1] == src.hu && uo.p[2] == src.hv) {
            const dim3 tg = tile_grid(vb, kPX, kPY);
            const int ntiles = (int)(tg.x * tg.y);
            int dev = 0, sms = 0;
            cudaError_t e = cudaGetDevice(&dev);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            auto k = k_hydro_persist<FAST, DivOut<double>>;
            e = ensure_smem(k, persist_smem_bytes());
            if (e != cudaSuccess) return e;
            StepCtl<double> ctl{};
            ctl.dx = dx;
            ctl.dy = dy;
            (void)np;
            const PersistMaps maps = persist_maps(src);
            k<<<(unsigned)(ntiles < sms ? ntiles : sms), kPN, persist_smem_bytes(), st>>>(
                src, Cells3W<double>{}, vb, (int)tg.x, ntiles, ctl, div, maps, nullptr, EpiOut<double>{});
            return cudaGetLastError();
        }
    }
    if (big_tile<R>(vb)) {
        constexpr int BX = BigTile<R>::X, BY = BigTile<R>::Y;
        const size_t sm = sizeof(HydroSmem<R, BX, BY>);
        cudaError_t e = ensure_smem(k_hydro_div<R, FAST, BX, BY>, sm);
        if (e != cudaSuccess) return e;
        k_hydro_div<R, FAST, BX, BY><<<tile_grid(vb, BX, BY), BX * BY, sm, st>>>(src, uo, np, div, vb, dx, dy);
        return cudaGetLastError();
    }
    const size_t sm = sizeof(HydroSmem<R>);
    cudaError_t e = ensure_smem(k_hydro_div<R, FAST>, sm);
    if (e != cudaSuccess) return e;
    k_hydro_div<R, FAST><<<tile_grid(vb, TX, TY), NT, sm, st>>>(src, uo, np, div, vb, dx, dy);
    return cudaGetLastError();
}

template <class R, bool FAST>
cudaError_t launch_hydro_update(const Cells3<R>& uo, const DivOut<R>& div, const Plane<R>& np, const Plane<R>& zp,
                                const Cells3W<R>& out, const IBox& vb, const StepCtl<R>& ctl, cudaStream_t st) {
    k_hydro_update<R, FAST><<<tile_grid(vb, TX, TY * ROWS_PER_THREAD), NT, 0, st>>>(uo, div, np, zp, out, vb, ctl);
    return cudaGetLastError();
}

template <class R, bool FAST>
cudaError_t launch_dt_reduce(const Cells3<R>& U, const Plane<R>& Z, const IBox& vb, R dx, R dy, DtAccum* acc,
                             cudaStream_t st) {
    // 1/dx, 1/dy correctly rounded on the host: the same values the device would compute
    k_dt_reduce<R, FAST><<<tile_grid(vb, TX, TY * ROWS_PER_THREAD), NT, 0, st>>>(U, Z, vb, dx, dy, R(1) / dx,
                                                                                 R(1) / dy, acc);
    return cudaGetLastError();
}

template <bool FAST>
cudaError_t launch_adj_forward(const LevelSrc<double>& src, const Cells3<double>& uo, const Plane<double>& np,
                               const Cells3W<double>& out, const IBox& vb, const StepCtl<double>& ctl,
                               const double* dt_fixed, unsigned* post_flags, const AdjRecord& rec, cudaStream_t st) {
    auto go = [&](auto shape) -> cudaError_t {
        constexpr int AX = decltype(shape)::X, AY = decltype(shape)::Y;
        const size_t sm = sizeof(HydroSmem<double, AX, AY>);
        cudaError_t e = ensure_smem(k_adj_forward<FAST, AX, AY>, sm);
        if (e != cudaSuccess) return e;
        k_adj_forward<FAST, AX, AY><<<tile_grid(vb, AX, AY), AX * AY, sm, st>>>(src, uo, np, out, vb, ctl, dt_fixed,
                                                                              post_flags, rec);
        return cudaGetLastError();
    };
    return big_tile<double>(vb) ? go(BigTile<double>{}) : go(SmallTile{});
}

template <bool FAST>
cudaError_t launch_adj_forward_rec(const LevelSrc<double>& src, const Cells3<double>& uo, const Plane<double>& np,
                                   const Cells3W<double>& out, const IBox& vb, double dx, double dy,
                                   const double* dt_fixed, unsigned* post_flags, const FaceRec& rec, cudaStream_t st) {
    auto go = [&](auto shape) -> cudaError_t {
        constexpr int AX = decltype(shape)::X, AY = decltype(shape)::Y;
        const size_t sm = sizeof(HydroSmem<double, AX, AY>);
        cudaError_t e = ensure_smem(k_adj_forward_rec<FAST, AX, AY>, sm);
        if (e != cudaSuccess) return e;
        k_adj_forward_rec<FAST, AX, AY><<<tile_grid(vb, AX, AY), AX * AY, sm, st>>>(src, uo, np, out, vb, dx, dy,
                                                                                  dt_fixed, post_flags, rec);
        return cudaGetLastError();
    };
    return big_tile<double>(vb) ? go(BigTile<double>{}) : go(SmallTile{});
}

template <bool FAST>
cudaError_t launch_adj_forward_linear(const LevelSrc<double>& src, const Cells3<double>& uo, const Plane<double>& np,
                                      const Cells3W<double>& out, const IBox& vb, double dx, double dy,
                                      const double* dt_fixed, cudaStream_t st) {
    auto go = [&](auto shape) -> cudaError_t {
        constexpr int AX = decltype(shape)::X, AY = decltype(shape)::Y;
        const size_t sm = sizeof(HydroSmem<double, AX, AY>);
        cudaError_t e = ensure_smem(k_adj_forward_linear<FAST, AX, AY>, sm);
        if (e != cudaSuccess) return e;
        k_adj_forward_linear<FAST, AX, AY><<<tile_grid(vb, AX, AY), AX * AY, sm, st>>>(src, uo, np, out, vb, dx, dy,
                                                                                     dt_fixed);
        return cudaGetLastError();
    };
    return big_tile<double>(vb) ? go(BigTile<double>{}) : go(SmallTile{});
}

// The fast form's reciprocal (rcp_nr, which == 0) or square root (fast_sqrt,
// which == 1) of n values, for checking them against IEEE division and sqrt.
// The fast form's FP64 building blocks on n points: op 0 rcp_nr, 1 fast_sqrt,
// 2 the van Leer slope of the triplet x[3i..3i+2], 3 rcp_fa, 4 fast_sqrt_fa.
template <bool FAST> __global__ void k_rcp_probe(long n, const double* x, double* y, int which) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    switch (which) {
        case 0: y[i] = rcp_nr(x[i]); break;
        case 1: y[i] = fast_sqrt(x[i]); break;
        case 2: y[i] = van_leer_slope<double, true>(x[3 * i], x[3 * i + 1], x[3 * i + 2]); break;
        case 3: y[i] = rcp_fa(x[i]); break;
        case 4: y[i] = fast_sqrt_fa(x[i]); break;
        default: y[i] = rcbrt_nr(x[i]); break;
    }
}
template <bool FAST> cudaError_t launch_rcp(long n, const double* x, double* y, int which, cudaStream_t st) {
    static_assert(FAST, "the reciprocal and square root belong to the fast form");
    if (n <= 0) return cudaSuccess;
    k_rcp_probe<FAST><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x, y, which);
    return cudaGetLastError();
}

template <class R, bool FAST>
cudaError_t launch_points(int method, long n, const R* st, const R* aux, R* out, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_points<R, FAST><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(method, n, st, aux, out);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_tag(int method, const V4<R>& U, const V4<R>& T, const V4<signed char>& tags, const IBox& vb, R dx,
                       R dy, R time, R h_th, R u_th, R z_th, signed char set_value, cudaStream_t st) {
    k_tag<R><<<tile_grid(vb, TX, TY), NT, 0, st>>>(method, U, T, tags, vb, dx, dy, time, h_th, u_th, z_th, set_value);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_derive_eta(const V4<R>& U, const V4<R>& T, const V4<R>& eta, const IBox& b, cudaStream_t st) {
    k_derive_eta<R><<<tile_grid(b, TX, TY), NT, 0, st>>>(U, T, eta, b);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_diagnostics(const Plane<R>& h, const Plane<R>& hu, const Plane<R>& hv, const Plane<R>& nr,
                               const IBox& b, R dA, double* part, double* out, cudaStream_t st) {
    const dim3 g = tile_grid(b, TX, TY);
    k_diag_partial<R><<<g, NT, 0, st>>>(h, hu, hv, nr, b, dA, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_diag_final<R><<<1, NT, 0, st>>>(part, (long long)g.x * g.y, out);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_average_down(const V4<R>& fine, const V4<R>& crse, const IBox& cb, int scomp, int ccomp,
                                int ncomp, int rx, int ry, cudaStream_t st) {
    const R volfrac = R(1.0) / R(rx * ry);
    k_average_down<R><<<tile_grid(cb, TX, TY), NT, 0, st>>>(fine, crse, cb, scomp, ccomp, ncomp, rx, ry, volfrac);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_masked_avgdown(const V4<R>& fine, const V4<R>& crse, const IBox& cb, int scomp, int ccomp,
                                  int ncomp, int rx, int ry, R fv, R nodata, cudaStream_t st) {
    k_masked_avgdown<R><<<tile_grid(cb, TX, TY), NT, 0, st>>>(fine, crse, cb, scomp, ccomp, ncomp, rx, ry, fv, nodata);
    return cudaGetLastError();
}

}  // namespace hx
