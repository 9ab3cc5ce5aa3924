// Internal view types shared by the kernels and the C-ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hx {

// The level kernels' default tile: 32 x 8 cells, one thread per cell (FP64
// boxes of 2048^2 cells and more take a 32 x 32 tile: BigTile in
// hx_kernels.cuh; the ensemble picks its shapes per member).
constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NT = TX * TY;
// Rows of cells per thread in the per-cell kernels (CFL reduction, split
// update): four 32 x 8 layers per block cut the blocks, and with them the
// block-level atomics on the one dt accumulator, by four.
constexpr int ROWS_PER_THREAD = 4;


// Read-only load: through the read-only data cache for plain reals, a plain
// load for other element types (the dual numbers of the tangent model).
template <class T> __device__ __forceinline__ T ld_ro(const T* p) { return *p; }
template <> __device__ __forceinline__ double ld_ro<double>(const double* p) { return __ldg(p); }
template <> __device__ __forceinline__ float ld_ro<float>(const float* p) { return __ldg(p); }

struct IBox {
    int lo0, lo1, hi0, hi1;
};

// Boxes (and levels) from 2048 x 2048 cells take the big FP64 tile (32 x 32, one block of 1024 threads per
// SM): the persistent kernels on whole levels, the 32 x 32 tile kernel on boxes.
constexpr long long kBigTileCells = 1ll << 22;

// Array4-like strided view: element (i, j, c) at p[(i-lo0) + (j-lo1)*js + c*ns].
template <class T> struct V4 {
    T* p;
    long long js, ns;
    int lo0, lo1, hi0, hi1, nc;
    __device__ __forceinline__ T ld(int i, int j, int c) const {
        return p[(long long)(i - lo0) + (long long)(j - lo1) * js + (long long)c * ns];
    }
    __device__ __forceinline__ T& ref(int i, int j, int c) const {
        return p[(long long)(i - lo0) + (long long)(j - lo1) * js + (long long)c * ns];
    }
};

// One plane read at valid cells: (i-lo0) + (j-lo1)*js.
template <class R> struct Plane {
    const R* p;
    long long js;
    int lo0, lo1;
    __device__ __forceinline__ R ld(int i, int j) const {
        return ld_ro(p + (long long)(i - lo0) + (long long)(j - lo1) * js);
    }
};

// Three planes read at valid cells (the stored state u_o).
template <class R> struct Cells3 {
    const R* p[3];
    long long js;
    int lo0, lo1;
    __device__ __forceinline__ R ld(int c, int i, int j) const {
        return ld_ro(p[c] + (long long)(i - lo0) + (long long)(j - lo1) * js);
    }
};

// Three planes written at valid cells (U_new).
template <class R> struct Cells3W {
    R* p[3];
    long long js;
    int lo0, lo1;
    __device__ __forceinline__ void st(int i, int j, R a, R b, R c) const {
        const long long o = (long long)(i - lo0) + (long long)(j - lo1) * js;
        p[0][o] = a;
        p[1][o] = b;
        p[2][o] = c;
    }
};

// The advance epilogue: what the update of a step writes beside the state.
// eta (null: none) receives eta = h + z of every updated cell, the kernel of
// AmrMeshState::DeriveEtaFrom (src/state/AmrMeshState_AMR.cpp:203-224); part
// (null: none) receives 5 doubles per block of the conservation diagnostics
// of the updated state (AmrMeshState::ComputeMassDiagnostics,
// src/state/AmrMeshState_Utils.cpp:213-300), folded into out[5] after the step.
template <class R> struct EpiOut {
    R* eta;
    long long ejs;
    int elo0, elo1;
    double* part;
    double* out;
    R dA;
};
// A thread's running diagnostics: the four sums and min h as the bits of a
// positive double (whose order as integers is the order of the values).
struct DiagAcc {
    double m = 0.0, px = 0.0, py = 0.0, ke = 0.0;
    unsigned long long mn = 0x7fefffffffffffffull;  // DBL_MAX
};

// No flux-difference output (the fused step).
struct NoDiv {
    static constexpr bool on = false;
    template <class R> __device__ void st(int, int, R, R, R, R, R, R) const {}
};
// The six flux differences of every valid cell (dx0 dx1 dx2 dy0 dy1 dy2), for
// a step whose update runs once dt is known.
template <class R> struct DivOut {
    static constexpr bool on = true;
    R* p[6];
    long long js;
    int lo0, lo1;
    __device__ __forceinline__ void st(int i, int j, R a, R b, R c, R d, R e, R f) const {
        const long long o = (long long)(i - lo0) + (long long)(j - lo1) * js;
        p[0][o] = a; p[1][o] = b; p[2][o] = c; p[3][o] = d; p[4][o] = e; p[5][o] = f;
    }
};

// Optional hydrostatic face outputs: the FL/FR arrays (on), and/or the reflux
// flux 0.5 FL + 0.5 FR the flux registers receive (mean,
// src/solvers/HydrostaticRoe.cpp:612-627; the halves are exact, so the one
// rounding of the sum gives the reference's value with or without contraction).
template <class R> struct FaceOut {
    V4<R> FL[2], FR[2], Fm[2];
    int on, mean;
    __device__ __forceinline__ void put(int d, int gi, int gj, const R* l, const R* r) const {
        if (on)
            for (int k = 0; k < 3; ++k) { FL[d].ref(gi, gj, k) = l[k]; FR[d].ref(gi, gj, k) = r[k]; }
        if (mean)
            for (int k = 0; k < 3; ++k) Fm[d].ref(gi, gj, k) = R(0.5) * l[k] + R(0.5) * r[k];
    }
    // x face (gi, gj): FL = (F0, Fa, Fc), FR = (F0, Fb, Fc)
    __device__ __forceinline__ void store_x(int gi, int gj, const IBox& vb, R F0, R Fa, R Fb, R Fc, bool extra) const {
        if (!on && !mean) return;
        if (gi < vb.lo0 || gi > vb.hi0 + 1 || gj < vb.lo1 || gj > vb.hi1) return;
        if (extra && gi != vb.hi0 + 1) return;
        const R l[3] = {F0, Fa, Fc}, r[3] = {F0, Fb, Fc};
        put(0, gi, gj, l, r);
    }
    // y face: FL = (F0, Fa, Fb), FR = (F0, Fa, Fc)
    __device__ __forceinline__ void store_y(int gi, int gj, const IBox& vb, R F0, R Fa, R Fb, R Fc, bool extra) const {
        if (!on && !mean) return;
        if (gi < vb.lo0 || gi > vb.hi0 || gj < vb.lo1 || gj > vb.hi1 + 1) return;
        if (extra && gj != vb.hi1 + 1) return;
        const R l[3] = {F0, Fa, Fb}, r[3] = {F0, Fa, Fc};
        put(1, gi, gj, l, r);
    }
};

// Optional classic face outputs: the F, S-, S+ nodal arrays per direction
// (on), and/or the side-selected effective fluxes of the flux registers
// (src/solvers/Roe.cpp:369-388, 447-566): D- = F - S- (seen by the right
// cell), D+ = F + S+ (seen by the left cell).  Coarse register (crse_on): D+
// where the left cell is coarse and the right one covered by the finer level
// (mask 0 | 1), D- for 1 | 0, else 0.  Fine register (fine_on): D- on the
// grid box's low face, D+ on its high face, else 0.
template <class R> struct FaceOut9 {
    V4<R> F[2], Sm[2], Sp[2];
    V4<R> fc[2], ff[2];
    V4<int> mask;
    IBox grid;
    int on, crse_on, fine_on;
    __device__ __forceinline__ void put(int d, int gi, int gj, const R* f, const R* m, const R* p) const {
        if (on)
            for (int k = 0; k < 3; ++k) {
                F[d].ref(gi, gj, k) = f[k];
                Sm[d].ref(gi, gj, k) = m[k];
                Sp[d].ref(gi, gj, k) = p[k];
            }
        if (!crse_on && !fine_on) return;
        R Dm[3], Dp[3];
        for (int k = 0; k < 3; ++k) {  // LinComb(1.0, F, -1.0, S-) and LinComb(1.0, F, 1.0, S+): exact products
            Dm[k] = R(1.0) * f[k] + R(-1.0) * m[k];
            Dp[k] = R(1.0) * f[k] + R(1.0) * p[k];
        }
        if (crse_on) {
            const int left_is_fine = d == 0 ? mask.ld(gi - 1, gj, 0) : mask.ld(gi, gj - 1, 0);
            const int right_is_fine = mask.ld(gi, gj, 0);
            for (int k = 0; k < 3; ++k)
                fc[d].ref(gi, gj, k) = (left_is_fine == 0 && right_is_fine == 1)   ? Dp[k]
                                       : (left_is_fine == 1 && right_is_fine == 0) ? Dm[k]
                                                                                   : R(0.0);
        }
        if (fine_on) {
            const int face_idx = d == 0 ? gi : gj;
            const int i_low = d == 0 ? grid.lo0 : grid.lo1, i_high = (d == 0 ? grid.hi0 : grid.hi1) + 1;
            for (int k = 0; k < 3; ++k)
                ff[d].ref(gi, gj, k) = face_idx == i_low ? Dm[k] : (face_idx == i_high ? Dp[k] : R(0.0));
        }
    }
    __device__ __forceinline__ void store_x(int gi, int gj, const IBox& vb, const R* f, const R* m, const R* p,
                                            bool extra) const {
        if (!on && !crse_on && !fine_on) return;
        if (gi < vb.lo0 || gi > vb.hi0 + 1 || gj < vb.lo1 || gj > vb.hi1) return;
        if (extra && gi != vb.hi0 + 1) return;
        put(0, gi, gj, f, m, p);
    }
    __device__ __forceinline__ void store_y(int gi, int gj, const IBox& vb, const R* f, const R* m, const R* p,
                                            bool extra) const {
        if (!on && !crse_on && !fine_on) return;
        if (gi < vb.lo0 || gi > vb.hi0 || gj < vb.lo1 || gj > vb.hi1 + 1) return;
        if (extra && gj != vb.hi1 + 1) return;
        put(1, gi, gj, f, m, p);
    }
};

// Optional write-back of the rebuilt depth into U_old comp 0 on the box grown
// by one cell (the classic solver rebuilds in place, src/solvers/Roe.cpp:339).
// A grown-tile cell is written by the tile that owns it: its own columns/rows,
// plus the box's ghost ring next to them.
template <class R> struct RebuildOut {
    V4<R> U;
    int on;
    __device__ __forceinline__ void store(int gi, int gj, const IBox& vb, R hp) const {
        if (!on) return;
        const int tx0 = vb.lo0 + (int)blockIdx.x * 32, ty0 = vb.lo1 + (int)blockIdx.y * 8;
        int xa = tx0, xb = tx0 + 31, ya = ty0, yb = ty0 + 7;
        if (xb > vb.hi0) xb = vb.hi0;
        if (yb > vb.hi1) yb = vb.hi1;
        if (xa == vb.lo0) xa = vb.lo0 - 1;
        if (xb == vb.hi0) xb = vb.hi0 + 1;
        if (ya == vb.lo1) ya = vb.lo1 - 1;
        if (yb == vb.hi1) yb = vb.hi1 + 1;
        if (gi < xa || gi > xb || gj < ya || gj > yb) return;
        if (gi < U.lo0 || gi > U.hi0 || gj < U.lo1 || gj > U.hi1) return;
        U.ref(gi, gj, 0) = hp;
    }
};

// ---------------------------------------------------------------------------
// Sources of the grown tile.
// ---------------------------------------------------------------------------

// Physical-boundary codes of one side of the level (inputs file
// HydroEXA.lo_bc / hi_bc, include/boundaries/BCFill.H:35-138): 0 and 2 are
// walls (depth, eta mirrored; terrain always copied from the edge), anything
// else is open (every field copied from the edge cell).  The two walls differ
// in the BC records the momentum ghosts take:
//  - 0, the reference's wall: its per-step FillPatch fills hu, hv (components
//    1, 2) with BC-record offset 0 (include/utils/FillPatchUtils.H:128-129,
//    BCFill.H:244-264), so hu takes the scalar record (mirrored, never
//    negated) and hv the x-momentum record (negated across x walls only);
//  - 2, a closed wall (no counterpart in the reference's inputs): hu takes the
//    x-momentum record, hv the y-momentum record, each negated across the
//    walls normal to it.
// A cell outside in both directions takes the y rule applied to the x ghost,
// so its signs multiply (no stencil here reads such a corner cell).
constexpr int kBcWall = 0;
constexpr int kBcClosedWall = 2;
__host__ __device__ __forceinline__ bool bc_is_wall(int code) { return code == kBcWall || code == kBcClosedWall; }
// Sign flips of the momentum ghost read through an x mirror (xm, at a side of
// code cx) and/or a y mirror (ym, code cy).
__host__ __device__ __forceinline__ void ghost_momentum_signs(bool xm, int cx, bool ym, int cy, bool& neg_u,
                                                              bool& neg_v) {
    neg_u = xm && cx == kBcClosedWall;
    neg_v = (xm && cx == kBcWall) != (ym && cy == kBcClosedWall);
}
// The cell a ghost (i, j) reads its state from (mi, mj) and its terrain from
// (ei, ej), with the momentum sign flips.
__host__ __device__ __forceinline__ void ghost_source(int i, int j, int nx, int ny, int bc_xlo, int bc_xhi,
                                                      int bc_ylo, int bc_yhi, int& mi, int& mj, int& ei, int& ej,
                                                      bool& neg_u, bool& neg_v) {
    mi = i; mj = j;
    bool xm = false, ym = false;
    int cx = -1, cy = -1;
    if (i < 0) { cx = bc_xlo; if (bc_is_wall(cx)) { mi = -1 - i; xm = true; } else mi = 0; }
    else if (i >= nx) { cx = bc_xhi; if (bc_is_wall(cx)) { mi = 2 * nx - 1 - i; xm = true; } else mi = nx - 1; }
    if (j < 0) { cy = bc_ylo; if (bc_is_wall(cy)) { mj = -1 - j; ym = true; } else mj = 0; }
    else if (j >= ny) { cy = bc_yhi; if (bc_is_wall(cy)) { mj = 2 * ny - 1 - j; ym = true; } else mj = ny - 1; }
    ei = i < 0 ? 0 : (i >= nx ? nx - 1 : i);
    ej = j < 0 ? 0 : (j >= ny ? ny - 1 : j);
    ghost_momentum_signs(xm, cx, ym, cy, neg_u, neg_v);
}

// A whole level as one box with no stored ghosts: the physical-boundary ghost
// values of include/boundaries/BCFill.H:35-86 are generated here, by the
// rules of ghost_source (walls mirror, open sides copy the edge; momentum
// signs by the wall's BC records; terrain always copies the edge).
template <class R> struct LevelSrc {
    static constexpr bool kInterior = true;  // has interior() / fetch_in()
    const R* h; const R* hu; const R* hv; const R* z; const R* n;
    long long pitch;
    int nx, ny;
    int bc_xlo, bc_xhi, bc_ylo, bc_yhi;
    int glo0, glo1, ghi0, ghi1;  // grown region that may be fetched

    __device__ __forceinline__ bool inside(int i, int j) const {
        return i >= glo0 && i <= ghi0 && j >= glo1 && j <= ghi1;
    }
    // true when cells (i0, j0) .. (i1, j1) all lie in the level
    __device__ __forceinline__ bool interior(int i0, int j0, int i1, int j1) const {
        return i0 >= 0 && j0 >= 0 && i1 < nx && j1 < ny;
    }
    // (h, z, hu, hv) of a cell of the level, as stored
    __device__ __forceinline__ void fetch_in(int i, int j, R& hh, R& zz, R& qx, R& qy) const {
        const long long p = (long long)i + (long long)j * pitch;
        hh = ld_ro(h + p);
        zz = ld_ro(z + p);
        qx = ld_ro(hu + p);
        qy = ld_ro(hv + p);
    }
    // (eta, z, hu, hv, n) of any cell in the grown region.
    __device__ __forceinline__ void fetch(int i, int j, R& eta, R& zz, R& qx, R& qy, R& nn) const {
        int mi, mj, ei, ej;
        bool neg_u, neg_v;
        ghost_source(i, j, nx, ny, bc_xlo, bc_xhi, bc_ylo, bc_yhi, mi, mj, ei, ej, neg_u, neg_v);
        const long long pm = (long long)mi + (long long)mj * pitch;
        const long long pe = (long long)ei + (long long)ej * pitch;
        eta = ld_ro(h + pm) + ld_ro(z + pm);
        zz = ld_ro(z + pe);
        nn = ld_ro(n + pe);
        const R a = ld_ro(hu + pm), b = ld_ro(hv + pm);
        qx = neg_u ? -a : a;
        qy = neg_v ? -b : b;
    }
};

// A level of several boxes (a same-level BoxArray).  Each box keeps its own
// valid-cell arrays; a ghost of one box inside the domain is read from the
// box that owns that cell, found through a map of the domain at the boxes'
// common granularity, and one outside the domain follows the physical rules
// of LevelSrc (reflect / extrapolate, terrain always extrapolated) before the
// lookup.  This replaces the FillPatch of same-level and physical ghosts.
struct DevBox {
    const double *h[2], *hu[2], *hv[2];  // the two states of the time loop
    const double *z, *n;
    long long pitch;
    int lo0, lo1, hi0, hi1;
};
struct BoxSetSrc {
    static constexpr bool kInterior = true;  // has interior() / fetch_in()
    const DevBox* boxes;
    const int* map;   // box index of each g x g block of the domain
    int g, mnx;       // granularity, map row length
    int nx, ny;
    int bc_xlo, bc_xhi, bc_ylo, bc_yhi;
    int self, phase;  // the tile's box, which state is current
    int glo0, glo1, ghi0, ghi1;
    __device__ __forceinline__ bool inside(int i, int j) const {
        return i >= glo0 && i <= ghi0 && j >= glo1 && j <= ghi1;
    }
    __device__ __forceinline__ int owner(int i, int j) const {
        const DevBox& b = boxes[self];
        if (i >= b.lo0 && i <= b.hi0 && j >= b.lo1 && j <= b.hi1) return self;
        return ld_ro(map + (long long)(j / g) * mnx + i / g);
    }
    // true when cells (i0, j0) .. (i1, j1) all lie in the domain
    __device__ __forceinline__ bool interior(int i0, int j0, int i1, int j1) const {
        return i0 >= 0 && j0 >= 0 && i1 < nx && j1 < ny;
    }
    // (h, z, hu, hv) of a cell of the domain, as the box that owns it stores them
    __device__ __forceinline__ void fetch_in(int i, int j, double& hh, double& zz, double& qx, double& qy) const {
        const DevBox& b = boxes[owner(i, j)];
        const long long p = (long long)(i - b.lo0) + (long long)(j - b.lo1) * b.pitch;
        hh = ld_ro(b.h[phase] + p);
        zz = ld_ro(b.z + p);
        qx = ld_ro(b.hu[phase] + p);
        qy = ld_ro(b.hv[phase] + p);
    }
    __device__ __forceinline__ void fetch(int i, int j, double& eta, double& zz, double& qx, double& qy,
                                          double& nn) const {
        int mi, mj, ei, ej;
        bool neg_u, neg_v;
        ghost_source(i, j, nx, ny, bc_xlo, bc_xhi, bc_ylo, bc_yhi, mi, mj, ei, ej, neg_u, neg_v);
        const DevBox& bm = boxes[owner(mi, mj)];
        const DevBox& be = boxes[owner(ei, ej)];
        const long long pm = (long long)(mi - bm.lo0) + (long long)(mj - bm.lo1) * bm.pitch;
        const long long pe = (long long)(ei - be.lo0) + (long long)(ej - be.lo1) * be.pitch;
        eta = ld_ro(bm.h[phase] + pm) + ld_ro(bm.z + pm);
        zz = ld_ro(be.z + pe);
        nn = ld_ro(be.n + pe);
        const double a = ld_ro(bm.hu[phase] + pm), b = ld_ro(bm.hv[phase] + pm);
        qx = neg_u ? -a : a;
        qy = neg_v ? -b : b;
    }
};

// A box whose ghosts were filled by AMReX (FillPatch): read them as they are.
template <class R> struct BoxSrc {
    V4<R> eta, U, T;  // eta comp 0; U comps 1,2 (hu, hv); T comps 0,1 (z, n)
    int glo0, glo1, ghi0, ghi1;
    __device__ __forceinline__ bool inside(int i, int j) const {
        return i >= glo0 && i <= ghi0 && j >= glo1 && j <= ghi1;
    }
    __device__ __forceinline__ void fetch(int i, int j, R& e, R& zz, R& qx, R& qy, R& nn) const {
        e = eta.ld(i, j, 0);
        zz = T.ld(i, j, 0);
        nn = T.ld(i, j, 1);
        qx = U.ld(i, j, 1);
        qy = U.ld(i, j, 2);
    }
};

// Per-step control.  dt is either a host value (dt_in == nullptr) or cfl times
// the min CFL bound held in the accumulator dt_in (level time loop).
template <class R> struct StepCtl {
    R dt_host;
    R cfl;
    const struct DtAccum* dt_in;
    struct DtAccum* dt_out;       // next-step bound of the updated state (may be null)
    struct DtAccum* dt_reset;     // accumulator to clear for the step after next (may be null)
    unsigned* status;      // may be null
    R* time;               // simulated time, advanced by block 0 (may be null)
    R dx, dy;
};

// What a forward step of the adjoint's sweep records: the dt it used and h of
// its input state at the gauge cells (null pointers: nothing).
struct AdjRecord {
    double* dt;
    double* series;
    const long long* gauges;
    int ngauges;
};

// One member of a batched ensemble (device memory, one per instance).
template <class R> struct EnsInstance {
    R* st[2][3];          // state planes (h, hu, hv) for the two parities
    const R* z;
    const R* n;
    long long pitch;
    long long tile_base;  // queue index of the instance's first tile
    int nx, ny;
    R dx, dy;
    int bc[4];            // x-lo, x-hi, y-lo, y-hi codes
    int shape;            // tile shape id (HX_TILE_*)
    int tiles_x;
    struct DtAccum* slots;  // three accumulators
    unsigned* status;
    R* time;
};

}  // namespace hx
