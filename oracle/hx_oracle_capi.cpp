// C entry points of the CPU oracle (TEST INFRASTRUCTURE ONLY; see hx_oracle.hpp).
// Loaded with ctypes by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline; never by the product library.
//
// Planes are x-fastest with pitch nx (cell (i, j) at i + j * nx).  Boundary
// codes follow the inputs file (HydroEXA.lo_bc / hi_bc: 0 reflective wall,
// anything else transmissive).
#include "hx_oracle.hpp"

#include <omp.h>

using namespace hxo;

namespace {

template <class R>
Level<R> make_level(int nx, int ny, R dx, R dy, const int* lo, const int* hi) {
    Level<R> L;
    L.nx = nx; L.ny = ny; L.dx = dx; L.dy = dy;
    L.bc_lo[0] = lo[0]; L.bc_lo[1] = lo[1];
    L.bc_hi[0] = hi[0]; L.bc_hi[1] = hi[1];
    return L;
}

// Single-level time loop of the reference driver (src/HydroEXA.cpp:259-266,
// AmrMeshState_Physics.cpp:13-45 and :104-108 at one level): each step takes
// dt = cfl * min(per-cell bound) of the current state, aborts (status 1) when
// the minimum is below 1e-12, then advances.  The state is updated in place.
template <class R>
int run(int method, const Level<R>& L, R* h, R* hu, R* hv, const R* z, const R* n, int nsteps, R cfl, int mode,
        R* t_out, R* dt_last) {
    const size_t N = (size_t)L.nx * L.ny;
    std::vector<R> a(N), b(N), c(N);
    R t = 0;
    R dt = 0;
    for (int s = 0; s < nsteps; ++s) {
        R mn, mx;
        compute_dt(L, h, hu, hv, z, mn, mx);
        if (mn < 1.e-12) { if (t_out) *t_out = t; return 1; }
        dt = mn * cfl;
        if (method == 1) advance_hydrostatic(L, h, hu, hv, z, n, dt, a.data(), b.data(), c.data(), mode);
        else advance_classic(L, h, hu, hv, z, n, dt, a.data(), b.data(), c.data());
        std::copy(a.begin(), a.end(), h);
        std::copy(b.begin(), b.end(), hu);
        std::copy(c.begin(), c.end(), hv);
        t += dt;
    }
    if (t_out) *t_out = t;
    if (dt_last) *dt_last = dt;
    return 0;
}

}  // namespace

#define HXO_DEFINE(R, SUF)                                                                                          \
    extern "C" void hxo_roe_hydrostatic_points_##SUF(long n, const R* in, const R* nrm, R* F) {                   \
        for (long p = 0; p < n; ++p) {                                                                              \
            const R* q = in + 6 * p;                                                                                \
            R f[3];                                                                                                 \
            roe_hydrostatic<R>(q[0], q[1], q[2], q[3], q[4], q[5], f, nrm[2 * p], nrm[2 * p + 1]);                 \
            F[3 * p] = f[0]; F[3 * p + 1] = f[1]; F[3 * p + 2] = f[2];                                              \
        }                                                                                                           \
    }                                                                                                               \
    extern "C" void hxo_roe_classic_points_##SUF(long n, const R* in, const R* aux, R* F, R* Sm, R* Sp) {         \
        for (long p = 0; p < n; ++p) {                                                                              \
            const R* q = in + 10 * p;                                                                               \
            const R* a = aux + 4 * p;                                                                               \
            R f[3], sm[3], sp[3];                                                                                   \
            roe_classic<R>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], f, sm, sp, a[0], a[1], a[2], \
                           a[3]);                                                                                   \
            for (int c = 0; c < 3; ++c) { F[3 * p + c] = f[c]; Sm[3 * p + c] = sm[c]; Sp[3 * p + c] = sp[c]; }     \
        }                                                                                                           \
    }                                                                                                               \
    extern "C" void hxo_van_leer_slope_points_##SUF(long n, const R* q3, int mode, R* out) {                       \
        for (long p = 0; p < n; ++p) out[p] = van_leer_slope<R>(q3[3 * p], q3[3 * p + 1], q3[3 * p + 2], mode);     \
    }                                                                                                               \
    extern "C" void hxo_advance_hydrostatic_##SUF(int nx, int ny, R dx, R dy, const int* lo, const int* hi,        \
                                                  const R* h, const R* hu, const R* hv, const R* z, const R* n,     \
                                                  R dt, R* ho, R* huo, R* hvo, int mode) {                           \
        advance_hydrostatic<R>(make_level<R>(nx, ny, dx, dy, lo, hi), h, hu, hv, z, n, dt, ho, huo, hvo, mode);    \
    }                                                                                                               \
    extern "C" void hxo_advance_hydrostatic_faces_##SUF(int nx, int ny, R dx, R dy, const int* lo, const int* hi,  \
                                                        const R* h, const R* hu, const R* hv, const R* z,           \
                                                        const R* n, R dt, R* ho, R* huo, R* hvo, int mode, R* FLx,  \
                                                        R* FRx, R* FLy, R* FRy) {                                   \
        Faces<R> Fc;                                                                                                \
        advance_hydrostatic<R>(make_level<R>(nx, ny, dx, dy, lo, hi), h, hu, hv, z, n, dt, ho, huo, hvo, mode,     \
                               &Fc);                                                                                \
        std::copy(Fc.xa.begin(), Fc.xa.end(), FLx);                                                                 \
        std::copy(Fc.xb.begin(), Fc.xb.end(), FRx);                                                                 \
        std::copy(Fc.ya.begin(), Fc.ya.end(), FLy);                                                                 \
        std::copy(Fc.yb.begin(), Fc.yb.end(), FRy);                                                                 \
    }                                                                                                               \
    extern "C" void hxo_advance_classic_##SUF(int nx, int ny, R dx, R dy, const int* lo, const int* hi,            \
                                              const R* h, const R* hu, const R* hv, const R* z, const R* n, R dt,   \
                                              R* ho, R* huo, R* hvo) {                                              \
        advance_classic<R>(make_level<R>(nx, ny, dx, dy, lo, hi), h, hu, hv, z, n, dt, ho, huo, hvo);              \
    }                                                                                                               \
    extern "C" void hxo_advance_classic_faces_##SUF(int nx, int ny, R dx, R dy, const int* lo, const int* hi,      \
                                                    const R* h, const R* hu, const R* hv, const R* z, const R* n,   \
                                                    R dt, R* ho, R* huo, R* hvo, R* Fx, R* Smx, R* Spx, R* Fy,      \
                                                    R* Smy, R* Spy) {                                               \
        Faces<R> Fc;                                                                                                \
        advance_classic<R>(make_level<R>(nx, ny, dx, dy, lo, hi), h, hu, hv, z, n, dt, ho, huo, hvo, &Fc);         \
        std::copy(Fc.xa.begin(), Fc.xa.end(), Fx);                                                                  \
        std::copy(Fc.xb.begin(), Fc.xb.end(), Smx);                                                                 \
        std::copy(Fc.xc.begin(), Fc.xc.end(), Spx);                                                                 \
        std::copy(Fc.ya.begin(), Fc.ya.end(), Fy);                                                                  \
        std::copy(Fc.yb.begin(), Fc.yb.end(), Smy);                                                                 \
        std::copy(Fc.yc.begin(), Fc.yc.end(), Spy);                                                                 \
    }                                                                                                               \
    extern "C" void hxo_compute_dt_##SUF(int nx, int ny, R dx, R dy, const R* h, const R* hu, const R* hv,          \
                                         const R* z, R* dtmin, R* maxvel) {                                         \
        int lo[2] = {0, 0}, hi[2] = {0, 0};                                                                         \
        compute_dt<R>(make_level<R>(nx, ny, dx, dy, lo, hi), h, hu, hv, z, *dtmin, *maxvel);                        \
    }                                                                                                               \
    extern "C" int hxo_run_##SUF(int method, int nx, int ny, R dx, R dy, const int* lo, const int* hi, R* h, R* hu, \
                                 R* hv, const R* z, const R* n, int nsteps, R cfl, int mode, R* t_out,              \
                                 R* dt_last) {                                                                      \
        return run<R>(method, make_level<R>(nx, ny, dx, dy, lo, hi), h, hu, hv, z, n, nsteps, cfl, mode, t_out,    \
                      dt_last);                                                                                     \
    }                                                                                                               \
    extern "C" void hxo_tag_cells_##SUF(int variant, const R* U, long long ujs, long long uns, int ulo0, int ulo1,  \
                                        const R* T, long long tjs, long long tns, int tlo0, int tlo1,               \
                                        signed char* tags, long long gjs, int glo0, int glo1, int vlo0, int vlo1,   \
                                        int vhi0, int vhi1, R dx, R dy, R time, R h_th, R u_th, R z_th,             \
                                        signed char set_value) {                                                    \
        View<const R> Uv{U, ujs, uns, ulo0, ulo1};                                                                  \
        View<const R> Tv{T, tjs, tns, tlo0, tlo1};                                                                  \
        View<signed char> Gv{tags, gjs, 0, glo0, glo1};                                                             \
        tag_cells<R>(variant, Uv, Tv, Gv, vlo0, vlo1, vhi0, vhi1, dx, dy, time, h_th, u_th, z_th, set_value);       \
    }                                                                                                               \
    extern "C" void hxo_masked_average_down_##SUF(const R* fine, long long fjs, long long fns, int flo0, int flo1,  \
                                                  R* crse, long long cjs, long long cns, int clo0, int clo1,        \
                                                  int bx_lo0, int bx_lo1, int bx_hi0, int bx_hi1, int ncomp, int rx,\
                                                  int ry, R fv, R nodata) {                                         \
        View<const R> Fv{fine, fjs, fns, flo0, flo1};                                                               \
        View<R> Cv{crse, cjs, cns, clo0, clo1};                                                                     \
        masked_average_down<R>(Fv, Cv, bx_lo0, bx_lo1, bx_hi0, bx_hi1, ncomp, rx, ry, fv, nodata);                 \
    }                                                                                                               \
    extern "C" void hxo_average_down_##SUF(const R* fine, long long fjs, long long fns, int flo0, int flo1,          \
                                           R* crse, long long cjs, long long cns, int clo0, int clo1, int bx_lo0,    \
                                           int bx_lo1, int bx_hi0, int bx_hi1, int scomp, int ccomp, int ncomp,      \
                                           int rx, int ry) {                                                         \
        View<const R> Fv{fine, fjs, fns, flo0, flo1};                                                               \
        View<R> Cv{crse, cjs, cns, clo0, clo1};                                                                     \
        average_down<R>(Fv, Cv, bx_lo0, bx_lo1, bx_hi0, bx_hi1, scomp, ccomp, ncomp, rx, ry);                       \
    }                                                                                                               \
    extern "C" void hxo_mass_diagnostics_##SUF(int nx, int ny, long long pitch, const R* h, const R* hu,            \
                                               const R* hv, const R* n, R dx, R dy, double* out) {                  \
        mass_diagnostics<R>(nx, ny, pitch, h, hu, hv, n, dx, dy, out);                                              \
    }                                                                                                               \
    extern "C" void hxo_derive_eta_##SUF(long long count, const R* h, const R* z, R* eta) {                         \
        derive_eta<R>(count, h, z, eta);                                                                            \
    }

HXO_DEFINE(double, f64)
HXO_DEFINE(float, f32)

extern "C" void hxo_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
extern "C" int hxo_max_threads() { return omp_get_max_threads(); }
