// C-ABI layer: argument checks, view conversion and launches.  Sees only the
// launcher declarations (hx_launch.h), never the kernel bodies, so each
// arithmetic form is compiled exactly once with its own flags.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "hx_launch.h"

using namespace hx;

namespace {

thread_local std::string g_err;
std::atomic<unsigned long long> g_launches{0};

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int launched(cudaError_t e, const char* what, int n = 1) {
    if (e != cudaSuccess) return fail(HX_ERR_LAUNCH, "%s: %s", what, cudaGetErrorString(e));
    g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed);
    return HX_OK;
}

template <class A> struct Elem;
template <> struct Elem<hx_array4_f64> { using T = double; };
template <> struct Elem<hx_array4_f32> { using T = float; };
template <> struct Elem<hx_array4_i8> { using T = signed char; };
template <> struct Elem<hx_array4_i32> { using T = int; };

template <class A> V4<typename Elem<A>::T> to_v4(const A& a) {
    V4<typename Elem<A>::T> v;
    v.p = a.p;
    v.js = a.jstride;
    v.ns = a.nstride;
    v.lo0 = a.lo[0];
    v.lo1 = a.lo[1];
    v.hi0 = a.hi[0];
    v.hi1 = a.hi[1];
    v.nc = a.ncomp;
    return v;
}

// The view must hold comps [0, ncomp) over [lo0-g, hi0+g] x [lo1-g, hi1+g].
template <class A> bool covers(const A* a, const hx_box& b, int g, int ncomp, const char* name) {
    if (!a || !a->p) { fail(HX_ERR_ARG, "%s: null view", name); return false; }
    if (a->ncomp < ncomp) { fail(HX_ERR_ARG, "%s: needs %d components, has %d", name, ncomp, a->ncomp); return false; }
    if (a->lo[0] > b.lo[0] - g || a->lo[1] > b.lo[1] - g || a->hi[0] < b.hi[0] + g || a->hi[1] < b.hi[1] + g) {
        fail(HX_ERR_ARG, "%s: view [%d,%d]x[%d,%d] does not cover [%d,%d]x[%d,%d]", name, a->lo[0], a->hi[0], a->lo[1],
             a->hi[1], b.lo[0] - g, b.hi[0] + g, b.lo[1] - g, b.hi[1] + g);
        return false;
    }
    if (a->jstride < (int64_t)(a->hi[0] - a->lo[0] + 1)) { fail(HX_ERR_ARG, "%s: jstride too small", name); return false; }
    return true;
}

bool box_ok(const hx_box& b) {
    if (b.hi[0] < b.lo[0] || b.hi[1] < b.lo[1]) { fail(HX_ERR_ARG, "empty box"); return false; }
    return true;
}

IBox ibox(const hx_box& b) { return IBox{b.lo[0], b.lo[1], b.hi[0], b.hi[1]}; }

template <class A> Cells3<typename Elem<A>::T> cells3(const A& a) {
    Cells3<typename Elem<A>::T> c;
    for (int k = 0; k < 3; ++k) c.p[k] = a.p + (int64_t)k * a.nstride;
    c.js = a.jstride;
    c.lo0 = a.lo[0];
    c.lo1 = a.lo[1];
    return c;
}
template <class A> Cells3W<typename Elem<A>::T> cells3w(const A& a) {
    Cells3W<typename Elem<A>::T> c;
    for (int k = 0; k < 3; ++k) c.p[k] = a.p + (int64_t)k * a.nstride;
    c.js = a.jstride;
    c.lo0 = a.lo[0];
    c.lo1 = a.lo[1];
    return c;
}
template <class A> Plane<typename Elem<A>::T> plane(const A& a, int comp) {
    Plane<typename Elem<A>::T> p;
    p.p = a.p + (int64_t)comp * a.nstride;
    p.js = a.jstride;
    p.lo0 = a.lo[0];
    p.lo1 = a.lo[1];
    return p;
}

template <class R> StepCtl<R> host_ctl(R dt, R dx, R dy, hx_dt_accum* next_dt, uint32_t* status) {
    StepCtl<R> c;
    c.dt_host = dt;
    c.cfl = R(1);
    c.dt_in = nullptr;
    c.dt_out = reinterpret_cast<DtAccum*>(next_dt);
    c.dt_reset = nullptr;
    c.status = status;
    c.time = nullptr;
    c.dx = dx;
    c.dy = dy;
    return c;
}

// ---------------------------------------------------------------- box forms
template <class R, class A>
int advance_box_hydro(const A* eta, const A* Ue, const A* Te, const A* Uo, A* Un, hx_box vb, R dt, R dx, R dy,
                      const A* FL, const A* FR, hx_dt_accum* nd, uint32_t* status, int arith, cudaStream_t st,
                      const A* Fm = nullptr, const EpiOut<R>* epi = nullptr) {
    if (!box_ok(vb)) return HX_ERR_ARG;
    if (!covers(eta, vb, 2, 1, "eta_ext") || !covers(Ue, vb, 2, 3, "U_ext") || !covers(Te, vb, 2, 2, "T_ext") ||
        !covers(Uo, vb, 0, 3, "U_old") || !covers(Un, vb, 0, 3, "U_new"))
        return HX_ERR_ARG;
    if (!(dx > R(0)) || !(dy > R(0))) return fail(HX_ERR_ARG, "dx, dy must be positive");
    FaceOut<R> fo{};
    fo.on = 0;
    if (FL || FR) {
        if (!FL || !FR) return fail(HX_ERR_ARG, "FL and FR come together");
        hx_box bx{{vb.lo[0], vb.lo[1]}, {vb.hi[0] + 1, vb.hi[1]}};
        hx_box by{{vb.lo[0], vb.lo[1]}, {vb.hi[0], vb.hi[1] + 1}};
        if (!covers(&FL[0], bx, 0, 3, "FL[x]") || !covers(&FR[0], bx, 0, 3, "FR[x]") ||
            !covers(&FL[1], by, 0, 3, "FL[y]") || !covers(&FR[1], by, 0, 3, "FR[y]"))
            return HX_ERR_ARG;
        for (int d = 0; d < 2; ++d) { fo.FL[d] = to_v4(FL[d]); fo.FR[d] = to_v4(FR[d]); }
        fo.on = 1;
    }
    if (Fm) {
        hx_box bx{{vb.lo[0], vb.lo[1]}, {vb.hi[0] + 1, vb.hi[1]}};
        hx_box by{{vb.lo[0], vb.lo[1]}, {vb.hi[0], vb.hi[1] + 1}};
        if (!covers(&Fm[0], bx, 0, 3, "Freg[x]") || !covers(&Fm[1], by, 0, 3, "Freg[y]")) return HX_ERR_ARG;
        for (int d = 0; d < 2; ++d) fo.Fm[d] = to_v4(Fm[d]);
        fo.mean = 1;
    }
    BoxSrc<R> src;
    src.eta = to_v4(*eta);
    src.U = to_v4(*Ue);
    src.T = to_v4(*Te);
    src.glo0 = vb.lo[0] - 2; src.glo1 = vb.lo[1] - 2; src.ghi0 = vb.hi[0] + 2; src.ghi1 = vb.hi[1] + 2;
    const StepCtl<R> ctl = host_ctl<R>(dt, dx, dy, nd, status);
    cudaError_t e = (arith == HX_ARITH_EXACT)
                        ? launch_hydro<R, false, BoxSrc<R>>(src, cells3(*Uo), plane(*Te, 1), cells3w(*Un), fo, ibox(vb), ctl, st, epi)
                        : launch_hydro<R, true, BoxSrc<R>>(src, cells3(*Uo), plane(*Te, 1), cells3w(*Un), fo, ibox(vb), ctl, st, epi);
    return launched(e, "hx_advance_box_hydrostatic");
}

// The epilogue's outputs over the valid box vb: eta (one component covering vb)
// and the diagnostics with their work buffer; false (error set) when a given
// output is malformed or neither is given.
template <class R, class A>
bool epi_out(A* eta, double* diag, void* work, hx_box vb, R dA, EpiOut<R>& e, const char* who) {
    e = EpiOut<R>{};
    if (!eta && !diag) { fail(HX_ERR_ARG, "%s: neither eta nor diagnostics asked for", who); return false; }
    if (eta) {
        if (!covers(eta, vb, 0, 1, "eta_new")) return false;
        e.eta = eta->p;
        e.ejs = eta->jstride;
        e.elo0 = eta->lo[0];
        e.elo1 = eta->lo[1];
    }
    if (diag) {
        if (!work) { fail(HX_ERR_ARG, "%s: diagnostics need a work buffer", who); return false; }
        e.part = static_cast<double*>(work);
        e.out = diag;
    }
    e.dA = dA;
    return true;
}

template <class R, class A>
int advance_box_hydro_epi(const A* eta, const A* Ue, const A* Te, const A* Uo, A* Un, hx_box vb, R dt, R dx, R dy,
                          hx_dt_accum* nd, uint32_t* status, int arith, A* eta_new, double* diag, void* work,
                          cudaStream_t st) {
    if (!box_ok(vb)) return HX_ERR_ARG;
    EpiOut<R> e;
    if (!epi_out<R>(eta_new, diag, work, vb, dx * dy, e, "hx_advance_box_hydrostatic_epilogue")) return HX_ERR_ARG;
    return advance_box_hydro<R, A>(eta, Ue, Te, Uo, Un, vb, dt, dx, dy, nullptr, nullptr, nd, status, arith, st,
                                   nullptr, &e);
}

template <class R, class A>
int advance_box_roe(const A* eta, A* Uo, const A* T, A* Un, hx_box vb, R dt, R dx, R dy, const A* F, const A* Sm,
                    const A* Sp, hx_dt_accum* nd, uint32_t* status, int arith, cudaStream_t st,
                    const hx_array4_i32* mask = nullptr, const hx_box* grid = nullptr, const A* fc = nullptr,
                    const A* ff = nullptr) {
    if (!box_ok(vb)) return HX_ERR_ARG;
    if (!covers(eta, vb, 1, 1, "eta") || !covers(Uo, vb, 1, 3, "U_old") || !covers(T, vb, 1, 2, "T") ||
        !covers(Un, vb, 0, 3, "U_new"))
        return HX_ERR_ARG;
    if (!(dx > R(0)) || !(dy > R(0))) return fail(HX_ERR_ARG, "dx, dy must be positive");
    FaceOut9<R> fo{};
    fo.on = 0;
    if (F || Sm || Sp) {
        if (!F || !Sm || !Sp) return fail(HX_ERR_ARG, "F, Sm and Sp come together");
        hx_box bx{{vb.lo[0], vb.lo[1]}, {vb.hi[0] + 1, vb.hi[1]}};
        hx_box by{{vb.lo[0], vb.lo[1]}, {vb.hi[0], vb.hi[1] + 1}};
        for (int d = 0; d < 2; ++d) {
            const hx_box& b = d ? by : bx;
            if (!covers(&F[d], b, 0, 3, "F") || !covers(&Sm[d], b, 0, 3, "Sm") || !covers(&Sp[d], b, 0, 3, "Sp"))
                return HX_ERR_ARG;
            fo.F[d] = to_v4(F[d]); fo.Sm[d] = to_v4(Sm[d]); fo.Sp[d] = to_v4(Sp[d]);
        }
        fo.on = 1;
    }
    if (fc || ff) {
        hx_box bx{{vb.lo[0], vb.lo[1]}, {vb.hi[0] + 1, vb.hi[1]}};
        hx_box by{{vb.lo[0], vb.lo[1]}, {vb.hi[0], vb.hi[1] + 1}};
        if (fc) {
            if (!mask) return fail(HX_ERR_ARG, "flux_crse needs fine_mask");
            if (!covers(mask, vb, 1, 1, "fine_mask") || !covers(&fc[0], bx, 0, 3, "flux_crse[x]") ||
                !covers(&fc[1], by, 0, 3, "flux_crse[y]"))
                return HX_ERR_ARG;
            fo.mask = to_v4(*mask);
            for (int d = 0; d < 2; ++d) fo.fc[d] = to_v4(fc[d]);
            fo.crse_on = 1;
        }
        if (ff) {
            if (!grid || grid->hi[0] < grid->lo[0] || grid->hi[1] < grid->lo[1])
                return fail(HX_ERR_ARG, "flux_fine needs the grid box");
            if (!covers(&ff[0], bx, 0, 3, "flux_fine[x]") || !covers(&ff[1], by, 0, 3, "flux_fine[y]"))
                return HX_ERR_ARG;
            fo.grid = ibox(*grid);
            for (int d = 0; d < 2; ++d) fo.ff[d] = to_v4(ff[d]);
            fo.fine_on = 1;
        }
    }
    BoxSrc<R> src;
    src.eta = to_v4(*eta);
    src.U = to_v4(*Uo);
    src.T = to_v4(*T);
    src.glo0 = vb.lo[0] - 1; src.glo1 = vb.lo[1] - 1; src.ghi0 = vb.hi[0] + 1; src.ghi1 = vb.hi[1] + 1;
    RebuildOut<R> hb;
    hb.U = to_v4(*Uo);
    hb.on = 1;
    const StepCtl<R> ctl = host_ctl<R>(dt, dx, dy, nd, status);
    cudaError_t e = (arith == HX_ARITH_EXACT)
                        ? launch_classic<R, false, BoxSrc<R>>(src, cells3w(*Un), fo, hb, ibox(vb), ctl, st)
                        : launch_classic<R, true, BoxSrc<R>>(src, cells3w(*Un), fo, hb, ibox(vb), ctl, st);
    return launched(e, "hx_advance_box_roe");
}

template <class R, class A>
int dt_reduce_box(const A* U, const A* T, hx_box vb, R dx, R dy, hx_dt_accum* acc, cudaStream_t st) {
    if (!box_ok(vb)) return HX_ERR_ARG;
    if (!covers(U, vb, 0, 3, "U") || !covers(T, vb, 0, 1, "T")) return HX_ERR_ARG;
    if (!acc) return fail(HX_ERR_ARG, "null accumulator");
    // exact form: the bound is a monotone function of exactly rounded terms
    return launched(launch_dt_reduce<R, false>(cells3(*U), plane(*T, 0), ibox(vb), dx, dy,
                                               reinterpret_cast<DtAccum*>(acc), st),
                    "hx_dt_reduce_box");
}

template <class R, class A>
int tag_box(int method, const A* U, const A* T, hx_array4_i8* tags, hx_box vb, R dx, R dy, R time, R hth, R uth,
            R zth, signed char setv, cudaStream_t st) {
    if (!box_ok(vb)) return HX_ERR_ARG;
    if (method != HX_METHOD_ROE && method != HX_METHOD_HYDROSTATIC_ROE) return fail(HX_ERR_ARG, "unknown method");
    if (!covers(U, vb, 1, 3, "U") || !covers(T, vb, 1, 1, "T") || !covers(tags, vb, 0, 1, "tags")) return HX_ERR_ARG;
    return launched(launch_tag<R>(method, to_v4(*U), to_v4(*T), to_v4(*tags), ibox(vb), dx, dy, time, hth, uth, zth,
                                  setv, st),
                    "hx_tag_box");
}

template <class R, class A>
int avgdown_box(const A* fine, A* crse, hx_box cb, int scomp, int ccomp, int ncomp, int rx, int ry, cudaStream_t st) {
    if (!box_ok(cb)) return HX_ERR_ARG;
    if (rx < 1 || ry < 1 || ncomp < 1 || scomp < 0 || ccomp < 0) return fail(HX_ERR_ARG, "bad ratio or components");
    hx_box fb{{cb.lo[0] * rx, cb.lo[1] * ry}, {cb.hi[0] * rx + rx - 1, cb.hi[1] * ry + ry - 1}};
    if (!covers(fine, fb, 0, scomp + ncomp, "fine") || !covers(crse, cb, 0, ccomp + ncomp, "crse")) return HX_ERR_ARG;
    return launched(launch_average_down<R>(to_v4(*fine), to_v4(*crse), ibox(cb), scomp, ccomp, ncomp, rx, ry, st),
                    "hx_average_down_box");
}

template <class R, class A>
int mavg_box(const A* fine, A* crse, hx_box cb, int scomp, int ccomp, int ncomp, int rx, int ry, R fv, R nodata,
             cudaStream_t st) {
    if (!box_ok(cb)) return HX_ERR_ARG;
    if (rx < 1 || ry < 1 || ncomp < 1 || scomp < 0 || ccomp < 0) return fail(HX_ERR_ARG, "bad ratio or components");
    hx_box fb{{cb.lo[0] * rx, cb.lo[1] * ry}, {cb.hi[0] * rx + rx - 1, cb.hi[1] * ry + ry - 1}};
    if (!covers(fine, fb, 0, scomp + ncomp, "fine") || !covers(crse, cb, 0, ccomp + ncomp, "crse")) return HX_ERR_ARG;
    return launched(launch_masked_avgdown<R>(to_v4(*fine), to_v4(*crse), ibox(cb), scomp, ccomp, ncomp, rx, ry, fv,
                                             nodata, st),
                    "hx_masked_average_down_box");
}

template <class R, class A>
int eta_box(const A* U, const A* T, A* eta, hx_box b, cudaStream_t st) {
    if (!box_ok(b)) return HX_ERR_ARG;
    if (!covers(U, b, 0, 1, "U") || !covers(T, b, 0, 1, "terrain") || !covers(eta, b, 0, 1, "eta")) return HX_ERR_ARG;
    return launched(launch_derive_eta<R>(to_v4(*U), to_v4(*T), to_v4(*eta), ibox(b), st), "hx_derive_eta_box");
}

template <class R, class A>
Plane<R> comp_plane(const A* a, int c) {
    return Plane<R>{a->p + (long long)c * a->nstride, a->jstride, a->lo[0], a->lo[1]};
}

long long diag_blocks(hx_box b) {
    return (long long)((b.hi[0] - b.lo[0] + TX) / TX) * (long long)((b.hi[1] - b.lo[1] + TY) / TY);
}

template <class R, class A>
int diag_box(const A* U, const A* T, hx_box b, R dx, R dy, double* out, void* work, cudaStream_t st) {
    if (!box_ok(b)) return HX_ERR_ARG;
    if (!out || !work) return fail(HX_ERR_ARG, "hx_diagnostics: null output or work");
    if (!covers(U, b, 0, 3, "U") || !covers(T, b, 0, 2, "terrain")) return HX_ERR_ARG;
    const R dA = dx * dy;
    return launched(launch_diagnostics<R>(comp_plane<R>(U, 0), comp_plane<R>(U, 1), comp_plane<R>(U, 2),
                                          comp_plane<R>(T, 1), ibox(b), dA, static_cast<double*>(work), out, st),
                    "hx_diagnostics_box");
}

// ---------------------------------------------------------------- level forms
template <class L> bool level_ok(const L* lv) {
    if (!lv || !lv->h || !lv->hu || !lv->hv || !lv->z || !lv->n) { fail(HX_ERR_ARG, "level: null plane"); return false; }
    if (lv->nx < 2 || lv->ny < 2) { fail(HX_ERR_ARG, "level: nx, ny must be >= 2"); return false; }
    if (lv->pitch < lv->nx) { fail(HX_ERR_ARG, "level: pitch < nx"); return false; }
    if (!(lv->dx > 0) || !(lv->dy > 0)) { fail(HX_ERR_ARG, "level: dx, dy must be positive"); return false; }
    return true;
}

template <class R, class L> LevelSrc<R> level_src(const L* lv, int g) {
    LevelSrc<R> s;
    s.h = lv->h; s.hu = lv->hu; s.hv = lv->hv; s.z = lv->z; s.n = lv->n;
    s.pitch = lv->pitch;
    s.nx = lv->nx; s.ny = lv->ny;
    s.bc_xlo = lv->bc_lo[0]; s.bc_ylo = lv->bc_lo[1]; s.bc_xhi = lv->bc_hi[0]; s.bc_yhi = lv->bc_hi[1];
    s.glo0 = -g; s.glo1 = -g; s.ghi0 = lv->nx - 1 + g; s.ghi1 = lv->ny - 1 + g;
    return s;
}

// One step of the level, or of its rows j0..j1 (the rest of the level is read
// as halo, nothing outside the rows is written).
template <class R, class L>
int level_advance(int method, const L* lv, const StepCtl<R>& ctl, R* ho, R* huo, R* hvo, int arith, cudaStream_t st,
                  int j0 = 0, int j1 = -1, const EpiOut<R>* epi = nullptr) {
    const IBox vb{0, j0, lv->nx - 1, j1 < 0 ? lv->ny - 1 : j1};
    Cells3W<R> out;
    out.p[0] = ho; out.p[1] = huo; out.p[2] = hvo;
    out.js = lv->pitch; out.lo0 = 0; out.lo1 = 0;
    cudaError_t e;
    if (method == HX_METHOD_HYDROSTATIC_ROE) {
        Cells3<R> uo;
        uo.p[0] = lv->h; uo.p[1] = lv->hu; uo.p[2] = lv->hv;
        uo.js = lv->pitch; uo.lo0 = 0; uo.lo1 = 0;
        Plane<R> np{lv->n, lv->pitch, 0, 0};
        FaceOut<R> fo{};
        fo.on = 0;
        const LevelSrc<R> src = level_src<R>(lv, 2);
        e = (arith == HX_ARITH_EXACT) ? launch_hydro<R, false, LevelSrc<R>>(src, uo, np, out, fo, vb, ctl, st, epi)
                                      : launch_hydro<R, true, LevelSrc<R>>(src, uo, np, out, fo, vb, ctl, st, epi);
    } else {
        FaceOut9<R> fo{};
        fo.on = 0;
        RebuildOut<R> hb{};
        hb.on = 0;
        const LevelSrc<R> src = level_src<R>(lv, 1);
        e = (arith == HX_ARITH_EXACT) ? launch_classic<R, false, LevelSrc<R>>(src, out, fo, hb, vb, ctl, st)
                                      : launch_classic<R, true, LevelSrc<R>>(src, out, fo, hb, vb, ctl, st);
    }
    return launched(e, "hx_level_advance");
}

template <class R, class L>
int level_advance_epi(const L* lv, R dt, R* ho, R* huo, R* hvo, hx_dt_accum* nd, uint32_t* status, int arith,
                      R* eta_out, double* diag, void* work, cudaStream_t st) {
    if (!level_ok(lv)) return HX_ERR_ARG;
    if (!ho || !huo || !hvo) return fail(HX_ERR_ARG, "null output planes");
    EpiOut<R> e{};
    if (!eta_out && !diag) return fail(HX_ERR_ARG, "hx_level_advance_epilogue: neither eta nor diagnostics asked for");
    if (diag && !work) return fail(HX_ERR_ARG, "hx_level_advance_epilogue: diagnostics need a work buffer");
    e.eta = eta_out;
    e.ejs = lv->pitch;
    e.part = diag ? static_cast<double*>(work) : nullptr;
    e.out = diag;
    e.dA = lv->dx * lv->dy;
    return level_advance<R>(HX_METHOD_HYDROSTATIC_ROE, lv, host_ctl<R>(dt, lv->dx, lv->dy, nd, status), ho, huo, hvo,
                            arith, st, 0, -1, &e);
}

template <class R, class L>
int level_dt(const L* lv, hx_dt_accum* acc, cudaStream_t st, int arith = HX_ARITH_EXACT, int j0 = 0, int j1 = -1) {
    if (!level_ok(lv)) return HX_ERR_ARG;
    if (!acc) return fail(HX_ERR_ARG, "null accumulator");
    Cells3<R> U;
    U.p[0] = lv->h; U.p[1] = lv->hu; U.p[2] = lv->hv;
    U.js = lv->pitch; U.lo0 = 0; U.lo1 = 0;
    Plane<R> Z{lv->z, lv->pitch, 0, 0};
    const IBox vb{0, j0, lv->nx - 1, j1 < 0 ? lv->ny - 1 : j1};  // rows j0..j1 (all by default)
    DtAccum* a = reinterpret_cast<DtAccum*>(acc);
    return launched(arith == HX_ARITH_EXACT ? launch_dt_reduce<R, false>(U, Z, vb, lv->dx, lv->dy, a, st)
                                            : launch_dt_reduce<R, true>(U, Z, vb, lv->dx, lv->dy, a, st),
                    "hx_level_dt_reduce");
}

constexpr int64_t kRunWork = 3 * (int64_t)sizeof(DtAccum);

template <class R, class L>
int level_run(int method, L* lv, R* ha, R* hua, R* hva, int nsteps, R cfl, void* work, uint32_t* status, R* time_dev,
              int arith, int* final_in_alt, cudaStream_t st) {
    if (!level_ok(lv)) return HX_ERR_ARG;
    if (!ha || !hua || !hva) return fail(HX_ERR_ARG, "null alternate planes");
    if (!work) return fail(HX_ERR_ARG, "null work buffer");
    if (nsteps < 0) return fail(HX_ERR_ARG, "nsteps < 0");
    if (!(cfl > R(0))) return fail(HX_ERR_ARG, "cfl must be positive");
    if (method != HX_METHOD_ROE && method != HX_METHOD_HYDROSTATIC_ROE) return fail(HX_ERR_ARG, "unknown method");
    DtAccum* slot = reinterpret_cast<DtAccum*>(work);
    cudaError_t e = cudaMemsetAsync(slot, 0, 2 * sizeof(DtAccum), st);
    if (e != cudaSuccess) return fail(HX_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
    int rc = level_dt<R>(lv, reinterpret_cast<hx_dt_accum*>(&slot[0]), st, arith);
    if (rc) return rc;
    const R* A[3] = {lv->h, lv->hu, lv->hv};
    R* B[3] = {ha, hua, hva};
    L cur = *lv;
    for (int s = 0; s < nsteps; ++s) {
        StepCtl<R> ctl;
        ctl.dt_host = R(0);
        ctl.cfl = cfl;
        ctl.dt_in = &slot[s % 3];
        ctl.dt_out = s + 1 < nsteps ? &slot[(s + 1) % 3] : nullptr;  // no step reads the last one's bound
        ctl.dt_reset = &slot[(s + 2) % 3];
        ctl.status = status;
        ctl.time = time_dev;
        ctl.dx = lv->dx;
        ctl.dy = lv->dy;
        const bool even = (s % 2) == 0;
        cur.h = even ? A[0] : B[0];
        cur.hu = even ? A[1] : B[1];
        cur.hv = even ? A[2] : B[2];
        R* o0 = even ? B[0] : const_cast<R*>(A[0]);
        R* o1 = even ? B[1] : const_cast<R*>(A[1]);
        R* o2 = even ? B[2] : const_cast<R*>(A[2]);
        rc = level_advance<R>(method, &cur, ctl, o0, o1, o2, arith, st);
        if (rc) return rc;
    }
    if (final_in_alt) *final_in_alt = nsteps % 2;
    return HX_OK;
}

template <class R> int accum_read(const hx_dt_accum* acc, R* dtmin, R* maxvel, cudaStream_t st) {
    if (!acc) return fail(HX_ERR_ARG, "null accumulator");
    DtAccum h;
    cudaError_t e = cudaMemcpyAsync(&h, acc, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(HX_ERR_CUDA, "accumulator read: %s", cudaGetErrorString(e));
    if (dtmin) *dtmin = accum_dt_min<R>(h.rate_bits, h.flags);
    if (maxvel) *maxvel = from_bits<R>(h.maxvel_bits);
    return (h.flags & DTF_NAN) ? (int)HX_STATUS_NAN : (int)HX_OK;
}

// ---------------------------------------------------------------- host form
// Device buffers of the host-buffer entry, kept between calls, and three
// streams: uploads and downloads (one each: a copy engine does not interleave
// two streams' queues, so bands go in order on one) and the CFL reduction of
// the uploaded level, at the highest priority, so that its few blocks are
// scheduled ahead of the flux work queued on the caller's stream.  (The
// split bands' updates run on the caller's stream once dt is known: on a
// stream of their own they only got the GPU between two of the persistent
// flux kernels, which hold every SM, and their bands went down late.)
constexpr int kHostBands = 10;  // at most: a short first and last band, up to eight between
constexpr int kHeadRows = 2;  // rows of the next band the flux differences of a band read (the MUSCL reach)
// Share of the rows whose first step is split (flux differences as the rows land, the update once dt is
// known), before a call has measured this host: on GB300 the upload of the level (40 B per cell at
// ~210 GB/s) takes about as long as the flux work of 45% of the rows (~3.1 us per row of 8192 cells).
constexpr double kSplitFrac = 0.45;
// The split share for the next call from this call's upload time and the fused bands' time per row: the
// split flux work should last as long as the upload (dt is known when the last rows have landed), less a
// tenth for the split bands' flux-difference planes; halfway from the current share, within [0.15, 0.85].
double next_split_frac(double cur, double up_ms, double fused_ms, int fused_rows, int ny) {
    if (!(up_ms > 0) || !(fused_ms > 0) || fused_rows <= 0 || ny <= 0) return cur;
    double f = 0.9 * up_ms / (fused_ms / fused_rows * ny);
    f = f < 0.15 ? 0.15 : (f > 0.85 ? 0.85 : f);
    return 0.5 * (cur + f);
}
// One cache per device and thread: the buffers, streams and events are created
// with their device current and used only while it is current.
struct HostCache {
    int device = -1;  // ordinal the resources belong to
    void* base = nullptr;
    size_t bytes = 0;
    static constexpr int kStreams = 3;
    cudaStream_t cs[kStreams] = {nullptr, nullptr, nullptr};  // uploads, downloads, CFL reduction
    // start, dt known, (spare), four joins; per band: landed, head landed, (spare), computed
    cudaEvent_t ev[7 + 4 * kHostBands] = {};
    // timing marks of the split first step (start, uploads done, split updates done, fused bands done) and
    // the share of the rows it splits, adjusted after each call to the host's own copy rate
    cudaEvent_t tev[4] = {};
    double split_frac = kSplitFrac;
    bool streams_ok = false;
    bool ensure_streams() {
        if (streams_ok) return true;
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return false;
        for (int k = 0; k < kStreams; ++k)
            if (cudaStreamCreateWithPriority(&cs[k], cudaStreamNonBlocking, k >= 2 ? greatest : least) != cudaSuccess)
                return false;
        for (auto& e : ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
        for (auto& e : tev)
            if (cudaEventCreate(&e) != cudaSuccess) return false;
        streams_ok = true;
        return true;
    }
    // Frees with the owning device current, then restores the caller's device.
    // At thread or process exit the CUDA runtime may already be shut down;
    // the calls then fail harmlessly and the driver reclaims the memory.
    void release() {
        if (!base && !streams_ok) return;
        int prev = -1;
        const bool switched = device >= 0 && cudaGetDevice(&prev) == cudaSuccess && prev != device &&
                              cudaSetDevice(device) == cudaSuccess;
        if (base) cudaFree(base);
        base = nullptr;
        bytes = 0;
        if (streams_ok) {
            for (auto& e : ev) cudaEventDestroy(e);
            for (auto& e : tev) cudaEventDestroy(e);
            for (auto& c : cs) cudaStreamDestroy(c);
        }
        streams_ok = false;
        if (switched) cudaSetDevice(prev);
    }
    ~HostCache() { release(); }
};
constexpr int kMaxHostDevices = 64;
thread_local HostCache g_host[kMaxHostDevices];

// The calling thread's cache for the current device (null: no usable device).
HostCache* host_cache() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxHostDevices) return nullptr;
    g_host[dev].device = dev;
    return &g_host[dev];
}

// Row bands of the host-buffer run over ny rows: a short first band (the only
// upload the flux work waits for in full) and a short last band (the only
// download not hidden under flux work), each ~1/32 of the rows, and up to
// eight between them.  Band b is rows starts[b] .. starts[b + 1] - 1; starts
// has room for kHostBands + 1 entries.  Returns the number of bands.  Every
// band but the last holds at least kHeadRows rows: a remainder shorter than
// that before the last band joins the band ahead of it.
int host_bands(int ny, int* starts) {
    const int edge = ((ny + 31) / 32 + TY - 1) / TY * TY;
    const int mid = ny - 2 * edge;
    const int m = mid > 0 ? ((mid + 7) / 8 + TY - 1) / TY * TY : TY;  // a multiple of TY, >= TY
    int nb = 0;
    starts[nb++] = 0;
    for (int s = edge; s < ny - edge; s += m) starts[nb++] = s;
    if (ny - edge > starts[nb - 1]) {
        if (ny - edge - starts[nb - 1] >= kHeadRows) starts[nb++] = ny - edge;
        else if (nb > 1) starts[nb - 1] = ny - edge;  // (a first band that short: no split at all)
    }
    starts[nb] = ny;
    return nb;
}

// The band holding row r (rows 0 .. ny - 1).
int band_of(int r, int nb, const int* starts) {
    int b = 0;
    while (b + 1 < nb && starts[b + 1] <= r) ++b;
    return b;
}

}  // namespace

namespace hx {
// Shared with the other C-ABI translation units: launch counting and the
// thread's last error text.
void note_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
int set_error(int code, const char* msg) { return fail(code, "%s", msg); }
// The persistent level kernel's extra expected staging bytes (hx_debug_staging_extra_bytes).
unsigned& staging_test_extra_bytes() {
    static unsigned extra = 0;
    return extra;
}
}  // namespace hx

// ============================================================================
extern "C" {

const char* hx_version(void) { return "hydroexa_gb300 0.1.0 (sm_103a)"; }
const char* hx_last_error(void) { return g_err.c_str(); }
uint64_t hx_launch_count(void) { return g_launches.load(); }

int hx_status_clear(uint32_t* s, hx_stream_t st) {
    if (!s) return fail(HX_ERR_ARG, "null status");
    cudaError_t e = cudaMemsetAsync(s, 0, sizeof(uint32_t), (cudaStream_t)st);
    return e == cudaSuccess ? HX_OK : fail(HX_ERR_CUDA, "status clear: %s", cudaGetErrorString(e));
}

int hx_status_read(const uint32_t* s, hx_stream_t st) {
    if (!s) return fail(HX_ERR_ARG, "null status");
    uint32_t v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, s, sizeof v, cudaMemcpyDeviceToHost, (cudaStream_t)st);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)st);
    if (e != cudaSuccess) return fail(HX_ERR_CUDA, "status read: %s", cudaGetErrorString(e));
    return (int)(v & 0x7fffffffu);
}

int64_t hx_dt_accum_bytes(void) { return (int64_t)sizeof(DtAccum); }

int hx_dt_accum_reset(hx_dt_accum* acc, hx_stream_t st) {
    if (!acc) return fail(HX_ERR_ARG, "null accumulator");
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(DtAccum), (cudaStream_t)st);
    return e == cudaSuccess ? HX_OK : fail(HX_ERR_CUDA, "accumulator reset: %s", cudaGetErrorString(e));
}
int hx_dt_accum_read_f64(const hx_dt_accum* a, double* m, double* v, hx_stream_t st) {
    return accum_read<double>(a, m, v, (cudaStream_t)st);
}
int hx_dt_accum_read_f32(const hx_dt_accum* a, float* m, float* v, hx_stream_t st) {
    return accum_read<float>(a, m, v, (cudaStream_t)st);
}

int hx_advance_box_hydrostatic_f64(const hx_array4_f64* eta, const hx_array4_f64* Ue, const hx_array4_f64* Te,
                                   const hx_array4_f64* Uo, hx_array4_f64* Un, hx_box vb, double dt, double dx,
                                   double dy, const hx_array4_f64* FL, const hx_array4_f64* FR, hx_dt_accum* nd,
                                   uint32_t* status, int arith, hx_stream_t st) {
    return advance_box_hydro<double>(eta, Ue, Te, Uo, Un, vb, dt, dx, dy, FL, FR, nd, status, arith, (cudaStream_t)st);
}
int hx_advance_box_hydrostatic_f32(const hx_array4_f32* eta, const hx_array4_f32* Ue, const hx_array4_f32* Te,
                                   const hx_array4_f32* Uo, hx_array4_f32* Un, hx_box vb, float dt, float dx,
                                   float dy, const hx_array4_f32* FL, const hx_array4_f32* FR, hx_dt_accum* nd,
                                   uint32_t* status, int arith, hx_stream_t st) {
    return advance_box_hydro<float>(eta, Ue, Te, Uo, Un, vb, dt, dx, dy, FL, FR, nd, status, arith, (cudaStream_t)st);
}
int hx_advance_box_hydrostatic_epilogue_f64(const hx_array4_f64* eta, const hx_array4_f64* Ue,
                                            const hx_array4_f64* Te, const hx_array4_f64* Uo, hx_array4_f64* Un,
                                            hx_box vb, double dt, double dx, double dy, hx_dt_accum* nd,
                                            uint32_t* status, int arith, hx_array4_f64* eta_new, double* diag,
                                            void* work, hx_stream_t st) {
    return advance_box_hydro_epi<double>(eta, Ue, Te, Uo, Un, vb, dt, dx, dy, nd, status, arith, eta_new, diag, work,
                                         (cudaStream_t)st);
}
int hx_advance_box_hydrostatic_epilogue_f32(const hx_array4_f32* eta, const hx_array4_f32* Ue,
                                            const hx_array4_f32* Te, const hx_array4_f32* Uo, hx_array4_f32* Un,
                                            hx_box vb, float dt, float dx, float dy, hx_dt_accum* nd,
                                            uint32_t* status, int arith, hx_array4_f32* eta_new, double* diag,
                                            void* work, hx_stream_t st) {
    return advance_box_hydro_epi<float>(eta, Ue, Te, Uo, Un, vb, dt, dx, dy, nd, status, arith, eta_new, diag, work,
                                        (cudaStream_t)st);
}
int hx_advance_box_roe_f64(const hx_array4_f64* eta, hx_array4_f64* Uo, const hx_array4_f64* T, hx_array4_f64* Un,
                           hx_box vb, double dt, double dx, double dy, const hx_array4_f64* F,
                           const hx_array4_f64* Sm, const hx_array4_f64* Sp, hx_dt_accum* nd, uint32_t* status,
                           int arith, hx_stream_t st) {
    return advance_box_roe<double>(eta, Uo, T, Un, vb, dt, dx, dy, F, Sm, Sp, nd, status, arith, (cudaStream_t)st);
}
int hx_advance_box_roe_f32(const hx_array4_f32* eta, hx_array4_f32* Uo, const hx_array4_f32* T, hx_array4_f32* Un,
                           hx_box vb, float dt, float dx, float dy, const hx_array4_f32* F, const hx_array4_f32* Sm,
                           const hx_array4_f32* Sp, hx_dt_accum* nd, uint32_t* status, int arith, hx_stream_t st) {
    return advance_box_roe<float>(eta, Uo, T, Un, vb, dt, dx, dy, F, Sm, Sp, nd, status, arith, (cudaStream_t)st);
}
int hx_advance_box_hydrostatic_reflux_f64(const hx_array4_f64* eta, const hx_array4_f64* Ue,
                                          const hx_array4_f64* Te, const hx_array4_f64* Uo, hx_array4_f64* Un,
                                          hx_box vb, double dt, double dx, double dy, const hx_array4_f64* Freg,
                                          hx_dt_accum* nd, uint32_t* status, int arith, hx_stream_t st) {
    if (!Freg) return fail(HX_ERR_ARG, "hx_advance_box_hydrostatic_reflux: null Freg");
    return advance_box_hydro<double, hx_array4_f64>(eta, Ue, Te, Uo, Un, vb, dt, dx, dy, nullptr, nullptr, nd, status,
                                                    arith, (cudaStream_t)st, Freg);
}
int hx_advance_box_hydrostatic_reflux_f32(const hx_array4_f32* eta, const hx_array4_f32* Ue,
                                          const hx_array4_f32* Te, const hx_array4_f32* Uo, hx_array4_f32* Un,
                                          hx_box vb, float dt, float dx, float dy, const hx_array4_f32* Freg,
                                          hx_dt_accum* nd, uint32_t* status, int arith, hx_stream_t st) {
    if (!Freg) return fail(HX_ERR_ARG, "hx_advance_box_hydrostatic_reflux: null Freg");
    return advance_box_hydro<float, hx_array4_f32>(eta, Ue, Te, Uo, Un, vb, dt, dx, dy, nullptr, nullptr, nd, status,
                                                   arith, (cudaStream_t)st, Freg);
}
int hx_advance_box_roe_reflux_f64(const hx_array4_f64* eta, hx_array4_f64* Uo, const hx_array4_f64* T,
                                  hx_array4_f64* Un, hx_box vb, double dt, double dx, double dy,
                                  const hx_array4_i32* fine_mask, hx_box grid_box, const hx_array4_f64* flux_crse,
                                  const hx_array4_f64* flux_fine, hx_dt_accum* nd, uint32_t* status, int arith,
                                  hx_stream_t st) {
    if (!flux_crse && !flux_fine) return fail(HX_ERR_ARG, "hx_advance_box_roe_reflux: no register output");
    return advance_box_roe<double, hx_array4_f64>(eta, Uo, T, Un, vb, dt, dx, dy, nullptr, nullptr, nullptr, nd, status,
                                                  arith, (cudaStream_t)st, fine_mask, &grid_box, flux_crse, flux_fine);
}
int hx_advance_box_roe_reflux_f32(const hx_array4_f32* eta, hx_array4_f32* Uo, const hx_array4_f32* T,
                                  hx_array4_f32* Un, hx_box vb, float dt, float dx, float dy,
                                  const hx_array4_i32* fine_mask, hx_box grid_box, const hx_array4_f32* flux_crse,
                                  const hx_array4_f32* flux_fine, hx_dt_accum* nd, uint32_t* status, int arith,
                                  hx_stream_t st) {
    if (!flux_crse && !flux_fine) return fail(HX_ERR_ARG, "hx_advance_box_roe_reflux: no register output");
    return advance_box_roe<float, hx_array4_f32>(eta, Uo, T, Un, vb, dt, dx, dy, nullptr, nullptr, nullptr, nd, status,
                                                 arith, (cudaStream_t)st, fine_mask, &grid_box, flux_crse, flux_fine);
}
int hx_dt_reduce_box_f64(const hx_array4_f64* U, const hx_array4_f64* T, hx_box vb, double dx, double dy,
                         hx_dt_accum* acc, hx_stream_t st) {
    return dt_reduce_box<double>(U, T, vb, dx, dy, acc, (cudaStream_t)st);
}
int hx_dt_reduce_box_f32(const hx_array4_f32* U, const hx_array4_f32* T, hx_box vb, float dx, float dy,
                         hx_dt_accum* acc, hx_stream_t st) {
    return dt_reduce_box<float>(U, T, vb, dx, dy, acc, (cudaStream_t)st);
}
int hx_tag_box_f64(int method, const hx_array4_f64* U, const hx_array4_f64* T, hx_array4_i8* tags, hx_box vb,
                   double dx, double dy, double time, double h, double u, double z, signed char sv, hx_stream_t st) {
    return tag_box<double>(method, U, T, tags, vb, dx, dy, time, h, u, z, sv, (cudaStream_t)st);
}
int hx_tag_box_f32(int method, const hx_array4_f32* U, const hx_array4_f32* T, hx_array4_i8* tags, hx_box vb,
                   float dx, float dy, float time, float h, float u, float z, signed char sv, hx_stream_t st) {
    return tag_box<float>(method, U, T, tags, vb, dx, dy, time, h, u, z, sv, (cudaStream_t)st);
}
int hx_masked_average_down_box_f64(const hx_array4_f64* fine, hx_array4_f64* crse, hx_box cb, int scomp, int ccomp,
                                   int ncomp, int rx, int ry, double fv, double nodata, hx_stream_t st) {
    return mavg_box<double>(fine, crse, cb, scomp, ccomp, ncomp, rx, ry, fv, nodata, (cudaStream_t)st);
}
int hx_masked_average_down_box_f32(const hx_array4_f32* fine, hx_array4_f32* crse, hx_box cb, int scomp, int ccomp,
                                   int ncomp, int rx, int ry, float fv, float nodata, hx_stream_t st) {
    return mavg_box<float>(fine, crse, cb, scomp, ccomp, ncomp, rx, ry, fv, nodata, (cudaStream_t)st);
}

int hx_average_down_box_f64(const hx_array4_f64* fine, hx_array4_f64* crse, hx_box cb, int scomp, int ccomp,
                            int ncomp, int rx, int ry, hx_stream_t st) {
    return avgdown_box<double>(fine, crse, cb, scomp, ccomp, ncomp, rx, ry, (cudaStream_t)st);
}
int hx_average_down_box_f32(const hx_array4_f32* fine, hx_array4_f32* crse, hx_box cb, int scomp, int ccomp,
                            int ncomp, int rx, int ry, hx_stream_t st) {
    return avgdown_box<float>(fine, crse, cb, scomp, ccomp, ncomp, rx, ry, (cudaStream_t)st);
}

int hx_derive_eta_box_f64(const hx_array4_f64* U, const hx_array4_f64* T, hx_array4_f64* eta, hx_box b,
                          hx_stream_t st) {
    return eta_box<double>(U, T, eta, b, (cudaStream_t)st);
}
int hx_derive_eta_box_f32(const hx_array4_f32* U, const hx_array4_f32* T, hx_array4_f32* eta, hx_box b,
                          hx_stream_t st) {
    return eta_box<float>(U, T, eta, b, (cudaStream_t)st);
}
int64_t hx_diagnostics_work_bytes(hx_box b) {
    if (b.hi[0] < b.lo[0] || b.hi[1] < b.lo[1]) return 0;
    return 5 * (int64_t)sizeof(double) * diag_blocks(b);
}
int hx_diagnostics_box_f64(const hx_array4_f64* U, const hx_array4_f64* T, hx_box b, double dx, double dy,
                           double* out, void* work, hx_stream_t st) {
    return diag_box<double>(U, T, b, dx, dy, out, work, (cudaStream_t)st);
}
int hx_diagnostics_box_f32(const hx_array4_f32* U, const hx_array4_f32* T, hx_box b, float dx, float dy,
                           double* out, void* work, hx_stream_t st) {
    return diag_box<float>(U, T, b, dx, dy, out, work, (cudaStream_t)st);
}
int hx_level_diagnostics_f64(const hx_level_f64* L, double* out, void* work, hx_stream_t st) {
    if (!level_ok(L)) return HX_ERR_ARG;
    if (!out || !work) return fail(HX_ERR_ARG, "hx_level_diagnostics: null output or work");
    const IBox b{0, 0, L->nx - 1, L->ny - 1};
    auto pl = [&](const double* p) { return Plane<double>{p, L->pitch, 0, 0}; };
    return launched(launch_diagnostics<double>(pl(L->h), pl(L->hu), pl(L->hv), pl(L->n), b, L->dx * L->dy,
                                               static_cast<double*>(work), out, (cudaStream_t)st),
                    "hx_level_diagnostics_f64");
}

int hx_level_advance_f64(int method, const hx_level_f64* L, double dt, double* ho, double* huo, double* hvo,
                         hx_dt_accum* nd, uint32_t* status, int arith, hx_stream_t st) {
    if (!level_ok(L)) return HX_ERR_ARG;
    if (!ho || !huo || !hvo) return fail(HX_ERR_ARG, "null output planes");
    if (method != HX_METHOD_ROE && method != HX_METHOD_HYDROSTATIC_ROE) return fail(HX_ERR_ARG, "unknown method");
    return level_advance<double>(method, L, host_ctl<double>(dt, L->dx, L->dy, nd, status), ho, huo, hvo, arith,
                                 (cudaStream_t)st);
}
int hx_level_advance_f32(int method, const hx_level_f32* L, float dt, float* ho, float* huo, float* hvo,
                         hx_dt_accum* nd, uint32_t* status, int arith, hx_stream_t st) {
    if (!level_ok(L)) return HX_ERR_ARG;
    if (!ho || !huo || !hvo) return fail(HX_ERR_ARG, "null output planes");
    if (method != HX_METHOD_ROE && method != HX_METHOD_HYDROSTATIC_ROE) return fail(HX_ERR_ARG, "unknown method");
    return level_advance<float>(method, L, host_ctl<float>(dt, L->dx, L->dy, nd, status), ho, huo, hvo, arith,
                                (cudaStream_t)st);
}
int hx_level_advance_epilogue_f64(const hx_level_f64* L, double dt, double* ho, double* huo, double* hvo,
                                  hx_dt_accum* nd, uint32_t* status, int arith, double* eta_out, double* diag,
                                  void* work, hx_stream_t st) {
    return level_advance_epi<double>(L, dt, ho, huo, hvo, nd, status, arith, eta_out, diag, work, (cudaStream_t)st);
}
int hx_level_advance_epilogue_f32(const hx_level_f32* L, float dt, float* ho, float* huo, float* hvo,
                                  hx_dt_accum* nd, uint32_t* status, int arith, float* eta_out, double* diag,
                                  void* work, hx_stream_t st) {
    return level_advance_epi<float>(L, dt, ho, huo, hvo, nd, status, arith, eta_out, diag, work, (cudaStream_t)st);
}
int hx_level_dt_reduce_f64(const hx_level_f64* L, hx_dt_accum* acc, hx_stream_t st) {
    return level_dt<double>(L, acc, (cudaStream_t)st);
}
int hx_level_dt_reduce_f32(const hx_level_f32* L, hx_dt_accum* acc, hx_stream_t st) {
    return level_dt<float>(L, acc, (cudaStream_t)st);
}

int64_t hx_level_run_work_bytes(void) { return kRunWork; }

int hx_level_run_f64(int method, hx_level_f64* L, double* ha, double* hua, double* hva, int nsteps, double cfl,
                     void* work, uint32_t* status, double* time_dev, int arith, int* fin, hx_stream_t st) {
    return level_run<double>(method, L, ha, hua, hva, nsteps, cfl, work, status, time_dev, arith, fin,
                             (cudaStream_t)st);
}
int hx_level_run_f32(int method, hx_level_f32* L, float* ha, float* hua, float* hva, int nsteps, float cfl,
                     void* work, uint32_t* status, float* time_dev, int arith, int* fin, hx_stream_t st) {
    return level_run<float>(method, L, ha, hua, hva, nsteps, cfl, work, status, time_dev, arith, fin,
                            (cudaStream_t)st);
}

int hx_level_run_host_f64(int method, int nx, int ny, double dx, double dy, const int32_t bc_lo[2],
                          const int32_t bc_hi[2], double* h, double* hu, double* hv, const double* z, const double* n,
                          int nsteps, double cfl, int arith, double* time_out, hx_stream_t stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (nx < 2 || ny < 2) return fail(HX_ERR_ARG, "nx, ny must be >= 2");
    if (!h || !hu || !hv || !z || !n || !bc_lo || !bc_hi) return fail(HX_ERR_ARG, "null host buffer");
    if (nsteps < 0) return fail(HX_ERR_ARG, "nsteps < 0");
    if (!(cfl > 0)) return fail(HX_ERR_ARG, "cfl must be positive");
    if (method != HX_METHOD_ROE && method != HX_METHOD_HYDROSTATIC_ROE) return fail(HX_ERR_ARG, "unknown method");
    // the hydrostatic first step is split: flux differences as the rows land, the update once dt is known
    const bool split = method == HX_METHOD_HYDROSTATIC_ROE && nsteps >= 1;
    const size_t N = (size_t)nx * ny, pb = N * sizeof(double);
    const size_t need = (split ? 14 : 8) * pb + 512;
    HostCache* hc = host_cache();
    if (!hc) return fail(HX_ERR_CUDA, "hx_level_run_host_f64: no current CUDA device");
    if (hc->bytes < need) {
        if (hc->base) cudaFree(hc->base);
        hc->base = nullptr;
        hc->bytes = 0;
        cudaError_t e = cudaMalloc(&hc->base, need);
        if (e != cudaSuccess) return fail(HX_ERR_CUDA, "device buffers: %s", cudaGetErrorString(e));
        hc->bytes = need;
    }
    if (!hc->ensure_streams()) return fail(HX_ERR_CUDA, "copy streams could not be created");
    cudaStream_t* cs = hc->cs;
    cudaEvent_t* ev = hc->ev;
    // an error after work was queued returns once the queued copies have finished with the caller's buffers
    auto drain = [&](int r) -> int {
        for (int k = 0; k < HostCache::kStreams; ++k) cudaStreamSynchronize(cs[k]);
        cudaStreamSynchronize(st);
        return r;
    };
    double* d = (double*)hc->base;
    double* P[14];
    for (int k = 0; k < 14; ++k) P[k] = d + k * N;
    char* tail = (char*)(d + (split ? 14 : 8) * N);
    uint32_t* status = (uint32_t*)tail;
    double* tdev = (double*)(tail + 64);
    DtAccum* slot = reinterpret_cast<DtAccum*>(tail + 128);
    const double* src[5] = {h, hu, hv, z, n};
    hx_level_f64 L{P[0], P[1], P[2], P[3], P[4], (int64_t)nx, nx, ny, dx, dy, {bc_lo[0], bc_lo[1]}, {bc_hi[0], bc_hi[1]}};
    const bool fast = arith != HX_ARITH_EXACT;
    DivOut<double> div{{P[8], P[9], P[10], P[11], P[12], P[13]}, (long long)nx, 0, 0};
    Cells3<double> uo;
    uo.p[0] = P[0]; uo.p[1] = P[1]; uo.p[2] = P[2];
    uo.js = nx; uo.lo0 = 0; uo.lo1 = 0;
    const Plane<double> np{P[4], (long long)nx, 0, 0}, zp{P[3], (long long)nx, 0, 0};
    int starts[kHostBands + 1];
    const int nbands = host_bands(ny, starts);
    auto rows = [&](int b, int& j0, int& j1) { j0 = starts[b]; j1 = starts[b + 1] - 1; };
    auto flux_band = [&](int b) -> int {  // flux differences of band b (rows to the head of b+1 have landed)
        int j0, j1;
        rows(b, j0, j1);
        const LevelSrc<double> lsrc = level_src<double>(&L, 2);
        const IBox vb{0, j0, nx - 1, j1};
        return launched(fast ? launch_hydro_split<double, true>(lsrc, uo, np, div, vb, dx, dy, st)
                             : launch_hydro_split<double, false>(lsrc, uo, np, div, vb, dx, dy, st),
                        "hx_level_run_host_f64 (flux differences)");
    };
    // Upload in row bands (stream up), after the caller's earlier work; from the second band on, a band's
    // first kHeadRows rows go up ahead of the rest.  The CFL reduction of each band runs as soon as its rows
    // have landed.  Split: the reduction on its own high-priority stream (dts), while st runs each split
    // band's flux differences once the head of the band after it has landed, then (dt known) the split
    // bands' updates and the later bands' fused steps; each band's rows go down (stream down) as soon as
    // they are final, under the rest of the step.
    cudaStream_t up = cs[0], down = cs[1], dts = cs[2];
    cudaEvent_t ev_start = ev[0], ev_dt = ev[1];
    cudaEvent_t* ev_join = ev + 3;
    cudaEvent_t* ev_up = ev + 7;
    cudaEvent_t* ev_head = ev + 7 + kHostBands;
    cudaEvent_t* ev_k = ev + 7 + 3 * kHostBands;
    cudaError_t e = cudaMemsetAsync(tail, 0, 128 + 3 * sizeof(DtAccum), st);
    if (e == cudaSuccess) e = cudaEventRecord(ev_start, st);
    if (e == cudaSuccess && split) e = cudaEventRecord(hc->tev[0], st);
    for (int k = 0; k < HostCache::kStreams && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(cs[k], ev_start, 0);
    int rc = HX_OK;
    cudaStream_t dstream = split ? dts : st;
    auto upload = [&](int r0, int r1) -> cudaError_t {  // rows r0..r1 of the five planes
        cudaError_t r = cudaSuccess;
        for (int k = 0; k < 5 && r == cudaSuccess; ++k)
            r = cudaMemcpyAsync(P[k] + (size_t)r0 * nx, src[k] + (size_t)r0 * nx,
                                (size_t)(r1 - r0 + 1) * nx * sizeof(double), cudaMemcpyHostToDevice, up);
        return r;
    };
    for (int b = 0; b < nbands && e == cudaSuccess && rc == HX_OK; ++b) {
        int j0, j1;
        rows(b, j0, j1);
        int jr = j0;  // the rows after the head
        if (b > 0) {
            jr = j0 + kHeadRows <= j1 ? j0 + kHeadRows : j1 + 1;
            e = upload(j0, jr - 1);
            if (e == cudaSuccess) e = cudaEventRecord(ev_head[b], up);
        }
        if (e == cudaSuccess && jr <= j1) e = upload(jr, j1);
        if (e == cudaSuccess) e = cudaEventRecord(ev_up[b], up);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(dstream, ev_up[b], 0);
        if (e == cudaSuccess)
            rc = level_dt<double>(&L, reinterpret_cast<hx_dt_accum*>(&slot[0]), dstream, arith, j0, j1);
    }
    if (e == cudaSuccess && split) e = cudaEventRecord(ev_dt, dts);
    if (e == cudaSuccess && split) e = cudaEventRecord(hc->tev[1], up);
    if (e != cudaSuccess) return drain(fail(HX_ERR_CUDA, "upload: %s", cudaGetErrorString(e)));
    if (rc) return drain(rc);
    const double* A[3] = {P[0], P[1], P[2]};
    double* B[3] = {P[5], P[6], P[7]};
    hx_level_f64 cur = L;
    const double* res[3] = {P[0], P[1], P[2]};
    double* dst[3] = {h, hu, hv};
    // step s's controls; b > 0 leaves the clock and the slot reset to band 0
    auto step_ctl = [&](int s, int b) {
        StepCtl<double> c;
        c.dt_host = 0.0; c.cfl = cfl;
        c.dt_in = &slot[s % 3]; c.dt_out = s + 1 < nsteps ? &slot[(s + 1) % 3] : nullptr;
        c.dt_reset = b ? nullptr : &slot[(s + 2) % 3];
        c.status = status; c.time = b ? nullptr : tdev; c.dx = dx; c.dy = dy;
        return c;
    };
    // band b's rows of o, after the work queued so far on stream after
    auto download = [&](int b, double* const* o, cudaStream_t after) -> cudaError_t {
        int j0, j1;
        rows(b, j0, j1);
        cudaError_t r = cudaEventRecord(ev_k[b], after);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(down, ev_k[b], 0);
        for (int k = 0; k < 3 && r == cudaSuccess; ++k)
            r = cudaMemcpyAsync(dst[k] + (size_t)j0 * nx, o[k] + (size_t)j0 * nx,
                                (size_t)(j1 - j0 + 1) * nx * sizeof(double), cudaMemcpyDeviceToHost, down);
        return r;
    };
    int s0 = 0, split_rows = 0;  // split_rows: the rows of the fused bands of the split step
    if (split) {
        double* o[3] = {B[0], B[1], B[2]};
        Cells3W<double> ow;
        ow.p[0] = o[0]; ow.p[1] = o[1]; ow.p[2] = o[2];
        ow.js = nx; ow.lo0 = 0; ow.lo1 = 0;
        // The bands ahead of kf are split: their flux differences run as their rows land.  kf is the first
        // band starting past the split share of the rows (kSplitFrac until a call has measured this host,
        // then next_split_frac), so that dt -- whose reduction runs on its own stream as the rows land, in
        // the gaps between the flux kernels -- is known when that work ends.  Then, on the caller's stream,
        // the split bands' updates (short: their rows start going down at once, under the rest of the step)
        // and the later bands through the fused kernel in one pass, without the flux-difference planes and
        // the separate update (the same arithmetic, so the share changes the timing only).
        int kf = nbands;
        for (int b = 1; b < nbands; ++b)
            if ((double)starts[b] >= hc->split_frac * ny) {
                kf = b;
                break;
            }
        for (int b = 0; b < kf && rc == HX_OK && e == cudaSuccess; ++b) {
            // the flux differences of band b read rows up to kHeadRows past its last row: wait for the upload
            // event that covers the last of them (the head of the band holding it, or that whole band; rows
            // go up in order on one stream, so every earlier row has landed too)
            int j0, j1;
            rows(b, j0, j1);
            const int r = j1 + kHeadRows < ny ? j1 + kHeadRows : ny - 1;
            const int c = band_of(r, nbands, starts);
            e = cudaStreamWaitEvent(st, (c > b && r < starts[c] + kHeadRows) ? ev_head[c] : ev_up[c], 0);
            if (e == cudaSuccess) rc = flux_band(b);
        }
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_dt, 0);  // dt of the whole level
        for (int b = 0; b < kf && rc == HX_OK && e == cudaSuccess; ++b) {
            int j0, j1;
            rows(b, j0, j1);
            const IBox vb{0, j0, nx - 1, j1};
            rc = launched(fast ? launch_hydro_update<double, true>(uo, div, np, zp, ow, vb, step_ctl(0, b), st)
                               : launch_hydro_update<double, false>(uo, div, np, zp, ow, vb, step_ctl(0, b), st),
                          "hx_level_run_host_f64 (update)");
            if (rc == HX_OK && nsteps == 1) e = download(b, o, st);
        }
        if (e == cudaSuccess && rc == HX_OK) e = cudaEventRecord(hc->tev[2], st);
        for (int b = kf; b < nbands && rc == HX_OK && e == cudaSuccess; ++b) {
            int j0, j1;
            rows(b, j0, j1);
            rc = level_advance<double>(method, &L, step_ctl(0, b), o[0], o[1], o[2], arith, st, j0, j1);
            if (rc == HX_OK && nsteps == 1) e = download(b, o, st);
        }
        if (e == cudaSuccess && rc == HX_OK) e = cudaEventRecord(hc->tev[3], st);
        if (e != cudaSuccess) return drain(fail(HX_ERR_CUDA, "split step: %s", cudaGetErrorString(e)));
        if (rc) return drain(rc);
        res[0] = o[0]; res[1] = o[1]; res[2] = o[2];
        s0 = 1;
        split_rows = kf < nbands ? ny - starts[kf] : 0;
    }
    // the other steps; the last one in row bands, each band's rows going down while the next computes
    for (int s = s0; s < nsteps; ++s) {
        const bool even = (s % 2) == 0;
        cur.h = even ? A[0] : B[0];
        cur.hu = even ? A[1] : B[1];
        cur.hv = even ? A[2] : B[2];
        double* o[3] = {even ? B[0] : const_cast<double*>(A[0]), even ? B[1] : const_cast<double*>(A[1]),
                        even ? B[2] : const_cast<double*>(A[2])};
        res[0] = o[0]; res[1] = o[1]; res[2] = o[2];
        const bool last = s == nsteps - 1;
        for (int b = 0; b < (last ? nbands : 1); ++b) {
            int j0 = 0, j1 = ny - 1;
            if (last) rows(b, j0, j1);
            rc = level_advance<double>(method, &cur, step_ctl(s, b), o[0], o[1], o[2], arith, st, j0, j1);
            if (rc) return drain(rc);
            if (!last) continue;
            e = download(b, o, st);
            if (e != cudaSuccess) return drain(fail(HX_ERR_CUDA, "download: %s", cudaGetErrorString(e)));
        }
    }
    if (nsteps == 0) {
        e = cudaEventRecord(ev_k[0], st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(down, ev_k[0], 0);
        for (int k = 0; k < 3 && e == cudaSuccess; ++k)
            e = cudaMemcpyAsync(dst[k], res[k], pb, cudaMemcpyDeviceToHost, down);
    }
    for (int k = 0; k < HostCache::kStreams && e == cudaSuccess; ++k) e = cudaEventRecord(ev_join[k], cs[k]);
    for (int k = 0; k < HostCache::kStreams && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(st, ev_join[k], 0);
    uint32_t sv = 0;
    double tv = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&sv, status, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tv, tdev, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return drain(fail(HX_ERR_CUDA, "download: %s", cudaGetErrorString(e)));
    if (split && split_rows > 0) {  // the marks are complete: st has joined every stream
        float up_ms = 0.f, fused_ms = 0.f;
        if (cudaEventElapsedTime(&up_ms, hc->tev[0], hc->tev[1]) == cudaSuccess &&
            cudaEventElapsedTime(&fused_ms, hc->tev[2], hc->tev[3]) == cudaSuccess)
            hc->split_frac = next_split_frac(hc->split_frac, up_ms, fused_ms, split_rows, ny);
        else
            cudaGetLastError();  // a mark that was not recorded: keep the share, clear the error
    }
    if (time_out) *time_out = tv;
    return (int)sv;
}

void hx_host_cache_release(void) {
    for (auto& c : g_host) c.release();
}

double hx_debug_host_split_frac(void) {
    HostCache* hc = host_cache();
    return hc ? hc->split_frac : -1.0;
}

int hx_debug_host_bands(int ny, int* starts, int max_bands) {
    if (ny < 2) return fail(HX_ERR_ARG, "ny must be >= 2");
    if (!starts || max_bands < kHostBands) return fail(HX_ERR_ARG, "starts needs room for %d bands", kHostBands);
    return host_bands(ny, starts);
}

int hx_level_tangent_f64(const hx_level_f64* L, double dt, double ddt, double* oh, double* ohu, double* ohv,
                         hx_stream_t s) {
    if (!level_ok(L)) return HX_ERR_ARG;
    if (!oh || !ohu || !ohv) return fail(HX_ERR_ARG, "hx_level_tangent_f64: null output planes");
    LevelSrc<Dual> src;
    src.h = reinterpret_cast<const Dual*>(L->h);
    src.hu = reinterpret_cast<const Dual*>(L->hu);
    src.hv = reinterpret_cast<const Dual*>(L->hv);
    src.z = reinterpret_cast<const Dual*>(L->z);
    src.n = reinterpret_cast<const Dual*>(L->n);
    src.pitch = L->pitch;
    src.nx = L->nx; src.ny = L->ny;
    src.bc_xlo = L->bc_lo[0]; src.bc_ylo = L->bc_lo[1]; src.bc_xhi = L->bc_hi[0]; src.bc_yhi = L->bc_hi[1];
    src.glo0 = -2; src.glo1 = -2; src.ghi0 = L->nx + 1; src.ghi1 = L->ny + 1;
    Cells3<Dual> uo;
    uo.p[0] = src.h; uo.p[1] = src.hu; uo.p[2] = src.hv;
    uo.js = L->pitch; uo.lo0 = 0; uo.lo1 = 0;
    Plane<Dual> np{src.n, L->pitch, 0, 0};
    Cells3W<Dual> out;
    out.p[0] = reinterpret_cast<Dual*>(oh);
    out.p[1] = reinterpret_cast<Dual*>(ohu);
    out.p[2] = reinterpret_cast<Dual*>(ohv);
    out.js = L->pitch; out.lo0 = 0; out.lo1 = 0;
    const IBox vb{0, 0, L->nx - 1, L->ny - 1};
    return launched(launch_tangent(src, uo, np, out, vb, Dual(dt, ddt), L->dx, L->dy, (cudaStream_t)s),
                    "hx_level_tangent_f64");
}

int hx_debug_roe_points_f64(int method, int arith, long n, const double* st, const double* aux, double* out,
                            hx_stream_t s) {
    if (n < 0 || (n > 0 && (!st || !aux || !out))) return fail(HX_ERR_ARG, "bad point arrays");
    cudaError_t e = arith == HX_ARITH_EXACT ? launch_points<double, false>(method, n, st, aux, out, (cudaStream_t)s)
                                            : launch_points<double, true>(method, n, st, aux, out, (cudaStream_t)s);
    return launched(e, "hx_debug_roe_points");
}
int hx_debug_roe_points_f32(int method, int arith, long n, const float* st, const float* aux, float* out,
                            hx_stream_t s) {
    if (n < 0 || (n > 0 && (!st || !aux || !out))) return fail(HX_ERR_ARG, "bad point arrays");
    cudaError_t e = arith == HX_ARITH_EXACT ? launch_points<float, false>(method, n, st, aux, out, (cudaStream_t)s)
                                            : launch_points<float, true>(method, n, st, aux, out, (cudaStream_t)s);
    return launched(e, "hx_debug_roe_points");
}

int hx_debug_rcp_f64(long n, const double* x, double* y, hx_stream_t s) {
    if (n < 0 || (n > 0 && (!x || !y))) return fail(HX_ERR_ARG, "bad reciprocal arrays");
    return launched(launch_rcp<true>(n, x, y, 0, (cudaStream_t)s), "hx_debug_rcp_f64");
}

int hx_debug_sqrt_f64(long n, const double* x, double* y, hx_stream_t s) {
    if (n < 0 || (n > 0 && (!x || !y))) return fail(HX_ERR_ARG, "bad square-root arrays");
    return launched(launch_rcp<true>(n, x, y, 1, (cudaStream_t)s), "hx_debug_sqrt_f64");
}

int hx_debug_staging_extra_bytes(unsigned bytes) {
    const unsigned old = staging_test_extra_bytes();
    staging_test_extra_bytes() = bytes;
    return (int)old;
}

int hx_debug_fast_op_f64(int op, long n, const double* x, double* y, hx_stream_t s) {
    if (op < HX_FAST_OP_RCP || op > HX_FAST_OP_RCBRT) return fail(HX_ERR_ARG, "unknown fast-form operation");
    if (n < 0 || (n > 0 && (!x || !y))) return fail(HX_ERR_ARG, "bad operand arrays");
    return launched(launch_rcp<true>(n, x, y, op, (cudaStream_t)s), "hx_debug_fast_op_f64");
}

}  // extern "C"
