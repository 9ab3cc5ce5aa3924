// A single-level, single-box driver around the reference's own solver code,
// compiled verbatim from the reference tree with the host-only AMReX stand-in
// in ref_shim/: SolverVariant (include/solvers/SolverVariant.H), the two
// solvers (src/solvers/HydrostaticRoe.cpp, src/solvers/Roe.cpp, compiled as
// their own translation units) and the physical-boundary filler HydroPhysBC
// (include/boundaries/BCFill.H).  TEST INFRASTRUCTURE: built into oracle/_ref/
// by oracle/build_ref.sh, used to pin the oracle and to write tests/golden.
//
// What this file restates from the reference's AMR driver, at one level:
//  - the state and its BC records: U (3 comps), Eta (1), terrain (2), one ghost
//    each (AmrMeshState_Init.cpp:23-26); U_bcs = scalar, x-velocity,
//    y-velocity; Eta_bcs = scalar; terrain always extrapolated (:41-71);
//  - ComputeDt -> solver.compute_dt on U_new (AmrMeshState_Physics.cpp:13-19);
//  - the step: t_old = t_new, t_new += dt, compute_fluxes(ctx, 0, dt, t_old),
//    then Eta = h + z of U_new on the grown box (Physics.cpp:100-108, :153-172,
//    AmrMeshState_AMR.cpp:197-224);
//  - the three FillPatch services at level 0 (AmrMeshState_AMR.cpp:667-775 with
//    include/utils/FillPatchUtils.H): FillPatchSingleLevel copies the source's
//    valid cells into the destination (or exchanges ghosts when the source is
//    the destination: nothing to exchange on one box) and then calls the
//    physical-boundary functor as physbc(mf, dcomp, ncomp, mf's ghosts, time,
//    0) -- the BC-record offset is 0, as FillPatchFrom passes it.  The sources
//    are U_old (time = t_old), Eta derived from U_old on the grown box, and the
//    terrain.
#include <solvers/SolverVariant.H>
#include <boundaries/BCFill.H>

#include <cstring>

#include "ref_names.h"

namespace {

using amrex::Real;

struct OneLevel {
    int nx, ny;
    amrex::Box dom;
    amrex::Vector<amrex::Geometry> geom;
    amrex::Vector<amrex::BoxArray> grids;
    amrex::Vector<amrex::DistributionMapping> dmap;
    amrex::Vector<amrex::MultiFab> U_new, U_old, Eta, Terrain, EtaScratch;
    amrex::Vector<amrex::BCRec> U_bcs, Eta_bcs, Terrain_bcs;
    HydroPhysBC U_physbc, Eta_physbc, Terrain_physbc;
    amrex::Vector<std::unique_ptr<amrex::FluxRegister>> regs;
    amrex::Vector<Real> t_new{Real(0)}, t_old{Real(0)};
    SolverVariant solver;

    OneLevel(int method, int nx_, int ny_, Real dx, Real dy, const int* lo, const int* hi)
        : nx(nx_), ny(ny_), dom(amrex::IntVect(0, 0), amrex::IntVect(nx_ - 1, ny_ - 1)) {
        geom.emplace_back(dom, dx, dy);
        grids.emplace_back(dom);
        dmap.resize(1);
        U_new.resize(1); U_old.resize(1); Eta.resize(1); Terrain.resize(1); EtaScratch.resize(1);
        U_new[0].define(grids[0], dmap[0], 3, 1);
        U_old[0].define(grids[0], dmap[0], 3, 1);
        Eta[0].define(grids[0], dmap[0], 1, 1);
        EtaScratch[0].define(grids[0], dmap[0], 1, 1);
        Terrain[0].define(grids[0], dmap[0], 2, 1);
        BCParams bp;
        bp.lo_bc[0] = lo[0]; bp.lo_bc[1] = lo[1];
        bp.hi_bc[0] = hi[0]; bp.hi_bc[1] = hi[1];
        U_bcs.resize(3); Eta_bcs.resize(1); Terrain_bcs.resize(2);
        SetScalarBC(U_bcs[0], bp);
        SetXVelocityBC(U_bcs[1], bp);
        SetYVelocityBC(U_bcs[2], bp);
        SetScalarBC(Eta_bcs[0], bp);
        BCParams tp;
        for (int k = 0; k < AMREX_SPACEDIM; ++k) { tp.lo_bc[k] = 1; tp.hi_bc[k] = 1; }
        SetScalarBC(Terrain_bcs[0], tp);
        SetScalarBC(Terrain_bcs[1], tp);
        U_physbc.define(geom[0], U_bcs);
        Eta_physbc.define(geom[0], Eta_bcs);
        Terrain_physbc.define(geom[0], Terrain_bcs);
        regs.resize(1);
        if (method == 1) solver = SolverVariant(HydrostaticRoe{});
        else solver = SolverVariant(Roe{});
        solver.resize_flux_buffers(1);
    }

    // valid cells of comp c of mf <- plane (x fastest, pitch nx)
    void put(amrex::MultiFab& mf, int c, const Real* plane) {
        auto a = mf[0].array();
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) a(i, j, 0, c) = plane[i + (size_t)j * nx];
    }
    void get(const amrex::MultiFab& mf, int c, Real* plane) const {
        auto a = mf[0].const_array();
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) plane[i + (size_t)j * nx] = a(i, j, 0, c);
    }
    void load(const Real* h, const Real* hu, const Real* hv, const Real* z, const Real* n) {
        for (auto* U : {&U_new[0], &U_old[0]}) {
            U->setVal(Real(0));
            put(*U, 0, h); put(*U, 1, hu); put(*U, 2, hv);
        }
        Terrain[0].setVal(Real(0));
        put(Terrain[0], 0, z); put(Terrain[0], 1, n);
        // the terrain's ghost ring as the level creation leaves it (extrapolated)
        Terrain_physbc(Terrain[0], 0, 2, Terrain[0].nGrowVect(), Real(0), 0);
        derive_eta(U_new[0], Eta[0]);
    }
    // DeriveEtaFrom: eta = h + z on the grown box (AmrMeshState_AMR.cpp:203-224)
    void derive_eta(const amrex::MultiFab& U, amrex::MultiFab& dst) {
        for (amrex::MFIter mfi(dst); mfi.isValid(); ++mfi) {
            auto u = U.const_array(mfi);
            auto z = Terrain[0].const_array(mfi);
            auto e = dst.array(mfi);
            amrex::ParallelFor(mfi.growntilebox(), [=](int i, int j, int k) { e(i, j, k, 0) = u(i, j, k, 0) + z(i, j, k, 0); });
        }
    }
    // FillPatchSingleLevel at level 0 from one source at the fill time
    static void fill_single(amrex::MultiFab& mf, const amrex::MultiFab& src, int comp, int ncomp, HydroPhysBC& physbc,
                            Real time) {
        if (&mf != &src) {
            for (amrex::MFIter mfi(mf); mfi.isValid(); ++mfi) {
                auto d = mf.array(mfi);
                auto s = src.const_array(mfi);
                for (int c = comp; c < comp + ncomp; ++c)
                    amrex::ParallelFor(mfi.validbox(), [=](int i, int j, int k) { d(i, j, k, c) = s(i, j, k, c); });
            }
        }
        physbc(mf, comp, ncomp, mf.nGrowVect(), time, 0);
    }

    SolverContext context() {
        return SolverContext{
            U_new, U_old, Eta, Terrain, t_new, t_old, geom, grids, dmap,
            [](int) { return amrex::IntVect(2, 2); },
            U_bcs, Terrain_bcs, Eta_bcs, regs, false, 0,
            [this](int, Real time, amrex::MultiFab& mf, const amrex::Vector<amrex::BCRec>&, int icomp, int ncomp) {
                fill_single(mf, U_old[0], icomp, ncomp, U_physbc, time);
            },
            [this](int, Real time, amrex::MultiFab& mf, const amrex::Vector<amrex::BCRec>&, int icomp, int ncomp) {
                fill_single(mf, Terrain[0], icomp, ncomp, Terrain_physbc, time);
            },
            [this](int, Real time, amrex::MultiFab& mf, const amrex::Vector<amrex::BCRec>&, int icomp, int ncomp) {
                derive_eta(U_old[0], EtaScratch[0]);
                fill_single(mf, EtaScratch[0], icomp, ncomp, Eta_physbc, time);
            },
            [](const amrex::MultiFab& mf, const amrex::BoxArray&, const amrex::IntVect&, int, int) {
                return amrex::iMultiFab(mf.boxArray(), mf.DistributionMap(), 1, 1);
            }};
    }

    Real compute_dt(Real cfl) {
        amrex::Vector<Real> dt(1);
        amrex::Vector<amrex::IntVect> ratio;
        solver.compute_dt(dt, U_new, Terrain, geom, ratio, 0, cfl);
        return dt[0];
    }
    void step(Real dt) {
        t_old[0] = t_new[0];
        t_new[0] += dt;
        solver.compute_fluxes(context(), 0, dt, t_old[0]);
        derive_eta(U_new[0], Eta[0]);
    }
};

}  // namespace

extern "C" {

// The single-level time loop of the reference (HydroEXA::Compute at one level):
// nsteps of ComputeDt + the level advance, the state updated in place.
// Returns 0, or 1 when compute_dt aborts on a collapsed dt (the state is then
// the last one reached), or 2 on any other error (message in err, 256 bytes).
int HXREF_NAME(hxref_level_run)(int method, int nx, int ny, Real dx, Real dy, const int* lo, const int* hi, Real* h,
                                Real* hu, Real* hv, const Real* z, const Real* n, int nsteps, Real cfl, Real* t_out,
                                Real* dt_last, char* err) {
    try {
        OneLevel L(method, nx, ny, dx, dy, lo, hi);
        L.load(h, hu, hv, z, n);
        Real dt = 0;
        int rc = 0;
        for (int s = 0; s < nsteps; ++s) {
            try {
                dt = L.compute_dt(cfl);
            } catch (const std::runtime_error& e) {
                if (std::strstr(e.what(), "dt collapsed")) { rc = 1; break; }
                throw;
            }
            L.step(dt);
        }
        L.get(L.U_new[0], 0, h); L.get(L.U_new[0], 1, hu); L.get(L.U_new[0], 2, hv);
        if (t_out) *t_out = L.t_new[0];
        if (dt_last) *dt_last = dt;
        return rc;
    } catch (const std::exception& e) {
        if (err) { std::strncpy(err, e.what(), 255); err[255] = 0; }
        return 2;
    }
}

// One level advance by a given dt: out = the state after compute_fluxes.
int HXREF_NAME(hxref_level_advance)(int method, int nx, int ny, Real dx, Real dy, const int* lo, const int* hi,
                                    const Real* h, const Real* hu, const Real* hv, const Real* z, const Real* n,
                                    Real dt, Real* oh, Real* ohu, Real* ohv, char* err) {
    try {
        OneLevel L(method, nx, ny, dx, dy, lo, hi);
        L.load(h, hu, hv, z, n);
        L.step(dt);
        L.get(L.U_new[0], 0, oh); L.get(L.U_new[0], 1, ohu); L.get(L.U_new[0], 2, ohv);
        return 0;
    } catch (const std::exception& e) {
        if (err) { std::strncpy(err, e.what(), 255); err[255] = 0; }
        return 2;
    }
}

// compute_dt_level (cfl applied): returns 0, 1 on a collapsed dt, 2 on error.
int HXREF_NAME(hxref_level_dt)(int method, int nx, int ny, Real dx, Real dy, const Real* h, const Real* hu,
                               const Real* hv, const Real* z, Real cfl, Real* dt_out, char* err) {
    const int lo[2] = {0, 0}, hi[2] = {0, 0};
    try {
        OneLevel L(method, nx, ny, dx, dy, lo, hi);
        std::vector<Real> zero((size_t)nx * ny, Real(0));
        L.load(h, hu, hv, z, zero.data());
        *dt_out = L.solver.compute_dt_level(L.U_new, L.Terrain, L.geom, 0, cfl);
        return 0;
    } catch (const std::runtime_error& e) {
        if (std::strstr(e.what(), "dt collapsed")) return 1;
        if (err) { std::strncpy(err, e.what(), 255); err[255] = 0; }
        return 2;
    } catch (const std::exception& e) {
        if (err) { std::strncpy(err, e.what(), 255); err[255] = 0; }
        return 2;
    }
}

// tag_cells at level 0 on a box of nx x ny valid cells whose state and terrain
// are given with one ghost cell (planes of (nx + 2) x (ny + 2), x fastest,
// element (i, j) at (i + 1) + (j + 1) (nx + 2)); tags (nx x ny) are cleared,
// then set to TagBox::SET where the reference tags.
int HXREF_NAME(hxref_tag_cells)(int method, int nx, int ny, Real dx, Real dy, const Real* Ug, const Real* Tg,
                                Real time, Real h_th, Real u_th, Real z_th, signed char* tags, char* err) {
    const int lo[2] = {0, 0}, hi[2] = {0, 0};
    try {
        OneLevel L(method, nx, ny, dx, dy, lo, hi);
        const size_t gp = (size_t)(nx + 2) * (ny + 2);
        auto U = L.U_new[0][0].array();
        auto T = L.Terrain[0][0].array();
        for (int j = -1; j <= ny; ++j)
            for (int i = -1; i <= nx; ++i) {
                const size_t o = (size_t)(i + 1) + (size_t)(j + 1) * (nx + 2);
                for (int c = 0; c < 3; ++c) U(i, j, 0, c) = Ug[o + c * gp];
                for (int c = 0; c < 2; ++c) T(i, j, 0, c) = Tg[o + c * gp];
            }
        amrex::TagBoxArray tb(L.grids[0], L.dmap[0], 0);
        tb.setVal(amrex::TagBox::CLEAR);
        PhysicsParameters pp;
        pp.h_grad_thresh = {h_th};
        pp.umag_grad_thresh = {u_th};
        pp.z_grad_thresh = {z_th};
        L.solver.tag_cells(tb, L.U_new[0], L.Terrain[0], L.geom[0], 0, time, pp);
        auto t = tb[0].const_array();
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) tags[i + (size_t)j * nx] = (signed char)t(i, j, 0);
        return 0;
    } catch (const std::exception& e) {
        if (err) { std::strncpy(err, e.what(), 255); err[255] = 0; }
        return 2;
    }
}

}  // extern "C"
