/*
 * hydroexa_gb300.h -- C ABI of the GB300 (sm_103a) per-level advance of HydroEXA.
 *
 * The entry points replace the per-box bodies of the reference solver's
 * operator surface (include/solvers/BaseSolver.H:57-191, dispatched by
 * include/solvers/SolverVariant.H:45-192).  A C++ SolverVariant alternative
 * keeps AMReX's FillPatch, flux registers and clustering and calls these once
 * per MFIter box, passing the Array4 of each MultiFab as an hx_array4_* view.
 *
 * Conventions
 *  - Views are borrowed device pointers.  Element (i, j, comp) of a view is
 *    p[(i - lo[0]) + (j - lo[1]) * jstride + comp * nstride], exactly the
 *    layout of amrex::Array4 (x fastest, ghosts included in [lo, hi]).
 *  - Every call is stream-ordered and asynchronous on the given stream and
 *    allocates nothing.  Calls on different streams are independent.
 *  - Return value: HX_OK, or a negative argument/launch error detected on the
 *    host (HX_ERR_ARG, HX_ERR_LAUNCH).  Every view is checked on the host
 *    against the stencil the call reads (the valid box grown by the ghosts it
 *    needs, the components, the row stride): a view that falls short returns
 *    HX_ERR_ARG with the reason in hx_last_error(), before anything is
 *    launched -- the role of AMREX_ASSERT_WITH_MESSAGE in
 *    src/solvers/HydrostaticRoe.cpp:411-413.  Numerical conditions found on
 *    the device (dt collapse, NaN) are OR-ed into a device status word, read
 *    with hx_status_read(); the adapter maps a nonzero status to amrex::Abort,
 *    as the reference does (src/solvers/HydrostaticRoe.cpp:77-80).  Where a
 *    call takes the status word as optional and it is passed as NULL, those
 *    conditions are not reported (a collapsed dt chain still stops the later
 *    steps of a device time loop).
 *  - The dt reduction is a device accumulator (hx_dt_accum) so a whole time
 *    loop can run without a host round trip; hx_dt_accum_read() is the
 *    synchronising read that replaces ReduceOps::value().
 *
 * Precision: every entry has an _f64 form (the reference's DOUBLE build) and
 * an _f32 form (SINGLE build).  Arithmetic: HX_ARITH_EXACT repeats the
 * reference's operation order with no multiply-add contraction (bit-for-bit
 * the reference's host arithmetic up to cbrt); HX_ARITH_FAST shares
 * reciprocals and square roots between terms, takes them (and the Manning
 * factor's h^(-1/3)) from float seeds with one FP64 Newton step (within
 * 2^-42) and contracts multiply-adds,
 * agreeing with the exact form to a few 1e-15 relative per step (bound:
 * 1e-12 per step); its time step follows the exact form's to a few ulps.
 */
#ifndef HYDROEXA_GB300_H
#define HYDROEXA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* hx_stream_t; /* same handle as cudaStream_t */

enum {
    HX_OK = 0,
    HX_ERR_ARG = -1,
    HX_ERR_LAUNCH = -2,
    HX_ERR_CUDA = -3,
};

/* Device status bits (OR-ed). */
enum {
    HX_STATUS_DT_COLLAPSE = 1, /* min CFL bound < 1e-12 (HydrostaticRoe.cpp:77, Roe.cpp:88) */
    HX_STATUS_NAN = 2,         /* a NaN or Inf appeared in an updated state */
    HX_STATUS_STAGING_TIMEOUT = 4, /* the level kernel's TMA staging wait ran out (about a second); the step
                                      is incomplete (not expected: a fault of the copy hardware or driver) */
};

enum { HX_ARITH_EXACT = 0, HX_ARITH_FAST = 1 };
enum { HX_METHOD_ROE = 0, HX_METHOD_HYDROSTATIC_ROE = 1 };
/*
 * Physical-boundary codes of the level calls, one per side (bc_lo[dir],
 * bc_hi[dir]), as the inputs file gives them (HydroEXA.lo_bc / hi_bc,
 * include/boundaries/BCFill.H:35-138): 0 a wall, anything else open (every
 * field copied from the edge cell).  At a wall eta and depth are mirrored and
 * the terrain copied from the edge, and the momenta follow the BC records the
 * reference's time loop applies to them: its per-step FillPatch fills hu, hv
 * with BC-record offset 0 (include/utils/FillPatchUtils.H:128-129,
 * BCFill.H:244-264), so hu is mirrored without a sign change on every wall
 * and hv is negated across x walls only -- mass and momentum cross such a
 * wall once flow reaches it, as in the reference.
 * HX_BC_CLOSED_WALL (no counterpart in the reference's inputs) is the wall
 * with each momentum's own record: hu negated across x walls, hv across y
 * walls, so nothing crosses it.  The box calls read the ghosts the caller
 * filled and take no codes.
 */
enum { HX_BC_REFLECTIVE = 0, HX_BC_TRANSMISSIVE = 1, HX_BC_CLOSED_WALL = 2 };

typedef struct hx_array4_f64 {
    double* p;
    int64_t jstride;
    int64_t nstride;
    int32_t lo[2];
    int32_t hi[2];
    int32_t ncomp;
} hx_array4_f64;

typedef struct hx_array4_f32 {
    float* p;
    int64_t jstride;
    int64_t nstride;
    int32_t lo[2];
    int32_t hi[2];
    int32_t ncomp;
} hx_array4_f32;

typedef struct hx_array4_i8 {
    signed char* p;
    int64_t jstride;
    int64_t nstride;
    int32_t lo[2];
    int32_t hi[2];
    int32_t ncomp;
} hx_array4_i8;

typedef struct hx_array4_i32 {
    int32_t* p;
    int64_t jstride;
    int64_t nstride;
    int32_t lo[2];
    int32_t hi[2];
    int32_t ncomp;
} hx_array4_i32;

/* Inclusive cell box, like amrex::Box in 2-D. */
typedef struct hx_box {
    int32_t lo[2];
    int32_t hi[2];
} hx_box;

/* Device-resident dt accumulator: min per-cell CFL bound and max(|u|,|v|),
 * both before the CFL factor, as in compute_dt_Impl's ReduceOps<Min,Max>.
 * Opaque; 64-byte aligned device memory of hx_dt_accum_bytes() bytes. */
typedef struct hx_dt_accum hx_dt_accum;

/* ---- library ------------------------------------------------------------ */

/* Version string and the last host-side error message of this thread. */
const char* hx_version(void);
const char* hx_last_error(void);
/* Number of kernels this library launched since load (all entry points). */
uint64_t hx_launch_count(void);

/* Device status word: one uint32 of device memory owned by the caller. */
int hx_status_clear(uint32_t* status_dev, hx_stream_t stream);
/* Synchronises the stream and returns the status bits (or a negative error). */
int hx_status_read(const uint32_t* status_dev, hx_stream_t stream);

/* dt accumulator in caller-owned device memory of hx_dt_accum_bytes() bytes. */
int64_t hx_dt_accum_bytes(void);
int hx_dt_accum_reset(hx_dt_accum* acc, hx_stream_t stream);
/* Synchronising read (the ReduceOps::value() of compute_dt_Impl). */
int hx_dt_accum_read_f64(const hx_dt_accum* acc, double* dt_min, double* max_vel, hx_stream_t stream);
int hx_dt_accum_read_f32(const hx_dt_accum* acc, float* dt_min, float* max_vel, hx_stream_t stream);

/* ---- per-box operators (AMReX keeps the ghost fill) ---------------------- */

/*
 * Hydrostatic-Roe advance of one box (replaces the per-box body of
 * HydrostaticRoe::compute_fluxes_Impl, src/solvers/HydrostaticRoe.cpp:484-606:
 * h rebuild, x and y dual face fluxes, update with Manning friction and dry
 * clamp), fused into one kernel.
 *   eta_ext  free surface, >= 2 ghosts filled (FillPatchEta)
 *   U_ext    comps 1,2 = hu, hv with >= 2 ghosts filled (FillPatch)
 *   T_ext    comps 0,1 = z, Manning n with >= 2 ghosts filled (FillPatchTerrain)
 *   U_old    the stored state of the valid box (comp 0 is the stored depth)
 *   U_new    destination, valid box
 *   FL/FR    optional (NULL) nodal face arrays for reflux, 3 comps each,
 *            [0] = x faces, [1] = y faces (HydrostaticRoe.cpp:442-454)
 *   next_dt  optional: min CFL bound / max|vel| of U_new are folded in
 *            (compute_dt_Impl of the next step, fused)
 *   status   optional device status word
 */
int hx_advance_box_hydrostatic_f64(const hx_array4_f64* eta_ext, const hx_array4_f64* U_ext,
                                   const hx_array4_f64* T_ext, const hx_array4_f64* U_old, hx_array4_f64* U_new,
                                   hx_box valid, double dt, double dx, double dy, const hx_array4_f64* FL,
                                   const hx_array4_f64* FR, hx_dt_accum* next_dt, uint32_t* status, int arith,
                                   hx_stream_t stream);
int hx_advance_box_hydrostatic_f32(const hx_array4_f32* eta_ext, const hx_array4_f32* U_ext,
                                   const hx_array4_f32* T_ext, const hx_array4_f32* U_old, hx_array4_f32* U_new,
                                   hx_box valid, float dt, float dx, float dy, const hx_array4_f32* FL,
                                   const hx_array4_f32* FR, hx_dt_accum* next_dt, uint32_t* status, int arith,
                                   hx_stream_t stream);

/*
 * Classic Roe advance of one box (replaces Roe::compute_fluxes_Impl's per-box
 * body, src/solvers/Roe.cpp:327-434: in-place h rebuild on the grown tile,
 * first-order F / S- / S+ faces, four-term update).
 *   eta      free surface with >= 1 ghost (FillPatchEta)
 *   U_old    comps 1,2 with >= 1 ghost (FillPatch); comp 0 is overwritten on
 *            the grown box with max(0, eta - z), as the reference does
 *   T        z, n with >= 1 ghost
 *   F, Sm, Sp optional nodal face arrays ([0] x, [1] y) for the reflux
 *            selection (Roe.cpp:369-388)
 */
int hx_advance_box_roe_f64(const hx_array4_f64* eta, hx_array4_f64* U_old, const hx_array4_f64* T,
                           hx_array4_f64* U_new, hx_box valid, double dt, double dx, double dy,
                           const hx_array4_f64* F, const hx_array4_f64* Sm, const hx_array4_f64* Sp,
                           hx_dt_accum* next_dt, uint32_t* status, int arith, hx_stream_t stream);
int hx_advance_box_roe_f32(const hx_array4_f32* eta, hx_array4_f32* U_old, const hx_array4_f32* T,
                           hx_array4_f32* U_new, hx_box valid, float dt, float dx, float dy,
                           const hx_array4_f32* F, const hx_array4_f32* Sm, const hx_array4_f32* Sp,
                           hx_dt_accum* next_dt, uint32_t* status, int arith, hx_stream_t stream);

/* ---- reflux: the flux-register fluxes emitted by the advance kernels ------ */

/*
 * Hydrostatic advance that writes, instead of FL and FR, the one flux the
 * registers receive, Freg[d] = 0.5 FL + 0.5 FR on the box's nodal faces ([0] x,
 * [1] y) -- the flux-register preparation of HydrostaticRoe::compute_fluxes_Impl
 * (src/solvers/HydrostaticRoe.cpp:612-627) fused into the face loop.  The
 * caller passes Freg to FluxRegister::CrseInit (scale -dt dA) / FineAdd
 * (scale dt dA) as the reference does.  Other arguments as
 * hx_advance_box_hydrostatic_*.
 */
int hx_advance_box_hydrostatic_reflux_f64(const hx_array4_f64* eta_ext, const hx_array4_f64* U_ext,
                                          const hx_array4_f64* T_ext, const hx_array4_f64* U_old,
                                          hx_array4_f64* U_new, hx_box valid, double dt, double dx, double dy,
                                          const hx_array4_f64* Freg, hx_dt_accum* next_dt, uint32_t* status,
                                          int arith, hx_stream_t stream);
int hx_advance_box_hydrostatic_reflux_f32(const hx_array4_f32* eta_ext, const hx_array4_f32* U_ext,
                                          const hx_array4_f32* T_ext, const hx_array4_f32* U_old,
                                          hx_array4_f32* U_new, hx_box valid, float dt, float dx, float dy,
                                          const hx_array4_f32* Freg, hx_dt_accum* next_dt, uint32_t* status,
                                          int arith, hx_stream_t stream);
/*
 * Classic Roe advance that writes the side-selected effective fluxes of the
 * flux registers (src/solvers/Roe.cpp:369-388 and 447-566) instead of F, S-,
 * S+, on the box's nodal faces ([0] x, [1] y, 3 comps):
 *   D- = F - S- (the flux the right cell saw), D+ = F + S+ (the left cell's).
 *   flux_crse (optional): with fine_mask (one int comp, 0 = coarse, 1 = covered
 *     by the next finer level, >= 1 ghost: amrex::makeFineMask(U, fine grids,
 *     ratio, 0, 1)), D+ where the left cell is coarse and the right covered,
 *     D- where the left is covered and the right coarse, 0 elsewhere.
 *   flux_fine (optional): D- on faces at the low end of grid_box (the box's
 *     grid, which may extend beyond a tile), D+ at its high end, 0 elsewhere.
 * Other arguments as hx_advance_box_roe_*.
 */
int hx_advance_box_roe_reflux_f64(const hx_array4_f64* eta, hx_array4_f64* U_old, const hx_array4_f64* T,
                                  hx_array4_f64* U_new, hx_box valid, double dt, double dx, double dy,
                                  const hx_array4_i32* fine_mask, hx_box grid_box, const hx_array4_f64* flux_crse,
                                  const hx_array4_f64* flux_fine, hx_dt_accum* next_dt, uint32_t* status, int arith,
                                  hx_stream_t stream);
int hx_advance_box_roe_reflux_f32(const hx_array4_f32* eta, hx_array4_f32* U_old, const hx_array4_f32* T,
                                  hx_array4_f32* U_new, hx_box valid, float dt, float dx, float dy,
                                  const hx_array4_i32* fine_mask, hx_box grid_box, const hx_array4_f32* flux_crse,
                                  const hx_array4_f32* flux_fine, hx_dt_accum* next_dt, uint32_t* status, int arith,
                                  hx_stream_t stream);

/*
 * Per-cell CFL bound of one box folded into acc (replaces the ReduceOps pass of
 * compute_dt_Impl, src/solvers/HydrostaticRoe.cpp:19-65 and
 * src/solvers/Roe.cpp:20-76; the two are arithmetically identical).
 */
int hx_dt_reduce_box_f64(const hx_array4_f64* U, const hx_array4_f64* T, hx_box valid, double dx, double dy,
                         hx_dt_accum* acc, hx_stream_t stream);
int hx_dt_reduce_box_f32(const hx_array4_f32* U, const hx_array4_f32* T, hx_box valid, float dx, float dy,
                         hx_dt_accum* acc, hx_stream_t stream);

/*
 * Gradient tagging of one box (replaces tag_cells_Impl:
 * src/solvers/HydrostaticRoe.cpp:88-171 when method is
 * HX_METHOD_HYDROSTATIC_ROE, src/solvers/Roe.cpp:100-181 when HX_METHOD_ROE).
 * U and T must cover one ghost around the box.  Writes set_value
 * (amrex::TagBox::SET) to tagged cells only.
 */
int hx_tag_box_f64(int method, const hx_array4_f64* U, const hx_array4_f64* T, hx_array4_i8* tags, hx_box valid,
                   double dx, double dy, double time, double h_thresh, double umag_thresh, double z_thresh,
                   signed char set_value, hx_stream_t stream);
int hx_tag_box_f32(int method, const hx_array4_f32* U, const hx_array4_f32* T, hx_array4_i8* tags, hx_box valid,
                   float dx, float dy, float time, float h_thresh, float umag_thresh, float z_thresh,
                   signed char set_value, hx_stream_t stream);

/*
 * NODATA-aware volume-weighted restriction of the coarse box crse_box
 * (replaces the kernel of amrex::masked_average_down,
 * src/utils/MaskedAverageDown.cpp:45-60 and include/utils/MaskedAverageDown.H:64-104).
 * Components scomp..scomp+ncomp-1 of fine go to ccomp.. of crse.
 */
int hx_masked_average_down_box_f64(const hx_array4_f64* fine, hx_array4_f64* crse, hx_box crse_box, int scomp,
                                   int ccomp, int ncomp, int rx, int ry, double fine_volume, double nodata,
                                   hx_stream_t stream);
int hx_masked_average_down_box_f32(const hx_array4_f32* fine, hx_array4_f32* crse, hx_box crse_box, int scomp,
                                   int ccomp, int ncomp, int rx, int ry, float fine_volume, float nodata,
                                   hx_stream_t stream);

/*
 * Conservative restriction of the coarse box crse_box: each coarse value is the
 * mean of its rx*ry fine values, summed rows outer, columns inner, times
 * 1/(rx*ry) (replaces amrex::average_down as AmrMeshState::AverageDownTo and
 * AverageDown call it on the state, src/state/AmrMeshState_AMR.cpp:828-844;
 * Cartesian geometry).  Components scomp.. of fine go to ccomp.. of crse.
 */
int hx_average_down_box_f64(const hx_array4_f64* fine, hx_array4_f64* crse, hx_box crse_box, int scomp, int ccomp,
                            int ncomp, int rx, int ry, hx_stream_t stream);
int hx_average_down_box_f32(const hx_array4_f32* fine, hx_array4_f32* crse, hx_box crse_box, int scomp, int ccomp,
                            int ncomp, int rx, int ry, hx_stream_t stream);

/* ---- eta and the conservation diagnostics ---------------------------------- */

/*
 * eta = h + z on box b, ghosts included where the views cover them: the kernel
 * of AmrMeshState::DeriveEtaFrom (src/state/AmrMeshState_AMR.cpp:203-224).
 */
int hx_derive_eta_box_f64(const hx_array4_f64* U, const hx_array4_f64* terrain, hx_array4_f64* eta, hx_box b,
                          hx_stream_t stream);
int hx_derive_eta_box_f32(const hx_array4_f32* U, const hx_array4_f32* terrain, hx_array4_f32* eta, hx_box b,
                          hx_stream_t stream);

/*
 * The per-box reduction of AmrMeshState::ComputeMassDiagnostics
 * (src/state/AmrMeshState_Utils.cpp:242-298) over the valid box b: out (device,
 * 5 doubles) = {mass, x-momentum, y-momentum, kinetic energy, min h} summed
 * over cells that are not NODATA (roughness == -9999) and wet (h > 0), each
 * cell's terms in the reference's types and order, the sums carried in double
 * in a fixed order (deterministic).  min h is DBL_MAX / FLT_MAX when no cell
 * counts.  work: hx_diagnostics_work_bytes(b) bytes of device memory.  The
 * reference assigns each box's result to the level's total instead of adding
 * it (AmrMeshState_Utils.cpp:293-296), so with several boxes per level it
 * reports the last box only; an adapter reproducing that keeps the last
 * call's output, one summing the level adds the per-box outputs.
 */
int64_t hx_diagnostics_work_bytes(hx_box b);
int hx_diagnostics_box_f64(const hx_array4_f64* U, const hx_array4_f64* terrain, hx_box b, double dx, double dy,
                           double* out, void* work, hx_stream_t stream);
int hx_diagnostics_box_f32(const hx_array4_f32* U, const hx_array4_f32* terrain, hx_box b, float dx, float dy,
                           double* out, void* work, hx_stream_t stream);

/*
 * The hydrostatic step with its epilogue: hx_advance_box_hydrostatic_* (no face
 * arrays) whose update also writes, from the values it stores in U_new,
 *  - eta_new (not NULL; one component covering the valid box): eta = h + z of
 *    every valid cell, the kernel of DeriveEtaFrom (AmrMeshState_AMR.cpp:219)
 *    on the valid box.  The reference derives eta on the grown box and then
 *    fills the ghost ring (FillBoundary); that ring is the caller's fill here.
 *  - diag_out (not NULL; device, 5 doubles): the diagnostics of the updated
 *    state on the valid box, as hx_diagnostics_box_* defines them, with work of
 *    hx_diagnostics_work_bytes(valid) bytes.
 * Neither output needs another pass over the box.  HX_ARITH_EXACT: every
 * cell's terms are hx_diagnostics_box_*'s; on boxes below 2048 x 2048 cells
 * the blocks are its blocks too and the result is identical to it, on larger
 * ones only the sums' order differs.  HX_ARITH_FAST (double): h, hu, hv and
 * (hu^2 + hv^2) / h are summed unscaled (the reciprocal within 2^-44) and
 * scaled by dA and 0.5 dA once per block: within 1e-12 relative of the exact
 * sums, min h identical.  At least one of eta_new and diag_out is given.
 */
int hx_advance_box_hydrostatic_epilogue_f64(const hx_array4_f64* eta_ext, const hx_array4_f64* U_ext,
                                            const hx_array4_f64* T_ext, const hx_array4_f64* U_old,
                                            hx_array4_f64* U_new, hx_box valid, double dt, double dx, double dy,
                                            hx_dt_accum* next_dt, uint32_t* status, int arith,
                                            hx_array4_f64* eta_new, double* diag_out, void* work,
                                            hx_stream_t stream);
int hx_advance_box_hydrostatic_epilogue_f32(const hx_array4_f32* eta_ext, const hx_array4_f32* U_ext,
                                            const hx_array4_f32* T_ext, const hx_array4_f32* U_old,
                                            hx_array4_f32* U_new, hx_box valid, float dt, float dx, float dy,
                                            hx_dt_accum* next_dt, uint32_t* status, int arith,
                                            hx_array4_f32* eta_new, double* diag_out, void* work,
                                            hx_stream_t stream);

/* ---- single-box level with the physical boundary fused into the loader --- */

/*
 * A whole level held as one box [0,nx) x [0,ny) with no ghost cells: planes
 * h, hu, hv (state) and z, n (terrain), each with row pitch `pitch` elements.
 * The ghost values the reference's FillPatch + HydroPhysBC produce at the
 * domain edge (include/boundaries/BCFill.H:35-86,159-181: wall = mirror, normal
 * momentum negated; open = copy edge; terrain always copies the edge) are
 * generated inside the tile loader instead of stored.
 */
typedef struct hx_level_f64 {
    const double* h;
    const double* hu;
    const double* hv;
    const double* z;
    const double* n;
    int64_t pitch;
    int32_t nx, ny;
    double dx, dy;
    int32_t bc_lo[2];
    int32_t bc_hi[2];
} hx_level_f64;

typedef struct hx_level_f32 {
    const float* h;
    const float* hu;
    const float* hv;
    const float* z;
    const float* n;
    int64_t pitch;
    int32_t nx, ny;
    float dx, dy;
    int32_t bc_lo[2];
    int32_t bc_hi[2];
} hx_level_f32;

/* One advance of the level by dt (host value); writes h/hu/hv_out (same pitch). */
int hx_level_advance_f64(int method, const hx_level_f64* L, double dt, double* h_out, double* hu_out,
                         double* hv_out, hx_dt_accum* next_dt, uint32_t* status, int arith, hx_stream_t stream);
int hx_level_advance_f32(int method, const hx_level_f32* L, float dt, float* h_out, float* hu_out, float* hv_out,
                         hx_dt_accum* next_dt, uint32_t* status, int arith, hx_stream_t stream);

/*
 * One hydrostatic advance of the level with the epilogue of
 * hx_advance_box_hydrostatic_epilogue_*: eta_out (not NULL; same pitch) = h + z
 * of the updated state, diag_out (not NULL; device, 5 doubles) = its
 * diagnostics as hx_level_diagnostics_f64 defines them, work of
 * hx_diagnostics_work_bytes of the box (0,0)-(nx-1,ny-1) bytes.  Levels from
 * 2048 x 2048 cells run the persistent kernel with the epilogue in it.
 */
int hx_level_advance_epilogue_f64(const hx_level_f64* L, double dt, double* h_out, double* hu_out, double* hv_out,
                                  hx_dt_accum* next_dt, uint32_t* status, int arith, double* eta_out,
                                  double* diag_out, void* work, hx_stream_t stream);
int hx_level_advance_epilogue_f32(const hx_level_f32* L, float dt, float* h_out, float* hu_out, float* hv_out,
                                  hx_dt_accum* next_dt, uint32_t* status, int arith, float* eta_out,
                                  double* diag_out, void* work, hx_stream_t stream);

/* compute_dt_Impl over the level (no ghosts needed). */
int hx_level_dt_reduce_f64(const hx_level_f64* L, hx_dt_accum* acc, hx_stream_t stream);
int hx_level_dt_reduce_f32(const hx_level_f32* L, hx_dt_accum* acc, hx_stream_t stream);
/* hx_diagnostics_box_f64 over a whole single-box level (work: hx_diagnostics_work_bytes of
 * the box (0,0)-(nx-1,ny-1)). */
int hx_level_diagnostics_f64(const hx_level_f64* level, double* out, void* work, hx_stream_t stream);

/*
 * nsteps of the single-level time loop of the reference driver
 * (src/HydroEXA.cpp:259-266 with AmrMeshState::ComputeDt and AdvanceLevel at
 * one level): dt = cfl * min CFL bound of the current state, status
 * HX_STATUS_DT_COLLAPSE if that minimum is below 1e-12, then advance.  The dt
 * chain stays on the device (three rotating accumulators in `work`, the next
 * step's bound fused into each advance), so the loop issues one kernel per
 * step and can be captured in a CUDA graph.  The state ping-pongs between the
 * level's planes and (h_alt, hu_alt, hv_alt); *final_in_alt reports where the
 * last state is.  time_dev (optional, 1 value) accumulates the simulated time.
 * work: caller-owned device memory of hx_level_run_work_bytes() bytes.
 */
int64_t hx_level_run_work_bytes(void);
int hx_level_run_f64(int method, hx_level_f64* L, double* h_alt, double* hu_alt, double* hv_alt, int nsteps,
                     double cfl, void* work, uint32_t* status, double* time_dev, int arith, int* final_in_alt,
                     hx_stream_t stream);
int hx_level_run_f32(int method, hx_level_f32* L, float* h_alt, float* hu_alt, float* hv_alt, int nsteps,
                     float cfl, void* work, uint32_t* status, float* time_dev, int arith, int* final_in_alt,
                     hx_stream_t stream);

/*
 * Host-buffer form of hx_level_run for callers whose level lives in host
 * memory: copies h, hu, hv, z, n (host, pitch nx) to the device, runs nsteps,
 * copies the state back.  Device buffers, streams and events are created by
 * the call on the current device and cached per thread and per device for
 * the next call of that size on that device (hx_host_cache_release frees the
 * calling thread's caches on every device).  The copies overlap the computation in row bands, and they can only
 * when the host buffers are page-locked (cudaHostAlloc or cudaHostRegister).
 * The hydrostatic first step of the leading bands computes its flux differences
 * as the rows land and updates once the level's dt is known; the share of rows
 * so split follows each call's measured upload and compute times (the cache
 * keeps it; hx_debug_host_split_frac reads it) and does not change the result.
 * The call returns once the state is back in h, hu, hv: the status bits
 * (>= 0) or a negative error.
 */
int hx_level_run_host_f64(int method, int nx, int ny, double dx, double dy, const int32_t bc_lo[2],
                          const int32_t bc_hi[2], double* h, double* hu, double* hv, const double* z,
                          const double* n, int nsteps, double cfl, int arith, double* time_out, hx_stream_t stream);
void hx_host_cache_release(void);

/* ---- batched ensemble ---------------------------------------------------- */

/*
 * Many independent single-box levels (scenarios of any sizes) advanced
 * together: one persistent kernel per step drains a tile queue spanning every
 * member, each member keeps its own CFL dt chain, status word and clock, and
 * the steps are replayed from a CUDA graph.  No counterpart in the reference
 * (which advances one hierarchy per process); per member the arithmetic is
 * exactly that of hx_level_run_f64.
 */
/* Tile shapes: 256-cell tiles on 256-thread blocks, several per SM, for small
 * and medium members; HX_TILE_32x32 on 1024-thread blocks, one per SM, for
 * large members (fewer halo cells, slopes and faces per cell). */
enum { HX_TILE_32x8 = 0, HX_TILE_16x16 = 1, HX_TILE_64x4 = 2, HX_TILE_32x32 = 3 };

typedef struct hx_ensemble_member_f64 {
    hx_level_f64 level; /* state (advanced in place, see final_in_alt), terrain, geometry, BC codes */
    double* h_alt;      /* ping-pong planes with the level's pitch */
    double* hu_alt;
    double* hv_alt;
    int32_t tile_shape; /* HX_TILE_*: chosen per size class by the autotuner */
} hx_ensemble_member_f64;

/* Device scratch for n members (descriptor table, dt accumulators, queue). */
int64_t hx_ensemble_work_bytes(int n);
/* Total queue length (tiles) of a member list. */
int hx_ensemble_tiles(int n, const hx_ensemble_member_f64* members, int64_t* tiles);
/*
 * nsteps for every member.  status: n device words (cleared by the caller),
 * time_dev: n device doubles.  use_graph != 0 replays the launches from a CUDA
 * graph.  *final_in_alt = 1 when the results are in the alternate planes.
 */
int hx_ensemble_run_f64(int n, const hx_ensemble_member_f64* members, int nsteps, double cfl, void* work,
                        uint32_t* status, double* time_dev, int arith, int use_graph, int* final_in_alt,
                        hx_stream_t stream);

/*
 * Allocation-free form of hx_level_run_f64.  No counterpart in the reference:
 * it is for callers that cannot allocate device memory of their own.  HydroEXA
 * runs on AMReX, whose arena reserves most of the GPU's memory at start-up
 * (three quarters by default) and serves all later requests itself, so a
 * cudaMalloc issued by a library in the middle of the time loop can fail or
 * compete with the arena; other host codes forbid allocation once their loop
 * has started.  This call allocates nothing: the scratch the loop needs (the
 * alternate state planes it ping-pongs into and the three rotating CFL
 * accumulators) is one fixed array inside this library,
 * 256 bytes + 3 x HX_STATIC_RUN_MAX_CELLS doubles (6 MiB), which every GPU that
 * loads the library holds until the process exits.
 *   - The level must satisfy ny * pitch <= HX_STATIC_RUN_MAX_CELLS (512 x 512);
 *     a larger one is rejected with HX_ERR_ARG and an explanatory
 *     hx_last_error().  Use hx_level_run_f64 with your own scratch for it.
 *   - The state is advanced in place: level->h, hu, hv hold the result in
 *     their valid cells (nx of each pitch-long row; row padding is not
 *     touched).  The arithmetic form applies to the first CFL reduction and to
 *     every step, as in hx_level_run_f64, and the result is that call's.
 *     status and time_dev are optional caller-owned device words; without a
 *     status word a dt collapse goes to a word inside the array and is not
 *     reported.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current and caches it; make that
 *     first call before any stream capture.
 *   - Every call uses the same array and each call clears the accumulators it
 *     needs when it starts.  Calls that overlap on the GPU -- on two streams, or
 *     from two host threads -- race on the array and corrupt each other.
 */
#define HX_STATIC_RUN_MAX_CELLS 262144
int hx_level_run_static_f64(int method, hx_level_f64* level, int nsteps, double cfl, uint32_t* status,
                            double* time_dev, int arith, hx_stream_t stream);

/* ---- adjoint of the hydrostatic-Roe time loop ---------------------------- */

/*
 * Gradient of the gauge misfit J = sum_{n=1..N} sum_g (h^n_g - href^n_g)^2 of
 * an N-step hydrostatic-Roe run (device CFL chain) with
 * respect to the initial state (h, hu, hv) and the bed z.  No counterpart in the
 * reference, which runs forward only.  The adjoint is hand-written: a reverse
 * kernel of the whole step (van Leer limiter and MUSCL reconstruction, the Roe
 * flux taking the forward's entropy-fix and dry branches, the hydrostatic cap
 * and pressure correction, the update, Manning factor and dry clamp) plus the
 * dependence of each step's dt on the cell that set the CFL bound.
 *   checkpoint_every = 0: every state is kept (N + 5 states in work);
 *   k > 0: every k-th state is kept and each k-step segment is recomputed once
 *   in the reverse sweep, on a second stream while the previous segment is
 *   reversed (N/k + 2k + 9 states in work);
 *   k < 0: binomial checkpointing with -k snapshot slots (Griewank's revolve
 *   schedule: the fewest recomputed steps for that memory; -k + 8 states in
 *   work).  hx_adjoint_recompute_steps gives the forward steps the reverse
 *   sweep recomputes under each choice.
 * hx_adjoint_forward_f64 runs the forward sweep: the level's planes are the
 * initial state (not modified); series (device, N x ngauges) receives h at the
 * gauge cells (cell index i + j * pitch) after every step.
 * hx_adjoint_reverse_f64 then returns seed * dJ/d(h0, hu0, hv0, z) (device
 * planes with the level's pitch), with the same work buffer and arguments.
 * arith (HX_ARITH_FAST / HX_ARITH_EXACT) selects the forward's arithmetic
 * form; the reverse recomputes the forward's values in the same form so that
 * it takes the same branches.  HX_ARITH_EXACT runs the trajectory of
 * hx_level_run_f64 with HX_ARITH_EXACT bit for bit (and of the tangent-linear
 * step's value part).
 * options of hx_adjoint_work_bytes_f64, and the same bit OR-ed into arith of
 * the reverse: HX_ADJ_FACE_RECORDS (fast form, k > 0) makes the segment
 * recompute record each face's Roe intermediates (square roots, shared
 * reciprocal, Roe averages, fixed speeds, wave strengths; 11 doubles and a
 * flag byte per face) and each cell's van Leer slopes with their reciprocals,
 * 2 k steps' worth in work, so the reverse reads them instead of evaluating
 * them again; the gradient agrees with the unrecorded reverse to rounding.
 * Ignored for k <= 0 and the exact form.
 * Restriction: nx % 32 != 1 and ny % 16 != 1.
 */
#define HX_ADJ_FACE_RECORDS 0x100
int64_t hx_adjoint_work_bytes_f64(int nx, int ny, int64_t pitch, int nsteps, int checkpoint_every, int options);
int64_t hx_adjoint_recompute_steps(int nsteps, int checkpoint_every);
int hx_adjoint_forward_f64(const hx_level_f64* level, int nsteps, double cfl, int ngauges, const int64_t* gauge_cells,
                           double* series, int checkpoint_every, int arith, void* work, uint32_t* status,
                           hx_stream_t stream);
int hx_adjoint_reverse_f64(const hx_level_f64* level, int nsteps, double cfl, int ngauges,
                           const int64_t* gauge_cells, const double* href, double seed, int checkpoint_every,
                           int arith, void* work, double* grad_h, double* grad_hu, double* grad_hv, double* grad_z,
                           hx_stream_t stream);
/*
 * One reverse step at a fixed dt: (lam_h, lam_hu, lam_hv) = lambda^{n+1}
 * (device planes) -> out = lambda^n, zbar += dJ/dz, *dtbar (device) = dJ/d dt.
 * work: hx_adjoint_work_bytes_f64(nx, ny, pitch, 1, 0, 0) bytes.
 */
int hx_adjoint_step_f64(const hx_level_f64* level, double dt, const double* lam_h, const double* lam_hu,
                        const double* lam_hv, double* out_h, double* out_hu, double* out_hv, double* zbar,
                        double* dtbar, int arith, void* work, hx_stream_t stream);

/* ---- diagnostics --------------------------------------------------------- */

/*
 * Tangent-linear step at fixed dt, computed by carrying (value, derivative)
 * pairs through the exact arithmetic form: every plane of the level (h, hu, hv,
 * z, n) and of the outputs holds interleaved pairs, pitch counted in pairs;
 * ddt is the derivative of dt.  The independent check of the adjoint.
 */
int hx_level_tangent_f64(const hx_level_f64* level_pairs, double dt, double ddt, double* out_h, double* out_hu,
                         double* out_hv, hx_stream_t stream);

/* ---- multi-box level (same-level ghosts without FillPatch) ------------------- */

/*
 * One box of a level: its valid cells lo..hi (level cell coordinates), state
 * (h, hu, hv) and a second state for the time loop, terrain (z, n), planes of
 * (hi[1]-lo[1]+1) rows x pitch elements.
 */
typedef struct hx_levelbox_f64 {
    double *h, *hu, *hv;
    double *h_alt, *hu_alt, *hv_alt;
    const double *z, *n;
    int64_t pitch;
    int32_t lo[2], hi[2];
} hx_levelbox_f64;

/* ---- native plotfile ------------------------------------------------------ */

/* One box of one level: device planes of the state and the terrain with a row
 * pitch (doubles), covering cells lo..hi of the level's index space. */
typedef struct hx_plotbox_f64 {
    const double *h, *hu, *hv, *z, *n;
    int64_t pitch;
    int32_t lo[2], hi[2];
} hx_plotbox_f64;

/* One level: its boxes, domain box, cell size, step count and refinement ratio
 * to the next finer level (unused on the finest). */
typedef struct hx_plotlevel_f64 {
    const hx_plotbox_f64* boxes;
    int32_t nboxes;
    int32_t domain_lo[2], domain_hi[2];
    double dx, dy;
    int32_t ref_ratio;
    int32_t istep;
} hx_plotlevel_f64;

/*
 * AMReX native plotfile (HyperCLaw-V1.1) of the levels' state and terrain
 * (replaces WriteNativePlotfile, src/io/NativePlotFile.cpp:19-97, which calls
 * amrex::WriteMultiLevelPlotfile): directory <prefix><iteration as 5 digits>
 * with Header, Level_<l>/Cell_H and Level_<l>/Cell_D_00000; variables
 * h_fluid, hu_momentum, hv_momentum, z_bathymetry, extra_comp_4 (terrain
 * component 1, the Manning coefficient, as the reference names it).  Copies from
 * the device on stream through pinned staging; returns once the files are
 * written.
 */
int hx_write_plotfile_f64(const char* prefix, int iteration, double time, int nlevels,
                          const hx_plotlevel_f64* levels, const double prob_lo[2], const double prob_hi[2],
                          hx_stream_t stream);

/*
 * The single-level time loop of hx_level_run_f64 (hydrostatic-Roe) on a level
 * given as several boxes that tile the domain (0,0)-(nx-1,ny-1) -- the
 * same-level BoxArray of AMReX.  The ghosts a box needs are read straight
 * from the boxes that own those cells, and physical-boundary ghosts follow
 * the BCFill rules: the FillPatch of same-level and physical ghosts
 * (src/state/AmrMeshState_AMR.cpp:667-767, include/boundaries/BCFill.H:211-296)
 * and the U_ext / Terrain_ext / Eta_ext copies (HydrostaticRoe.cpp:456-500)
 * are not needed.  Each step is one launch over the tiles of all boxes with
 * one CFL chain for the level (levels from 2048 x 2048 cells: 32 x 32 tiles
 * walked by one block per SM, each tile staged from the boxes that own its
 * cells; below that, 32 x 8 tiles one block each); results equal the
 * single-box run bit for bit.
 * Boxes must not overlap and must cover the domain (coarse-fine ghosts still
 * need FillPatch).  On return *final_in_alt says which state of each box
 * holds the result.  work: hx_boxlevel_work_bytes bytes of device memory.
 */
int64_t hx_boxlevel_work_bytes(int nboxes, const hx_levelbox_f64* boxes, int nx, int ny);
int hx_boxlevel_run_f64(int nboxes, const hx_levelbox_f64* boxes, int nx, int ny, double dx, double dy,
                        const int32_t bc_lo[2], const int32_t bc_hi[2], int nsteps, double cfl, int arith, void* work,
                        uint32_t* status, double* time_dev, int* final_in_alt, hx_stream_t stream);

/* ---- the FP64 roof --------------------------------------------------------- */

/*
 * Measured FMA issue rates of the current GPU (thread instructions per second,
 * best of three launches of register-only FMA chains): DFMA, and FFMA when
 * ffma_per_s is not NULL.  The fused FP64 kernels are bound by FP64 issue on
 * GB300; bench.py reports their FP64-pipe fraction against this rate.
 * Synchronises the stream; allocates a few MB for the duration of the call.
 */
int hx_measure_fp64_rate(double* dfma_per_s, double* ffma_per_s, hx_stream_t stream);

/* ---- diagnostics (points) ------------------------------------------------ */

/*
 * Evaluate the device Riemann solvers on arrays of face states (device
 * memory), for checking them against golden vectors.  method
 * HX_METHOD_HYDROSTATIC_ROE: states (n, 6) = (hi hui hvi hj huj hvj), aux
 * (n, 2) = face normal, out (n, 3) = F (include/solvers/kernels/HydrostaticRoe.H:44).
 * method HX_METHOD_ROE: states (n, 10) = (hi hui hvi zi ni hj huj hvj zj nj),
 * aux (n, 4) = (dt dx nx ny), out (3, n, 3) = F, S-, S+
 * (include/solvers/kernels/Roe.H:51).  Normals must be (1,0) or (0,1).
 */
int hx_debug_roe_points_f64(int method, int arith, long n, const double* states, const double* aux, double* out,
                            hx_stream_t stream);
int hx_debug_roe_points_f32(int method, int arith, long n, const float* states, const float* aux, float* out,
                            hx_stream_t stream);
/* The fast form's FP64 reciprocal of n device values (to check it against IEEE division). */
int hx_debug_rcp_f64(long n, const double* x, double* y, hx_stream_t stream);
/* The fast form's FP64 square root of n device values (to check it against the IEEE square root). */
int hx_debug_sqrt_f64(long n, const double* x, double* y, hx_stream_t stream);
/* The fast form's FP64 building blocks on n device points (to check their
 * error bounds): HX_FAST_OP_RCP and HX_FAST_OP_SQRT (one Newton step, the
 * face flux's), HX_FAST_OP_SLOPE (the van Leer slope of the triplets
 * x[3i], x[3i+1], x[3i+2]: x holds 3n values), HX_FAST_OP_RCP_FAITHFUL and
 * HX_FAST_OP_SQRT_FAITHFUL (the CFL rate's, within an ulp), HX_FAST_OP_RCBRT
 * (h^(-1/3) of the Manning factor, for depths within the float range).  y holds
 * n values. */
enum {
    HX_FAST_OP_RCP = 0,
    HX_FAST_OP_SQRT = 1,
    HX_FAST_OP_SLOPE = 2,
    HX_FAST_OP_RCP_FAITHFUL = 3,
    HX_FAST_OP_SQRT_FAITHFUL = 4,
    HX_FAST_OP_RCBRT = 5
};
int hx_debug_fast_op_f64(int op, long n, const double* x, double* y, hx_stream_t stream);
/* Test setting of the persistent level kernel's TMA staging: the next launches wait for this many bytes
 * more than the tiles bring, so the bounded wait runs out (about a second per block) and the step ends with
 * HX_STATUS_STAGING_TIMEOUT; 0 (the default) restores normal operation.  Returns the previous value. */
int hx_debug_staging_extra_bytes(unsigned bytes);
/* The row bands hx_level_run_host_f64 uses for ny rows (host only, no GPU):
 * writes band starts into starts[0..n] (starts[n] = ny) and returns n, at
 * most 10; max_bands must be at least 10. */
int hx_debug_host_bands(int ny, int* starts, int max_bands);
/* The share of the rows whose first step hx_level_run_host_f64 splits on the
 * calling thread's current device (0.45 before a call; afterwards the value
 * each call sets from its measured upload and compute times, within
 * [0.15, 0.85]); -1 without a usable device. */
double hx_debug_host_split_frac(void);

#ifdef __cplusplus
}
#endif

#endif /* HYDROEXA_GB300_H */
