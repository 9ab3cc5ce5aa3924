// Launcher declarations.  Definitions live in hx_kernels.cuh and are
// explicitly instantiated by hx_exact.cu (compiled --fmad=false, FAST=false)
// and hx_fast.cu (FAST=true), so this header never instantiates a kernel.
#pragma once

#include "hx_device.cuh"
#include "hx_internal.h"

namespace hx {

// One hydrostatic step; epi (not null): with the advance epilogue (eta and the
// conservation diagnostics of the updated state, folded into epi->out).
template <class R, bool FAST, class Src>
cudaError_t launch_hydro(const Src& src, const Cells3<R>& uo, const Plane<R>& np, const Cells3W<R>& out,
                         const FaceOut<R>& fo, const IBox& vb, const StepCtl<R>& ctl, cudaStream_t st,
                         const EpiOut<R>* epi = nullptr);

template <class R, bool FAST, class Src>
cudaError_t launch_classic(const Src& src, const Cells3W<R>& out, const FaceOut9<R>& fo, const RebuildOut<R>& hb,
                           const IBox& vb, const StepCtl<R>& ctl, cudaStream_t st);

// One hydrostatic step of a multi-box level over its tile table: 32 x 8 tiles one block each, or (big)
// 32 x 32 tiles walked by the persistent kernel.
template <bool FAST>
cudaError_t launch_boxlevel(const BoxSetSrc& src, const int* tiles, int ntiles, const StepCtl<double>& ctl,
                            cudaStream_t st, bool big);

// The hydrostatic step in two launches: flux differences (no dt), then the
// update once dt is known (same arithmetic as launch_hydro).
template <class R, bool FAST>
cudaError_t launch_hydro_split(const LevelSrc<R>& src, const Cells3<R>& uo, const Plane<R>& np, const DivOut<R>& div,
                               const IBox& vb, R dx, R dy, cudaStream_t st);
template <class R, bool FAST>
cudaError_t launch_hydro_update(const Cells3<R>& uo, const DivOut<R>& div, const Plane<R>& np, const Plane<R>& zp,
                                const Cells3W<R>& out, const IBox& vb, const StepCtl<R>& ctl, cudaStream_t st);

template <class R, bool FAST>
cudaError_t launch_dt_reduce(const Cells3<R>& U, const Plane<R>& Z, const IBox& vb, R dx, R dy, DtAccum* acc,
                             cudaStream_t st);

template <class R, bool FAST>
cudaError_t launch_points(int method, long n, const R* st, const R* aux, R* out, cudaStream_t stream);
template <bool FAST> cudaError_t launch_rcp(long n, const double* x, double* y, int which, cudaStream_t st);

template <class R>
cudaError_t launch_tag(int method, const V4<R>& U, const V4<R>& T, const V4<signed char>& tags, const IBox& vb, R dx,
                       R dy, R time, R h_th, R u_th, R z_th, signed char set_value, cudaStream_t st);

template <class R>
cudaError_t launch_masked_avgdown(const V4<R>& fine, const V4<R>& crse, const IBox& cb, int scomp, int ccomp,
                                  int ncomp, int rx, int ry, R fv, R nodata, cudaStream_t st);

template <class R>
cudaError_t launch_average_down(const V4<R>& fine, const V4<R>& crse, const IBox& cb, int scomp, int ccomp,
                                int ncomp, int rx, int ry, cudaStream_t st);

template <class R>
cudaError_t launch_derive_eta(const V4<R>& U, const V4<R>& T, const V4<R>& eta, const IBox& b, cudaStream_t st);

template <class R>
cudaError_t launch_diagnostics(const Plane<R>& h, const Plane<R>& hu, const Plane<R>& hv, const Plane<R>& nr,
                               const IBox& b, R dA, double* part, double* out, cudaStream_t st);

template <class R, bool FAST>
cudaError_t launch_ensemble(const EnsInstance<R>* inst, int ninst, long long total_tiles, int step, R cfl,
                           unsigned long long* queue, int grid, cudaStream_t st);

template <class R, bool FAST> int ensemble_blocks_per_sm();
// The large members on 32 x 32 tiles (queue counters queue[2], queue[3]), one CTA per SM.
template <class R, bool FAST>
cudaError_t launch_ensemble_big(const EnsInstance<R>* inst, int ninst, long long total_tiles, int step, R cfl,
                               unsigned long long* queue, int grid, cudaStream_t st);

// Forward step of the adjoint's sweeps: the tile body with dt from the device
// chain (dt_fixed == nullptr; the step's dt is resolved from ctl) or from
// *dt_fixed (segment recompute), recording in *post_flags whether any cell took
// the Manning factor (1) or the dry clamp (2).
template <bool FAST>
cudaError_t launch_adj_forward(const LevelSrc<double>& src, const Cells3<double>& uo, const Plane<double>& np,
                               const Cells3W<double>& out, const IBox& vb, const StepCtl<double>& ctl,
                               const double* dt_fixed, unsigned* post_flags, const AdjRecord& rec, cudaStream_t st);
// The flux update alone at *dt_fixed (the state before friction and clamp).
template <bool FAST>
cudaError_t launch_adj_forward_linear(const LevelSrc<double>& src, const Cells3<double>& uo, const Plane<double>& np,
                                      const Cells3W<double>& out, const IBox& vb, double dx, double dy,
                                      const double* dt_fixed, cudaStream_t st);

cudaError_t launch_tangent(const LevelSrc<Dual>& src, const Cells3<Dual>& uo, const Plane<Dual>& np,
                           const Cells3W<Dual>& out, const IBox& vb, Dual dt, double dx, double dy, cudaStream_t st);

inline dim3 tile_grid(const IBox& b, int tx, int ty) {
    return dim3((unsigned)((b.hi0 - b.lo0 + 1 + tx - 1) / tx), (unsigned)((b.hi1 - b.lo1 + 1 + ty - 1) / ty));
}

}  // namespace hx
