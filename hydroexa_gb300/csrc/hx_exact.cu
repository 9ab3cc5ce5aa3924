// Exact arithmetic form: compiled with --fmad=false so that every product and
// sum is rounded separately, as in the reference's host build.  Also home of
// the kernels that must be bit-exact in any build (tags, restriction).
#include "hx_kernels.cuh"

namespace hx {
#define HX_INST(R)                                                                                             \
    template cudaError_t launch_hydro<R, false, LevelSrc<R>>(                                                  \
        const LevelSrc<R>&, const Cells3<R>&, const Plane<R>&, const Cells3W<R>&, const FaceOut<R>&,           \
        const IBox&, const StepCtl<R>&, cudaStream_t, const EpiOut<R>*);                                       \
    template cudaError_t launch_hydro<R, false, BoxSrc<R>>(                                                    \
        const BoxSrc<R>&, const Cells3<R>&, const Plane<R>&, const Cells3W<R>&, const FaceOut<R>&,             \
        const IBox&, const StepCtl<R>&, cudaStream_t, const EpiOut<R>*);                                       \
    template cudaError_t launch_classic<R, false, LevelSrc<R>>(const LevelSrc<R>&, const Cells3W<R>&,         \
                                                               const FaceOut9<R>&, const RebuildOut<R>&,       \
                                                               const IBox&, const StepCtl<R>&, cudaStream_t);  \
    template cudaError_t launch_classic<R, false, BoxSrc<R>>(const BoxSrc<R>&, const Cells3W<R>&,             \
                                                             const FaceOut9<R>&, const RebuildOut<R>&,         \
                                                             const IBox&, const StepCtl<R>&, cudaStream_t);    \
    template cudaError_t launch_dt_reduce<R, false>(const Cells3<R>&, const Plane<R>&, const IBox&, R, R,      \
                                                    DtAccum*, cudaStream_t);                                   \
    template cudaError_t launch_tag<R>(int, const V4<R>&, const V4<R>&, const V4<signed char>&, const IBox&, R, \
                                       R, R, R, R, R, signed char, cudaStream_t);                              \
    template cudaError_t launch_masked_avgdown<R>(const V4<R>&, const V4<R>&, const IBox&, int, int, int, int,  \
                                                  int, R, R, cudaStream_t);                                     \
    template cudaError_t launch_average_down<R>(const V4<R>&, const V4<R>&, const IBox&, int, int, int, int, int,  \
                                                cudaStream_t);                                                    \
    template cudaError_t launch_derive_eta<R>(const V4<R>&, const V4<R>&, const V4<R>&, const IBox&,          \
                                              cudaStream_t);                                                    \
    template cudaError_t launch_diagnostics<R>(const Plane<R>&, const Plane<R>&, const Plane<R>&,             \
                                               const Plane<R>&, const IBox&, R, double*, double*, cudaStream_t);
HX_INST(double)
HX_INST(float)
#undef HX_INST
template cudaError_t launch_ensemble<double, false>(const EnsInstance<double>*, int, long long, int, double, unsigned long long*, int, cudaStream_t);
template cudaError_t launch_ensemble_big<double, false>(const EnsInstance<double>*, int, long long, int, double, unsigned long long*, int, cudaStream_t);
template int ensemble_blocks_per_sm<double, false>();
template cudaError_t launch_boxlevel<false>(const BoxSetSrc&, const int*, int, const StepCtl<double>&, cudaStream_t,
                                            bool);
template cudaError_t launch_hydro_split<double, false>(const LevelSrc<double>&, const Cells3<double>&,
                                                      const Plane<double>&, const DivOut<double>&, const IBox&,
                                                      double, double, cudaStream_t);
template cudaError_t launch_hydro_update<double, false>(const Cells3<double>&, const DivOut<double>&,
                                                       const Plane<double>&, const Plane<double>&,
                                                       const Cells3W<double>&, const IBox&, const StepCtl<double>&,
                                                       cudaStream_t);
template cudaError_t launch_adj_forward<false>(const LevelSrc<double>&, const Cells3<double>&, const Plane<double>&,
                                              const Cells3W<double>&, const IBox&, const StepCtl<double>&,
                                              const double*, unsigned*, const AdjRecord&, cudaStream_t);
template cudaError_t launch_adj_forward_linear<false>(const LevelSrc<double>&, const Cells3<double>&,
                                                     const Plane<double>&, const Cells3W<double>&, const IBox&, double,
                                                     double, const double*, cudaStream_t);
template cudaError_t launch_points<double, false>(int, long, const double*, const double*, double*, cudaStream_t);
template cudaError_t launch_points<float, false>(int, long, const float*, const float*, float*, cudaStream_t);
}  // namespace hx

// ---------------------------------------------------------------------------
// Tangent-linear step: the exact tile body carried on dual numbers.
// ---------------------------------------------------------------------------
namespace hx {
__global__ void __launch_bounds__(NT) k_hydro_tangent(LevelSrc<Dual> src, Cells3<Dual> uo, Plane<Dual> np,
                                                      Cells3W<Dual> out, IBox vb, Dual dt, double dx, double dy) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HydroSmem<Dual>& S = *reinterpret_cast<HydroSmem<Dual>*>(smem_raw);
    FaceOut<Dual> fo{};
    fo.on = 0;
    hydro_tile_body<Dual, false, TX, TY, NT>(S, src, uo, np, out, fo, vb, vb.lo0 + (int)blockIdx.x * TX,
                                             vb.lo1 + (int)blockIdx.y * TY, dt, Dual(dx), Dual(dy), nullptr, nullptr);
}

cudaError_t launch_tangent(const LevelSrc<Dual>& src, const Cells3<Dual>& uo, const Plane<Dual>& np,
                           const Cells3W<Dual>& out, const IBox& vb, Dual dt, double dx, double dy, cudaStream_t st) {
    const size_t sm = sizeof(HydroSmem<Dual>);
    cudaError_t e = ensure_smem(k_hydro_tangent, sm);
    if (e != cudaSuccess) return e;
    k_hydro_tangent<<<tile_grid(vb, TX, TY), NT, sm, st>>>(src, uo, np, out, vb, dt, dx, dy);
    return cudaGetLastError();
}
}  // namespace hx
