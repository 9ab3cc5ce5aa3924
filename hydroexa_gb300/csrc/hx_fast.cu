// Fast arithmetic form: shared reciprocals and square roots, contracted
// multiply-adds (nvcc's default --fmad=true).
#include "hx_kernels.cuh"

namespace hx {
#define HX_INST(R)                                                                                             \
    template cudaError_t launch_hydro<R, true, LevelSrc<R>>(                                                   \
        const LevelSrc<R>&, const Cells3<R>&, const Plane<R>&, const Cells3W<R>&, const FaceOut<R>&,           \
        const IBox&, const StepCtl<R>&, cudaStream_t, const EpiOut<R>*);                                       \
    template cudaError_t launch_hydro<R, true, BoxSrc<R>>(                                                     \
        const BoxSrc<R>&, const Cells3<R>&, const Plane<R>&, const Cells3W<R>&, const FaceOut<R>&,             \
        const IBox&, const StepCtl<R>&, cudaStream_t, const EpiOut<R>*);                                       \
    template cudaError_t launch_classic<R, true, LevelSrc<R>>(const LevelSrc<R>&, const Cells3W<R>&,          \
                                                              const FaceOut9<R>&, const RebuildOut<R>&,        \
                                                              const IBox&, const StepCtl<R>&, cudaStream_t);   \
    template cudaError_t launch_classic<R, true, BoxSrc<R>>(const BoxSrc<R>&, const Cells3W<R>&,              \
                                                            const FaceOut9<R>&, const RebuildOut<R>&,          \
                                                            const IBox&, const StepCtl<R>&, cudaStream_t);     \
    template cudaError_t launch_dt_reduce<R, true>(const Cells3<R>&, const Plane<R>&, const IBox&, R, R,       \
                                                   DtAccum*, cudaStream_t);
HX_INST(double)
HX_INST(float)
#undef HX_INST
template cudaError_t launch_ensemble<double, true>(const EnsInstance<double>*, int, long long, int, double, unsigned long long*, int, cudaStream_t);
template cudaError_t launch_ensemble_big<double, true>(const EnsInstance<double>*, int, long long, int, double, unsigned long long*, int, cudaStream_t);
template int ensemble_blocks_per_sm<double, true>();
template cudaError_t launch_boxlevel<true>(const BoxSetSrc&, const int*, int, const StepCtl<double>&, cudaStream_t,
                                            bool);
template cudaError_t launch_hydro_split<double, true>(const LevelSrc<double>&, const Cells3<double>&,
                                                      const Plane<double>&, const DivOut<double>&, const IBox&,
                                                      double, double, cudaStream_t);
template cudaError_t launch_hydro_update<double, true>(const Cells3<double>&, const DivOut<double>&,
                                                       const Plane<double>&, const Plane<double>&,
                                                       const Cells3W<double>&, const IBox&, const StepCtl<double>&,
                                                       cudaStream_t);
template cudaError_t launch_adj_forward<true>(const LevelSrc<double>&, const Cells3<double>&, const Plane<double>&,
                                              const Cells3W<double>&, const IBox&, const StepCtl<double>&,
                                              const double*, unsigned*, const AdjRecord&, cudaStream_t);
template cudaError_t launch_adj_forward_rec<true>(const LevelSrc<double>&, const Cells3<double>&, const Plane<double>&,
                                                  const Cells3W<double>&, const IBox&, double, double, const double*,
                                                  unsigned*, const FaceRec&, cudaStream_t);
template cudaError_t launch_adj_forward_linear<true>(const LevelSrc<double>&, const Cells3<double>&,
                                                     const Plane<double>&, const Cells3W<double>&, const IBox&, double,
                                                     double, const double*, cudaStream_t);
template cudaError_t launch_rcp<true>(long, const double*, double*, int, cudaStream_t);
template cudaError_t launch_points<double, true>(int, long, const double*, const double*, double*, cudaStream_t);
template cudaError_t launch_points<float, true>(int, long, const float*, const float*, float*, cudaStream_t);
}  // namespace hx
