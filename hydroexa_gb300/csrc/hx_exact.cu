// Exact arithmetic form: compiled with --fmad=false so that every product and
// sum is rounded separately, as in the reference's host build.  Also home of
// the kernels that must be bit-exact in any build (tags, restriction).
#include "hx_kernels.cuh"

namespace hx {
#define HX_INST(R)                                                                                             \
    template cudaError_t launch_hydro<R, false, LevelSrc<R>>(const LevelSrc<R>&, const Cells3<R>&,            \
                                                             const Plane<R>&, const Cells3W<R>&,               \
                                                             const FaceOut<R>&, const IBox&, const StepCtl<R>&, \
                                                             cudaStream_t);                                    \
    template cudaError_t launch_hydro<R, false, BoxSrc<R>>(const BoxSrc<R>&, const Cells3<R>&, const Plane<R>&, \
                                                           const Cells3W<R>&, const FaceOut<R>&, const IBox&,  \
                                                           const StepCtl<R>&, cudaStream_t);                   \
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
                                                  int, R, R, cudaStream_t);
HX_INST(double)
HX_INST(float)
#undef HX_INST
template cudaError_t launch_points<double, false>(int, long, const double*, const double*, double*, cudaStream_t);
template cudaError_t launch_points<float, false>(int, long, const float*, const float*, float*, cudaStream_t);
}  // namespace hx
