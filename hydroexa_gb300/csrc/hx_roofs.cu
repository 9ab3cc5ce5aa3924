// The FP64 issue roof of the GPU the library runs on: the rate of dependent-
// chain-free FMA instructions (DFMA, and FFMA for comparison), timed with CUDA
// events.  On GB300 the per-level advance is bound by FP64 issue rather than by
// HBM, so this rate -- not the copy bandwidth -- is the roof its FP64-pipe
// fraction is reported against.
#include <cuda_runtime.h>

#include "hydroexa_gb300.h"

namespace hx {
int set_error(int code, const char* msg);
}

namespace {

constexpr int kChains = 8, kUnroll = 16;

// Each thread keeps kChains independent FMA chains in registers; one store per
// thread (the grid covers out exactly) keeps the work live.
template <class T>
__global__ void __launch_bounds__(256) k_fma_chains(T* out, int iters, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = T(threadIdx.x) * T(1e-3) + T(c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T>
double fma_rate(int sms, int iters, cudaStream_t st, cudaError_t& e) {
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    e = cudaMallocAsync(&out, sizeof(T) * blocks * threads, st);
    if (e != cudaSuccess) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {  // the first launch warms the clocks up
        cudaEventRecord(e0, st);
        k_fma_chains<T><<<blocks, threads, 0, st>>>(out, iters, T(0.999999), T(1e-7));
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        const double n = (double)blocks * threads * iters * kUnroll * kChains;
        if (e == cudaSuccess && ms > 0.f && n / (ms * 1e-3) > best) best = n / (ms * 1e-3);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, st);
    cudaStreamSynchronize(st);
    return best;
}

}  // namespace

extern "C" int hx_measure_fp64_rate(double* dfma_per_s, double* ffma_per_s, hx_stream_t stream) {
    if (!dfma_per_s) return hx::set_error(HX_ERR_ARG, "hx_measure_fp64_rate: null output");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return hx::set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    *dfma_per_s = fma_rate<double>(sms, 2000, st, e);
    if (e == cudaSuccess && ffma_per_s) *ffma_per_s = fma_rate<float>(sms, 8000, st, e);
    if (e != cudaSuccess) return hx::set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    return HX_OK;
}
