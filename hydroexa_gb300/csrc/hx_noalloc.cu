// hx_level_run_static_f64: the single-level time loop for callers that cannot
// allocate device memory.
//
// HydroEXA runs on AMReX, whose arena takes most of the GPU's memory when the
// run starts (three quarters of it by default) and hands it out itself; a
// library that calls cudaMalloc on its own during the time loop can fail there
// or fight the arena for memory, and some host codes simply forbid allocation
// once their loop has started.  This entry point needs no allocation at all:
// the scratch the loop needs -- the alternate state planes it ping-pongs into
// and the three rotating CFL accumulators -- lives in the fixed array below,
// which every GPU that loads this library holds until the process exits.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "hx_launch.h"

namespace hx {
void note_launches(int n);          // hx_capi.cu
int set_error(int code, const char* msg);  // hx_capi.cu
}  // namespace hx

using namespace hx;

namespace {

constexpr long long kMaxCells = HX_STATIC_RUN_MAX_CELLS;
constexpr size_t kHeadBytes = 256;  // 3 accumulators (192 B), a status word, padding
constexpr size_t kScratchBytes = kHeadBytes + 3 * (size_t)kMaxCells * sizeof(double);

// The scratch.  In host code this name is only a stand-in for the device
// symbol: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_run_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (with that device current) and cached.
int scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(HX_ERR_ARG, "hx_level_run_static_f64: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_run_scratch);
        if (e != cudaSuccess || !p) {
            char msg[256];
            snprintf(msg, sizeof msg, "hx_level_run_static_f64: cudaGetSymbolAddress failed: %s",
                     cudaGetErrorString(e));
            return set_error(HX_ERR_CUDA, msg);
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return HX_OK;
}

}  // namespace

extern "C" int hx_level_run_static_f64(int method, hx_level_f64* L, int nsteps, double cfl, uint32_t* status,
                                       double* time_dev, int arith, hx_stream_t stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!L || !L->h || !L->hu || !L->hv || !L->z || !L->n)
        return set_error(HX_ERR_ARG, "hx_level_run_static_f64: null level plane");
    if (L->nx < 2 || L->ny < 2 || L->pitch < L->nx || !(L->dx > 0) || !(L->dy > 0))
        return set_error(HX_ERR_ARG, "hx_level_run_static_f64: bad level geometry");
    if (method != HX_METHOD_ROE && method != HX_METHOD_HYDROSTATIC_ROE)
        return set_error(HX_ERR_ARG, "hx_level_run_static_f64: unknown method");
    if (nsteps < 0 || !(cfl > 0)) return set_error(HX_ERR_ARG, "hx_level_run_static_f64: nsteps < 0 or cfl <= 0");
    const long long cells = (long long)L->ny * (long long)L->pitch;
    if (cells > kMaxCells) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "hx_level_run_static_f64: level of %lld cells (ny x pitch) exceeds the static scratch of %lld cells; "
                 "use hx_level_run_f64 with caller-provided scratch",
                 cells, kMaxCells);
        return set_error(HX_ERR_ARG, msg);
    }
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    DtAccum* slot = reinterpret_cast<DtAccum*>(base);
    uint32_t* own_status = reinterpret_cast<uint32_t*>(static_cast<char*>(base) + 3 * sizeof(DtAccum));
    double* alt = reinterpret_cast<double*>(static_cast<char*>(base) + kHeadBytes);
    uint32_t* stw = status ? status : own_status;

    // The array keeps whatever the previous call left: clear the accumulators
    // and the internal status word; the alternate planes are written by the
    // first step before anything reads them.
    cudaError_t e = cudaMemsetAsync(base, 0, kHeadBytes, st);
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));

    const IBox vb{0, 0, L->nx - 1, L->ny - 1};
    {
        Cells3<double> U;
        U.p[0] = L->h; U.p[1] = L->hu; U.p[2] = L->hv;
        U.js = L->pitch; U.lo0 = 0; U.lo1 = 0;
        Plane<double> Z{L->z, L->pitch, 0, 0};
        // the same arithmetic form as the steps, as hx_level_run_f64 does
        e = arith == HX_ARITH_EXACT ? launch_dt_reduce<double, false>(U, Z, vb, L->dx, L->dy, &slot[0], st)
                                    : launch_dt_reduce<double, true>(U, Z, vb, L->dx, L->dy, &slot[0], st);
        if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
        note_launches(1);
    }
    double* A[3] = {const_cast<double*>(L->h), const_cast<double*>(L->hu), const_cast<double*>(L->hv)};
    double* B[3] = {alt, alt + cells, alt + 2 * cells};
    const int g = (method == HX_METHOD_HYDROSTATIC_ROE) ? 2 : 1;
    for (int s = 0; s < nsteps; ++s) {
        const bool even = (s % 2) == 0;
        double* const* in = even ? A : B;
        double* const* out = even ? B : A;
        StepCtl<double> ctl;
        ctl.dt_host = 0.0;
        ctl.cfl = cfl;
        ctl.dt_in = &slot[s % 3];
        ctl.dt_out = s + 1 < nsteps ? &slot[(s + 1) % 3] : nullptr;
        ctl.dt_reset = &slot[(s + 2) % 3];
        ctl.status = stw;
        ctl.time = time_dev;
        ctl.dx = L->dx;
        ctl.dy = L->dy;
        LevelSrc<double> src;
        src.h = in[0]; src.hu = in[1]; src.hv = in[2]; src.z = L->z; src.n = L->n;
        src.pitch = L->pitch;
        src.nx = L->nx; src.ny = L->ny;
        src.bc_xlo = L->bc_lo[0]; src.bc_ylo = L->bc_lo[1]; src.bc_xhi = L->bc_hi[0]; src.bc_yhi = L->bc_hi[1];
        src.glo0 = -g; src.glo1 = -g; src.ghi0 = L->nx - 1 + g; src.ghi1 = L->ny - 1 + g;
        Cells3W<double> o;
        o.p[0] = out[0]; o.p[1] = out[1]; o.p[2] = out[2];
        o.js = L->pitch; o.lo0 = 0; o.lo1 = 0;
        if (method == HX_METHOD_HYDROSTATIC_ROE) {
            Cells3<double> uo;
            uo.p[0] = in[0]; uo.p[1] = in[1]; uo.p[2] = in[2];
            uo.js = L->pitch; uo.lo0 = 0; uo.lo1 = 0;
            Plane<double> np{L->n, L->pitch, 0, 0};
            FaceOut<double> fo{};
            fo.on = 0;
            e = arith == HX_ARITH_EXACT ? launch_hydro<double, false, LevelSrc<double>>(src, uo, np, o, fo, vb, ctl, st)
                                        : launch_hydro<double, true, LevelSrc<double>>(src, uo, np, o, fo, vb, ctl, st);
        } else {
            FaceOut9<double> fo{};
            fo.on = 0;
            RebuildOut<double> hb{};
            hb.on = 0;
            e = arith == HX_ARITH_EXACT ? launch_classic<double, false, LevelSrc<double>>(src, o, fo, hb, vb, ctl, st)
                                        : launch_classic<double, true, LevelSrc<double>>(src, o, fo, hb, vb, ctl, st);
        }
        if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
        note_launches(1);
    }
    // An odd number of steps leaves the result in the scratch: copy its valid
    // cells back (nx of every pitch-long row; the caller's row padding is left
    // as it was).
    if (nsteps % 2) {
        const size_t row = (size_t)L->nx * sizeof(double), pitch = (size_t)L->pitch * sizeof(double);
        for (int k = 0; k < 3 && e == cudaSuccess; ++k)
            e = cudaMemcpy2DAsync(A[k], pitch, B[k], pitch, row, (size_t)L->ny, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    }
    return HX_OK;
}
