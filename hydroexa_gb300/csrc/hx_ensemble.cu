// C-ABI of the batched ensemble: many independent single-box levels advanced
// together, one persistent launch per step, steps replayed from a CUDA graph.
#include <cstdio>
#include <vector>

#include "hx_launch.h"

namespace hx {
void note_launches(int n);                  // hx_capi.cu
int set_error(int code, const char* msg);  // hx_capi.cu

}  // namespace hx

using namespace hx;

namespace {

constexpr int kPeriod = 6;  // parity repeats every 2 steps, dt slots every 3

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Layout {
    size_t desc, slots, queue, total;
};

Layout layout(int n) {
    Layout L;
    L.desc = 0;
    L.slots = align256((size_t)n * sizeof(EnsInstance<double>));
    L.queue = L.slots + align256((size_t)n * 3 * sizeof(DtAccum));
    L.total = L.queue + 256;
    return L;
}

int tile_w(int shape) { return shape == HX_TILE_16x16 ? 16 : (shape == HX_TILE_64x4 ? 64 : 32); }
int tile_h(int shape) {
    return shape == HX_TILE_16x16 ? 16 : (shape == HX_TILE_64x4 ? 4 : (shape == HX_TILE_32x32 ? 32 : 8));
}

int err(int code, const char* fmt, int a) {
    char buf[256];
    snprintf(buf, sizeof buf, fmt, a);
    return set_error(code, buf);
}

}  // namespace

extern "C" int64_t hx_ensemble_work_bytes(int n) { return n > 0 ? (int64_t)layout(n).total : 0; }

extern "C" int hx_ensemble_run_f64(int n, const hx_ensemble_member_f64* members, int nsteps, double cfl, void* work,
                                   uint32_t* status, double* time_dev, int arith, int use_graph, int* final_in_alt,
                                   hx_stream_t stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n <= 0 || !members || !work || !status || !time_dev) return set_error(HX_ERR_ARG, "hx_ensemble_run_f64: bad arguments");
    if (nsteps < 0 || !(cfl > 0)) return set_error(HX_ERR_ARG, "hx_ensemble_run_f64: nsteps < 0 or cfl <= 0");
    const Layout Lw = layout(n);
    char* base = static_cast<char*>(work);
    EnsInstance<double>* desc = reinterpret_cast<EnsInstance<double>*>(base + Lw.desc);
    DtAccum* slots = reinterpret_cast<DtAccum*>(base + Lw.slots);
    unsigned long long* queue = reinterpret_cast<unsigned long long*>(base + Lw.queue);

    // the table holds the 256-thread members first, then the 32 x 32 ones; each group numbers its own tiles
    std::vector<EnsInstance<double>> host((size_t)n);
    int nbig = 0;
    for (int i = 0; i < n; ++i) nbig += members[i].tile_shape == HX_TILE_32x32 ? 1 : 0;
    const int nsmall = n - nbig;
    long long tiles = 0, tiles_big = 0;
    int ks = 0, kb = nsmall;
    for (int i = 0; i < n; ++i) {
        const hx_ensemble_member_f64& m = members[i];
        const hx_level_f64& L = m.level;
        if (!L.h || !L.hu || !L.hv || !L.z || !L.n || !m.h_alt || !m.hu_alt || !m.hv_alt)
            return err(HX_ERR_ARG, "hx_ensemble_run_f64: member %d has a null plane", i);
        if (L.nx < 2 || L.ny < 2 || L.pitch < L.nx || !(L.dx > 0) || !(L.dy > 0))
            return err(HX_ERR_ARG, "hx_ensemble_run_f64: member %d has a bad geometry", i);
        if (m.tile_shape < 0 || m.tile_shape > HX_TILE_32x32)
            return err(HX_ERR_ARG, "hx_ensemble_run_f64: member %d has an unknown tile shape", i);
        const bool big = m.tile_shape == HX_TILE_32x32;
        EnsInstance<double>& I = host[(size_t)(big ? kb++ : ks++)];
        I.st[0][0] = const_cast<double*>(L.h);
        I.st[0][1] = const_cast<double*>(L.hu);
        I.st[0][2] = const_cast<double*>(L.hv);
        I.st[1][0] = m.h_alt;
        I.st[1][1] = m.hu_alt;
        I.st[1][2] = m.hv_alt;
        I.z = L.z;
        I.n = L.n;
        I.pitch = L.pitch;
        I.nx = L.nx;
        I.ny = L.ny;
        I.dx = L.dx;
        I.dy = L.dy;
        I.bc[0] = L.bc_lo[0]; I.bc[1] = L.bc_hi[0]; I.bc[2] = L.bc_lo[1]; I.bc[3] = L.bc_hi[1];
        I.shape = m.tile_shape;
        const int tw = tile_w(m.tile_shape), th = tile_h(m.tile_shape);
        I.tiles_x = (L.nx + tw - 1) / tw;
        long long& count = big ? tiles_big : tiles;
        I.tile_base = count;
        count += (long long)I.tiles_x * ((L.ny + th - 1) / th);
        I.slots = slots + 3 * (size_t)i;
        I.status = status + i;
        I.time = time_dev + i;
    }
    cudaError_t e = cudaMemcpyAsync(desc, host.data(), host.size() * sizeof(host[0]), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + Lw.slots, 0, Lw.total - Lw.slots, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host table must outlive the copy
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));

    // each member's first CFL bound
    for (int i = 0; i < n; ++i) {
        const hx_level_f64& L = members[i].level;
        Cells3<double> U;
        U.p[0] = L.h; U.p[1] = L.hu; U.p[2] = L.hv;
        U.js = L.pitch; U.lo0 = 0; U.lo1 = 0;
        Plane<double> Z{L.z, L.pitch, 0, 0};
        const IBox vb{0, 0, L.nx - 1, L.ny - 1};
        e = arith == HX_ARITH_EXACT ? launch_dt_reduce<double, false>(U, Z, vb, L.dx, L.dy, &slots[3 * i], st)
                                    : launch_dt_reduce<double, true>(U, Z, vb, L.dx, L.dy, &slots[3 * i], st);
        if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    }
    note_launches(n);

    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = arith == HX_ARITH_EXACT ? ensemble_blocks_per_sm<double, false>() : ensemble_blocks_per_sm<double, true>();
    if (per_sm <= 0 || sms <= 0) return set_error(HX_ERR_LAUNCH, "hx_ensemble_run_f64: occupancy query failed");
    long long g = (long long)per_sm * sms;
    const int grid = (int)(g < tiles ? g : tiles);
    const int grid_big = (int)(sms < tiles_big ? sms : tiles_big);

    // one step: the 256-thread members, then the 32 x 32 ones (each group drains its own tile queue)
    int per_step = 0;
    auto launch = [&](int step, cudaStream_t s) {
        cudaError_t r = cudaSuccess;
        per_step = 0;
        if (nsmall > 0) {
            r = arith == HX_ARITH_EXACT ? launch_ensemble<double, false>(desc, nsmall, tiles, step, cfl, queue, grid, s)
                                        : launch_ensemble<double, true>(desc, nsmall, tiles, step, cfl, queue, grid, s);
            ++per_step;
        }
        if (r == cudaSuccess && nbig > 0) {
            const EnsInstance<double>* db = desc + nsmall;
            r = arith == HX_ARITH_EXACT
                    ? launch_ensemble_big<double, false>(db, nbig, tiles_big, step, cfl, queue, grid_big, s)
                    : launch_ensemble_big<double, true>(db, nbig, tiles_big, step, cfl, queue, grid_big, s);
            ++per_step;
        }
        return r;
    };

    int done = 0;
    if (use_graph && nsteps >= kPeriod) {
        cudaStream_t cap = nullptr;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (int s = 0; s < kPeriod && e == cudaSuccess; ++s) e = launch(s, cap);
            cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
            if (e == cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        const int reps = nsteps / kPeriod;
        for (int r = 0; r < reps && e == cudaSuccess; ++r) e = cudaGraphLaunch(exec, st);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
        if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
        done = reps * kPeriod;
        note_launches(done * per_step);
    }
    for (int s = done; s < nsteps; ++s) {
        e = launch(s, st);
        if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
        note_launches(per_step);
    }
    if (final_in_alt) *final_in_alt = nsteps % 2;
    return HX_OK;
}

extern "C" int hx_ensemble_tiles(int n, const hx_ensemble_member_f64* members, int64_t* tiles) {
    if (n < 0 || (n > 0 && !members) || !tiles) return set_error(HX_ERR_ARG, "hx_ensemble_tiles: bad arguments");
    long long t = 0;
    for (int i = 0; i < n; ++i) {
        const int s = members[i].tile_shape;
        t += (long long)((members[i].level.nx + tile_w(s) - 1) / tile_w(s)) *
             ((members[i].level.ny + tile_h(s) - 1) / tile_h(s));
    }
    *tiles = t;
    return HX_OK;
}
