// C-ABI of the multi-box level: a same-level BoxArray advanced without
// FillPatch.  The host checks that the boxes tile the domain, builds the map
// from g x g blocks of the domain to boxes (g: the greatest common divisor of
// the box corners) and the table of the tiles of all boxes -- 32 x 8, or on
// levels of 2048^2 cells and more 32 x 32 for the persistent kernel, as the
// single-box level takes them; each step is one launch over that table, with
// one dt chain for the level.
#include <cstring>
#include <numeric>
#include <vector>

#include "hx_launch.h"

namespace hx {
void note_launches(int n);
int set_error(int code, const char* msg);
extern template cudaError_t launch_dt_reduce<double, false>(const Cells3<double>&, const Plane<double>&, const IBox&,
                                                            double, double, DtAccum*, cudaStream_t);
extern template cudaError_t launch_dt_reduce<double, true>(const Cells3<double>&, const Plane<double>&, const IBox&,
                                                           double, double, DtAccum*, cudaStream_t);
}  // namespace hx

using namespace hx;

namespace {

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Plan {
    int g = 0, mnx = 0, mny = 0;
    bool big = false;  // 32 x 32 tiles and the persistent kernel
    std::vector<int> map, tiles;
    size_t off_boxes = 0, off_map = 0, off_tiles = 0, total = 0;
};

int make_plan(int nb, const hx_levelbox_f64* boxes, int nx, int ny, Plan& P) {
    if (nb < 1 || !boxes || nx < 2 || ny < 2) return set_error(HX_ERR_ARG, "boxlevel: no boxes or bad domain");
    int g = std::gcd(nx, ny);
    for (int k = 0; k < nb; ++k) {
        const hx_levelbox_f64& b = boxes[k];
        if (b.lo[0] < 0 || b.lo[1] < 0 || b.hi[0] >= nx || b.hi[1] >= ny || b.hi[0] < b.lo[0] || b.hi[1] < b.lo[1])
            return set_error(HX_ERR_ARG, "boxlevel: a box lies outside the domain");
        if (!b.h || !b.hu || !b.hv || !b.z || !b.n || !b.h_alt || !b.hu_alt || !b.hv_alt)
            return set_error(HX_ERR_ARG, "boxlevel: null plane");
        if (b.pitch < b.hi[0] - b.lo[0] + 1) return set_error(HX_ERR_ARG, "boxlevel: pitch below the box width");
        g = std::gcd(g, std::gcd(std::gcd(b.lo[0], b.lo[1]), std::gcd(b.hi[0] + 1, b.hi[1] + 1)));
    }
    P.g = g;
    P.big = (long long)nx * (long long)ny >= kBigTileCells;
    const int tx = P.big ? 32 : TX, ty = P.big ? 32 : TY;
    P.mnx = nx / g;
    P.mny = ny / g;
    P.map.assign((size_t)P.mnx * P.mny, -1);
    for (int k = 0; k < nb; ++k) {
        const hx_levelbox_f64& b = boxes[k];
        for (int j = b.lo[1] / g; j <= b.hi[1] / g; ++j)
            for (int i = b.lo[0] / g; i <= b.hi[0] / g; ++i) {
                int& m = P.map[(size_t)j * P.mnx + i];
                if (m != -1) return set_error(HX_ERR_ARG, "boxlevel: boxes overlap");
                m = k;
            }
        for (int y0 = b.lo[1]; y0 <= b.hi[1]; y0 += ty)
            for (int x0 = b.lo[0]; x0 <= b.hi[0]; x0 += tx) {
                P.tiles.push_back(k);
                P.tiles.push_back(x0);
                P.tiles.push_back(y0);
            }
    }
    for (int m : P.map)
        if (m < 0) return set_error(HX_ERR_ARG, "boxlevel: the boxes do not cover the domain (coarse-fine ghosts "
                                                "need FillPatch)");
    size_t o = 256;  // three dt accumulators
    P.off_boxes = o; o += al256(sizeof(DevBox) * nb);
    P.off_map = o; o += al256(sizeof(int) * P.map.size());
    P.off_tiles = o; o += al256(sizeof(int) * P.tiles.size());
    P.total = o;
    return HX_OK;
}

}  // namespace

extern "C" int64_t hx_boxlevel_work_bytes(int nboxes, const hx_levelbox_f64* boxes, int nx, int ny) {
    Plan P;
    if (make_plan(nboxes, boxes, nx, ny, P) != HX_OK) return 0;
    return (int64_t)P.total;
}

extern "C" int hx_boxlevel_run_f64(int nboxes, const hx_levelbox_f64* boxes, int nx, int ny, double dx, double dy,
                                   const int32_t bc_lo[2], const int32_t bc_hi[2], int nsteps, double cfl, int arith,
                                   void* work, uint32_t* status, double* time_dev, int* final_in_alt,
                                   hx_stream_t stream) {
    cudaStream_t st = (cudaStream_t)stream;
    Plan P;
    int rc = make_plan(nboxes, boxes, nx, ny, P);
    if (rc) return rc;
    if (!work || !bc_lo || !bc_hi || nsteps < 0 || !(cfl > 0) || !(dx > 0) || !(dy > 0))
        return set_error(HX_ERR_ARG, "boxlevel: bad arguments");
    char* base = static_cast<char*>(work);
    DtAccum* slot = reinterpret_cast<DtAccum*>(base);
    std::vector<DevBox> db((size_t)nboxes);
    for (int k = 0; k < nboxes; ++k) {
        const hx_levelbox_f64& b = boxes[k];
        DevBox& d = db[(size_t)k];
        d.h[0] = b.h; d.hu[0] = b.hu; d.hv[0] = b.hv;
        d.h[1] = b.h_alt; d.hu[1] = b.hu_alt; d.hv[1] = b.hv_alt;
        d.z = b.z; d.n = b.n;
        d.pitch = b.pitch;
        d.lo0 = b.lo[0]; d.lo1 = b.lo[1]; d.hi0 = b.hi[0]; d.hi1 = b.hi[1];
    }
    // plan to the device (pageable sources: the copies complete before the call returns them)
    cudaError_t e = cudaMemsetAsync(base, 0, 256, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + P.off_boxes, db.data(), sizeof(DevBox) * db.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + P.off_map, P.map.data(), sizeof(int) * P.map.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + P.off_tiles, P.tiles.data(), sizeof(int) * P.tiles.size(), cudaMemcpyHostToDevice,
                            st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    int launches = 0;
    // CFL bound of the initial state, box by box into slot 0
    for (int k = 0; k < nboxes && e == cudaSuccess; ++k) {
        const DevBox& d = db[(size_t)k];
        Cells3<double> U;
        U.p[0] = d.h[0]; U.p[1] = d.hu[0]; U.p[2] = d.hv[0];
        U.js = d.pitch; U.lo0 = d.lo0; U.lo1 = d.lo1;
        const Plane<double> Z{d.z, d.pitch, d.lo0, d.lo1};
        const IBox vb{d.lo0, d.lo1, d.hi0, d.hi1};
        e = arith == HX_ARITH_EXACT ? launch_dt_reduce<double, false>(U, Z, vb, dx, dy, &slot[0], st)
                                    : launch_dt_reduce<double, true>(U, Z, vb, dx, dy, &slot[0], st);
        ++launches;
    }
    BoxSetSrc src;
    src.boxes = reinterpret_cast<const DevBox*>(base + P.off_boxes);
    src.map = reinterpret_cast<const int*>(base + P.off_map);
    src.g = P.g; src.mnx = P.mnx;
    src.nx = nx; src.ny = ny;
    src.bc_xlo = bc_lo[0]; src.bc_ylo = bc_lo[1]; src.bc_xhi = bc_hi[0]; src.bc_yhi = bc_hi[1];
    src.self = 0;
    src.glo0 = -2; src.glo1 = -2; src.ghi0 = nx + 1; src.ghi1 = ny + 1;
    const int* tiles = reinterpret_cast<const int*>(base + P.off_tiles);
    const int ntiles = (int)(P.tiles.size() / 3);
    for (int s = 0; s < nsteps && e == cudaSuccess; ++s) {
        StepCtl<double> ctl;
        ctl.dt_host = 0.0; ctl.cfl = cfl;
        ctl.dt_in = &slot[s % 3]; ctl.dt_out = s + 1 < nsteps ? &slot[(s + 1) % 3] : nullptr;
        ctl.dt_reset = &slot[(s + 2) % 3];
        ctl.status = status; ctl.time = time_dev; ctl.dx = dx; ctl.dy = dy;
        src.phase = s % 2;
        e = arith == HX_ARITH_EXACT ? launch_boxlevel<false>(src, tiles, ntiles, ctl, st, P.big)
                                    : launch_boxlevel<true>(src, tiles, ntiles, ctl, st, P.big);
        ++launches;
    }
    note_launches(launches);
    if (e != cudaSuccess) return set_error(HX_ERR_LAUNCH, cudaGetErrorString(e));
    if (final_in_alt) *final_in_alt = nsteps % 2;
    return HX_OK;
}
