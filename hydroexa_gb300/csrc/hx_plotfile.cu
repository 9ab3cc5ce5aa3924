// C-ABI of the native plotfile writer: the level planes (h, hu, hv, z, n) of
// every box of every level, copied from the device and written in AMReX's
// native plotfile layout (HyperCLaw-V1.1), as WriteNativePlotfile does with
// amrex::WriteMultiLevelPlotfile (src/io/NativePlotFile.cpp:19-97).
//
//   <prefix><iteration, 5 digits>/Header
//   <prefix><iteration, 5 digits>/Level_<l>/Cell_H
//   <prefix><iteration, 5 digits>/Level_<l>/Cell_D_00000
//
// One data file per level (the boxes of one writer), each box a FAB: a text
// header naming the real format (64-bit IEEE, little-endian byte order), the
// box and the component count, then the components one after another, x
// fastest.  Copies go through one pinned staging buffer, two boxes in flight:
// the next box is copied while the current one is written.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hydroexa_gb300.h"
#include "hx_internal.h"

namespace hx {
int set_error(int code, const char* msg);
}  // namespace hx

using namespace hx;

namespace {

constexpr int kComps = 5;
const char* const kVarNames[kComps] = {"h_fluid", "hu_momentum", "hv_momentum", "z_bathymetry", "extra_comp_4"};

bool make_dir(const std::string& d) { return mkdir(d.c_str(), 0755) == 0 || errno == EEXIST; }

std::string box_str(const int32_t lo[2], const int32_t hi[2]) {
    char b[96];
    std::snprintf(b, sizeof b, "((%d,%d) (%d,%d) (0,0))", lo[0], lo[1], hi[0], hi[1]);
    return b;
}

std::string real_str(double v) {
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", v);
    return b;
}

struct Staging {
    double* p[2] = {nullptr, nullptr};
    size_t cap = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Staging() {
        for (int k = 0; k < 2; ++k) {
            if (p[k]) cudaFreeHost(p[k]);
            if (ev[k]) cudaEventDestroy(ev[k]);
        }
    }
    cudaError_t init(size_t doubles) {
        cap = doubles;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaMallocHost(&p[k], doubles * sizeof(double));
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
        return e;
    }
};

size_t box_cells(const hx_plotbox_f64& b) { return (size_t)(b.hi[0] - b.lo[0] + 1) * (size_t)(b.hi[1] - b.lo[1] + 1); }

// The five planes of box b into host buffer dst (component-major, x fastest).
cudaError_t copy_box(const hx_plotbox_f64& b, double* dst, cudaStream_t st) {
    const size_t w = (size_t)(b.hi[0] - b.lo[0] + 1), h = (size_t)(b.hi[1] - b.lo[1] + 1);
    const double* src[kComps] = {b.h, b.hu, b.hv, b.z, b.n};
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < kComps && e == cudaSuccess; ++c)
        e = cudaMemcpy2DAsync(dst + c * w * h, w * sizeof(double), src[c], (size_t)b.pitch * sizeof(double),
                              w * sizeof(double), h, cudaMemcpyDeviceToHost, st);
    return e;
}

int check_levels(int nlevels, const hx_plotlevel_f64* levels) {
    if (nlevels < 1 || !levels) return set_error(HX_ERR_ARG, "plotfile: no levels");
    for (int l = 0; l < nlevels; ++l) {
        const hx_plotlevel_f64& L = levels[l];
        if (L.nboxes < 1 || !L.boxes) return set_error(HX_ERR_ARG, "plotfile: a level without boxes");
        if (L.domain_hi[0] < L.domain_lo[0] || L.domain_hi[1] < L.domain_lo[1] || !(L.dx > 0) || !(L.dy > 0))
            return set_error(HX_ERR_ARG, "plotfile: bad level domain or cell size");
        if (l + 1 < nlevels && L.ref_ratio < 1) return set_error(HX_ERR_ARG, "plotfile: bad refinement ratio");
        for (int k = 0; k < L.nboxes; ++k) {
            const hx_plotbox_f64& b = L.boxes[k];
            if (!b.h || !b.hu || !b.hv || !b.z || !b.n) return set_error(HX_ERR_ARG, "plotfile: null plane");
            if (b.hi[0] < b.lo[0] || b.hi[1] < b.lo[1] || b.lo[0] < L.domain_lo[0] || b.lo[1] < L.domain_lo[1] ||
                b.hi[0] > L.domain_hi[0] || b.hi[1] > L.domain_hi[1])
                return set_error(HX_ERR_ARG, "plotfile: a box lies outside its level's domain");
            if (b.pitch < b.hi[0] - b.lo[0] + 1) return set_error(HX_ERR_ARG, "plotfile: pitch below the box width");
        }
    }
    return HX_OK;
}

// Level l's data file and FabArray header; the per-box minima and maxima go to mins/maxs.
int write_level(const std::string& dir, const hx_plotlevel_f64& L, Staging& S, cudaStream_t st) {
    const std::string dfile = dir + "/Cell_D_00000";
    FILE* f = std::fopen(dfile.c_str(), "wb");
    if (!f) return set_error(HX_ERR_ARG, "plotfile: cannot create a data file");
    std::vector<long long> offs((size_t)L.nboxes);
    std::vector<double> mins((size_t)L.nboxes * kComps), maxs((size_t)L.nboxes * kComps);
    cudaError_t e = copy_box(L.boxes[0], S.p[0], st);
    if (e == cudaSuccess) e = cudaEventRecord(S.ev[0], st);
    int rc = HX_OK;
    for (int k = 0; k < L.nboxes && e == cudaSuccess && rc == HX_OK; ++k) {
        const int cur = k & 1;
        if (k + 1 < L.nboxes) {  // the next box's copy runs while this one is written
            e = copy_box(L.boxes[k + 1], S.p[cur ^ 1], st);
            if (e == cudaSuccess) e = cudaEventRecord(S.ev[cur ^ 1], st);
        }
        if (e == cudaSuccess) e = cudaEventSynchronize(S.ev[cur]);
        if (e != cudaSuccess) break;
        const hx_plotbox_f64& b = L.boxes[k];
        const size_t n = box_cells(b);
        offs[(size_t)k] = std::ftell(f);
        const std::string head = std::string("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))") +
                                 box_str(b.lo, b.hi) + " " + std::to_string(kComps) + "\n";
        if (std::fwrite(head.data(), 1, head.size(), f) != head.size() ||
            std::fwrite(S.p[cur], sizeof(double), kComps * n, f) != kComps * n) {
            rc = set_error(HX_ERR_ARG, "plotfile: short write");
            break;
        }
        for (int c = 0; c < kComps; ++c) {
            const double* v = S.p[cur] + c * n;
            double mn = v[0], mx = v[0];
            for (size_t i = 1; i < n; ++i) {
                mn = v[i] < mn ? v[i] : mn;
                mx = v[i] > mx ? v[i] : mx;
            }
            mins[(size_t)k * kComps + c] = mn;
            maxs[(size_t)k * kComps + c] = mx;
        }
    }
    std::fclose(f);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(st);
        return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc) {
        cudaStreamSynchronize(st);
        return rc;
    }
    std::string h = "1\n0\n" + std::to_string(kComps) + "\n0\n(" + std::to_string(L.nboxes) + " 0\n";
    for (int k = 0; k < L.nboxes; ++k) h += box_str(L.boxes[k].lo, L.boxes[k].hi) + "\n";
    h += ")\n" + std::to_string(L.nboxes) + "\n";
    for (int k = 0; k < L.nboxes; ++k) h += "FabOnDisk: Cell_D_00000 " + std::to_string(offs[(size_t)k]) + "\n";
    for (const std::vector<double>* mm : {&mins, &maxs}) {
        h += "\n" + std::to_string(L.nboxes) + "," + std::to_string(kComps) + "\n";
        for (int k = 0; k < L.nboxes; ++k) {
            for (int c = 0; c < kComps; ++c) h += real_str((*mm)[(size_t)k * kComps + c]) + ",";
            h += "\n";
        }
    }
    FILE* hf = std::fopen((dir + "/Cell_H").c_str(), "w");
    if (!hf) return set_error(HX_ERR_ARG, "plotfile: cannot create a FabArray header");
    const bool ok = std::fwrite(h.data(), 1, h.size(), hf) == h.size();
    std::fclose(hf);
    return ok ? HX_OK : set_error(HX_ERR_ARG, "plotfile: short write");
}

}  // namespace

extern "C" int hx_write_plotfile_f64(const char* prefix, int iteration, double time, int nlevels,
                                     const hx_plotlevel_f64* levels, const double prob_lo[2],
                                     const double prob_hi[2], hx_stream_t stream) {
    if (!prefix || !prob_lo || !prob_hi || iteration < 0) return set_error(HX_ERR_ARG, "plotfile: bad arguments");
    int rc = check_levels(nlevels, levels);
    if (rc) return rc;
    char num[16];
    std::snprintf(num, sizeof num, "%05d", iteration);  // amrex::Concatenate(prefix, iteration, 5)
    const std::string root = std::string(prefix) + num;
    if (!make_dir(root)) return set_error(HX_ERR_ARG, "plotfile: cannot create the plotfile directory");
    size_t most = 0;
    for (int l = 0; l < nlevels; ++l)
        for (int k = 0; k < levels[l].nboxes; ++k) most = std::max(most, box_cells(levels[l].boxes[k]));
    Staging S;
    cudaError_t e = S.init(most * kComps);
    if (e != cudaSuccess) return set_error(HX_ERR_CUDA, cudaGetErrorString(e));
    const cudaStream_t st = (cudaStream_t)stream;
    for (int l = 0; l < nlevels && rc == HX_OK; ++l) {
        const std::string ld = root + "/Level_" + std::to_string(l);
        if (!make_dir(ld)) return set_error(HX_ERR_ARG, "plotfile: cannot create a level directory");
        rc = write_level(ld, levels[l], S, st);
    }
    if (rc) return rc;
    // the plotfile header
    std::string h = "HyperCLaw-V1.1\n" + std::to_string(kComps) + "\n";
    for (int c = 0; c < kComps; ++c) h += std::string(kVarNames[c]) + "\n";
    h += "2\n" + real_str(time) + "\n" + std::to_string(nlevels - 1) + "\n";
    h += real_str(prob_lo[0]) + " " + real_str(prob_lo[1]) + " \n";
    h += real_str(prob_hi[0]) + " " + real_str(prob_hi[1]) + " \n";
    for (int l = 0; l + 1 < nlevels; ++l) h += std::to_string(levels[l].ref_ratio) + " ";
    h += "\n";
    for (int l = 0; l < nlevels; ++l) h += box_str(levels[l].domain_lo, levels[l].domain_hi) + " ";
    h += "\n";
    for (int l = 0; l < nlevels; ++l) h += std::to_string(levels[l].istep) + " ";
    h += "\n";
    for (int l = 0; l < nlevels; ++l) h += real_str(levels[l].dx) + " " + real_str(levels[l].dy) + " \n";
    h += "0\n0\n";  // Cartesian coordinates, no boundary width
    for (int l = 0; l < nlevels; ++l) {
        const hx_plotlevel_f64& L = levels[l];
        h += std::to_string(l) + " " + std::to_string(L.nboxes) + " " + real_str(time) + "\n";
        h += std::to_string(L.istep) + "\n";
        for (int k = 0; k < L.nboxes; ++k) {
            const hx_plotbox_f64& b = L.boxes[k];
            h += real_str(prob_lo[0] + b.lo[0] * L.dx) + " " + real_str(prob_lo[0] + (b.hi[0] + 1) * L.dx) + "\n";
            h += real_str(prob_lo[1] + b.lo[1] * L.dy) + " " + real_str(prob_lo[1] + (b.hi[1] + 1) * L.dy) + "\n";
        }
        h += "Level_" + std::to_string(l) + "/Cell\n";
    }
    FILE* f = std::fopen((root + "/Header").c_str(), "w");
    if (!f) return set_error(HX_ERR_ARG, "plotfile: cannot create the header");
    const bool ok = std::fwrite(h.data(), 1, h.size(), f) == h.size();
    std::fclose(f);
    return ok ? HX_OK : set_error(HX_ERR_ARG, "plotfile: short write");
}
