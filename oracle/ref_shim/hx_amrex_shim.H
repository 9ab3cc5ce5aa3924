// Host-only, single-process stand-in for the parts of AMReX that the
// reference's per-box solver drivers use (src/solvers/HydrostaticRoe.cpp,
// src/solvers/Roe.cpp, include/boundaries/BCFill.H, include/solvers/*.H,
// include/utils/Logging.H), so that those files compile verbatim on the host.
// TEST INFRASTRUCTURE: built by oracle/build_ref.sh into oracle/_ref/ only.
//
// AMReX itself is a third-party dependency that the reference does not vendor
// (tpl/amrex is an empty submodule with no pinned commit).  What is restated
// here is AMReX's documented behaviour on one box, one rank, no tiling, no
// GPU: Box / BoxArray index arithmetic, FabArray storage with ghost cells,
// MFIter over the boxes, ParallelFor as the loop k, j, i (i fastest),
// ReduceOps as a sequential fold, MultiFab::LinComb as a*x + b*y per element,
// and FilccCell's per-direction ghost rules (foextrap copies the edge cell,
// reflect_even mirrors, reflect_odd mirrors with a sign change; the BCRec of
// destination component n is bcr[bcomp + n - dcomp]; x is applied before y).
// Only what those files need exists; parallel communication is the identity.
#pragma once

#include <AMReX_REAL.H>

#include <array>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#define AMREX_D_DECL(a, b, c) a, b
#define AMREX_ASSERT(x) ((void)0)
#define AMREX_ASSERT_WITH_MESSAGE(x, msg) ((void)0)
#define AMREX_ALWAYS_ASSERT(x) \
    do { if (!(x)) throw std::runtime_error("assertion failed: " #x); } while (0)
#define AMREX_ALWAYS_ASSERT_WITH_MESSAGE(x, msg) \
    do { if (!(x)) throw std::runtime_error(msg); } while (0)
#define BL_PROFILE(x) ((void)0)
#define BL_ASSERT(x) ((void)0)
#define AMREX_GPU_HOST
#define AMREX_PRAGMA_SIMD

namespace amrex {

using Long = long long;
template <class T> using Vector = std::vector<T>;
template <class T, std::size_t N> using Array = std::array<T, N>;
template <class T, std::size_t N> using GpuArray = std::array<T, N>;

[[noreturn]] inline void Abort(const std::string& msg) { throw std::runtime_error(msg); }
[[noreturn]] inline void Error(const std::string& msg) { throw std::runtime_error(msg); }

inline std::ostream& OutStream() { return std::cout; }
inline std::ostream& ErrorStream() { return std::cerr; }
struct Print {
    template <class T> Print& operator<<(const T& v) { std::cout << v; return *this; }
};

namespace ParallelContext {
inline bool IOProcessorSub() { return true; }
}
namespace ParallelDescriptor {
inline bool IOProcessor() { return true; }
template <class T> inline void ReduceRealMin(T*, int) {}
template <class T> inline void ReduceRealMin(T&) {}
template <class T> inline void ReduceRealMax(T*, int) {}
}  // namespace ParallelDescriptor

// Inputs-file parameters: none are set, so every query reports "absent".
class ParmParse {
public:
    explicit ParmParse(const std::string& = std::string()) {}
    template <class T> bool query(const char*, T&) const { return false; }
};

// ---------------------------------------------------------------- index space
struct Dim3 {
    int x, y, z;
};

struct IntVect {
    int v[3] = {0, 0, 0};
    IntVect() = default;
    IntVect(int i, int j) : v{i, j, 0} {}
    IntVect(int i, int j, int k) : v{i, j, k} {}
    int operator[](int d) const { return v[d]; }
    int& operator[](int d) { return v[d]; }
    bool allLE(const IntVect& o) const { return v[0] <= o[0] && v[1] <= o[1]; }
    static IntVect TheZeroVector() { return IntVect(0, 0); }
    static IntVect TheUnitVector() { return IntVect(1, 1); }
    static IntVect TheDimensionVector(int d) { IntVect r; r[d] = 1; return r; }
};

// Cell (false) or node (true) centring per direction.
struct IndexType {
    bool node[2] = {false, false};
    IndexType() = default;
    explicit IndexType(const IntVect& t) : node{t[0] != 0, t[1] != 0} {}
    bool nodeCentered(int d) const { return node[d]; }
    bool operator==(const IndexType& o) const { return node[0] == o.node[0] && node[1] == o.node[1]; }
};

class Box {
public:
    IntVect lo, hi;
    IndexType typ;
    Box() : lo(0, 0), hi(-1, -1) {}
    Box(const IntVect& l, const IntVect& h, IndexType t = IndexType()) : lo(l), hi(h), typ(t) {}
    const IntVect& smallEnd() const { return lo; }
    const IntVect& bigEnd() const { return hi; }
    int smallEnd(int d) const { return lo[d]; }
    int bigEnd(int d) const { return hi[d]; }
    int length(int d) const { return hi[d] - lo[d] + 1; }
    bool ok() const { return hi[0] >= lo[0] && hi[1] >= lo[1]; }
    IndexType ixType() const { return typ; }
    Box& grow(int d, int n) { lo[d] -= n; hi[d] += n; return *this; }
    Box& grow(int n) { return grow(0, n).grow(1, n); }
    Box& grow(const IntVect& n) { return grow(0, n[0]).grow(1, n[1]); }
    // cell -> node in direction d: one more index at the high end
    Box& surroundingNodes(int d) {
        if (!typ.node[d]) { hi[d] += 1; typ.node[d] = true; }
        return *this;
    }
    bool contains(const IntVect& p) const {
        return p[0] >= lo[0] && p[0] <= hi[0] && p[1] >= lo[1] && p[1] <= hi[1];
    }
    bool contains(const Box& b) const { return contains(b.lo) && contains(b.hi); }
};

inline Box grow(const Box& b, int n) { Box r = b; return r.grow(n); }
inline Box grow(const Box& b, const IntVect& n) { Box r = b; return r.grow(n); }
inline Box surroundingNodes(const Box& b, int d) { Box r = b; return r.surroundingNodes(d); }
inline Box convert(const Box& b, IndexType t) {
    Box r = b;
    for (int d = 0; d < 2; ++d) {
        if (t.node[d] && !r.typ.node[d]) r.surroundingNodes(d);
        else if (!t.node[d] && r.typ.node[d]) { r.hi[d] -= 1; r.typ.node[d] = false; }
    }
    return r;
}

class BoxArray {
public:
    std::vector<Box> boxes;
    BoxArray() = default;
    explicit BoxArray(const Box& b) : boxes{b} {}
    int size() const { return (int)boxes.size(); }
    const Box& operator[](int i) const { return boxes[i]; }
    IndexType ixType() const { return boxes.empty() ? IndexType() : boxes[0].typ; }
    BoxArray& surroundingNodes(int d) {
        for (auto& b : boxes) b.surroundingNodes(d);
        return *this;
    }
};
inline BoxArray convert(const BoxArray& ba, const IntVect& t) {
    BoxArray r = ba;
    for (auto& b : r.boxes) b = convert(b, IndexType(t));
    return r;
}

struct DistributionMapping {};
struct Periodicity {};

class Geometry {
public:
    Box dom;
    Real dx[2] = {Real(1), Real(1)};
    Geometry() = default;
    Geometry(const Box& d, Real cx, Real cy) : dom(d), dx{cx, cy} {}
    Real CellSize(int d) const { return dx[d]; }
    GpuArray<Real, 2> CellSizeArray() const { return {dx[0], dx[1]}; }
    const Box& Domain() const { return dom; }
    bool isAllPeriodic() const { return false; }
    bool isPeriodic(int) const { return false; }
    Periodicity periodicity() const { return {}; }
};

// ------------------------------------------------------------------ storage
template <class T> struct Array4 {
    T* p = nullptr;
    Long jstride = 0, kstride = 0, nstride = 0;
    Dim3 begin{0, 0, 0}, end{1, 1, 1};
    int ncomp = 0;
    Array4() = default;
    Array4(T* ptr, Dim3 lo, Dim3 hi_plus_one, int nc)
        : p(ptr), jstride(hi_plus_one.x - lo.x), kstride(jstride * (hi_plus_one.y - lo.y)),
          nstride(kstride * (hi_plus_one.z - lo.z)), begin(lo), end(hi_plus_one), ncomp(nc) {}
    template <class U, class = std::enable_if_t<std::is_same_v<const U, T> && !std::is_same_v<U, T>>>
    Array4(const Array4<U>& o)
        : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride), begin(o.begin), end(o.end),
          ncomp(o.ncomp) {}
    T& operator()(int i, int j, int k, int n) const {
        return p[(i - begin.x) + (Long)(j - begin.y) * jstride + (Long)(k - begin.z) * kstride + (Long)n * nstride];
    }
    T& operator()(int i, int j, int k) const { return (*this)(i, j, k, 0); }
};

// One box of ncomp components with its ghost ring (box = valid box grown).
template <class T> class BaseFab {
public:
    Box bx;
    int nc = 0;
    std::vector<T> data;
    BaseFab() = default;
    BaseFab(const Box& b, int ncomp) : bx(b), nc(ncomp), data((size_t)b.length(0) * b.length(1) * ncomp, T(0)) {}
    const Box& box() const { return bx; }
    int nComp() const { return nc; }
    Array4<T> array() { return Array4<T>(data.data(), lo3(), hi3(), nc); }
    Array4<T const> array() const { return Array4<T const>(data.data(), lo3(), hi3(), nc); }
    Array4<T const> const_array() const { return array(); }
    void setVal(T v) { std::fill(data.begin(), data.end(), v); }

private:
    Dim3 lo3() const { return {bx.lo[0], bx.lo[1], 0}; }
    Dim3 hi3() const { return {bx.hi[0] + 1, bx.hi[1] + 1, 1}; }
};
using FArrayBox = BaseFab<Real>;
using IArrayBox = BaseFab<int>;

class TagBox : public BaseFab<char> {
public:
    enum TagVal { CLEAR = 0, BUF = 1, SET = 2 };
    using BaseFab<char>::BaseFab;
};

class MFIter;

class FabArrayBase {
public:
    BoxArray ba;
    DistributionMapping dm;
    int nc = 0;
    IntVect ng;
    const BoxArray& boxArray() const { return ba; }
    const DistributionMapping& DistributionMap() const { return dm; }
    int nComp() const { return nc; }
    int nGrow() const { return ng[0]; }
    IntVect nGrowVect() const { return ng; }
    int size() const { return ba.size(); }
};

template <class FAB> class FabArray : public FabArrayBase {
public:
    using value_type = typename std::remove_reference_t<decltype(std::declval<FAB>().data[0])>;
    std::vector<FAB> fabs;
    FabArray() = default;
    FabArray(const BoxArray& b, const DistributionMapping& d, int ncomp, int ngrow) { define(b, d, ncomp, ngrow); }
    FabArray(const BoxArray& b, const DistributionMapping& d, int ncomp, const IntVect& ngrow) {
        define(b, d, ncomp, ngrow);
    }
    void define(const BoxArray& b, const DistributionMapping& d, int ncomp, int ngrow) {
        define(b, d, ncomp, IntVect(ngrow, ngrow));
    }
    void define(const BoxArray& b, const DistributionMapping& d, int ncomp, const IntVect& ngrow) {
        ba = b; dm = d; nc = ncomp; ng = ngrow;
        fabs.clear();
        for (const Box& x : b.boxes) fabs.emplace_back(amrex::grow(x, ngrow), ncomp);
    }
    void clear() { fabs.clear(); ba = BoxArray(); nc = 0; }
    bool ok() const { return !fabs.empty(); }
    FAB& operator[](const MFIter& m);
    const FAB& operator[](const MFIter& m) const;
    FAB& operator[](int i) { return fabs[i]; }
    const FAB& operator[](int i) const { return fabs[i]; }
    auto array(const MFIter& m);
    auto array(const MFIter& m) const;
    auto const_array(const MFIter& m) const;
    void setVal(value_type v) { for (auto& f : fabs) f.setVal(v); }
    void FillBoundary(const Periodicity& = Periodicity()) {}  // one box, no periodic directions: nothing to exchange
};

class MultiFab : public FabArray<FArrayBox> {
public:
    using FabArray<FArrayBox>::FabArray;
    // dst(dstcomp + n) = a * x(xcomp + n) + b * y(ycomp + n) over each valid box grown by nghost
    static void LinComb(MultiFab& dst, Real a, const MultiFab& x, int xcomp, Real b, const MultiFab& y, int ycomp,
                        int dstcomp, int ncomp, int nghost);
};
using iMultiFab = FabArray<IArrayBox>;

class TagBoxArray : public FabArray<TagBox> {
public:
    TagBoxArray() = default;
    TagBoxArray(const BoxArray& b, const DistributionMapping& d, int ngrow = 0) { define(b, d, 1, ngrow); }
};

// Iterates the boxes of a FabArray, one tile per box (no tiling).
class MFIter {
public:
    const FabArrayBase* fa;
    int idx = 0;
    explicit MFIter(const FabArrayBase& f, bool /*tiling*/ = false) : fa(&f) {}
    bool isValid() const { return idx < fa->size(); }
    MFIter& operator++() { ++idx; return *this; }
    int index() const { return idx; }
    Box validbox() const { return fa->ba[idx]; }
    Box tilebox() const { return validbox(); }
    Box growntilebox() const { return amrex::grow(validbox(), fa->ng); }
    Box growntilebox(int n) const { return amrex::grow(validbox(), n); }
    Box nodaltilebox(int d) const { return amrex::convert(tilebox(), IndexType(IntVect::TheDimensionVector(d))); }
    Box fabbox() const { return growntilebox(); }
};
inline bool TilingIfNotGPU() { return false; }

template <class FAB> FAB& FabArray<FAB>::operator[](const MFIter& m) { return fabs[m.index()]; }
template <class FAB> const FAB& FabArray<FAB>::operator[](const MFIter& m) const { return fabs[m.index()]; }
template <class FAB> auto FabArray<FAB>::array(const MFIter& m) { return fabs[m.index()].array(); }
template <class FAB> auto FabArray<FAB>::array(const MFIter& m) const { return fabs[m.index()].const_array(); }
template <class FAB> auto FabArray<FAB>::const_array(const MFIter& m) const { return fabs[m.index()].const_array(); }

// ------------------------------------------------------------------- loops
template <class F> void ParallelFor(const Box& b, F&& f) {
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
        for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, 0);
}

inline void MultiFab::LinComb(MultiFab& dst, Real a, const MultiFab& x, int xcomp, Real b, const MultiFab& y,
                              int ycomp, int dstcomp, int ncomp, int nghost) {
    for (MFIter mfi(dst); mfi.isValid(); ++mfi) {
        const Box bx = mfi.growntilebox(nghost);
        auto d = dst.array(mfi);
        auto xa = x.const_array(mfi);
        auto ya = y.const_array(mfi);
        for (int n = 0; n < ncomp; ++n)
            ParallelFor(bx, [&](int i, int j, int k) {
                d(i, j, k, dstcomp + n) = a * xa(i, j, k, xcomp + n) + b * ya(i, j, k, ycomp + n);
            });
    }
}

// ReduceOps<ReduceOpMin, ReduceOpMax> / ReduceData<Real, Real>: a sequential
// fold from the identity of each operation.
struct ReduceOpMin {
    template <class T> static T init() { return std::numeric_limits<T>::max(); }
    template <class T> static void update(T& d, const T& s) { d = (s < d) ? s : d; }
};
struct ReduceOpMax {
    template <class T> static T init() { return std::numeric_limits<T>::lowest(); }
    template <class T> static void update(T& d, const T& s) { d = (d < s) ? s : d; }
};
template <class... Ts> using GpuTuple = std::tuple<Ts...>;
template <std::size_t I, class... Ts> auto get(const std::tuple<Ts...>& t) { return std::get<I>(t); }

template <class... Ops> class ReduceOps;
template <class... Ts> class ReduceData {
public:
    using Type = GpuTuple<Ts...>;
    Type acc;
    template <class R> explicit ReduceData(R&) { acc = R::template identity<Ts...>(); }
    Type value() const { return acc; }
};
template <class... Ops> class ReduceOps {
public:
    template <class... Ts> static GpuTuple<Ts...> identity() { return GpuTuple<Ts...>(Ops::template init<Ts>()...); }
    template <class D, class F> void eval(const Box& b, D& d, F&& f) {
        ParallelFor(b, [&](int i, int j, int k) { fold(d.acc, f(i, j, k), std::index_sequence_for<Ops...>{}); });
    }

private:
    template <class Tup, std::size_t... I> static void fold(Tup& acc, const Tup& v, std::index_sequence<I...>) {
        (Ops::update(std::get<I>(acc), std::get<I>(v)), ...);
    }
};

// -------------------------------------------------------------- boundaries
namespace BCType {
enum : int { bogus = -666, reflect_odd = -1, int_dir = 0, reflect_even = 1, foextrap = 2, ext_dir = 3, hoextrap = 4 };
}

class BCRec {
public:
    int lo_[2] = {BCType::bogus, BCType::bogus}, hi_[2] = {BCType::bogus, BCType::bogus};
    void setLo(int d, int v) { lo_[d] = v; }
    void setHi(int d, int v) { hi_[d] = v; }
    int lo(int d) const { return lo_[d]; }
    int hi(int d) const { return hi_[d]; }
};

namespace Gpu {
template <class T> using DeviceVector = std::vector<T>;
struct HostToDevice {};
constexpr HostToDevice hostToDevice{};
template <class It, class Out> void copy(HostToDevice, It first, It last, Out dst) { std::copy(first, last, dst); }
inline bool notInLaunchRegion() { return true; }
}  // namespace Gpu

// The ghost rules of one cell outside the domain: for each destination
// component n, BCRec bcr[bcomp + n - dcomp]; the x rule, then the y rule, each
// reading the cell it copies from at the state it has when the rule runs.
struct FilccCell {
    void operator()(const IntVect& iv, Array4<Real> const& q, int dcomp, int numcomp, Box const& domain,
                    const BCRec* bcr, int bcomp) const {
        const int i = iv[0], j = iv[1], k = 0;
        const int ilo = domain.lo[0], ihi = domain.hi[0], jlo = domain.lo[1], jhi = domain.hi[1];
        for (int n = dcomp; n < dcomp + numcomp; ++n) {
            const BCRec& bc = bcr[bcomp + n - dcomp];
            if (i < ilo) side(q, bc.lo(0), i, j, k, n, ilo, 2 * ilo - i - 1, j, j);
            else if (i > ihi) side(q, bc.hi(0), i, j, k, n, ihi, 2 * ihi - i + 1, j, j);
            if (j < jlo) side(q, bc.lo(1), i, j, k, n, i, i, jlo, 2 * jlo - j - 1, true);
            else if (j > jhi) side(q, bc.hi(1), i, j, k, n, i, i, jhi, 2 * jhi - j + 1, true);
        }
    }

private:
    // x rules read (edge, j) / (mirror, j); y rules read (i, edge) / (i, mirror)
    static void side(Array4<Real> const& q, int type, int i, int j, int k, int n, int ex, int mx, int ey, int my,
                     bool ydir = false) {
        const int ei = ydir ? i : ex, ej = ydir ? ey : j;
        const int mi = ydir ? i : mx, mj = ydir ? my : j;
        switch (type) {
            case BCType::foextrap: q(i, j, k, n) = q(ei, ej, k, n); break;
            case BCType::reflect_even: q(i, j, k, n) = q(mi, mj, k, n); break;
            case BCType::reflect_odd: q(i, j, k, n) = -q(mi, mj, k, n); break;
            default:
                throw std::runtime_error("FilccCell: boundary type not supported by the host stand-in");
        }
    }
};

// --------------------------------------------------------- flux registers
// Records what the solver hands over (the face fluxes and the scale), so a
// harness can compare them; AMReX's register arithmetic is not restated.
class FluxRegister {
public:
    enum FrOp { COPY = 0, ADD = 1 };
    MultiFab crse[2], fine[2];
    Real crse_scale[2] = {0, 0}, fine_scale[2] = {0, 0};
    int crse_calls = 0, fine_calls = 0;
    void setVal(Real) {}
    void CrseInit(const MultiFab& mf, int dir, int srccomp, int destcomp, int numcomp, Real mult, FrOp = COPY) {
        (void)srccomp; (void)destcomp; (void)numcomp;
        crse[dir] = mf;
        crse_scale[dir] = mult;
        ++crse_calls;
    }
    void FineAdd(const MultiFab& mf, int dir, int srccomp, int destcomp, int numcomp, Real mult) {
        (void)srccomp; (void)destcomp; (void)numcomp;
        fine[dir] = mf;
        fine_scale[dir] = mult;
        ++fine_calls;
    }
};

}  // namespace amrex
