// Host-only stand-in providing the few AMReX types the reference's
// masked_avgdown_with_vol kernel touches: Array4 (strided 4-D view), IntVect,
// and forward declarations for the whole-MultiFab driver's signature.
#pragma once
#include <AMReX_REAL.H>
namespace amrex {
struct IntVect {
    int v[3] = {0, 0, 0};
    int operator[](int d) const { return v[d]; }
    int& operator[](int d) { return v[d]; }
};
template <class T> struct Array4 {
    T* p = nullptr;
    long long jstride = 0, kstride = 0, nstride = 0;
    int lo0 = 0, lo1 = 0, lo2 = 0;
    T& operator()(int i, int j, int k, int n) const {
        return p[(i - lo0) + (long long)(j - lo1) * jstride + (long long)(k - lo2) * kstride + (long long)n * nstride];
    }
    T& operator()(int i, int j, int k) const { return (*this)(i, j, k, 0); }
};
class MultiFab;
class Geometry;
}  // namespace amrex
