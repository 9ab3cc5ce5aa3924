// Minimal stand-in for the AMReX header of the same name, so that the
// reference's header-only point kernels compile on the host without AMReX.
// REAL_T selects the precision (the reference's DOUBLE/SINGLE build option).
#pragma once
#include <cmath>
#include <cstdlib>
#include <algorithm>
#ifndef HXREF_REAL_T
#define HXREF_REAL_T double
#endif
#define AMREX_SPACEDIM 2
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST_DEVICE
#define AMREX_FORCE_INLINE inline
namespace amrex { using Real = HXREF_REAL_T; }
