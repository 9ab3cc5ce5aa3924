// Host-only stand-in: the reference kernels need only the qualifier macros.
#pragma once
#include <AMReX_REAL.H>
