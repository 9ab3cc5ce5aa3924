// Host-only stand-in: qualifier macros only.
#pragma once
#include <AMReX_REAL.H>
