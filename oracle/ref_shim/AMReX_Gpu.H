// Host-only stand-in: every AMReX name the reference drivers use is in hx_amrex_shim.H.
#pragma once
#include "hx_amrex_shim.H"
