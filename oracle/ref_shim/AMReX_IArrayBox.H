// Host-only stand-in (nothing needed from it by the restriction kernel).
#pragma once
#include <AMReX_FArrayBox.H>
