#include <vector>
// Exports the reference's cell-local NODATA-aware restriction
// (include/utils/MaskedAverageDown.H:64-104), compiled verbatim from the
// reference tree through the host-only shim in ref_shim/, for pinning the
// oracle.  TEST INFRASTRUCTURE: built into oracle/_ref/ by oracle/build_ref.sh.
#include <utils/MaskedAverageDown.H>
#include "ref_names.h"

// fine: (nxf x nyf x ncomp) x-fastest, crse: (nxc x nyc x ncomp); all volumes fv.
extern "C" void HXREF_NAME(hxref_masked_avgdown)(int nxf, int nyf, int ncomp, const amrex::Real* fine, int rx, int ry,
                                                  amrex::Real fv, amrex::Real nodata, amrex::Real* crse) {
    const int nxc = nxf / rx, nyc = nyf / ry;
    std::vector<amrex::Real> vol((size_t)nxf * nyf, fv);
    amrex::Array4<amrex::Real const> f;
    f.p = fine; f.jstride = nxf; f.kstride = (long long)nxf * nyf; f.nstride = (long long)nxf * nyf;
    amrex::Array4<amrex::Real const> v;
    v.p = vol.data(); v.jstride = nxf; v.kstride = (long long)nxf * nyf; v.nstride = 0;
    amrex::Array4<amrex::Real> c;
    c.p = crse; c.jstride = nxc; c.kstride = (long long)nxc * nyc; c.nstride = (long long)nxc * nyc;
    amrex::IntVect r; r[0] = rx; r[1] = ry; r[2] = 1;
    for (int n = 0; n < ncomp; ++n)
        for (int j = 0; j < nyc; ++j)
            for (int i = 0; i < nxc; ++i) amrex::masked_avgdown_with_vol(i, j, 0, n, c, f, v, 0, 0, r, nodata);
}
