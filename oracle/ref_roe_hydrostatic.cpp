// Exports the reference's homogeneous Roe point kernel
// (include/solvers/kernels/HydrostaticRoe.H:44-159), compiled verbatim from the
// reference tree through the host-only shim in ref_shim/, for pinning the
// oracle.  TEST INFRASTRUCTURE: built into oracle/_ref/ by oracle/build_ref.sh.
#include <solvers/kernels/HydrostaticRoe.H>
#include "ref_names.h"

extern "C" void HXREF_NAME(hxref_roe_hydrostatic)(long n, const amrex::Real* in, const amrex::Real* nrm,
                                                   amrex::Real* F) {
    for (long p = 0; p < n; ++p) {
        const amrex::Real* q = in + 6 * p;
        amrex::Real f[3] = {};
        roeSolver(q[0], q[1], q[2], q[3], q[4], q[5], f, amrex::Real(0), amrex::Real(1), nrm[2 * p],
                  nrm[2 * p + 1]);
        F[3 * p] = f[0]; F[3 * p + 1] = f[1]; F[3 * p + 2] = f[2];
    }
}
