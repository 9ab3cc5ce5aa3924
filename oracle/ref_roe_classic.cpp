// Exports the reference's classic Roe point kernel
// (include/solvers/kernels/Roe.H:51-309), compiled verbatim from the reference
// tree through the host-only shim in ref_shim/, for pinning the oracle.
// TEST INFRASTRUCTURE: built into oracle/_ref/ by oracle/build_ref.sh.
#include <solvers/kernels/Roe.H>
#include "ref_names.h"

// in: n x 10 (hi hui hvi zi ni hj huj hvj zj nj); aux: n x 4 (dt dx nx ny)
extern "C" void HXREF_NAME(hxref_roe_classic)(long n, const amrex::Real* in, const amrex::Real* aux,
                                               amrex::Real* F, amrex::Real* Sm, amrex::Real* Sp) {
    for (long p = 0; p < n; ++p) {
        const amrex::Real* q = in + 10 * p;
        const amrex::Real* a = aux + 4 * p;
        amrex::Real f[3] = {}, sm[3] = {}, sp[3] = {};
        roeSolver(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], f, sm, sp, a[0], a[1], a[2], a[3]);
        for (int c = 0; c < 3; ++c) { F[3 * p + c] = f[c]; Sm[3 * p + c] = sm[c]; Sp[3 * p + c] = sp[c]; }
    }
}
