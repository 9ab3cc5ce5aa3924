#!/bin/sh
# Compiles parts of the reference verbatim from the reference source tree,
# through the host-only AMReX stand-in in oracle/ref_shim/, into oracle/_ref/:
#  - libhx_ref.so: the header-only point kernels (Riemann solvers, the masked
#    restriction), FP64 and FP32;
#  - libhx_ref_level_{f64,f32}.so and libhx_ref_level_fabs_{f64,f32}.so: the
#    per-box solver drivers src/solvers/HydrostaticRoe.cpp and
#    src/solvers/Roe.cpp with SolverVariant and BCFill.H, driven by
#    ref_level.cpp at one level.  The vanLeerLimiter's unqualified abs()
#    (HydrostaticRoe.cpp:176) binds to C's int abs(int) with these headers;
#    the _fabs libraries are the same sources with <math.h> included first,
#    which binds it to the floating abs (what device code and any build whose
#    headers pull in <math.h> get).  Linked -Bsymbolic, so each library keeps
#    its own copies of the reference's functions.
# Used only to pin the oracle and to generate the committed golden vectors;
# needs the reference tree (default /root/reference, or $HX_REFERENCE_ROOT).
# The rest of the reference (AMR hierarchy, I/O) needs AMReX, MPI and HDF5 and
# is not built.
# "build_ref.sh --root" prints the reference tree it would use and exits 0, or
# exits 1 without output when there is none (the other tools ask it, so this
# recipe is the one place that knows where the tree lives).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${HX_REFERENCE_ROOT:-/root/reference}
if [ "$1" = "--root" ]; then
  [ -d "$REF/include/solvers/kernels" ] || exit 1
  echo "$REF"
  exit 0
fi
[ -d "$REF/include/solvers/kernels" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-O2 -ffp-contract=off -fPIC -std=c++20 -I$HERE/ref_shim -I$REF/include -I$HERE"
objs=""
for src in ref_roe_hydrostatic ref_roe_classic ref_masked_avgdown; do
  $CXX $FLAGS -c "$HERE/$src.cpp" -o "$OUT/${src}_f64.o"
  $CXX $FLAGS -DHXREF_SINGLE -DHXREF_REAL_T=float -c "$HERE/$src.cpp" -o "$OUT/${src}_f32.o"
  objs="$objs $OUT/${src}_f64.o $OUT/${src}_f32.o"
done
$CXX -shared -o "$OUT/libhx_ref.so" $objs
# the per-box drivers: (abs binding) x (precision), each its own library
for abs in int fabs; do
  for prec in f64 f32; do
    extra=""
    [ "$abs" = fabs ] && extra="-include math.h"
    [ "$prec" = f32 ] && extra="$extra -DHXREF_SINGLE -DHXREF_REAL_T=float"
    tag="${abs}_${prec}"
    lobjs=""
    for src in "$REF/src/solvers/HydrostaticRoe.cpp" "$REF/src/solvers/Roe.cpp" "$HERE/ref_level.cpp"; do
      o="$OUT/$(basename "$src" .cpp)_${tag}.o"
      $CXX $FLAGS $extra -c "$src" -o "$o" &
      lobjs="$lobjs $o"
    done
    wait
    name=libhx_ref_level_${prec}.so
    [ "$abs" = fabs ] && name=libhx_ref_level_fabs_${prec}.so
    $CXX -shared -Wl,-Bsymbolic -o "$OUT/$name" $lobjs
  done
done
echo "$OUT/libhx_ref.so"
