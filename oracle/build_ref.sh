#!/bin/sh
# Compiles the reference's header-only point kernels (Riemann solvers and the
# masked restriction) verbatim from the reference source tree, through the
# host-only AMReX shim in oracle/ref_shim/, into oracle/_ref/libhx_ref.so.
# Used only to pin the oracle and to generate the committed golden vectors;
# needs the reference tree (default /root/reference, or $HX_REFERENCE_ROOT).
# The rest of the reference (the AMReX-based drivers) needs AMReX, MPI and HDF5
# and is not buildable here.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${HX_REFERENCE_ROOT:-/root/reference}
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
echo "$OUT/libhx_ref.so"
