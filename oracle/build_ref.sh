#!/bin/sh
# Compiles the reference's own Kronecker matvec, src/expv/source/hamvec_func3.cpp,
# straight from the read-only reference tree into oracle/_ref/libref_hamvec.so,
# with oracle/ref_shim/mkl.h standing in for MKL's cblas_zcopy/zaxpy/zgemm.
# TEST INFRASTRUCTURE ONLY (a pin for the matvec).  Nothing else in the
# reference builds here: its Krylov drivers and Expokit are Fortran (no
# gfortran) and the C++ layers need armadillo, boost and MPI.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${OOPS_REFERENCE_ROOT:-/root/reference}
SRC="$REF/src/expv/source/hamvec_func3.cpp"
if [ ! -f "$SRC" ]; then
  echo "build_ref.sh: $SRC not present; skipping the reference matvec" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -O2 -fPIC -ffp-contract=off -shared -w -I"$HERE/ref_shim" -o "$HERE/_ref/libref_hamvec.so" "$SRC"
echo "built $HERE/_ref/libref_hamvec.so"
