#!/bin/sh
# TEST INFRASTRUCTURE ONLY: compiles parity pins from the reference's own
# sources, read in place from the reference tree named by OOPS_REFERENCE_ROOT
# (nothing is built when it is unset or absent), into oracle/_ref/:
#   libref_hamvec.so  the Kronecker matvec, src/expv/source/hamvec_func3.cpp,
#                     with oracle/ref_shim/mkl.h for MKL's cblas_zcopy/zaxpy/zgemm;
#   ref_pin           the spin, cluster and physics sources (Spin.cpp,
#                     SpinData.cpp, misc.cpp, lattice.cpp, SpinSource.cpp,
#                     SpinCollection.cpp, SpinClusterIndex.cpp,
#                     SpinClusterAlgorithm.cpp, SpinCluster.cpp) linked with
#                     oracle/ref_pin.cpp, with oracle/ref_shim/armadillo;
#   ref_cce_pin       the CCE reduction, src/source/app/cce.cpp (with the same
#                     spin and cluster sources), linked with
#                     oracle/ref_cce_pin.cpp; oracle/ref_shim/include/app/cce.h
#                     stands in for the application header (no boost, MPI or
#                     application class tree).
# The Krylov drivers and Expokit are Fortran (no gfortran here) and the rest
# of the application layer needs boost, MPI and its class tree, so it is not
# built.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${OOPS_REFERENCE_ROOT:-}
if [ -z "$REF" ] || [ ! -d "$REF/src" ]; then
  echo "build_ref.sh: OOPS_REFERENCE_ROOT does not name a reference tree; skipping the pins" >&2
  exit 0
fi
S="$REF/src"
mkdir -p "$HERE/_ref"
${CXX:-g++} -O2 -fPIC -ffp-contract=off -shared -w -I"$HERE/ref_shim" -o "$HERE/_ref/libref_hamvec.so" \
  "$S/expv/source/hamvec_func3.cpp"
${CXX:-g++} -O2 -std=c++14 -ffp-contract=off -w -I"$HERE/ref_shim" -I"$S" -o "$HERE/_ref/ref_pin" \
  "$HERE/ref_pin.cpp" \
  "$S/source/spin/Spin/Spin.cpp" "$S/source/spin/Spin/SpinData.cpp" \
  "$S/source/misc/misc.cpp" "$S/source/misc/lattice.cpp" \
  "$S/source/spin/SpinCollection/SpinSource.cpp" "$S/source/spin/SpinCollection/SpinCollection.cpp" \
  "$S/source/spin/SpinCluster/SpinClusterIndex.cpp" "$S/source/spin/SpinCluster/SpinClusterAlgorithm.cpp" \
  "$S/source/spin/SpinCluster/SpinCluster.cpp"
${CXX:-g++} -O2 -std=c++14 -ffp-contract=off -w -I"$HERE/ref_shim" -I"$S" -o "$HERE/_ref/ref_cce_pin" \
  "$HERE/ref_cce_pin.cpp" "$S/source/app/cce.cpp" \
  "$S/source/spin/Spin/Spin.cpp" "$S/source/spin/Spin/SpinData.cpp" \
  "$S/source/misc/misc.cpp" "$S/source/misc/lattice.cpp" \
  "$S/source/spin/SpinCollection/SpinSource.cpp" "$S/source/spin/SpinCollection/SpinCollection.cpp" \
  "$S/source/spin/SpinCluster/SpinClusterIndex.cpp" "$S/source/spin/SpinCluster/SpinClusterAlgorithm.cpp" \
  "$S/source/spin/SpinCluster/SpinCluster.cpp"
echo "built $HERE/_ref/libref_hamvec.so, $HERE/_ref/ref_pin and $HERE/_ref/ref_cce_pin"
