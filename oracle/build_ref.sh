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
#                     application class tree);
#   ref_ensemble_pin  the whole ensemble-CCE application path: ensemble_cce.cpp,
#                     cce.cpp, DefectCenter.cpp, the quantum operator, state and
#                     evolution classes, KronProd/spkron, MatExp and the spin
#                     sources, linked with oracle/ref_ensemble_pin.cpp; the
#                     stand-ins of oracle/ref_shim replace armadillo, boost's
#                     variables_map, MPI, logging and MATLAB's mat.h, and
#                     expokit's Fortran ZGPADM is the oracle's C restatement
#                     (oracle.c, orc_padm);
#   ref_expv_pin      the same sources with oracle/ref_expv_pin.cpp: what the
#                     reference's MatExpVector hands main_mkl_ for a cluster's
#                     NV-conditional Hamiltonian (the drop-in's arguments);
#   ref_single_pin    the same sources and single_sample_cce.cpp with
#                     oracle/ref_single_pin.cpp: whole single-sample CCE runs;
#   ref_export_pin    ref_ensemble_pin with cce.cpp compiled with HAS_MATLAB:
#                     the reference's CCE::export_mat_file runs into the
#                     recording stand-in of oracle/ref_shim/mat.h (the result
#                     file's variables).
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
  "$S/source/quantum/QuantumState/QuantumState.cpp" "$S/source/quantum/QuantumState/PureState.cpp" \
  "$S/source/spin/Spin/Spin.cpp" "$S/source/spin/Spin/SpinData.cpp" \
  "$S/source/misc/misc.cpp" "$S/source/misc/lattice.cpp" \
  "$S/source/spin/SpinCollection/SpinSource.cpp" "$S/source/spin/SpinCollection/SpinCollection.cpp" \
  "$S/source/spin/SpinCluster/SpinClusterIndex.cpp" "$S/source/spin/SpinCluster/SpinClusterAlgorithm.cpp" \
  "$S/source/spin/SpinCluster/SpinCluster.cpp"
${CC:-gcc} -O2 -std=c99 -ffp-contract=off -c "$HERE/oracle.c" -o "$HERE/_ref/oracle_pin.o"
${CXX:-g++} -O2 -std=c++14 -ffp-contract=off -w -I"$HERE/ref_shim" -I"$HERE" -I"$S" -o "$HERE/_ref/ref_ensemble_pin" \
  "$HERE/ref_ensemble_pin.cpp" "$S/source/app/ensemble_cce.cpp" "$S/source/app/cce.cpp" \
  "$S/source/app/DefectCenter.cpp" \
  "$S/source/quantum/QuantumEvolution/QuantumEvolution.cpp" \
  "$S/source/quantum/QuantumEvolution/QuantumEvolutionAlgorithm.cpp" \
  "$S/source/quantum/QuantumOperator/QuantumOperator.cpp" \
  "$S/source/quantum/QuantumOperator/HilbertSpaceOperator.cpp" \
  "$S/source/quantum/QuantumOperator/LiouvilleSpaceOperator.cpp" \
  "$S/source/quantum/QuantumState/QuantumState.cpp" "$S/source/quantum/QuantumState/PureState.cpp" \
  "$S/source/quantum/QuantumState/MixedState.cpp" \
  "$S/source/spin/SpinInteraction/SpinInteraction.cpp" \
  "$S/source/spin/SpinInteraction/SpinInteractionComponent.cpp" \
  "$S/source/spin/SpinInteraction/SpinState.cpp" \
  "$S/source/kron/KronProd.cpp" "$S/source/kron/spkron.cpp" "$S/source/math/MatExp.cpp" \
  "$S/source/spin/Spin/Spin.cpp" "$S/source/spin/Spin/SpinData.cpp" \
  "$S/source/misc/misc.cpp" "$S/source/misc/lattice.cpp" \
  "$S/source/spin/SpinCollection/SpinSource.cpp" "$S/source/spin/SpinCollection/SpinCollection.cpp" \
  "$S/source/spin/SpinCluster/SpinClusterIndex.cpp" "$S/source/spin/SpinCluster/SpinClusterAlgorithm.cpp" \
  "$S/source/spin/SpinCluster/SpinCluster.cpp" "$HERE/_ref/oracle_pin.o" -lm
APP_BASE="$S/source/app/ensemble_cce.cpp $S/source/app/DefectCenter.cpp
  $S/source/quantum/QuantumEvolution/QuantumEvolution.cpp $S/source/quantum/QuantumEvolution/QuantumEvolutionAlgorithm.cpp
  $S/source/quantum/QuantumOperator/QuantumOperator.cpp $S/source/quantum/QuantumOperator/HilbertSpaceOperator.cpp
  $S/source/quantum/QuantumOperator/LiouvilleSpaceOperator.cpp
  $S/source/quantum/QuantumState/QuantumState.cpp $S/source/quantum/QuantumState/PureState.cpp
  $S/source/quantum/QuantumState/MixedState.cpp
  $S/source/spin/SpinInteraction/SpinInteraction.cpp $S/source/spin/SpinInteraction/SpinInteractionComponent.cpp
  $S/source/spin/SpinInteraction/SpinState.cpp
  $S/source/kron/KronProd.cpp $S/source/kron/spkron.cpp $S/source/math/MatExp.cpp
  $S/source/spin/Spin/Spin.cpp $S/source/spin/Spin/SpinData.cpp $S/source/misc/misc.cpp $S/source/misc/lattice.cpp
  $S/source/spin/SpinCollection/SpinSource.cpp $S/source/spin/SpinCollection/SpinCollection.cpp
  $S/source/spin/SpinCluster/SpinClusterIndex.cpp $S/source/spin/SpinCluster/SpinClusterAlgorithm.cpp
  $S/source/spin/SpinCluster/SpinCluster.cpp"
APP_SRCS="$S/source/app/cce.cpp $APP_BASE"
# shellcheck disable=SC2086
${CXX:-g++} -O2 -std=c++14 -ffp-contract=off -w -I"$HERE/ref_shim" -I"$HERE" -I"$S" -o "$HERE/_ref/ref_expv_pin" \
  "$HERE/ref_expv_pin.cpp" $APP_SRCS -lm
# shellcheck disable=SC2086
${CXX:-g++} -O2 -std=c++14 -ffp-contract=off -w -I"$HERE/ref_shim" -I"$HERE" -I"$S" -o "$HERE/_ref/ref_single_pin" \
  "$HERE/ref_single_pin.cpp" "$S/source/app/single_sample_cce.cpp" $APP_SRCS "$HERE/_ref/oracle_pin.o" -lm
# cce.cpp alone with HAS_MATLAB: its export_mat_file is the code recorded
${CXX:-g++} -O2 -std=c++14 -ffp-contract=off -w -DHAS_MATLAB -I"$HERE/ref_shim" -I"$HERE" -I"$S" \
  -c "$S/source/app/cce.cpp" -o "$HERE/_ref/cce_export.o"
# shellcheck disable=SC2086
${CXX:-g++} -O2 -std=c++14 -ffp-contract=off -w -DOOPS_PIN_EXPORT -I"$HERE/ref_shim" -I"$HERE" -I"$S" \
  -o "$HERE/_ref/ref_export_pin" "$HERE/ref_ensemble_pin.cpp" "$HERE/_ref/cce_export.o" $APP_BASE \
  "$HERE/_ref/oracle_pin.o" -lm
echo "built $HERE/_ref/libref_hamvec.so, ref_pin, ref_cce_pin, ref_ensemble_pin, ref_expv_pin, ref_single_pin and ref_export_pin"
