#!/bin/sh
# Builds oracle/_ref/libsimall_ref.so: the SimAll reference's own hot-path
# sources, compiled where they lie, plus oracle/ref_driver.cpp (a C-callable
# test driver).  Test infrastructure only; the product never loads it.
#
# Reference files compiled (paths inside the reference tree):
#   src/solver/LinearSolvers.cpp   (see the one patch below)
#   src/solver/AMGPreconditioner.cpp, src/solver/SimpleAlgorithm.cpp,
#   src/solver/PisoAlgorithm.cpp, src/solver/PimpleAlgorithm.cpp,
#   src/solver/Gradient.cpp, src/meshing/MeshStorage.cpp,
#   src/meshing/CartesianMesher.cpp, src/meshing/Connectivity.cpp,
#   src/meshing/MeshOps.cpp, src/meshing/MeshQuality.cpp,
#   src/adjoint/DiscreteAdjoint.cpp, src/core/PluginLoader.cpp,
#   src/core/PluginRegistry.cpp, src/io/Checkpoint.cpp,
#   src/optimization/SimpTopology.cpp, and the GPU facade's host path (no
#   SIMALL_HAVE_CUDA): src/gpu/CgGpu.cpp, src/gpu/GpuKernels.cpp,
#   src/gpu/CudaContext.cpp, src/gpu/DeviceMemoryPool.cpp
#
# Patch: LinearSolvers.cpp assigns util::aligned_vector<int> to std::vector<int>
# at :85-86 and :170-171, which g++ 13 rejects.  A scratch copy written into
# oracle/_ref/ replaces each of those four assignments with .assign(begin,end);
# behaviour is unchanged.
#
# Usage: sh oracle/build_ref.sh [reference-root]
# The root is the argument, else $SIMALL_REFERENCE, else /root/reference.  Exit
# status 2 when no reference tree is there (e.g. on the GPU host).  The root
# compiled is recorded in oracle/_ref/REFERENCE_ROOT for the tests that compile
# against the reference's headers.
set -eu
REF=${1:-${SIMALL_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/solver/LinearSolvers.cpp" ]; then
    echo "build_ref.sh: reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
printf '%s\n' "$REF" > "$OUT/REFERENCE_ROOT"
sed -e 's/^        rowPtr_ = A\.rowPtr;$/        rowPtr_.assign(A.rowPtr.begin(), A.rowPtr.end());/' \
    -e 's/^        colIdx_ = A\.colIdx;$/        colIdx_.assign(A.colIdx.begin(), A.colIdx.end());/' \
    "$REF/src/solver/LinearSolvers.cpp" > "$OUT/LinearSolvers_patched.cpp"

CXX=${CXX:-g++}
FLAGS="-std=c++20 -O3 -fPIC -ffp-contract=off -w -Wno-psabi -I$REF/src -I$REF"
SRCS="$OUT/LinearSolvers_patched.cpp
$REF/src/solver/AMGPreconditioner.cpp
$REF/src/solver/SimpleAlgorithm.cpp
$REF/src/solver/PisoAlgorithm.cpp
$REF/src/solver/PimpleAlgorithm.cpp
$REF/src/solver/Gradient.cpp
$REF/src/meshing/MeshStorage.cpp
$REF/src/meshing/CartesianMesher.cpp
$REF/src/meshing/Connectivity.cpp
$REF/src/meshing/MeshOps.cpp
$REF/src/meshing/MeshQuality.cpp
$REF/src/adjoint/DiscreteAdjoint.cpp
$REF/src/core/PluginLoader.cpp
$REF/src/core/PluginRegistry.cpp
$REF/src/io/Checkpoint.cpp
$REF/src/optimization/SimpTopology.cpp
$REF/src/gpu/CgGpu.cpp
$REF/src/gpu/GpuKernels.cpp
$REF/src/gpu/CudaContext.cpp
$REF/src/gpu/DeviceMemoryPool.cpp
$HERE/ref_driver.cpp"
pids=""
objs=""
i=0
for s in $SRCS; do
    o="$OUT/obj_$i.o"
    $CXX $FLAGS -c "$s" -o "$o" &
    pids="$pids $!"
    objs="$objs $o"
    i=$((i + 1))
done
for p in $pids; do wait "$p"; done
$CXX -shared -o "$OUT/libsimall_ref.so.tmp" $objs -lpthread -ldl
mv "$OUT/libsimall_ref.so.tmp" "$OUT/libsimall_ref.so"
echo "built $OUT/libsimall_ref.so"
