#!/bin/sh
# Builds the reference's own CUDA library (seepage_flows_cuda) for sm_103a,
# with its own arithmetic flags (-use_fast_math, seepage_flows_cuda/
# CMakeLists.txt:23), linked with the driver oracle/ref_gpu_driver.cu into
# baseline/_ref/libsfrefgpu.so. Test and measurement infrastructure only: the
# product never loads it.
#
# Two steps, each done where it can be:
#   stage   where the reference sources are mounted: copy seepage_flows_cuda/
#           into baseline/_ref/seepage_flows_cuda (git-ignored; it travels with
#           the working tree to the GPU machine) and apply the two source
#           patches its Windows-era code needs under g++/nvcc on Linux:
#             * cuda_sf_particles.cuh:31-33: CCCL tuples have no member get<N>();
#               data.get<N>() -> thrust::get<N>(data);
#             * cuda_base_system.{cuh,cu}: the solver argument is a non-const
#               reference bound to an rvalue (cuda_sf_system.cu:27, an MSVC
#               extension); it is taken by value instead (the constructor moves
#               it either way).
#           The std::powf / std::sqrtf names and the size_t atomicAdd come from
#           the forced-include prelude oracle/ref_shim/device_prelude.h, the
#           Linux <kiri_pbs_cuda/string.h> includes from oracle/ref_shim.
#   build   wherever the staged copy exists: nvcc of its 14 translation units
#           and the driver, in parallel.
#
#   SF_REFERENCE_ROOT  root of the sph_seepage_flows sources (default: the
#                      mount point of this build container, /root/reference)
#   CUDA_HOME          CUDA toolkit (default /usr/local/cuda)
#   SF_REF_ARCH        -gencode argument (default arch=compute_103a,code=sm_103a)
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(dirname "$HERE")
REF=${SF_REFERENCE_ROOT:-/root/reference}
CUDA=${CUDA_HOME:-/usr/local/cuda}
ARCH=${SF_REF_ARCH:-arch=compute_103a,code=sm_103a}
DST="$ROOT/baseline/_ref"
SFC="$DST/seepage_flows_cuda"
LIB="$DST/libsfrefgpu.so"

if [ -d "$REF/seepage_flows_cuda/include/kiri_pbs_cuda" ]; then
    mkdir -p "$DST"
    rm -rf "$SFC.tmp"
    cp -R "$REF/seepage_flows_cuda" "$SFC.tmp"
    sed -i 's/data\.get<\([0-9]\)>()/thrust::get<\1>(data)/g' \
        "$SFC.tmp/include/kiri_pbs_cuda/particle/cuda_sf_particles.cuh"
    sed -i 's/CudaBaseSolverPtr &solver/CudaBaseSolverPtr solver/' \
        "$SFC.tmp/include/kiri_pbs_cuda/system/cuda_base_system.cuh" \
        "$SFC.tmp/src/kiri_pbs_cuda/system/cuda_base_system.cu"
    grep -q "thrust::get<0>(data)" "$SFC.tmp/include/kiri_pbs_cuda/particle/cuda_sf_particles.cuh"
    grep -q "CudaBaseSolverPtr solver" "$SFC.tmp/src/kiri_pbs_cuda/system/cuda_base_system.cu"
    if [ -d "$SFC" ] && diff -rq "$SFC" "$SFC.tmp" > /dev/null 2>&1; then
        rm -rf "$SFC.tmp"
    else
        rm -rf "$SFC"
        mv "$SFC.tmp" "$SFC"
    fi
fi
if [ ! -d "$SFC/src" ]; then
    echo "build_ref_cuda.sh: no staged reference library under $SFC; skipping" >&2
    exit 0
fi
NVCC="$CUDA/bin/nvcc"
[ -x "$NVCC" ] || NVCC=nvcc
OBJ="$DST/obj"
mkdir -p "$OBJ"
FLAGS="-gencode $ARCH -O3 -std=c++17 --expt-extended-lambda --expt-relaxed-constexpr -use_fast_math \
    -Xcompiler -fPIC -w -I $HERE/ref_shim -I $SFC/include -I $ROOT/include -include $HERE/ref_shim/device_prelude.h"
SRCS=$(cd "$SFC/src" && find . -name '*.cu' -o -name '*.cpp' | sort)
NEWEST=$(ls -t "$HERE/ref_gpu_driver.cu" "$HERE/build_ref_cuda.sh" "$HERE/ref_shim/device_prelude.h" | head -1)
if [ -f "$LIB" ] && [ "$LIB" -nt "$NEWEST" ] && [ -z "$(find "$SFC" -newer "$LIB" -type f | head -1)" ]; then
    echo "$LIB is up to date"
    exit 0
fi
pids=""
objs=""
for s in $SRCS; do
    o="$OBJ/$(echo "$s" | sed 's|^\./||; s|/|_|g').o"
    objs="$objs $o"
    # shellcheck disable=SC2086
    "$NVCC" $FLAGS -x cu -c "$SFC/src/$s" -o "$o" &
    pids="$pids $!"
done
# shellcheck disable=SC2086
"$NVCC" $FLAGS -x cu -c "$HERE/ref_gpu_driver.cu" -o "$OBJ/ref_gpu_driver.o" &
pids="$pids $!"
fail=0
for p in $pids; do wait "$p" || fail=1; done
if [ "$fail" -ne 0 ]; then
    echo "build_ref_cuda.sh: nvcc failed" >&2
    exit 1
fi
# shellcheck disable=SC2086
"$NVCC" -gencode "$ARCH" -shared -o "$LIB" $objs "$OBJ/ref_gpu_driver.o"
echo "built $LIB"
