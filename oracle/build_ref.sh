#!/bin/sh
# Builds the reference harness oracle/_ref/libsfref.so: the sph_seepage_flows
# kernel headers and emitter sources compiled in place as host C++ (test
# infrastructure; see oracle/ref_harness.cpp), and the partio harness
# oracle/_ref/libpartioref.so: the partio .bgeo reader and writer the
# reference vendors (extlib/include/partio), compiled in place (see
# oracle/partio_harness.cpp). Needs the reference sources, which exist only
# where they are mounted; elsewhere this script does nothing.
#
#   SF_REFERENCE_ROOT  root of the sph_seepage_flows sources (default /root/reference)
#   CUDA_HOME          CUDA toolkit (default /usr/local/cuda; only its headers are used)
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${SF_REFERENCE_ROOT:-/root/reference}
CUDA=${CUDA_HOME:-/usr/local/cuda}
SFC="$REF/seepage_flows_cuda"
if [ ! -d "$SFC/include/kiri_pbs_cuda" ]; then
    echo "build_ref.sh: reference sources not found under $REF; skipping" >&2
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
EMIT="$SFC/src/kiri_pbs_cuda/emitter"
${CXX:-g++} -std=c++17 -O2 -ffp-contract=off -fopenmp -fPIC -shared -w \
    -I "$HERE/ref_shim" -I "$SFC/include" -I "$CUDA/include" -I "$CUDA/include/cccl" \
    -include "$HERE/ref_shim/host_prelude.h" \
    "$HERE/ref_harness.cpp" \
    "$EMIT/cuda_boundary_emitter.cpp" "$EMIT/cuda_emitter.cpp" "$EMIT/cuda_volume_emitter.cpp" \
    -o "$OUT/libsfref.so"
echo "built $OUT/libsfref.so"
P="$REF/extlib/include/partio"
if [ -f "$P/io/BGEO.cpp" ]; then
    ${CXX:-g++} -std=c++17 -O2 -fPIC -shared -w -I "$P" -I "$P/core" -I "$P/io" \
        "$HERE/partio_harness.cpp" "$P/io/BGEO.cpp" "$P/io/ZIP.cpp" "$P/core/Particle.cpp" \
        "$P/core/ParticleHeaders.cpp" "$P/core/ParticleSimple.cpp" "$P/core/ParticleSimpleInterleave.cpp" \
        "$P/core/ParticleCaching.cpp" -o "$OUT/libpartioref.so"
    echo "built $OUT/libpartioref.so"
fi
