/* Forced-include prelude for building the reference's CUDA library with
 * nvcc on Linux (oracle/build_ref_cuda.sh; test and measurement
 * infrastructure only). It supplies two things the reference's sources
 * expect from their original Windows toolchain:
 *   - the std::powf / std::sqrtf names (libstdc++ does not declare them in
 *     namespace std; cuda_dem_solver_common_gpu.cuh:40 and
 *     cuda_volume_emitter.cpp:74,124,162 use them);
 *   - atomicAdd on a size_t counter (cuda_neighbor_searcher_gpu.cuh:23),
 *     where size_t is unsigned long, which has no CUDA overload: the same
 *     64-bit atomic on its unsigned long long view. */
#ifndef SF_REF_DEVICE_PRELUDE_H
#define SF_REF_DEVICE_PRELUDE_H
#include <cuda_runtime.h>
#include <cmath>
#include <math.h>
namespace std {
using ::powf;
using ::sqrtf;
}
#ifdef __CUDACC__
static_assert(sizeof(unsigned long) == sizeof(unsigned long long), "LP64 expected");
__device__ __forceinline__ unsigned long atomicAdd(unsigned long* address, unsigned long val) {
    return static_cast<unsigned long>(
        atomicAdd(reinterpret_cast<unsigned long long*>(address), static_cast<unsigned long long>(val)));
}
#endif
#endif
