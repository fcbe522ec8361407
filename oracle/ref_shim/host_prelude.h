/* Forced-include prelude for compiling the reference's CUDA kernel headers as
 * host C++ (the reference harness under oracle/). It supplies what nvcc would:
 * the launch built-ins as per-thread host variables, __umul24, and the
 * std::powf / std::sqrtf names the reference uses (libstdc++ does not declare
 * them in namespace std). Test infrastructure only. */
#ifndef SF_REF_HOST_PRELUDE_H
#define SF_REF_HOST_PRELUDE_H
#include <cuda_runtime.h>
#include <cmath>
#include <math.h>
namespace std {
using ::powf;
using ::sqrtf;
}
struct sfref_dim3 {
    unsigned int x, y, z;
};
extern thread_local sfref_dim3 sfref_blockIdx, sfref_blockDim, sfref_threadIdx;
#define blockIdx sfref_blockIdx
#define blockDim sfref_blockDim
#define threadIdx sfref_threadIdx
static inline unsigned int __umul24(unsigned int a, unsigned int b) { return a * b; }
#endif
