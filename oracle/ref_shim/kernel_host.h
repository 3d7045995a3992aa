/* Host execution of the reference's __global__ kernels (test infrastructure,
 * oracle build only).  Force-included before a reference kernel file whose
 * launchers (the `extern "C"` functions with <<<...>>> launches) are cut off;
 * the harness then runs each kernel body once per (block, thread) index:
 *   - threadIdx / blockIdx / blockDim / gridDim are thread-local variables
 *     the harness sets before each call;
 *   - a texture reference is a pointer the harness binds (cudaBindTexture
 *     semantics) and tex1Dfetch reads element i through it;
 *   - __syncthreads() is a barrier over the host threads running one block,
 *     and extern __shared__ arrays are buffers the harness owns per block.
 * Written from the public CUDA programming model, not from NVIDIA headers. */
#ifndef FG_SHIM_KERNEL_HOST_H
#define FG_SHIM_KERNEL_HOST_H

#include <math.h>
#include "vector_types.h"
#include "vector_functions.h"

struct fg_idx3 {
    unsigned int x, y, z;
};
extern thread_local fg_idx3 threadIdx, blockIdx, blockDim, gridDim;

void fg_syncthreads();
#define __syncthreads() fg_syncthreads()

enum cudaTextureReadMode { cudaReadModeElementType = 0 };
template <class T, int dim = 1, cudaTextureReadMode mode = cudaReadModeElementType>
struct texture {
    const T *bound = nullptr;
};
template <class T, int dim, cudaTextureReadMode mode>
static inline T tex1Dfetch(const texture<T, dim, mode> &t, int i)
{
    return t.bound[i];
}

/* __umul24: the product of the low 24 bits of a and b, low 32 bits kept */
static inline unsigned int __umul24(unsigned int a, unsigned int b) { return (a & 0xffffffu) * (b & 0xffffffu); }

/* CUDA's overloads of max/min for mixed float/double arguments resolve to the
 * double versions */
static inline double max(double a, double b) { return a > b ? a : b; }
static inline double min(double a, double b) { return a < b ? a : b; }

#endif
