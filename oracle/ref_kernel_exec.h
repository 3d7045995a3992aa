/* Test infrastructure, not product code.
 *
 * Host execution of a reference kernel's launch grid, for the harnesses that
 * drive the reference's __global__ functions compiled through
 * ref_shim/kernel_host.h.  Included by exactly one translation unit of each
 * harness library (it defines the thread-local launch indices). */
#ifndef FG_REF_KERNEL_EXEC_H
#define FG_REF_KERNEL_EXEC_H

#include <stdlib.h>
#include <barrier>
#include <thread>
#include <vector>
#include "kernel_host.h"

thread_local fg_idx3 threadIdx, blockIdx, blockDim, gridDim;
static thread_local std::barrier<> *fg_block_barrier = nullptr;

/* __syncthreads(): the barrier of the block this host thread runs in; a
 * kernel run index by index (each_index) reaching one is a harness error */
void fg_syncthreads()
{
    if (!fg_block_barrier) abort();
    fg_block_barrier->arrive_and_wait();
}

/* A kernel that reads only blockDim.x * blockIdx.x + threadIdx.x and has no
 * barrier: one call per index i (blockDim 1, blockIdx i), indices in
 * parallel. */
template <class Fn>
static void each_index(unsigned int n, Fn &&fn)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; i++) {
        blockDim = fg_idx3{1u, 1u, 1u};
        gridDim = fg_idx3{n, 1u, 1u};
        threadIdx = fg_idx3{0u, 0u, 0u};
        blockIdx = fg_idx3{(unsigned int)i, 0u, 0u};
        fn();
    }
}

/* A kernel with barriers or shared memory: the launch's blocks one after
 * another, each as `bdim` host threads that share a barrier (and whatever
 * shared buffer the harness gives the block). */
template <class Fn>
static void each_block(unsigned int nblocks, unsigned int bdim, Fn &&fn)
{
    for (unsigned int b = 0; b < nblocks; b++) {
        std::barrier<> bar((std::ptrdiff_t)bdim);
        std::vector<std::thread> th;
        th.reserve(bdim);
        for (unsigned int t = 0; t < bdim; t++)
            th.emplace_back([&, b, t] {
                blockDim = fg_idx3{bdim, 1u, 1u};
                gridDim = fg_idx3{nblocks, 1u, 1u};
                blockIdx = fg_idx3{b, 0u, 0u};
                threadIdx = fg_idx3{t, 0u, 0u};
                fg_block_barrier = &bar;
                fn();
                fg_block_barrier = nullptr;
            });
        for (auto &x : th) x.join();
    }
}

#endif
