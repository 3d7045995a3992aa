/* FP64 conservation diagnostics per scene: fluid mass, momentum, kinetic
 * energy and first moment, the bodies' momentum, angular momentum and
 * kinetic energy.  Sums run in FP64 in a fixed order (a tree inside each
 * 128-particle work item, then the work items of a scene in sequence), so
 * the figures are reproducible bit for bit.  The reference has no such
 * diagnostic; it reads the same state its integrators write
 * (SPHIntegrateK, K_FluidSim.cu:418-438; IntegrateRBK,
 * K_RigidBodySim.cu:160-262). */
#include <cuda_runtime.h>
#include <stdint.h>
#include "fg_device.cuh"
#include "fg_kernels.h"

namespace fg {

#define DIAG_PART 9 /* count, mass, px, py, pz, ke, mx, my, mz */

__global__ void __launch_bounds__(FG_CHUNK) k_diag_partial(const FgWork *__restrict__ work, uint32_t nwork,
                                                          uint32_t n_single, const FgScene *__restrict__ table,
                                                          const __grid_constant__ FgScene single,
                                                          const float4 *__restrict__ pos,
                                                          const float4 *__restrict__ vel, double *__restrict__ part)
{
    __shared__ double s[DIAG_PART][FG_CHUNK];
    for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        const FgWork it = fg_work(work, w, n_single);
        const FgScene *S = fg_scene(table, &single, it.scene);
        double v[DIAG_PART];
#pragma unroll
        for (int q = 0; q < DIAG_PART; q++) v[q] = 0.0;
        if (threadIdx.x < it.count) {
            const float4 p = __ldg(pos + it.first + threadIdx.x);
            if (p.w > 0.0f) {
                const float4 u = __ldg(vel + it.first + threadIdx.x);
                const double m = (double)S->mass;
                const double ux = u.x, uy = u.y, uz = u.z;
                v[0] = 1.0;
                v[1] = m;
                v[2] = m * ux;
                v[3] = m * uy;
                v[4] = m * uz;
                v[5] = 0.5 * m * (ux * ux + uy * uy + uz * uz);
                v[6] = m * (double)p.x;
                v[7] = m * (double)p.y;
                v[8] = m * (double)p.z;
            }
        }
#pragma unroll
        for (int q = 0; q < DIAG_PART; q++) s[q][threadIdx.x] = v[q];
        __syncthreads();
        for (uint32_t h = FG_CHUNK / 2; h; h >>= 1) {
            if (threadIdx.x < h)
#pragma unroll
                for (int q = 0; q < DIAG_PART; q++) s[q][threadIdx.x] += s[q][threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x < DIAG_PART) part[(size_t)w * DIAG_PART + threadIdx.x] = s[threadIdx.x][0];
        __syncthreads();
    }
}

/* One thread per scene: its work items in order, then its bodies. */
__global__ void k_diag_final(const FgScene *__restrict__ table, const __grid_constant__ FgScene single,
                             uint32_t nscenes, const uint32_t *__restrict__ work_first,
                             const double *__restrict__ part, const FgD4 *__restrict__ bv,
                             const FgD4 *__restrict__ bL, const double *__restrict__ bmass, double *__restrict__ out)
{
    const uint32_t sc = blockIdx.x * blockDim.x + threadIdx.x;
    if (sc >= nscenes) return;
    const FgScene *S = table ? table + sc : &single;
    double acc[FG_DIAG_VALUES];
    for (int q = 0; q < FG_DIAG_VALUES; q++) acc[q] = 0.0;
    for (uint32_t w = work_first[sc]; w < work_first[sc + 1]; w++)
        for (int q = 0; q < DIAG_PART; q++) acc[q] += part[(size_t)w * DIAG_PART + q];
    for (uint32_t b = S->body_base; b < S->body_base + S->nbodies; b++) {
        const double M = bmass[b];
        const FgD4 v = bv[b], L = bL[b];
        acc[9] += M * v.x;
        acc[10] += M * v.y;
        acc[11] += M * v.z;
        acc[12] += L.x;
        acc[13] += L.y;
        acc[14] += L.z;
        acc[15] += 0.5 * M * (v.x * v.x + v.y * v.y + v.z * v.z);
    }
    for (int q = 0; q < FG_DIAG_VALUES; q++) out[(size_t)sc * FG_DIAG_VALUES + q] = acc[q];
}

void launch_diagnostics(const Launch &L, uint32_t nscenes, const uint32_t *work_first, const float4 *pos,
                        const float4 *vel, const FgD4 *bv, const FgD4 *bL, const double *bmass, double *part,
                        double *out)
{
    if (L.nwork)
        k_diag_partial<<<grid_for(L.nwork, 8), FG_CHUNK, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single,
                                                                        pos, vel, part);
    if (nscenes)
        k_diag_final<<<(nscenes + 63) / 64, 64, 0, L.stream>>>(L.table, *L.single, nscenes, work_first, part, bv, bL,
                                                              bmass, out);
}

} // namespace fg
