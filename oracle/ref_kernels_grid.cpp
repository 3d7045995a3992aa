/* Test infrastructure, not product code.
 *
 * Runs the reference's own hash-grid kernels on the host: the __global__
 * section of GPU_Kernels/K_HashGrid.cu (up to its first `extern "C"`
 * launcher, compiled where it lies through oracle/ref_shim/kernel_host.h, see
 * oracle/Makefile target `refk`), launched as its launchers launch them
 * (K_HashGrid.cu:207-318): 128-thread blocks, the block's shared hash buffer
 * of 129 words, start pre-filled with 0xffffffff, textures bound to the
 * unsorted arrays.  The blocks of the range kernels run as real thread
 * groups with a barrier (ref_kernel_exec.h).
 *
 * Kernels driven (paths relative to the reference project):
 *   GPU_Kernels/K_HashGrid.cu:26-38    CalcHashKeyK
 *   GPU_Kernels/K_HashGrid.cu:43-63    CalcHashKeyWithOffsetK
 *   GPU_Kernels/K_HashGrid.cu:70-133   FindCellOffsetOrderinPosVelK
 *   GPU_Kernels/K_HashGrid.cu:140-197  FindCellOffsetOrderingPosK
 */
#include <string.h>
#include "ref_kernel_exec.h"

extern texture<float4, 1, cudaReadModeElementType> oldPosTex;
extern texture<float4, 1, cudaReadModeElementType> oldVelTex;

namespace SimulationLib {
namespace DataStructure {
void CalcHashKeyK(unsigned int *, unsigned int *, float4 *, unsigned int, float3, int);
void CalcHashKeyWithOffsetK(unsigned int *, unsigned int *, float4 *, float4 *, float4 *, float4 *, unsigned int,
                            float3, int);
void FindCellOffsetOrderinPosVelK(unsigned int *, unsigned int *, unsigned int *, unsigned int *, float4 *,
                                  float4 *, float4 *, float4 *, unsigned int);
void FindCellOffsetOrderingPosK(unsigned int *, unsigned int *, unsigned int *, unsigned int *, float4 *, float4 *,
                                unsigned int);
/* the kernels' `extern __shared__ unsigned int sharedHash[]` (blockSize + 1
 * words); blocks run one at a time */
unsigned int sharedHash[129];
} // namespace DataStructure
} // namespace SimulationLib

namespace G = SimulationLib::DataStructure;

static const unsigned int BLOCK = 128;

static unsigned int blocks_for(unsigned int n) { return (n + BLOCK - 1) / BLOCK; }

extern "C" {

/* gCalcHashKey (K_HashGrid.cu:207-216) */
void refk_calc_hash_key(unsigned int *keys, unsigned int *ids, float4 *pos, unsigned int n, unsigned int nb,
                        const float *cell3)
{
    const float3 c = make_float3(cell3[0], cell3[1], cell3[2]);
    each_index(n, [&] { G::CalcHashKeyK(keys, ids, pos, n, c, (int)nb); });
}

/* gCalcHashKeyWithOffset (K_HashGrid.cu:221-233) */
void refk_calc_hash_key_with_offset(unsigned int *keys, unsigned int *ids, float4 *cm, float4 *q, float4 *local,
                                    float4 *world, unsigned int n, const float *cell3, int nb)
{
    const float3 c = make_float3(cell3[0], cell3[1], cell3[2]);
    each_index(n, [&] { G::CalcHashKeyWithOffsetK(keys, ids, cm, q, local, world, n, c, nb); });
}

/* gFindCellOffsetOrderingPosVel (K_HashGrid.cu:238-280) */
void refk_find_cell_offset_pos_vel(unsigned int *start, unsigned int *end, unsigned int *keys, unsigned int *ids,
                                   float4 *pos, float4 *spos, float4 *vel, float4 *svel, unsigned int n,
                                   unsigned int nb)
{
    memset(start, 0xff, sizeof(unsigned int) * nb);
    oldPosTex.bound = pos;
    oldVelTex.bound = vel;
    each_block(blocks_for(n), BLOCK,
               [&] { G::FindCellOffsetOrderinPosVelK(start, end, keys, ids, pos, spos, vel, svel, n); });
}

/* gFindCellOffsetOrderingPos (K_HashGrid.cu:286-318) */
void refk_find_cell_offset_pos(unsigned int *start, unsigned int *end, unsigned int *keys, unsigned int *ids,
                               float4 *pos, float4 *spos, unsigned int n, unsigned int nb)
{
    memset(start, 0xff, sizeof(unsigned int) * nb);
    oldPosTex.bound = pos;
    each_block(blocks_for(n), BLOCK, [&] { G::FindCellOffsetOrderingPosK(start, end, keys, ids, pos, spos, n); });
}

} /* extern "C" */
