/* Test infrastructure, not product code.
 *
 * Runs the reference's own SPH kernels on the host: the __global__ section of
 * GPU_Kernels/K_FluidSim.cu (lines 1 up to the first `extern "C"` launcher,
 * compiled where it lies through oracle/ref_shim/kernel_host.h, see
 * oracle/Makefile target `refk`), driven once per particle index the way its
 * launchers (K_FluidSim.cu:488-691) drive them: textures bound to the same
 * arrays, the same arguments.  The result, oracle/_ref/libfgrefk_fluid.so,
 * produces tests/golden/ref_kernels.npz, which pins the oracle's restatement
 * of the kernel loops (27-bucket traversal order, self exclusion, scatter by
 * id, the static/dynamic rigid-grid terms) bit for bit.
 *
 * Kernels driven (paths relative to the reference project):
 *   GPU_Kernels/K_FluidSim.cu:210-254  CalculateMassDensityK   (launcher :488-517)
 *   GPU_Kernels/K_FluidSim.cu:260-309  SPHCalculateForcesK     (launcher :522-565)
 *   GPU_Kernels/K_FluidSim.cu:315-413  SPHCalculateForcesWithSRBK (launcher :614-680)
 *   GPU_Kernels/K_FluidSim.cu:418-477  SPHIntegrateK           (launcher :570-585)
 */
#include <string.h>
#include "ref_kernel_exec.h"
#include "ApplicationData.cuh"

extern texture<float4, 1, cudaReadModeElementType> oldPosTex;
extern texture<float4, 1, cudaReadModeElementType> oldVelTex;
extern texture<float2, 1, cudaReadModeElementType> densityFieldTex;
extern texture<uint, 1, cudaReadModeElementType> cellStartTex;
extern texture<uint, 1, cudaReadModeElementType> cellEndTex;

namespace SimulationLib {
namespace Fluid {
extern Simulation::Application::KernelsCache dKernelsCache;
extern Simulation::Application::CommonFluidParams dCommonFluidParams;
void CalculateMassDensityK(float4 *, float2 *, unsigned int *, unsigned int *, unsigned int *, unsigned int, float,
                           float, float);
void SPHCalculateForcesK(float4 *, float4 *, float4 *, float2 *, unsigned int *, unsigned int *, float4 *,
                         unsigned int *, float, unsigned int, float);
void SPHCalculateForcesWithSRBK(float4 *, float4 *, float4 *, float4 *, float2 *, unsigned int *, unsigned int *,
                                unsigned int *, unsigned int, float, float, float, float4 *, unsigned int *,
                                unsigned int *, unsigned int, float, float, float, float3, int3, float4 *, float4 *,
                                unsigned int *, unsigned int *, unsigned int, bool, bool);
void SPHIntegrateK(float4 *, float4 *, float4 *, float2 *, unsigned int *, unsigned int *, unsigned int);
} // namespace Fluid
} // namespace SimulationLib

namespace F = SimulationLib::Fluid;

extern "C" {

unsigned int refk_params_size() { return (unsigned int)sizeof(Simulation::Application::CommonFluidParams); }
unsigned int refk_kernels_cache_size() { return (unsigned int)sizeof(Simulation::Application::KernelsCache); }

/* gInitializeCommonFluidParams / gInitializeKernelParams (K_FluidSim.cu:590-609) */
void refk_set_params(const void *common, const void *kc)
{
    memcpy(&F::dCommonFluidParams, common, sizeof(F::dCommonFluidParams));
    memcpy(&F::dKernelsCache, kc, sizeof(F::dKernelsCache));
}

/* gCalcMassDensity (K_FluidSim.cu:488-517) */
void refk_density(float4 *spos, float2 *dp, unsigned int *start, unsigned int *end, unsigned int n, float gas,
                  float rest, float mass)
{
    oldPosTex.bound = spos;
    cellStartTex.bound = start;
    cellEndTex.bound = end;
    each_index(n, [&] { F::CalculateMassDensityK(spos, dp, nullptr, start, end, n, gas, rest, mass); });
}

/* gSPHCalculateForces (K_FluidSim.cu:522-565) */
void refk_forces(float4 *spos, float4 *svel, float2 *dp, unsigned int *start, unsigned int *end, float4 *newvel,
                 unsigned int *ids, float mass, unsigned int n, float visc)
{
    oldPosTex.bound = spos;
    oldVelTex.bound = svel;
    densityFieldTex.bound = dp;
    cellStartTex.bound = start;
    cellEndTex.bound = end;
    each_index(n, [&] { F::SPHCalculateForcesK(spos, svel, nullptr, dp, start, end, newvel, ids, mass, n, visc); });
}

/* gSPHCalculateForcesWithSRB (K_FluidSim.cu:614-680); cell3 / rel3 are the
 * rigid grid's cell size and the fluid-to-rigid cell relation */
void refk_forces_srb(float4 *spos, float4 *svel, float4 *newvel, float2 *dp, unsigned int *ids,
                     unsigned int *start, unsigned int *end, unsigned int n, float mass, float visc,
                     float fluid_radius, float rb_radius, float kspring, float kdamping, const float *cell3,
                     const int *rel3, float4 *s_pos, unsigned int *s_start, unsigned int *s_end, unsigned int s_nb,
                     float4 *d_pos, float4 *d_vel, unsigned int *d_start, unsigned int *d_end, unsigned int d_nb,
                     int use_static, int use_dynamic)
{
    oldPosTex.bound = spos;
    oldVelTex.bound = svel;
    densityFieldTex.bound = dp;
    cellStartTex.bound = start;
    cellEndTex.bound = end;
    const float3 cell = make_float3(cell3[0], cell3[1], cell3[2]);
    const int3 rel = make_int3(rel3[0], rel3[1], rel3[2]);
    each_index(n, [&] {
        F::SPHCalculateForcesWithSRBK(spos, svel, newvel, nullptr, dp, ids, start, end, n, mass, visc, fluid_radius,
                                      s_pos, s_start, s_end, s_nb, rb_radius, kspring, kdamping, cell, rel, d_pos,
                                      d_vel, d_start, d_end, d_nb, use_static != 0, use_dynamic != 0);
    });
}

/* gSPHIntegrate (K_FluidSim.cu:570-585), in place on pos */
void refk_integrate(float4 *pos, float4 *vel, unsigned int n)
{
    each_index(n, [&] { F::SPHIntegrateK(pos, vel, nullptr, nullptr, nullptr, nullptr, n); });
}

} /* extern "C" */
