/* Test infrastructure, not product code.
 *
 * Runs the reference's own rigid-body kernels on the host: the __global__
 * section of GPU_Kernels/K_RigidBodySim.cu (up to its first `extern "C"`
 * launcher, compiled where it lies through oracle/ref_shim/kernel_host.h, see
 * oracle/Makefile target `refk`), one call per index as its launchers
 * (K_RigidBodySim.cu:273-400) launch them.  None of the three uses a barrier.
 *
 * Kernels driven (paths relative to the reference project):
 *   GPU_Kernels/K_RigidBodySim.cu:18-61    CalculateRigidBodyForcesFromRBK
 *   GPU_Kernels/K_RigidBodySim.cu:66-99    CalculateRBForcesFromFluidsK
 *   GPU_Kernels/K_RigidBodySim.cu:160-262  IntegrateRBK
 */
#include <stddef.h>
#include "ref_kernel_exec.h"

namespace SimulationLib {
namespace RigidBody {
void CalculateRigidBodyForcesFromRBK(float4 *, float4 *, float4 *, float4 *, float4 *, unsigned int *,
                                     unsigned int *, unsigned int, float3, float, int, int, float4 *, unsigned int *,
                                     unsigned int *, float, float, int);
void CalculateRBForcesFromFluidsK(float4 *, float4 *, float4 *, float4 *, float4 *, unsigned int *, unsigned int *,
                                  unsigned int, float3, float, int, float4 *, float4 *, uint *, uint *, float, float3,
                                  uint, int3, float, float);
void IntegrateRBK(float4 *, float *, float4 *, float4 *, size_t, float, float4, float3, float3, float4 *, float4 *,
                  float4 *, float4 *, float4 *, float);
} // namespace RigidBody
} // namespace SimulationLib

namespace RB = SimulationLib::RigidBody;

static float3 f3(const float *p) { return make_float3(p[0], p[1], p[2]); }

extern "C" {

/* gCalculateRigidBodyForcesFromRB (K_RigidBodySim.cu:273-304) */
void refk_rb_forces_from_rb(float4 *pos, float4 *bvel, float4 *bcm, float4 *torque, float4 *force,
                            unsigned int *start, unsigned int *end, unsigned int n, const float *cell3, float radius,
                            int rb_nb, int srb_nb, float4 *srb_pos, unsigned int *srb_start, unsigned int *srb_end,
                            float k, float kd, int nsrb)
{
    const float3 c = f3(cell3);
    each_index(n, [&] {
        RB::CalculateRigidBodyForcesFromRBK(pos, bvel, bcm, torque, force, start, end, n, c, radius, rb_nb, srb_nb,
                                            srb_pos, srb_start, srb_end, k, kd, nsrb);
    });
}

/* gCalculateRBForcesFromFluids (K_RigidBodySim.cu:309-340) */
void refk_rb_forces_from_fluids(float4 *pos, float4 *bvel, float4 *bcm, float4 *force, float4 *torque,
                                unsigned int *start, unsigned int *end, unsigned int n, const float *cell3,
                                float radius, int rb_nb, float4 *sph_pos, float4 *sph_vel, unsigned int *sph_start,
                                unsigned int *sph_end, float sph_radius, const float *sph_cell3,
                                unsigned int sph_nb, const int *rel3, float k, float kd)
{
    const float3 c = f3(cell3), sc = f3(sph_cell3);
    const int3 rel = make_int3(rel3[0], rel3[1], rel3[2]);
    each_index(n, [&] {
        RB::CalculateRBForcesFromFluidsK(pos, bvel, bcm, force, torque, start, end, n, c, radius, rb_nb, sph_pos,
                                         sph_vel, sph_start, sph_end, sph_radius, sc, sph_nb, rel, k, kd);
    });
}

/* gIntegrateRB (K_RigidBodySim.cu:381-400) */
void refk_integrate_rb(float4 *x, float *mass, float4 *v, float4 *f, unsigned int nrb, float dt, const float *ext4,
                       const float *min3, const float *max3, float4 *L, float4 *t, float4 *inertia, float4 *q,
                       float4 *inv, float vlimit)
{
    const float4 ext = make_float4(ext4[0], ext4[1], ext4[2], ext4[3]);
    const float3 mn = f3(min3), mx = f3(max3);
    each_index(nrb, [&] {
        RB::IntegrateRBK(x, mass, v, f, (size_t)nrb, dt, ext, mn, mx, L, t, inertia, q, inv, vlimit);
    });
}

} /* extern "C" */
