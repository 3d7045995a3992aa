/* fluidgrid_gb300 -- drop-in replacements of the reference's extern "C"
 * kernel launchers (GPU_Kernels/K_HashGrid.cuh, K_FluidSim.cuh,
 * K_RigidBodySim.cuh of FluidGrid).
 *
 * Same symbol names, argument lists and by-value struct layouts as the
 * reference, so the reference's host code (GPUSPHFluid,
 * HeterogeneousSimulator, RigidBodySimulator) links against
 * libfluidgrid_gb300.so unchanged.  Pointers are device pointers owned by the
 * caller; work is enqueued on the legacy default stream like the reference.
 * The launchers return void as there; fgc_last_status() reports the status
 * of the most recent call on this thread (0 = success).
 *
 * Differences a caller can observe: none in keys, sort order, start/end
 * entries or sorted gathers (bit-identical); density, forces and rigid
 * contact agree within the tolerances of the parity tests; gSort sorts the
 * full 32-bit key like thrust::sort_by_key and allocates its scratch once
 * (grow-only cache), not per call.
 */
#ifndef FLUIDGRID_REFERENCE_H
#define FLUIDGRID_REFERENCE_H

#include <stddef.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif
#include <vector_types.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Layout of Simulation::Application::CommonFluidParams
 * (ApplicationData.cuh:46-67); passed by value like the reference type. */
typedef struct fgr_common_fluid_params {
    float3 cell_size;
    int3 bucket_size;
    unsigned int keyBits;
    float kernel_radius;
    float kernel_radius_squared;
    float pointRadius;
    float pointScale;
    float velocity_limit;
    float3 volume_min;
    float3 volume_max;
    float3 global_external_force;
    float simulation_scale;
    float deltaTimeIntegration;
    int3 fluid_to_srb_relation;
} fgr_common_fluid_params;

/* Layout of Simulation::Application::KernelsCache (ApplicationData.cuh:107-112). */
typedef struct fgr_kernels_cache {
    float kPoly6;
    float kSpikyGradient;
    float kViscosityLaplacian;
} fgr_kernels_cache;

/* ---- K_HashGrid.cuh ---- */

/* replaces gCalcHashKey, K_HashGrid.cuh:5-8 / K_HashGrid.cu:207-216 */
void gCalcHashKey(unsigned int *hashKey, unsigned int *particleID, float4 *positions, unsigned int numParticles,
                  unsigned int numBuckets, float3 cell_size);

/* replaces gCalcHashKeyWithOffset, K_HashGrid.cuh:10-20 / K_HashGrid.cu:221-233 */
void gCalcHashKeyWithOffset(unsigned int *_out_hashKey, unsigned int *_out_particleID, float4 *_in_vectorOffset,
                            float4 *_in_orientation, float4 *_in_vectorPos, float4 *_out_positions,
                            unsigned int _in_numParticles, float3 _in_cellSize, int _in_hashTableSize);

/* replaces gFindCellOffsetOrderingPosVel, K_HashGrid.cuh:23-33 / K_HashGrid.cu:238-281 */
void gFindCellOffsetOrderingPosVel(unsigned int *gridPosStart, unsigned int *gridPosEnd, unsigned int *hashTable,
                                   unsigned int *particleID, float4 *particlePositions,
                                   float4 *orderedParticlePositions, float4 *particleVel, float4 *particleOrderedVel,
                                   unsigned int numParticles, unsigned int numBuckets);

/* replaces gFindCellOffsetOrderingPos, K_HashGrid.cuh:37-56 / K_HashGrid.cu:287-318 */
void gFindCellOffsetOrderingPos(unsigned int *gridPosStart, unsigned int *gridPosEnd, unsigned int *hashTable,
                                unsigned int *particleID, float4 *particlePositions, float4 *orderedParticlePositions,
                                unsigned int numParticles, unsigned int numBuckets);

/* ---- K_FluidSim.cuh ---- */

/* replaces gCalcMassDensity, K_FluidSim.cuh:7-16 / K_FluidSim.cu:488-518 */
void gCalcMassDensity(float4 *orderedPositions, float2 *mass_pressure, unsigned int *hashTable,
                      unsigned int *gridStart, unsigned int *gridEnd, int numParticles, float gasConstant,
                      float restDensity, float mass);

/* replaces gInitializeKernelParams, K_FluidSim.cuh:18-19 / K_FluidSim.cu:602-609 */
void gInitializeKernelParams(fgr_kernels_cache _hKernelsCache);

/* replaces gSPHCalculateForces, K_FluidSim.cuh:21-32 / K_FluidSim.cu:527-566 */
void gSPHCalculateForces(float4 *orderedPositions, float4 *orderedVelocity, float4 *forces,
                         float2 *density_pressure, unsigned int *gridStart, unsigned int *gridEnd, float4 *vel,
                         unsigned int *particleId, unsigned int numParticles, float mass, float viscosity);

/* replaces gSPHIntegrate, K_FluidSim.cuh:34-41 / K_FluidSim.cu:571-586 */
void gSPHIntegrate(float4 *_in_sph_positions, float4 *_in_sph_velocity, float4 *_in_sph_forces,
                   unsigned int _in_num_particles, float2 *_in_density_press, unsigned int *_in_grid_start,
                   unsigned int *_in_grid_end);

/* replaces gInitializeCommonFluidParams, K_FluidSim.cuh:43-44 / K_FluidSim.cu:591-597 */
void gInitializeCommonFluidParams(fgr_common_fluid_params hFluidParams);

/* replaces gSPHCalculateForcesWithSRB, K_FluidSim.cuh:46-78 / K_FluidSim.cu:615-680 */
void gSPHCalculateForcesWithSRB(float4 *oldPositions, float4 *oldVelocity, float4 *forces, float4 *newVel,
                                float2 *density_pressure, unsigned int *particleId, unsigned int *gridStart,
                                unsigned int *gridEnd, unsigned int numParticles, float mass, float kViscosity,
                                float _in_sph_particle_radius, int3 _in_cell_size_relation,
                                float _in_srb_particle_radius, float3 _in_srb_cell_size, float _in_kspring,
                                float _in_kdamping, float4 *_in_srb_positions, unsigned int *_in_srb_start_offset,
                                unsigned int *_in_srb_end_offset, unsigned int _in_srb_num_buckets,
                                float4 *_in_rb_positions, float4 *_in_rb_velocities,
                                unsigned int *_in_rb_start_offset, unsigned int *_in_rb_end_offset,
                                unsigned int _in_rb_num_buckets, bool useStaticRB, bool useDynamicRB);

/* replaces gSort, K_FluidSim.cuh:81 / K_FluidSim.cu:685-691 (thrust::sort_by_key) */
void gSort(unsigned int *_key, unsigned int *_values, int _numParticles);

/* ---- K_RigidBodySim.cuh ---- */

/* replaces gCalculateRigidBodyForcesFromRB, K_RigidBodySim.cuh:5-24 / K_RigidBodySim.cu:273-303 */
void gCalculateRigidBodyForcesFromRB(float4 *_in_RBPositions, float4 *_in_RBVelocites, float4 *_in_RBCMPosition,
                                     float4 *_out_torque, float4 *_out_Forces, unsigned int *_in_RBGridStart,
                                     unsigned int *_in_RBGridEnd, unsigned int _in_NumParticles, float3 _in_CellSize,
                                     float _in_Radius, int _in_RBHashTableSize, int _in_SRBHashTableSize,
                                     float4 *_in_SRBPositions, unsigned int *_in_SRBGridStart,
                                     unsigned int *_in_SRBGridEnd, float _in_RBkSpring, float _in_RBkDamping,
                                     int _in_numSRB);

/* replaces gCalculateRigidBodyForcesFromFluids, K_RigidBodySim.cuh:27-50 / K_RigidBodySim.cu:309-342 */
void gCalculateRigidBodyForcesFromFluids(float4 *_in_RBPositions, float4 *_in_RBVelocites, float4 *_in_RBCMPos,
                                         float4 *_out_Forces, float4 *_out_torque, unsigned int *_in_RBGridStart,
                                         unsigned int *_in_RBGridEnd, unsigned int _in_NumParticles,
                                         float3 _in_CellSize, float _in_Radius, int _in_RBHashTableSize,
                                         float4 *_in_sph_particles, float4 *_in_sph_velocities,
                                         unsigned int *_in_sph_grid_start, unsigned int *_in_sph_grid_end,
                                         float _in_sph_particle_radius, float3 _in_sph_cell_size,
                                         unsigned int _in_sph_num_buckets, int3 _in_cell_size_relation,
                                         float _in_sph_kSpring, float _in_sph_kDamping);

/* replaces gCopyRBDataToParticle, K_RigidBodySim.cuh:52-55 / K_RigidBodySim.cu:344-352 */
void gCopyRBDataToParticle(unsigned int *_out_force_rb, unsigned int *_out_force_index,
                           float4 *_in_rb_particle_forces, size_t num_particles);

/* replaces gReorderForceTorque, K_RigidBodySim.cuh:57-59 / K_RigidBodySim.cu:354-366 */
void gReorderForceTorque(float4 *_out_force, float4 *_out_torque, float4 *_in_force, float4 *_in_torque,
                         unsigned int *_in_ordered_index, unsigned int _num_values);

/* replaces gAddForceTorque, K_RigidBodySim.cuh:61-63 / K_RigidBodySim.cu:368-377 */
void gAddForceTorque(float4 *_in_sum_force, float4 *_in_sum_torque, float4 *_in_ordened_force,
                     float4 *_out_to_force, float4 *_out_to_torque, int *_in_sum_offset, size_t num_rigid_body);

/* replaces gIntegrateRB, K_RigidBodySim.cuh:64-67 / K_RigidBodySim.cu:381-392 */
void gIntegrateRB(float4 *_in_RBPosition, float *_in_mass, float4 *_in_RBVelocities, float4 *_in_rbforces,
                  size_t num_rb, float _elapsed_time_in_seconds, float4 _in_external_force, float3 min_volume,
                  float3 max_volume, float4 *_angular_momentum, float4 *_torque, float4 *_inertia_tensor,
                  float4 *_orientation, float4 *_inv_inertia_tensor, float velocity_limit);

/* ---- stand-ins for the CUDPP calls of RigidBodySimulator.cpp ---- */

/* replaces cudppSort(plan, keys, values, keyBits, n) (key/value radix sort,
 * RigidBodySimulator.cpp:195-196, 469-470, 542-543): stable, in place */
void fgc_sort_pairs(unsigned int *keys, unsigned int *values, unsigned int keyBits, unsigned int n);

/* replaces cudppSegmentedScan (CUDPP_FLOAT4, CUDPP_ADD, forward inclusive,
 * RigidBodySimulator.cpp:279-285, 551-554) */
void fgc_segmented_scan_float4(float4 *out, const float4 *in, const unsigned int *flags, unsigned int n);

/* status of the last launcher call on this thread: 0 ok, else an fg_status */
int fgc_last_status(void);

#ifdef __cplusplus
}
#endif

#endif
