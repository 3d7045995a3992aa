/* Drop-in launchers with the reference's extern "C" names and signatures
 * (declared in include/fluidgrid_reference.h).  Each builds a one-scene
 * FgScene from the parameters the reference uses for that launcher -- the
 * arguments, plus CommonFluidParams/KernelsCache stored by
 * gInitializeCommonFluidParams/gInitializeKernelParams as the reference keeps
 * them in __constant__ memory and in its ApplicationData singleton
 * (K_FluidSim.cu:37-40, 502-507) -- and launches the GB300 kernels on the
 * legacy default stream. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <mutex>
#include "fg_types.h"
#include "fg_kernels.h"
#include "fg_engine.h"
#include "../../include/fluidgrid_gb300.h"
#include "../../include/fluidgrid_reference.h"

namespace {

fgr_common_fluid_params g_params;
fgr_kernels_cache g_kc;
bool g_have_params = false, g_have_kc = false;
std::mutex g_mu;
thread_local int g_status = 0;

struct SortCache {
    uint32_t *k = nullptr, *v = nullptr, *h = nullptr;
    size_t cap = 0;
} g_sort;

bool is_pow2(uint32_t v) { return v && !(v & (v - 1)); }

/* one-scene FgScene from the stored CommonFluidParams + KernelsCache */
FgScene fluid_scene()
{
    FgScene S;
    memset(&S, 0, sizeof(S));
    const fgr_common_fluid_params &p = g_params;
    S.cell[0] = p.cell_size.x; S.cell[1] = p.cell_size.y; S.cell[2] = p.cell_size.z;
    S.nb = (uint32_t)(p.bucket_size.x * p.bucket_size.y * p.bucket_size.z);
    S.nb_mask = is_pow2(S.nb) ? S.nb - 1 : 0;
    S.h = p.kernel_radius;
    S.h2 = p.kernel_radius_squared;
    S.scale = p.simulation_scale;
    S.dt = p.deltaTimeIntegration;
    S.dt_over_scale = p.deltaTimeIntegration / p.simulation_scale;
    S.vlimit = p.velocity_limit;
    S.vmin[0] = p.volume_min.x; S.vmin[1] = p.volume_min.y; S.vmin[2] = p.volume_min.z;
    S.vmax[0] = p.volume_max.x; S.vmax[1] = p.volume_max.y; S.vmax[2] = p.volume_max.z;
    S.gravity[0] = p.global_external_force.x;
    S.gravity[1] = p.global_external_force.y;
    S.gravity[2] = p.global_external_force.z;
    S.kpoly6 = g_kc.kPoly6;
    S.kspiky = g_kc.kSpikyGradient;
    S.kvisc = g_kc.kViscosityLaplacian;
    /* literals of SPHCalculateForcesK (K_FluidSim.cu:289-293) */
    S.wall_dist = 0.003043174f;
    S.wall_stiff = 20000.0f;
    S.wall_damp = 256.0f;
    S.noslip_min[0] = -11.0f; S.noslip_min[1] = -40.0f; S.noslip_min[2] = -11.0f;
    S.noslip_max[0] = 11.0f; S.noslip_max[1] = 200.0f; S.noslip_max[2] = 11.0f;
    S.fric_kin = 0.0f;
    S.fric_static = 0.0f;
    return S;
}

fg::Launch single_launch(const FgScene *S, uint32_t n)
{
    fg::Launch L{}; /* default launch shape: 64 CTAs of 128 threads per SM */
    L.table = nullptr;
    L.single = S;
    L.work = nullptr;
    L.nwork = (n + FG_CHUNK - 1) / FG_CHUNK;
    L.n = n;
    L.stream = 0;
    return L;
}

void finish()
{
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        fg::set_error("launcher", e);
        g_status = FG_E_CUDA;
    } else {
        g_status = FG_OK;
    }
}

int ensure_sort(size_t n)
{
    if (n <= g_sort.cap) return FG_OK;
    cudaFree(g_sort.k);
    cudaFree(g_sort.v);
    cudaFree(g_sort.h);
    g_sort.k = g_sort.v = g_sort.h = nullptr;
    g_sort.cap = 0;
    if (cudaMalloc(&g_sort.k, 4 * n) != cudaSuccess || cudaMalloc(&g_sort.v, 4 * n) != cudaSuccess ||
        cudaMalloc(&g_sort.h, 4 * fg::radix_hist_words((uint32_t)n)) != cudaSuccess) {
        fg::set_error_msg("gSort scratch allocation failed");
        return FG_E_OOM;
    }
    g_sort.cap = n;
    return FG_OK;
}

void sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t bits, uint32_t n)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!n) { g_status = FG_OK; return; }
    int r = ensure_sort(n);
    if (r != FG_OK) { g_status = r; return; }
    fg::RadixScratch rs{g_sort.k, g_sort.v, g_sort.h};
    fg::radix_sort(keys, vals, keys, vals, n, bits, 8, rs, 0);
    finish();
}

} // namespace

extern "C" {

void gInitializeCommonFluidParams(fgr_common_fluid_params hFluidParams)
{
    g_params = hFluidParams;
    g_have_params = true;
    g_status = FG_OK;
}

void gInitializeKernelParams(fgr_kernels_cache _hKernelsCache)
{
    g_kc = _hKernelsCache;
    g_have_kc = true;
    g_status = FG_OK;
}

void gCalcHashKey(unsigned int *hashKey, unsigned int *particleID, float4 *positions, unsigned int numParticles,
                  unsigned int numBuckets, float3 cell_size)
{
    if (!numParticles) { g_status = FG_OK; return; }
    if (!numBuckets) { g_status = FG_E_INVALID; return; }
    FgScene S;
    memset(&S, 0, sizeof(S));
    S.cell[0] = cell_size.x; S.cell[1] = cell_size.y; S.cell[2] = cell_size.z;
    S.nb = numBuckets;
    S.nb_mask = is_pow2(numBuckets) ? numBuckets - 1 : 0;
    fg::launch_hash(single_launch(&S, numParticles), positions, hashKey, particleID);
    finish();
}

void gCalcHashKeyWithOffset(unsigned int *_out_hashKey, unsigned int *_out_particleID, float4 *_in_vectorOffset,
                            float4 *_in_orientation, float4 *_in_vectorPos, float4 *_out_positions,
                            unsigned int _in_numParticles, float3 _in_cellSize, int _in_hashTableSize)
{
    if (!_in_numParticles) { g_status = FG_OK; return; }
    if (_in_hashTableSize <= 0) { g_status = FG_E_INVALID; return; }
    FgScene S;
    memset(&S, 0, sizeof(S));
    S.rb_cell[0] = _in_cellSize.x; S.rb_cell[1] = _in_cellSize.y; S.rb_cell[2] = _in_cellSize.z;
    S.rb_nb = (uint32_t)_in_hashTableSize;
    S.rb_nb_mask = is_pow2(S.rb_nb) ? S.rb_nb - 1 : 0;
    fg::launch_hash_with_offset(single_launch(&S, _in_numParticles), _in_vectorPos, _in_vectorOffset, _in_orientation,
                                _out_positions, _out_hashKey, _out_particleID, nullptr);
    finish();
}

void gFindCellOffsetOrderingPosVel(unsigned int *gridPosStart, unsigned int *gridPosEnd, unsigned int *hashTable,
                                   unsigned int *particleID, float4 *particlePositions,
                                   float4 *orderedParticlePositions, float4 *particleVel, float4 *particleOrderedVel,
                                   unsigned int numParticles, unsigned int numBuckets)
{
    cudaMemsetAsync(gridPosStart, 0xff, 4 * (size_t)numBuckets, 0);
    fg::launch_cell_ranges(hashTable, particleID, particlePositions, particleVel, gridPosStart, gridPosEnd,
                           orderedParticlePositions, particleOrderedVel, numParticles, 0);
    finish();
}

void gFindCellOffsetOrderingPos(unsigned int *gridPosStart, unsigned int *gridPosEnd, unsigned int *hashTable,
                                unsigned int *particleID, float4 *particlePositions, float4 *orderedParticlePositions,
                                unsigned int numParticles, unsigned int numBuckets)
{
    cudaMemsetAsync(gridPosStart, 0xff, 4 * (size_t)numBuckets, 0);
    fg::launch_cell_ranges(hashTable, particleID, particlePositions, nullptr, gridPosStart, gridPosEnd,
                           orderedParticlePositions, nullptr, numParticles, 0);
    finish();
}

void gSort(unsigned int *_key, unsigned int *_values, int _numParticles)
{
    if (_numParticles < 0) { g_status = FG_E_INVALID; return; }
    sort_pairs(_key, _values, 32, (uint32_t)_numParticles);
}

void gCalcMassDensity(float4 *orderedPositions, float2 *mass_pressure, unsigned int *hashTable,
                      unsigned int *gridStart, unsigned int *gridEnd, int numParticles, float gasConstant,
                      float restDensity, float mass)
{
    (void)hashTable;
    if (!g_have_params || !g_have_kc) { g_status = FG_E_STATE; return; }
    if (numParticles <= 0) { g_status = FG_OK; return; }
    FgScene S = fluid_scene();
    fg::launch_density(single_launch(&S, (uint32_t)numParticles), orderedPositions, gridStart, gridEnd,
                       mass_pressure, gasConstant, restDensity, mass, 1);
    finish();
}

void gSPHCalculateForces(float4 *orderedPositions, float4 *orderedVelocity, float4 *forces,
                         float2 *density_pressure, unsigned int *gridStart, unsigned int *gridEnd, float4 *vel,
                         unsigned int *particleId, unsigned int numParticles, float mass, float viscosity)
{
    (void)forces;
    if (!g_have_params || !g_have_kc) { g_status = FG_E_STATE; return; }
    if (!numParticles) { g_status = FG_OK; return; }
    FgScene S = fluid_scene();
    fg::ForceOut o;
    o.vel = vel;
    o.pos = nullptr;
    fg::launch_forces(single_launch(&S, numParticles), orderedPositions, orderedVelocity, density_pressure, gridStart,
                      gridEnd, particleId, o, nullptr, nullptr, mass, viscosity, 1);
    finish();
}

void gSPHIntegrate(float4 *_in_sph_positions, float4 *_in_sph_velocity, float4 *_in_sph_forces,
                   unsigned int _in_num_particles, float2 *_in_density_press, unsigned int *_in_grid_start,
                   unsigned int *_in_grid_end)
{
    (void)_in_sph_forces; (void)_in_density_press; (void)_in_grid_start; (void)_in_grid_end;
    if (!g_have_params) { g_status = FG_E_STATE; return; }
    if (!_in_num_particles) { g_status = FG_OK; return; }
    FgScene S = fluid_scene();
    fg::launch_integrate(single_launch(&S, _in_num_particles), _in_sph_positions, _in_sph_velocity);
    finish();
}

void gSPHCalculateForcesWithSRB(float4 *oldPositions, float4 *oldVelocity, float4 *forces, float4 *newVel,
                                float2 *density_pressure, unsigned int *particleId, unsigned int *gridStart,
                                unsigned int *gridEnd, unsigned int numParticles, float mass, float kViscosity,
                                float _in_sph_particle_radius, int3 _in_cell_size_relation,
                                float _in_srb_particle_radius, float3 _in_srb_cell_size, float _in_kspring,
                                float _in_kdamping, float4 *_in_srb_positions, unsigned int *_in_srb_start_offset,
                                unsigned int *_in_srb_end_offset, unsigned int _in_srb_num_buckets,
                                float4 *_in_rb_positions, float4 *_in_rb_velocities,
                                unsigned int *_in_rb_start_offset, unsigned int *_in_rb_end_offset,
                                unsigned int _in_rb_num_buckets, bool useStaticRB, bool useDynamicRB)
{
    (void)forces;
    if (!g_have_params || !g_have_kc) { g_status = FG_E_STATE; return; }
    if (!numParticles) { g_status = FG_OK; return; }
    /* search half-widths of 0..8 cells per axis, as for world scenes */
    if (_in_cell_size_relation.x < 0 || _in_cell_size_relation.x > 8 || _in_cell_size_relation.y < 0 ||
        _in_cell_size_relation.y > 8 || _in_cell_size_relation.z < 0 || _in_cell_size_relation.z > 8) {
        g_status = FG_E_INVALID;
        return;
    }
    FgScene S = fluid_scene();
    S.fluid_radius = _in_sph_particle_radius;
    S.rb_radius = _in_srb_particle_radius;
    S.rb_cell[0] = _in_srb_cell_size.x; S.rb_cell[1] = _in_srb_cell_size.y; S.rb_cell[2] = _in_srb_cell_size.z;
    S.f2r_rel[0] = _in_cell_size_relation.x;
    S.f2r_rel[1] = _in_cell_size_relation.y;
    S.f2r_rel[2] = _in_cell_size_relation.z;
    S.ck = _in_kspring;
    S.ckd = _in_kdamping;
    S.fluid_eps = 0.003f; /* K_FluidSim.cu:378, 386 */
    S.flags = FG_SCENE_HAS_RB;
    fg::RigidGrid dyn, sta;
    memset(&dyn, 0, sizeof(dyn));
    memset(&sta, 0, sizeof(sta));
    dyn.spos = _in_rb_positions;
    dyn.start = _in_rb_start_offset;
    dyn.end = _in_rb_end_offset;
    dyn.body_vel = _in_rb_velocities;
    dyn.own_geometry = 1;
    dyn.nb = _in_rb_num_buckets;
    dyn.mask = is_pow2(_in_rb_num_buckets) ? _in_rb_num_buckets - 1 : 0;
    sta.spos = _in_srb_positions;
    sta.start = _in_srb_start_offset;
    sta.end = _in_srb_end_offset;
    sta.own_geometry = 1;
    sta.nb = _in_srb_num_buckets;
    sta.mask = is_pow2(_in_srb_num_buckets) ? _in_srb_num_buckets - 1 : 0;
    fg::ForceOut o;
    o.vel = newVel;
    o.pos = nullptr;
    fg::launch_forces(single_launch(&S, numParticles), oldPositions, oldVelocity, density_pressure, gridStart,
                      gridEnd, particleId, o, useDynamicRB ? &dyn : nullptr, useStaticRB ? &sta : nullptr, mass,
                      kViscosity, 1);
    finish();
}

void gCalculateRigidBodyForcesFromRB(float4 *_in_RBPositions, float4 *_in_RBVelocites, float4 *_in_RBCMPosition,
                                     float4 *_out_torque, float4 *_out_Forces, unsigned int *_in_RBGridStart,
                                     unsigned int *_in_RBGridEnd, unsigned int _in_NumParticles, float3 _in_CellSize,
                                     float _in_Radius, int _in_RBHashTableSize, int _in_SRBHashTableSize,
                                     float4 *_in_SRBPositions, unsigned int *_in_SRBGridStart,
                                     unsigned int *_in_SRBGridEnd, float _in_RBkSpring, float _in_RBkDamping,
                                     int _in_numSRB)
{
    if (!_in_NumParticles) { g_status = FG_OK; return; }
    FgScene S;
    memset(&S, 0, sizeof(S));
    S.rb_cell[0] = _in_CellSize.x; S.rb_cell[1] = _in_CellSize.y; S.rb_cell[2] = _in_CellSize.z;
    S.rb_nb = (uint32_t)_in_RBHashTableSize;
    S.rb_nb_mask = is_pow2(S.rb_nb) ? S.rb_nb - 1 : 0;
    S.rb_radius = _in_Radius;
    S.rbrb_k = _in_RBkSpring;
    S.rbrb_kd = _in_RBkDamping;
    S.rbrb_eps = 0.001f; /* K_RigidBodySim.cu:42, 50 */
    fg::RigidGrid sta;
    memset(&sta, 0, sizeof(sta));
    sta.spos = _in_SRBPositions;
    sta.start = _in_SRBGridStart;
    sta.end = _in_SRBGridEnd;
    sta.own_geometry = 1;
    sta.nb = (uint32_t)_in_SRBHashTableSize;
    sta.mask = is_pow2(sta.nb) ? sta.nb - 1 : 0;
    fg::launch_rb_from_rb(single_launch(&S, _in_NumParticles), _in_RBPositions, nullptr, _in_RBVelocites,
                          _in_RBCMPosition, _in_RBGridStart, _in_RBGridEnd, _out_Forces, _out_torque,
                          _in_numSRB > 0 ? &sta : nullptr, 0);
    finish();
}

void gCalculateRigidBodyForcesFromFluids(float4 *_in_RBPositions, float4 *_in_RBVelocites, float4 *_in_RBCMPos,
                                         float4 *_out_Forces, float4 *_out_torque, unsigned int *_in_RBGridStart,
                                         unsigned int *_in_RBGridEnd, unsigned int _in_NumParticles,
                                         float3 _in_CellSize, float _in_Radius, int _in_RBHashTableSize,
                                         float4 *_in_sph_particles, float4 *_in_sph_velocities,
                                         unsigned int *_in_sph_grid_start, unsigned int *_in_sph_grid_end,
                                         float _in_sph_particle_radius, float3 _in_sph_cell_size,
                                         unsigned int _in_sph_num_buckets, int3 _in_cell_size_relation,
                                         float _in_sph_kSpring, float _in_sph_kDamping)
{
    (void)_in_RBGridStart; (void)_in_RBGridEnd; (void)_in_CellSize; (void)_in_RBHashTableSize;
    if (!_in_NumParticles) { g_status = FG_OK; return; }
    if (!_in_sph_num_buckets) { g_status = FG_E_INVALID; return; }
    FgScene S;
    memset(&S, 0, sizeof(S));
    S.cell[0] = _in_sph_cell_size.x; S.cell[1] = _in_sph_cell_size.y; S.cell[2] = _in_sph_cell_size.z;
    S.nb = _in_sph_num_buckets;
    S.nb_mask = is_pow2(S.nb) ? S.nb - 1 : 0;
    S.r2f_rel[0] = _in_cell_size_relation.x;
    S.r2f_rel[1] = _in_cell_size_relation.y;
    S.r2f_rel[2] = _in_cell_size_relation.z;
    S.rb_radius = _in_Radius;
    S.fluid_radius = _in_sph_particle_radius;
    S.ck = _in_sph_kSpring;
    S.ckd = _in_sph_kDamping;
    S.rb_eps = 0.0001f; /* K_RigidBodySim.cu:87 */
    fg::launch_rb_from_fluid(single_launch(&S, _in_NumParticles), _in_RBPositions, nullptr, _in_RBVelocites,
                             _in_RBCMPos, _in_sph_particles, _in_sph_velocities, _in_sph_grid_start, _in_sph_grid_end,
                             _out_Forces, _out_torque, 0);
    finish();
}

void gCopyRBDataToParticle(unsigned int *_out_force_rb, unsigned int *_out_force_index,
                           float4 *_in_rb_particle_forces, size_t num_particles)
{
    fg::launch_copy_rb_data_to_particle(_out_force_rb, _out_force_index, _in_rb_particle_forces,
                                        (uint32_t)num_particles, 0);
    finish();
}

void gReorderForceTorque(float4 *_out_force, float4 *_out_torque, float4 *_in_force, float4 *_in_torque,
                         unsigned int *_in_ordered_index, unsigned int _num_values)
{
    fg::launch_reorder_force_torque(_out_force, _out_torque, _in_force, _in_torque, _in_ordered_index, _num_values,
                                    0);
    finish();
}

void gAddForceTorque(float4 *_in_sum_force, float4 *_in_sum_torque, float4 *_in_ordened_force,
                     float4 *_out_to_force, float4 *_out_to_torque, int *_in_sum_offset, size_t num_rigid_body)
{
    fg::launch_add_force_torque(_in_sum_force, _in_sum_torque, _in_ordened_force, _out_to_force, _out_to_torque,
                                _in_sum_offset, (uint32_t)num_rigid_body, 0);
    finish();
}

void gIntegrateRB(float4 *_in_RBPosition, float *_in_mass, float4 *_in_RBVelocities, float4 *_in_rbforces,
                  size_t num_rb, float _elapsed_time_in_seconds, float4 _in_external_force, float3 min_volume,
                  float3 max_volume, float4 *_angular_momentum, float4 *_torque, float4 *_inertia_tensor,
                  float4 *_orientation, float4 *_inv_inertia_tensor, float velocity_limit)
{
    fg::launch_integrate_rb_f32(_in_RBPosition, _in_mass, _in_RBVelocities, _in_rbforces, (uint32_t)num_rb,
                                _elapsed_time_in_seconds, _in_external_force, min_volume, max_volume,
                                _angular_momentum, _torque, _inertia_tensor, _orientation, _inv_inertia_tensor,
                                velocity_limit, 0);
    finish();
}

void fgc_sort_pairs(unsigned int *keys, unsigned int *values, unsigned int keyBits, unsigned int n)
{
    if (keyBits > 32) keyBits = 32;
    sort_pairs(keys, values, keyBits, n);
}

void fgc_segmented_scan_float4(float4 *out, const float4 *in, const unsigned int *flags, unsigned int n)
{
    fg::launch_segmented_sum(in, flags, out, n, 0);
    finish();
}

int fgc_last_status(void) { return g_status; }

} /* extern "C" */
