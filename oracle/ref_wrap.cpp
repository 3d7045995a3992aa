/* Test infrastructure, not product code.
 *
 * Compiles the reference's own __device__ helper files verbatim as host C++
 * (through the self-written headers in oracle/ref_shim) and exports C entry
 * points around them.  The result, oracle/_ref/libfgref.so, is built only where
 * the reference sources are present; it produces the golden vectors under
 * tests/golden/ that pin the oracle's restatement of these helpers.
 *
 * Helpers wrapped (paths relative to the reference project):
 *   GPU_Kernels/K_DeviceFunctions.cu:17-26   HashKeyD
 *   GPU_Kernels/K_DeviceFunctions.cu:113-159 ProcessCollisionForcesD (+ ProcessCellForcesD :32-106)
 *   GPU_Kernels/K_Boundaries_Walls.cu:8-65   calculateWallsNoPenetrationForce
 *   GPU_Kernels/K_Boundaries_Walls.cu:68-125 calculateWallsNoSlipForce
 *   GPU_Kernels/K_MathUtils.cu:160-181       Quaternion_ProductD / Quaternion_TransformPointD
 *   GPU_Kernels/K_MathUtils.cu:72-82         Quaternion_NormalizeD
 *   GPU_Kernels/K_MathUtils.cu:211-236       AngularVelocityD
 *   GPU_Kernels/K_MathUtils.cu:57-62         Vec3CrossD
 */
#include "K_DeviceFunctions.cu"
#include "K_Boundaries_Walls.cu"
#include "K_MathUtils.cu"

static float3 f3(const float *p) { return make_float3(p[0], p[1], p[2]); }
static float4 f4(const float *p) { return make_float4(p[0], p[1], p[2], p[3]); }
static void put3(float *o, float3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
static void put4(float *o, float4 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }

extern "C" {

unsigned int ref_hash_key(const float *pos3, const float *cell3, int nbuckets)
{
    return SimulationLib::Common::HashKeyD(f3(pos3), f3(cell3), nbuckets);
}

void ref_walls_no_penetration(const float *pos3, const float *vel3, const float *min3,
                              const float *max3, float bdist, float stiff, float damp,
                              float scale, float *out3)
{
    put3(out3, calculateWallsNoPenetrationForce(f3(pos3), f3(vel3), f3(min3), f3(max3),
                                                bdist, stiff, damp, scale));
}

void ref_walls_no_slip(const float *pos3, const float *vel3, const float *force3,
                       const float *min3, const float *max3, float bdist, float fkin,
                       float fstatic, float scale, float *out3)
{
    put3(out3, calculateWallsNoSlipForce(f3(pos3), f3(vel3), f3(force3), f3(min3), f3(max3),
                                         bdist, fkin, fstatic, scale));
}

/* pos4/vel4: the querying sphere; coll_pos4: sorted collection (float4[n]);
 * coll_vel4: per-particle or per-body velocities (float4) or NULL. */
void ref_process_collision_forces(const float *pos4, const float *vel4, float radius,
                                  const float *coll_pos4, const float *coll_vel4,
                                  float coll_radius, float kspring, float kdamp,
                                  const int *rel3, const unsigned int *start,
                                  const unsigned int *end, const float *cell3,
                                  unsigned int nbuckets, int w_rb_index, int check_group,
                                  int group, float eps, float *out3)
{
    int3 rel = make_int3(rel3[0], rel3[1], rel3[2]);
    float3 r = SimulationLib::Common::ProcessCollisionForcesD(
        f4(pos4), f4(vel4), radius, (float4 *)coll_pos4, (float4 *)coll_vel4, coll_radius,
        kspring, kdamp, rel, (unsigned int *)start, (unsigned int *)end, f3(cell3), nbuckets,
        w_rb_index != 0, check_group != 0, group, eps);
    put3(out3, r);
}

void ref_quat_product(const float *q1, const float *q2, float *out4)
{
    put4(out4, SimulationLib::MathUtils::Quaternion_ProductD(f4(q1), f4(q2)));
}

void ref_quat_transform_point(const float *pos4, const float *q4, float *out4)
{
    put4(out4, SimulationLib::MathUtils::Quaternion_TransformPointD(f4(pos4), f4(q4)));
}

void ref_quat_normalize(const float *q4, float *out4)
{
    put4(out4, SimulationLib::MathUtils::Quaternion_NormalizeD(f4(q4)));
}

void ref_vec3_cross(const float *a4, const float *b4, float *out4)
{
    put4(out4, SimulationLib::MathUtils::Vec3CrossD(f4(a4), f4(b4)));
}

/* inv_inertia12: three float4 rows. */
void ref_angular_velocity(const float *inv_inertia12, const float *L4, const float *q4, float *out4)
{
    float4 rows[3] = {f4(inv_inertia12), f4(inv_inertia12 + 4), f4(inv_inertia12 + 8)};
    float4 r = SimulationLib::MathUtils::AngularVelocityD(rows, f4(L4), f4(q4));
    /* AngularVelocityD leaves .w unset; report 0 like the caller does. */
    r.w = 0.0f;
    put4(out4, r);
}

} /* extern "C" */
