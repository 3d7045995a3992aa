/* Pair terms and rigid contact shared by the SPH force kernels. */
#ifndef FG_SPH_COMMON_CUH
#define FG_SPH_COMMON_CUH

#include "fg_device.cuh"
#include "fg_kernels.h"

namespace fg {

/* Rigid-sphere contact of one fluid particle against a rigid grid
 * (ProcessCollisionForcesD with the per-body velocity of w, eps from the
 * scene).  Skipped when the particle is outside the scene's sphere AABB
 * grown by the contact distance: there every candidate is out of range, so
 * the sum is exactly zero as in the reference. */
__device__ __forceinline__ float3 fg_fluid_rigid_contact(const FgScene *S, uint32_t scene, float4 p, float4 v,
                                                         const RigidGrid &G, bool dynamic)
{
    float3 acc = make_float3(0.f, 0.f, 0.f);
    const float mind = S->fluid_radius + S->rb_radius + S->fluid_eps;
    if (G.aabb) {
        const int *bx = G.aabb + 6 * scene;
        if (p.x < fg_ord_float(bx[0]) - mind || p.y < fg_ord_float(bx[1]) - mind ||
            p.z < fg_ord_float(bx[2]) - mind || p.x > fg_ord_float(bx[3]) + mind ||
            p.y > fg_ord_float(bx[4]) + mind || p.z > fg_ord_float(bx[5]) + mind)
            return acc;
    }
    const float3 P = make_float3(p.x, p.y, p.z);
    const float3 V = make_float3(v.x, v.y, v.z);
    const int rx = S->f2r_rel[0], ry = S->f2r_rel[1], rz = S->f2r_rel[2];
    for (int z = -rz; z <= rz; z++) {
        const uint32_t hz = fg_axis_hash_rel(p.z, S->rb_cell[2], z, FG_PZ);
        for (int y = -ry; y <= ry; y++) {
            const uint32_t hy = fg_axis_hash_rel(p.y, S->rb_cell[1], y, FG_PY);
            for (int x = -rx; x <= rx; x++) {
                const uint32_t hx = fg_axis_hash_rel(p.x, S->rb_cell[0], x, FG_PX);
                const uint32_t b = G.own_geometry ? fg_bucket(hx, hy, hz, G.nb, G.mask)
                                                  : S->rb_bucket_base + fg_bucket(hx, hy, hz, S->rb_nb, S->rb_nb_mask);
                const uint32_t st = __ldg(G.start + b);
                if (st == FG_EMPTY) continue;
                const uint32_t en = __ldg(G.end + b);
                for (uint32_t j = st; j < en; j++) {
                    const float4 q = __ldg(G.spos + j);
                    const float4 vq = dynamic ? __ldg(G.body_vel + (int)q.w) : make_float4(0.f, 0.f, 0.f, 0.f);
                    fg_contact(acc, P, V, q, vq, mind, S->ck, S->ckd);
                }
            }
        }
    }
    return acc;
}

/* Pressure + viscosity of neighbour j on i (SPHCalculatePressureForceD +
 * SPHCalculateViscosityForceD): d = p_i - p_j (scaled), r2 = |d|^2 <= h^2. */
__device__ __forceinline__ void fg_pair(float &fx, float &fy, float &fz, float dx, float dy, float dz, float r2,
                                        float h, float kspiky, float kv, float rho_i, float P_i, float4 vi,
                                        float rho_j, float P_j, float4 vj)
{
    const float il = rsqrtf(r2);
    const float l = r2 * il;
    const float hl = h - l;
    const float irr = __frcp_rn(rho_i * rho_j);
    /* pressure: -(d/l) kSpiky (h-l)^2 (Pi+Pj)/(rho_i rho_j) */
    const float cp = -(kspiky * hl * hl) * ((P_i + P_j) * irr) * il;
    /* viscosity: (vj-vi)/(rho_i rho_j) kVisc (h-l) mu */
    const float cv = (kv * hl) * irr;
    fx += dx * cp + (vj.x - vi.x) * cv;
    fy += dy * cp + (vj.y - vi.y) * cv;
    fz += dz * cp + (vj.z - vi.z) * cv;
}

/* Tail of SPHCalculateForcesK / SPHCalculateForcesWithSRBK
 * (K_FluidSim.cu:287-307, 389-411): F = internal*mass + gravity (+ rigid
 * contact), walls, force clamp, newVel[id] = vel + F*dt, optional fused
 * SPHIntegrateK (:438) with each operation rounded on its own. */
__device__ __forceinline__ void fg_force_tail(const FgScene *S, uint32_t scene, float4 p, float4 v, bool active,
                                              float fx, float fy, float fz, float mass, const RigidGrid *dyn,
                                              const RigidGrid *sta, uint32_t oi, float4 *__restrict__ vel_out,
                                              float4 *__restrict__ pos_out)
{
    float3 F = make_float3(0.f, 0.f, 0.f);
    if (active) {
        F = make_float3(fx * mass + S->gravity[0], fy * mass + S->gravity[1], fz * mass + S->gravity[2]);
        if (sta) {
            const float3 c = fg_fluid_rigid_contact(S, scene, p, v, *sta, false);
            F.x += c.x; F.y += c.y; F.z += c.z;
        }
        if (dyn && (S->flags & FG_SCENE_HAS_RB)) {
            const float3 c = fg_fluid_rigid_contact(S, scene, p, v, *dyn, true);
            F.x += c.x; F.y += c.y; F.z += c.z;
        }
        const float3 wl = fg_walls(*S, make_float3(p.x, p.y, p.z), make_float3(v.x, v.y, v.z));
        F.x += wl.x; F.y += wl.y; F.z += wl.z;
        const float speed = sqrtf(F.x * F.x + F.y * F.y + F.z * F.z);
        if (speed > S->vlimit) {
            const float t = S->vlimit / speed;
            F.x *= t; F.y *= t; F.z *= t;
        }
    }
    const float dt = S->dt;
    float4 nv;
    nv.x = v.x + F.x * dt;
    nv.y = v.y + F.y * dt;
    nv.z = v.z + F.z * dt;
    nv.w = v.w + 0.0f;
    vel_out[oi] = nv;
    if (pos_out && active) {
        const float c = S->dt_over_scale;
        float4 np;
        np.x = __fadd_rn(p.x, __fmul_rn(nv.x, c));
        np.y = __fadd_rn(p.y, __fmul_rn(nv.y, c));
        np.z = __fadd_rn(p.z, __fmul_rn(nv.z, c));
        np.w = __fadd_rn(p.w, __fmul_rn(nv.w, c));
        pos_out[oi] = np;
    }
}

} // namespace fg

#endif
