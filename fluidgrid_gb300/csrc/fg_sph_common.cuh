/* Neighbour walks, pair terms and rigid contact shared by the SPH kernels. */
#ifndef FG_SPH_COMMON_CUH
#define FG_SPH_COMMON_CUH

#include "fg_device.cuh"
#include "fg_kernels.h"

namespace fg {

/* Visit the particles of the 27 neighbour buckets in the reference's order
 * (z outer, x inner, each from -1 to 1; ascending sorted index inside a
 * bucket).  The buckets are taken a row (three x offsets) at a time: the
 * row's three start and three end words are loaded together, so a row costs
 * one memory latency instead of six dependent ones.  One runtime loop with
 * the per-axis hashes selected from registers keeps the code compact (an
 * unrolled walk multiplies the body 27 times and thrashes the instruction
 * cache) and uses no local memory. */
template <typename Fn, typename End>
__device__ __forceinline__ void fg_walk27(float px, float py, float pz, const FgScene *S,
                                          const uint32_t *__restrict__ start, const uint32_t *__restrict__ end,
                                          Fn &&fn, End &&bucket_end)
{
    uint32_t hx[3], hy[3], hz[3];
    fg_neighbour_hashes(px, py, pz, S->cell, hx, hy, hz);
    const uint32_t hx0 = hx[0], hx1 = hx[1], hx2 = hx[2], hy0 = hy[0], hy1 = hy[1], hy2 = hy[2];
    const uint32_t hz0 = hz[0], hz1 = hz[1], hz2 = hz[2];
    const uint32_t nb = S->nb, mask = S->nb_mask, bb = S->bucket_base;
#pragma unroll 1
    for (int r = 0; r < 9; r++) {
        const uint32_t yh = fg_sel3(hy0, hy1, hy2, r % 3), zh = fg_sel3(hz0, hz1, hz2, r / 3);
        const uint32_t b0 = bb + fg_bucket(hx0, yh, zh, nb, mask);
        const uint32_t b1 = bb + fg_bucket(hx1, yh, zh, nb, mask);
        const uint32_t b2 = bb + fg_bucket(hx2, yh, zh, nb, mask);
        const uint32_t s0 = __ldg(start + b0), s1 = __ldg(start + b1), s2 = __ldg(start + b2);
        const uint32_t e0 = __ldg(end + b0), e1 = __ldg(end + b1), e2 = __ldg(end + b2);
#pragma unroll 1
        for (int x = 0; x < 3; x++) {
            const uint32_t st = fg_sel3(s0, s1, s2, x);
            if (st == FG_EMPTY) continue; /* end of an empty bucket is stale */
            const uint32_t en = fg_sel3(e0, e1, e2, x);
#pragma unroll 2
            for (uint32_t j = st; j < en; j++) fn(j);
            bucket_end();
        }
    }
}

/* The same walk with nothing to do at the end of a bucket. */
template <typename Fn>
__device__ __forceinline__ void fg_walk27(float px, float py, float pz, const FgScene *S,
                                          const uint32_t *__restrict__ start, const uint32_t *__restrict__ end,
                                          Fn &&fn)
{
    fg_walk27(px, py, pz, S, start, end, fn, [] {});
}

/* One target's state in a density pass: the sum of (h^2 - l^2)^3 over the
 * candidates with l <= h (an exact 0 at l = h, so the sum equals the
 * reference's l < h sum) and the force pass's neighbour list (every visit
 * with l <= h, the target's own entries included: testing j != i in the
 * force pass, which waits on memory, is cheaper than in this issue-bound
 * branch), stored two entries (8 bytes) at a time.  The terms of one bucket
 * (a few in range) are added plainly; each bucket's partial is then added to
 * the total with Kahan compensation, which keeps the hot in-range branch to
 * one addition.  Every operation is rounded on its own, so any kernel that
 * visits the same candidates in the same order produces the same bits. */
struct DensityAcc {
    float s, c;          /* Kahan sum and compensation over bucket partials */
    float b;             /* plain sum of the current bucket's terms */
    uint32_t dcnt, cnt;  /* density visits (without a list), list entries */
    uint32_t q2, q3;     /* the last two list entries (q3 the newest) */

    __device__ __forceinline__ void init()
    {
        s = c = b = 0.0f;
        dcnt = cnt = 0;
        q2 = q3 = 0;
    }

    /* fold the finished bucket's partial into the compensated total */
    __device__ __forceinline__ void end_bucket()
    {
        const float y = __fsub_rn(b, c);
        const float u = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(u, s), y);
        s = u;
        b = 0.0f;
    }

    template <bool LIST>
    __device__ __forceinline__ void visit(float4 q, uint32_t j, float px, float py, float pz, float scale, float h2,
                                          uint32_t *lp, uint32_t cap)
    {
        const float dx = fmaf(-q.x, scale, px), dy = fmaf(-q.y, scale, py), dz = fmaf(-q.z, scale, pz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
        if (r2 <= h2) {
            const float t = __fsub_rn(h2, r2);
            b = __fadd_rn(b, __fmul_rn(__fmul_rn(t, t), t));
            if (!LIST) dcnt++; /* with a list every visit is an entry: cnt counts them */
            if (LIST) {
                q2 = q3;
                q3 = j;
                cnt++;
                if ((cnt & 1u) == 0u && cnt <= cap) fg_st_list2(lp + cnt - 2u, q2, q3);
            }
        }
    }

    /* store an odd last entry (q3) and pad the list to a whole group of
     * four with the target's own index, which the force pass skips, so it
     * reads only whole groups */
    __device__ __forceinline__ void flush(uint32_t *lp, uint32_t cap, uint32_t self) const
    {
        if (cnt > cap) return;
        const uint32_t r = cnt & 3u;
        if (r == 1u) {
            fg_st_list2(lp + cnt - 1u, q3, self);
            fg_st_list2(lp + cnt + 1u, self, self);
        } else if (r == 2u) {
            fg_st_list2(lp + cnt, self, self);
        } else if (r == 3u) {
            fg_st_list2(lp + cnt - 1u, q3, self);
        }
    }
};

/* CalculateMassDensityK's output (K_FluidSim.cu:244-251): (max(1, rho),
 * k (rho - rho0)) with rho = m kPoly6 sum, each operation rounded alone. */
__device__ __forceinline__ float2 fg_density_out(float mass, float kpoly6, float gas, float rest, float sum)
{
    const float rho = __fmul_rn(__fmul_rn(mass, kpoly6), sum);
    return make_float2(fmaxf(1.0f, rho), __fmul_rn(gas, __fsub_rn(rho, rest)));
}

/* scene owning a global bucket key (scenes are ordered by bucket_base) */
__device__ __forceinline__ uint32_t cc_scene_of(const FgScene *table, uint32_t nscenes, uint32_t key)
{
    if (!table) return 0;
    uint32_t lo = 0, hi = nscenes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&table[mid].bucket_base) <= key) lo = mid;
        else hi = mid;
    }
    return lo;
}

/* The 9 per-axis neighbour cell indices that determine a particle's 27
 * buckets (fg_neighbour_hashes before the prime products). */
struct Sig {
    int v[9];
};

__device__ __forceinline__ Sig cc_sig(float px, float py, float pz, const float *cell)
{
    Sig s;
#pragma unroll
    for (int o = -1; o <= 1; o++) {
        s.v[o + 1] = fg_axis_index_off(px, cell[0], o);
        s.v[o + 4] = fg_axis_index_off(py, cell[1], o);
        s.v[o + 7] = fg_axis_index_off(pz, cell[2], o);
    }
    return s;
}

/* Lanes 0..26 return bucket k = lane's (z, y, x) = (lane/9, lane/3 % 3,
 * lane % 3) start and count; lanes 27..31 return count 0. */
__device__ __forceinline__ void cc_bucket_of_lane(const Sig &s, const FgScene *S, const uint32_t *__restrict__ start,
                                                  const uint32_t *__restrict__ end, int lane, uint32_t &st,
                                                  uint32_t &cnt)
{
    st = 0;
    cnt = 0;
    if (lane < 27) {
        const int z = lane / 9, y = (lane / 3) % 3, x = lane % 3;
        const uint32_t hx = fg_sel3((uint32_t)s.v[0], (uint32_t)s.v[1], (uint32_t)s.v[2], x) * FG_PX;
        const uint32_t hy = fg_sel3((uint32_t)s.v[3], (uint32_t)s.v[4], (uint32_t)s.v[5], y) * FG_PY;
        const uint32_t hz = fg_sel3((uint32_t)s.v[6], (uint32_t)s.v[7], (uint32_t)s.v[8], z) * FG_PZ;
        const uint32_t b = S->bucket_base + fg_bucket(hx, hy, hz, S->nb, S->nb_mask);
        const uint32_t a = __ldg(start + b);
        const uint32_t z1 = __ldg(end + b); /* independent of `a`: one memory latency, not two */
        if (a != FG_EMPTY) {
            st = a;
            cnt = z1 - a;
        }
    }
}

__device__ __forceinline__ uint32_t cc_excl_scan(uint32_t v, int lane, uint32_t &total)
{
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

__device__ __forceinline__ float cc_sum(float v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* widest search half-width whose bucket rows the contact walk loads together */
#define FG_CONTACT_ROW_MAX 2

/* Whether a fluid particle lies outside the bodies' AABB of its scene grown
 * by the contact distance: its contact sum is then exactly zero. */
/* Rigid-sphere contact of one fluid particle against a rigid grid
 * (ProcessCollisionForcesD with the per-body velocity of w, eps from the
 * scene).  Skipped when the particle is outside the scene's sphere AABB
 * grown by the contact distance: there every candidate is out of range, so
 * the sum is exactly zero as in the reference. */
__device__ __forceinline__ bool fg_contact_outside(const FgScene *S, uint32_t scene, float4 p, const RigidGrid &G)
{
    if (!G.aabb) return false;
    const float mind = S->fluid_radius + S->rb_radius + S->fluid_eps;
    const int *bx = G.aabb + 6 * scene;
    return p.x < fg_ord_float(bx[0]) - mind || p.y < fg_ord_float(bx[1]) - mind ||
           p.z < fg_ord_float(bx[2]) - mind || p.x > fg_ord_float(bx[3]) + mind ||
           p.y > fg_ord_float(bx[4]) + mind || p.z > fg_ord_float(bx[5]) + mind;
}

__device__ __forceinline__ float3 fg_fluid_rigid_contact(const FgScene *S, uint32_t scene, float4 p, float4 v,
                                                         const RigidGrid &G, bool dynamic)
{
    float3 acc = make_float3(0.f, 0.f, 0.f);
    const float mind = S->fluid_radius + S->rb_radius + S->fluid_eps;
    if (fg_contact_outside(S, scene, p, G)) return acc;
    const float3 P = make_float3(p.x, p.y, p.z);
    const float3 V = make_float3(v.x, v.y, v.z);
    const int rx = S->f2r_rel[0], ry = S->f2r_rel[1], rz = S->f2r_rel[2];
    auto bucket = [&](uint32_t hx, uint32_t hy, uint32_t hz) {
        return G.own_geometry ? fg_bucket(hx, hy, hz, G.nb, G.mask)
                              : S->rb_bucket_base + fg_bucket(hx, hy, hz, S->rb_nb, S->rb_nb_mask);
    };
    auto visit = [&](uint32_t st, uint32_t en) {
        for (uint32_t j = st; j < en; j++) {
            const float4 q = __ldg(G.spos + j);
            const float4 vq = dynamic ? __ldg(G.body_vel + (int)q.w) : make_float4(0.f, 0.f, 0.f, 0.f);
            fg_contact(acc, P, V, q, vq, mind, S->ck, S->ckd);
        }
    };
    if (rx >= 0 && rx <= FG_CONTACT_ROW_MAX) {
        /* the same buckets in the same order, with the x hashes computed
         * once and each x row's bucket ranges loaded together: a particle
         * near a body pays one memory latency per row instead of one per
         * bucket (125 buckets at the default half-width of 2) */
        uint32_t hx[2 * FG_CONTACT_ROW_MAX + 1];
#pragma unroll
        for (int k = 0; k <= 2 * FG_CONTACT_ROW_MAX; k++)
            hx[k] = k <= 2 * rx ? fg_axis_hash_rel(p.x, S->rb_cell[0], k - rx, FG_PX) : 0u;
        for (int z = -rz; z <= rz; z++) {
            const uint32_t hz = fg_axis_hash_rel(p.z, S->rb_cell[2], z, FG_PZ);
            for (int y = -ry; y <= ry; y++) {
                const uint32_t hy = fg_axis_hash_rel(p.y, S->rb_cell[1], y, FG_PY);
                uint32_t st[2 * FG_CONTACT_ROW_MAX + 1], en[2 * FG_CONTACT_ROW_MAX + 1];
#pragma unroll
                for (int k = 0; k <= 2 * FG_CONTACT_ROW_MAX; k++) {
                    st[k] = FG_EMPTY;
                    en[k] = 0u;
                    if (k <= 2 * rx) {
                        const uint32_t b = bucket(hx[k], hy, hz);
                        st[k] = __ldg(G.start + b);
                        en[k] = __ldg(G.end + b);
                    }
                }
#pragma unroll
                for (int k = 0; k <= 2 * FG_CONTACT_ROW_MAX; k++)
                    if (st[k] != FG_EMPTY) visit(st[k], en[k]);
            }
        }
        return acc;
    }
    /* wider half-widths: one bucket at a time */
    for (int z = -rz; z <= rz; z++) {
        const uint32_t hz = fg_axis_hash_rel(p.z, S->rb_cell[2], z, FG_PZ);
        for (int y = -ry; y <= ry; y++) {
            const uint32_t hy = fg_axis_hash_rel(p.y, S->rb_cell[1], y, FG_PY);
            for (int x = -rx; x <= rx; x++) {
                const uint32_t b = bucket(fg_axis_hash_rel(p.x, S->rb_cell[0], x, FG_PX), hy, hz);
                const uint32_t st = __ldg(G.start + b);
                if (st != FG_EMPTY) visit(st, __ldg(G.end + b));
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
    /* every operation rounded on its own: the same bits in every kernel */
    const float il = fg_rsqrt_approx(r2);
    const float l = __fmul_rn(r2, il);
    const float hl = __fsub_rn(h, l);
    const float irr = fg_rcp_approx(__fmul_rn(rho_i, rho_j)); /* rho >= 1: no denormal or overflow range */
    /* pressure: -(d/l) kSpiky (h-l)^2 (Pi+Pj)/(rho_i rho_j) */
    const float cp = __fmul_rn(__fmul_rn(-__fmul_rn(__fmul_rn(kspiky, hl), hl), __fmul_rn(__fadd_rn(P_i, P_j), irr)),
                               il);
    /* viscosity: (vj-vi)/(rho_i rho_j) kVisc (h-l) mu */
    const float cv = __fmul_rn(__fmul_rn(kv, hl), irr);
    fx = __fadd_rn(fx, __fmaf_rn(__fsub_rn(vj.x, vi.x), cv, __fmul_rn(dx, cp)));
    fy = __fadd_rn(fy, __fmaf_rn(__fsub_rn(vj.y, vi.y), cv, __fmul_rn(dy, cp)));
    fz = __fadd_rn(fz, __fmaf_rn(__fsub_rn(vj.z, vi.z), cv, __fmul_rn(dz, cp)));
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
