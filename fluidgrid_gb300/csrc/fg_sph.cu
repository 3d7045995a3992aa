/* SPH density, forces and integration on GB300.
 *
 * Semantics follow GPU_Kernels/K_FluidSim.cu:
 *   density   CalculateMassDensityK + ProcessMassDensityGridD (:46-79, :210-254)
 *   forces    SPHCalculateForcesK / SPHCalculateForcesWithSRBK with
 *             CalculateFluidInternalForcesD, SPHCalculatePressureForceD,
 *             SPHCalculateViscosityForceD (:85-205, :260-413), walls from
 *             K_Boundaries_Walls.cu, rigid contact ProcessCollisionForcesD
 *             (K_DeviceFunctions.cu:32-159)
 *   integrate SPHIntegrateK (:418-438)
 * The 27 neighbour buckets are visited exactly as the reference visits them
 * (z-y-x order, same hashed buckets, a bucket reached twice is summed twice);
 * bucket indices are bit-exact.  Pair arithmetic is reorganised for the
 * GPU: squared-distance tests, rsqrt/rcp instead of divides, compensated
 * density sums (plain within a bucket, Kahan across buckets); the results
 * agree with the reference arithmetic to the tolerances the parity tests
 * state.
 *
 * One thread per particle in sorted order: neighbouring lanes share cells,
 * so neighbour loads broadcast from L1 and sorted float4 loads coalesce.
 * In the world pipeline the density pass is the only one that walks the
 * ~216 candidates of the 27 buckets (~1,000 once the block compresses): it
 * records each particle's in-range visits (in visit order, duplicates and
 * the particle itself included) in the particle's own list, buffered in
 * registers and stored two entries at a time, together with a packed
 * 32-byte record per particle.  The force pass then loops over the ~30-110
 * listed neighbours per particle with all lanes busy, one 256-bit record
 * load each, instead of re-walking the candidates where almost every warp
 * iteration would run the pair math for a few lanes. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include "fg_device.cuh"
#include "fg_kernels.h"
#include "fg_sph_common.cuh"

namespace fg {

/* 16 CTAs of 128 threads per SM (32 registers): the walk's per-row state
 * spills to L1, but the candidate loop keeps its values in registers, and
 * the full 64 warps per SM hide the candidate loads and the in-range
 * branch's divergence better than 8 CTAs at 64 registers (0.85 -> 0.71 ms
 * on the 1M-particle dam break). */
/* Work items are FG_CHUNK particles whatever the block size: a CTA of
 * BLOCK < FG_CHUNK threads takes an item in FG_CHUNK / BLOCK passes, one of
 * BLOCK > FG_CHUNK threads takes BLOCK / FG_CHUNK items at once.  Every
 * particle's arithmetic is the same for every block size. */
#define FG_ITEMS_PER_CTA(B) ((B) >= FG_CHUNK ? (B) / FG_CHUNK : 1u)
#define FG_PASSES(B) ((B) >= FG_CHUNK ? 1u : FG_CHUNK / (B))

template <bool LIST, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 2048 / BLOCK) k_density(const FgWork *__restrict__ work, uint32_t nwork,
                                                     uint32_t n_single, const FgScene *__restrict__ table,
                                                     const __grid_constant__ FgScene single,
                                                     const float4 *__restrict__ spos,
                                                     const float4 *__restrict__ svel,
                                                     const uint32_t *__restrict__ start,
                                                     const uint32_t *__restrict__ end, float2 *__restrict__ dp,
                                                     float gas_o, float rest_o, float mass_o, int use_o,
                                                     const __grid_constant__ NbrList list, TargetOrder ord,
                                                     unsigned long long *__restrict__ pairs)
{
    constexpr uint32_t IPC = FG_ITEMS_PER_CTA(BLOCK), PASSES = FG_PASSES(BLOCK);
    const uint32_t sub = IPC > 1u ? threadIdx.x / FG_CHUNK : 0u;
    const uint32_t lt = IPC > 1u ? threadIdx.x % FG_CHUNK : threadIdx.x;
    const uint32_t cap = LIST ? __ldg(list.cap) : 0u;
    unsigned long long pc = 0; /* in-range density visits of this thread */
    uint32_t mx = 0;           /* largest list count of this thread */
    uint32_t ovf = 0;          /* targets of this thread with more entries than slots */
    for (uint32_t w = blockIdx.x * IPC + sub; w < nwork; w += gridDim.x * IPC)
#pragma unroll 1
    for (uint32_t ps = 0; ps < PASSES; ps++) {
        const uint32_t tid = lt + ps * BLOCK;
        FgWork it = fg_work(work, w, n_single);
        const bool valid = tid < it.count;
        const FgScene *S = fg_scene(table, &single, it.scene);
        const uint32_t tpos = it.first + tid; /* target slot */
        const uint32_t i = (ord.tord && valid) ? __ldg(ord.inv + __ldg(ord.tord + tpos)) : tpos;
        const float4 p = valid ? spos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool active = valid && p.w > 0.0f; /* inactive: density not written */
        DensityAcc acc;
        acc.init();
        /* lists by sorted index: the force pass may visit the targets in another order */
        uint32_t *lp = LIST ? list.idx + (size_t)i * list.stride : nullptr;
        if (active) {
            const float scale = S->scale, h2 = S->h2;
            const float px = p.x * scale, py = p.y * scale, pz = p.z * scale;
            fg_walk27(
                p.x, p.y, p.z, S, start, end,
                [&](uint32_t j) { acc.visit<LIST>(__ldg(spos + j), j, px, py, pz, scale, h2, lp, cap); },
                [&] { acc.end_bucket(); });
            if (LIST) acc.flush(lp, cap, i);
            const float mass = use_o ? mass_o : S->mass;
            const float gas = use_o ? gas_o : S->gas;
            const float rest = use_o ? rest_o : S->rest;
            const float2 d = fg_density_out(mass, S->kpoly6, gas, rest, acc.s);
            dp[i] = d;
            if (LIST) {
                const float4 v = __ldg(svel + i);
                list.rec[2 * i] = make_float4(p.x, p.y, p.z, d.x);
                list.rec[2 * i + 1] = make_float4(v.x, v.y, v.z, d.y);
            }
        } else if (LIST && valid) {
            /* inactive particles stay neighbours with their stale density */
            const float2 d = dp[i];
            const float4 v = __ldg(svel + i);
            list.rec[2 * i] = make_float4(p.x, p.y, p.z, d.x);
            list.rec[2 * i + 1] = make_float4(v.x, v.y, v.z, d.y);
        }
        const uint32_t cnt = acc.cnt, dcnt = LIST ? acc.cnt : acc.dcnt;
        if (LIST && valid) list.cnt[i] = cnt;
        pc += dcnt;
        mx = max(mx, cnt);
        ovf += (LIST && cnt > cap) ? 1u : 0u;
    }
    /* once per warp: in-range pair visits (self included) for reporting, and
     * the largest list count for the capacity check */
    const uint32_t lane = threadIdx.x & 31u;
    if (pairs) {
#pragma unroll
        for (int o = 16; o; o >>= 1) pc += __shfl_xor_sync(0xffffffffu, pc, o);
        if (lane == 0 && pc) atomicAdd(pairs, pc);
    }
    if (LIST && list.max_count) {
        mx = __reduce_max_sync(0xffffffffu, mx);
        if (lane == 0 && mx) atomicMax(list.max_count, mx);
    }
    if (LIST && list.overflow) {
        ovf = __reduce_add_sync(0xffffffffu, ovf);
        if (lane == 0 && ovf) atomicAdd(list.overflow, (unsigned long long)ovf);
    }
}

void launch_density(const Launch &L, const float4 *spos, const uint32_t *start, const uint32_t *end, float2 *dp,
                    float gas_o, float rest_o, float mass_o, int use_o, const float4 *svel, const NbrList *list,
                    TargetOrder ord, unsigned long long *pairs)
{
    if (!L.nwork) return;
    NbrList none;
    memset(&none, 0, sizeof(none));
    const NbrList &nl = list ? *list : none;
    const uint32_t B = L.block ? L.block : FG_CHUNK;
    const uint32_t ipc = FG_ITEMS_PER_CTA(B);
    /* ctas_per_sm counts CTAs of FG_CHUNK threads: the same threads per SM
     * for every block size */
    const int per_sm = (int)(((L.ctas_per_sm ? L.ctas_per_sm : 64u) * FG_CHUNK) / B);
    const uint32_t g = grid_for((L.nwork + ipc - 1u) / ipc, per_sm > 0 ? per_sm : 1);
#define FG_DENSITY(LI, BL)                                                                                        \
    k_density<LI, BL><<<g, BL, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, spos, svel, start, end, dp, \
                                              gas_o, rest_o, mass_o, use_o, nl, ord, pairs)
    if (B == 64u) {
        if (list) FG_DENSITY(true, 64); else FG_DENSITY(false, 64);
    } else if (B == 256u) {
        if (list) FG_DENSITY(true, 256); else FG_DENSITY(false, 256);
    } else {
        if (list) FG_DENSITY(true, 128); else FG_DENSITY(false, 128);
    }
#undef FG_DENSITY
}

struct RigidArgs {
    RigidGrid dyn;
    RigidGrid sta;
    int use_dyn, use_sta;
};

template <bool LIST, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 768 / BLOCK) k_forces(const FgWork *__restrict__ work, uint32_t nwork,
                                                    uint32_t n_single, const FgScene *__restrict__ table,
                                                    const __grid_constant__ FgScene single,
                                                    const float4 *__restrict__ spos, const float4 *__restrict__ svel,
                                                    const float2 *__restrict__ dp,
                                                    const uint32_t *__restrict__ start,
                                                    const uint32_t *__restrict__ end,
                                                    const uint32_t *__restrict__ ids, float4 *__restrict__ vel_out,
                                                    float4 *__restrict__ pos_out,
                                                    const __grid_constant__ RigidArgs R, float mass_o, float visc_o,
                                                    int use_o, const __grid_constant__ NbrList list, TargetOrder ord)
{
    constexpr uint32_t IPC = FG_ITEMS_PER_CTA(BLOCK), PASSES = FG_PASSES(BLOCK);
    const uint32_t sub = IPC > 1u ? threadIdx.x / FG_CHUNK : 0u;
    const uint32_t lt = IPC > 1u ? threadIdx.x % FG_CHUNK : threadIdx.x;
    for (uint32_t w = blockIdx.x * IPC + sub; w < nwork; w += gridDim.x * IPC)
#pragma unroll 1
    for (uint32_t ps = 0; ps < PASSES; ps++) {
        const uint32_t tid = lt + ps * BLOCK;
        FgWork it = fg_work(work, w, n_single);
        if (tid >= it.count) continue;
        const FgScene *S = fg_scene(table, &single, it.scene);
        const uint32_t tpos = it.first + tid; /* target slot */
        const uint32_t pid = ord.tord ? __ldg(ord.tord + tpos) : 0u;
        const uint32_t i = ord.tord ? __ldg(ord.inv + pid) : tpos;
        const float4 p = spos[i];
        const float4 v = svel[i];
        float3 F = make_float3(0.f, 0.f, 0.f);
        if (p.w > 0.0f) {
            const float scale = S->scale, h = S->h, h2 = S->h2;
            const float mass = use_o ? mass_o : S->mass;
            const float visc = use_o ? visc_o : S->visc;
            const float kspiky = S->kspiky, kv = S->kvisc * visc;
            const float px = p.x * scale, py = p.y * scale, pz = p.z * scale;
            float fx = 0.f, fy = 0.f, fz = 0.f;
            if (LIST) {
                const float4 r0 = list.rec[2 * i], r1 = list.rec[2 * i + 1];
                const float rho_i = r0.w, P_i = r1.w;
                const uint32_t c = list.cnt[i];
                if (c <= __ldg(list.cap)) {
                    /* in-range visits in walk order (the target's own
                     * entries skipped) */
                    const uint32_t *nl = list.idx + (size_t)i * list.stride;
                    /* the list is padded with i to whole groups of four */
                    const uint32_t c4 = (c + 3u) & ~3u;
                    /* four 32-byte records in flight, one 256-bit load each,
                     * their target's own entries skipped */
                    auto group = [&](const uint4 q) {
                        const uint32_t jj[4] = {q.x, q.y, q.z, q.w};
                        float4 a[4], b[4];
#pragma unroll
                        for (int e = 0; e < 4; e++) fg_ld_rec(list.rec + 2 * jj[e], a[e], b[e]);
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            if (jj[e] != i) {
                                const float dx = fmaf(-a[e].x, scale, px), dy = fmaf(-a[e].y, scale, py),
                                            dz = fmaf(-a[e].z, scale, pz);
                                const float r2 = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
                                fg_pair(fx, fy, fz, dx, dy, dz, r2, h, kspiky, kv, rho_i, P_i, v, a[e].w, b[e].w,
                                        b[e]);
                            }
                        }
                    };
                    /* eight indices (one sector, 32-byte aligned: the stride
                     * is a multiple of 8) per load, the next eight loading
                     * while these records do */
                    uint4 qa = make_uint4(0u, 0u, 0u, 0u), qb = qa;
                    if (c4) fg_ld_idx8(nl, qa, qb);
                    for (uint32_t k = 0; k < c4; k += 8) {
                        const uint4 ca = qa, cb = qb;
                        if (k + 8u < c4) fg_ld_idx8(nl + k + 8u, qa, qb);
                        group(ca);
                        if (k + 4u < c4) group(cb);
                    }
                } else {
                    /* more in-range visits than list slots: walk the buckets */
                    fg_walk27(p.x, p.y, p.z, S, start, end, [&](uint32_t j) {
                        if (j == i) return;
                        const float4 q0 = __ldg(list.rec + 2 * j);
                        const float dx = fmaf(-q0.x, scale, px), dy = fmaf(-q0.y, scale, py),
                                    dz = fmaf(-q0.z, scale, pz);
                        const float r2 = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
                        if (r2 <= h2) {
                            const float4 q1 = __ldg(list.rec + 2 * j + 1);
                            fg_pair(fx, fy, fz, dx, dy, dz, r2, h, kspiky, kv, rho_i, P_i, v, q0.w, q1.w, q1);
                        }
                    });
                }
            } else {
                const float2 di = dp[i];
                fg_walk27(p.x, p.y, p.z, S, start, end, [&](uint32_t j) {
                    if (j == i) return;
                    const float4 q = __ldg(spos + j);
                    const float dx = fmaf(-q.x, scale, px), dy = fmaf(-q.y, scale, py), dz = fmaf(-q.z, scale, pz);
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
                    if (r2 <= h2) {
                        const float4 vj = __ldg(svel + j);
                        const float2 dj = __ldg(dp + j);
                        fg_pair(fx, fy, fz, dx, dy, dz, r2, h, kspiky, kv, di.x, di.y, v, dj.x, dj.y, vj);
                    }
                });
            }
            F = make_float3(fx * mass + S->gravity[0], fy * mass + S->gravity[1], fz * mass + S->gravity[2]);
            if (R.use_sta) {
                float3 c = fg_fluid_rigid_contact(S, it.scene, p, v, R.sta, false);
                F.x += c.x; F.y += c.y; F.z += c.z;
            }
            if (R.use_dyn && (S->flags & FG_SCENE_HAS_RB)) {
                float3 c = make_float3(0.f, 0.f, 0.f);
                if (!R.dyn.pre) {
                    c = fg_fluid_rigid_contact(S, it.scene, p, v, R.dyn, true);
                } else if (!fg_contact_outside(S, it.scene, p, R.dyn)) {
                    const float4 q = R.dyn.pre[ord.tord ? pid : __ldg(ids + i)];
                    c = make_float3(q.x, q.y, q.z);
                }
                F.x += c.x; F.y += c.y; F.z += c.z;
            }
            const float3 wl = fg_walls(*S, make_float3(p.x, p.y, p.z), make_float3(v.x, v.y, v.z));
            F.x += wl.x; F.y += wl.y; F.z += wl.z;
            const float sp2 = F.x * F.x + F.y * F.y + F.z * F.z;
            const float speed = sqrtf(sp2);
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
        const uint32_t oi = ord.tord ? pid : __ldg(ids + i);
        vel_out[oi] = nv;
        if (pos_out && p.w > 0.0f) {
            /* SPHIntegrateK fused: pos += vel * (dt / scale), unfused rounding */
            const float c = S->dt_over_scale;
            float4 np;
            np.x = __fadd_rn(p.x, __fmul_rn(nv.x, c));
            np.y = __fadd_rn(p.y, __fmul_rn(nv.y, c));
            np.z = __fadd_rn(p.z, __fmul_rn(nv.z, c));
            np.w = __fadd_rn(p.w, __fmul_rn(nv.w, c));
            pos_out[oi] = np;
        }
    }
}

void launch_forces(const Launch &L, const float4 *spos, const float4 *svel, const float2 *dp, const uint32_t *start,
                   const uint32_t *end, const uint32_t *ids, ForceOut out, const RigidGrid *rigid,
                   const RigidGrid *statics, float mass_o, float visc_o, int use_o, const NbrList *list,
                   TargetOrder ord)
{
    if (!L.nwork) return;
    RigidArgs R;
    memset(&R, 0, sizeof(R));
    if (rigid) { R.dyn = *rigid; R.use_dyn = 1; }
    if (statics) { R.sta = *statics; R.use_sta = 1; }
    NbrList none;
    memset(&none, 0, sizeof(none));
    const NbrList &nl = list ? *list : none;
    const uint32_t B = L.block ? L.block : FG_CHUNK;
    const uint32_t ipc = FG_ITEMS_PER_CTA(B);
    const int per_sm = (int)(((L.ctas_per_sm ? L.ctas_per_sm : 64u) * FG_CHUNK) / B);
    const uint32_t g = grid_for((L.nwork + ipc - 1u) / ipc, per_sm > 0 ? per_sm : 1);
#define FG_FORCES(LI, BL)                                                                                        \
    k_forces<LI, BL><<<g, BL, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, spos, svel, dp, start, end, \
                                             ids, out.vel, out.pos, R, mass_o, visc_o, use_o, nl, ord)
    if (B == 64u) {
        if (list) FG_FORCES(true, 64); else FG_FORCES(false, 64);
    } else if (B == 256u) {
        if (list) FG_FORCES(true, 256); else FG_FORCES(false, 256);
    } else {
        if (list) FG_FORCES(true, 128); else FG_FORCES(false, 128);
    }
#undef FG_FORCES
}

/* The fluid side of the fluid/rigid contact ahead of the force pass, by
 * particle id from the step's unsorted positions and velocities (the sorted
 * copies hold the same bits), so it runs right after the rigid-sphere grid
 * beside the fluid hash and sort.  Inside the force pass, the few particles
 * near a body walked (2r+1)^3 rigid buckets while the rest of their warps and
 * CTAs waited at 80 registers a thread.  The force pass adds the stored sum
 * where it added the walked one: the same bits. */
__global__ void __launch_bounds__(FG_CHUNK) k_fluid_contact(const FgWork *__restrict__ work, uint32_t nwork,
                                                           uint32_t n_single, const FgScene *__restrict__ table,
                                                           const __grid_constant__ FgScene single,
                                                           const float4 *__restrict__ pos,
                                                           const float4 *__restrict__ vel,
                                                           const __grid_constant__ RigidGrid G,
                                                           float4 *__restrict__ out)
{
    for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        const FgWork it = fg_work(work, w, n_single);
        if (threadIdx.x >= it.count) continue;
        const FgScene *S = fg_scene(table, &single, it.scene);
        if (!(S->flags & FG_SCENE_HAS_RB)) continue;
        const uint32_t id = it.first + threadIdx.x;
        const float4 p = pos[id];
        if (!(p.w > 0.0f) || fg_contact_outside(S, it.scene, p, G)) continue;
        const float3 c = fg_fluid_rigid_contact(S, it.scene, p, vel[id], G, true);
        out[id] = make_float4(c.x, c.y, c.z, 0.0f);
    }
}

void launch_fluid_contact(const Launch &L, const float4 *pos, const float4 *vel, const RigidGrid &G, float4 *out)
{
    if (!L.nwork) return;
    k_fluid_contact<<<grid_for(L.nwork, 16), FG_CHUNK, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, pos,
                                                                     vel, G, out);
}

/* SPHIntegrateK (K_FluidSim.cu:418-438): pos += vel*(dt/scale) for active
 * particles, all four components, each operation rounded separately. */
__global__ void __launch_bounds__(FG_CHUNK) k_integrate(const FgWork *__restrict__ work, uint32_t nwork,
                                                       uint32_t n_single, const FgScene *__restrict__ table,
                                                       const __grid_constant__ FgScene single,
                                                       float4 *__restrict__ pos, const float4 *__restrict__ vel)
{
    for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        FgWork it = fg_work(work, w, n_single);
        if (threadIdx.x >= it.count) continue;
        const FgScene *S = fg_scene(table, &single, it.scene);
        const uint32_t i = it.first + threadIdx.x;
        float4 p = pos[i];
        if (p.w > 0.0f) {
            const float4 v = __ldg(vel + i);
            const float c = S->dt_over_scale;
            p.x = __fadd_rn(p.x, __fmul_rn(v.x, c));
            p.y = __fadd_rn(p.y, __fmul_rn(v.y, c));
            p.z = __fadd_rn(p.z, __fmul_rn(v.z, c));
            p.w = __fadd_rn(p.w, __fmul_rn(v.w, c));
            pos[i] = p;
        }
    }
}

void launch_integrate(const Launch &L, float4 *pos, const float4 *vel)
{
    if (!L.nwork) return;
    k_integrate<<<grid_for(L.nwork, 16), FG_CHUNK, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, pos,
                                                                  vel);
}

} // namespace fg
