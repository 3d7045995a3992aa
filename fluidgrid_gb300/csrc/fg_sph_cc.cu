/* Cell-cooperative SPH density and forces: one warp per occupied bucket run.
 *
 * Same semantics as fg_sph.cu (GPU_Kernels/K_FluidSim.cu:46-413): every
 * particle sums over the particles of the 27 buckets hashed from its own
 * position (duplicate buckets summed twice, z-y-x visit order), bucket ids
 * bit-exact.  The work is organised around the sorted bucket runs instead of
 * one thread per particle:
 *
 *  - the ranges pass appends the first sorted index of every occupied bucket
 *    (a "run") to a list;
 *  - a warp takes a run; its particles (the targets) are grouped by their 27
 *    neighbour buckets, which are identical for all particles of one cell
 *    (checked per particle through the 9 per-axis cell indices, so a particle
 *    whose offsets round into a different cell, or a bucket shared by two
 *    cells, forms its own group);
 *  - the warp stages the group's candidates -- the particles of the 27
 *    buckets, bucket by bucket, with coalesced loads -- into shared memory
 *    (in chunks of CC_CAP if there are more);
 *  - density: for each target the 32 lanes test 32 candidates at a time from
 *    shared memory and a warp reduction sums the compensated partials;
 *  - forces: for each target the lanes test candidates, compact the in-range
 *    ones with a warp ballot into a shared queue, and then evaluate the pair
 *    terms with all lanes busy, followed by a warp reduction.
 * Neighbour data is read from HBM once per run instead of once per target,
 * and no lane idles through another lane's pair arithmetic. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include "fg_device.cuh"
#include "fg_kernels.h"
#include "fg_sph_common.cuh"

namespace fg {

/* warps (bucket runs in flight) per CTA: 1, 2 or 4, an autotuner dimension */
#define CC_CAP 256

struct CcArgs {
    const uint32_t *runs;  /* first sorted index of each occupied bucket */
    const uint32_t *nruns; /* device counter */
    const uint32_t *keys;  /* sorted global bucket keys */
    uint32_t nscenes;
};

/* Stage candidates [c0, c0 + mc) of the 27-bucket sequence into shared
 * memory.  st/off are lane-resident (lane k holds bucket k); they are
 * published to the warp's shared table tab (27 offsets, 27 starts) so every
 * lane can place any candidate with a 5-step binary search and issue its
 * load independently -- one memory latency per 32 candidates instead of one
 * per bucket. */
template <bool REC>
__device__ __forceinline__ void cc_stage(uint32_t st, uint32_t off, uint32_t c0, uint32_t mc, int lane,
                                         const float4 *__restrict__ spos, const float4 *__restrict__ rec,
                                         float4 *s0, float4 *s1, uint32_t *sj, uint32_t *tab)
{
    if (lane < 27) {
        tab[lane] = off;
        tab[32 + lane] = st;
    }
    __syncwarp();
#pragma unroll 2
    for (uint32_t c = lane; c < mc; c += 32) {
        const uint32_t g = c0 + c;
        /* largest k with off_k <= g (empty buckets share the next offset) */
        uint32_t lo = 0, hi = 27;
#pragma unroll
        for (int it = 0; it < 5; it++) {
            const uint32_t mid = (lo + hi) >> 1;
            if (hi - lo > 1) {
                if (tab[mid] <= g) lo = mid;
                else hi = mid;
            }
        }
        const uint32_t j = tab[32 + lo] + (g - tab[lo]);
        if (REC) {
            s0[c] = __ldg(rec + 2 * j);
            s1[c] = __ldg(rec + 2 * j + 1);
            sj[c] = j;
        } else {
            s0[c] = __ldg(spos + j);
        }
    }
    __syncwarp();
}

template <int CC_WARPS>
__global__ void __launch_bounds__(CC_WARPS * 32) k_density_cc(const FgScene *__restrict__ table,
                                                             const __grid_constant__ FgScene single,
                                                             const __grid_constant__ CcArgs A,
                                                             const float4 *__restrict__ spos,
                                                             const float4 *__restrict__ svel,
                                                             const uint32_t *__restrict__ start,
                                                             const uint32_t *__restrict__ end,
                                                             float2 *__restrict__ dp, float4 *__restrict__ rec)
{
    __shared__ float4 s_cand[CC_WARPS][CC_CAP];
    __shared__ uint32_t s_tab[CC_WARPS][64];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float4 *cand = s_cand[wid];
    const uint32_t nruns = *A.nruns;
    for (uint32_t r = blockIdx.x * CC_WARPS + wid; r < nruns; r += gridDim.x * CC_WARPS) {
        const uint32_t s0 = __ldg(A.runs + r);
        const uint32_t key = __ldg(A.keys + s0);
        const uint32_t e = __ldg(end + key);
        const FgScene *S = table ? table + cc_scene_of(table, A.nscenes, key) : &single;
        const float scale = S->scale, h2 = S->h2;
        for (uint32_t t0 = s0; t0 < e; t0 += 32) {
            const uint32_t tc = min(32u, e - t0);
            const bool valid = (uint32_t)lane < tc;
            const uint32_t ti = t0 + lane;
            const float4 p = valid ? spos[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
            const bool active = valid && p.w > 0.0f;
            const Sig sig = cc_sig(p.x, p.y, p.z, S->cell);
            float acc = 0.0f; /* this lane's target total */
            uint32_t todo = __ballot_sync(0xffffffffu, active);
            while (todo) {
                const int leader = __ffs(todo) - 1;
                Sig ls;
                bool same = active;
#pragma unroll
                for (int q = 0; q < 9; q++) {
                    ls.v[q] = __shfl_sync(0xffffffffu, sig.v[q], leader);
                    same = same && (ls.v[q] == sig.v[q]);
                }
                const uint32_t G = __ballot_sync(0xffffffffu, same) & todo;
                todo &= ~G;
                uint32_t st, cnt;
                cc_bucket_of_lane(ls, S, start, end, lane, st, cnt);
                uint32_t M;
                const uint32_t off = cc_excl_scan(cnt, lane, M);
                for (uint32_t c0 = 0; c0 < M; c0 += CC_CAP) {
                    const uint32_t mc = min((uint32_t)CC_CAP, M - c0);
                    cc_stage<false>(st, off, c0, mc, lane, spos, nullptr, cand, nullptr, nullptr, s_tab[wid]);
                    uint32_t g = G;
                    while (g) {
                        const int t = __ffs(g) - 1;
                        g &= g - 1;
                        const float tx = __shfl_sync(0xffffffffu, p.x, t) * scale;
                        const float ty = __shfl_sync(0xffffffffu, p.y, t) * scale;
                        const float tz = __shfl_sync(0xffffffffu, p.z, t) * scale;
                        float ks = 0.0f, kc = 0.0f; /* Kahan partial over this lane's candidates */
                        for (uint32_t c = lane; c < mc; c += 32) {
                            const float4 q = cand[c];
                            const float dx = fmaf(-q.x, scale, tx), dy = fmaf(-q.y, scale, ty),
                                        dz = fmaf(-q.z, scale, tz);
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
                            if (r2 < h2) {
                                const float tt = h2 - r2;
                                const float y = tt * tt * tt - kc;
                                const float sum = ks + y;
                                kc = (sum - ks) - y;
                                ks = sum;
                            }
                        }
                        const float tot = cc_sum(ks - kc);
                        if (lane == t) acc += tot;
                    }
                    __syncwarp();
                }
            }
            if (valid) {
                float2 d;
                if (active) {
                    const float rho = (S->mass * S->kpoly6) * acc;
                    d = make_float2(fmaxf(1.0f, rho), S->gas * (rho - S->rest));
                    dp[ti] = d;
                } else {
                    d = dp[ti]; /* inactive: not written, stays a neighbour with its old value */
                }
                const float4 v = __ldg(svel + ti);
                rec[2 * ti] = make_float4(p.x, p.y, p.z, d.x);
                rec[2 * ti + 1] = make_float4(v.x, v.y, v.z, d.y);
            }
        }
    }
}

struct CcForceArgs {
    RigidGrid dyn;
    int use_dyn;
    float4 *vel_out;
    float4 *pos_out; /* null: no fused integration */
    const uint32_t *ids;
};

template <int CC_WARPS>
__global__ void __launch_bounds__(CC_WARPS * 32) k_forces_cc(const FgScene *__restrict__ table,
                                                            const __grid_constant__ FgScene single,
                                                            const __grid_constant__ CcArgs A,
                                                            const float4 *__restrict__ spos,
                                                            const float4 *__restrict__ svel,
                                                            const float4 *__restrict__ rec,
                                                            const uint32_t *__restrict__ start,
                                                            const uint32_t *__restrict__ end,
                                                            const __grid_constant__ CcForceArgs O)
{
    __shared__ float4 s_c0[CC_WARPS][CC_CAP];
    __shared__ float4 s_c1[CC_WARPS][CC_CAP];
    __shared__ uint32_t s_cj[CC_WARPS][CC_CAP];
    __shared__ uint16_t s_q[CC_WARPS][CC_CAP];
    __shared__ uint32_t s_tab[CC_WARPS][64];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    float4 *c0s = s_c0[wid], *c1s = s_c1[wid];
    uint32_t *cjs = s_cj[wid];
    uint16_t *qs = s_q[wid];
    const uint32_t nruns = *A.nruns;
    for (uint32_t r = blockIdx.x * CC_WARPS + wid; r < nruns; r += gridDim.x * CC_WARPS) {
        const uint32_t s0 = __ldg(A.runs + r);
        const uint32_t key = __ldg(A.keys + s0);
        const uint32_t e = __ldg(end + key);
        const uint32_t scene = table ? cc_scene_of(table, A.nscenes, key) : 0u;
        const FgScene *S = table ? table + scene : &single;
        const float scale = S->scale, h = S->h, h2 = S->h2;
        const float kspiky = S->kspiky, kv = S->kvisc * S->visc;
        for (uint32_t t0 = s0; t0 < e; t0 += 32) {
            const uint32_t tc = min(32u, e - t0);
            const bool valid = (uint32_t)lane < tc;
            const uint32_t ti = t0 + lane;
            const float4 p = valid ? spos[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 v = valid ? svel[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float rho = valid ? __ldg(rec + 2 * ti).w : 1.0f;
            const float prs = valid ? __ldg(rec + 2 * ti + 1).w : 0.0f;
            const bool active = valid && p.w > 0.0f;
            const Sig sig = cc_sig(p.x, p.y, p.z, S->cell);
            float fx = 0.f, fy = 0.f, fz = 0.f; /* this lane's target sum */
            uint32_t todo = __ballot_sync(0xffffffffu, active);
            while (todo) {
                const int leader = __ffs(todo) - 1;
                Sig ls;
                bool same = active;
#pragma unroll
                for (int q = 0; q < 9; q++) {
                    ls.v[q] = __shfl_sync(0xffffffffu, sig.v[q], leader);
                    same = same && (ls.v[q] == sig.v[q]);
                }
                const uint32_t G = __ballot_sync(0xffffffffu, same) & todo;
                todo &= ~G;
                uint32_t st, cnt;
                cc_bucket_of_lane(ls, S, start, end, lane, st, cnt);
                uint32_t M;
                const uint32_t off = cc_excl_scan(cnt, lane, M);
                for (uint32_t c0 = 0; c0 < M; c0 += CC_CAP) {
                    const uint32_t mc = min((uint32_t)CC_CAP, M - c0);
                    cc_stage<true>(st, off, c0, mc, lane, nullptr, rec, c0s, c1s, cjs, s_tab[wid]);
                    uint32_t g = G;
                    while (g) {
                        const int t = __ffs(g) - 1;
                        g &= g - 1;
                        const float tx = __shfl_sync(0xffffffffu, p.x, t) * scale;
                        const float ty = __shfl_sync(0xffffffffu, p.y, t) * scale;
                        const float tz = __shfl_sync(0xffffffffu, p.z, t) * scale;
                        const float4 tv = make_float4(__shfl_sync(0xffffffffu, v.x, t), __shfl_sync(0xffffffffu, v.y, t),
                                                      __shfl_sync(0xffffffffu, v.z, t), 0.0f);
                        const float trho = __shfl_sync(0xffffffffu, rho, t);
                        const float tprs = __shfl_sync(0xffffffffu, prs, t);
                        const uint32_t tj = t0 + (uint32_t)t;
                        /* test and compact the in-range candidates (j != i, l <= h) */
                        uint32_t qn = 0;
                        for (uint32_t cb = 0; cb < mc; cb += 32) {
                            const uint32_t c = cb + lane;
                            bool in = false;
                            if (c < mc) {
                                const float4 q = c0s[c];
                                const float dx = fmaf(-q.x, scale, tx), dy = fmaf(-q.y, scale, ty),
                                            dz = fmaf(-q.z, scale, tz);
                                const float r2 = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
                                in = (r2 <= h2) && (cjs[c] != tj);
                            }
                            const uint32_t m = __ballot_sync(0xffffffffu, in);
                            if (in) qs[qn + __popc(m & lt)] = (uint16_t)c;
                            qn += __popc(m);
                        }
                        __syncwarp();
                        float px = 0.f, py = 0.f, pz = 0.f;
                        for (uint32_t k = lane; k < qn; k += 32) {
                            const uint32_t c = qs[k];
                            const float4 q0 = c0s[c], q1 = c1s[c];
                            const float dx = fmaf(-q0.x, scale, tx), dy = fmaf(-q0.y, scale, ty),
                                        dz = fmaf(-q0.z, scale, tz);
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
                            fg_pair(px, py, pz, dx, dy, dz, r2, h, kspiky, kv, trho, tprs, tv, q0.w, q1.w, q1);
                        }
                        px = cc_sum(px);
                        py = cc_sum(py);
                        pz = cc_sum(pz);
                        if (lane == t) {
                            fx += px;
                            fy += py;
                            fz += pz;
                        }
                        __syncwarp();
                    }
                    __syncwarp();
                }
            }
            if (valid)
                fg_force_tail(S, scene, p, v, active, fx, fy, fz, S->mass, O.use_dyn ? &O.dyn : nullptr, nullptr,
                              __ldg(O.ids + ti), O.vel_out, O.pos_out);
        }
    }
}

void launch_density_cc(const FgScene *table, const FgScene *single, uint32_t nscenes, const uint32_t *runs,
                       const uint32_t *nruns, const uint32_t *keys, const float4 *spos, const float4 *svel,
                       const uint32_t *start, const uint32_t *end, float2 *dp, float4 *rec, uint32_t n,
                       cudaStream_t s, uint32_t warps)
{
    if (!n) return;
    CcArgs A;
    A.runs = runs;
    A.nruns = nruns;
    A.keys = keys;
    A.nscenes = nscenes;
    /* 32 warps per SM whatever the CTA size */
    if (warps == 1u) k_density_cc<1><<<sm_count() * 32u, 32, 0, s>>>(table, *single, A, spos, svel, start, end, dp, rec);
    else if (warps == 2u) k_density_cc<2><<<sm_count() * 16u, 64, 0, s>>>(table, *single, A, spos, svel, start, end, dp, rec);
    else k_density_cc<4><<<sm_count() * 8u, 128, 0, s>>>(table, *single, A, spos, svel, start, end, dp, rec);
}

void launch_forces_cc(const FgScene *table, const FgScene *single, uint32_t nscenes, const uint32_t *runs,
                      const uint32_t *nruns, const uint32_t *keys, const float4 *spos, const float4 *svel,
                      const float4 *rec, const uint32_t *start, const uint32_t *end, const uint32_t *ids,
                      ForceOut out, const RigidGrid *rigid, uint32_t n, cudaStream_t s, uint32_t warps)
{
    if (!n) return;
    CcArgs A;
    A.runs = runs;
    A.nruns = nruns;
    A.keys = keys;
    A.nscenes = nscenes;
    CcForceArgs O;
    memset(&O, 0, sizeof(O));
    if (rigid) {
        O.dyn = *rigid;
        O.use_dyn = 1;
    }
    O.vel_out = out.vel;
    O.pos_out = out.pos;
    O.ids = ids;
    /* 16 warps per SM whatever the CTA size */
    if (warps == 1u) k_forces_cc<1><<<sm_count() * 16u, 32, 0, s>>>(table, *single, A, spos, svel, rec, start, end, O);
    else if (warps == 2u) k_forces_cc<2><<<sm_count() * 8u, 64, 0, s>>>(table, *single, A, spos, svel, rec, start, end, O);
    else k_forces_cc<4><<<sm_count() * 4u, 128, 0, s>>>(table, *single, A, spos, svel, rec, start, end, O);
}

} // namespace fg
