/* Rigid-body side of the two-way fluid/rigid coupling on GB300.
 *
 *   k_rb_from_fluid   CalculateRBForcesFromFluidsK (K_RigidBodySim.cu:66-99)
 *   k_rb_from_rb      CalculateRigidBodyForcesFromRBK (K_RigidBodySim.cu:18-61)
 *   k_body_update     applyForces' per-body sum (RigidBodySimulator.cpp:522-566:
 *                     sort by body, segmented scan, AddForceTorqueK) as one
 *                     deterministic FP64 block reduction per body, followed by
 *                     IntegrateRBK (K_RigidBodySim.cu:160-262) in FP64
 *   k_integrate_rb_f32  IntegrateRBK with the reference's FP32 arithmetic
 *   k_copy_rb_data / k_reorder_ft / k_segsum / k_add_ft
 *                     the reference's reduction data flow for the drop-in
 *                     launchers (K_RigidBodySim.cu:102-155 + CUDPP scan). */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include "fg_device.cuh"
#include "fg_kernels.h"

namespace fg {

/* Contact sum of one rigid sphere against the fluid grid, then force and
 * torque written at the sphere's unsorted index (body-contiguous).  One warp
 * per sphere, so a few thousand spheres still fill the GPU: the lanes take
 * the (2r+1)^3 fluid buckets in turn and a fixed shuffle tree adds their
 * partial sums (deterministic; the FP32 terms are the reference's, their
 * summation order differs).  CTA = RBF_WARPS warps; CTA c takes spheres
 * RBF_WARPS (c % 32) + warp of work item c / 32. */
#define RBF_WARPS 4
__global__ void __launch_bounds__(RBF_WARPS * 32) k_rb_from_fluid(const FgWork *__restrict__ work, uint32_t nwork,
                                                                 uint32_t n_single, const FgScene *__restrict__ table,
                                                                 const __grid_constant__ FgScene single,
                                                                 const float4 *__restrict__ rb_spos,
                                                                 const uint32_t *__restrict__ rb_ids,
                                                                 const float4 *__restrict__ body_vel,
                                                                 const float4 *__restrict__ body_cm,
                                                                 const float4 *__restrict__ fl_spos,
                                                                 const float4 *__restrict__ fl_svel,
                                                                 const uint32_t *__restrict__ fl_start,
                                                                 const uint32_t *__restrict__ fl_end,
                                                                 float4 *__restrict__ force,
                                                                 float4 *__restrict__ torque, int add)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t w = blockIdx.x >> 5;
    if (w >= nwork) return;
    const FgWork it = fg_work(work, w, n_single);
    const uint32_t k = ((blockIdx.x & 31u) * RBF_WARPS) + (uint32_t)wid;
    if (k >= it.count) return; /* warp-uniform */
    const FgScene *S = fg_scene(table, &single, it.scene);
    const uint32_t i = it.first + k;
    const float4 p = rb_spos[i];
    const int b = (int)p.w;
    const float4 vb = __ldg(body_vel + b);
    const float3 P = make_float3(p.x, p.y, p.z), V = make_float3(vb.x, vb.y, vb.z);
    const float mind = S->rb_radius + S->fluid_radius + S->rb_eps;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    const int rx = S->r2f_rel[0], ry = S->r2f_rel[1], rz = S->r2f_rel[2];
    const int nx = 2 * rx + 1, ny = 2 * ry + 1, nz = 2 * rz + 1;
    for (int q = lane; q < nx * ny * nz; q += 32) {
        const int z = q / (nx * ny) - rz, y = (q / nx) % ny - ry, x = q % nx - rx;
        const uint32_t bk = S->bucket_base + fg_bucket(fg_axis_hash_rel(p.x, S->cell[0], x, FG_PX),
                                                       fg_axis_hash_rel(p.y, S->cell[1], y, FG_PY),
                                                       fg_axis_hash_rel(p.z, S->cell[2], z, FG_PZ), S->nb, S->nb_mask);
        const uint32_t st = __ldg(fl_start + bk);
        if (st == FG_EMPTY) continue;
        const uint32_t en = __ldg(fl_end + bk);
        for (uint32_t j = st; j < en; j++)
            fg_contact(acc, P, V, __ldg(fl_spos + j), __ldg(fl_svel + j), mind, S->ck, S->ckd);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
    }
    if (lane) return;
    const float4 cm = __ldg(body_cm + b);
    const float lw = (float)(b - (int)S->body_base); /* the reference stores the body index in w */
    const float dx = p.x - cm.x, dy = p.y - cm.y, dz = p.z - cm.z;
    float4 f = make_float4(acc.x, acc.y, acc.z, lw);
    float4 t = make_float4(dy * acc.z - dz * acc.y, dz * acc.x - dx * acc.z, dx * acc.y - dy * acc.x, lw);
    const uint32_t oi = rb_ids ? __ldg(rb_ids + i) : i;
    if (add) {
        const float4 f0 = force[oi], t0 = torque[oi];
        f.x += f0.x; f.y += f0.y; f.z += f0.z;
        t.x += t0.x; t.y += t0.y; t.z += t0.z;
    }
    force[oi] = f;
    torque[oi] = t;
}

void launch_rb_from_fluid(const Launch &L, const float4 *rb_spos, const uint32_t *rb_ids, const float4 *body_vel,
                          const float4 *body_cm, const float4 *fl_spos, const float4 *fl_svel,
                          const uint32_t *fl_start, const uint32_t *fl_end, float4 *force, float4 *torque, int add)
{
    if (!L.nwork) return;
    /* a work item holds up to FG_CHUNK spheres: FG_CHUNK / RBF_WARPS CTAs */
    k_rb_from_fluid<<<L.nwork * (FG_CHUNK / RBF_WARPS), RBF_WARPS * 32, 0, L.stream>>>(
        L.work, L.nwork, L.n, L.table, *L.single, rb_spos, rb_ids, body_vel, body_cm, fl_spos, fl_svel, fl_start,
        fl_end, force, torque, add);
}

/* Sphere/sphere contact between different bodies of one scene (same rigid
 * grid, half-width 1, spheres of the own body skipped) and, optionally,
 * against a static sphere grid (no velocity, no grouping). */
struct StaticArg {
    RigidGrid g;
    int use;
};

__global__ void __launch_bounds__(FG_CHUNK) k_rb_from_rb(const FgWork *__restrict__ work, uint32_t nwork,
                                                        uint32_t n_single, const FgScene *__restrict__ table,
                                                        const __grid_constant__ FgScene single,
                                                        const float4 *__restrict__ rb_spos,
                                                        const uint32_t *__restrict__ rb_ids,
                                                        const float4 *__restrict__ body_vel,
                                                        const float4 *__restrict__ body_cm,
                                                        const uint32_t *__restrict__ rb_start,
                                                        const uint32_t *__restrict__ rb_end,
                                                        float4 *__restrict__ force, float4 *__restrict__ torque,
                                                        const __grid_constant__ StaticArg sta, int add)
{
    for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        FgWork it = fg_work(work, w, n_single);
        if (threadIdx.x >= it.count) continue;
        const FgScene *S = fg_scene(table, &single, it.scene);
        const uint32_t i = it.first + threadIdx.x;
        const float4 p = rb_spos[i];
        const int b = (int)p.w;
        const float4 vb = __ldg(body_vel + b);
        const float4 cm = __ldg(body_cm + b);
        const float3 P = make_float3(p.x, p.y, p.z), V = make_float3(vb.x, vb.y, vb.z);
        const float mind = S->rb_radius + S->rb_radius + S->rbrb_eps;
        float3 acc = make_float3(0.f, 0.f, 0.f);
        for (int z = -1; z <= 1; z++) {
            const uint32_t hz = fg_axis_hash_rel(p.z, S->rb_cell[2], z, FG_PZ);
            for (int y = -1; y <= 1; y++) {
                const uint32_t hy = fg_axis_hash_rel(p.y, S->rb_cell[1], y, FG_PY);
                for (int x = -1; x <= 1; x++) {
                    const uint32_t hx = fg_axis_hash_rel(p.x, S->rb_cell[0], x, FG_PX);
                    const uint32_t bk = S->rb_bucket_base + fg_bucket(hx, hy, hz, S->rb_nb, S->rb_nb_mask);
                    const uint32_t st = __ldg(rb_start + bk);
                    if (st == FG_EMPTY) continue;
                    const uint32_t en = __ldg(rb_end + bk);
                    for (uint32_t j = st; j < en; j++) {
                        const float4 q = __ldg(rb_spos + j);
                        if ((int)q.w == b) continue;
                        fg_contact(acc, P, V, q, __ldg(body_vel + (int)q.w), mind, S->rbrb_k, S->rbrb_kd);
                    }
                }
            }
        }
        if (sta.use) {
            for (int z = -1; z <= 1; z++) {
                const uint32_t hz = fg_axis_hash_rel(p.z, S->rb_cell[2], z, FG_PZ);
                for (int y = -1; y <= 1; y++) {
                    const uint32_t hy = fg_axis_hash_rel(p.y, S->rb_cell[1], y, FG_PY);
                    for (int x = -1; x <= 1; x++) {
                        const uint32_t hx = fg_axis_hash_rel(p.x, S->rb_cell[0], x, FG_PX);
                        const uint32_t bk = fg_bucket(hx, hy, hz, sta.g.nb, sta.g.mask);
                        const uint32_t st = __ldg(sta.g.start + bk);
                        if (st == FG_EMPTY) continue;
                        const uint32_t en = __ldg(sta.g.end + bk);
                        for (uint32_t j = st; j < en; j++)
                            fg_contact(acc, P, V, __ldg(sta.g.spos + j), make_float4(0.f, 0.f, 0.f, 0.f), mind,
                                       S->rbrb_k, S->rbrb_kd);
                    }
                }
            }
        }
        const float dx = p.x - cm.x, dy = p.y - cm.y, dz = p.z - cm.z;
        const uint32_t oi = rb_ids ? __ldg(rb_ids + i) : i;
        const float tx = dy * acc.z - dz * acc.y, ty = dz * acc.x - dx * acc.z, tz = dx * acc.y - dy * acc.x;
        if (add) {
            float4 f = force[oi], t = torque[oi];
            f.x += acc.x; f.y += acc.y; f.z += acc.z;
            t.x += tx; t.y += ty; t.z += tz;
            force[oi] = f;
            torque[oi] = t;
        } else {
            const float lw = (float)(b - (int)S->body_base);
            force[oi] = make_float4(acc.x, acc.y, acc.z, lw);
            torque[oi] = make_float4(tx, ty, tz, lw);
        }
    }
}

void launch_rb_from_rb(const Launch &L, const float4 *rb_spos, const uint32_t *rb_ids, const float4 *body_vel,
                       const float4 *body_cm, const uint32_t *rb_start, const uint32_t *rb_end, float4 *force,
                       float4 *torque, const RigidGrid *statics, int add)
{
    if (!L.nwork) return;
    StaticArg sa;
    memset(&sa, 0, sizeof(sa));
    if (statics) { sa.g = *statics; sa.use = 1; }
    k_rb_from_rb<<<grid_for(L.nwork, 16), FG_CHUNK, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, rb_spos,
                                                                   rb_ids, body_vel, body_cm, rb_start, rb_end, force,
                                                                   torque, sa, add);
}

/* ---------------------------------------------------------- FP64 bodies */

__device__ __forceinline__ FgD4 fg_d4(double x, double y, double z, double w)
{
    FgD4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}

struct d4 {
    double x, y, z, w;
};
__device__ __forceinline__ d4 qprod_d(d4 a, d4 b)
{
    d4 r;
    double dotv = a.x * b.x + a.y * b.y + a.z * b.z;
    r.w = a.w * b.w - dotv;
    r.x = (a.w * b.x) + (b.w * a.x) + (a.y * b.z - a.z * b.y);
    r.y = (a.w * b.y) + (b.w * a.y) + (a.z * b.x - a.x * b.z);
    r.z = (a.w * b.z) + (b.w * a.z) + (a.x * b.y - a.y * b.x);
    return r;
}

#define BODY_THREADS 256

/* FP64 partial force/torque sums of one body's spheres: chunk blockIdx.x of
 * FG_BODY_CHUNKS, body blockIdx.y; threads stride the chunk, then a warp
 * shuffle tree and the warps in order (deterministic). */
__global__ void __launch_bounds__(BODY_THREADS) k_body_partial(const uint32_t *__restrict__ body_first,
                                                              const uint32_t *__restrict__ body_count,
                                                              const float4 *__restrict__ force,
                                                              const float4 *__restrict__ torque,
                                                              double *__restrict__ partial)
{
    __shared__ double s_red[BODY_THREADS / 32][8];
    const uint32_t b = blockIdx.y, c = blockIdx.x;
    const uint32_t first = body_first[b], cnt = body_count[b];
    const uint32_t per = (cnt + FG_BODY_CHUNKS - 1) / FG_BODY_CHUNKS;
    const uint32_t lo = min(cnt, c * per), hi = min(cnt, lo + per);
    double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t k = lo + threadIdx.x; k < hi; k += BODY_THREADS) {
        const float4 f = __ldg(force + first + k), t = __ldg(torque + first + k);
        a[0] += f.x; a[1] += f.y; a[2] += f.z; a[3] += f.w;
        a[4] += t.x; a[5] += t.y; a[6] += t.z; a[7] += t.w;
    }
#pragma unroll
    for (int q = 0; q < 8; q++)
#pragma unroll
        for (int o = 16; o; o >>= 1) a[q] += __shfl_xor_sync(0xffffffffu, a[q], o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 8; q++) s_red[wid][q] = a[q];
    __syncthreads();
    if (threadIdx.x < 8) {
        double v = 0.0;
        for (int wv = 0; wv < BODY_THREADS / 32; wv++) v += s_red[wv][threadIdx.x];
        partial[((size_t)b * FG_BODY_CHUNKS + c) * 8 + threadIdx.x] = v;
    }
}

__global__ void __launch_bounds__(BODY_THREADS) k_body_update(const FgScene *__restrict__ table,
                                                             const __grid_constant__ FgScene single,
                                                             const uint32_t *__restrict__ body_scene,
                                                             const uint32_t *__restrict__ body_first,
                                                             const uint32_t *__restrict__ body_count,
                                                             uint32_t nbodies, const float4 *__restrict__ force,
                                                             const float4 *__restrict__ torque, BodyState st,
                                                             int integrate)
{
    __shared__ double s_red[BODY_THREADS / 32][8];
    for (uint32_t b = blockIdx.x; b < nbodies; b += gridDim.x) {
        const uint32_t first = body_first[b], cnt = st.partial ? 0u : body_count[b];
        double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (uint32_t k = threadIdx.x; k < cnt; k += BODY_THREADS) {
            float4 f = __ldg(force + first + k), t = __ldg(torque + first + k);
            a[0] += f.x; a[1] += f.y; a[2] += f.z; a[3] += f.w;
            a[4] += t.x; a[5] += t.y; a[6] += t.z; a[7] += t.w;
        }
#pragma unroll
        for (int c = 0; c < 8; c++)
#pragma unroll
            for (int o = 16; o; o >>= 1) a[c] += __shfl_xor_sync(0xffffffffu, a[c], o);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 8; c++) s_red[wid][c] = a[c];
        __syncthreads();
        if (threadIdx.x == 0) {
            double F[4] = {0, 0, 0, 0}, T[4] = {0, 0, 0, 0};
            if (st.partial) {
                const double *pp = st.partial + (size_t)b * FG_BODY_CHUNKS * 8;
                for (int ch = 0; ch < FG_BODY_CHUNKS; ch++)
                    for (int c = 0; c < 4; c++) {
                        F[c] += pp[ch * 8 + c];
                        T[c] += pp[ch * 8 + 4 + c];
                    }
            } else {
                for (int wv = 0; wv < BODY_THREADS / 32; wv++)
                    for (int c = 0; c < 4; c++) {
                        F[c] += s_red[wv][c];
                        T[c] += s_red[wv][4 + c];
                    }
            }
            st.force_sum[b] = fg_d4(F[0], F[1], F[2], F[3]);
            st.torque_sum[b] = fg_d4(T[0], T[1], T[2], T[3]);
            /* mass 0: a static body (the reference's "static" rigid-body
             * file type), never integrated */
            if (integrate && st.mass[b] != 0.0) {
                const FgScene *S = table ? table + body_scene[b] : &single;
                /* IntegrateRBK in double */
                const double vl = S->rb_vlimit;
                double spd = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3]);
                if (spd > vl) {
                    double t = vl / spd;
                    for (int c = 0; c < 4; c++) F[c] *= t;
                }
                const double dt = S->rb_dt, m = st.mass[b];
                FgD4 x = st.x[b], v = st.v[b], L = st.L[b], q4 = st.q[b];
                double acc[4];
                for (int c = 0; c < 4; c++) acc[c] = ((F[c] + (double)S->rb_gravity[c]) / m) * dt;
                v.x += acc[0] * dt; v.y += acc[1] * dt; v.z += acc[2] * dt; v.w += acc[3] * dt;
                x.x += v.x * dt; x.y += v.y * dt; x.z += v.z * dt;
                const double damp = (double)0.9f;
                L.x = (L.x + T[0] * dt) * damp;
                L.y = (L.y + T[1] * dt) * damp;
                L.z = (L.z + T[2] * dt) * damp;
                L.w = (L.w + T[3] * dt) * damp;
                /* AngularVelocityD: R * Iinv * R^T * L */
                const double *I = st.inv_inertia + 9 * b;
                d4 q = {q4.x, q4.y, q4.z, q4.w};
                double R[3][3];
                R[0][0] = 1.0 - (2.0 * q.y * q.y) - (2.0 * q.z * q.z);
                R[0][1] = (2.0 * q.x * q.y) + (2.0 * q.w * q.z);
                R[0][2] = (2.0 * q.x * q.z) - (2.0 * q.w * q.y);
                R[1][0] = (2.0 * q.x * q.y) - (2.0 * q.w * q.z);
                R[1][1] = 1.0 - (2.0 * q.x * q.x) - (2.0 * q.z * q.z);
                R[1][2] = (2.0 * q.y * q.z) + (2.0 * q.w * q.x);
                R[2][0] = (2.0 * q.x * q.z) + (2.0 * q.w * q.y);
                R[2][1] = (2.0 * q.y * q.z) - (2.0 * q.w * q.x);
                R[2][2] = 1.0 - (2.0 * q.x * q.x) - (2.0 * q.y * q.y);
                double Tm[3][3], G[3][3];
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++)
                        Tm[r][c] = R[r][0] * I[0 * 3 + c] + R[r][1] * I[1 * 3 + c] + R[r][2] * I[2 * 3 + c];
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) G[r][c] = Tm[r][0] * R[c][0] + Tm[r][1] * R[c][1] + Tm[r][2] * R[c][2];
                d4 om;
                om.x = G[0][0] * L.x + G[0][1] * L.y + G[0][2] * L.z;
                om.y = G[1][0] * L.x + G[1][1] * L.y + G[1][2] * L.z;
                om.z = G[2][0] * L.x + G[2][1] * L.y + G[2][2] * L.z;
                om.w = 0.0;
                om = qprod_d(om, q);
                const double half = (double)0.5f, tenth = (double)0.1f;
                om.x *= half; om.y *= half; om.z *= half; om.w *= half;
                d4 ws = {om.x * dt * tenth, om.y * dt * tenth, om.z * dt * tenth, om.w * dt * tenth};
                d4 dq = qprod_d(ws, q);
                q.x += dq.x; q.y += dq.y; q.z += dq.z; q.w += dq.w;
                double nrm = sqrt(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
                q.x /= nrm; q.y /= nrm; q.z /= nrm; q.w /= nrm;
                const double rest = (double)-0.7f;
                if (x.y < (double)S->rb_vmin[1]) { x.y = S->rb_vmin[1]; v.y *= rest; }
                if (x.x <= (double)S->rb_vmin[0]) { x.x = S->rb_vmin[0]; v.x *= rest; }
                else if (x.x >= (double)S->rb_vmax[0]) { x.x = S->rb_vmax[0]; v.x *= rest; }
                if (x.z <= (double)S->rb_vmin[2]) { x.z = S->rb_vmin[2]; v.z *= rest; }
                else if (x.z >= (double)S->rb_vmax[2]) { x.z = S->rb_vmax[2]; v.z *= rest; }
                st.x[b] = x;
                st.v[b] = v;
                st.L[b] = L;
                st.q[b] = fg_d4(q.x, q.y, q.z, q.w);
                st.x_f[b] = make_float4((float)x.x, (float)x.y, (float)x.z, (float)x.w);
                st.v_f[b] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
                st.q_f[b] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
            }
        }
        __syncthreads();
    }
}

void launch_body_update(const FgScene *table, const FgScene *single, const uint32_t *body_scene,
                        const uint32_t *body_first, const uint32_t *body_count, uint32_t nbodies,
                        const float4 *force, const float4 *torque, BodyState st, int integrate, cudaStream_t s)
{
    if (!nbodies) return;
    if (st.partial && nbodies <= 65535u)
        k_body_partial<<<dim3(FG_BODY_CHUNKS, nbodies), BODY_THREADS, 0, s>>>(body_first, body_count, force, torque,
                                                                            st.partial);
    else
        st.partial = nullptr;
    k_body_update<<<grid_for(nbodies, 4), BODY_THREADS, 0, s>>>(table, *single, body_scene, body_first, body_count,
                                                                nbodies, force, torque, st, integrate);
}

/* ---------------------------------------------- FP32 IntegrateRBK (exact) */
__device__ __forceinline__ float4 f4add(float4 a, float4 b)
{
    return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 f4muls(float4 a, float s)
{
    return make_float4(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}

__global__ void k_integrate_rb_f32(float4 *__restrict__ X, const float *__restrict__ mass, float4 *__restrict__ V,
                                   const float4 *__restrict__ Fin, uint32_t nrb, float dt, float4 ext, float3 vmin,
                                   float3 vmax, float4 *__restrict__ Lm, const float4 *__restrict__ Tq,
                                   float4 *__restrict__ Q, const float4 *__restrict__ inv, float vlimit)
{
    uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nrb) return;
    float4 F = Fin[idx];
    float spd = __fsqrt_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(F.x, F.x), __fmul_rn(F.y, F.y)),
                                               __fmul_rn(F.z, F.z)),
                                     __fmul_rn(F.w, F.w)));
    if (spd > vlimit) F = f4muls(F, __fdiv_rn(vlimit, spd));
    float4 pos = X[idx];
    float m = mass[idx];
    float4 fe = f4add(F, ext);
    float4 acc = make_float4(__fmul_rn(__fdiv_rn(fe.x, m), dt), __fmul_rn(__fdiv_rn(fe.y, m), dt),
                             __fmul_rn(__fdiv_rn(fe.z, m), dt), __fmul_rn(__fdiv_rn(fe.w, m), dt));
    float4 vel = f4add(V[idx], f4muls(acc, dt));
    pos.x = __fadd_rn(pos.x, __fmul_rn(vel.x, dt));
    pos.y = __fadd_rn(pos.y, __fmul_rn(vel.y, dt));
    pos.z = __fadd_rn(pos.z, __fmul_rn(vel.z, dt));
    float4 L = f4add(Lm[idx], f4muls(Tq[idx], dt));
    L = f4muls(L, 0.9f);
    Lm[idx] = L;
    /* AngularVelocityD */
    float4 q = Q[idx];
    float R[3][3];
    R[0][0] = __fsub_rn(__fsub_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, q.y), q.y)), __fmul_rn(__fmul_rn(2.0f, q.z), q.z));
    R[0][1] = __fadd_rn(__fmul_rn(__fmul_rn(2.0f, q.x), q.y), __fmul_rn(__fmul_rn(2.0f, q.w), q.z));
    R[0][2] = __fsub_rn(__fmul_rn(__fmul_rn(2.0f, q.x), q.z), __fmul_rn(__fmul_rn(2.0f, q.w), q.y));
    R[1][0] = __fsub_rn(__fmul_rn(__fmul_rn(2.0f, q.x), q.y), __fmul_rn(__fmul_rn(2.0f, q.w), q.z));
    R[1][1] = __fsub_rn(__fsub_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, q.x), q.x)), __fmul_rn(__fmul_rn(2.0f, q.z), q.z));
    R[1][2] = __fadd_rn(__fmul_rn(__fmul_rn(2.0f, q.y), q.z), __fmul_rn(__fmul_rn(2.0f, q.w), q.x));
    R[2][0] = __fadd_rn(__fmul_rn(__fmul_rn(2.0f, q.x), q.z), __fmul_rn(__fmul_rn(2.0f, q.w), q.y));
    R[2][1] = __fsub_rn(__fmul_rn(__fmul_rn(2.0f, q.y), q.z), __fmul_rn(__fmul_rn(2.0f, q.w), q.x));
    R[2][2] = __fsub_rn(__fsub_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, q.x), q.x)), __fmul_rn(__fmul_rn(2.0f, q.y), q.y));
    float I[3][3];
    for (int r = 0; r < 3; r++) {
        float4 row = inv[idx * 3 + r];
        I[r][0] = row.x; I[r][1] = row.y; I[r][2] = row.z;
    }
    float Tm[3][3], G[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            Tm[r][c] = __fadd_rn(__fadd_rn(__fmul_rn(R[r][0], I[0][c]), __fmul_rn(R[r][1], I[1][c])),
                                 __fmul_rn(R[r][2], I[2][c]));
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            G[r][c] = __fadd_rn(__fadd_rn(__fmul_rn(Tm[r][0], R[c][0]), __fmul_rn(Tm[r][1], R[c][1])),
                                __fmul_rn(Tm[r][2], R[c][2]));
    float4 om;
    om.x = __fadd_rn(__fadd_rn(__fmul_rn(G[0][0], L.x), __fmul_rn(G[0][1], L.y)), __fmul_rn(G[0][2], L.z));
    om.y = __fadd_rn(__fadd_rn(__fmul_rn(G[1][0], L.x), __fmul_rn(G[1][1], L.y)), __fmul_rn(G[1][2], L.z));
    om.z = __fadd_rn(__fadd_rn(__fmul_rn(G[2][0], L.x), __fmul_rn(G[2][1], L.y)), __fmul_rn(G[2][2], L.z));
    om.w = 0.0f;
    om = f4muls(fg_qprod_rn(om, q), 0.5f);
    float4 dq = fg_qprod_rn(f4muls(f4muls(om, dt), 0.1f), q);
    q = f4add(q, dq);
    float nrm = __fsqrt_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(q.w, q.w), __fmul_rn(q.x, q.x)),
                                               __fmul_rn(q.y, q.y)),
                                     __fmul_rn(q.z, q.z)));
    q = make_float4(__fdiv_rn(q.x, nrm), __fdiv_rn(q.y, nrm), __fdiv_rn(q.z, nrm), __fdiv_rn(q.w, nrm));
    Q[idx] = q;
    if (pos.y < vmin.y) { pos.y = vmin.y; vel.y = __fmul_rn(vel.y, -0.7f); }
    if (pos.x <= vmin.x) { pos.x = vmin.x; vel.x = __fmul_rn(vel.x, -0.7f); }
    else if (pos.x >= vmax.x) { pos.x = vmax.x; vel.x = __fmul_rn(vel.x, -0.7f); }
    if (pos.z <= vmin.z) { pos.z = vmin.z; vel.z = __fmul_rn(vel.z, -0.7f); }
    else if (pos.z >= vmax.z) { pos.z = vmax.z; vel.z = __fmul_rn(vel.z, -0.7f); }
    X[idx] = pos;
    V[idx] = vel;
}

void launch_integrate_rb_f32(float4 *x, const float *mass, float4 *v, const float4 *f, uint32_t nrb, float dt,
                             float4 ext, float3 vmin, float3 vmax, float4 *L, const float4 *t, const float4 *inertia,
                             float4 *q, const float4 *inv, float vlimit, cudaStream_t s)
{
    (void)inertia;
    if (!nrb) return;
    k_integrate_rb_f32<<<(nrb + 127) / 128, 128, 0, s>>>(x, mass, v, f, nrb, dt, ext, vmin, vmax, L, t, q, inv,
                                                         vlimit);
}

/* ------------------------------- reference reduction data flow (drop-in) */

__global__ void k_copy_rb_data(uint32_t *key, uint32_t *idx, const float4 *force, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        key[i] = (uint32_t)force[i].w;
        idx[i] = i;
    }
}

void launch_copy_rb_data_to_particle(uint32_t *key, uint32_t *idx, const float4 *force, uint32_t n, cudaStream_t s)
{
    if (!n) return;
    k_copy_rb_data<<<grid_for((n + 255) / 256, 8), 256, 0, s>>>(key, idx, force, n);
}

__global__ void k_reorder_ft(float4 *fo, float4 *to, const float4 *fi, const float4 *ti, const uint32_t *order,
                             uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t o = order[i];
        fo[i] = fi[o];
        to[i] = ti[o];
    }
}

void launch_reorder_force_torque(float4 *fo, float4 *to, const float4 *fi, const float4 *ti, const uint32_t *order,
                                 uint32_t n, cudaStream_t s)
{
    if (!n) return;
    k_reorder_ft<<<grid_for((n + 255) / 256, 8), 256, 0, s>>>(fo, to, fi, ti, order, n);
}

/* Inclusive forward segmented sum of float4 (segment heads flagged with a
 * non-zero flag), one CTA walking the array in 1024-element chunks with a
 * carried segment total. */
__global__ void __launch_bounds__(1024) k_segsum(const float4 *__restrict__ in, const uint32_t *__restrict__ flags,
                                                 float4 *__restrict__ out, uint32_t n)
{
    __shared__ float4 s_v[32];
    __shared__ uint32_t s_f[32];
    __shared__ float4 s_carry;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    for (uint32_t base = 0; base < n; base += 1024) {
        uint32_t i = base + threadIdx.x;
        float4 v = i < n ? in[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t f = i < n ? (flags[i] ? 1u : 0u) : 0u;
        /* warp segmented inclusive scan */
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            float4 u = make_float4(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o),
                                   __shfl_up_sync(0xffffffffu, v.z, o), __shfl_up_sync(0xffffffffu, v.w, o));
            uint32_t g = __shfl_up_sync(0xffffffffu, f, o);
            if (lane >= (uint32_t)o && !f) {
                v.x += u.x; v.y += u.y; v.z += u.z; v.w += u.w;
            }
            if (lane >= (uint32_t)o) f |= g;
        }
        if (lane == 31) { s_v[wid] = v; s_f[wid] = f; }
        __syncthreads();
        if (wid == 0) {
            float4 wv = s_v[lane];
            uint32_t wf = s_f[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                float4 u = make_float4(__shfl_up_sync(0xffffffffu, wv.x, o), __shfl_up_sync(0xffffffffu, wv.y, o),
                                       __shfl_up_sync(0xffffffffu, wv.z, o), __shfl_up_sync(0xffffffffu, wv.w, o));
                uint32_t g = __shfl_up_sync(0xffffffffu, wf, o);
                if (lane >= (uint32_t)o && !wf) {
                    wv.x += u.x; wv.y += u.y; wv.z += u.z; wv.w += u.w;
                }
                if (lane >= (uint32_t)o) wf |= g;
            }
            /* exclusive prefix for warp `lane` (carry from previous chunk) */
            float4 pv = make_float4(__shfl_up_sync(0xffffffffu, wv.x, 1), __shfl_up_sync(0xffffffffu, wv.y, 1),
                                    __shfl_up_sync(0xffffffffu, wv.z, 1), __shfl_up_sync(0xffffffffu, wv.w, 1));
            uint32_t pf = __shfl_up_sync(0xffffffffu, wf, 1);
            float4 c = s_carry;
            __syncwarp();
            if (lane == 0) { pv = c; pf = 0; }
            else if (!pf) { pv.x += c.x; pv.y += c.y; pv.z += c.z; pv.w += c.w; }
            s_v[lane] = pv;
            if (lane == 31) {
                float4 last = wv;
                if (!wf) { last.x += c.x; last.y += c.y; last.z += c.z; last.w += c.w; }
                s_carry = last;
            }
        }
        __syncthreads();
        if (i < n) {
            if (!f) {
                float4 p = s_v[wid];
                v.x += p.x; v.y += p.y; v.z += p.z; v.w += p.w;
            }
            out[i] = v;
        }
        __syncthreads();
    }
}

void launch_segmented_sum(const float4 *in, const uint32_t *flags, float4 *out, uint32_t n, cudaStream_t s)
{
    if (!n) return;
    k_segsum<<<1, 1024, 0, s>>>(in, flags, out, n);
}

__global__ void k_add_ft(const float4 *sum_f, const float4 *sum_t, const float4 *ordered_f, float4 *out_f,
                         float4 *out_t, const int *offsets, uint32_t nrb)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrb) return;
    int o = offsets[i];
    int b = (int)ordered_f[o].w;
    float4 f = sum_f[o], t = sum_t[o];
    float4 a = out_f[b], c = out_t[b];
    out_f[b] = make_float4(a.x + f.x, a.y + f.y, a.z + f.z, a.w + f.w);
    out_t[b] = make_float4(c.x + t.x, c.y + t.y, c.z + t.z, c.w + t.w);
}

void launch_add_force_torque(const float4 *sum_f, const float4 *sum_t, const float4 *ordered_f, float4 *out_f,
                             float4 *out_t, const int *offsets, uint32_t nrb, cudaStream_t s)
{
    if (!nrb) return;
    k_add_ft<<<(nrb + 127) / 128, 128, 0, s>>>(sum_f, sum_t, ordered_f, out_f, out_t, offsets, nrb);
}

} // namespace fg
