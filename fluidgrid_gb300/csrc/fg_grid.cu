/* Hash-grid build on GB300: particle hash, stable key/index radix sort, cell
 * start/end ranges with the sorted gather of position and velocity.
 *
 * Follows the reference's grid build (GPU_Kernels/K_HashGrid.cu:26-197 and the
 * thrust/CUDPP key-value sorts, K_FluidSim.cu:685-691,
 * RigidBodySimulator.cpp:195-196) with identical results: keys bit-exact,
 * ascending key order with ties in particle-index order, same start/end
 * entries.  All kernels stream coalesced 16-byte loads; the sort is a
 * reduce-then-scan LSD radix sort whose CTAs never wait on one another. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include "fg_device.cuh"
#include "fg_kernels.h"

namespace fg {

int sm_count()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = 152;
    }
    return sms;
}

uint32_t grid_for(uint32_t nwork, int ctas_per_sm)
{
    uint32_t cap = (uint32_t)sm_count() * (uint32_t)ctas_per_sm;
    return std::max(1u, std::min(nwork, cap));
}

/* ------------------------------------------------------------- hashing */

/* CalcHashKeyK (K_HashGrid.cu:26-38): key = bucket_base + HashKeyD(pos),
 * id = particle index.  With cnt, also the counting sort's first pass (as
 * k_bs_count): cnt[key] += 1 by L2 atomics, one per run of equal keys in a
 * warp, and off[i] = the count found there. */
__global__ void __launch_bounds__(FG_CHUNK) k_hash(const FgWork *__restrict__ work, uint32_t nwork, uint32_t n_single,
                                                  const FgScene *__restrict__ table,
                                                  const __grid_constant__ FgScene single,
                                                  const float4 *__restrict__ pos, uint32_t *__restrict__ keys,
                                                  uint32_t *__restrict__ ids, uint32_t *__restrict__ cnt,
                                                  uint32_t *__restrict__ off)
{
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        FgWork it = fg_work(work, w, n_single);
        const FgScene *S = fg_scene(table, &single, it.scene);
        const bool valid = threadIdx.x < it.count;
        const uint32_t i = it.first + threadIdx.x;
        uint32_t k = 0;
        if (valid) {
            float4 p = __ldg(pos + i);
            k = S->bucket_base + fg_hash(p.x, p.y, p.z, S->cell, S->nb, S->nb_mask);
            keys[i] = k;
            if (ids) ids[i] = i;
        }
        if (cnt) { /* uniform: every lane of the warp gets here */
            const uint32_t act = __ballot_sync(0xffffffffu, valid);
            if (valid) {
                const uint32_t peers = __match_any_sync(act, k);
                const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
                uint32_t o = 0;
                if (lane == leader) o = atomicAdd(cnt + k, (uint32_t)__popc(peers));
                off[i] = __shfl_sync(peers, o, leader) + (uint32_t)__popc(peers & ((1u << lane) - 1u));
            }
        }
    }
}

void launch_hash(const Launch &L, const float4 *pos, uint32_t *keys, uint32_t *ids, uint32_t *cnt, uint32_t *off)
{
    if (!L.nwork) return;
    k_hash<<<grid_for(L.nwork, 64), FG_CHUNK, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, pos, keys,
                                                             ids, cnt, off);
}

/* CalcHashKeyWithOffsetK (K_HashGrid.cu:43-63): world = conj(q)*p*q + cm of
 * the sphere's body (w = body index), key of the world position in the
 * rigid grid.  Optionally grows the per-scene AABB of sphere centres (six
 * ordered ints: min xyz, max xyz). */
__global__ void __launch_bounds__(FG_CHUNK) k_hash_offset(const FgWork *__restrict__ work, uint32_t nwork,
                                                         uint32_t n_single, const FgScene *__restrict__ table,
                                                         const __grid_constant__ FgScene single,
                                                         const float4 *__restrict__ local,
                                                         const float4 *__restrict__ cm,
                                                         const float4 *__restrict__ q, float4 *__restrict__ world,
                                                         uint32_t *__restrict__ keys, uint32_t *__restrict__ ids,
                                                         int *__restrict__ aabb)
{
    for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        FgWork it = fg_work(work, w, n_single);
        const FgScene *S = fg_scene(table, &single, it.scene);
        bool ok = threadIdx.x < it.count;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ok) {
            uint32_t i = it.first + threadIdx.x;
            float4 p = __ldg(local + i);
            int b = (int)p.w;
            float4 t = fg_qtransform_rn(p, __ldg(q + b));
            float4 o = __ldg(cm + b);
            a.x = __fadd_rn(t.x, o.x);
            a.y = __fadd_rn(t.y, o.y);
            a.z = __fadd_rn(t.z, o.z);
            a.w = p.w;
            world[i] = a;
            keys[i] = S->rb_bucket_base + fg_hash(a.x, a.y, a.z, S->rb_cell, S->rb_nb, S->rb_nb_mask);
            if (ids) ids[i] = i;
        }
        if (aabb) {
            /* warp-reduce then one atomic per warp per bound */
            float mn[3] = {ok ? a.x : 3.0e38f, ok ? a.y : 3.0e38f, ok ? a.z : 3.0e38f};
            float mx[3] = {ok ? a.x : -3.0e38f, ok ? a.y : -3.0e38f, ok ? a.z : -3.0e38f};
#pragma unroll
            for (int d = 0; d < 3; d++)
#pragma unroll
                for (int o = 16; o; o >>= 1) {
                    mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
                    mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
                }
            if ((threadIdx.x & 31) == 0 && (threadIdx.x >> 5) * 32 < it.count) {
                int *bx = aabb + 6 * it.scene;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    atomicMin(bx + d, fg_float_ord(mn[d]));
                    atomicMax(bx + 3 + d, fg_float_ord(mx[d]));
                }
            }
        }
    }
}

void launch_hash_with_offset(const Launch &L, const float4 *local, const float4 *cm, const float4 *q, float4 *world,
                             uint32_t *keys, uint32_t *ids, int *aabb)
{
    if (!L.nwork) return;
    k_hash_offset<<<grid_for(L.nwork, 16), FG_CHUNK, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, local,
                                                                    cm, q, world, keys, ids, aabb);
}

/* ----------------------------------------------------------- radix sort
 * LSD radix sort, up to 8 bits per pass, tiles of RS_TILE keys:
 *   upsweep   per-tile digit counts          hist[d * T + t]
 *   scan      per digit, exclusive over tiles  (one CTA per digit) + totals
 *   downsweep stable in-tile ranking (warp match_any), shared-memory
 *             staging in digit order, coalesced scatter.
 * Ranks within a tile follow particle order (warp w holds keys
 * [w*512, w*512+512) of the tile, item k of lane l is key w*512 + 32k + l and
 * items are ranked k-major, lane-minor), so each pass is stable. */

#define RS_THREADS 256
#define RS_ITEMS 8
#define RS_TILE (RS_THREADS * RS_ITEMS)
static_assert(RS_TILE == FG_RS_TILE, "scratch sizes elsewhere assume FG_RS_TILE keys per tile");
#define RS_RADIX 256
#define RS_WARPS (RS_THREADS / 32)

size_t radix_hist_words(uint32_t n)
{
    size_t tiles = ((size_t)n + RS_TILE - 1) / RS_TILE;
    return (size_t)RS_RADIX * std::max<size_t>(tiles, 1) + RS_RADIX;
}

int radix_passes(uint32_t bits, uint32_t digit_bits)
{
    if (digit_bits < 1) digit_bits = 1;
    if (digit_bits > 8) digit_bits = 8;
    return (int)((bits + digit_bits - 1) / digit_bits);
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_upsweep(const uint32_t *__restrict__ keys, uint32_t n,
                                                          uint32_t shift, uint32_t mask, uint32_t *__restrict__ hist,
                                                          uint32_t T)
{
    __shared__ uint32_t cnt[RS_RADIX];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t i = base + (size_t)k * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(__ldg(keys + i) >> shift) & mask], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * T + blockIdx.x] = cnt[threadIdx.x];
}

/* block-wide exclusive scan of one value per thread (RS_THREADS threads) */
__device__ __forceinline__ uint32_t rs_block_excl(uint32_t v, uint32_t *s_warp, uint32_t &total)
{
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < RS_WARPS ? s_warp[lane] : 0;
        uint32_t u = t;
#pragma unroll
        for (int o = 1; o < RS_WARPS; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
            if (lane >= (uint32_t)o) u += y;
        }
        if (lane < RS_WARPS) s_warp[lane] = u - t;
        if (lane == RS_WARPS - 1) s_warp[RS_WARPS] = u;
    }
    __syncthreads();
    uint32_t r = x - v + s_warp[wid];
    total = s_warp[RS_WARPS];
    __syncthreads();
    return r;
}

/* One CTA per digit: exclusive scan of hist[d*T .. d*T+T) in place. */
__global__ void __launch_bounds__(RS_THREADS) k_rs_scan(uint32_t *__restrict__ hist, uint32_t T,
                                                       uint32_t *__restrict__ totals)
{
    __shared__ uint32_t s_warp[RS_WARPS + 1];
    uint32_t *h = hist + (size_t)blockIdx.x * T;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < T; base += RS_THREADS) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < T ? h[i] : 0;
        uint32_t tot;
        uint32_t e = rs_block_excl(v, s_warp, tot);
        if (i < T) h[i] = e + carry;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_downsweep(const uint32_t *__restrict__ kin,
                                                            const uint32_t *__restrict__ vin,
                                                            uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                            uint32_t n, uint32_t shift, uint32_t mask,
                                                            const uint32_t *__restrict__ hist,
                                                            const uint32_t *__restrict__ totals, uint32_t T)
{
    __shared__ uint32_t s_keys[RS_TILE];
    __shared__ uint32_t s_vals[RS_TILE];
    __shared__ uint32_t s_whist[RS_WARPS][RS_RADIX];
    __shared__ uint32_t s_goff[RS_RADIX];
    __shared__ uint32_t s_tstart[RS_RADIX];
    __shared__ uint32_t s_warp[RS_WARPS + 1];

    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const size_t base = (size_t)blockIdx.x * RS_TILE;

    /* global offset of each digit for this tile */
    {
        uint32_t tot;
        uint32_t gb = rs_block_excl(totals[tid], s_warp, tot);
        s_goff[tid] = gb + hist[(size_t)tid * T + blockIdx.x];
    }
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) s_whist[w][tid] = 0;
    __syncthreads();

    uint32_t key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t i = base + (size_t)wid * (32 * RS_ITEMS) + (size_t)k * 32 + lane;
        bool valid = i < n;
        key[k] = valid ? __ldg(kin + i) : 0xffffffffu;
        val[k] = valid ? (vin ? __ldg(vin + i) : (uint32_t)i) : 0u;
        uint32_t active = __ballot_sync(0xffffffffu, valid);
        uint32_t r = 0;
        if (valid) {
            uint32_t d = (key[k] >> shift) & mask;
            uint32_t peers = __match_any_sync(active, d);
            uint32_t leader = __ffs(peers) - 1;
            uint32_t b = 0;
            if (lane == leader) {
                b = s_whist[wid][d];
                s_whist[wid][d] = b + __popc(peers);
            }
            b = __shfl_sync(active, b, leader);
            r = b + __popc(peers & lt);
        }
        rank[k] = r;
        __syncwarp();
    }
    __syncthreads();
    /* per digit: exclusive over warps, tile count */
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
        uint32_t c = s_whist[w][tid];
        s_whist[w][tid] = run;
        run += c;
    }
    {
        uint32_t tot;
        uint32_t ts = rs_block_excl(run, s_warp, tot);
        s_tstart[tid] = ts;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t i = base + (size_t)wid * (32 * RS_ITEMS) + (size_t)k * 32 + lane;
        if (i < n) {
            uint32_t d = (key[k] >> shift) & mask;
            uint32_t p = s_tstart[d] + s_whist[wid][d] + rank[k];
            s_keys[p] = key[k];
            s_vals[p] = val[k];
        }
    }
    __syncthreads();
    uint32_t tile_n = (n - base) < (size_t)RS_TILE ? (uint32_t)(n - base) : (uint32_t)RS_TILE;
    for (uint32_t i = tid; i < tile_n; i += RS_THREADS) {
        uint32_t kk = s_keys[i];
        uint32_t d = (kk >> shift) & mask;
        uint32_t g = s_goff[d] + (i - s_tstart[d]);
        kout[g] = kk;
        vout[g] = s_vals[i];
    }
}

__global__ void k_iota_copy(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                            uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        kout[i] = kin[i];
        vout[i] = vin ? vin[i] : i;
    }
}

cudaError_t radix_sort(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out,
                       uint32_t n, uint32_t bits, uint32_t digit_bits, const RadixScratch &s, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (digit_bits < 1) digit_bits = 1;
    if (digit_bits > 8) digit_bits = 8;
    const int P = radix_passes(bits, digit_bits);
    if (P == 0) {
        if (keys_in != keys_out || vals_in != vals_out || !vals_in)
            k_iota_copy<<<grid_for((n + 255) / 256, 8), 256, 0, st>>>(keys_in, vals_in, keys_out, vals_out, n);
        return cudaSuccess;
    }
    const uint32_t T = (n + RS_TILE - 1) / RS_TILE;
    uint32_t *totals = s.hist + (size_t)RS_RADIX * T;
    const bool inplace = (keys_in == keys_out);
    /* choose the first destination so the last pass lands in *_out */
    const uint32_t *kin = keys_in;
    const uint32_t *vin = vals_in;
    bool to_out = (P % 2 == 1) && !inplace;
    for (int p = 0; p < P; p++) {
        uint32_t shift = (uint32_t)p * digit_bits;
        uint32_t b = std::min(digit_bits, bits - shift);
        uint32_t mask = (1u << b) - 1u;
        uint32_t *ko = to_out ? keys_out : s.keys_alt;
        uint32_t *vo = to_out ? vals_out : s.vals_alt;
        k_rs_upsweep<<<T, RS_THREADS, 0, st>>>(kin, n, shift, mask, s.hist, T);
        k_rs_scan<<<RS_RADIX, RS_THREADS, 0, st>>>(s.hist, T, totals);
        k_rs_downsweep<<<T, RS_THREADS, 0, st>>>(kin, vin, ko, vo, n, shift, mask, s.hist, totals, T);
        kin = ko;
        vin = vo;
        to_out = !to_out;
    }
    cudaError_t e = cudaSuccess;
    if (kin != keys_out) {
        e = cudaMemcpyAsync(keys_out, kin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
        const cudaError_t e2 = cudaMemcpyAsync(vals_out, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = e2;
    }
    return e;
}

/* ------------------------------------------- counting sort by bucket
 * Sort variant 2.  The keys are bucket indices below B (the world's total
 * buckets), so the sort counts instead of ranking digits:
 *   end[] zeroed, then k_bs_count (or k_hash, when the step hashes right
 *           before) adds every particle to end[key] (L2 atomics, one per run
 *           of equal keys in a warp) and keeps the count it found there as
 *           the particle's offset in its bucket;
 *   k_bs_tile_sums: the sum of each tile of BS_TILE counts;
 *   k_bs_offsets: per tile, the preceding tiles' sums plus the exclusive
 *           prefix inside the tile give P; start[k] = P[k] for an occupied
 *           bucket, FG_EMPTY for an empty one; end[k] = P[k] + count;
 *   k_bs_scatter: slot = start[key] + offset: keys_out[slot] = key,
 *           tmp[slot] = particle index (in arrival order inside a bucket);
 *   k_bs_rank: the stable order inside each bucket: particle e's rank is
 *           the number of smaller particle indices in its bucket (a bucket
 *           of L particles costs L loads per particle, as the density walk
 *           over that bucket does), vals_out[start + rank] = e;
 *           k_bs_rank_reorder also does the ranges pass's gathers there.
 * The result is the stable sort: (key, particle index) ascending, and the
 * cell ranges come with it. */
#define BS_THREADS 256
#define BS_ITEMS 8
#define BS_TILE (BS_THREADS * BS_ITEMS)
static_assert(BS_THREADS == RS_THREADS, "the tile scans use rs_block_excl");

__global__ void __launch_bounds__(256) k_bs_count(const uint32_t *__restrict__ keys, uint32_t n,
                                                 uint32_t *__restrict__ cnt, uint32_t *__restrict__ off)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    /* warp-uniform loop: a warp's 32 indices are consecutive */
    for (uint32_t b0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); b0 < n; b0 += stride) {
        const uint32_t i = b0 + lane;
        const bool valid = i < n;
        const uint32_t act = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            const uint32_t k = __ldg(keys + i);
            const uint32_t peers = __match_any_sync(act, k);
            const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
            uint32_t o = 0;
            if (lane == leader) o = atomicAdd(cnt + k, (uint32_t)__popc(peers));
            off[i] = __shfl_sync(peers, o, leader) + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        }
    }
}

/* one CTA per tile: the sum of its BS_TILE counts (coalesced reads) */
__global__ void __launch_bounds__(BS_THREADS) k_bs_tile_sums(const uint32_t *__restrict__ cnt, uint32_t nb,
                                                            uint32_t *__restrict__ tsum)
{
    __shared__ uint32_t s_warp[RS_WARPS + 1];
    const size_t base = (size_t)blockIdx.x * BS_TILE;
    uint32_t v = 0;
#pragma unroll
    for (int k = 0; k < BS_ITEMS; k++) {
        const size_t i = base + (size_t)k * BS_THREADS + threadIdx.x;
        if (i < nb) v += __ldg(cnt + i);
    }
    uint32_t tot;
    rs_block_excl(v, s_warp, tot);
    if (threadIdx.x == 0) tsum[blockIdx.x] = tot;
}

/* one CTA per tile: the tile's base (the preceding tiles' sums), then the
 * exclusive prefix of its counts in order, staged through shared memory so
 * that every global read and write is coalesced */
__global__ void __launch_bounds__(BS_THREADS) k_bs_offsets(uint32_t *__restrict__ cnt_end, uint32_t nb,
                                                          const uint32_t *__restrict__ tsum,
                                                          uint32_t *__restrict__ start)
{
    __shared__ uint32_t s_c[BS_TILE];
    __shared__ uint32_t s_warp[RS_WARPS + 1];
    const size_t base = (size_t)blockIdx.x * BS_TILE;
    /* the tile's base: the sum of all earlier tiles */
    uint32_t pre = 0;
    for (uint32_t t = threadIdx.x; t < blockIdx.x; t += BS_THREADS) pre += __ldg(tsum + t);
    uint32_t tbase;
    rs_block_excl(pre, s_warp, tbase);
#pragma unroll
    for (int k = 0; k < BS_ITEMS; k++) {
        const size_t i = base + (size_t)k * BS_THREADS + threadIdx.x;
        s_c[k * BS_THREADS + threadIdx.x] = i < nb ? cnt_end[i] : 0u;
    }
    __syncthreads();
    /* thread t scans items t*BS_ITEMS .. +BS_ITEMS of the tile */
    uint32_t c[BS_ITEMS], v = 0;
#pragma unroll
    for (int k = 0; k < BS_ITEMS; k++) {
        c[k] = s_c[threadIdx.x * BS_ITEMS + k];
        v += c[k];
    }
    uint32_t tot;
    uint32_t p = rs_block_excl(v, s_warp, tot) + tbase;
#pragma unroll
    for (int k = 0; k < BS_ITEMS; k++) {
        s_c[threadIdx.x * BS_ITEMS + k] = p; /* the bucket's first index */
        p += c[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BS_ITEMS; k++) {
        const size_t i = base + (size_t)k * BS_THREADS + threadIdx.x;
        if (i < nb) {
            const uint32_t first = s_c[k * BS_THREADS + threadIdx.x];
            const uint32_t count = cnt_end[i];
            start[i] = count ? first : FG_EMPTY;
            cnt_end[i] = first + count;
        }
    }
}

__global__ void __launch_bounds__(256) k_bs_scatter(const uint32_t *__restrict__ keys,
                                                   const uint32_t *__restrict__ off, uint32_t n,
                                                   const uint32_t *__restrict__ start,
                                                   uint32_t *__restrict__ keys_out, uint32_t *__restrict__ tmp)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = __ldg(keys + i);
        const uint32_t slot = __ldg(start + k) + __ldg(off + i);
        keys_out[slot] = k;
        tmp[slot] = i;
    }
}

__global__ void __launch_bounds__(256) k_bs_rank(const uint32_t *__restrict__ keys_out,
                                                const uint32_t *__restrict__ tmp, uint32_t n,
                                                const uint32_t *__restrict__ start, const uint32_t *__restrict__ end,
                                                uint32_t *__restrict__ vals_out)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const uint32_t k = __ldg(keys_out + s);
        const uint32_t st = __ldg(start + k), en = __ldg(end + k);
        const uint32_t e = __ldg(tmp + s);
        uint32_t r = 0;
        for (uint32_t f = st; f < en; f++) r += __ldg(tmp + f) < e ? 1u : 0u;
        vals_out[st + r] = e;
    }
}

/* k_bs_rank and the ranges pass's reorder in one: the particle's sorted
 * index p = start + rank gets its id, position and velocity, inv[id] = p,
 * and a rank-0 particle appends its bucket's first index to runs (in no
 * particular order, as the ranges pass does). */
__global__ void __launch_bounds__(256) k_bs_rank_reorder(const uint32_t *__restrict__ keys_out,
                                                        const uint32_t *__restrict__ tmp, uint32_t n,
                                                        const uint32_t *__restrict__ start,
                                                        const uint32_t *__restrict__ end,
                                                        uint32_t *__restrict__ vals_out, BucketReorder R)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t b0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); b0 < n; b0 += stride) {
        const uint32_t s = b0 + lane;
        const bool valid = s < n;
        uint32_t st = 0, r = 0;
        if (valid) {
            const uint32_t k = __ldg(keys_out + s);
            st = __ldg(start + k);
            const uint32_t en = __ldg(end + k);
            const uint32_t e = __ldg(tmp + s);
            for (uint32_t f = st; f < en; f++) r += __ldg(tmp + f) < e ? 1u : 0u;
            const uint32_t p = st + r;
            vals_out[p] = e;
            R.spos[p] = __ldg(R.pos + e);
            if (R.vel) R.svel[p] = __ldg(R.vel + e);
            if (R.inv) R.inv[e] = p;
        }
        if (R.runs) {
            const bool head = valid && r == 0u;
            const uint32_t m = __ballot_sync(0xffffffffu, head);
            uint32_t base = 0;
            if (lane == 0 && m) base = atomicAdd(R.nruns, (uint32_t)__popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (head) R.runs[base + __popc(m & ((1u << lane) - 1u))] = st;
        }
    }
}

bool bucket_sort(const uint32_t *keys_in, uint32_t *keys_out, uint32_t *vals_out, uint32_t n, uint32_t nbuckets,
                 uint32_t *start, uint32_t *end, const RadixScratch &s, uint32_t scratch_words, cudaStream_t st,
                 const BucketReorder *reorder, bool counted)
{
    const uint32_t T = (nbuckets + BS_TILE - 1) / BS_TILE;
    if (!nbuckets || (size_t)T > scratch_words) return false; /* the tile sums would not fit */
    const uint32_t g = grid_for((n + 255) / 256, 8);
    if (!counted) {
        cudaMemsetAsync(end, 0, sizeof(uint32_t) * (size_t)nbuckets, st);
        if (n) k_bs_count<<<g, 256, 0, st>>>(keys_in, n, end, s.keys_alt);
    }
    k_bs_tile_sums<<<T, BS_THREADS, 0, st>>>(end, nbuckets, s.hist);
    k_bs_offsets<<<T, BS_THREADS, 0, st>>>(end, nbuckets, s.hist, start);
    if (n) {
        k_bs_scatter<<<g, 256, 0, st>>>(keys_in, s.keys_alt, n, start, keys_out, s.vals_alt);
        if (reorder)
            k_bs_rank_reorder<<<g, 256, 0, st>>>(keys_out, s.vals_alt, n, start, end, vals_out, *reorder);
        else
            k_bs_rank<<<g, 256, 0, st>>>(keys_out, s.vals_alt, n, start, end, vals_out);
    }
    return true;
}

/* ---------------------------------------------------------- onesweep
 * Stable LSD radix sort with one kernel per digit pass, after one histogram
 * kernel for all passes (decoupled look-back):
 *   k_os_hist  global digit counts of every pass (one read of the keys)
 *   k_os_scan  exclusive digit bases of every pass
 *   k_os_pass  per tile of RS_TILE keys, taken in launch order through a
 *              counter: rank the keys in the tile exactly as k_rs_downsweep
 *              does, publish the tile's per-digit counts, add up the
 *              preceding tiles' counts by looking back until a tile whose
 *              inclusive prefix is known, publish this tile's inclusive
 *              prefix, scatter.
 * A tile waits only on tiles taken before it, which publish their counts
 * before they wait themselves, so every wait ends; each wait is bounded all
 * the same, and one that gives up sets FG_DEV_SORT_TIMEOUT and goes on. */
#define OS_MAX_PASSES 6
#define OS_AGG 0x40000000u
#define OS_INC 0x80000000u
#define OS_CNT 0x3fffffffu
#define OS_SPIN_LIMIT (1u << 22)
#define OS_WINDOW 8

static uint32_t os_tiles(uint32_t n) { return std::max<uint32_t>((n + RS_TILE - 1) / RS_TILE, 1u); }

size_t onesweep_words(uint32_t n)
{
    /* status words [pass][tile][digit], digit counts/bases [pass][digit], tile counters */
    return (size_t)OS_MAX_PASSES * RS_RADIX * os_tiles(n) + (size_t)OS_MAX_PASSES * RS_RADIX + 32;
}

__global__ void __launch_bounds__(RS_THREADS) k_os_hist(const uint32_t *__restrict__ keys, uint32_t n,
                                                       uint32_t bits, uint32_t db, uint32_t passes,
                                                       uint32_t *__restrict__ counts)
{
    __shared__ uint32_t h[OS_MAX_PASSES][RS_RADIX];
#pragma unroll
    for (int p = 0; p < OS_MAX_PASSES; p++) h[p][threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = __ldg(keys + i);
        for (uint32_t p = 0; p < passes; p++) {
            const uint32_t shift = p * db, b = min(db, bits - shift);
            atomicAdd(&h[p][(k >> shift) & ((1u << b) - 1u)], 1u);
        }
    }
    __syncthreads();
    for (uint32_t p = 0; p < passes; p++) {
        const uint32_t v = h[p][threadIdx.x];
        if (v) atomicAdd(&counts[p * RS_RADIX + threadIdx.x], v);
    }
}

/* one CTA per pass: counts -> exclusive digit bases, in place */
__global__ void __launch_bounds__(RS_THREADS) k_os_scan(uint32_t *__restrict__ counts)
{
    __shared__ uint32_t s_warp[RS_WARPS + 1];
    uint32_t *c = counts + blockIdx.x * RS_RADIX;
    uint32_t tot;
    const uint32_t e = rs_block_excl(c[threadIdx.x], s_warp, tot);
    c[threadIdx.x] = e;
}

__global__ void __launch_bounds__(RS_THREADS) k_os_pass(const uint32_t *__restrict__ kin,
                                                       const uint32_t *__restrict__ vin,
                                                       uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                       uint32_t n, uint32_t shift, uint32_t mask,
                                                       uint32_t *__restrict__ status,
                                                       const uint32_t *__restrict__ bases,
                                                       uint32_t *__restrict__ tile_ctr, uint32_t *__restrict__ err,
                                                       uint32_t spin_limit)
{
    __shared__ uint32_t s_keys[RS_TILE];
    __shared__ uint32_t s_vals[RS_TILE];
    __shared__ uint32_t s_whist[RS_WARPS][RS_RADIX];
    __shared__ uint32_t s_goff[RS_RADIX];
    __shared__ uint32_t s_tstart[RS_RADIX];
    __shared__ uint32_t s_warp[RS_WARPS + 1];
    __shared__ uint32_t s_tile;

    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) s_whist[w][tid] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const size_t base = (size_t)tile * RS_TILE;

    uint32_t key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t i = base + (size_t)wid * (32 * RS_ITEMS) + (size_t)k * 32 + lane;
        bool valid = i < n;
        key[k] = valid ? __ldg(kin + i) : 0xffffffffu;
        val[k] = valid ? (vin ? __ldg(vin + i) : (uint32_t)i) : 0u;
        uint32_t active = __ballot_sync(0xffffffffu, valid);
        uint32_t r = 0;
        if (valid) {
            uint32_t d = (key[k] >> shift) & mask;
            uint32_t peers = __match_any_sync(active, d);
            uint32_t leader = __ffs(peers) - 1;
            uint32_t b = 0;
            if (lane == leader) {
                b = s_whist[wid][d];
                s_whist[wid][d] = b + __popc(peers);
            }
            b = __shfl_sync(active, b, leader);
            r = b + __popc(peers & lt);
        }
        rank[k] = r;
        __syncwarp();
    }
    __syncthreads();
    /* per digit: exclusive over warps, tile count */
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
        uint32_t c = s_whist[w][tid];
        s_whist[w][tid] = run;
        run += c;
    }
    /* publish this tile's count of digit tid, then look back */
    uint32_t *mine = status + (size_t)tile * RS_RADIX + tid;
    uint32_t excl = 0;
    if (tile == 0) {
        atomicExch(mine, OS_INC | run);
    } else {
        atomicExch(mine, OS_AGG | run);
        /* look back OS_WINDOW tiles per round trip: add aggregates from the
         * nearest tile outwards until an inclusive prefix; a tile that has
         * not published yet ends the round, which resumes there */
        int k = (int)tile - 1;
        uint32_t spins = 0;
        bool found = false;
        while (!found) {
            uint32_t v[OS_WINDOW];
#pragma unroll
            for (int q = 0; q < OS_WINDOW; q++)
                v[q] = (k - q >= 0) ? *(volatile const uint32_t *)(status + (size_t)(k - q) * RS_RADIX + tid)
                                    : OS_INC; /* before tile 0: an empty inclusive prefix */
            int used = 0;
            bool stalled = false;
#pragma unroll
            for (int q = 0; q < OS_WINDOW; q++) {
                if (found || stalled) continue;
                if (v[q] & OS_INC) {
                    excl += v[q] & OS_CNT;
                    found = true;
                } else if (v[q] & OS_AGG) {
                    excl += v[q] & OS_CNT;
                    used++;
                } else {
                    stalled = true;
                }
            }
            k -= used;
            if (stalled && ++spins > spin_limit) {
                atomicOr(err, FG_DEV_SORT_TIMEOUT);
                break;
            }
        }
        atomicExch(mine, OS_INC | (excl + run));
    }
    s_goff[tid] = __ldg(bases + tid) + excl;
    {
        uint32_t tot;
        s_tstart[tid] = rs_block_excl(run, s_warp, tot);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t i = base + (size_t)wid * (32 * RS_ITEMS) + (size_t)k * 32 + lane;
        if (i < n) {
            uint32_t d = (key[k] >> shift) & mask;
            uint32_t p = s_tstart[d] + s_whist[wid][d] + rank[k];
            s_keys[p] = key[k];
            s_vals[p] = val[k];
        }
    }
    __syncthreads();
    const uint32_t tile_n = (n - base) < (size_t)RS_TILE ? (uint32_t)(n - base) : (uint32_t)RS_TILE;
    for (uint32_t i = tid; i < tile_n; i += RS_THREADS) {
        uint32_t kk = s_keys[i];
        uint32_t d = (kk >> shift) & mask;
        uint32_t g = s_goff[d] + (i - s_tstart[d]);
        if (g < n) { /* only a wait that gave up leaves g unchecked */
            kout[g] = kk;
            vout[g] = s_vals[i];
        }
    }
}

bool onesweep_sort(const uint32_t *keys_in, uint32_t *keys_out, uint32_t *vals_out, uint32_t n, uint32_t bits,
                   uint32_t digit_bits, const RadixScratch &s, uint32_t *os, uint32_t *err, cudaStream_t st)
{
    if (digit_bits < 1) digit_bits = 1;
    if (digit_bits > 8) digit_bits = 8;
    const int P = radix_passes(bits, digit_bits);
    if (P < 1 || P > OS_MAX_PASSES || n == 0 || keys_in == keys_out) return false;
    const uint32_t T = os_tiles(n);
    uint32_t *status = os;                                        /* [P][T][256] */
    uint32_t *counts = os + (size_t)OS_MAX_PASSES * RS_RADIX * T; /* [P][256] */
    uint32_t *ctr = counts + (size_t)OS_MAX_PASSES * RS_RADIX;    /* [P] */
    cudaMemsetAsync(status, 0, 4 * ((size_t)P * RS_RADIX * T), st);
    cudaMemsetAsync(counts, 0, 4 * ((size_t)OS_MAX_PASSES * RS_RADIX + 32), st);
    k_os_hist<<<grid_for((n + RS_THREADS - 1) / RS_THREADS, 4), RS_THREADS, 0, st>>>(keys_in, n, bits, digit_bits,
                                                                                     (uint32_t)P, counts);
    k_os_scan<<<P, RS_THREADS, 0, st>>>(counts);
    const uint32_t *kin = keys_in;
    const uint32_t *vin = nullptr;
    bool to_out = (P % 2 == 1);
    for (int p = 0; p < P; p++) {
        const uint32_t shift = (uint32_t)p * digit_bits;
        const uint32_t b = std::min(digit_bits, bits - shift);
        const uint32_t mask = (1u << b) - 1u;
        uint32_t *ko = to_out ? keys_out : s.keys_alt;
        uint32_t *vo = to_out ? vals_out : s.vals_alt;
        k_os_pass<<<T, RS_THREADS, 0, st>>>(kin, vin, ko, vo, n, shift, mask, status + (size_t)p * RS_RADIX * T,
                                            counts + (size_t)p * RS_RADIX, ctr + p, err, OS_SPIN_LIMIT);
        kin = ko;
        vin = vo;
        to_out = !to_out;
    }
    return true;
}

/* Self-test of the look-back's bounded wait: one CTA takes tile 1 of a
 * two-tile sort whose tile 0 never publishes, waits spin_limit rounds, sets
 * FG_DEV_SORT_TIMEOUT and returns; every access stays inside the buffers
 * (the scatter skips the positions a wait that gave up leaves unchecked). */
int bounded_wait_selftest(uint32_t spin_limit, uint32_t *flags)
{
    const uint32_t n = 2 * RS_TILE;
    uint32_t *buf = nullptr;
    const size_t words = 3 * (size_t)n + 2 * RS_RADIX + RS_RADIX + 2;
    if (cudaMalloc(&buf, 4 * words) != cudaSuccess) return -1;
    uint32_t *keys = buf, *kout = buf + n, *vout = buf + 2 * n;
    uint32_t *status = buf + 3 * (size_t)n, *bases = status + 2 * RS_RADIX, *ctr = bases + RS_RADIX, *err = ctr + 1;
    cudaMemset(buf, 0, 4 * words);
    const uint32_t one = 1; /* the only CTA takes tile 1 */
    cudaMemcpy(ctr, &one, 4, cudaMemcpyHostToDevice);
    k_os_pass<<<1, RS_THREADS>>>(keys, nullptr, kout, vout, n, 0, 0xffu, status, bases, ctr, err, spin_limit);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(flags, err, 4, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    return e == cudaSuccess ? 0 : -1;
}

/* ------------------------------------------------------ ranges + reorder
 * FindCellOffsetOrderinPosVelK / FindCellOffsetOrderingPosK
 * (K_HashGrid.cu:70-197): start[key] at the first index of each key run,
 * end[previous key] = that index, end[last key] = n; sorted gather of
 * position (and velocity). */
__global__ void __launch_bounds__(256) k_cell_ranges(const uint32_t *__restrict__ keys,
                                                    const uint32_t *__restrict__ ids,
                                                    const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                                    uint32_t *__restrict__ start, uint32_t *__restrict__ end,
                                                    float4 *__restrict__ spos, float4 *__restrict__ svel, uint32_t n,
                                                    uint32_t *__restrict__ inv, uint32_t *__restrict__ runs,
                                                    uint32_t *__restrict__ nruns)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = __ldg(keys + i);
        uint32_t prev = i > 0 ? __ldg(keys + i - 1) : k;
        const bool head = (i == 0 || k != prev);
        if (head) {
            start[k] = i;
            if (i > 0) end[prev] = i;
        }
        if (runs) {
            /* append run heads, one atomic per warp */
            const uint32_t act = __activemask();
            const uint32_t m = __ballot_sync(act, head);
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(act) - 1;
            uint32_t base = 0;
            if (lane == leader && m) base = atomicAdd(nruns, (uint32_t)__popc(m));
            base = __shfl_sync(act, base, leader);
            if (head) runs[base + __popc(m & ((1u << lane) - 1u))] = i;
        }
        if (i == n - 1) end[k] = n;
        uint32_t id = __ldg(ids + i);
        spos[i] = __ldg(pos + id);
        if (vel) svel[i] = __ldg(vel + id);
        if (inv) inv[id] = i; /* particle -> sorted index */
    }
}

void launch_cell_ranges(const uint32_t *keys, const uint32_t *ids, const float4 *pos, const float4 *vel,
                        uint32_t *start, uint32_t *end, float4 *spos, float4 *svel, uint32_t n, cudaStream_t st,
                        uint32_t *inv, uint32_t *runs, uint32_t *nruns)
{
    if (!n) return;
    k_cell_ranges<<<grid_for((n + 255) / 256, 32), 256, 0, st>>>(keys, ids, pos, vel, start, end, spos, svel, n,
                                                                inv, runs, nruns);
}

/* ------------------------------------------------ spatial target order
 * Density and force kernels process their targets in a spatially coherent
 * order so that a CTA's particles share neighbour cells and the neighbour
 * loads hit L1 (the hashed bucket order scatters a CTA over random cells).
 * The key is the scene id above a Morton code of the particle's cell,
 * counted from the scene's volume_min and clamped to 2^bits cells per axis;
 * a particle outside that range only loses locality, never correctness. */
__device__ __forceinline__ uint32_t fg_spread3(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void __launch_bounds__(FG_CHUNK) k_morton_keys(const FgWork *__restrict__ work, uint32_t nwork,
                                                         uint32_t n_single, const FgScene *__restrict__ table,
                                                         const __grid_constant__ FgScene single,
                                                         const float4 *__restrict__ pos, uint32_t *__restrict__ keys,
                                                         uint32_t bits, uint32_t scene_shift)
{
    const int lim = (1 << bits) - 1;
    for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        FgWork it = fg_work(work, w, n_single);
        if (threadIdx.x >= it.count) continue;
        const FgScene *S = fg_scene(table, &single, it.scene);
        const uint32_t t = it.first + threadIdx.x;
        const float4 p = __ldg(pos + t);
        int c[3];
        const float q[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            /* the hash grid's own cell index (relative to the scene's lower
             * corner): a Morton cell is exactly one hashed cell, so a run of
             * targets shares its 27 buckets as in bucket order */
            const int v = fg_axis_index(q[a], S->cell[a]) - fg_axis_index(S->vmin[a], S->cell[a]) + 2;
            c[a] = v < 0 ? 0 : (v > lim ? lim : v);
        }
        const uint32_t m = (fg_spread3((uint32_t)c[0]) | (fg_spread3((uint32_t)c[1]) << 1) |
                            (fg_spread3((uint32_t)c[2]) << 2));
        keys[t] = (scene_shift < 32 ? (it.scene << scene_shift) : 0u) | m;
    }
}

void launch_morton_keys(const Launch &L, const float4 *pos, uint32_t *keys, uint32_t bits, uint32_t scene_shift)
{
    if (!L.nwork) return;
    k_morton_keys<<<grid_for(L.nwork, 16), FG_CHUNK, 0, L.stream>>>(L.work, L.nwork, L.n, L.table, *L.single, pos,
                                                                    keys, bits, scene_shift);
}

/* ------------------------------------------ rigid-sphere grid per scene
 * The sort + start/end of FindCellOffsetOrderingPosK (K_HashGrid.cu:140-197)
 * for the rigid-sphere grid, in one CTA per scene when every scene has at
 * most FG_RB_SCENE_MAX spheres.  The scene's (key, index) pairs are sorted
 * as 64-bit words by a bitonic network in shared memory -- the index in the
 * low word makes the order the stable one, so keys, ids and ranges equal the
 * radix path's bit for bit.  A scene's spheres and rigid buckets are its own
 * ranges of the global arrays, and the global stable order is the scenes'
 * orders one after another (keys carry the scene's rigid bucket base). */
__global__ void __launch_bounds__(1024) k_rb_sort_ranges(const FgScene *__restrict__ table,
                                                        const __grid_constant__ FgScene single,
                                                        const uint32_t *__restrict__ keys_u,
                                                        const float4 *__restrict__ world,
                                                        uint32_t *__restrict__ keys, uint32_t *__restrict__ ids,
                                                        float4 *__restrict__ spos, uint32_t *__restrict__ rstart,
                                                        uint32_t *__restrict__ rend)
{
    __shared__ unsigned long long s[FG_RB_SCENE_MAX];
    const FgScene *S = table ? table + blockIdx.x : &single;
    const uint32_t n = S->nsph, base = S->sph_base;
    if (!(S->flags & FG_SCENE_HAS_RB)) return; /* the scene has no rigid buckets */
    for (uint32_t b = threadIdx.x; b < S->rb_nb; b += blockDim.x) rstart[S->rb_bucket_base + b] = FG_EMPTY;
    if (!n) return;
    uint32_t P = 1;
    while (P < n) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x)
        s[i] = i < n ? (((unsigned long long)__ldg(keys_u + base + i) << 32) | i) : ~0ull;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1)
        for (uint32_t j = k >> 1; j; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const unsigned long long a = s[i], c = s[l];
                    if ((a > c) == ((i & k) == 0)) {
                        s[i] = c;
                        s[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const unsigned long long v = s[i];
        const uint32_t key = (uint32_t)(v >> 32), id = base + (uint32_t)(v & 0xffffffffu);
        keys[base + i] = key;
        ids[base + i] = id;
        spos[base + i] = __ldg(world + id);
        const uint32_t prev = i ? (uint32_t)(s[i - 1] >> 32) : key;
        if (i == 0 || key != prev) {
            rstart[key] = base + i;
            if (i) rend[prev] = base + i;
        }
        if (i == n - 1) rend[key] = base + n;
    }
}

void launch_rb_sort_ranges(const FgScene *table, const FgScene *single, uint32_t nscenes, const uint32_t *keys_u,
                           const float4 *world, uint32_t *keys, uint32_t *ids, float4 *spos, uint32_t *rstart,
                           uint32_t *rend, cudaStream_t s)
{
    if (!nscenes) return;
    k_rb_sort_ranges<<<nscenes, 1024, 0, s>>>(table, *single, keys_u, world, keys, ids, spos, rstart, rend);
}

__global__ void k_fill(uint32_t *buf, size_t words, uint32_t v)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        buf[i] = v;
}

void launch_fill(uint32_t *buf, size_t words, uint32_t v, cudaStream_t s)
{
    if (!words) return;
    k_fill<<<grid_for((uint32_t)std::min<size_t>((words + 255) / 256, 1u << 30), 8), 256, 0, s>>>(buf, words, v);
}

} // namespace fg
