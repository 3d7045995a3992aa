/* Device helpers shared by the GB300 SPH kernels. */
#ifndef FG_DEVICE_CUH
#define FG_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include "fg_types.h"

#define FG_EMPTY 0xffffffffu

/* ------------------------------------------------------------ hashing
 * Bucket hash of GPU_Kernels/K_DeviceFunctions.cu:17-26, bit-exact:
 * i = (int)((p + 5000) / cell) per axis with IEEE round-to-nearest add and
 * divide (explicit intrinsics, so no contraction or approximate divide can
 * change a cell index), truncation toward zero with saturation (cvt.rzi),
 * wrapping int32 products with the three primes, XOR, unsigned modulo. */
__device__ __forceinline__ int fg_axis_index(float p, float cell)
{
    return __float2int_rz(__fdiv_rn(__fadd_rn(p, 5000.0f), cell));
}

/* Neighbour-cell index along one axis: the reference hashes pos + cell*o
 * (K_FluidSim.cu:191-195); cell*o is exact for o in {-1,0,1}. */
__device__ __forceinline__ int fg_axis_index_off(float p, float cell, int o)
{
    float a = (o == 0) ? p : (o < 0 ? __fsub_rn(p, cell) : __fadd_rn(p, cell));
    return fg_axis_index(a, cell);
}

__device__ __forceinline__ uint32_t fg_bucket(uint32_t hx, uint32_t hy, uint32_t hz, uint32_t nb, uint32_t mask)
{
    uint32_t h = hx ^ hy ^ hz;
    return mask ? (h & mask) : (h % nb);
}

#define FG_PX 73856093u
#define FG_PY 19349663u
#define FG_PZ 83492791u

__device__ __forceinline__ uint32_t fg_hash(float x, float y, float z, const float *cell, uint32_t nb,
                                            uint32_t mask)
{
    return fg_bucket((uint32_t)fg_axis_index(x, cell[0]) * FG_PX, (uint32_t)fg_axis_index(y, cell[1]) * FG_PY,
                     (uint32_t)fg_axis_index(z, cell[2]) * FG_PZ, nb, mask);
}

/* Hashed products of the 3 neighbour indices along each axis (o = -1,0,1).
 * The 27 neighbour buckets are fg_bucket(hx[x], hy[y], hz[z]). */
__device__ __forceinline__ void fg_neighbour_hashes(float px, float py, float pz, const float *cell, uint32_t hx[3],
                                                    uint32_t hy[3], uint32_t hz[3])
{
#pragma unroll
    for (int o = -1; o <= 1; o++) {
        hx[o + 1] = (uint32_t)fg_axis_index_off(px, cell[0], o) * FG_PX;
        hy[o + 1] = (uint32_t)fg_axis_index_off(py, cell[1], o) * FG_PY;
        hz[o + 1] = (uint32_t)fg_axis_index_off(pz, cell[2], o) * FG_PZ;
    }
}

/* Same for a search half-width r (ProcessCollisionForcesD,
 * K_DeviceFunctions.cu:139-149): offset o*cell with o in [-r, r].  o*cell is
 * evaluated as the reference does (float multiply), then added. */
__device__ __forceinline__ uint32_t fg_axis_hash_rel(float p, float cell, int o, uint32_t prime)
{
    float off = __fmul_rn(cell, (float)o);
    return (uint32_t)fg_axis_index(__fadd_rn(p, off), cell) * prime;
}

/* One 32-byte neighbour record (two float4) in a single 256-bit load of
 * read-only data; p must be 32-byte aligned. */
__device__ __forceinline__ void fg_ld_rec(const float4 *p, float4 &a, float4 &b)
{
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

/* Eight list entries (one 32-byte sector) in a single 256-bit load of
 * read-only data; p must be 32-byte aligned.  A list is read once: the load
 * skips L1 and marks its L2 lines evict-first, so the lists stream past the
 * particle records instead of pushing them out of L2. */
__device__ __forceinline__ void fg_ld_idx8(const uint32_t *p, uint4 &a, uint4 &b)
{
    asm("ld.global.nc.L1::no_allocate.L2::evict_first.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
        : "l"(p));
}

/* Two list entries stored with the streaming (evict-first) policy: a list
 * is written once by the density pass and read once by the force pass. */
__device__ __forceinline__ void fg_st_list2(uint32_t *p, uint32_t a, uint32_t b)
{
    /* no memory clobber: no kernel reads a list it writes */
    asm volatile("st.global.cs.v2.b32 [%0], {%1, %2};" ::"l"(p), "r"(a), "r"(b));
}

/* select one of three register values without local-memory indexing */
__device__ __forceinline__ uint32_t fg_sel3(uint32_t a0, uint32_t a1, uint32_t a2, int k)
{
    return k == 0 ? a0 : (k == 1 ? a1 : a2);
}

/* ------------------------------------------------------- work items */

/* Resolve work item w to (scene, first, count).  With no table, the single
 * scene's particles [0, n) are cut into FG_CHUNK-sized items. */
__device__ __forceinline__ FgWork fg_work(const FgWork *table, uint32_t w, uint32_t n_single)
{
    if (table) return table[w];
    FgWork r;
    r.scene = 0;
    r.first = w * FG_CHUNK;
    uint32_t left = n_single - r.first;
    r.count = left < FG_CHUNK ? left : FG_CHUNK;
    r.pad = 0;
    return r;
}

__device__ __forceinline__ const FgScene *fg_scene(const FgScene *table, const FgScene *single, uint32_t s)
{
    return table ? table + s : single;
}

/* ------------------------------------------------- exact quaternion math
 * Quaternion_ProductD / Quaternion_TransformPointD
 * (GPU_Kernels/K_MathUtils.cu:57-70, 160-181) in IEEE single precision with
 * every operation rounded on its own, so rigid-sphere world positions (and
 * the bucket keys hashed from them) are bit-identical to the source order. */
__device__ __forceinline__ float4 fg_qprod_rn(float4 a, float4 b)
{
    float dotv = __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
    float w = __fsub_rn(__fmul_rn(a.w, b.w), dotv);
    float cx = __fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y));
    float cy = __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z));
    float cz = __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x));
    float4 r;
    r.x = __fadd_rn(__fadd_rn(__fmul_rn(a.w, b.x), __fmul_rn(b.w, a.x)), cx);
    r.y = __fadd_rn(__fadd_rn(__fmul_rn(a.w, b.y), __fmul_rn(b.w, a.y)), cy);
    r.z = __fadd_rn(__fadd_rn(__fmul_rn(a.w, b.z), __fmul_rn(b.w, a.z)), cz);
    r.w = w;
    return r;
}

__device__ __forceinline__ float4 fg_qtransform_rn(float4 p, float4 q)
{
    p.w = 0.0f;
    float4 cq = make_float4(-q.x, -q.y, -q.z, q.w);
    return fg_qprod_rn(fg_qprod_rn(cq, p), q);
}

/* ------------------------------------------------------------ walls
 * calculateWallsNoPenetrationForce / calculateWallsNoSlipForce
 * (GPU_Kernels/K_Boundaries_Walls.cu:8-125) with calculateRepulsionForce /
 * calculateFrictionForce (K_Boundaries_Common.cu:12-82). */
__device__ __forceinline__ void fg_wall_push(float3 &f, float d, float nx, float ny, float nz, float3 v,
                                             float stiff, float damp)
{
    float c = stiff * d - damp * (nx * v.x + ny * v.y + nz * v.z);
    f.x += c * nx;
    f.y += c * ny;
    f.z += c * nz;
}

__device__ __forceinline__ void fg_wall_friction(float3 &f, float nx, float ny, float nz, float3 v, float fkin,
                                                 float fstatic)
{
    float vn = nx * v.x + ny * v.y + nz * v.z;
    float tx = v.x - v.x * vn, ty = v.y - v.y * vn, tz = v.z - v.z * vn;
    float s = ((tx + ty + tz) / 3.0f > fstatic) ? 1.0f : fkin;
    f.x += s * -tx;
    f.y += s * -ty;
    f.z += s * -tz;
}

/* Single-instruction approximations (PTX rsqrt.approx.ftz / rcp.approx.ftz)
 * for operands that are never denormal: a squared pair distance (or 0 for
 * coincident particles, giving +inf as before) and a density product >= 1. */
__device__ __forceinline__ float fg_rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float fg_rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float3 fg_walls(const FgScene &S, float3 p, float3 v)
{
    const float eps = 0.00001f;
    float3 f = make_float3(0.f, 0.f, 0.f);
    float d;
    d = S.wall_dist - (p.y - S.vmin[1]) * S.scale;
    if (d > eps) fg_wall_push(f, d, 0.f, 1.f, 0.f, v, S.wall_stiff, S.wall_damp);
    d = S.wall_dist - (S.vmax[1] - p.y) * S.scale;
    if (d > eps) fg_wall_push(f, d, 0.f, -1.f, 0.f, v, S.wall_stiff, S.wall_damp);
    d = S.wall_dist - (p.z - S.vmin[2]) * S.scale;
    if (d > eps) fg_wall_push(f, d, 0.f, 0.f, 1.f, v, S.wall_stiff, S.wall_damp);
    d = S.wall_dist - (S.vmax[2] - p.z) * S.scale;
    if (d > eps) fg_wall_push(f, d, 0.f, 0.f, -1.f, v, S.wall_stiff, S.wall_damp);
    d = S.wall_dist - (p.x - S.vmin[0]) * S.scale;
    if (d > eps) fg_wall_push(f, d, 1.f, 0.f, 0.f, v, S.wall_stiff, S.wall_damp);
    d = S.wall_dist - (S.vmax[0] - p.x) * S.scale;
    if (d > eps) fg_wall_push(f, d, -1.f, 0.f, 0.f, v, S.wall_stiff, S.wall_damp);
    /* no-slip walls of the literal box (friction uses the velocity only) */
    d = S.wall_dist - (p.y - S.noslip_min[1]) * S.scale;
    if (d > eps) fg_wall_friction(f, 0.f, 1.f, 0.f, v, S.fric_kin, S.fric_static);
    d = S.wall_dist - (S.noslip_max[1] - p.y) * S.scale;
    if (d > eps) fg_wall_friction(f, 0.f, -1.f, 0.f, v, S.fric_kin, S.fric_static);
    d = S.wall_dist - (p.z - S.noslip_min[2]) * S.scale;
    if (d > eps) fg_wall_friction(f, 0.f, 0.f, 1.f, v, S.fric_kin, S.fric_static);
    d = S.wall_dist - (S.noslip_max[2] - p.z) * S.scale;
    if (d > eps) fg_wall_friction(f, 0.f, 0.f, -1.f, v, S.fric_kin, S.fric_static);
    d = S.wall_dist - (p.x - S.noslip_min[0]) * S.scale;
    if (d > eps) fg_wall_friction(f, 1.f, 0.f, 0.f, v, S.fric_kin, S.fric_static);
    d = S.wall_dist - (S.noslip_max[0] - p.x) * S.scale;
    if (d > eps) fg_wall_friction(f, -1.f, 0.f, 0.f, v, S.fric_kin, S.fric_static);
    return f;
}

/* ------------------------------------------------- sphere contact
 * One candidate of ProcessCellForcesD (K_DeviceFunctions.cu:82-100):
 * contact when |q - p| < mind, force (k*lg - kd*dot(n, vq - vp)) * n with
 * n = (q - p)/lg. */
__device__ __forceinline__ void fg_contact(float3 &acc, float3 p, float3 vp, float4 q, float4 vq, float mind,
                                           float k, float kd)
{
    float rx = q.x - p.x, ry = q.y - p.y, rz = q.z - p.z;
    float lg = sqrtf(rx * rx + ry * ry + rz * rz);
    if (lg < mind) {
        float inv = 1.0f / lg;
        float nx = rx * inv, ny = ry * inv, nz = rz * inv;
        float c = k * lg - kd * (nx * (vq.x - vp.x) + ny * (vq.y - vp.y) + nz * (vq.z - vp.z));
        acc.x += c * nx;
        acc.y += c * ny;
        acc.z += c * nz;
    }
}

/* float atomics on the ordered-int encoding (for bounding boxes) */
__device__ __forceinline__ int fg_float_ord(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fg_ord_float(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

#endif
