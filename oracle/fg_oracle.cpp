/* FluidGrid SPH hot path -- CPU oracle.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only the tests, the smoke check and
 * the CPU-baseline leg of the benchmark load this library, and only as the
 * checker / the timed CPU restatement of the reference.  The product path
 * (fluidgrid_gb300) never calls into it.
 *
 * A line-by-line restatement of the reference's kernel arithmetic as plain
 * host loops (OpenMP over particles).  Every function names the reference
 * file:line it follows (paths relative to the reference project).  FP32
 * functions evaluate each operation in IEEE single precision in the
 * reference's source order; the library is compiled with -ffp-contract=off so
 * nothing is fused.  FP64 instantiations keep the FP32 hash and the FP32
 * neighbour-inclusion tests (so the neighbour sets are identical) and carry
 * every accumulated quantity in double.
 *
 * Pinning, both bit for bit against golden vectors in tests/golden:
 *   - the restated helpers (HashKeyD, wall forces, collision forces,
 *     quaternion math) against the reference's own helper source files
 *     compiled on the host (oracle/ref_wrap.cpp, ref_helpers.npz);
 *   - the restated kernels (density, forces with and without the rigid
 *     grids, integration, hashing, cell ranges, rigid contact and rigid
 *     integration) against the reference's own __global__ kernels run on the
 *     host (oracle/ref_kernels_*.cpp over the kernel sections of
 *     K_FluidSim.cu, K_HashGrid.cu and K_RigidBodySim.cu, ref_kernels.npz).
 * Library math the source calls (powf, sqrtf) is the host C library's on both
 * sides; sqrtf is exact, and the GPU's own powf may differ from the host's in
 * the last bit.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint32_t u32;

/* ------------------------------------------------------------------ types */

struct fgo_float3 { float x, y, z; };
struct fgo_int3 { int x, y, z; };

/* Field order and sizes of Simulation::Application::CommonFluidParams
 * (ApplicationData.cuh:46-67). */
struct fgo_common_fluid_params {
    fgo_float3 cell_size;
    fgo_int3 bucket_size;
    u32 keyBits;
    float kernel_radius;
    float kernel_radius_squared;
    float pointRadius;
    float pointScale;
    float velocity_limit;
    fgo_float3 volume_min;
    fgo_float3 volume_max;
    fgo_float3 global_external_force;
    float simulation_scale;
    float deltaTimeIntegration;
    fgo_int3 fluid_to_srb_relation;
};

/* Simulation::Application::KernelsCache (ApplicationData.cuh:107-112). */
struct fgo_kernels_cache { float kPoly6, kSpikyGradient, kViscosityLaplacian; };

template <typename R> struct V3 { R x, y, z; };
template <typename R> struct V4 { R x, y, z, w; };
typedef V3<float> f3;
typedef V4<float> f4;

template <typename R> static inline V3<R> mk3(R x, R y, R z) { V3<R> v; v.x = x; v.y = y; v.z = z; return v; }
template <typename R> static inline V3<R> add(V3<R> a, V3<R> b) { return mk3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename R> static inline V3<R> sub(V3<R> a, V3<R> b) { return mk3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename R> static inline V3<R> mul(V3<R> a, R s) { return mk3<R>(a.x * s, a.y * s, a.z * s); }
template <typename R> static inline V3<R> smul(R s, V3<R> a) { return mk3<R>(s * a.x, s * a.y, s * a.z); }
template <typename R> static inline V3<R> dvs(V3<R> a, R s) { return mk3<R>(a.x / s, a.y / s, a.z / s); }
template <typename R> static inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float len(f3 v) { return sqrtf(dot(v, v)); }
static inline double len(V3<double> v) { return std::sqrt(dot(v, v)); }
template <typename R> static inline V3<R> xyz(const float *p) { return mk3<R>((R)p[0], (R)p[1], (R)p[2]); }
template <typename R> static inline V3<R> cvt(f3 a) { return mk3<R>((R)a.x, (R)a.y, (R)a.z); }

/* ------------------------------------------------------------------ hash */

/* C float->int conversion with the saturation the GPU's cvt.rzi.s32.f32 uses
 * (values beyond int range clamp, NaN gives 0). */
static inline int f2i_sat(float q)
{
    if (q != q) return 0;
    if (q >= 2147483648.0f) return std::numeric_limits<int>::max();
    if (q <= -2147483648.0f) return std::numeric_limits<int>::min();
    return (int)q;
}

/* HashKeyD, GPU_Kernels/K_DeviceFunctions.cu:17-26.  The int32 products wrap
 * (unsigned arithmetic here); the modulo is unsigned. */
static inline u32 hash_key(float px, float py, float pz, float cx, float cy, float cz, u32 nb)
{
    int x = f2i_sat((px + 5000.0f) / cx);
    int y = f2i_sat((py + 5000.0f) / cy);
    int z = f2i_sat((pz + 5000.0f) / cz);
    u32 h = ((u32)x * 73856093u) ^ ((u32)y * 19349663u) ^ ((u32)z * 83492791u);
    return h % nb;
}

/* The neighbour-bucket hash used inside the 27-cell loops:
 * HashKeyD(make_float3(pos) + cell*(x,y,z), cell, nb)
 * (K_FluidSim.cu:191-195, 237-240; K_DeviceFunctions.cu:146-149). */
static inline u32 hash_offset(f3 p, f3 cell, int xo, int yo, int zo, u32 nb)
{
    float ox = cell.x * (float)xo, oy = cell.y * (float)yo, oz = cell.z * (float)zo;
    return hash_key(p.x + ox, p.y + oy, p.z + oz, cell.x, cell.y, cell.z, nb);
}

static inline f3 cell_of(const fgo_common_fluid_params *p) { return mk3<float>(p->cell_size.x, p->cell_size.y, p->cell_size.z); }
static inline u32 nbuckets_of(const fgo_common_fluid_params *p)
{
    /* CommonFluidParams::getNumBuckets, ApplicationData.cuh:63-66 */
    return (u32)(p->bucket_size.x * p->bucket_size.y * p->bucket_size.z);
}

/* ------------------------------------------------------- boundary forces */

static const float WALL_EPS = 0.00001f; /* EPSILON, K_Boundaries_Walls.cu:6 */

/* calculateRepulsionForce, K_Boundaries_Common.cu:12-23 */
template <typename R>
static inline V3<R> repulsion(V3<R> vel, V3<R> n, R dist, R damp, R stiff)
{
    return smul<R>(stiff * dist - damp * dot(n, vel), n);
}

/* calculateWallsNoPenetrationForce, K_Boundaries_Walls.cu:8-65 */
template <typename R>
static V3<R> walls_no_penetration(V3<R> pos, V3<R> vel, V3<R> gmin, V3<R> gmax, R bd, R stiff, R damp, R scale)
{
    V3<R> f = mk3<R>(0, 0, 0);
    R d;
    d = bd - ((pos.y - gmin.y) * scale);
    if (d > (R)WALL_EPS) f = add(f, repulsion<R>(vel, mk3<R>(0, 1, 0), d, damp, stiff));
    d = bd - ((gmax.y - pos.y) * scale);
    if (d > (R)WALL_EPS) f = add(f, repulsion<R>(vel, mk3<R>(0, -1, 0), d, damp, stiff));
    d = bd - ((pos.z - gmin.z) * scale);
    if (d > (R)WALL_EPS) f = add(f, repulsion<R>(vel, mk3<R>(0, 0, 1), d, damp, stiff));
    d = bd - ((gmax.z - pos.z) * scale);
    if (d > (R)WALL_EPS) {
        V3<R> n = mk3<R>(0, 0, -1);
        R adj = stiff * d - damp * dot(n, vel);
        f = add(f, smul<R>(adj, n));
    }
    d = bd - ((pos.x - gmin.x) * scale);
    if (d > (R)WALL_EPS) f = add(f, repulsion<R>(vel, mk3<R>(1, 0, 0), d, damp, stiff));
    d = bd - ((gmax.x - pos.x) * scale);
    if (d > (R)WALL_EPS) f = add(f, repulsion<R>(vel, mk3<R>(-1, 0, 0), d, damp, stiff));
    return f;
}

/* calculateFrictionForce, K_Boundaries_Common.cu:48-82.  Only the velocity
 * terms reach the result (f_n / f_t are computed and discarded there). */
template <typename R>
static inline V3<R> friction(V3<R> vel, V3<R> n, R fkin, R fstatic)
{
    V3<R> v_n = mul<R>(vel, dot(n, vel));
    V3<R> v_t = sub(vel, v_n);
    if ((v_t.x + v_t.y + v_t.z) / (R)3.0f > fstatic)
        return mk3<R>(-v_t.x, -v_t.y, -v_t.z);
    return smul<R>(fkin, mk3<R>(-v_t.x, -v_t.y, -v_t.z));
}

/* calculateWallsNoSlipForce, K_Boundaries_Walls.cu:68-125 */
template <typename R>
static V3<R> walls_no_slip(V3<R> pos, V3<R> vel, V3<R> gmin, V3<R> gmax, R bd, R fkin, R fstatic, R scale)
{
    V3<R> f = mk3<R>(0, 0, 0);
    R d;
    d = bd - ((pos.y - gmin.y) * scale);
    if (d > (R)WALL_EPS) f = add(f, friction<R>(vel, mk3<R>(0, 1, 0), fkin, fstatic));
    d = bd - ((gmax.y - pos.y) * scale);
    if (d > (R)WALL_EPS) f = add(f, friction<R>(vel, mk3<R>(0, -1, 0), fkin, fstatic));
    d = bd - ((pos.z - gmin.z) * scale);
    if (d > (R)WALL_EPS) f = add(f, friction<R>(vel, mk3<R>(0, 0, 1), fkin, fstatic));
    d = bd - ((gmax.z - pos.z) * scale);
    if (d > (R)WALL_EPS) f = add(f, friction<R>(vel, mk3<R>(0, 0, -1), fkin, fstatic));
    d = bd - ((pos.x - gmin.x) * scale);
    if (d > (R)WALL_EPS) f = add(f, friction<R>(vel, mk3<R>(1, 0, 0), fkin, fstatic));
    d = bd - ((gmax.x - pos.x) * scale);
    if (d > (R)WALL_EPS) f = add(f, friction<R>(vel, mk3<R>(-1, 0, 0), fkin, fstatic));
    return f;
}

/* Literal wall constants of SPHCalculateForcesK, K_FluidSim.cu:289-293. */
static const float WALL_DIST = 0.003043174f;
static const float WALL_STIFF = 20000.0f;
static const float WALL_DAMP = 256.0f;

/* Walls + clamp block shared by both force kernels (K_FluidSim.cu:287-303
 * and :389-406).  `total` enters as internal*mass + gravity (+ contact). */
template <typename R>
static V3<R> walls_and_clamp(V3<R> total, f3 pos, f3 vel, const fgo_common_fluid_params *p)
{
    V3<R> P = cvt<R>(pos), V = cvt<R>(vel);
    V3<R> vmin = mk3<R>(p->volume_min.x, p->volume_min.y, p->volume_min.z);
    V3<R> vmax = mk3<R>(p->volume_max.x, p->volume_max.y, p->volume_max.z);
    R scale = p->simulation_scale;
    V3<R> wall = walls_no_penetration<R>(P, V, vmin, vmax, (R)WALL_DIST, (R)WALL_STIFF, (R)WALL_DAMP, scale);
    /* the friction call receives total + wallAvoid but only uses velocity */
    wall = add(wall, walls_no_slip<R>(P, V, mk3<R>(-11.0f, -40.0f, -11.0f), mk3<R>(11.0f, 200.0f, 11.0f),
                                      (R)WALL_DIST, (R)0, (R)0, scale));
    total = add(total, wall);
    R speed = len(total);
    if (speed > (R)p->velocity_limit) {
        R t = (R)p->velocity_limit / speed;
        total = mul<R>(total, t);
    }
    return total;
}

/* ------------------------------------------------- collision (contacts) */

/* ProcessCellForcesD + ProcessCollisionForcesD, K_DeviceFunctions.cu:32-159.
 * Inclusion (lg < minimum distance) is decided in FP32; the accumulated
 * force is carried in R. */
template <typename R>
static V3<R> collision_forces(f4 pos, f4 vel, float radius, const f4 *cpos, const f4 *cvel,
                              float cradius, float k, float kd, fgo_int3 rel, const u32 *start,
                              const u32 *end, f3 cell, u32 nb, bool w_rb_index, bool check_group,
                              int group, float eps)
{
    V3<R> out = mk3<R>(0, 0, 0);
    f3 P = mk3<float>(pos.x, pos.y, pos.z);
    float mind = radius + cradius + eps;
    for (int z = -rel.z; z <= rel.z; z++)
        for (int y = -rel.y; y <= rel.y; y++)
            for (int x = -rel.x; x <= rel.x; x++) {
                u32 b = hash_offset(P, cell, x, y, z, nb);
                V3<R> tf = mk3<R>(0, 0, 0);
                if (start[b] != 0xffffffffu) {
                    for (u32 i = start[b]; i < end[b]; i++) {
                        f4 q = cpos[i];
                        f4 v = {0.0f, 0.0f, 0.0f, 0.0f};
                        if (check_group && ((int)q.w) == group) continue;
                        if (cvel) v = w_rb_index ? cvel[(int)q.w] : cvel[i];
                        f3 rd = sub(mk3<float>(q.x, q.y, q.z), P);
                        float lg = len(rd);
                        if (lg < mind) {
                            V3<R> RD = cvt<R>(rd);
                            R LG = (R)lg;
                            if (sizeof(R) == 8) {
                                RD = mk3<R>((R)q.x - (R)P.x, (R)q.y - (R)P.y, (R)q.z - (R)P.z);
                                LG = len(RD);
                            }
                            V3<R> n = dvs<R>(RD, LG);
                            V3<R> rv = sub(xyz<R>(&v.x), xyz<R>(&vel.x));
                            tf = add(tf, repulsion<R>(rv, n, LG, (R)kd, (R)k));
                        }
                    }
                }
                out = add(out, tf);
            }
    return out;
}

/* ------------------------------------------------------------ quaternions */

/* Vec3CrossD / Vec3DotD / Quaternion_ProductD / Quaternion_TransformPointD /
 * Quaternion_NormalizeD / Quaternion_ToMatrixD / MatrixMultD /
 * AngularVelocityD, GPU_Kernels/K_MathUtils.cu:20-236 (restated for R). */
template <typename R> static inline V4<R> mk4(R x, R y, R z, R w) { V4<R> v; v.x = x; v.y = y; v.z = z; v.w = w; return v; }
template <typename R> static inline V4<R> cross4(V4<R> a, V4<R> b)
{
    return mk4<R>((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x), (R)0);
}
template <typename R> static inline V4<R> qprod(V4<R> a, V4<R> b)
{
    R w = a.w * b.w - (a.x * b.x + a.y * b.y + a.z * b.z);
    V4<R> c = cross4(a, b);
    return mk4<R>((a.w * b.x) + (b.w * a.x) + c.x, (a.w * b.y) + (b.w * a.y) + c.y,
                  (a.w * b.z) + (b.w * a.z) + c.z, w);
}
template <typename R> static inline V4<R> qtransform(V4<R> pos, V4<R> q)
{
    pos.w = 0;
    V4<R> cq = mk4<R>(-q.x, -q.y, -q.z, q.w);
    return qprod(qprod(cq, pos), q);
}
template <typename R> static inline V4<R> qnormalize(V4<R> q)
{
    R norm = std::sqrt(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
    q.x /= norm; q.y /= norm; q.z /= norm; q.w /= norm;
    return q;
}
template <typename R> static void qmatrix(V4<R> q, R m[3][3])
{
    m[0][0] = (R)1 - ((R)2 * q.y * q.y) - ((R)2 * q.z * q.z);
    m[0][1] = ((R)2 * q.x * q.y) + ((R)2 * q.w * q.z);
    m[0][2] = ((R)2 * q.x * q.z) - ((R)2 * q.w * q.y);
    m[1][0] = ((R)2 * q.x * q.y) - ((R)2 * q.w * q.z);
    m[1][1] = (R)1 - ((R)2 * q.x * q.x) - ((R)2 * q.z * q.z);
    m[1][2] = ((R)2 * q.y * q.z) + ((R)2 * q.w * q.x);
    m[2][0] = ((R)2 * q.x * q.z) + ((R)2 * q.w * q.y);
    m[2][1] = ((R)2 * q.y * q.z) - ((R)2 * q.w * q.x);
    m[2][2] = (R)1 - ((R)2 * q.x * q.x) - ((R)2 * q.y * q.y);
}
template <typename R> static void mmul(R a[3][3], R b[3][3], R r[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
}
template <typename R> static V4<R> angular_velocity(const R inv[3][3], V4<R> L, V4<R> q)
{
    R m[3][3], mt[3][3], t[3][3], g[3][3], ii[3][3];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) ii[i][j] = inv[i][j];
    qmatrix(q, m);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) mt[i][j] = m[j][i];
    mmul(m, ii, t);
    mmul(t, mt, g);
    return mk4<R>(g[0][0] * L.x + g[0][1] * L.y + g[0][2] * L.z,
                  g[1][0] * L.x + g[1][1] * L.y + g[1][2] * L.z,
                  g[2][0] * L.x + g[2][1] * L.y + g[2][2] * L.z, (R)0);
}

/* ====================================================================== */
#define FGO_API extern "C"

FGO_API int fgo_version(void) { return 3; }

FGO_API int fgo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

FGO_API void fgo_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---- restated helpers, exposed for the golden-vector tests ---- */

FGO_API u32 fgo_hash_key(const float *pos3, const float *cell3, int nb)
{
    return hash_key(pos3[0], pos3[1], pos3[2], cell3[0], cell3[1], cell3[2], (u32)nb);
}

FGO_API void fgo_walls_no_penetration(const float *pos3, const float *vel3, const float *min3, const float *max3,
                              float bd, float stiff, float damp, float scale, float *out3)
{
    f3 r = walls_no_penetration<float>(xyz<float>(pos3), xyz<float>(vel3), xyz<float>(min3), xyz<float>(max3),
                                       bd, stiff, damp, scale);
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

FGO_API void fgo_walls_no_slip(const float *pos3, const float *vel3, const float *force3, const float *min3,
                       const float *max3, float bd, float fkin, float fstatic, float scale, float *out3)
{
    (void)force3;
    f3 r = walls_no_slip<float>(xyz<float>(pos3), xyz<float>(vel3), xyz<float>(min3), xyz<float>(max3),
                                bd, fkin, fstatic, scale);
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

FGO_API void fgo_process_collision_forces(const float *pos4, const float *vel4, float radius, const float *cpos4,
                                  const float *cvel4, float cradius, float k, float kd, const int *rel3,
                                  const u32 *start, const u32 *end, const float *cell3, u32 nb, int w_rb,
                                  int check_group, int group, float eps, float *out3)
{
    fgo_int3 rel = {rel3[0], rel3[1], rel3[2]};
    f3 r = collision_forces<float>(*(const f4 *)pos4, *(const f4 *)vel4, radius, (const f4 *)cpos4,
                                   (const f4 *)cvel4, cradius, k, kd, rel, start, end, xyz<float>(cell3), nb,
                                   w_rb != 0, check_group != 0, group, eps);
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

FGO_API void fgo_quat_product(const float *a, const float *b, float *out4)
{
    f4 r = qprod(*(const f4 *)a, *(const f4 *)b);
    memcpy(out4, &r, 16);
}
FGO_API void fgo_quat_transform_point(const float *p, const float *q, float *out4)
{
    f4 r = qtransform(*(const f4 *)p, *(const f4 *)q);
    memcpy(out4, &r, 16);
}
FGO_API void fgo_quat_normalize(const float *q, float *out4)
{
    f4 r = qnormalize(*(const f4 *)q);
    memcpy(out4, &r, 16);
}
FGO_API void fgo_vec3_cross(const float *a, const float *b, float *out4)
{
    f4 r = cross4(*(const f4 *)a, *(const f4 *)b);
    memcpy(out4, &r, 16);
}
FGO_API void fgo_angular_velocity(const float *inv12, const float *L4, const float *q4, float *out4)
{
    float inv[3][3];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) inv[i][j] = inv12[i * 4 + j];
    f4 r = angular_velocity<float>(inv, *(const f4 *)L4, *(const f4 *)q4);
    memcpy(out4, &r, 16);
}

/* ---- KernelsCache, HeterogeneousSimulator.cpp:33-42 ----
 * kPoly6 = 315/(64*PI*h^9), kSpiky = -45/(PI*h^6), kVisc = 45/(PI*h^6),
 * PI = 3.14159265f (ApplicationData.cuh:18); pow() in double, stored as float. */
FGO_API void fgo_compute_kernels_cache(float h, fgo_kernels_cache *out)
{
    const float PI = 3.14159265f;
    out->kPoly6 = (float)(315.0f / ((double)(64.0f * PI) * std::pow((double)h, 9)));
    out->kSpikyGradient = (float)(-(45.0f / ((double)PI * std::pow((double)h, 6))));
    out->kViscosityLaplacian = (float)(45.0f / ((double)PI * std::pow((double)h, 6)));
}

/* ---- CalcHashKeyK, K_HashGrid.cu:26-38 ---- */
FGO_API void fgo_calc_hash_key(u32 *keys, u32 *ids, const float *pos4, int n, u32 nb, float cx, float cy, float cz)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        const float *p = pos4 + 4 * (size_t)i;
        ids[i] = (u32)i;
        keys[i] = hash_key(p[0], p[1], p[2], cx, cy, cz, nb);
    }
}

/* ---- CalcHashKeyWithOffsetK, K_HashGrid.cu:43-63 ---- */
FGO_API void fgo_calc_hash_key_with_offset(u32 *keys, u32 *ids, const float *offset4, const float *orient4,
                                   const float *local4, float *out4, int n, float cx, float cy, float cz, int nb)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        f4 pos = ((const f4 *)local4)[i];
        int oi = (int)pos.w;
        f4 q = ((const f4 *)orient4)[oi];
        f4 o = ((const f4 *)offset4)[oi];
        f4 t = qtransform(pos, q);
        f4 a = mk4<float>(t.x + o.x, t.y + o.y, t.z + o.z, t.w + o.w);
        a.w = pos.w;
        ids[i] = (u32)i;
        ((f4 *)out4)[i] = a;
        keys[i] = hash_key(a.x, a.y, a.z, cx, cy, cz, (u32)nb);
    }
}

/* ---- gSort, K_FluidSim.cu:685-691 (thrust::sort_by_key on u32 keys, a
 * stable radix sort) and the CUDPP key/value radix sort of the rigid-body
 * grids (RigidBodySimulator.cpp:195-196, 469-470): ascending key, ties in
 * input order.  Restated as a stable counting sort over the key range. */
FGO_API void fgo_sort_pairs(u32 *keys, u32 *vals, int n)
{
    if (n <= 1) return;
    u32 kmax = 0;
    for (int i = 0; i < n; i++) kmax = std::max(kmax, keys[i]);
    if ((size_t)kmax + 1 > (size_t)16 * (size_t)n + (1u << 22)) {
        std::vector<uint64_t> kv((size_t)n);
        for (int i = 0; i < n; i++) kv[i] = ((uint64_t)keys[i] << 32) | (uint64_t)i;
        std::sort(kv.begin(), kv.end());
        std::vector<u32> v2(vals, vals + n);
        for (int i = 0; i < n; i++) {
            keys[i] = (u32)(kv[i] >> 32);
            vals[i] = v2[(u32)kv[i]];
        }
        return;
    }
    std::vector<u32> cnt((size_t)kmax + 2, 0);
    for (int i = 0; i < n; i++) cnt[keys[i] + 1]++;
    for (size_t b = 1; b < cnt.size(); b++) cnt[b] += cnt[b - 1];
    std::vector<u32> k2((size_t)n), v2((size_t)n);
    for (int i = 0; i < n; i++) {
        u32 d = cnt[keys[i]]++;
        k2[d] = keys[i];
        v2[d] = vals[i];
    }
    memcpy(keys, k2.data(), sizeof(u32) * (size_t)n);
    memcpy(vals, v2.data(), sizeof(u32) * (size_t)n);
}

/* ---- gFindCellOffsetOrderingPosVel / gFindCellOffsetOrderingPos,
 * K_HashGrid.cu:238-318 (memset of start to 0xffffffff) and the kernels
 * FindCellOffsetOrderinPosVelK :70-133 / FindCellOffsetOrderingPosK
 * :140-197.  `end` entries of empty buckets are left untouched, as there.
 * vel4/svel4 may be NULL (positions only). */
FGO_API void fgo_find_cell_offset(u32 *start, u32 *end, const u32 *keys, const u32 *ids, const float *pos4,
                          float *spos4, const float *vel4, float *svel4, int n, u32 nb)
{
    memset(start, 0xff, sizeof(u32) * (size_t)nb);
    for (int i = 0; i < n; i++) {
        u32 h = keys[i];
        if (i == 0 || h != keys[i - 1]) {
            start[h] = (u32)i;
            if (i > 0) end[keys[i - 1]] = (u32)i;
        }
        if (i == n - 1) end[h] = (u32)i + 1;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        u32 s = ids[i];
        memcpy(spos4 + 4 * (size_t)i, pos4 + 4 * (size_t)s, 16);
        if (vel4 && svel4) memcpy(svel4 + 4 * (size_t)i, vel4 + 4 * (size_t)s, 16);
    }
}

/* ---- CalculateMassDensityK + ProcessMassDensityGridD,
 * K_FluidSim.cu:210-254 and :46-79.  Per bucket a partial sum starting at 0,
 * partials added in z-y-x order.  dp of inactive particles is not written.
 * If pairs_out != NULL, the number of in-range (l < h) pair visits is added to
 * pairs_out[0]. */
template <typename R>
static void density_impl(const float *spos4, R *dp2, const u32 *start, const u32 *end, int n,
                         const fgo_common_fluid_params *p, const fgo_kernels_cache *kc, float gas, float rest,
                         float mass, long long *pairs_out)
{
    const f3 cell = cell_of(p);
    const u32 nb = nbuckets_of(p);
    const float scale = p->simulation_scale, h = p->kernel_radius, h2 = p->kernel_radius_squared;
    long long pairs = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : pairs)
    for (int i = 0; i < n; i++) {
        const f4 pos = ((const f4 *)spos4)[i];
        if (!(pos.w > 0.0f)) continue;
        const f3 P = mk3<float>(pos.x, pos.y, pos.z);
        R md = 0;
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    u32 b = hash_offset(P, cell, x, y, z, nb);
                    R part = 0;
                    u32 st = start[b];
                    if (st != 0xffffffffu) {
                        f3 p1 = mul<float>(P, scale);
                        u32 en = end[b];
                        for (u32 j = st; j < en; j++) {
                            const f4 q = ((const f4 *)spos4)[j];
                            f3 p2 = mul<float>(mk3<float>(q.x, q.y, q.z), scale);
                            f3 diff = sub(p1, p2);
                            float l = len(diff);
                            if (l < h) {
                                pairs++;
                                if (sizeof(R) == 4) {
                                    /* powf as the source calls it (the host C library's) */
                                    part += (R)((mass * kc->kPoly6) * powf(h2 - (l * l), 3.0f));
                                } else {
                                    V3<R> d = mk3<R>((R)P.x * scale - (R)q.x * scale, (R)P.y * scale - (R)q.y * scale,
                                                     (R)P.z * scale - (R)q.z * scale);
                                    R t = (R)h2 - dot(d, d);
                                    part += ((R)mass * (R)kc->kPoly6) * (t * t * t);
                                }
                            }
                        }
                    }
                    md += part;
                }
        R dpx = (R)std::fmax(1.0, (double)md);
        dp2[2 * (size_t)i] = dpx;
        dp2[2 * (size_t)i + 1] = (R)gas * (md - (R)rest);
    }
    if (pairs_out) pairs_out[0] += pairs;
}

FGO_API void fgo_density_f32(const float *spos4, float *dp2, const u32 *start, const u32 *end, int n,
                     const fgo_common_fluid_params *p, const fgo_kernels_cache *kc, float gas, float rest,
                     float mass, long long *pairs_out)
{
    density_impl<float>(spos4, dp2, start, end, n, p, kc, gas, rest, mass, pairs_out);
}

FGO_API void fgo_density_f64(const float *spos4, double *dp2, const u32 *start, const u32 *end, int n,
                     const fgo_common_fluid_params *p, const fgo_kernels_cache *kc, float gas, float rest,
                     float mass, long long *pairs_out)
{
    density_impl<double>(spos4, dp2, start, end, n, p, kc, gas, rest, mass, pairs_out);
}

/* Rigid-body contact inputs of SPHCalculateForcesWithSRBK
 * (K_FluidSim.cu:315-348).  Grid pointers may be NULL when the flag is 0. */
struct fgo_contact_grid {
    const float *pos4;   /* sorted sphere positions, w = body index (dynamic) */
    const float *vel4;   /* per-body velocities (dynamic) or NULL (static) */
    const u32 *start;
    const u32 *end;
    u32 nbuckets;
    int use;
};
struct fgo_contact_params {
    float fluid_radius;  /* fluidParticleRadius */
    float rb_radius;     /* _in_srb_particle_radius */
    float kspring, kdamping;
    float cell[3];       /* _in_srb_cell_size */
    int rel[3];          /* _in_srb_cell_size_relation */
    float eps;           /* 0.003 in the reference call */
};

/* ---- SPHCalculateForcesK / SPHCalculateForcesWithSRBK with
 * CalculateFluidInternalForcesD, SPHCalculateInternalForcesD,
 * SPHCalculatePressureForceD, SPHCalculateViscosityForceD:
 * K_FluidSim.cu:85-205, 260-309, 315-413.  Writes newvel[ids[i]].  R = float
 * reproduces the FP32 arithmetic; R = double carries the pair terms and sums in
 * double (neighbour inclusion still decided in FP32). */
template <typename R>
static void forces_impl(const float *spos4, const float *svel4, const float *dp2f, const double *dp2d,
                        const u32 *start, const u32 *end, R *newvel4, const u32 *ids, float mass, int n,
                        float visc, const fgo_common_fluid_params *p, const fgo_kernels_cache *kc,
                        const fgo_contact_params *cp, const fgo_contact_grid *sgrid,
                        const fgo_contact_grid *dgrid)
{
    const f3 cell = cell_of(p);
    const u32 nb = nbuckets_of(p);
    const float scale = p->simulation_scale, h = p->kernel_radius;
    const R dt = (R)p->deltaTimeIntegration;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; i++) {
        const f4 pos = ((const f4 *)spos4)[i];
        const f4 vel = ((const f4 *)svel4)[i];
        V3<R> total = mk3<R>(0, 0, 0);
        if (pos.w > 0.0f) {
            const f3 P = mk3<float>(pos.x, pos.y, pos.z);
            V3<R> internal = mk3<R>(0, 0, 0);
            for (int z = -1; z <= 1; z++)
                for (int y = -1; y <= 1; y++)
                    for (int x = -1; x <= 1; x++) {
                        u32 b = hash_offset(P, cell, x, y, z, nb);
                        V3<R> tf = mk3<R>(0, 0, 0);
                        u32 st = start[b];
                        if (st != 0xffffffffu) {
                            f3 p1 = mul<float>(P, scale);
                            R d1x = dp2d ? (R)dp2d[2 * (size_t)i] : (R)dp2f[2 * (size_t)i];
                            R d1y = dp2d ? (R)dp2d[2 * (size_t)i + 1] : (R)dp2f[2 * (size_t)i + 1];
                            const f4 v1 = vel;
                            u32 en = end[b];
                            for (u32 j = st; j < en; j++) {
                                if (j == (u32)i) continue;
                                const f4 q = ((const f4 *)spos4)[j];
                                const f4 v2 = ((const f4 *)svel4)[j];
                                R d2x = dp2d ? (R)dp2d[2 * (size_t)j] : (R)dp2f[2 * (size_t)j];
                                R d2y = dp2d ? (R)dp2d[2 * (size_t)j + 1] : (R)dp2f[2 * (size_t)j + 1];
                                f3 p2 = mul<float>(mk3<float>(q.x, q.y, q.z), scale);
                                f3 diff = sub(p1, p2);
                                float l = len(diff);
                                if (l > h) continue; /* both terms return 0 */
                                if (sizeof(R) == 4) {
                                    /* pressure :107-120 */
                                    float pp = ((float)d1y + (float)d2y) / ((float)d1x * (float)d2x);
                                    float r = kc->kSpikyGradient * ((h - l) * (h - l));
                                    f3 pf = mul<float>(mul<float>(mul<float>(dvs<float>(diff, l), r), pp), -1.0f);
                                    tf = add(tf, cvt<R>(pf));
                                    /* viscosity :85-102 */
                                    float lap = kc->kViscosityLaplacian * (h - l);
                                    float den = (float)d1x * (float)d2x;
                                    f3 vf = mk3<float>(((v2.x - v1.x) / den) * lap * visc,
                                                       ((v2.y - v1.y) / den) * lap * visc,
                                                       ((v2.z - v1.z) / den) * lap * visc);
                                    tf = add(tf, cvt<R>(vf));
                                } else {
                                    V3<R> D = mk3<R>((R)P.x * scale - (R)q.x * scale, (R)P.y * scale - (R)q.y * scale,
                                                     (R)P.z * scale - (R)q.z * scale);
                                    R L = std::sqrt(dot(D, D));
                                    R H = (R)h;
                                    R pp = (d1y + d2y) / (d1x * d2x);
                                    R r = (R)kc->kSpikyGradient * ((H - L) * (H - L));
                                    tf = add(tf, mul<R>(dvs<R>(D, L), -(r * pp)));
                                    R lap = (R)kc->kViscosityLaplacian * (H - L);
                                    R den = d1x * d2x;
                                    tf = add(tf, mk3<R>(((R)v2.x - (R)v1.x) / den * lap * (R)visc,
                                                        ((R)v2.y - (R)v1.y) / den * lap * (R)visc,
                                                        ((R)v2.z - (R)v1.z) / den * lap * (R)visc));
                                }
                            }
                        }
                        internal = add(internal, tf);
                    }
            V3<R> external = mk3<R>(0, 0, 0);
            if (cp) {
                f3 ccell = mk3<float>(cp->cell[0], cp->cell[1], cp->cell[2]);
                fgo_int3 rel = {cp->rel[0], cp->rel[1], cp->rel[2]};
                if (sgrid && sgrid->use)
                    external = add(external, collision_forces<R>(pos, vel, cp->fluid_radius, (const f4 *)sgrid->pos4,
                                                                 nullptr, cp->rb_radius, cp->kspring, cp->kdamping, rel,
                                                                 sgrid->start, sgrid->end, ccell, sgrid->nbuckets,
                                                                 false, false, 0, cp->eps));
                if (dgrid && dgrid->use)
                    external = add(external, collision_forces<R>(pos, vel, cp->fluid_radius, (const f4 *)dgrid->pos4,
                                                                 (const f4 *)dgrid->vel4, cp->rb_radius, cp->kspring,
                                                                 cp->kdamping, rel, dgrid->start, dgrid->end, ccell,
                                                                 dgrid->nbuckets, true, false, 0, cp->eps));
            }
            V3<R> g = mk3<R>(p->global_external_force.x, p->global_external_force.y, p->global_external_force.z);
            total = add(add(mul<R>(internal, (R)mass), g), external);
            total = walls_and_clamp<R>(total, P, mk3<float>(vel.x, vel.y, vel.z), p);
        }
        u32 oi = ids[i];
        R *o = newvel4 + 4 * (size_t)oi;
        o[0] = (R)vel.x + total.x * dt;
        o[1] = (R)vel.y + total.y * dt;
        o[2] = (R)vel.z + total.z * dt;
        o[3] = (R)vel.w + (R)0.0f;
    }
}

FGO_API void fgo_forces_f32(const float *spos4, const float *svel4, const float *dp2, const u32 *start, const u32 *end,
                    float *newvel4, const u32 *ids, float mass, int n, float visc, const fgo_common_fluid_params *p,
                    const fgo_kernels_cache *kc)
{
    forces_impl<float>(spos4, svel4, dp2, nullptr, start, end, newvel4, ids, mass, n, visc, p, kc, nullptr,
                       nullptr, nullptr);
}

FGO_API void fgo_forces_f64(const float *spos4, const float *svel4, const double *dp2, const u32 *start, const u32 *end,
                    double *newvel4, const u32 *ids, float mass, int n, float visc, const fgo_common_fluid_params *p,
                    const fgo_kernels_cache *kc)
{
    forces_impl<double>(spos4, svel4, nullptr, dp2, start, end, newvel4, ids, mass, n, visc, p, kc, nullptr,
                        nullptr, nullptr);
}

/* FP64 forces from the FP32 density field (stage parity from identical state) */
FGO_API void fgo_forces_f64_fdp(const float *spos4, const float *svel4, const float *dp2, const u32 *start, const u32 *end,
                        double *newvel4, const u32 *ids, float mass, int n, float visc,
                        const fgo_common_fluid_params *p, const fgo_kernels_cache *kc,
                        const fgo_contact_params *cp, const fgo_contact_grid *sgrid, const fgo_contact_grid *dgrid)
{
    forces_impl<double>(spos4, svel4, dp2, nullptr, start, end, newvel4, ids, mass, n, visc, p, kc, cp, sgrid,
                        dgrid);
}

FGO_API void fgo_forces_srb_f32(const float *spos4, const float *svel4, const float *dp2, const u32 *start,
                        const u32 *end, float *newvel4, const u32 *ids, float mass, int n, float visc,
                        const fgo_common_fluid_params *p, const fgo_kernels_cache *kc, const fgo_contact_params *cp,
                        const fgo_contact_grid *sgrid, const fgo_contact_grid *dgrid)
{
    forces_impl<float>(spos4, svel4, dp2, nullptr, start, end, newvel4, ids, mass, n, visc, p, kc, cp, sgrid,
                       dgrid);
}

/* ---- SPHIntegrateK, K_FluidSim.cu:418-438 (pos += vel*(dt/scale), all four
 * components, active particles only) ---- */
FGO_API void fgo_integrate_f32(float *pos4, const float *vel4, int n, const fgo_common_fluid_params *p)
{
    const float c = p->deltaTimeIntegration / p->simulation_scale;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        float *q = pos4 + 4 * (size_t)i;
        const float *v = vel4 + 4 * (size_t)i;
        if (q[3] > 0.0f) {
            q[0] = q[0] + v[0] * c;
            q[1] = q[1] + v[1] * c;
            q[2] = q[2] + v[2] * c;
            q[3] = q[3] + v[3] * c;
        }
    }
}

/* ---- CalculateRBForcesFromFluidsK, K_RigidBodySim.cu:66-99 ----
 * force4/torque4 get w = (float)(int)pos.w (the body index).  R = double
 * writes double outputs. */
template <typename R>
static void rb_from_fluid_impl(const float *rbpos4, const float *rbvel4, const float *rbcm4, R *force4, R *torque4,
                               int n, float radius, const float *sph_pos4, const float *sph_vel4, const u32 *sph_start,
                               const u32 *sph_end, float sph_radius, const float *sph_cell3, u32 sph_nb,
                               const int *rel3, float k, float kd)
{
    fgo_int3 rel = {rel3[0], rel3[1], rel3[2]};
    f3 cell = xyz<float>(sph_cell3);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        f4 pos = ((const f4 *)rbpos4)[i];
        int b = (int)pos.w;
        f4 vel = ((const f4 *)rbvel4)[b];
        f4 cm = ((const f4 *)rbcm4)[b];
        V3<R> tot = collision_forces<R>(pos, vel, radius, (const f4 *)sph_pos4, (const f4 *)sph_vel4, sph_radius, k,
                                        kd, rel, sph_start, sph_end, cell, sph_nb, false, false, 0, 0.0001f);
        R *F = force4 + 4 * (size_t)i;
        F[0] = tot.x; F[1] = tot.y; F[2] = tot.z; F[3] = (R)(float)b;
        V4<R> dir = mk4<R>((R)pos.x - (R)cm.x, (R)pos.y - (R)cm.y, (R)pos.z - (R)cm.z, (R)pos.w - (R)cm.w);
        if (sizeof(R) == 4) dir = mk4<R>((R)(pos.x - cm.x), (R)(pos.y - cm.y), (R)(pos.z - cm.z), (R)(pos.w - cm.w));
        V4<R> t = cross4(dir, mk4<R>(tot.x, tot.y, tot.z, (R)0));
        R *T = torque4 + 4 * (size_t)i;
        T[0] = t.x; T[1] = t.y; T[2] = t.z; T[3] = (R)(float)b;
    }
}

FGO_API void fgo_rb_forces_from_fluids_f32(const float *rbpos4, const float *rbvel4, const float *rbcm4, float *force4,
                                   float *torque4, int n, float radius, const float *sph_pos4, const float *sph_vel4,
                                   const u32 *sph_start, const u32 *sph_end, float sph_radius, const float *sph_cell3,
                                   u32 sph_nb, const int *rel3, float k, float kd)
{
    rb_from_fluid_impl<float>(rbpos4, rbvel4, rbcm4, force4, torque4, n, radius, sph_pos4, sph_vel4, sph_start,
                              sph_end, sph_radius, sph_cell3, sph_nb, rel3, k, kd);
}

FGO_API void fgo_rb_forces_from_fluids_f64(const float *rbpos4, const float *rbvel4, const float *rbcm4, double *force4,
                                   double *torque4, int n, float radius, const float *sph_pos4, const float *sph_vel4,
                                   const u32 *sph_start, const u32 *sph_end, float sph_radius, const float *sph_cell3,
                                   u32 sph_nb, const int *rel3, float k, float kd)
{
    rb_from_fluid_impl<double>(rbpos4, rbvel4, rbcm4, force4, torque4, n, radius, sph_pos4, sph_vel4, sph_start,
                               sph_end, sph_radius, sph_cell3, sph_nb, rel3, k, kd);
}

/* ---- CalculateRigidBodyForcesFromRBK, K_RigidBodySim.cu:18-61 ---- */
FGO_API void fgo_rb_forces_from_rb_f32(const float *rbpos4, const float *rbvel4, const float *rbcm4, float *torque4,
                               float *force4, const u32 *rb_start, const u32 *rb_end, int n, const float *cell3,
                               float radius, int rb_nb, int srb_nb, const float *srbpos4, const u32 *srb_start,
                               const u32 *srb_end, float k, float kd, int nsrb)
{
    fgo_int3 one = {1, 1, 1};
    f3 cell = xyz<float>(cell3);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        f4 pos = ((const f4 *)rbpos4)[i];
        int b = (int)pos.w;
        f4 vel = ((const f4 *)rbvel4)[b];
        f4 cm = ((const f4 *)rbcm4)[b];
        f3 tot = collision_forces<float>(pos, vel, radius, (const f4 *)rbpos4, (const f4 *)rbvel4, radius, k, kd, one,
                                         rb_start, rb_end, cell, (u32)rb_nb, true, true, b, 0.001f);
        if (nsrb > 0)
            tot = add(tot, collision_forces<float>(pos, vel, radius, (const f4 *)srbpos4, nullptr, radius, k, kd, one,
                                                   srb_start, srb_end, cell, (u32)srb_nb, false, false, 0, 0.001f));
        float *F = force4 + 4 * (size_t)i;
        F[0] = tot.x; F[1] = tot.y; F[2] = tot.z; F[3] = (float)b;
        f4 dir = mk4<float>(pos.x - cm.x, pos.y - cm.y, pos.z - cm.z, pos.w - cm.w);
        f4 t = cross4(dir, mk4<float>(tot.x, tot.y, tot.z, 0.0f));
        float *T = torque4 + 4 * (size_t)i;
        T[0] = t.x; T[1] = t.y; T[2] = t.z; T[3] = (float)b;
    }
}

/* ---- applyForces, RigidBodySimulator.cpp:522-566: per-body sum of the
 * sphere forces and torques (CopyRBDataToParticleK / ReorderForceTorqueK /
 * segmented scan / AddForceTorqueK, K_RigidBodySim.cu:102-155), grouped by
 * the body index in force.w; added into body_force4/body_torque4.  Summed in
 * double in sphere order. */
FGO_API void fgo_rb_reduce_f64(const float *force4, const float *torque4, int n, int nbodies, double *body_force4,
                       double *body_torque4)
{
    for (int i = 0; i < n; i++) {
        int b = (int)force4[4 * (size_t)i + 3];
        if (b < 0 || b >= nbodies) continue;
        for (int c = 0; c < 4; c++) {
            body_force4[4 * b + c] += (double)force4[4 * (size_t)i + c];
            body_torque4[4 * b + c] += (double)torque4[4 * (size_t)i + c];
        }
    }
}

/* ---- IntegrateRBK, K_RigidBodySim.cu:160-262 (with AngularVelocityD,
 * Quaternion_ProductD, Quaternion_NormalizeD from K_MathUtils.cu).  State
 * arrays of type R (float4 or double4 rows); inertia rows 3 per body.  The
 * force/torque inputs are the per-body sums. */
template <typename R>
static void integrate_rb_impl(R *x4, const float *mass, R *v4, const R *f4in, int nrb, float dt, const float *ext4,
                              const float *min3, const float *max3, R *L4, const R *t4, R *q4, const R *inv12,
                              float vlimit)
{
    for (int b = 0; b < nrb; b++) {
        V4<R> F = mk4<R>(f4in[4 * b], f4in[4 * b + 1], f4in[4 * b + 2], f4in[4 * b + 3]);
        R spd = std::sqrt(F.x * F.x + F.y * F.y + F.z * F.z + F.w * F.w);
        if (spd > (R)vlimit) {
            R t = (R)vlimit / spd;
            F = mk4<R>(F.x * t, F.y * t, F.z * t, F.w * t);
        }
        V4<R> pos = mk4<R>(x4[4 * b], x4[4 * b + 1], x4[4 * b + 2], x4[4 * b + 3]);
        R m = (R)mass[b];
        R DT = (R)dt;
        V4<R> E = mk4<R>((R)ext4[0], (R)ext4[1], (R)ext4[2], (R)ext4[3]);
        V4<R> acc = mk4<R>(((F.x + E.x) / m) * DT, ((F.y + E.y) / m) * DT, ((F.z + E.z) / m) * DT,
                           ((F.w + E.w) / m) * DT);
        V4<R> vel = mk4<R>(v4[4 * b] + acc.x * DT, v4[4 * b + 1] + acc.y * DT, v4[4 * b + 2] + acc.z * DT,
                           v4[4 * b + 3] + acc.w * DT);
        pos.x += vel.x * DT;
        pos.y += vel.y * DT;
        pos.z += vel.z * DT;
        for (int c = 0; c < 4; c++) L4[4 * b + c] += t4[4 * b + c] * DT;
        const R damp = (R)0.9f;
        for (int c = 0; c < 4; c++) L4[4 * b + c] *= damp;
        R inv[3][3];
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) inv[i][j] = inv12[12 * b + 4 * i + j];
        V4<R> q = mk4<R>(q4[4 * b], q4[4 * b + 1], q4[4 * b + 2], q4[4 * b + 3]);
        V4<R> w = angular_velocity<R>(inv, mk4<R>(L4[4 * b], L4[4 * b + 1], L4[4 * b + 2], L4[4 * b + 3]), q);
        w.w = 0;
        w = qprod(w, q);
        const R half = (R)0.5f;
        w = mk4<R>(w.x * half, w.y * half, w.z * half, w.w * half);
        const R tenth = (R)0.1f;
        V4<R> ws = mk4<R>(w.x * DT * tenth, w.y * DT * tenth, w.z * DT * tenth, w.w * DT * tenth);
        V4<R> dq = qprod(ws, q);
        q = mk4<R>(q.x + dq.x, q.y + dq.y, q.z + dq.z, q.w + dq.w);
        q = qnormalize(q);
        q4[4 * b] = q.x; q4[4 * b + 1] = q.y; q4[4 * b + 2] = q.z; q4[4 * b + 3] = q.w;
        const R rest = (R)-0.7f;
        if (pos.y < (R)min3[1]) { pos.y = (R)min3[1]; vel.y *= rest; }
        if (pos.x <= (R)min3[0]) { pos.x = (R)min3[0]; vel.x *= rest; }
        else if (pos.x >= (R)max3[0]) { pos.x = (R)max3[0]; vel.x *= rest; }
        if (pos.z <= (R)min3[2]) { pos.z = (R)min3[2]; vel.z *= rest; }
        else if (pos.z >= (R)max3[2]) { pos.z = (R)max3[2]; vel.z *= rest; }
        x4[4 * b] = pos.x; x4[4 * b + 1] = pos.y; x4[4 * b + 2] = pos.z; x4[4 * b + 3] = pos.w;
        v4[4 * b] = vel.x; v4[4 * b + 1] = vel.y; v4[4 * b + 2] = vel.z; v4[4 * b + 3] = vel.w;
    }
}

FGO_API void fgo_integrate_rb_f32(float *x4, const float *mass, float *v4, const float *f4in, int nrb, float dt,
                          const float *ext4, const float *min3, const float *max3, float *L4, const float *t4,
                          float *q4, const float *inv12, float vlimit)
{
    integrate_rb_impl<float>(x4, mass, v4, f4in, nrb, dt, ext4, min3, max3, L4, t4, q4, inv12, vlimit);
}

FGO_API void fgo_integrate_rb_f64(double *x4, const float *mass, double *v4, const double *f4in, int nrb, float dt,
                          const float *ext4, const float *min3, const float *max3, double *L4, const double *t4,
                          double *q4, const double *inv12, float vlimit)
{
    integrate_rb_impl<double>(x4, mass, v4, f4in, nrb, dt, ext4, min3, max3, L4, t4, q4, inv12, vlimit);
}

/* ---- RigidBodySimulator::generateCollisionData, RigidBodySimulator.cpp:334-477
 * (CPU side): the OpenMP broad phase over dynamic bodies (its bounding-box
 * test is disabled in the reference, so every body with a partner is
 * collided) and the host gather of the collided bodies' local sphere offsets
 * (w = body index) and segment-head flags.  Returns the number of gathered
 * spheres; out_flags may be NULL.  `partner` says whether each body has a
 * partner (another dynamic body, a static body, or the fluid). */
FGO_API int fgo_rb_collision_gather(const float *local4, const u32 *body_first, const u32 *body_count, const int *partner,
                            int nbodies, float *out4, u32 *out_flags, int *out_last)
{
    std::vector<int> collided((size_t)nbodies, 0);
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nbodies; b++) collided[b] = partner[b] ? 1 : 0;
    int off = 0, nc = 0;
    for (int b = 0; b < nbodies; b++) {
        if (!collided[b]) continue;
        memcpy(out4 + 4 * (size_t)off, local4 + 4 * (size_t)body_first[b], 16 * (size_t)body_count[b]);
        if (out_flags)
            for (u32 j = 0; j < body_count[b]; j++) out_flags[off + j] = (j == 0) ? 1u : 0u;
        off += (int)body_count[b];
        if (out_last) out_last[nc] = off - 1;
        nc++;
    }
    return off;
}

