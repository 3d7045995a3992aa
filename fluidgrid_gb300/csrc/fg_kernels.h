/* Host-side launch wrappers of the GB300 SPH kernels (internal). */
#ifndef FG_KERNELS_H
#define FG_KERNELS_H

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include "fg_types.h"

namespace fg {

/* Launch geometry: work items of FG_CHUNK particles; grids are sized in
 * multiples of the SM count (persistent grid-stride loops). */
struct Launch {
    const FgScene *table;  /* device scene table, or nullptr for one scene */
    const FgScene *single; /* host copy used when table == nullptr (passed by value) */
    const FgWork *work;    /* device work table, or nullptr (single scene) */
    uint32_t nwork;        /* work items */
    uint32_t n;            /* particles (single-scene mode) */
    cudaStream_t stream;
    uint32_t ctas_per_sm;  /* density/force grids: CTAs of FG_CHUNK threads per SM (0 = 64) */
    uint32_t block;        /* density/force grids: threads per CTA, 64, 128 or 256 (0 = FG_CHUNK) */
};

int sm_count();
uint32_t grid_for(uint32_t nwork, int ctas_per_sm);

/* ---- grid build (fg_grid.cu) ---- */
/* cnt/off (optional): the counting sort's first pass fused in (cnt zeroed
 * over the world's buckets by the caller; off = its s.keys_alt) */
void launch_hash(const Launch &L, const float4 *pos, uint32_t *keys, uint32_t *ids, uint32_t *cnt = nullptr,
                 uint32_t *off = nullptr);
void launch_hash_with_offset(const Launch &L, const float4 *local, const float4 *cm, const float4 *q,
                             float4 *world, uint32_t *keys, uint32_t *ids, int *aabb /* 6 ints per scene or null */);

/* keys per radix tile (one CTA of the upsweep/downsweep); the histogram
 * holds 256 counts per tile plus 256 digit totals */
#define FG_RS_TILE 2048u
struct RadixScratch {
    uint32_t *keys_alt;
    uint32_t *vals_alt;
    uint32_t *hist; /* >= radix_hist_words(n) words */
};
size_t radix_hist_words(uint32_t n);
int radix_passes(uint32_t bits, uint32_t digit_bits);
/* One-kernel-per-pass variant (decoupled look-back) for the world's fluid
 * sort: same result as radix_sort with vals_in = 0..n-1.  os is
 * onesweep_words(n) words of scratch; err receives FG_DEV_SORT_TIMEOUT if a
 * bounded wait gives up.  Returns false (and does nothing) when the pass
 * count exceeds what the scratch holds; the caller then uses radix_sort. */
size_t onesweep_words(uint32_t n);
int bounded_wait_selftest(uint32_t spin_limit, uint32_t *flags);
bool onesweep_sort(const uint32_t *keys_in, uint32_t *keys_out, uint32_t *vals_out, uint32_t n, uint32_t bits,
                   uint32_t digit_bits, const RadixScratch &s, uint32_t *os, uint32_t *err, cudaStream_t st);
/* Stable ascending sort of (key, value) by the low `bits` bits of the key.
 * vals_in == nullptr means values 0..n-1.  keys_out/vals_out may alias
 * keys_in/vals_in (in-place).  Returns the status of the device-to-device
 * copies an odd pass count in place ends with (kernel launch errors are
 * left for cudaGetLastError). */
cudaError_t radix_sort(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out,
                uint32_t n, uint32_t bits, uint32_t digit_bits, const RadixScratch &s, cudaStream_t st);

/* Counting sort by bucket (keys below nbuckets): the same result as
 * radix_sort with vals_in = 0..n-1, and it writes start[] (0xffffffff for
 * empty buckets) and end[] of every occupied bucket of [0, nbuckets) on the
 * way.  Uses s.keys_alt and s.vals_alt (n words each) and s.hist
 * (scratch_words words; returns false, doing nothing, when the
 * ceil(nbuckets / 2048) tile sums exceed them). */
struct BucketReorder {
    const float4 *pos, *vel; /* unsorted (vel may be null) */
    float4 *spos, *svel;
    uint32_t *inv, *runs, *nruns; /* optional; nruns zeroed by the caller */
};
/* With reorder, the stable rank also does launch_cell_ranges' gathers
 * (sorted position and velocity, inv, run heads): no ranges pass needed.
 * counted: launch_hash already counted the keys into end[] and left the
 * arrival offsets in s.keys_alt. */
bool bucket_sort(const uint32_t *keys_in, uint32_t *keys_out, uint32_t *vals_out, uint32_t n, uint32_t nbuckets,
                 uint32_t *start, uint32_t *end, const RadixScratch &s, uint32_t scratch_words, cudaStream_t st,
                 const BucketReorder *reorder = nullptr, bool counted = false);

/* start[] must be pre-filled with 0xffffffff over the bucket range.
 * inv (optional) receives particle -> sorted index; runs (optional) receives
 * the first sorted index of every occupied bucket, in no particular order,
 * counted in *nruns (zeroed by the caller). */
void launch_cell_ranges(const uint32_t *keys, const uint32_t *ids, const float4 *pos, const float4 *vel,
                        uint32_t *start, uint32_t *end, float4 *spos, float4 *svel, uint32_t n, cudaStream_t st,
                        uint32_t *inv = nullptr, uint32_t *runs = nullptr, uint32_t *nruns = nullptr);

/* Rigid-sphere grid of every scene (sort by key, ids, sorted positions,
 * start/end) in one CTA per scene; valid when no scene has more than
 * FG_RB_SCENE_MAX spheres.  keys_u are global rigid bucket ids. */
#define FG_RB_SCENE_MAX 4096u
void launch_rb_sort_ranges(const FgScene *table, const FgScene *single, uint32_t nscenes, const uint32_t *keys_u,
                           const float4 *world, uint32_t *keys, uint32_t *ids, float4 *spos, uint32_t *rstart,
                           uint32_t *rend, cudaStream_t s);

/* Spatial (Morton) keys of the unsorted particles: scene id << scene_shift |
 * Morton code of the cell with `bits` bits per axis (bits <= 10). */
void launch_morton_keys(const Launch &L, const float4 *pos, uint32_t *keys, uint32_t bits, uint32_t scene_shift);


/* Target order of the density/force passes: target slot t processes the
 * particle tord[t] (a particle id, scene-contiguous), found in sorted order
 * at inv[tord[t]].  tord == nullptr: slot t is sorted index t. */
struct TargetOrder {
    const uint32_t *tord;
    const uint32_t *inv;
};

/* ---- SPH (fg_sph.cu) ---- */

/* In-range neighbour lists recorded by the density pass and consumed by the
 * force pass: every in-range visit (l <= h, the target's own entries and
 * duplicate bucket visits kept) in the bucket walk's order; the force pass
 * skips j == i.  Target slot t owns idx[t * stride, (t + 1) * stride) and
 * stores at most cap entries there; cap lives in device memory, so the host
 * changes it between steps without touching a captured graph.  The density pass writes two entries (8 bytes) at a time,
 * so a 32-byte sector is completed by four stores of one thread rather than
 * eight scattered 4-byte ones; the force pass reads four at a time.
 * cnt[t] may exceed cap; then the force pass re-walks the buckets.
 * rec[2i] = (x, y, z, rho_i), rec[2i+1] = (vx, vy, vz, P_i): one 32-byte
 * sector per neighbour gather. */
struct NbrList {
    uint32_t *idx;
    uint32_t *cnt;
    float4 *rec;
    uint32_t stride;              /* slots per target in idx, a multiple of 4 */
    const uint32_t *cap;          /* device word: entries a target may store (<= stride) */
    uint32_t *max_count;          /* optional: atomicMax of cnt */
    unsigned long long *overflow; /* optional: targets with cnt > cap */
};

void launch_density(const Launch &L, const float4 *spos, const uint32_t *start, const uint32_t *end, float2 *dp,
                    float gas_override, float rest_override, float mass_override, int use_override,
                    const float4 *svel = nullptr, const NbrList *list = nullptr,
                    TargetOrder ord = TargetOrder{nullptr, nullptr}, unsigned long long *pairs = nullptr);

struct RigidGrid {
    const float4 *spos;     /* sorted sphere positions, w = body index */
    const uint32_t *start;  /* rigid bucket table */
    const uint32_t *end;
    const float4 *body_vel; /* per-body velocity (float); null = static grid */
    const int *aabb;        /* per scene ordered-int AABB of sphere centres, or null */
    int own_geometry;       /* 1: bucket count below (bucket base 0); 0: the scene's rigid grid */
    uint32_t nb, mask;
    /* the force pass: each fluid particle's contact with this grid, by
     * particle id, written by launch_fluid_contact for the particles inside
     * the bodies' grown AABB; null = the force pass walks the grid itself */
    const float4 *pre;
};

struct ForceOut {
    float4 *vel;  /* unsorted velocity, written at ids[i] */
    float4 *pos;  /* unsorted position; non-null = fused integration */
};

void launch_forces(const Launch &L, const float4 *spos, const float4 *svel, const float2 *dp, const uint32_t *start,
                   const uint32_t *end, const uint32_t *ids, ForceOut out, const RigidGrid *rigid,
                   const RigidGrid *statics, float mass_override, float visc_override, int use_override,
                   const NbrList *list = nullptr, TargetOrder ord = TargetOrder{nullptr, nullptr});

/* The fluid side of the fluid/rigid contact as its own pass, over the
 * unsorted particles: for every active fluid particle of a scene with bodies
 * that lies inside the bodies' AABB grown by the contact distance, out[id] =
 * its contact with grid G (ProcessCollisionForcesD).  The force pass then
 * reads it (G.pre). */
void launch_fluid_contact(const Launch &L, const float4 *pos, const float4 *vel, const RigidGrid &G, float4 *out);

void launch_integrate(const Launch &L, float4 *pos, const float4 *vel);

/* ---- cell-cooperative density/forces (fg_sph_cc.cu): one warp per bucket
 * run, neighbour candidates staged in shared memory.  rec receives / holds
 * the packed per-particle records (x, y, z, rho), (vx, vy, vz, P). */
void launch_density_cc(const FgScene *table, const FgScene *single, uint32_t nscenes, const uint32_t *runs,
                       const uint32_t *nruns, const uint32_t *keys, const float4 *spos, const float4 *svel,
                       const uint32_t *start, const uint32_t *end, float2 *dp, float4 *rec, uint32_t n,
                       cudaStream_t s, uint32_t warps = 4);
void launch_forces_cc(const FgScene *table, const FgScene *single, uint32_t nscenes, const uint32_t *runs,
                      const uint32_t *nruns, const uint32_t *keys, const float4 *spos, const float4 *svel,
                      const float4 *rec, const uint32_t *start, const uint32_t *end, const uint32_t *ids,
                      ForceOut out, const RigidGrid *rigid, uint32_t n, cudaStream_t s, uint32_t warps = 4);

/* ---- rigid bodies (fg_rigid.cu) ---- */
void launch_rb_from_fluid(const Launch &Lrb, const float4 *rb_spos, const uint32_t *rb_ids, const float4 *body_vel,
                          const float4 *body_cm, const float4 *fl_spos, const float4 *fl_svel,
                          const uint32_t *fl_start, const uint32_t *fl_end, float4 *force, float4 *torque,
                          int add);

/* add = 1: accumulate xyz into force/torque at the sphere's unsorted index;
 * add = 0: write (w = body index).  statics: optional static sphere grid
 * (numSRB > 0 in the reference). */
void launch_rb_from_rb(const Launch &Lrb, const float4 *rb_spos, const uint32_t *rb_ids, const float4 *body_vel,
                       const float4 *body_cm, const uint32_t *rb_start, const uint32_t *rb_end, float4 *force,
                       float4 *torque, const RigidGrid *statics, int add);

struct BodyState {
    FgD4 *x, *v, *q, *L;  /* FP64 state per body */
    const double *inv_inertia; /* 9 per body, row-major */
    const double *mass;
    float4 *x_f, *v_f, *q_f; /* FP32 mirrors read by the contact kernels */
    FgD4 *force_sum, *torque_sum; /* FP64 per-body sums (diagnostic output) */
    double *partial;              /* FG_BODY_CHUNKS x 8 FP64 partial sums per body, or null */
};

/* Per body: FP64 sum of its spheres' force/torque (unsorted, body-contiguous
 * sphere ranges) followed by the FP64 body integrator.  With st.partial the
 * sum is spread over FG_BODY_CHUNKS CTAs per body and added in a fixed order. */
#define FG_BODY_CHUNKS 16
void launch_body_update(const FgScene *table, const FgScene *single, const uint32_t *body_scene,
                        const uint32_t *body_first, const uint32_t *body_count, uint32_t nbodies,
                        const float4 *force, const float4 *torque, BodyState st, int integrate, cudaStream_t s);

/* FP32 body integrator with the reference's arithmetic (IntegrateRBK). */
void launch_integrate_rb_f32(float4 *x, const float *mass, float4 *v, const float4 *f, uint32_t nrb, float dt,
                             float4 ext, float3 vmin, float3 vmax, float4 *L, const float4 *t,
                             const float4 *inertia, float4 *q, const float4 *inv, float vlimit, cudaStream_t s);

/* reduction helpers with the reference's data flow */
void launch_copy_rb_data_to_particle(uint32_t *key, uint32_t *idx, const float4 *force, uint32_t n, cudaStream_t s);
void launch_reorder_force_torque(float4 *fo, float4 *to, const float4 *fi, const float4 *ti, const uint32_t *order,
                                 uint32_t n, cudaStream_t s);
void launch_segmented_sum(const float4 *in, const uint32_t *flags, float4 *out, uint32_t n, cudaStream_t s);
void launch_add_force_torque(const float4 *sum_f, const float4 *sum_t, const float4 *ordered_f, float4 *out_f,
                             float4 *out_t, const int *offsets, uint32_t nrb, cudaStream_t s);

/* ---- FP64 conservation diagnostics (fg_diag.cu) ----
 * out[scene * FG_DIAG_VALUES + q], q as the FG_DIAG_* enum of the public
 * header; work_first[s]..work_first[s+1] are scene s's work items; part holds
 * 9 doubles per work item. */
#define FG_DIAG_VALUES 16 /* = FG_DIAG_COUNT of the public header */
void launch_diagnostics(const Launch &L, uint32_t nscenes, const uint32_t *work_first, const float4 *pos,
                        const float4 *vel, const FgD4 *bv, const FgD4 *bL, const double *bmass, double *part,
                        double *out);

/* L2 flush helper used by the benchmark */
void launch_fill(uint32_t *buf, size_t words, uint32_t v, cudaStream_t s);

} // namespace fg

#endif
