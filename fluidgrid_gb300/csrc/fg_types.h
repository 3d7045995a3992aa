/* Host/device POD types of the GB300 SPH engine.
 *
 * A "world" is a packed set of independent scenes stepped together (one
 * scene is the plain drop-in step).  Scene s owns
 *   particles   [pbase, pbase + n)           in every per-particle array,
 *   buckets     [bucket_base, bucket_base+nb) in the fluid start/end tables,
 *   spheres     [sph_base, sph_base + nsph)   of rigid-body surface spheres,
 *   rb buckets  [rb_bucket_base, +rb_nb)      in the rigid-body start/end tables,
 *   bodies      [body_base, body_base + nbodies).
 * Sort keys are global bucket ids (bucket_base + local hash), so one stable
 * sort over all particles groups them by scene and then by bucket, and the
 * order inside a scene equals that scene sorted alone.
 */
#ifndef FG_TYPES_H
#define FG_TYPES_H

#include <stdint.h>

#define FG_CHUNK 128u /* particles per work item (one CTA) */

/* FP64 4-vector (rigid-body state). */
struct alignas(16) FgD4 {
    double x, y, z, w;
};

/* Per-scene constants resident in the device scene table. */
struct FgScene {
    /* fluid hash grid (CommonFluidParams.cell_size / bucket_size) */
    float cell[3];
    uint32_t nb;          /* numBuckets of the scene */
    uint32_t nb_mask;     /* nb-1 when nb is a power of two, else 0 */
    uint32_t bucket_base; /* first global bucket id */
    uint32_t pbase;       /* first particle */
    uint32_t n;           /* particles */
    /* SPH constants (CommonFluidParams, FluidParams, KernelsCache) */
    float h, h2, scale, dt, dt_over_scale, vlimit;
    float vmin[3], vmax[3], gravity[3];
    float mass, rest, gas, visc;
    float kpoly6, kspiky, kvisc;
    /* boundary literals of SPHCalculateForcesK (K_FluidSim.cu:289-293) */
    float wall_dist, wall_stiff, wall_damp;
    float noslip_min[3], noslip_max[3];
    float fric_kin, fric_static;
    /* rigid-body contact */
    uint32_t sph_base, nsph;      /* surface spheres of this scene */
    uint32_t body_base, nbodies;  /* bodies of this scene */
    uint32_t rb_nb, rb_nb_mask, rb_bucket_base;
    float rb_cell[3];
    int f2r_rel[3];   /* fluid -> rigid grid search half-width (fluid_to_srb_relation) */
    int r2f_rel[3];   /* rigid -> fluid grid search half-width (rb_to_fluid_relation) */
    float fluid_radius, rb_radius;
    float ck, ckd;            /* fluid/rigid contact spring, damping */
    float fluid_eps, rb_eps;  /* 0.003 fluid side, 0.0001 rigid side */
    float rbrb_k, rbrb_kd, rbrb_eps; /* rigid/rigid contact */
    float rb_gravity[4];
    float rb_vlimit, rb_dt;
    float rb_vmin[3], rb_vmax[3];
    uint32_t flags;
    uint32_t pad[3];
};

#define FG_SCENE_HAS_RB 1u      /* scene has dynamic bodies */
#define FG_SCENE_RB_RB 2u       /* rigid/rigid contact enabled */

/* Work item: a chunk of up to FG_CHUNK particles (or spheres) of one scene. */
struct FgWork {
    uint32_t scene;
    uint32_t first;
    uint32_t count;
    uint32_t pad;
};

/* Device status word written by kernels (never trapped on the device). */
#define FG_DEV_OK 0u
#define FG_DEV_NONFINITE 1u
#define FG_DEV_SORT_TIMEOUT 2u /* a one-pass radix sort gave up waiting on a preceding tile */
#define FG_DEV_RANGE 2u

#endif
