/* fluidgrid_gb300 -- C ABI of the GB300 SPH step engine.
 *
 * A world is a packed set of independent scenes that advance together, one
 * step = the reference's HeterogeneousSimulator::doTimeStep for every scene
 * (HeterogeneousSimulator.cpp:54-127) with the two-way rigid-body coupling of
 * its commented block (:57-126, RigidBodySimulator.cpp:334-611):
 *   hash -> stable key/index radix sort -> cell start/end + sorted gather ->
 *   density -> [rigid spheres: transform+hash -> sort -> ranges -> contact
 *   from fluid] -> pressure+viscosity+walls+contact forces with fused
 *   integration -> FP64 per-body reduction + body integration.
 * A world of one scene is the plain drop-in step; many scenes give the
 * batched form (one launch per stage for all scenes).
 *
 * Every call returns an fg_status.  Plain pointers and sizes only; device
 * buffers belong to the world, host buffers to the caller.  Calls on one
 * world are not thread-safe; different worlds are independent.
 */
#ifndef FLUIDGRID_GB300_H
#define FLUIDGRID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *fg_stream_t; /* a cudaStream_t; NULL = the world creates its own */

typedef enum fg_status {
    FG_OK = 0,
    FG_E_INVALID = 1,    /* bad argument */
    FG_E_CUDA = 2,       /* CUDA runtime error (see fg_last_error) */
    FG_E_OOM = 3,        /* device allocation failed */
    FG_E_BUDGET = 4,     /* request exceeds the HBM budget */
    FG_E_NONFINITE = 5,  /* a kernel produced NaN/Inf state */
    FG_E_TIMEOUT = 6,    /* a bounded device wait gave up */
    FG_E_STATE = 7,      /* call not valid in the current state */
    FG_E_UNSUPPORTED = 8,
    FG_E_NOLIB = 9       /* CUDA driver/device unavailable */
} fg_status;

/* One rigid body: surface spheres in body coordinates and its state.
 * RigidBody (Simulators/RigidBody.cpp:55-126) + RigidBodySimulator::addElement
 * (RigidBodySimulator.cpp:76-132). */
typedef struct fg_body_desc {
    uint32_t n_spheres;
    const float *local_spheres; /* host float4[n_spheres]: x,y,z (w ignored) */
    float mass;            /* 0 = static body: never integrated (contact at zero velocity) */
    float position[3];     /* centre of mass */
    float orientation[4];  /* quaternion x,y,z,w */
    float inv_inertia[9];  /* row-major body-frame inverse inertia */
} fg_body_desc;

/* One scene.  Fields mirror CommonFluidParams / FluidParams /
 * CommonRigidBodyParams (ApplicationData.cuh:32-102) plus the constants the
 * reference writes as literals in its kernels (defaults from
 * fg_scene_desc_defaults equal those literals). */
typedef struct fg_scene_desc {
    uint32_t n_particles;
    const float *positions;  /* host float4[n]: x,y,z,w (w > 0 = active) */
    const float *velocities; /* host float4[n], or NULL for zero */
    float cell_size[3];
    int32_t bucket_size[3];  /* numBuckets = product */
    float kernel_radius;
    float velocity_limit;
    float volume_min[3], volume_max[3];
    float gravity[3];
    float simulation_scale;
    float dt;
    float mass, rest_density, gas_constant, viscosity;
    /* K_FluidSim.cu:289-293 literals */
    float wall_distance, wall_stiffness, wall_damping;
    float noslip_min[3], noslip_max[3];
    float friction_kinetic, friction_static;
    /* rigid bodies */
    uint32_t n_bodies;
    const fg_body_desc *bodies;
    float fluid_radius;           /* fluid particle contact radius */
    float rb_radius;              /* surface sphere radius (rigid grid cell) */
    int32_t rb_bucket_size[3];
    int32_t fluid_to_rb_relation[3];
    int32_t rb_to_fluid_relation[3];
    float contact_kspring, contact_kdamping;
    float fluid_contact_eps;      /* 0.003 (K_FluidSim.cu:386) */
    float rb_contact_eps;         /* 0.0001 (K_RigidBodySim.cu:87) */
    int32_t rb_rb_contact;        /* sphere/sphere contact between bodies */
    float rbrb_kspring, rbrb_kdamping, rbrb_eps; /* eps 0.001 (K_RigidBodySim.cu:42) */
    float rb_gravity[4];
    float rb_velocity_limit;
    float rb_dt;
    float rb_volume_min[3], rb_volume_max[3];
} fg_scene_desc;

void fg_scene_desc_defaults(fg_scene_desc *d);

typedef struct fg_world fg_world;

int fg_world_create(const fg_scene_desc *scenes, uint32_t nscenes, fg_stream_t stream, fg_world **out);
int fg_world_destroy(fg_world *w);

/* Enqueue nsteps steps on the world's stream (CUDA-graph replay after the
 * first call).  Returns without waiting. */
int fg_world_step(fg_world *w, uint32_t nsteps);
/* One stage of a step, enqueued on the world's stream on its own, for host
 * code that sequences the step itself as the reference's two-way step does
 * (HeterogeneousSimulator.cpp:57-126, RigidBodySimulator.cpp:313-611).
 * Stages run in this order; FG_RUN_INTEGRATE ends the step.  A stage whose
 * inputs were not made earlier in the same step returns FG_E_STATE (the
 * rigid stages do nothing in a world without bodies), and fg_world_step
 * returns FG_E_STATE while a staged step is unfinished.  The kernels are
 * those of fg_world_step, so a staged step gives the same bits; no graph is
 * captured and no autotuning round runs.  flags: FG_RUN_WITH_CONTACT for
 * FG_RUN_FORCES adds the rigid contact term (a whole step always does). */
enum {
    FG_RUN_NEIGHBOURHOOD = 1, /* hash, sort, cell ranges + sorted gather */
    FG_RUN_DENSITY = 2,
    FG_RUN_RB_GRID = 3,        /* sphere world positions, keys, sort, ranges */
    FG_RUN_RB_FROM_FLUID = 4,  /* sphere force/torque from the fluid */
    FG_RUN_RB_FROM_RB = 5,     /* + sphere/sphere contact between bodies */
    FG_RUN_FORCES = 6,         /* pressure, viscosity, walls (+ contact): velocities */
    FG_RUN_BODY_SUMS = 7,      /* FP64 per-body force/torque sums */
    FG_RUN_BODY_INTEGRATE = 8, /* FP64 body integration */
    FG_RUN_INTEGRATE = 9       /* particle positions; ends the step */
};
enum { FG_RUN_WITH_CONTACT = 1 };
int fg_world_run_stage(fg_world *w, int stage, int flags);
/* Wait for the world's stream; returns FG_E_NONFINITE if the last
 * fg_world_check found NaN/Inf, FG_E_CUDA on a CUDA error. */
int fg_world_sync(fg_world *w);
/* Scan every scene's state for NaN/Inf (enqueued; result seen at sync). */
int fg_world_check(fg_world *w);

/* Whole-world state in packed scene-major order (host float4 arrays of
 * fg_world_particles() entries).  Copies are enqueued on the world's stream;
 * pinned host memory makes them asynchronous. */
int fg_world_upload(fg_world *w, const float *pos4, const float *vel4);
int fg_world_download(fg_world *w, float *pos4, float *vel4);
/* One scene's state (scene-local arrays of n_particles entries). */
int fg_world_scene_upload(fg_world *w, uint32_t scene, const float *pos4, const float *vel4);
int fg_world_scene_download(fg_world *w, uint32_t scene, float *pos4, float *vel4);

uint32_t fg_world_particles(const fg_world *w);
uint32_t fg_world_scenes(const fg_world *w);
uint32_t fg_world_spheres(const fg_world *w);
uint32_t fg_world_bodies(const fg_world *w);
/* scene layout: first particle, particle count, first global bucket,
 * buckets, first sphere, spheres, first body, bodies */
int fg_world_scene_layout(const fg_world *w, uint32_t scene, uint32_t out[8]);

/* Device buffers of a world (for drop-in callers and parity checks). */
typedef enum fg_buffer_id {
    FG_BUF_POS = 0, FG_BUF_VEL, FG_BUF_KEYS_UNSORTED, FG_BUF_KEYS, FG_BUF_IDS, FG_BUF_START, FG_BUF_END,
    FG_BUF_SPOS, FG_BUF_SVEL, FG_BUF_DP,
    FG_BUF_RB_LOCAL, FG_BUF_RB_WORLD, FG_BUF_RB_KEYS_UNSORTED, FG_BUF_RB_KEYS, FG_BUF_RB_IDS, FG_BUF_RB_START,
    FG_BUF_RB_END, FG_BUF_RB_SPOS, FG_BUF_RB_FORCE, FG_BUF_RB_TORQUE,
    FG_BUF_BODY_X, FG_BUF_BODY_V, FG_BUF_BODY_Q, FG_BUF_BODY_L, FG_BUF_BODY_FSUM, FG_BUF_BODY_TSUM,
    FG_BUF_BODY_XF, FG_BUF_BODY_VF, FG_BUF_BODY_QF, FG_BUF_BODY_MASS, FG_BUF_BODY_INV_INERTIA,
    FG_BUF_COUNT
} fg_buffer_id;
int fg_world_buffer(fg_world *w, int id, void **dev_ptr, size_t *bytes);

/* Stage control for parity checks: run only the stages whose bit is set in
 * `mask` for the next fg_world_step calls (default: all).  Bits follow the
 * step order below. */
enum {
    FG_STAGE_HASH = 1, FG_STAGE_SORT = 2, FG_STAGE_RANGES = 4, FG_STAGE_DENSITY = 8,
    FG_STAGE_RB_GRID = 16, FG_STAGE_RB_CONTACT = 32, FG_STAGE_FORCES = 64, FG_STAGE_BODIES = 128,
    FG_STAGE_ALL = 255
};
int fg_world_set_stages(fg_world *w, uint32_t mask);
/* 0 = fused forces+integration (default), 1 = separate SPHIntegrateK pass */
int fg_world_set_fused_integrate(fg_world *w, int fused);
/* radix digit width 1..8 (autotuned default) */
int fg_world_set_sort_digit_bits(fg_world *w, uint32_t bits);
/* 1 = capture steps in a CUDA graph (default), 0 = direct launches */
int fg_world_set_graphs(fg_world *w, int on);
/* Tunables (they change how work is scheduled, not which neighbours are
 * summed):
 *   FG_OPT_KERNEL         density/force kernels:
 *                         1 = one thread per particle with in-range
 *                             neighbour lists recorded by the density pass
 *                             (default);
 *                         0 = one thread per particle walking the 27 buckets
 *                             in both passes;
 *                         2 = one warp per run, one target at a time
 *   FG_OPT_NEIGHBOR_LIST  1 = kernel 1, 0 = kernel 0
 *   FG_OPT_TARGET_ORDER   kernels 0/1: 1 = targets in Morton order of their
 *                         cells, 0 = hashed bucket order, 2 = Morton order in
 *                         the force pass only (default, server worlds too): the
 *                         density pass walks in bucket order, where a warp's
 *                         lanes share their buckets, and the force pass's
 *                         lanes, spatially close, share neighbour records
 *   FG_OPT_ORDER_PERIOD   steps between refreshes of the Morton order (16)
 *   FG_OPT_DIGIT_BITS     radix digit width 1..8
 *   FG_OPT_AUTOTUNE_PERIOD  every this many steps the autotuner runs one
 *                         (real) step per candidate value of one tunable
 *                         under CUDA events and keeps the fastest (0 = off;
 *                         default 25): the best choice changes as a scene
 *                         compresses
 *   FG_OPT_AUTOTUNE_KERNELS bit mask of candidate kernels (default 0x2:
 *                         kernel 1 only, so results never depend on timing)
 *   FG_OPT_LIST_CAP       kernel 1: neighbour-list slots per particle, a
 *                         multiple of 4 (default 160, at most 2048; values
 *                         round up to a multiple of 4; a particle with more
 *                         in-range visits re-walks its buckets in the force
 *                         pass; a value beyond the allocation reallocates
 *                         the lists with 1.5x headroom, one within it changes
 *                         nothing but the limit; setting it turns
 *                         FG_OPT_LIST_AUTOGROW off)
 *   FG_OPT_LIST_AUTOGROW  kernel 1: 1 = every 25 steps grow the capacity to
 *                         1.125x the largest in-range count seen (default)
 *   FG_OPT_GRAPH_STEPS    steps captured in one CUDA graph launch (1..64,
 *                         default 1); such a launch never spans an
 *                         autotuning round or a list capacity check
 *   FG_OPT_CTAS_PER_SM    kernels 0/1: CTAs per SM of the persistent
 *                         128-thread density/force grids (0 = 64; the
 *                         autotuner tries 16, 32 and 64)
 *   FG_OPT_AUTOTUNE_TILES bit mask of the tunables the autotuner varies:
 *                         1 = CTAs per SM, 2 = radix digit width, 4 = the
 *                         sort variant of FG_OPT_ONE_PASS_SORT, 8 = block
 *                         size, 16 = runs per CTA (default 31)
 *   FG_OPT_BLOCK_SIZE     kernels 0/1: threads per CTA of the density/force
 *                         grids, 64, 128 (default) or 256; work items stay
 *                         128 particles (two passes of a 64-thread CTA, two
 *                         items per 256-thread CTA) and the threads per SM
 *                         stay those of FG_OPT_CTAS_PER_SM
 *   FG_OPT_RUNS_PER_CTA   kernel 2: bucket runs in flight per CTA (one warp
 *                         each), 1, 2 or 4 (default)
 *   FG_OPT_ONE_PASS_SORT  the fluid sort's variant: 0 = upsweep, scan and
 *                         downsweep kernels per digit pass; 1 = one kernel
 *                         per pass (decoupled look-back); 2 = counting by
 *                         bucket (a histogram of the keys, a scan that
 *                         writes the cell ranges, a scatter, a stable rank
 *                         inside each bucket).  Default: 2 for worlds with at
 *                         most 64 buckets per particle, else 0.  The same
 *                         order and cell ranges from each.
 * Kernels 0 and 1 (with either target order) produce bit-identical states;
 * kernel 2 sums the same terms in another order.  No kernel's results depend
 * on CTAs per SM or digit width, and kernel 1's not on the list capacity
 * either (the list holds the bucket walk's order). */
enum {
    FG_OPT_NEIGHBOR_LIST = 1, FG_OPT_TARGET_ORDER = 2, FG_OPT_ORDER_PERIOD = 3, FG_OPT_DIGIT_BITS = 4,
    FG_OPT_KERNEL = 5, FG_OPT_AUTOTUNE_PERIOD = 6, FG_OPT_AUTOTUNE_KERNELS = 7, FG_OPT_LIST_CAP = 8,
    FG_OPT_CTAS_PER_SM = 10, FG_OPT_AUTOTUNE_TILES = 11, FG_OPT_LIST_AUTOGROW = 12, FG_OPT_GRAPH_STEPS = 13,
    FG_OPT_ONE_PASS_SORT = 14, FG_OPT_BLOCK_SIZE = 16, FG_OPT_RUNS_PER_CTA = 17
};
#define FG_NUM_KERNELS 3
int fg_world_set_option(fg_world *w, int option, int value);
int fg_world_get_option(const fg_world *w, int option, int *value);
/* In-range pair visits (self and duplicate-bucket visits included) counted by
 * the density pass and the steps run since the last reset (synchronises the
 * world's stream). */
int fg_world_counters(fg_world *w, int reset, uint64_t *pair_visits, uint64_t *steps);
/* kernel 1: particles whose in-range visits exceeded the list capacity, summed
 * over the steps since the last reset (synchronises the world's stream) */
int fg_world_list_overflows(fg_world *w, int reset, uint64_t *particles);
/* steps run with each kernel so far and the last autotuning trial times */
int fg_world_tuning_stats(const fg_world *w, uint32_t steps_per_kernel[FG_NUM_KERNELS],
                          float last_trial_ms[FG_NUM_KERNELS]);

/* number of kernel launches one step enqueues */
uint32_t fg_world_launches_per_step(const fg_world *w);
/* kernel launches this world has enqueued or replayed so far: every step's,
 * the target-order refreshes and the L2 flushes of fg_world_timed_steps */
int fg_world_kernel_launches(const fg_world *w, uint64_t *count);

/* ---- measurement (CUDA events on the world's stream) ----
 * One step in direct-launch mode with an event pair around each stage,
 * after rewriting a flush_bytes buffer (0 = no flush); stage_ms[k] receives
 * the time of stage bit k (0 if not run). */
int fg_world_stage_profile(fg_world *w, size_t flush_bytes, float stage_ms[8]);
/* nsteps steps (graph replay), each bracketed by events; before each step a
 * flush_bytes buffer is rewritten so no step starts with a warm L2.
 * ms[k] = duration of step k. */
int fg_world_timed_steps(fg_world *w, uint32_t nsteps, size_t flush_bytes, float *ms);
/* FP64 conservation diagnostics, per scene FG_DIAG_COUNT doubles summed on
 * the GPU in a fixed order (reproducible bit for bit): out[scene *
 * FG_DIAG_COUNT + q].  Synchronises the world's stream. */
enum {
    FG_DIAG_ACTIVE = 0,         /* active particles (w > 0) */
    FG_DIAG_MASS = 1,           /* sum m */
    FG_DIAG_MOMENTUM = 2,       /* sum m v (3) */
    FG_DIAG_KINETIC = 5,        /* sum m |v|^2 / 2 */
    FG_DIAG_MOMENT = 6,         /* sum m x (3): centre of mass times mass */
    FG_DIAG_BODY_MOMENTUM = 9,  /* sum M v of the bodies (3) */
    FG_DIAG_BODY_ANGULAR = 12,  /* sum L of the bodies (3) */
    FG_DIAG_BODY_KINETIC = 15,  /* sum M |v|^2 / 2 of the bodies */
    FG_DIAG_COUNT = 16
};
int fg_world_diagnostics(fg_world *w, double *out);
/* nblocks blocks of steps_per_block steps each (multi-step graphs apply),
 * each block bracketed by events; ms[k] = duration of block k. */
int fg_world_timed_blocks(fg_world *w, uint32_t nblocks, uint32_t steps_per_block, size_t flush_bytes, float *ms);
/* End to end through host memory: per step, copy positions and velocities
 * from host_pos4/host_vel4 to the device, step, copy them back to
 * out_pos4/out_vel4 (in and out may be the same buffers); ms[k] = device
 * time of step k including its copies.  With pinned host buffers
 * (fg_host_alloc) the copies run inside the step's graph: the velocity
 * upload beside the hash and sort, and each step's velocity download beside
 * the next step's position upload (the last one at the end of the call).
 * Every output has landed when the call returns. */
int fg_world_e2e_steps(fg_world *w, uint32_t nsteps, const float *host_pos4, const float *host_vel4,
                       float *out_pos4, float *out_vel4, float *ms);
void *fg_host_alloc(size_t bytes); /* pinned host memory, NULL on failure */
int fg_host_free(void *p);
int fg_set_device(int device);
/* FP32 FMA throughput of the current device (register-resident loop), in
 * TFLOP/s; used as the FP32 roofline denominator. */
int fg_probe_fp32_peak(float *tflops);

/* Stable in-place sort of n (key, value) pairs by the low keyBits bits of the
 * key -- the same result as fgc_sort_pairs -- without allocating: its scratch
 * is a fixed 8,913,920-byte (8.91 MB) array inside the library (held on every
 * GPU that loads it), for callers that cannot call cudaMalloc/cudaFree while they sort (a
 * host that gives all device memory to its own pool, a step loop that must
 * not wait for the allocator).  No counterpart in the reference.
 * n <= 1,048,576 (larger n -> FG_E_INVALID).  All calls share the scratch:
 * calls that overlap on the GPU race, so serialise them.  Each call outside
 * stream capture looks up the scratch address on the current device; a call
 * during capture reuses the last one, so make the first call on a device
 * before any stream capture (else FG_E_STATE).
 * Work is enqueued on `stream` (NULL = legacy default stream). */
int fg_sort_pairs_noalloc(unsigned int *keys, unsigned int *values, unsigned int keyBits, unsigned int n,
                          fg_stream_t stream);

/* Self-test of the bounded waits in the one-pass sort's look-back: runs one
 * tile whose predecessor never publishes, so its wait gives up after
 * spin_limit rounds; *flags receives the device status bits it set (2 = the
 * sort's wait gave up).  The context stays usable afterwards. */
int fg_selftest_bounded_wait(unsigned int spin_limit, unsigned int *flags);

/* ---- served form: continuous batching of scenes (no reference
 * counterpart; each scene's step is HeterogeneousSimulator::doTimeStep) ----
 * Requests -- a scene and a step count -- queue on the host.  Every
 * fg_server_step admits queued requests in arrival order while the resident
 * scenes' device bytes stay within hbm_budget_bytes, their particles within
 * max_particles (if set) and the predicted step time within target_step_ms
 * (if set), skipping requests that do not fit yet; a younger request passes
 * the oldest only if it finishes before the oldest can fit (backfilling),
 * advances every resident scene by one step in the same launches, and
 * retires scenes that reached their step count (their final state is kept
 * on the host until fg_server_result releases it).  A scene's result is the
 * same bits as the scene stepped alone in a one-scene world. */
typedef struct fg_server fg_server;
typedef struct fg_server_config {
    size_t hbm_budget_bytes;      /* device bytes the resident scenes may use */
    uint32_t max_particles;       /* particles advanced per step, 0 = no limit (default 1,200,000;
                                     a larger scene is refused with FG_E_BUDGET) */
    uint32_t max_admit_per_step;  /* 0 = no limit */
    int use_graphs;               /* replay captured steps while the resident set is stable */
    int grow_via_host;            /* 1: when the world grows, always park the state on the host
                                     (otherwise only when both worlds would not fit) */
    int pipeline_depth;           /* steps fg_server_step may leave running on the device (0 =
                                     return after each step finishes); a change of the resident
                                     set, a retirement or a result waits for all of them */
    float target_step_ms;         /* per-step work budget: a request is admitted only while the
                                     predicted device time of one step over the resident scenes
                                     stays within it (an empty server admits any request); the
                                     prediction is a fixed 0.1 ms plus a per-particle rate learned
                                     from the finished steps; 0 = no time budget (default 1.1) */
    float head_wait_s;            /* once the oldest queued request has waited this long and does
                                     not fit, it gets a reservation: a younger request is admitted
                                     only if it fits now and finishes before enough resident scenes
                                     have left for the oldest to fit (backfilling); default 0 */
    int autotune_period;          /* steps between autotuning rounds of the resident world; 0 = no
                                     autotuning (default: a round's trial steps of other launch
                                     shapes land in the step latency; measured on the C5 arrivals,
                                     off gave 3% more throughput and a lower p99) */
} fg_server_config;
enum { FG_REQ_QUEUED = 0, FG_REQ_ACTIVE = 1, FG_REQ_DONE = 2 };
typedef struct fg_server_step_info {
    uint32_t active_scenes;   /* scenes advanced by this step */
    uint32_t admitted;        /* of which newly admitted */
    uint32_t finished;        /* scenes that reached their step count */
    uint32_t queued;          /* requests still waiting */
    uint64_t active_particles;
    float step_ms;            /* device time of the step (CUDA events); with pipeline_depth > 0,
                                 of the newest step that has finished (0 if none has) */
    float pad_;
    double wall_ms;           /* host time of fg_server_step (admission, layout, step, retirement) */
    size_t resident_bytes;
} fg_server_step_info;
typedef struct fg_request_info {
    int state;                /* FG_REQ_* */
    uint32_t steps_done, steps_total, n_particles;
    double submit_s, admit_s, done_s; /* host clock, seconds since fg_server_create */
    size_t resident_bytes;    /* budget charge while resident */
} fg_request_info;
typedef struct fg_server_stats_info {
    uint64_t steps, particle_steps;
    uint32_t queued, active;
    size_t resident_bytes;    /* budget charge of the resident scenes */
    uint64_t resident_particles;
    size_t device_bytes;      /* bytes the server's world holds (capacity) */
} fg_server_stats_info;
/* 120 GiB budget, graphs on, 850k particles and a predicted 0.9 ms per step */
void fg_server_config_defaults(fg_server_config *cfg);
int fg_server_create(const fg_server_config *cfg, fg_stream_t stream, fg_server **out);
void fg_server_destroy(fg_server *s);
/* Copies the description and its arrays.  FG_E_BUDGET if the scene alone
 * exceeds the budget. */
int fg_server_submit(fg_server *s, const fg_scene_desc *scene, uint32_t steps, uint64_t *request_id);
int fg_server_step(fg_server *s, fg_server_step_info *info);
int fg_server_request(const fg_server *s, uint64_t request_id, fg_request_info *info);
/* Final positions and velocities (n x float4 each, either may be NULL) of a
 * finished request; release = 1 forgets the request.  FG_E_STATE if it has
 * not finished. */
int fg_server_result(fg_server *s, uint64_t request_id, float *pos4, float *vel4, int release);
int fg_server_stats(const fg_server *s, fg_server_stats_info *stats);
/* Request ids of the resident scenes (the ones the next step advances), at
 * most `cap` of them; *count receives how many are resident. */
int fg_server_active(const fg_server *s, uint64_t *ids, uint32_t cap, uint32_t *count);

/* Small helpers so callers without a CUDA runtime binding can move data. */
int fg_memcpy_d2h(void *dst, const void *src, size_t bytes);
int fg_memcpy_h2d(void *dst, const void *src, size_t bytes);
int fg_device_synchronize(void);
const char *fg_last_error(void);
const char *fg_version(void);

#ifdef __cplusplus
}
#endif

#endif
