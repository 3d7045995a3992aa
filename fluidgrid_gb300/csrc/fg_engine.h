/* World engine internals (host side). */
#ifndef FG_ENGINE_H
#define FG_ENGINE_H

#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <vector>
#include "fg_types.h"
#include "fg_kernels.h"

struct fg_scene_desc;

namespace fg {

#define FG_LIST_CAP_DEFAULT 160u
#define FG_LIST_CAP_MAX 2048u
#define FG_LIST_CHECK_PERIOD 25u
/* list strides are multiples of 8 entries: the force pass reads each list
 * eight entries (one 32-byte sector) at a time from its start */
static_assert(FG_LIST_CAP_DEFAULT % 8u == 0u && FG_LIST_CAP_MAX % 8u == 0u, "list strides must be multiples of 8");

void set_error(const char *what, cudaError_t e);
void set_error_msg(const char *what);
void fill_scene(FgScene &S, const fg_scene_desc &d);
int validate(const fg_scene_desc &d);

/* Element capacities of a world's buffers. */
struct Capacity {
    uint64_t particles = 0, buckets = 0, spheres = 0, bodies = 0, rb_buckets = 0, scenes = 0;
    uint64_t work = 0, work_sph = 0; /* FG_CHUNK work items */
    bool fits(const Capacity &o) const;
    bool too_large() const;
};

/* worlds with at most this many buckets per particle count their keys
 * (sort variant 2) by default */
#define FG_BUCKET_SORT_RATIO 64

struct World {
    /* layout */
    uint32_t nscenes = 0, n = 0, total_buckets = 0, nspheres = 0, nbodies = 0, total_rb_buckets = 0;
    uint32_t nwork = 0, nwork_sph = 0;
    uint32_t key_bits = 0, rb_key_bits = 0, digit_bits = 8;
    bool single = true;
    bool any_rb_rb = false;
    bool rb_small_scenes = true; /* every scene has <= FG_RB_SCENE_MAX spheres: one-CTA rigid grid */
    std::vector<FgScene> scenes_h;
    FgScene *scenes_d = nullptr;
    FgWork *work_d = nullptr, *work_sph_d = nullptr;
    /* fluid */
    float4 *pos = nullptr, *vel = nullptr, *spos = nullptr, *svel = nullptr;
    float2 *dp = nullptr;
    uint32_t *keys_u = nullptr, *keys = nullptr, *ids = nullptr, *start = nullptr, *end = nullptr;
    RadixScratch rs{nullptr, nullptr, nullptr};
    uint32_t *os_scratch = nullptr; /* one-pass sort: tile status words, digit bases, tile counters */
    bool one_pass_sort = false; /* measured slower on the 1M dam break (0.088 vs 0.076 ms) */
    /* counting sort by bucket (sort variant 2); set_layout turns it on when
     * the world has at most FG_BUCKET_SORT_RATIO buckets per particle */
    bool bucket_sort_on = false;
    bool sort_chosen = false; /* the variant was set explicitly: set_layout keeps it */
    bool counted_ranges = false; /* this step's sort wrote start/end */
    bool fused_ranges = false;   /* ... and did the ranges pass's reorder */
    int sort_variant() const { return bucket_sort_on ? 2 : (one_pass_sort ? 1 : 0); }
    void set_sort_variant(int v)
    {
        one_pass_sort = (v == 1);
        bucket_sort_on = (v == 2);
    }
    void enqueue_sort(bool with_ranges = false);
    void enqueue_hash(const Launch &L, bool sort_follows);
    bool counted_in_hash = false; /* this step's hash pass counted the keys for the counting sort */
    /* the counting sort's tile sums fit the radix scratch */
    bool bucket_sort_fits() const
    {
        const uint64_t tiles = ((uint64_t)total_buckets + FG_RS_TILE - 1) / FG_RS_TILE;
        return total_buckets && tiles <= radix_hist_words((uint32_t)std::max<uint64_t>(cap.particles, 1));
    }
    uint32_t sort_launches() const;
    NbrList nbr{nullptr, nullptr, nullptr, 0, nullptr, nullptr}; /* density -> forces neighbour lists */
    uint32_t list_cap_alloc = 0; /* list slots per particle allocated (the stride) */
    uint32_t list_cap = 0;       /* entries a particle may store (<= list_cap_alloc) */
    uint32_t *list_cap_d = nullptr; /* the same, in device memory for the kernels */
    uint32_t *inv = nullptr;  /* particle -> sorted index (written by the ranges pass) */
    uint32_t *tord = nullptr; /* spatial target order (particle ids, scene-contiguous) */
    /* default: Morton target order in the force pass only (FG_OPT_TARGET_ORDER 2) */
    bool use_list = true, use_order = true;
    bool order_forces_only = true;
    bool use_cc = false;       /* kernel 2: warp per bucket run, candidates staged in shared memory */
    uint32_t ctas_per_sm = 0;  /* CTAs per SM of the density/force grids (0 = 64) */
    uint32_t block = 128;      /* kernels 0/1: threads per CTA of the density/force grids (64, 128, 256) */
    uint32_t cc_warps = 4;     /* kernel 2: bucket runs (warps) per CTA (1, 2, 4) */
    int set_list_cap(uint32_t cap);
    uint32_t *runs = nullptr;  /* occupied-bucket run heads */
    uint32_t *nruns = nullptr; /* device counter */
    uint32_t order_period = 16, order_bits = 8, order_scene_shift = 24, order_key_bits = 24;
    uint64_t step_count = 0;
    uint64_t kernels_enqueued = 0; /* kernel launches enqueued or replayed so far */
    bool order_valid = false;
    void enqueue_order_refresh();
    /* the target order of the force pass, and of the density pass unless
     * the Morton order is the force pass's only; the neighbour lists are
     * indexed by sorted particle, so the two passes may differ */
    TargetOrder target_order() const
    {
        return (use_order && order_valid) ? TargetOrder{tord, inv} : TargetOrder{nullptr, nullptr};
    }
    TargetOrder density_order() const
    {
        return order_forces_only ? TargetOrder{nullptr, nullptr} : target_order();
    }
    bool order_refresh_due(uint64_t s) const;
    /* rigid */
    float4 *rb_local = nullptr, *rb_world = nullptr, *rb_spos = nullptr, *rb_force = nullptr, *rb_torque = nullptr;
    float4 *fcontact = nullptr; /* per sorted fluid particle: its contact with the bodies' spheres */
    uint32_t *rb_keys_u = nullptr, *rb_keys = nullptr, *rb_ids = nullptr, *rb_start = nullptr, *rb_end = nullptr;
    int *aabb = nullptr;
    FgD4 *bx = nullptr, *bv = nullptr, *bq = nullptr, *bL = nullptr, *bfs = nullptr, *bts = nullptr;
    double *body_part = nullptr; /* FG_BODY_CHUNKS x 8 FP64 partial sums per body */
    float4 *bxf = nullptr, *bvf = nullptr, *bqf = nullptr;
    float4 *bvf_next = nullptr; /* velocity mirror written beside the force pass */
    double *bmass = nullptr, *binv = nullptr;
    uint32_t *body_scene = nullptr, *body_first = nullptr, *body_count = nullptr;
    uint32_t *status_d = nullptr;
    unsigned long long *pair_counter = nullptr; /* in-range pair visits since the last reset */
    uint64_t counted_steps = 0;
    /* execution */
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaStream_t stream2 = nullptr; /* rigid-body branch of a full step */
    cudaEvent_t ev_fork = nullptr, ev_fluid_ready = nullptr, ev_rb_done = nullptr, ev_bodies_done = nullptr;
    cudaStream_t stream3 = nullptr; /* velocity upload of an end-to-end step */
    cudaEvent_t ev_io_fork = nullptr, ev_vel_in = nullptr, ev_pos_in = nullptr;
    void enqueue_rb_grid(cudaStream_t st, cudaEvent_t *ev, uint32_t &launches);
    void enqueue_rb_contact(cudaStream_t st, cudaEvent_t *ev, uint32_t &launches, bool with_fluid);
    void enqueue_fluid_contact(cudaStream_t st, uint32_t &launches);
    RigidGrid body_grid() const;
    bool fluid_contact_pass() const;
    void enqueue_bodies(cudaStream_t st, float4 *vf);
    /* kernels of one body update: the chunked FP64 partial sums (up to 65,535
     * bodies) and the update */
    uint32_t body_launches() const { return nbodies <= 65535u ? 2u : 1u; }
    uint32_t stages = 255;
    bool fused_integrate = true;
    bool use_graphs = true;
    /* one instantiated step graph per configuration signature */
    /* host buffers of an end-to-end step: the positions and velocities it
     * uploads before and downloads after (16 bytes per particle each) */
    struct StepIO {
        const void *hp = nullptr, *hv = nullptr;
        void *op = nullptr, *ov = nullptr;
        /* prev_vel: the step first downloads the previous step's velocities
         * (still in vel) to ov, beside its own position upload; defer_vel:
         * the step leaves its velocities for the next step (or the caller)
         * to download */
        bool prev_vel = false, defer_vel = false;
        bool operator==(const StepIO &o) const
        {
            return hp == o.hp && hv == o.hv && op == o.op && ov == o.ov && prev_vel == o.prev_vel &&
                   defer_vel == o.defer_vel;
        }
    };
    const StepIO *cur_io = nullptr; /* set while step() runs an end-to-end step */
    struct CachedGraph {
        uint64_t sig;
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        StepIO io;
    };
    std::vector<CachedGraph> graphs;
    /* graphs whose parameters a layout change or a list reallocation made
     * stale: a later capture with the same signature updates one in place
     * (cudaGraphExecUpdate) instead of instantiating a new one */
    std::vector<CachedGraph> stale;
    uint64_t graph_signature() const;
    int graph_for_current(cudaGraphExec_t *out, uint32_t nsteps = 1);
    uint32_t graph_steps = 1; /* steps per captured graph launch */
    bool host_boundary(uint64_t s) const;
    /* online autotuner: every tune_period steps, each candidate value of one
     * tunable (kernel, block warps, digit width; the tunable rotates) runs
     * one real step under CUDA events and the fastest is kept */
    uint32_t tune_period = 25;
    uint32_t tune_count[3] = {0, 0, 0}; /* steps run with kernel 0..2 */
    float tune_last_ms[3] = {0.f, 0.f, 0.f};
    uint32_t tune_kernels = 0x2; /* candidate kernels bit mask */
    uint32_t tune_tiles = 0x1f;  /* 1: CTAs per SM, 2: digit width, 4: sort variant, 8: block size,
                                    16: runs per CTA (kernel 2) */
    uint32_t tune_round = 0;
    unsigned long long *overflow_counter = nullptr; /* list overflows since the last reset */
    uint32_t *max_count = nullptr; /* largest list count since the last capacity check */
    bool list_autogrow = true;     /* grow the list capacity to the largest count seen */
    int check_list_cap();
    int current_kernel() const { return use_cc ? 2 : (use_list ? 1 : 0); }
    void set_kernel(int k)
    {
        use_cc = (k == 2);
        use_list = (k == 1);
    }
    bool needs_runs() const { return use_cc; }
#define FG_TUNE_MARGIN 0.015f
    struct TuneRound {
        bool active = false;
        int dim = 0, ncand = 0, idx = 0;
        int prev = 0; /* the tunable's value before the round */
        int cand[4] = {0, 0, 0, 0};
        cudaEvent_t ev[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    } tr;
    void tune_begin();
    void tune_apply(int dim, int v);
    int tune_finish();
    std::vector<void *> allocs;
    size_t device_bytes = 0;

    ~World();
    int alloc(void **p, size_t bytes);
    int create(const fg_scene_desc *d, uint32_t ns, cudaStream_t st);
    /* building blocks of create() that the server reuses */
    Capacity cap;
    static Capacity needs(const fg_scene_desc *d, uint32_t ns);
    static size_t footprint(const Capacity &c, uint32_t list_cap);
    int init_stream(cudaStream_t st);
    int reserve(const Capacity &c);
    int set_layout(const fg_scene_desc *d, uint32_t ns);
    int upload_scene(uint32_t s, const fg_scene_desc &d);
    void drop_graphs();  /* destroys every captured graph */
    void stale_graphs(); /* keeps them for in-place updates */
    /* FP64 conservation diagnostics */
    std::vector<uint32_t> work_first_h; /* scene s owns work items [first[s], first[s+1]) */
    uint32_t *diag_first = nullptr;
    double *diag_part = nullptr, *diag_out = nullptr;
    size_t diag_cap_work = 0, diag_cap_scenes = 0;
    int diagnostics(double *out);
    Launch fluid_launch() const;
    Launch sphere_launch() const;
    uint32_t enqueue_step(cudaEvent_t *stage_events = nullptr);
    uint32_t *flush_buf = nullptr;
    size_t flush_bytes = 0;
    int step(uint32_t nsteps, const StepIO *io = nullptr);
    /* One stage of a step enqueued on its own (FG_RUN_* of the public
     * header), in the order of the reference's step; staged_done holds the
     * FG_RUN_* bits (1 << stage) already run in the current step. */
    uint32_t staged_done = 0;
    int run_stage(int stage, int flags);
    int step_loop(uint32_t nsteps);
    uint32_t launches_per_step();
    int check();
    int sync();
    int ensure_flush(size_t bytes);
    int stage_profile(size_t flush_bytes, float *ms);
    int timed_steps(uint32_t nblocks, size_t flush_bytes, float *ms, uint32_t per_block = 1);
    int e2e_steps(uint32_t nsteps, const float *hp, const float *hv, float *op, float *ov, float *ms);
};

} // namespace fg

#endif
