/* Served form: continuous batching of independent scenes on one GPU.
 *
 * Requests (a scene plus a number of steps) queue on the host.  At every
 * server step, requests that fit the HBM budget, the limit of particles
 * advanced per step and the per-step time budget are admitted in arrival
 * order, skipping any that do not fit yet; finished scenes leave.  The time
 * budget bounds the latency of every resident scene's step: the step over
 * the resident set is predicted as a fixed 0.1 ms plus a per-particle rate
 * that an exponential average learns from the finished steps of at least
 * 100k particles.  When the oldest request does not fit (and has waited
 * head_wait_s, 0 by default), it gets a reservation: the number of steps
 * after which the resident scenes that finish first leave room for it; a
 * younger request is admitted only if it fits now and is done within that
 * many steps (backfilling).  So no request is passed over indefinitely, and
 * the GPU stays busy while the oldest waits.  When the resident set changes
 * the world is re-laid out in place -- the dynamic state of every continuing
 * scene (particle positions, velocities, densities, the bodies' FP64
 * motion) moves to its new offsets on the device, new scenes upload their
 * initial state -- and all resident scenes advance together in the world's
 * segment-aware launches.  A scene's arithmetic never depends on the other
 * scenes (sort keys are global bucket ids, every kernel reads only its own
 * scene's buckets), so each result equals the scene stepped alone.
 *
 * The reference has no serving layer; the per-scene step is
 * HeterogeneousSimulator::doTimeStep (HeterogeneousSimulator.cpp:54-127). */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <unordered_map>
#include <vector>
#include "../../include/fluidgrid_gb300.h"
#include "fg_engine.h"

namespace fg {

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            set_error(#call, e_);                                                                  \
            return (e_ == cudaErrorMemoryAllocation) ? FG_E_OOM : FG_E_CUDA;                       \
        }                                                                                          \
    } while (0)

struct Request {
    uint64_t id = 0;
    fg_scene_desc desc;
    std::vector<float> pos, vel;             /* initial state (host copies) */
    std::vector<fg_body_desc> bodies;
    std::vector<std::vector<float>> spheres; /* local sphere positions per body */
    uint32_t steps_total = 0, steps_done = 0;
    int state = FG_REQ_QUEUED;
    double t_submit = 0, t_admit = 0, t_done = 0;
    size_t bytes = 0;                        /* budget charge while resident */
    std::vector<float> out_pos, out_vel;     /* final state */
};

#define FG_SERVER_RING 16 /* pipeline_depth is clamped below this */
#define FG_STEP_FIXED_MS 0.1 /* predicted per-step time independent of the particle count */
#define FG_RATE_MIN_N 100000u /* steps of fewer particles do not update the learned rate */
/* neighbour-list slots per particle of a server world: they do not grow
 * (the budget charges them at admission), so they cover the compressed
 * phase's ~300 in-range visits; a particle with more walks its buckets in
 * the force pass */
#ifndef FG_SERVER_LIST_CAP
#define FG_SERVER_LIST_CAP 320u
#endif

struct Server {
    fg_server_config cfg;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::unique_ptr<World> w;
    std::deque<Request *> queue;
    std::vector<Request *> active;  /* wanted resident set, in layout order */
    std::vector<uint64_t> laid_out; /* request id of world scene s */
    std::map<uint64_t, std::unique_ptr<Request>> all;
    uint64_t next_id = 1;
    size_t resident = 0;
    uint64_t resident_particles = 0;
    /* step events: slot k % FG_SERVER_RING brackets step k */
    cudaEvent_t ev0[FG_SERVER_RING] = {}, ev1[FG_SERVER_RING] = {};
    uint64_t issued = 0, waited = 0; /* steps enqueued / steps whose end was waited for */
    float last_ms = 0.0f;           /* device time of the newest step waited for */
    uint64_t slot_n[FG_SERVER_RING] = {}; /* particles of the step in each event slot */
    double rate_ms = 0.9e-6;        /* learned device ms per particle of a step */
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    uint64_t steps = 0, particle_steps = 0;
    uint32_t stable_steps = 0; /* steps since the last re-layout */

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    ~Server()
    {
        w.reset();
        for (int k = 0; k < FG_SERVER_RING; k++) {
            if (ev0[k]) cudaEventDestroy(ev0[k]);
            if (ev1[k]) cudaEventDestroy(ev1[k]);
        }
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
    bool layout_current() const
    {
        if (!w || laid_out.size() != active.size()) return false;
        for (size_t s = 0; s < active.size(); s++)
            if (laid_out[s] != active[s]->id) return false;
        return true;
    }
    int relayout();
    int retire_finished();
    /* steps until the resident scenes that finish first leave room for a
     * scene of n particles and `bytes` device bytes */
    uint32_t steps_until_fits(uint64_t n, size_t bytes, uint64_t pcap) const
    {
        std::vector<std::pair<uint32_t, const Request *>> by_rem;
        for (const Request *a : active) by_rem.push_back({a->steps_total - a->steps_done, a});
        std::sort(by_rem.begin(), by_rem.end(),
                  [](const std::pair<uint32_t, const Request *> &x, const std::pair<uint32_t, const Request *> &y) {
                      return x.first < y.first;
                  });
        uint64_t np = resident_particles;
        size_t nb = resident;
        for (const auto &e : by_rem) {
            np -= e.second->desc.n_particles;
            nb -= e.second->bytes;
            if (np + n <= pcap && nb + bytes <= cfg.hbm_budget_bytes) return e.first;
        }
        return by_rem.empty() ? 0u : by_rem.back().first;
    }
    int step(fg_server_step_info *info);
    /* wait until at most `depth` enqueued steps are unfinished */
    int drain(uint64_t depth)
    {
        while (issued - waited > depth) {
            const int k = (int)(waited % FG_SERVER_RING);
            CK(cudaEventSynchronize(ev1[k]));
            CK(cudaEventElapsedTime(&last_ms, ev0[k], ev1[k]));
            if (slot_n[k] >= FG_RATE_MIN_N && last_ms > FG_STEP_FIXED_MS)
                rate_ms = 0.9 * rate_ms + 0.1 * ((double)last_ms - FG_STEP_FIXED_MS) / (double)slot_n[k];
            waited++;
        }
        return FG_OK;
    }
};

/* Device bytes one scene adds to a world at list capacity list_cap. */
static size_t scene_bytes(const fg_scene_desc &d, uint32_t list_cap)
{
    const Capacity c = World::needs(&d, 1);
    const Capacity z;
    return World::footprint(c, list_cap) - World::footprint(z, list_cap);
}

/* Make the world's scenes equal `active`: continuing scenes keep their
 * dynamic state, new scenes upload theirs. */
int Server::relayout()
{
    std::vector<fg_scene_desc> descs(active.size());
    for (size_t s = 0; s < active.size(); s++) descs[s] = active[s]->desc;
    const Capacity need = World::needs(descs.data(), (uint32_t)descs.size());
    std::unordered_map<uint64_t, uint32_t> where; /* request id -> current scene index */
    for (size_t o = 0; o < laid_out.size(); o++) where[laid_out[o]] = (uint32_t)o;
    std::vector<FgScene> old_scenes;
    if (w) old_scenes.assign(w->scenes_h.begin(), w->scenes_h.begin() + w->nscenes);
    if (drain(0) != FG_OK) return FG_E_CUDA;
    if (w) CK(cudaStreamSynchronize(stream));
    /* body motion of continuing scenes goes through the host (small) */
    std::vector<double> hx, hv, hq, hL;
    std::vector<float> hxf, hvf, hqf;
    if (w && w->nbodies) {
        const size_t B = w->nbodies;
        hx.resize(4 * B); hv.resize(4 * B); hq.resize(4 * B); hL.resize(4 * B);
        hxf.resize(4 * B); hvf.resize(4 * B); hqf.resize(4 * B);
        CK(cudaMemcpy(hx.data(), w->bx, 32 * B, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hv.data(), w->bv, 32 * B, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hq.data(), w->bq, 32 * B, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hL.data(), w->bL, 32 * B, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hxf.data(), w->bxf, 16 * B, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hvf.data(), w->bvf, 16 * B, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hqf.data(), w->bqf, 16 * B, cudaMemcpyDeviceToHost));
    }
    const float4 *src_pos = nullptr, *src_vel = nullptr;
    const float2 *src_dp = nullptr;
    std::vector<float4> host_pos, host_vel; /* growth through host memory */
    std::vector<float2> host_dp;
    std::unique_ptr<World> nw;
    World *dst = w.get();
    const bool grow = !w || !w->cap.fits(need) || (need.bodies && !w->rb_local);
    if (grow) {
        /* a new world with headroom; the old world is the source */
        Capacity c = need;
        c.scenes = std::max<uint64_t>(c.scenes, 16);
        if (w) {
            auto g = [](uint64_t want, uint64_t have) { return std::max<uint64_t>(want, have + have / 2); };
            c.particles = g(need.particles, w->cap.particles);
            c.buckets = g(need.buckets, w->cap.buckets);
            c.spheres = g(need.spheres, w->cap.spheres);
            c.bodies = g(need.bodies, w->cap.bodies);
            c.rb_buckets = g(need.rb_buckets, w->cap.rb_buckets);
            c.scenes = g(need.scenes, w->cap.scenes);
            c.work = g(need.work, w->cap.work);
            c.work_sph = g(need.work_sph, w->cap.work_sph);
        }
        const uint32_t lc = w ? w->list_cap_alloc : FG_SERVER_LIST_CAP;
        /* headroom only while the world stays within the budget */
        if (c.too_large() || World::footprint(c, lc) > cfg.hbm_budget_bytes) c = need;
        nw.reset(new World());
        int r = nw->init_stream(stream);
        if (r != FG_OK) return r;
        /* the budget charges list memory at the admission-time capacity: the
         * lists do not grow (denser particles walk their buckets instead) */
        nw->list_autogrow = false;
        nw->list_cap_alloc = lc;
        /* the force pass in Morton target order, the density pass in bucket
         * order (the world default): each re-layout rebuilds the order in its
         * next step (~0.1 ms), which the faster force pass repays */
        /* trials of slower launch shapes would land in the step latency */
        nw->tune_period = (uint32_t)std::max(cfg.autotune_period, 0);
        if (w) {
            nw->list_cap_alloc = w->list_cap_alloc;
            nw->digit_bits = w->digit_bits;
            nw->ctas_per_sm = w->ctas_per_sm;
            nw->block = w->block;
            nw->cc_warps = w->cc_warps;
            nw->use_graphs = w->use_graphs;
            size_t free_b = 0, total_b = 0;
            CK(cudaMemGetInfo(&free_b, &total_b));
            if (cfg.grow_via_host || World::footprint(c, nw->list_cap_alloc) + ((size_t)1 << 30) > free_b) {
                /* both worlds would not fit at once: park the state on the
                 * host, release the old world, then build the new one */
                const size_t n0 = w->n;
                host_pos.resize(n0);
                host_vel.resize(n0);
                host_dp.resize(n0);
                if (n0) {
                    CK(cudaMemcpy(host_pos.data(), w->pos, 16 * n0, cudaMemcpyDeviceToHost));
                    CK(cudaMemcpy(host_vel.data(), w->vel, 16 * n0, cudaMemcpyDeviceToHost));
                    CK(cudaMemcpy(host_dp.data(), w->dp, 8 * n0, cudaMemcpyDeviceToHost));
                }
                w.reset();
                src_pos = host_pos.data();
                src_vel = host_vel.data();
                src_dp = host_dp.data();
            } else {
                src_pos = w->pos;
                src_vel = w->vel;
                src_dp = w->dp;
            }
        }
        if ((r = nw->reserve(c)) != FG_OK) return r;
        dst = nw.get();
    } else if (w->n) {
        /* in place: stage the state in buffers the next step rewrites anyway */
        CK(cudaMemcpyAsync(w->spos, w->pos, 16 * (size_t)w->n, cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(w->svel, w->vel, 16 * (size_t)w->n, cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(w->nbr.rec, w->dp, 8 * (size_t)w->n, cudaMemcpyDeviceToDevice, stream));
        src_pos = w->spos;
        src_vel = w->svel;
        src_dp = (const float2 *)w->nbr.rec;
    }
    int r = dst->set_layout(descs.data(), (uint32_t)descs.size());
    if (r != FG_OK) return r;
    for (size_t s = 0; s < active.size(); s++) {
        const FgScene &S = dst->scenes_h[s];
        auto it = where.find(active[s]->id);
        if (it == where.end()) {
            if ((r = dst->upload_scene((uint32_t)s, descs[s])) != FG_OK) return r;
            continue;
        }
        const FgScene &O = old_scenes[it->second];
        if (S.n) {
            CK(cudaMemcpyAsync(dst->pos + S.pbase, src_pos + O.pbase, 16 * (size_t)S.n, cudaMemcpyDefault,
                               stream));
            CK(cudaMemcpyAsync(dst->vel + S.pbase, src_vel + O.pbase, 16 * (size_t)S.n, cudaMemcpyDefault,
                               stream));
            CK(cudaMemcpyAsync(dst->dp + S.pbase, src_dp + O.pbase, 8 * (size_t)S.n, cudaMemcpyDefault,
                               stream));
        }
        if (S.nbodies) {
            const size_t B = S.nbodies, ob = O.body_base, nb = S.body_base;
            CK(cudaMemcpyAsync(dst->bx + nb, hx.data() + 4 * ob, 32 * B, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(dst->bv + nb, hv.data() + 4 * ob, 32 * B, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(dst->bq + nb, hq.data() + 4 * ob, 32 * B, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(dst->bL + nb, hL.data() + 4 * ob, 32 * B, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(dst->bxf + nb, hxf.data() + 4 * ob, 16 * B, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(dst->bvf + nb, hvf.data() + 4 * ob, 16 * B, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(dst->bqf + nb, hqf.data() + 4 * ob, 16 * B, cudaMemcpyHostToDevice, stream));
        }
    }
    /* the host staging arrays and the old world must outlive the copies */
    CK(cudaStreamSynchronize(stream));
    if (grow) w = std::move(nw);
    laid_out.resize(active.size());
    for (size_t s = 0; s < active.size(); s++) laid_out[s] = active[s]->id;
    stable_steps = 0;
    return FG_OK;
}

/* Download the final state of scenes that reached their step count and
 * release their budget. */
int Server::retire_finished()
{
    bool any = false;
    for (auto *q : active)
        if (q->steps_done >= q->steps_total) any = true;
    if (!any) return FG_OK;
    if (drain(0) != FG_OK) return FG_E_CUDA;
    CK(cudaStreamSynchronize(stream));
    std::vector<Request *> keep;
    for (size_t s = 0; s < active.size(); s++) {
        Request *q = active[s];
        if (q->steps_done < q->steps_total) {
            keep.push_back(q);
            continue;
        }
        const FgScene &S = w->scenes_h[s];
        q->out_pos.resize(4 * (size_t)S.n);
        q->out_vel.resize(4 * (size_t)S.n);
        if (S.n) {
            CK(cudaMemcpy(q->out_pos.data(), w->pos + S.pbase, 16 * (size_t)S.n, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(q->out_vel.data(), w->vel + S.pbase, 16 * (size_t)S.n, cudaMemcpyDeviceToHost));
        }
        q->state = FG_REQ_DONE;
        q->t_done = now();
        resident -= q->bytes;
        resident_particles -= q->desc.n_particles;
    }
    active.swap(keep);
    return FG_OK;
}

int Server::step(fg_server_step_info *info)
{
    const double tw0 = now();
    uint32_t admitted = 0;
    /* admission: arrival order, a request that does not fit yet is skipped */
    const uint32_t lc = w ? w->list_cap_alloc : FG_SERVER_LIST_CAP;
    const double tnow = now();
    /* particles one step may advance: the particle limit and what the time
     * budget allows at the learned rate */
    uint64_t pcap = cfg.max_particles ? (uint64_t)cfg.max_particles : ~0ull;
    if (cfg.target_step_ms > 0.0f) {
        const double t = ((double)cfg.target_step_ms - FG_STEP_FIXED_MS) / rate_ms;
        pcap = std::min<uint64_t>(pcap, t > 0.0 ? (uint64_t)t : 0ull);
    }
    bool reserved = false; /* the oldest request waits for room: backfill only */
    uint32_t reserve_steps = 0;
    for (auto it = queue.begin(); it != queue.end();) {
        if (cfg.max_admit_per_step && admitted >= cfg.max_admit_per_step) break;
        Request *q = *it;
        const size_t b = scene_bytes(q->desc, lc);
        const bool fits = active.empty() ||
                          (resident + b <= cfg.hbm_budget_bytes && resident_particles + q->desc.n_particles <= pcap);
        /* with a reservation, a younger request runs only if it is done
         * before the oldest one can start */
        if (fits && (!reserved || q->steps_total <= reserve_steps)) {
            q->bytes = b;
            q->state = FG_REQ_ACTIVE;
            q->t_admit = now();
            resident += b;
            resident_particles += q->desc.n_particles;
            active.push_back(q);
            it = queue.erase(it);
            admitted++;
        } else {
            if (it == queue.begin() && !reserved && tnow - q->t_submit >= (double)cfg.head_wait_s) {
                /* reserve for the oldest request: the number of steps after
                 * which enough resident scenes have finished for it to fit */
                reserved = true;
                reserve_steps = steps_until_fits(q->desc.n_particles, b, pcap);
            }
            ++it;
        }
    }
    if (!layout_current()) {
        int r = relayout();
        if (r != FG_OK) return r;
    }
    float ms = 0.0f;
    uint64_t adv = 0;
    if (w && w->n) {
        /* a layout that just changed runs uncaptured; a stable one replays
         * its captured step */
        w->use_graphs = cfg.use_graphs && stable_steps >= 1;
        /* the slot about to be reused must hold a finished step */
        if (drain(FG_SERVER_RING - 1) != FG_OK) return FG_E_CUDA;
        const int k = (int)(issued % FG_SERVER_RING);
        slot_n[k] = w->n;
        CK(cudaEventRecord(ev0[k], w->stream));
        int r = w->step(1);
        if (r != FG_OK) return r;
        CK(cudaEventRecord(ev1[k], w->stream));
        issued++;
        const int depth = std::min(std::max(cfg.pipeline_depth, 0), FG_SERVER_RING - 1);
        if (drain((uint64_t)depth) != FG_OK) return FG_E_CUDA;
        ms = last_ms;
        adv = w->n;
    }
    for (auto *q : active) q->steps_done++;
    stable_steps++;
    steps++;
    particle_steps += adv;
    const uint32_t before = (uint32_t)active.size();
    int r = retire_finished();
    if (r != FG_OK) return r;
    if (info) {
        info->active_scenes = before;
        info->admitted = admitted;
        info->finished = before - (uint32_t)active.size();
        info->queued = (uint32_t)queue.size();
        info->active_particles = adv;
        info->step_ms = ms;
        info->wall_ms = 1e3 * (now() - tw0);
        info->resident_bytes = resident;
    }
    return FG_OK;
}

} // namespace fg

using namespace fg;

extern "C" {

void fg_server_config_defaults(fg_server_config *c)
{
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->hbm_budget_bytes = (size_t)120 << 30;
    c->use_graphs = 1;
    /* per-step work budget: at most 850k particles and a predicted 0.9 ms
     * per step; with backfilling this kept the C5 arrival workload's p99
     * step latency under 1.9 ms for every scene size (admitting by the HBM
     * budget alone: p99 210 ms) */
    c->max_particles = 1200000u;
    c->target_step_ms = 1.1f;
    c->head_wait_s = 0.0f;
}

int fg_server_create(const fg_server_config *cfg, fg_stream_t stream, fg_server **out)
{
    if (!cfg || !out) return FG_E_INVALID;
    *out = nullptr;
    std::unique_ptr<Server> s(new Server());
    s->cfg = *cfg;
    if (stream) {
        s->stream = (cudaStream_t)stream;
    } else {
        CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    for (int k = 0; k < FG_SERVER_RING; k++) {
        CK(cudaEventCreate(&s->ev0[k]));
        CK(cudaEventCreate(&s->ev1[k]));
    }
    *out = (fg_server *)s.release();
    return FG_OK;
}

void fg_server_destroy(fg_server *s) { delete (Server *)s; }

int fg_server_submit(fg_server *srv, const fg_scene_desc *d, uint32_t steps, uint64_t *request_id)
{
    if (!srv || !d || !steps) return FG_E_INVALID;
    Server *S = (Server *)srv;
    const int v = validate(*d);
    if (v != FG_OK) {
        set_error_msg("invalid scene description");
        return v;
    }
    std::unique_ptr<Request> q(new Request());
    q->desc = *d;
    const size_t n = d->n_particles;
    q->pos.assign(d->positions, d->positions + 4 * n);
    if (d->velocities) q->vel.assign(d->velocities, d->velocities + 4 * n);
    q->desc.positions = n ? q->pos.data() : nullptr;
    q->desc.velocities = d->velocities ? q->vel.data() : nullptr;
    q->bodies.assign(d->bodies, d->bodies + d->n_bodies);
    q->spheres.resize(d->n_bodies);
    for (uint32_t b = 0; b < d->n_bodies; b++) {
        const fg_body_desc &bd = d->bodies[b];
        q->spheres[b].assign(bd.local_spheres, bd.local_spheres + 4 * (size_t)bd.n_spheres);
        q->bodies[b].local_spheres = q->spheres[b].data();
    }
    q->desc.bodies = d->n_bodies ? q->bodies.data() : nullptr;
    const uint32_t lc = S->w ? S->w->list_cap_alloc : FG_SERVER_LIST_CAP;
    if (scene_bytes(q->desc, lc) > S->cfg.hbm_budget_bytes ||
        (S->cfg.max_particles && d->n_particles > S->cfg.max_particles)) {
        set_error_msg("scene alone exceeds the server budget");
        return FG_E_BUDGET;
    }
    q->id = S->next_id++;
    q->steps_total = steps;
    q->t_submit = S->now();
    if (request_id) *request_id = q->id;
    S->queue.push_back(q.get());
    S->all[q->id] = std::move(q);
    return FG_OK;
}

int fg_server_active(const fg_server *srv, uint64_t *ids, uint32_t cap, uint32_t *count)
{
    if (!srv || (cap && !ids)) return FG_E_INVALID;
    const Server *S = (const Server *)srv;
    const uint32_t n = (uint32_t)S->active.size();
    for (uint32_t k = 0; k < n && k < cap; k++) ids[k] = S->active[k]->id;
    if (count) *count = n;
    return FG_OK;
}

int fg_server_step(fg_server *srv, fg_server_step_info *info)
{
    if (!srv) return FG_E_INVALID;
    return ((Server *)srv)->step(info);
}

int fg_server_request(const fg_server *srv, uint64_t id, fg_request_info *info)
{
    if (!srv || !info) return FG_E_INVALID;
    const Server *S = (const Server *)srv;
    auto it = S->all.find(id);
    if (it == S->all.end()) return FG_E_INVALID;
    const Request &q = *it->second;
    info->state = q.state;
    info->steps_done = q.steps_done;
    info->steps_total = q.steps_total;
    info->n_particles = q.desc.n_particles;
    info->submit_s = q.t_submit;
    info->admit_s = q.t_admit;
    info->done_s = q.t_done;
    info->resident_bytes = q.bytes;
    return FG_OK;
}

int fg_server_result(fg_server *srv, uint64_t id, float *pos4, float *vel4, int release)
{
    if (!srv) return FG_E_INVALID;
    Server *S = (Server *)srv;
    auto it = S->all.find(id);
    if (it == S->all.end()) return FG_E_INVALID;
    Request &q = *it->second;
    if (q.state != FG_REQ_DONE) return FG_E_STATE;
    if (pos4 && !q.out_pos.empty()) memcpy(pos4, q.out_pos.data(), sizeof(float) * q.out_pos.size());
    if (vel4 && !q.out_vel.empty()) memcpy(vel4, q.out_vel.data(), sizeof(float) * q.out_vel.size());
    if (release) S->all.erase(it);
    return FG_OK;
}

int fg_server_stats(const fg_server *srv, fg_server_stats_info *st)
{
    if (!srv || !st) return FG_E_INVALID;
    const Server *S = (const Server *)srv;
    memset(st, 0, sizeof(*st));
    st->steps = S->steps;
    st->particle_steps = S->particle_steps;
    st->queued = (uint32_t)S->queue.size();
    st->active = (uint32_t)S->active.size();
    st->resident_bytes = S->resident;
    st->resident_particles = S->resident_particles;
    st->device_bytes = S->w ? S->w->device_bytes : 0;
    return FG_OK;
}

} // extern "C"
