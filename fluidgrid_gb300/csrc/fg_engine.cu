/* World engine: packed scenes, per-step orchestration, C ABI.
 *
 * Host side of the step.  Order per step (one launch per stage for all
 * scenes), following HeterogeneousSimulator::doTimeStep
 * (HeterogeneousSimulator.cpp:54-127) and the two-way rigid order of its
 * commented block with RigidBodySimulator (RigidBodySimulator.cpp:334-611):
 *   findFluidNeighbourhood  hash, sort, start/end + sorted gather (:131-150)
 *   calculateFluidDensity   (:153-159)
 *   generateCollisionData   sphere transform+hash, sort, ranges (:464-474)
 *   calculateRigidBodyForcesFromFluid (:503-520)
 *   calculateFluidForces(useDynamicRB) + integrateFluidForces (:161-212),
 *                           fused into one kernel
 *   applyForces + integrate (:522-611) as one FP64 kernel per body.
 * The per-stage device synchronisations of the reference are gone; stages
 * are stream-ordered and the whole step is replayed from a CUDA graph. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <stdio.h>
#include <math.h>
#include <algorithm>
#include <string>
#include <vector>
#include <mutex>
#include "fg_types.h"
#include "fg_kernels.h"
#include "fg_engine.h"
#include "fg_device.cuh"
#include "../../include/fluidgrid_gb300.h"

namespace fg {

/* One 32-bit device word set in stream order. */
__global__ void k_set_u32(uint32_t *p, uint32_t v) { *p = v; }

static thread_local std::string g_err;

void set_error(const char *what, cudaError_t e)
{
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    g_err = buf;
}

void set_error_msg(const char *what) { g_err = what; }

static uint32_t ceil_log2(uint64_t v)
{
    uint32_t b = 0;
    while ((1ull << b) < v) b++;
    return b;
}

static bool is_pow2(uint32_t v) { return v && !(v & (v - 1)); }

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            fg::set_error(#call, e_);                                                                  \
            return (e_ == cudaErrorMemoryAllocation) ? FG_E_OOM : FG_E_CUDA;                       \
        }                                                                                          \
    } while (0)

int World::alloc(void **p, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        set_error("cudaMalloc", e);
        *p = nullptr;
        return e == cudaErrorMemoryAllocation ? FG_E_OOM : FG_E_CUDA;
    }
    allocs.push_back(*p);
    device_bytes += bytes;
    return FG_OK;
}

World::~World()
{
    if (flush_buf) cudaFree(flush_buf);
    if (diag_first) cudaFree(diag_first);
    if (diag_part) cudaFree(diag_part);
    if (diag_out) cudaFree(diag_out);
    for (auto &e : tr.ev)
        if (e) cudaEventDestroy(e);
    drop_graphs();
    for (void *p : allocs) cudaFree(p);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_fluid_ready) cudaEventDestroy(ev_fluid_ready);
    if (ev_rb_done) cudaEventDestroy(ev_rb_done);
    if (ev_bodies_done) cudaEventDestroy(ev_bodies_done);
    if (ev_io_fork) cudaEventDestroy(ev_io_fork);
    if (ev_vel_in) cudaEventDestroy(ev_vel_in);
    if (ev_pos_in) cudaEventDestroy(ev_pos_in);
    if (stream2) cudaStreamDestroy(stream2);
    if (stream3) cudaStreamDestroy(stream3);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

void fill_scene(FgScene &S, const fg_scene_desc &d)
{
    memset(&S, 0, sizeof(S));
    for (int k = 0; k < 3; k++) S.cell[k] = d.cell_size[k];
    S.nb = (uint32_t)((int64_t)d.bucket_size[0] * d.bucket_size[1] * d.bucket_size[2]);
    S.nb_mask = is_pow2(S.nb) ? S.nb - 1 : 0;
    S.n = d.n_particles;
    S.h = d.kernel_radius;
    S.h2 = d.kernel_radius * d.kernel_radius;
    S.scale = d.simulation_scale;
    S.dt = d.dt;
    S.dt_over_scale = d.dt / d.simulation_scale;
    S.vlimit = d.velocity_limit;
    for (int k = 0; k < 3; k++) {
        S.vmin[k] = d.volume_min[k];
        S.vmax[k] = d.volume_max[k];
        S.gravity[k] = d.gravity[k];
        S.noslip_min[k] = d.noslip_min[k];
        S.noslip_max[k] = d.noslip_max[k];
    }
    S.mass = d.mass;
    S.rest = d.rest_density;
    S.gas = d.gas_constant;
    S.visc = d.viscosity;
    /* KernelsCache, HeterogeneousSimulator.cpp:33-42 (double pow, float store) */
    const float PI = 3.14159265f;
    double h = (double)d.kernel_radius;
    S.kpoly6 = (float)(315.0f / ((double)(64.0f * PI) * pow(h, 9)));
    S.kspiky = (float)(-(45.0f / ((double)PI * pow(h, 6))));
    S.kvisc = (float)(45.0f / ((double)PI * pow(h, 6)));
    S.wall_dist = d.wall_distance;
    S.wall_stiff = d.wall_stiffness;
    S.wall_damp = d.wall_damping;
    S.fric_kin = d.friction_kinetic;
    S.fric_static = d.friction_static;
    S.nbodies = d.n_bodies;
    S.rb_nb = (uint32_t)((int64_t)d.rb_bucket_size[0] * d.rb_bucket_size[1] * d.rb_bucket_size[2]);
    S.rb_nb_mask = is_pow2(S.rb_nb) ? S.rb_nb - 1 : 0;
    for (int k = 0; k < 3; k++) {
        S.rb_cell[k] = d.rb_radius;
        S.f2r_rel[k] = d.fluid_to_rb_relation[k];
        S.r2f_rel[k] = d.rb_to_fluid_relation[k];
        S.rb_vmin[k] = d.rb_volume_min[k];
        S.rb_vmax[k] = d.rb_volume_max[k];
    }
    S.fluid_radius = d.fluid_radius;
    S.rb_radius = d.rb_radius;
    S.ck = d.contact_kspring;
    S.ckd = d.contact_kdamping;
    S.fluid_eps = d.fluid_contact_eps;
    S.rb_eps = d.rb_contact_eps;
    S.rbrb_k = d.rbrb_kspring;
    S.rbrb_kd = d.rbrb_kdamping;
    S.rbrb_eps = d.rbrb_eps;
    for (int k = 0; k < 4; k++) S.rb_gravity[k] = d.rb_gravity[k];
    S.rb_vlimit = d.rb_velocity_limit;
    S.rb_dt = d.rb_dt;
    S.flags = 0;
    if (d.n_bodies) S.flags |= FG_SCENE_HAS_RB;
    if (d.rb_rb_contact) S.flags |= FG_SCENE_RB_RB;
}

int validate(const fg_scene_desc &d)
{
    if (d.n_particles && !d.positions) return FG_E_INVALID;
    for (int k = 0; k < 3; k++) {
        if (d.bucket_size[k] <= 0) return FG_E_INVALID;
        if (!(d.cell_size[k] > 0.0f)) return FG_E_INVALID;
    }
    int64_t nb = (int64_t)d.bucket_size[0] * d.bucket_size[1] * d.bucket_size[2];
    if (nb > 0x7fffffffLL) return FG_E_INVALID;
    if (!(d.kernel_radius > 0.0f) || !(d.simulation_scale != 0.0f)) return FG_E_INVALID;
    if (d.n_bodies) {
        if (!d.bodies) return FG_E_INVALID;
        for (int k = 0; k < 3; k++)
            if (d.rb_bucket_size[k] <= 0 || d.fluid_to_rb_relation[k] < 0 || d.rb_to_fluid_relation[k] < 0 ||
                d.fluid_to_rb_relation[k] > 8 || d.rb_to_fluid_relation[k] > 8)
                return FG_E_INVALID;
        if (!(d.rb_radius > 0.0f)) return FG_E_INVALID;
        int64_t rnb = (int64_t)d.rb_bucket_size[0] * d.rb_bucket_size[1] * d.rb_bucket_size[2];
        if (rnb > 0x7fffffffLL) return FG_E_INVALID;
        for (uint32_t b = 0; b < d.n_bodies; b++) {
            if (d.bodies[b].n_spheres && !d.bodies[b].local_spheres) return FG_E_INVALID;
            if (!(d.bodies[b].mass >= 0.0f)) return FG_E_INVALID; /* 0 = static body */
        }
    }
    return FG_OK;
}

static void build_work(std::vector<FgWork> &wt, uint32_t scene, uint32_t first, uint32_t n)
{
    for (uint32_t o = 0; o < n; o += FG_CHUNK) {
        FgWork w;
        w.scene = scene;
        w.first = first + o;
        w.count = std::min<uint32_t>(FG_CHUNK, n - o);
        w.pad = 0;
        wt.push_back(w);
    }
}

/* Element counts a set of scenes needs. */
Capacity World::needs(const fg_scene_desc *d, uint32_t ns)
{
    Capacity c;
    c.scenes = ns;
    for (uint32_t s = 0; s < ns; s++) {
        const uint64_t nb = (uint64_t)d[s].bucket_size[0] * d[s].bucket_size[1] * d[s].bucket_size[2];
        uint64_t sph = 0;
        for (uint32_t b = 0; b < d[s].n_bodies; b++) sph += d[s].bodies[b].n_spheres;
        c.particles += d[s].n_particles;
        c.buckets += nb;
        c.spheres += sph;
        c.bodies += d[s].n_bodies;
        if (d[s].n_bodies)
            c.rb_buckets += (uint64_t)d[s].rb_bucket_size[0] * d[s].rb_bucket_size[1] * d[s].rb_bucket_size[2];
        c.work += (d[s].n_particles + FG_CHUNK - 1) / FG_CHUNK;
        c.work_sph += (sph + FG_CHUNK - 1) / FG_CHUNK;
    }
    return c;
}

bool Capacity::fits(const Capacity &o) const
{
    return o.particles <= particles && o.buckets <= buckets && o.spheres <= spheres && o.bodies <= bodies &&
           o.rb_buckets <= rb_buckets && o.scenes <= scenes && o.work <= work && o.work_sph <= work_sph;
}

bool Capacity::too_large() const
{
    return particles >= 0x7fffffffULL || buckets >= 0x7fffffffULL || spheres >= 0x7fffffffULL ||
           rb_buckets >= 0x7fffffffULL;
}

/* Device bytes reserve(c) allocates (list capacity `list_cap` slots). */
size_t World::footprint(const Capacity &c, uint32_t list_cap)
{
    const size_t P = std::max<uint64_t>(c.particles, 1), S = std::max<uint64_t>(c.spheres, 1);
    const size_t M = std::max(P, S);
    size_t b = 0;
    b += P * (16 + 16 + 4 + 4 + 4 + 16 + 16 + 8); /* pos vel keys_u keys ids spos svel dp */
    b += M * 8 + 4 * radix_hist_words((uint32_t)M) + 4 * onesweep_words((uint32_t)P); /* sort scratch */
    b += P * (4 * (size_t)list_cap + 4 + 32);      /* lists, counts, records */
    b += P * 12;                                    /* runs, inv, tord */
    b += 8 * std::max<uint64_t>(c.buckets, 1);
    b += (sizeof(FgScene) + 24) * std::max<uint64_t>(c.scenes, 1);
    b += sizeof(FgWork) * (std::max<uint64_t>(c.work, 1) + std::max<uint64_t>(c.work_sph, 1));
    if (c.bodies) {
        b += P * 16; /* the fluid side of the contact */
        b += S * (16 * 6 + 12);
        b += 8 * std::max<uint64_t>(c.rb_buckets, 1);
        b += c.bodies * (32 * 6 + 16 * 3 + 8 + 72 + 12 + 8 * 8 * FG_BODY_CHUNKS);
    }
    return b;
}

/* Allocate every buffer for capacity c (once per World). */
int World::reserve(const Capacity &c)
{
    cap = c;
    int r;
    auto A = [&](void **p, size_t b) { return alloc(p, b); };
    const size_t Sc = std::max<uint64_t>(c.scenes, 1);
    if ((r = A((void **)&scenes_d, sizeof(FgScene) * Sc))) return r;
    if ((r = A((void **)&work_d, sizeof(FgWork) * std::max<uint64_t>(c.work, 1)))) return r;
    if ((r = A((void **)&work_sph_d, sizeof(FgWork) * std::max<uint64_t>(c.work_sph, 1)))) return r;
    const size_t N = std::max<uint64_t>(c.particles, 1);
    const size_t NB = std::max<uint64_t>(c.buckets, 1);
    if ((r = A((void **)&pos, 16 * N))) return r;
    if ((r = A((void **)&vel, 16 * N))) return r;
    if ((r = A((void **)&keys_u, 4 * N))) return r;
    if ((r = A((void **)&keys, 4 * N))) return r;
    if ((r = A((void **)&ids, 4 * N))) return r;
    if ((r = A((void **)&spos, 16 * N))) return r;
    if ((r = A((void **)&svel, 16 * N))) return r;
    if ((r = A((void **)&dp, 8 * N))) return r;
    if ((r = A((void **)&start, 4 * NB))) return r;
    if ((r = A((void **)&end, 4 * NB))) return r;
    const size_t M = std::max(N, (size_t)std::max<uint64_t>(c.spheres, 1));
    if ((r = A((void **)&rs.keys_alt, 4 * M))) return r;
    if ((r = A((void **)&rs.vals_alt, 4 * M))) return r;
    if ((r = A((void **)&rs.hist, 4 * radix_hist_words((uint32_t)M)))) return r;
    if ((r = A((void **)&os_scratch, 4 * onesweep_words((uint32_t)N)))) return r;
    if (!list_cap_alloc) list_cap_alloc = FG_LIST_CAP_DEFAULT;
    if ((r = A((void **)&nbr.idx, 4 * (size_t)list_cap_alloc * N))) return r;
    nbr.stride = list_cap_alloc;
    list_cap = list_cap_alloc;
    if ((r = A((void **)&nbr.cnt, 4 * N))) return r;
    if ((r = A((void **)&nbr.rec, 32 * N))) return r;
    if ((r = A((void **)&runs, 4 * N))) return r;
    if ((r = A((void **)&nruns, 16))) return r;
    if ((r = A((void **)&inv, 4 * N))) return r;
    if ((r = A((void **)&tord, 4 * N))) return r;
    if ((r = A((void **)&status_d, 64))) return r;
    CK(cudaMemsetAsync(status_d, 0, 64, stream));
    pair_counter = (unsigned long long *)(status_d + 8); /* 8-byte aligned slots of the status block */
    overflow_counter = (unsigned long long *)(status_d + 10);
    max_count = status_d + 12;
    list_cap_d = status_d + 13;
    nbr.cap = list_cap_d;
    k_set_u32<<<1, 1, 0, stream>>>(list_cap_d, list_cap);
    nbr.max_count = max_count;
    nbr.overflow = overflow_counter;
    CK(cudaMemsetAsync(dp, 0, 8 * N, stream));
    CK(cudaMemsetAsync(vel, 0, 16 * N, stream));
    CK(cudaMemsetAsync(end, 0, 4 * NB, stream));
    /* lists read before any density pass (stage-split calls) see zero
     * counts and in-range indices */
    CK(cudaMemsetAsync(nbr.cnt, 0, 4 * N, stream));
    CK(cudaMemsetAsync(nbr.idx, 0, 4 * (size_t)list_cap_alloc * N, stream));
    CK(cudaMemsetAsync(nbr.rec, 0, 32 * N, stream));
    if ((r = A((void **)&aabb, 24 * Sc))) return r;
    if (c.bodies) {
        const size_t S = std::max<uint64_t>(c.spheres, 1), B = c.bodies;
        const size_t RB = std::max<uint64_t>(c.rb_buckets, 1);
        if ((r = A((void **)&fcontact, 16 * N))) return r;
        if ((r = A((void **)&rb_local, 16 * S))) return r;
        if ((r = A((void **)&rb_world, 16 * S))) return r;
        if ((r = A((void **)&rb_keys_u, 4 * S))) return r;
        if ((r = A((void **)&rb_keys, 4 * S))) return r;
        if ((r = A((void **)&rb_ids, 4 * S))) return r;
        if ((r = A((void **)&rb_spos, 16 * S))) return r;
        if ((r = A((void **)&rb_force, 16 * S))) return r;
        if ((r = A((void **)&rb_torque, 16 * S))) return r;
        if ((r = A((void **)&rb_start, 4 * RB))) return r;
        if ((r = A((void **)&rb_end, 4 * RB))) return r;
        if ((r = A((void **)&bx, 32 * B))) return r;
        if ((r = A((void **)&bv, 32 * B))) return r;
        if ((r = A((void **)&bq, 32 * B))) return r;
        if ((r = A((void **)&bL, 32 * B))) return r;
        if ((r = A((void **)&bfs, 32 * B))) return r;
        if ((r = A((void **)&body_part, 8 * 8 * FG_BODY_CHUNKS * B))) return r;
        if ((r = A((void **)&bts, 32 * B))) return r;
        if ((r = A((void **)&bxf, 16 * B))) return r;
        if ((r = A((void **)&bvf, 16 * B))) return r;
        if ((r = A((void **)&bvf_next, 16 * B))) return r;
        if ((r = A((void **)&bqf, 16 * B))) return r;
        if ((r = A((void **)&bmass, 8 * B))) return r;
        if ((r = A((void **)&binv, 72 * B))) return r;
        if ((r = A((void **)&body_scene, 4 * B))) return r;
        if ((r = A((void **)&body_first, 4 * B))) return r;
        if ((r = A((void **)&body_count, 4 * B))) return r;
        CK(cudaMemsetAsync(rb_end, 0, 4 * RB, stream));
        CK(cudaMemsetAsync(bfs, 0, 32 * B, stream));
        CK(cudaMemsetAsync(bts, 0, 32 * B, stream));
    }
    return FG_OK;
}

/* Scene table, work tables and the static per-body and per-sphere data of
 * the scenes d[0..ns) (which must fit the capacity).  Dynamic state --
 * particle positions, velocities, densities and the bodies' motion -- is not
 * touched: upload_scene or a migration fills it. */
int World::set_layout(const fg_scene_desc *d, uint32_t ns)
{
    const Capacity need = needs(d, ns);
    if (need.too_large()) {
        set_error_msg("world too large");
        return FG_E_INVALID;
    }
    if (!cap.fits(need) || (need.bodies && !rb_local)) {
        set_error_msg("scenes exceed the world's capacity");
        return FG_E_BUDGET;
    }
    /* steps in flight read the tables rewritten below */
    CK(cudaStreamSynchronize(stream));
    nscenes = ns;
    scenes_h.assign(std::max<uint32_t>(ns, 1), FgScene{});
    uint64_t np = 0, nbk = 0, nsph = 0, nbod = 0, nrbk = 0;
    any_rb_rb = false;
    for (uint32_t s = 0; s < ns; s++) {
        FgScene &S = scenes_h[s];
        fill_scene(S, d[s]);
        S.pbase = (uint32_t)np;
        S.bucket_base = (uint32_t)nbk;
        S.sph_base = (uint32_t)nsph;
        S.body_base = (uint32_t)nbod;
        S.rb_bucket_base = (uint32_t)nrbk;
        uint64_t sph = 0;
        for (uint32_t b = 0; b < d[s].n_bodies; b++) sph += d[s].bodies[b].n_spheres;
        S.nsph = (uint32_t)sph;
        np += d[s].n_particles;
        nbk += S.nb;
        nsph += sph;
        nbod += d[s].n_bodies;
        if (d[s].n_bodies) nrbk += S.rb_nb;
        if (d[s].n_bodies && d[s].rb_rb_contact) any_rb_rb = true;
    }
    n = (uint32_t)np;
    rb_small_scenes = true;
    for (uint32_t s = 0; s < ns; s++)
        if (scenes_h[s].nsph > FG_RB_SCENE_MAX) rb_small_scenes = false;
    total_buckets = (uint32_t)nbk;
    /* the counting sort's work grows with the buckets, the radix sort's
     * with the particles and passes */
    if (!sort_chosen)
        set_sort_variant((total_buckets <= (uint64_t)FG_BUCKET_SORT_RATIO * std::max<uint32_t>(n, 1u) &&
                          bucket_sort_fits())
                             ? 2
                             : (one_pass_sort ? 1 : 0));
    nspheres = (uint32_t)nsph;
    nbodies = (uint32_t)nbod;
    total_rb_buckets = (uint32_t)nrbk;
    const uint32_t old_key_bits = key_bits;
    key_bits = ceil_log2(total_buckets);
    rb_key_bits = ceil_log2(std::max<uint32_t>(total_rb_buckets, 1));
    if (!digit_bits || key_bits != old_key_bits) {
        digit_bits = key_bits <= 16 ? std::max<uint32_t>(1, (key_bits + 1) / 2) : (key_bits + 2) / 3;
        if (digit_bits > 8) digit_bits = 8;
    }
    std::vector<FgWork> fw, sw;
    work_first_h.assign(ns + 1, 0);
    for (uint32_t s = 0; s < ns; s++) {
        work_first_h[s] = (uint32_t)fw.size();
        build_work(fw, s, scenes_h[s].pbase, scenes_h[s].n);
        build_work(sw, s, scenes_h[s].sph_base, scenes_h[s].nsph);
    }
    work_first_h[ns] = (uint32_t)fw.size();
    nwork = (uint32_t)fw.size();
    nwork_sph = (uint32_t)sw.size();
    single = (ns == 1);
    {
        const uint32_t sbits = ceil_log2(std::max<uint32_t>(ns, 1));
        order_bits = std::min<uint32_t>(10u, (32u - sbits) / 3u);
        order_scene_shift = 3u * order_bits;
        order_key_bits = order_scene_shift + sbits;
    }
    order_valid = false;
    if (ns) CK(cudaMemcpyAsync(scenes_d, scenes_h.data(), sizeof(FgScene) * ns, cudaMemcpyHostToDevice, stream));
    if (nwork) CK(cudaMemcpyAsync(work_d, fw.data(), sizeof(FgWork) * nwork, cudaMemcpyHostToDevice, stream));
    if (nwork_sph)
        CK(cudaMemcpyAsync(work_sph_d, sw.data(), sizeof(FgWork) * nwork_sph, cudaMemcpyHostToDevice, stream));
    if (nbodies) {
        const size_t S = nspheres, B = nbodies;
        std::vector<float> local(4 * std::max<size_t>(S, 1), 0.0f);
        std::vector<double> hm(B), hinv(9 * B);
        std::vector<uint32_t> hbs(B), hbf(B), hbc(B);
        uint32_t gb = 0, gs = 0;
        for (uint32_t s = 0; s < ns; s++)
            for (uint32_t b = 0; b < d[s].n_bodies; b++, gb++) {
                const fg_body_desc &bd = d[s].bodies[b];
                hbs[gb] = s;
                hbf[gb] = gs;
                hbc[gb] = bd.n_spheres;
                for (uint32_t k = 0; k < bd.n_spheres; k++, gs++) {
                    local[4 * gs + 0] = bd.local_spheres[4 * k + 0];
                    local[4 * gs + 1] = bd.local_spheres[4 * k + 1];
                    local[4 * gs + 2] = bd.local_spheres[4 * k + 2];
                    local[4 * gs + 3] = (float)gb; /* w = global body index */
                }
                hm[gb] = bd.mass;
                for (int c = 0; c < 9; c++) hinv[9 * gb + c] = bd.inv_inertia[c];
            }
        if (S) CK(cudaMemcpy(rb_local, local.data(), 16 * S, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(bmass, hm.data(), 8 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(binv, hinv.data(), 72 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(body_scene, hbs.data(), 4 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(body_first, hbf.data(), 4 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(body_count, hbc.data(), 4 * B, cudaMemcpyHostToDevice));
    }
    stale_graphs();
    return FG_OK;
}

/* Initial dynamic state of scene s from its description: positions,
 * velocities (zero if none) and the bodies at rest at their poses. */
int World::upload_scene(uint32_t s, const fg_scene_desc &d)
{
    const FgScene &S = scenes_h[s];
    if (S.n) {
        CK(cudaMemcpyAsync(pos + S.pbase, d.positions, 16 * (size_t)S.n, cudaMemcpyHostToDevice, stream));
        if (d.velocities)
            CK(cudaMemcpyAsync(vel + S.pbase, d.velocities, 16 * (size_t)S.n, cudaMemcpyHostToDevice, stream));
        else
            CK(cudaMemsetAsync(vel + S.pbase, 0, 16 * (size_t)S.n, stream));
        CK(cudaMemsetAsync(dp + S.pbase, 0, 8 * (size_t)S.n, stream));
    }
    if (S.nbodies) {
        const size_t B = S.nbodies;
        std::vector<double> hx(4 * B), hv(4 * B, 0.0), hq(4 * B), hL(4 * B, 0.0);
        std::vector<float> hxf(4 * B), hvf(4 * B, 0.0f), hqf(4 * B);
        for (uint32_t b = 0; b < S.nbodies; b++) {
            const fg_body_desc &bd = d.bodies[b];
            for (int c = 0; c < 3; c++) hx[4 * b + c] = bd.position[c];
            hx[4 * b + 3] = 0.0;
            for (int c = 0; c < 4; c++) hq[4 * b + c] = bd.orientation[c];
            for (int c = 0; c < 4; c++) {
                hxf[4 * b + c] = (float)hx[4 * b + c];
                hqf[4 * b + c] = (float)hq[4 * b + c];
            }
        }
        const size_t o = S.body_base;
        CK(cudaMemcpy(bx + o, hx.data(), 32 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(bv + o, hv.data(), 32 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(bq + o, hq.data(), 32 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(bL + o, hL.data(), 32 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(bxf + o, hxf.data(), 16 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(bvf + o, hvf.data(), 16 * B, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(bqf + o, hqf.data(), 16 * B, cudaMemcpyHostToDevice));
    }
    return FG_OK;
}

void World::drop_graphs()
{
    for (auto *v : {&graphs, &stale}) {
        for (auto &g : *v) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            if (g.graph) cudaGraphDestroy(g.graph);
        }
        v->clear();
    }
}

void World::stale_graphs()
{
    for (auto &g : graphs) stale.push_back(g);
    graphs.clear();
    /* bound the kept set: the oldest go first */
    while (stale.size() > 32) {
        if (stale.front().exec) cudaGraphExecDestroy(stale.front().exec);
        if (stale.front().graph) cudaGraphDestroy(stale.front().graph);
        stale.erase(stale.begin());
    }
}

int World::init_stream(cudaStream_t st)
{
    (void)sm_count(); /* cache the device query outside any graph capture */
    if (st) {
        stream = st;
        own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
    }
    CK(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_fluid_ready, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_rb_done, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_bodies_done, cudaEventDisableTiming));
    CK(cudaStreamCreateWithFlags(&stream3, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev_io_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_vel_in, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_pos_in, cudaEventDisableTiming));
    return FG_OK;
}

int World::create(const fg_scene_desc *d, uint32_t ns, cudaStream_t st)
{
    int r = init_stream(st);
    if (r != FG_OK) return r;
    for (uint32_t s = 0; s < ns; s++) {
        const int v = validate(d[s]);
        if (v != FG_OK) {
            set_error_msg("invalid scene description");
            return v;
        }
    }
    const Capacity c = needs(d, ns);
    if (c.too_large()) {
        set_error_msg("world too large");
        return FG_E_INVALID;
    }
    if ((r = reserve(c)) != FG_OK) return r;
    if ((r = set_layout(d, ns)) != FG_OK) return r;
    for (uint32_t s = 0; s < ns; s++)
        if ((r = upload_scene(s, d[s])) != FG_OK) return r;
    CK(cudaStreamSynchronize(stream));
    return FG_OK;
}

Launch World::fluid_launch() const
{
    Launch L{};
    L.table = single ? nullptr : scenes_d;
    L.single = &scenes_h[0];
    L.work = single ? nullptr : work_d;
    L.nwork = nwork;
    L.n = n;
    L.stream = stream;
    L.ctas_per_sm = ctas_per_sm;
    L.block = block;
    return L;
}

Launch World::sphere_launch() const
{
    Launch L{};
    L.table = single ? nullptr : scenes_d;
    L.single = &scenes_h[0];
    L.work = single ? nullptr : work_sph_d;
    L.nwork = nwork_sph;
    L.n = nspheres;
    L.stream = stream;
    L.ctas_per_sm = 0;
    return L;
}

/* Ordered-int AABB reset: mins to +big, maxes to -big. */
__global__ void k_aabb_reset(int *aabb, uint32_t ns)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * ns) aabb[i] = (i % 6) < 3 ? fg_float_ord(3.0e38f) : fg_float_ord(-3.0e38f);
}

/* Rigid-sphere grid of every scene: AABB, world positions and keys, sort,
 * start/end (the stage bit FG_STAGE_RB_GRID). */
void World::enqueue_rb_grid(cudaStream_t st, cudaEvent_t *ev, uint32_t &launches)
{
    if (!(stages & FG_STAGE_RB_GRID)) return;
    if (ev) cudaEventRecord(ev[8], st);
    Launch Ls = sphere_launch();
    Ls.stream = st;
    k_aabb_reset<<<(6 * nscenes + 127) / 128, 128, 0, st>>>(aabb, nscenes);
    launch_hash_with_offset(Ls, rb_local, bxf, bqf, rb_world, rb_keys_u, nullptr, aabb);
    if (rb_small_scenes) {
        launch_rb_sort_ranges(single ? nullptr : scenes_d, &scenes_h[0], nscenes, rb_keys_u, rb_world, rb_keys,
                              rb_ids, rb_spos, rb_start, rb_end, st);
        launches += 3;
    } else {
        radix_sort(rb_keys_u, nullptr, rb_keys, rb_ids, nspheres, rb_key_bits, 8, rs, st);
        cudaMemsetAsync(rb_start, 0xff, 4 * (size_t)total_rb_buckets, st);
        launch_cell_ranges(rb_keys, rb_ids, rb_world, nullptr, rb_start, rb_end, rb_spos, nullptr, nspheres, st);
        launches += 3 + 3 * radix_passes(rb_key_bits, 8);
    }
    if (ev) cudaEventRecord(ev[9], st);
}

/* Sphere forces and torques from the fluid (and from other bodies) (the
 * stage bit FG_STAGE_RB_CONTACT). */
/* The bodies' rigid-sphere grid as the fluid side of the contact reads it. */
RigidGrid World::body_grid() const
{
    RigidGrid G;
    memset(&G, 0, sizeof(G));
    G.spos = rb_spos;
    G.start = rb_start;
    G.end = rb_end;
    G.body_vel = bvf;
    G.aabb = aabb;
    return G;
}

/* Whether a whole step computes the fluid side of the contact in its own
 * pass (with the sphere side, beside the density pass) for the force pass to
 * read; kernel 2's force pass walks the rigid grid itself. */
bool World::fluid_contact_pass() const
{
    return nbodies > 0 && fcontact && !use_cc && (stages & FG_STAGE_RB_CONTACT);
}

void World::enqueue_rb_contact(cudaStream_t st, cudaEvent_t *ev, uint32_t &launches, bool with_fluid)
{
    if (!(stages & FG_STAGE_RB_CONTACT)) return;
    if (ev) cudaEventRecord(ev[10], st);
    Launch Ls = sphere_launch();
    Ls.stream = st;
    launch_rb_from_fluid(Ls, rb_spos, rb_ids, bvf, bxf, spos, svel, start, end, rb_force, rb_torque, 0);
    launches++;
    if (any_rb_rb) {
        launch_rb_from_rb(Ls, rb_spos, rb_ids, bvf, bxf, rb_start, rb_end, rb_force, rb_torque, nullptr, 1);
        launches++;
    }
    if (with_fluid) enqueue_fluid_contact(st, launches);
    if (ev) cudaEventRecord(ev[11], st);
}

/* The fluid side of the contact (by particle id, from the step's unsorted
 * state and the bodies' sphere grid) for the force pass to read. */
void World::enqueue_fluid_contact(cudaStream_t st, uint32_t &launches)
{
    if (!fluid_contact_pass()) return;
    Launch Lf = fluid_launch();
    Lf.stream = st;
    launch_fluid_contact(Lf, pos, vel, body_grid(), fcontact);
    launches++;
}

#define CK0(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) set_error(#call, e_);                                               \
    } while (0)

/* Per-body FP64 force/torque sums and the integration (the stage bit
 * FG_STAGE_BODIES); the FP32 velocity mirror goes to vf. */
void World::enqueue_bodies(cudaStream_t st, float4 *vf)
{
    BodyState b;
    b.x = bx; b.v = bv; b.q = bq; b.L = bL;
    b.inv_inertia = binv;
    b.mass = bmass;
    b.x_f = bxf; b.v_f = vf; b.q_f = bqf;
    b.force_sum = bfs; b.torque_sum = bts;
    b.partial = body_part;
    launch_body_update(single ? nullptr : scenes_d, &scenes_h[0], body_scene, body_first, body_count, nbodies,
                       rb_force, rb_torque, b, 1, st);
}

/* The fluid sort of the variant in use: keys_u -> keys, ids (and, for the
 * counting sort, start/end). */
uint32_t World::sort_launches() const
{
    /* the fused reorder included; the count runs in the hash pass when the
     * step hashes too */
    if (bucket_sort_on && bucket_sort_fits()) return n ? ((stages & FG_STAGE_HASH) ? 4u : 5u) : 2u;
    const uint32_t P = (uint32_t)radix_passes(key_bits, digit_bits);
    return (one_pass_sort && n && P <= 6) ? 2 + P : 3 * P;
}

/* The hash pass; when the counting sort follows, it counts the keys too. */
void World::enqueue_hash(const Launch &L, bool sort_follows)
{
    counted_in_hash = sort_follows && bucket_sort_on && bucket_sort_fits();
    if (counted_in_hash) {
        cudaMemsetAsync(end, 0, 4 * (size_t)total_buckets, stream);
        launch_hash(L, pos, keys_u, nullptr, end, rs.keys_alt);
    } else {
        launch_hash(L, pos, keys_u, nullptr);
    }
}

void World::enqueue_sort(bool with_ranges)
{
    /* with_ranges: the step's ranges pass follows directly; the counting
     * sort then does its reorder too (fused_ranges) */
    BucketReorder R{pos, vel, spos, svel, inv, needs_runs() ? runs : nullptr, nruns};
    if (bucket_sort_on && with_ranges && needs_runs()) cudaMemsetAsync(nruns, 0, 4, stream);
    const bool counted = counted_in_hash;
    counted_in_hash = false;
    if (bucket_sort_on &&
        bucket_sort(keys_u, keys, ids, n, total_buckets, start, end, rs,
                    (uint32_t)std::min<size_t>(radix_hist_words((uint32_t)std::max<uint64_t>(cap.particles, 1)),
                                               0xffffffffu),
                    stream, with_ranges ? &R : nullptr, counted)) {
        counted_ranges = true;
        fused_ranges = with_ranges;
        return;
    }
    if (one_pass_sort && onesweep_sort(keys_u, keys, ids, n, key_bits, digit_bits, rs, os_scratch, status_d, stream))
        return;
    radix_sort(keys_u, nullptr, keys, ids, n, key_bits, digit_bits, rs, stream);
}

uint32_t World::enqueue_step(cudaEvent_t *ev)
{
    /* ev: optional 16 events, (2k, 2k+1) bracket stage bit k */
    auto mark = [&](int k, int end_) {
        if (ev) cudaEventRecord(ev[2 * k + end_], stream);
    };
    uint32_t launches = 0;
    const Launch L = fluid_launch();
    const bool rb = nbodies > 0;
    /* the rigid-sphere grid needs only the previous step's body poses and the
     * fluid/sphere contact only the fluid grid: in a full step they run on a
     * second stream beside the fluid sort and density pass and join before
     * the force pass (parallel branches of the captured graph) */
    const uint32_t full = FG_STAGE_HASH | FG_STAGE_SORT | FG_STAGE_RANGES | FG_STAGE_RB_GRID | FG_STAGE_RB_CONTACT;
    const bool fork = rb && !ev && rb_small_scenes && stream2 && (stages & full) == full;
    if (fork) {
        CK0(cudaEventRecord(ev_fork, stream));
        CK0(cudaStreamWaitEvent(stream2, ev_fork, 0));
        enqueue_rb_grid(stream2, nullptr, launches);
    }
    /* end-to-end step: the velocities upload on a third stream while the
     * positions upload and the hash and sort run; the reorder waits for them */
    const size_t iob = 16 * (size_t)n;
    if (cur_io && iob) {
        CK0(cudaEventRecord(ev_io_fork, stream));
        CK0(cudaStreamWaitEvent(stream3, ev_io_fork, 0));
        /* the previous step's velocities go down while this step's
         * positions come up (the link carries both directions at once) */
        if (cur_io->prev_vel) CK0(cudaMemcpyAsync(cur_io->ov, vel, iob, cudaMemcpyDeviceToHost, stream3));
        CK0(cudaMemcpyAsync(vel, cur_io->hv, iob, cudaMemcpyHostToDevice, stream3));
        CK0(cudaEventRecord(ev_vel_in, stream3));
        CK0(cudaMemcpyAsync(pos, cur_io->hp, iob, cudaMemcpyHostToDevice, stream));
    }
    if (fork) {
        /* the fluid side of the contact follows the sphere grid on the second
         * stream, beside the hash and sort; an end-to-end step's pass waits
         * for the state's upload */
        if (cur_io && iob && fluid_contact_pass()) {
            CK0(cudaEventRecord(ev_pos_in, stream));
            CK0(cudaStreamWaitEvent(stream2, ev_pos_in, 0));
            CK0(cudaStreamWaitEvent(stream2, ev_vel_in, 0));
        }
        enqueue_fluid_contact(stream2, launches);
    }
    counted_in_hash = false;
    if (stages & FG_STAGE_HASH) {
        mark(0, 0);
        enqueue_hash(L, (stages & FG_STAGE_SORT) != 0);
        mark(0, 1);
        launches++;
    }
    counted_ranges = fused_ranges = false;
    if (stages & FG_STAGE_SORT) {
        mark(1, 0);
        /* an end-to-end step's ranges wait for the velocity upload: no fused reorder */
        enqueue_sort((stages & FG_STAGE_RANGES) && !(cur_io && iob));
        launches += sort_launches();
        mark(1, 1);
    }
    if (cur_io && iob) CK0(cudaStreamWaitEvent(stream, ev_vel_in, 0));
    if (stages & FG_STAGE_RANGES) {
        mark(2, 0);
        if (!fused_ranges) {
            /* the counting sort wrote start[] of every bucket already */
            if (!counted_ranges) cudaMemsetAsync(start, 0xff, 4 * (size_t)total_buckets, stream);
            if (needs_runs()) {
                cudaMemsetAsync(nruns, 0, 4, stream);
                launch_cell_ranges(keys, ids, pos, vel, start, end, spos, svel, n, stream, inv, runs, nruns);
            } else {
                launch_cell_ranges(keys, ids, pos, vel, start, end, spos, svel, n, stream, inv);
            }
            launches += 1;
        }
        mark(2, 1);
    }
    /* with a full step forked, the body reduction and integration follow the
     * contact on the second stream and overlap the force pass, which reads
     * only the spheres' grid and the bodies' old velocities (kept in bvf
     * until the step's end) */
    const bool fork_bodies = fork && (stages & (FG_STAGE_FORCES | FG_STAGE_BODIES)) ==
                                         (FG_STAGE_FORCES | FG_STAGE_BODIES);
    if (fork) {
        CK0(cudaEventRecord(ev_fluid_ready, stream));
        CK0(cudaStreamWaitEvent(stream2, ev_fluid_ready, 0));
        enqueue_rb_contact(stream2, nullptr, launches, false);
        CK0(cudaEventRecord(ev_rb_done, stream2));
        if (fork_bodies) {
            enqueue_bodies(stream2, bvf_next);
            launches += body_launches();
            CK0(cudaEventRecord(ev_bodies_done, stream2));
        }
    }
    if (stages & FG_STAGE_DENSITY) {
        mark(3, 0);
        if (use_cc)
            launch_density_cc(single ? nullptr : scenes_d, &scenes_h[0], nscenes, runs, nruns, keys, spos, svel, start,
                              end, dp, nbr.rec, n, stream, cc_warps);
        else
            launch_density(L, spos, start, end, dp, 0.f, 0.f, 0.f, 0, svel, use_list ? &nbr : nullptr,
                           density_order(), pair_counter);
        mark(3, 1);
        launches++;
    }
    if (rb && !fork) {
        enqueue_rb_grid(stream, ev, launches);
        enqueue_rb_contact(stream, ev, launches, true);
    }
    if (fork) CK0(cudaStreamWaitEvent(stream, ev_rb_done, 0));
    if (stages & FG_STAGE_FORCES) {
        mark(6, 0);
        RigidGrid G = body_grid();
        /* the fluid side of the contact ran as its own pass (enqueue_fluid_contact) */
        if (fluid_contact_pass()) G.pre = fcontact;
        ForceOut o;
        o.vel = vel;
        o.pos = fused_integrate ? pos : nullptr;
        if (use_cc)
            launch_forces_cc(single ? nullptr : scenes_d, &scenes_h[0], nscenes, runs, nruns, keys, spos, svel,
                             nbr.rec, start, end, ids, o, rb ? &G : nullptr, n, stream, cc_warps);
        else
            launch_forces(L, spos, svel, dp, start, end, ids, o, rb ? &G : nullptr, nullptr, 0.f, 0.f, 0,
                          use_list ? &nbr : nullptr, target_order());
        launches++;
        if (!fused_integrate) {
            launch_integrate(L, pos, vel);
            launches++;
        }
        mark(6, 1);
    }
    if (fork_bodies) {
        /* the body update ran beside the force pass; its velocity mirror
         * lands once the force pass has read the old one */
        CK0(cudaStreamWaitEvent(stream, ev_bodies_done, 0));
        CK0(cudaMemcpyAsync(bvf, bvf_next, 16 * (size_t)nbodies, cudaMemcpyDeviceToDevice, stream));
    } else if (rb && (stages & FG_STAGE_BODIES)) {
        mark(7, 0);
        enqueue_bodies(stream, bvf);
        mark(7, 1);
        launches += body_launches();
    }
    if (cur_io && iob) {
        CK0(cudaMemcpyAsync(cur_io->op, pos, iob, cudaMemcpyDeviceToHost, stream));
        if (!cur_io->defer_vel) CK0(cudaMemcpyAsync(cur_io->ov, vel, iob, cudaMemcpyDeviceToHost, stream));
    }
    return launches;
}

/* Spatial target order from the current particle positions: Morton keys of
 * the unsorted particles, stable sort by key with particle ids as values.
 * The sorted-key buffers of the step are free here (the step rewrites them
 * before reading), so they serve as key scratch. */
void World::enqueue_order_refresh()
{
    if (!n) return;
    launch_morton_keys(fluid_launch(), pos, keys, order_bits, order_scene_shift);
    radix_sort(keys, nullptr, keys_u, tord, n, order_key_bits, digit_bits, rs, stream);
    kernels_enqueued += 1 + 3 * (uint64_t)radix_passes(order_key_bits, digit_bits);
    order_valid = true;
}

uint64_t World::graph_signature() const
{
    /* every setting that changes the captured launches, each in its own bits */
    const bool ordered = use_order && order_valid;
    return (uint64_t)(stages & 0xffu) | (fused_integrate ? 0x100ull : 0ull) | ((uint64_t)(digit_bits & 0xfu) << 9) |
           (use_list ? 1ull << 16 : 0ull) | (ordered ? 1ull << 17 : 0ull) | (use_cc ? 1ull << 18 : 0ull) |
           ((ordered && order_forces_only) ? 1ull << 19 : 0ull) | ((uint64_t)(ctas_per_sm & 0x7fu) << 20) |
           (one_pass_sort ? 1ull << 27 : 0ull) | (bucket_sort_on ? 1ull << 28 : 0ull) |
           ((uint64_t)((block >> 6) & 0x7u) << 29) | ((uint64_t)(cc_warps & 0x7u) << 32) |
           ((uint64_t)nbr.stride << 40);
}

/* The capacity is a device word the kernels read, so changing it within the
 * allocation leaves every captured graph valid.  A capacity beyond the
 * allocation reallocates the lists with 1.5x headroom (the captured graphs
 * hold the old pointer and stride and are dropped), so a growing scene
 * reallocates a few times rather than at every capacity check. */
int World::set_list_cap(uint32_t slots)
{
    if (slots < 1 || slots > FG_LIST_CAP_MAX) return FG_E_INVALID;
    slots = (slots + 3u) & ~3u; /* the force pass reads lists four entries at a time */
    if (slots > list_cap_alloc) {
        const uint32_t grown = ((list_cap_alloc + list_cap_alloc / 2u) + 31u) & ~31u;
        /* a multiple of 8: every list starts on a 32-byte boundary */
        const uint32_t stride = std::max((slots + 7u) & ~7u, std::min(grown, FG_LIST_CAP_MAX));
        CK(cudaStreamSynchronize(stream));
        const size_t N = std::max<uint64_t>(cap.particles, 1);
        uint32_t *p = nullptr;
        /* not cleared: every step writes entries [0, cnt rounded up to 4)
         * before the force pass reads them */
        CK(cudaMalloc(&p, 4 * (size_t)stride * N));
        for (auto &a : allocs)
            if (a == (void *)nbr.idx) a = p;
        cudaFree(nbr.idx);
        device_bytes += 4 * (size_t)(stride - list_cap_alloc) * N;
        nbr.idx = p;
        nbr.stride = stride;
        list_cap_alloc = stride;
        stale_graphs(); /* every captured step holds the old list pointer */
    }
    if (slots != list_cap) {
        list_cap = slots;
        k_set_u32<<<1, 1, 0, stream>>>(list_cap_d, list_cap);
        CK(cudaGetLastError());
    }
    return FG_OK;
}

int World::graph_for_current(cudaGraphExec_t *out, uint32_t nsteps)
{
    const uint64_t sig = graph_signature() ^ ((uint64_t)(nsteps & 0xffu) << 56);
    const StepIO io = cur_io ? *cur_io : StepIO();
    for (auto &g : graphs)
        if (g.sig == sig && g.io == io) {
            *out = g.exec;
            return FG_OK;
        }
    CachedGraph g{sig, nullptr, nullptr, io};
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    for (uint32_t k = 0; k < nsteps; k++) enqueue_step();
    cudaError_t e = cudaStreamEndCapture(stream, &g.graph);
    if (e != cudaSuccess) {
        set_error("cudaStreamEndCapture", e);
        return FG_E_CUDA;
    }
    for (size_t k = 0; k < stale.size(); k++) {
        if (stale[k].sig != sig || !(stale[k].io == io)) continue;
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(stale[k].exec, g.graph, &info) == cudaSuccess) {
            g.exec = stale[k].exec;
            cudaGraphDestroy(stale[k].graph);
            stale.erase(stale.begin() + (long)k);
            graphs.push_back(g);
            *out = g.exec;
            return FG_OK;
        }
        cudaGetLastError(); /* another topology (e.g. another radix pass count): instantiate */
        cudaGraphExecDestroy(stale[k].exec);
        cudaGraphDestroy(stale[k].graph);
        stale.erase(stale.begin() + (long)k);
        break;
    }
    e = cudaGraphInstantiate(&g.exec, g.graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g.graph);
        set_error("cudaGraphInstantiate", e);
        return FG_E_CUDA;
    }
    graphs.push_back(g);
    *out = g.exec;
    return FG_OK;
}

/* Autotuning round: the candidate values of one tunable (rotating among the
 * kernel, the CTAs per SM of the density/force grids and the radix digit
 * width) each run one real step between CUDA events -- the state advances as
 * in any step -- and the fastest value is kept.  A round may span several
 * step() calls. */
void World::tune_begin()
{
    int dims[6], nd = 0;
    if (__builtin_popcount(tune_kernels & 0x7u) >= 2) dims[nd++] = 0;
    if ((tune_tiles & 1u) && !use_cc) dims[nd++] = 1;
    if (tune_tiles & 2u) dims[nd++] = 2;
    if (tune_tiles & 4u) dims[nd++] = 3;
    if ((tune_tiles & 8u) && !use_cc) dims[nd++] = 4;
    if ((tune_tiles & 16u) && use_cc) dims[nd++] = 5;
    tr.ncand = 0;
    if (!nd) return;
    tr.dim = dims[tune_round++ % (uint32_t)nd];
    if (tr.dim == 0) {
        for (int k = 0; k < 3; k++)
            if (tune_kernels & (1u << k)) tr.cand[tr.ncand++] = k;
    } else if (tr.dim == 1) {
        /* CTAs per SM of the 128-thread density/force grids */
        const int v[3] = {16, 32, 64};
        for (int k = 0; k < 3; k++) tr.cand[tr.ncand++] = v[k];
    } else if (tr.dim == 2) {
        for (int v = 6; v <= 8; v++) tr.cand[tr.ncand++] = v;
    } else if (tr.dim == 3) {
        /* the sort: three kernels per digit pass, one kernel per pass, or
         * counting by bucket (when the tile sums fit its scratch) */
        tr.cand[tr.ncand++] = 0;
        tr.cand[tr.ncand++] = 1;
        if (bucket_sort_fits()) tr.cand[tr.ncand++] = 2;
    } else if (tr.dim == 4) {
        /* threads per CTA of the density/force grids */
        const int v[3] = {64, 128, 256};
        for (int k = 0; k < 3; k++) tr.cand[tr.ncand++] = v[k];
    } else {
        /* bucket runs (warps) per CTA of kernel 2 */
        const int v[3] = {1, 2, 4};
        for (int k = 0; k < 3; k++) tr.cand[tr.ncand++] = v[k];
    }
    if (tr.ncand < 2) {
        tr.ncand = 0;
        return;
    }
    if (!tr.ev[0])
        for (auto &e : tr.ev)
            if (cudaEventCreate(&e) != cudaSuccess) {
                cudaGetLastError();
                tr.ncand = 0;
                return;
            }
    const int prev[6] = {current_kernel(), (int)ctas_per_sm, (int)digit_bits, sort_variant(), (int)block,
                         (int)cc_warps};
    tr.prev = prev[tr.dim];
    tr.idx = 0;
    tr.active = true;
}

void World::tune_apply(int dim, int v)
{
    if (dim == 0) set_kernel(v);
    else if (dim == 1) ctas_per_sm = (uint32_t)v;
    else if (dim == 2) digit_bits = (uint32_t)v;
    else if (dim == 3) set_sort_variant(v);
    else if (dim == 4) block = (uint32_t)v;
    else cc_warps = (uint32_t)v;
}

int World::tune_finish()
{
    tr.active = false;
    CK(cudaEventSynchronize(tr.ev[2 * tr.ncand - 1]));
    int best = tr.cand[0];
    float best_ms = 1e30f, cur_ms = -1.0f;
    for (int c = 0; c < tr.ncand; c++) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, tr.ev[2 * c], tr.ev[2 * c + 1]));
        if (tr.dim == 0) tune_last_ms[tr.cand[c]] = ms;
        if (tr.cand[c] == tr.prev) cur_ms = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best = tr.cand[c];
        }
    }
    /* one step per candidate is a noisy sample: the value in use stays
     * unless another is faster by more than 1.5% */
    if (cur_ms >= 0.0f && best != tr.prev && best_ms > cur_ms * (1.0f - FG_TUNE_MARGIN)) best = tr.prev;
    tune_apply(tr.dim, best);
    return FG_OK;
}

/* Every FG_LIST_CHECK_PERIOD steps (kernel 1): grow the neighbour-list
 * capacity to 1.125x the largest in-range count seen since the last check,
 * so the force pass walks lists instead of buckets as a scene compresses. */
int World::check_list_cap()
{
    uint32_t mx = 0;
    CK(cudaMemcpyAsync(&mx, max_count, 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    CK(cudaMemsetAsync(max_count, 0, 4, stream));
    if (mx <= list_cap) return FG_OK;
    const uint32_t want = std::min<uint32_t>(((mx + mx / 8u) + 31u) & ~31u, FG_LIST_CAP_MAX);
    if (want <= list_cap) return FG_OK;
    return set_list_cap(want);
}

/* Whether step s starts by refreshing the Morton target order. */
bool World::order_refresh_due(uint64_t s) const
{
    return use_order && !needs_runs() && (stages & FG_STAGE_DENSITY) &&
           (!order_valid || (order_period && s % order_period == 0));
}

/* Steps at which the host acts between steps (autotuning rounds, list
 * capacity checks): a multi-step graph never spans one. */
bool World::host_boundary(uint64_t s) const
{
    if (tune_period && s % tune_period == 0) return true;
    if (use_list && list_autogrow && s % FG_LIST_CHECK_PERIOD == 0) return true;
    if (order_refresh_due(s)) return true;
    return false;
}

int World::step(uint32_t nsteps, const StepIO *io)
{
    if (staged_done) {
        set_error_msg("a stage-by-stage step is in progress: finish it with FG_RUN_INTEGRATE");
        return FG_E_STATE;
    }
    cur_io = io;
    int r = step_loop(nsteps);
    cur_io = nullptr;
    return r;
}

int World::step_loop(uint32_t nsteps)
{
    for (uint32_t k = 0; k < nsteps; k++) {
        if (use_graphs && graph_steps > 1 && !cur_io && !tr.active && nsteps - k >= graph_steps &&
            !host_boundary(step_count)) {
            bool clear = true;
            for (uint32_t q = 1; q < graph_steps && clear; q++) clear = !host_boundary(step_count + q);
            if (clear) {
                /* graph_steps steps in one captured graph */
                cudaGraphExec_t ge = nullptr;
                int r = graph_for_current(&ge, graph_steps);
                if (r != FG_OK) return r;
                CK(cudaGraphLaunch(ge, stream));
                kernels_enqueued += (uint64_t)graph_steps * launches_per_step();
                tune_count[current_kernel()] += graph_steps;
                counted_steps += graph_steps;
                step_count += graph_steps;
                k += graph_steps - 1;
                continue;
            }
        }
        if (use_list && list_autogrow && step_count && (step_count % FG_LIST_CHECK_PERIOD == 0)) {
            int r = check_list_cap();
            if (r != FG_OK) return r;
        }
        if (!tr.active && tune_period && (step_count % tune_period == 0)) tune_begin();
        if (order_refresh_due(step_count)) enqueue_order_refresh();
        if (tr.active) tune_apply(tr.dim, tr.cand[tr.idx]);
        const int kused = current_kernel();
        /* the graph is found (or captured and instantiated) before a trial's
         * start event, so a candidate's first use is not charged the host
         * time of building its graph */
        cudaGraphExec_t ge = nullptr;
        if (use_graphs) {
            int r = graph_for_current(&ge);
            if (r != FG_OK) return r;
        }
        if (tr.active) CK(cudaEventRecord(tr.ev[2 * tr.idx], stream));
        if (!use_graphs) enqueue_step();
        else CK(cudaGraphLaunch(ge, stream));
        kernels_enqueued += launches_per_step();
        if (tr.active) {
            CK(cudaEventRecord(tr.ev[2 * tr.idx + 1], stream));
            if (++tr.idx == tr.ncand) {
                int r = tune_finish();
                if (r != FG_OK) return r;
            }
        }
        tune_count[kused]++;
        counted_steps++;
        step_count++;
    }
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        set_error("step", e);
        return FG_E_CUDA;
    }
    return FG_OK;
}

/* The stages of one step enqueued one call at a time, in the order of the
 * reference's two-way step (HeterogeneousSimulator.cpp:57-126 with
 * RigidBodySimulator.cpp:313-611): neighbourhood (hash, sort, ranges),
 * density, rigid-sphere grid, sphere forces from the fluid and from other
 * bodies, fluid forces (velocity only), per-body sums, body integration,
 * fluid integration.  The kernels are those of a whole step, so a staged
 * step gives the same bits; no graph is captured and no autotuning round
 * runs.  A stage whose inputs were not produced earlier in the same step
 * returns FG_E_STATE. */
int World::run_stage(int stage, int flags)
{
    auto bit = [](int s) { return 1u << s; };
    auto need = [&](uint32_t mask, const char *msg) {
        if ((staged_done & mask) == mask) return true;
        set_error_msg(msg);
        return false;
    };
    const bool rb = nbodies > 0;
    const Launch L = fluid_launch();
    switch (stage) {
    case FG_RUN_NEIGHBOURHOOD: {
        if (staged_done) {
            set_error_msg("FG_RUN_NEIGHBOURHOOD: the previous staged step has not reached FG_RUN_INTEGRATE");
            return FG_E_STATE;
        }
        if (tr.active) { /* a staged step is no autotuning trial: keep the value in use */
            tune_apply(tr.dim, tr.prev);
            tr.active = false;
        }
        if (use_list && list_autogrow && step_count && (step_count % FG_LIST_CHECK_PERIOD == 0)) {
            int r = check_list_cap();
            if (r != FG_OK) return r;
        }
        if (order_refresh_due(step_count)) enqueue_order_refresh();
        enqueue_hash(L, true);
        counted_ranges = fused_ranges = false;
        enqueue_sort(true);
        if (!fused_ranges) {
            if (!counted_ranges) cudaMemsetAsync(start, 0xff, 4 * (size_t)total_buckets, stream);
            if (needs_runs()) {
                cudaMemsetAsync(nruns, 0, 4, stream);
                launch_cell_ranges(keys, ids, pos, vel, start, end, spos, svel, n, stream, inv, runs, nruns);
            } else {
                launch_cell_ranges(keys, ids, pos, vel, start, end, spos, svel, n, stream, inv);
            }
        }
        break;
    }
    case FG_RUN_DENSITY:
        if (!need(bit(FG_RUN_NEIGHBOURHOOD), "FG_RUN_DENSITY needs FG_RUN_NEIGHBOURHOOD first")) return FG_E_STATE;
        if (use_cc)
            launch_density_cc(single ? nullptr : scenes_d, &scenes_h[0], nscenes, runs, nruns, keys, spos, svel, start,
                              end, dp, nbr.rec, n, stream, cc_warps);
        else
            launch_density(L, spos, start, end, dp, 0.f, 0.f, 0.f, 0, svel, use_list ? &nbr : nullptr,
                           density_order(), pair_counter);
        break;
    case FG_RUN_RB_GRID: {
        if (!rb) break;
        if (staged_done & bit(FG_RUN_BODY_INTEGRATE)) {
            set_error_msg("FG_RUN_RB_GRID must come before FG_RUN_BODY_INTEGRATE");
            return FG_E_STATE;
        }
        uint32_t launches = 0;
        const uint32_t keep = stages;
        stages = FG_STAGE_ALL;
        enqueue_rb_grid(stream, nullptr, launches);
        stages = keep;
        break;
    }
    case FG_RUN_RB_FROM_FLUID:
        if (!rb) break;
        if (!need(bit(FG_RUN_NEIGHBOURHOOD) | bit(FG_RUN_RB_GRID),
                  "FG_RUN_RB_FROM_FLUID needs FG_RUN_NEIGHBOURHOOD and FG_RUN_RB_GRID first"))
            return FG_E_STATE;
        launch_rb_from_fluid(sphere_launch(), rb_spos, rb_ids, bvf, bxf, spos, svel, start, end, rb_force, rb_torque,
                             0);
        break;
    case FG_RUN_RB_FROM_RB:
        if (!rb || !any_rb_rb) break;
        if (!need(bit(FG_RUN_RB_FROM_FLUID), "FG_RUN_RB_FROM_RB adds to FG_RUN_RB_FROM_FLUID: run that first"))
            return FG_E_STATE;
        launch_rb_from_rb(sphere_launch(), rb_spos, rb_ids, bvf, bxf, rb_start, rb_end, rb_force, rb_torque, nullptr,
                          1);
        break;
    case FG_RUN_FORCES: {
        if (!need(bit(FG_RUN_DENSITY), "FG_RUN_FORCES needs FG_RUN_DENSITY first")) return FG_E_STATE;
        const bool contact = rb && (flags & FG_RUN_WITH_CONTACT);
        if (contact && !need(bit(FG_RUN_RB_GRID), "FG_RUN_FORCES with contact needs FG_RUN_RB_GRID first"))
            return FG_E_STATE;
        if (staged_done & bit(FG_RUN_BODY_INTEGRATE)) {
            set_error_msg("FG_RUN_FORCES reads the bodies' old velocities: run it before FG_RUN_BODY_INTEGRATE");
            return FG_E_STATE;
        }
        const RigidGrid G = body_grid();
        ForceOut o;
        o.vel = vel;
        o.pos = nullptr; /* FG_RUN_INTEGRATE moves the particles */
        if (use_cc)
            launch_forces_cc(single ? nullptr : scenes_d, &scenes_h[0], nscenes, runs, nruns, keys, spos, svel,
                             nbr.rec, start, end, ids, o, contact ? &G : nullptr, n, stream, cc_warps);
        else
            launch_forces(L, spos, svel, dp, start, end, ids, o, contact ? &G : nullptr, nullptr, 0.f, 0.f, 0,
                          use_list ? &nbr : nullptr, target_order());
        break;
    }
    case FG_RUN_BODY_SUMS:
    case FG_RUN_BODY_INTEGRATE: {
        if (!rb) break;
        const uint32_t want = bit(FG_RUN_RB_FROM_FLUID) | (any_rb_rb ? bit(FG_RUN_RB_FROM_RB) : 0u) |
                              (stage == FG_RUN_BODY_INTEGRATE ? bit(FG_RUN_BODY_SUMS) | bit(FG_RUN_FORCES) : 0u);
        if (!need(want, stage == FG_RUN_BODY_SUMS
                            ? "FG_RUN_BODY_SUMS needs the sphere forces (FG_RUN_RB_FROM_FLUID, and FG_RUN_RB_FROM_RB "
                              "when bodies can touch) first"
                            : "FG_RUN_BODY_INTEGRATE needs FG_RUN_BODY_SUMS and FG_RUN_FORCES first"))
            return FG_E_STATE;
        BodyState b;
        b.x = bx; b.v = bv; b.q = bq; b.L = bL;
        b.inv_inertia = binv;
        b.mass = bmass;
        b.x_f = bxf; b.v_f = bvf; b.q_f = bqf;
        b.force_sum = bfs; b.torque_sum = bts;
        b.partial = body_part;
        launch_body_update(single ? nullptr : scenes_d, &scenes_h[0], body_scene, body_first, body_count, nbodies,
                           rb_force, rb_torque, b, stage == FG_RUN_BODY_INTEGRATE ? 1 : 0, stream);
        break;
    }
    case FG_RUN_INTEGRATE: {
        const uint32_t want = bit(FG_RUN_FORCES) | (rb ? bit(FG_RUN_BODY_INTEGRATE) : 0u);
        if (!need(want, "FG_RUN_INTEGRATE ends the step: it needs FG_RUN_FORCES (and FG_RUN_BODY_INTEGRATE with "
                        "bodies) first"))
            return FG_E_STATE;
        launch_integrate(L, pos, vel);
        cudaError_t e = cudaPeekAtLastError();
        if (e != cudaSuccess) {
            set_error("staged step", e);
            return FG_E_CUDA;
        }
        tune_count[current_kernel()]++;
        counted_steps++;
        step_count++;
        staged_done = 0;
        return FG_OK;
    }
    default:
        set_error_msg("unknown stage");
        return FG_E_INVALID;
    }
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        set_error("staged step", e);
        return FG_E_CUDA;
    }
    staged_done |= bit(stage);
    return FG_OK;
}

uint32_t World::launches_per_step()
{
    /* count by enqueueing into a capture-free dry description */
    uint32_t c = 0;
    if (stages & FG_STAGE_HASH) c += 1;
    if (stages & FG_STAGE_SORT) c += sort_launches();
    /* + one memset node; none with the counting sort's fused reorder */
    if ((stages & FG_STAGE_RANGES) && !(bucket_sort_on && bucket_sort_fits() && (stages & FG_STAGE_SORT))) c += 1;
    if (stages & FG_STAGE_DENSITY) c += 1;
    if (nbodies) {
        if (stages & FG_STAGE_RB_GRID) /* aabb reset, hash, sort + ranges */
            c += rb_small_scenes ? 3 : 3 + 3 * radix_passes(rb_key_bits, 8);
        if (stages & FG_STAGE_RB_CONTACT) c += 1 + (any_rb_rb ? 1 : 0) + (fluid_contact_pass() ? 1 : 0);
        if (stages & FG_STAGE_BODIES) c += body_launches();
    }
    if (stages & FG_STAGE_FORCES) c += fused_integrate ? 1 : 2;
    return c;
}

/* NaN/Inf scan of positions and velocities */
__global__ void k_check(const float4 *pos, const float4 *vel, uint32_t n, uint32_t *status)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = pos[i], v = vel[i];
        if (!isfinite(p.x) || !isfinite(p.y) || !isfinite(p.z) || !isfinite(v.x) || !isfinite(v.y) ||
            !isfinite(v.z))
            atomicOr(status, FG_DEV_NONFINITE);
    }
}

/* FP64 sums per scene (see fg_diag.cu); out: nscenes x FG_DIAG_COUNT. */
int World::diagnostics(double *out)
{
    const size_t nw = std::max<uint32_t>(nwork, 1), ns = std::max<uint32_t>(nscenes, 1);
    if (nw > diag_cap_work || ns > diag_cap_scenes) {
        if (diag_first) cudaFree(diag_first);
        if (diag_part) cudaFree(diag_part);
        if (diag_out) cudaFree(diag_out);
        diag_first = nullptr;
        diag_part = diag_out = nullptr;
        diag_cap_work = diag_cap_scenes = 0;
        CK(cudaMalloc(&diag_first, 4 * (ns + 1)));
        CK(cudaMalloc(&diag_part, 8 * 9 * nw));
        CK(cudaMalloc(&diag_out, 8 * FG_DIAG_VALUES * ns));
        diag_cap_work = nw;
        diag_cap_scenes = ns;
    }
    if (!nscenes) return FG_OK;
    CK(cudaMemcpyAsync(diag_first, work_first_h.data(), 4 * (nscenes + 1), cudaMemcpyHostToDevice, stream));
    launch_diagnostics(fluid_launch(), nscenes, diag_first, pos, vel, bv, bL, bmass, diag_part, diag_out);
    CK(cudaMemcpyAsync(out, diag_out, 8 * FG_DIAG_VALUES * (size_t)nscenes, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return FG_OK;
}

int World::check()
{
    if (!n) return FG_OK;
    k_check<<<grid_for((n + 255) / 256, 8), 256, 0, stream>>>(pos, vel, n, status_d);
    return FG_OK;
}

int World::sync()
{
    CK(cudaStreamSynchronize(stream));
    uint32_t st = 0;
    CK(cudaMemcpy(&st, status_d, 4, cudaMemcpyDeviceToHost));
    if (st & FG_DEV_NONFINITE) return FG_E_NONFINITE;
    if (st & FG_DEV_SORT_TIMEOUT) {
        set_error_msg("a one-pass radix sort gave up waiting on a preceding tile");
        return FG_E_TIMEOUT;
    }
    return FG_OK;
}

/* RAII event set */
struct Events {
    std::vector<cudaEvent_t> ev;
    explicit Events(size_t n) : ev(n, nullptr)
    {
        for (auto &e : ev) cudaEventCreate(&e);
    }
    ~Events()
    {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
};

int World::ensure_flush(size_t bytes)
{
    if (bytes <= flush_bytes) return FG_OK;
    if (flush_buf) cudaFree(flush_buf);
    flush_buf = nullptr;
    flush_bytes = 0;
    CK(cudaMalloc(&flush_buf, bytes));
    flush_bytes = bytes;
    return FG_OK;
}

int World::stage_profile(size_t fbytes, float *ms)
{
    Events E(16);
    for (int k = 0; k < 16; k++)
        if (!E.ev[k]) return FG_E_CUDA;
    if (fbytes) {
        int r = ensure_flush(fbytes);
        if (r != FG_OK) return r;
        launch_fill(flush_buf, fbytes / 4, 7u, stream);
    }
    for (int k = 0; k < 8; k++) ms[k] = 0.0f;
    if (use_order && !order_valid) enqueue_order_refresh();
    kernels_enqueued += enqueue_step(E.ev.data());
    step_count++;
    counted_steps++;
    tune_count[current_kernel()]++;
    CK(cudaStreamSynchronize(stream));
    for (int k = 0; k < 8; k++) {
        if (cudaEventQuery(E.ev[2 * k]) != cudaSuccess || cudaEventQuery(E.ev[2 * k + 1]) != cudaSuccess) {
            cudaGetLastError(); /* stage not run: events never recorded */
            continue;
        }
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, E.ev[2 * k], E.ev[2 * k + 1]) == cudaSuccess) ms[k] = t;
        else cudaGetLastError();
    }
    return FG_OK;
}

int World::timed_steps(uint32_t nsteps, size_t fbytes, float *ms, uint32_t per_block)
{
    if (fbytes) {
        int r = ensure_flush(fbytes);
        if (r != FG_OK) return r;
    }
    Events E(2 * (size_t)nsteps);
    for (uint32_t k = 0; k < nsteps; k++) {
        if (fbytes) {
            launch_fill(flush_buf, fbytes / 4, k, stream);
            kernels_enqueued++;
        }
        CK(cudaEventRecord(E.ev[2 * k], stream));
        int r = step(per_block);
        if (r != FG_OK) return r;
        CK(cudaEventRecord(E.ev[2 * k + 1], stream));
    }
    CK(cudaStreamSynchronize(stream));
    for (uint32_t k = 0; k < nsteps; k++) CK(cudaEventElapsedTime(&ms[k], E.ev[2 * k], E.ev[2 * k + 1]));
    return FG_OK;
}

static bool is_pinned(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

int World::e2e_steps(uint32_t nsteps, const float *hp, const float *hv, float *op, float *ov, float *ms)
{
    Events E(2 * (size_t)nsteps);
    StepIO io;
    io.hp = hp;
    io.hv = hv;
    io.op = op;
    io.ov = ov;
    /* pinned buffers: the copies belong to the step (captured with it, the
     * velocity upload beside the hash and sort, and each step's velocity
     * download carried into the next step beside its position upload; the
     * last one follows the last step); pageable ones are copied around it */
    const bool pinned = is_pinned(hp) && is_pinned(hv) && is_pinned(op) && is_pinned(ov);
    const size_t b = 16 * (size_t)n;
    for (uint32_t k = 0; k < nsteps; k++) {
        CK(cudaEventRecord(E.ev[2 * k], stream));
        if (pinned) {
            io.prev_vel = k > 0;
            io.defer_vel = true;
            int r = step(1, &io);
            if (r != FG_OK) return r;
            if (k + 1 == nsteps && b) CK(cudaMemcpyAsync(ov, vel, b, cudaMemcpyDeviceToHost, stream));
        } else {
            if (b) {
                CK(cudaMemcpyAsync(pos, hp, b, cudaMemcpyHostToDevice, stream));
                CK(cudaMemcpyAsync(vel, hv, b, cudaMemcpyHostToDevice, stream));
            }
            int r = step(1);
            if (r != FG_OK) return r;
            if (b) {
                CK(cudaMemcpyAsync(op, pos, b, cudaMemcpyDeviceToHost, stream));
                CK(cudaMemcpyAsync(ov, vel, b, cudaMemcpyDeviceToHost, stream));
            }
        }
        CK(cudaEventRecord(E.ev[2 * k + 1], stream));
    }
    CK(cudaStreamSynchronize(stream));
    for (uint32_t k = 0; k < nsteps; k++) CK(cudaEventElapsedTime(&ms[k], E.ev[2 * k], E.ev[2 * k + 1]));
    return FG_OK;
}

/* Register-resident FMA loop: 8 independent chains per thread. */
__global__ void k_fma_probe(float *out, int iters, float a, float b)
{
    float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
    float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678f) out[0] = s; /* keeps the loop alive */
}

int probe_fp32(float *tflops)
{
    float *d = nullptr;
    CK(cudaMalloc(&d, 16));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sm_count() * 8, threads = 256, iters = 4096;
    k_fma_probe<<<blocks, threads>>>(d, 64, 0.999f, 1e-6f); /* warm-up */
    cudaEventRecord(e0);
    k_fma_probe<<<blocks, threads>>>(d, iters, 0.999f, 1e-6f);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_error("fp32 probe", e);
        return FG_E_CUDA;
    }
    double flops = 2.0 * 8.0 * 16.0 * (double)iters * (double)blocks * (double)threads;
    *tflops = (float)(flops / (ms * 1e-3) / 1e12);
    return FG_OK;
}

} // namespace fg

/* ============================================================ C ABI */

using fg::World;

extern "C" {

void fg_scene_desc_defaults(fg_scene_desc *d)
{
    if (!d) return;
    memset(d, 0, sizeof(*d));
    const float h = 0.0457f;
    for (int k = 0; k < 3; k++) {
        d->cell_size[k] = h;
        d->bucket_size[k] = 64;
        d->volume_min[k] = 0.0f;
        d->volume_max[k] = 1.0f;
        d->rb_bucket_size[k] = 64;
        d->fluid_to_rb_relation[k] = 1;
        d->rb_to_fluid_relation[k] = 1;
        d->rb_volume_min[k] = 0.0f;
        d->rb_volume_max[k] = 1.0f;
    }
    d->gravity[1] = -9.8f;
    d->kernel_radius = h;
    d->velocity_limit = 600.0f;
    d->simulation_scale = 1.0f;
    d->dt = 0.003f;
    d->mass = 0.02f;
    d->rest_density = 998.29f;
    d->gas_constant = 3.0f;
    d->viscosity = 3.5f;
    /* SPHCalculateForcesK literals (K_FluidSim.cu:289-293) */
    d->wall_distance = 0.003043174f;
    d->wall_stiffness = 20000.0f;
    d->wall_damping = 256.0f;
    d->noslip_min[0] = -11.0f; d->noslip_min[1] = -40.0f; d->noslip_min[2] = -11.0f;
    d->noslip_max[0] = 11.0f; d->noslip_max[1] = 200.0f; d->noslip_max[2] = 11.0f;
    d->friction_kinetic = 0.0f;
    d->friction_static = 0.0f;
    d->fluid_radius = 0.25f * h;
    d->rb_radius = 0.5f * h;
    d->contact_kspring = -10.0f; /* HeterogeneousSimulator.cpp:180 */
    d->contact_kdamping = -5.0f;
    d->fluid_contact_eps = 0.003f;
    d->rb_contact_eps = 0.0001f;
    d->rbrb_kspring = -10.0f;
    d->rbrb_kdamping = -5.0f;
    d->rbrb_eps = 0.001f;
    d->rb_gravity[1] = -9.8f;
    d->rb_velocity_limit = 600.0f;
    d->rb_dt = 0.003f;
}

int fg_world_create(const fg_scene_desc *scenes, uint32_t nscenes, fg_stream_t stream, fg_world **out)
{
    if (!out || !scenes || nscenes == 0) return FG_E_INVALID;
    *out = nullptr;
    for (uint32_t s = 0; s < nscenes; s++) {
        int v = fg::validate(scenes[s]);
        if (v != FG_OK) {
            fg::set_error_msg("invalid scene description");
            return v;
        }
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        fg::set_error("cudaGetDeviceCount", e == cudaSuccess ? cudaErrorNoDevice : e);
        return FG_E_NOLIB;
    }
    World *w = new World();
    int r = w->create(scenes, nscenes, (cudaStream_t)stream);
    if (r != FG_OK) {
        delete w;
        return r;
    }
    for (uint32_t s = 0; s < nscenes; s++)
        if (scenes[s].n_bodies && scenes[s].rb_rb_contact) w->any_rb_rb = true;
    *out = (fg_world *)w;
    return FG_OK;
}

int fg_world_destroy(fg_world *w)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    cudaStreamSynchronize(W->stream);
    delete W;
    return FG_OK;
}

int fg_world_step(fg_world *w, uint32_t nsteps)
{
    if (!w) return FG_E_INVALID;
    return ((World *)w)->step(nsteps);
}

int fg_world_run_stage(fg_world *w, int stage, int flags)
{
    if (!w) return FG_E_INVALID;
    return ((World *)w)->run_stage(stage, flags);
}

int fg_world_sync(fg_world *w)
{
    if (!w) return FG_E_INVALID;
    return ((World *)w)->sync();
}

int fg_world_check(fg_world *w)
{
    if (!w) return FG_E_INVALID;
    return ((World *)w)->check();
}

int fg_world_upload(fg_world *w, const float *pos4, const float *vel4)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    if (!W->n) return FG_OK;
    if (pos4) CK(cudaMemcpyAsync(W->pos, pos4, 16 * (size_t)W->n, cudaMemcpyHostToDevice, W->stream));
    if (vel4) CK(cudaMemcpyAsync(W->vel, vel4, 16 * (size_t)W->n, cudaMemcpyHostToDevice, W->stream));
    return FG_OK;
}

int fg_world_download(fg_world *w, float *pos4, float *vel4)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    if (!W->n) return FG_OK;
    if (pos4) CK(cudaMemcpyAsync(pos4, W->pos, 16 * (size_t)W->n, cudaMemcpyDeviceToHost, W->stream));
    if (vel4) CK(cudaMemcpyAsync(vel4, W->vel, 16 * (size_t)W->n, cudaMemcpyDeviceToHost, W->stream));
    return FG_OK;
}

int fg_world_scene_upload(fg_world *w, uint32_t scene, const float *pos4, const float *vel4)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    if (scene >= W->nscenes) return FG_E_INVALID;
    const FgScene &S = W->scenes_h[scene];
    if (!S.n) return FG_OK;
    if (pos4) CK(cudaMemcpyAsync(W->pos + S.pbase, pos4, 16 * (size_t)S.n, cudaMemcpyHostToDevice, W->stream));
    if (vel4) CK(cudaMemcpyAsync(W->vel + S.pbase, vel4, 16 * (size_t)S.n, cudaMemcpyHostToDevice, W->stream));
    return FG_OK;
}

int fg_world_scene_download(fg_world *w, uint32_t scene, float *pos4, float *vel4)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    if (scene >= W->nscenes) return FG_E_INVALID;
    const FgScene &S = W->scenes_h[scene];
    if (!S.n) return FG_OK;
    if (pos4) CK(cudaMemcpyAsync(pos4, W->pos + S.pbase, 16 * (size_t)S.n, cudaMemcpyDeviceToHost, W->stream));
    if (vel4) CK(cudaMemcpyAsync(vel4, W->vel + S.pbase, 16 * (size_t)S.n, cudaMemcpyDeviceToHost, W->stream));
    return FG_OK;
}

uint32_t fg_world_particles(const fg_world *w) { return w ? ((const World *)w)->n : 0; }
uint32_t fg_world_scenes(const fg_world *w) { return w ? ((const World *)w)->nscenes : 0; }
uint32_t fg_world_spheres(const fg_world *w) { return w ? ((const World *)w)->nspheres : 0; }
uint32_t fg_world_bodies(const fg_world *w) { return w ? ((const World *)w)->nbodies : 0; }

int fg_world_scene_layout(const fg_world *w, uint32_t scene, uint32_t out[8])
{
    if (!w || !out) return FG_E_INVALID;
    const World *W = (const World *)w;
    if (scene >= W->nscenes) return FG_E_INVALID;
    const FgScene &S = W->scenes_h[scene];
    out[0] = S.pbase; out[1] = S.n; out[2] = S.bucket_base; out[3] = S.nb;
    out[4] = S.sph_base; out[5] = S.nsph; out[6] = S.body_base; out[7] = S.nbodies;
    return FG_OK;
}

int fg_world_buffer(fg_world *w, int id, void **dev_ptr, size_t *bytes)
{
    if (!w || !dev_ptr || !bytes) return FG_E_INVALID;
    World *W = (World *)w;
    const size_t N = W->n, B = W->total_buckets, S = W->nspheres, RB = W->total_rb_buckets, NB = W->nbodies;
    void *p = nullptr;
    size_t b = 0;
    switch (id) {
    case FG_BUF_POS: p = W->pos; b = 16 * N; break;
    case FG_BUF_VEL: p = W->vel; b = 16 * N; break;
    case FG_BUF_KEYS_UNSORTED: p = W->keys_u; b = 4 * N; break;
    case FG_BUF_KEYS: p = W->keys; b = 4 * N; break;
    case FG_BUF_IDS: p = W->ids; b = 4 * N; break;
    case FG_BUF_START: p = W->start; b = 4 * B; break;
    case FG_BUF_END: p = W->end; b = 4 * B; break;
    case FG_BUF_SPOS: p = W->spos; b = 16 * N; break;
    case FG_BUF_SVEL: p = W->svel; b = 16 * N; break;
    case FG_BUF_DP: p = W->dp; b = 8 * N; break;
    case FG_BUF_RB_LOCAL: p = W->rb_local; b = 16 * S; break;
    case FG_BUF_RB_WORLD: p = W->rb_world; b = 16 * S; break;
    case FG_BUF_RB_KEYS_UNSORTED: p = W->rb_keys_u; b = 4 * S; break;
    case FG_BUF_RB_KEYS: p = W->rb_keys; b = 4 * S; break;
    case FG_BUF_RB_IDS: p = W->rb_ids; b = 4 * S; break;
    case FG_BUF_RB_START: p = W->rb_start; b = 4 * RB; break;
    case FG_BUF_RB_END: p = W->rb_end; b = 4 * RB; break;
    case FG_BUF_RB_SPOS: p = W->rb_spos; b = 16 * S; break;
    case FG_BUF_RB_FORCE: p = W->rb_force; b = 16 * S; break;
    case FG_BUF_RB_TORQUE: p = W->rb_torque; b = 16 * S; break;
    case FG_BUF_BODY_X: p = W->bx; b = 32 * NB; break;
    case FG_BUF_BODY_V: p = W->bv; b = 32 * NB; break;
    case FG_BUF_BODY_Q: p = W->bq; b = 32 * NB; break;
    case FG_BUF_BODY_L: p = W->bL; b = 32 * NB; break;
    case FG_BUF_BODY_FSUM: p = W->bfs; b = 32 * NB; break;
    case FG_BUF_BODY_TSUM: p = W->bts; b = 32 * NB; break;
    case FG_BUF_BODY_XF: p = W->bxf; b = 16 * NB; break;
    case FG_BUF_BODY_VF: p = W->bvf; b = 16 * NB; break;
    case FG_BUF_BODY_QF: p = W->bqf; b = 16 * NB; break;
    case FG_BUF_BODY_MASS: p = W->bmass; b = 8 * NB; break;
    case FG_BUF_BODY_INV_INERTIA: p = W->binv; b = 72 * NB; break;
    default: return FG_E_INVALID;
    }
    *dev_ptr = p;
    *bytes = p ? b : 0;
    return FG_OK;
}

int fg_world_set_stages(fg_world *w, uint32_t mask)
{
    if (!w) return FG_E_INVALID;
    ((World *)w)->stages = mask & FG_STAGE_ALL;
    return FG_OK;
}

int fg_world_set_fused_integrate(fg_world *w, int fused)
{
    if (!w) return FG_E_INVALID;
    ((World *)w)->fused_integrate = fused != 0;
    return FG_OK;
}

int fg_world_set_sort_digit_bits(fg_world *w, uint32_t bits)
{
    if (!w || bits < 1 || bits > 8) return FG_E_INVALID;
    ((World *)w)->digit_bits = bits;
    return FG_OK;
}

int fg_world_set_graphs(fg_world *w, int on)
{
    if (!w) return FG_E_INVALID;
    ((World *)w)->use_graphs = on != 0;
    return FG_OK;
}

int fg_world_set_option(fg_world *w, int option, int value)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    switch (option) {
    case FG_OPT_NEIGHBOR_LIST: W->use_list = value != 0; return FG_OK;
    case FG_OPT_TARGET_ORDER:
        if (value < 0 || value > 2) return FG_E_INVALID;
        W->use_order = value != 0;
        W->order_forces_only = value == 2;
        return FG_OK;
    case FG_OPT_ORDER_PERIOD:
        if (value < 0) return FG_E_INVALID;
        W->order_period = (uint32_t)value;
        return FG_OK;
    case FG_OPT_DIGIT_BITS:
        if (value < 1 || value > 8) return FG_E_INVALID;
        W->digit_bits = (uint32_t)value;
        return FG_OK;
    case FG_OPT_KERNEL:
        if (value < 0 || value > 2) return FG_E_INVALID;
        W->set_kernel(value);
        return FG_OK;
    case FG_OPT_AUTOTUNE_PERIOD:
        if (value < 0) return FG_E_INVALID;
        W->tune_period = (uint32_t)value;
        return FG_OK;
    case FG_OPT_AUTOTUNE_KERNELS:
        if (value <= 0 || value > 7) return FG_E_INVALID;
        W->tune_kernels = (uint32_t)value;
        return FG_OK;
    case FG_OPT_LIST_CAP: {
        const int r = W->set_list_cap((uint32_t)std::max(value, 0));
        if (r == FG_OK) W->list_autogrow = false; /* an explicit capacity stays */
        return r;
    }
    case FG_OPT_LIST_AUTOGROW: W->list_autogrow = value != 0; return FG_OK;
    case FG_OPT_GRAPH_STEPS:
        if (value < 1 || value > 64) return FG_E_INVALID;
        W->graph_steps = (uint32_t)value;
        return FG_OK;
    case FG_OPT_ONE_PASS_SORT:
        if (value < 0 || value > 2) return FG_E_INVALID;
        W->set_sort_variant(value);
        W->sort_chosen = true;
        return FG_OK;
    case FG_OPT_BLOCK_SIZE:
        if (value != 64 && value != 128 && value != 256) return FG_E_INVALID;
        W->block = (uint32_t)value;
        return FG_OK;
    case FG_OPT_RUNS_PER_CTA:
        if (value != 1 && value != 2 && value != 4) return FG_E_INVALID;
        W->cc_warps = (uint32_t)value;
        return FG_OK;
    case FG_OPT_CTAS_PER_SM:
        if (value < 0 || value > 64) return FG_E_INVALID;
        W->ctas_per_sm = (uint32_t)value;
        return FG_OK;
    case FG_OPT_AUTOTUNE_TILES:
        if (value < 0 || value > 31) return FG_E_INVALID;
        W->tune_tiles = (uint32_t)value;
        return FG_OK;
    default: return FG_E_INVALID;
    }
}

int fg_world_counters(fg_world *w, int reset, uint64_t *pair_visits, uint64_t *steps)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    CK(cudaStreamSynchronize(W->stream));
    unsigned long long v = 0;
    CK(cudaMemcpy(&v, W->pair_counter, sizeof(v), cudaMemcpyDeviceToHost));
    if (pair_visits) *pair_visits = v;
    if (steps) *steps = W->counted_steps;
    if (reset) {
        CK(cudaMemset(W->pair_counter, 0, sizeof(v)));
        W->counted_steps = 0;
    }
    return FG_OK;
}

int fg_world_list_overflows(fg_world *w, int reset, uint64_t *particles)
{
    if (!w) return FG_E_INVALID;
    World *W = (World *)w;
    CK(cudaStreamSynchronize(W->stream));
    unsigned long long v = 0;
    CK(cudaMemcpy(&v, W->overflow_counter, sizeof(v), cudaMemcpyDeviceToHost));
    if (particles) *particles = v;
    if (reset) CK(cudaMemset(W->overflow_counter, 0, sizeof(v)));
    return FG_OK;
}

int fg_world_tuning_stats(const fg_world *w, uint32_t steps_per_kernel[FG_NUM_KERNELS],
                          float last_trial_ms[FG_NUM_KERNELS])
{
    if (!w) return FG_E_INVALID;
    const World *W = (const World *)w;
    for (int k = 0; k < FG_NUM_KERNELS; k++) {
        if (steps_per_kernel) steps_per_kernel[k] = W->tune_count[k];
        if (last_trial_ms) last_trial_ms[k] = W->tune_last_ms[k];
    }
    return FG_OK;
}

int fg_world_get_option(const fg_world *w, int option, int *value)
{
    if (!w || !value) return FG_E_INVALID;
    const World *W = (const World *)w;
    switch (option) {
    case FG_OPT_NEIGHBOR_LIST: *value = W->use_list ? 1 : 0; return FG_OK;
    case FG_OPT_TARGET_ORDER: *value = W->use_order ? (W->order_forces_only ? 2 : 1) : 0; return FG_OK;
    case FG_OPT_ORDER_PERIOD: *value = (int)W->order_period; return FG_OK;
    case FG_OPT_DIGIT_BITS: *value = (int)W->digit_bits; return FG_OK;
    case FG_OPT_KERNEL: *value = W->current_kernel(); return FG_OK;
    case FG_OPT_BLOCK_SIZE: *value = (int)W->block; return FG_OK;
    case FG_OPT_RUNS_PER_CTA: *value = (int)W->cc_warps; return FG_OK;
    case FG_OPT_AUTOTUNE_PERIOD: *value = (int)W->tune_period; return FG_OK;
    case FG_OPT_AUTOTUNE_KERNELS: *value = (int)W->tune_kernels; return FG_OK;
    case FG_OPT_LIST_CAP: *value = (int)W->list_cap; return FG_OK;
    case FG_OPT_LIST_AUTOGROW: *value = W->list_autogrow ? 1 : 0; return FG_OK;
    case FG_OPT_GRAPH_STEPS: *value = (int)W->graph_steps; return FG_OK;
    case FG_OPT_ONE_PASS_SORT: *value = W->sort_variant(); return FG_OK;
    case FG_OPT_CTAS_PER_SM: *value = (int)W->ctas_per_sm; return FG_OK;
    case FG_OPT_AUTOTUNE_TILES: *value = (int)W->tune_tiles; return FG_OK;
    default: return FG_E_INVALID;
    }
}

int fg_world_kernel_launches(const fg_world *w, uint64_t *count)
{
    if (!w || !count) return FG_E_INVALID;
    *count = ((const World *)w)->kernels_enqueued;
    return FG_OK;
}

uint32_t fg_world_launches_per_step(const fg_world *w)
{
    if (!w) return 0;
    return ((World *)w)->launches_per_step();
}

int fg_memcpy_d2h(void *dst, const void *src, size_t bytes)
{
    if (!bytes) return FG_OK;
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return FG_OK;
}

int fg_memcpy_h2d(void *dst, const void *src, size_t bytes)
{
    if (!bytes) return FG_OK;
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return FG_OK;
}

int fg_device_synchronize(void)
{
    CK(cudaDeviceSynchronize());
    return FG_OK;
}

int fg_world_stage_profile(fg_world *w, size_t flush_bytes, float stage_ms[8])
{
    if (!w || !stage_ms) return FG_E_INVALID;
    return ((World *)w)->stage_profile(flush_bytes, stage_ms);
}

int fg_world_timed_steps(fg_world *w, uint32_t nsteps, size_t flush_bytes, float *ms)
{
    if (!w || (!ms && nsteps)) return FG_E_INVALID;
    return ((World *)w)->timed_steps(nsteps, flush_bytes, ms);
}

int fg_world_timed_blocks(fg_world *w, uint32_t nblocks, uint32_t steps_per_block, size_t flush_bytes, float *ms)
{
    if (!w || (!ms && nblocks) || !steps_per_block) return FG_E_INVALID;
    return ((World *)w)->timed_steps(nblocks, flush_bytes, ms, steps_per_block);
}

int fg_world_diagnostics(fg_world *w, double *out)
{
    if (!w || !out) return FG_E_INVALID;
    return ((World *)w)->diagnostics(out);
}

int fg_world_e2e_steps(fg_world *w, uint32_t nsteps, const float *host_pos4, const float *host_vel4,
                       float *out_pos4, float *out_vel4, float *ms)
{
    if (!w || !host_pos4 || !host_vel4 || !out_pos4 || !out_vel4 || (!ms && nsteps)) return FG_E_INVALID;
    return ((World *)w)->e2e_steps(nsteps, host_pos4, host_vel4, out_pos4, out_vel4, ms);
}

void *fg_host_alloc(size_t bytes)
{
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

int fg_host_free(void *p)
{
    if (!p) return FG_OK;
    CK(cudaFreeHost(p));
    return FG_OK;
}

int fg_set_device(int device)
{
    CK(cudaSetDevice(device));
    return FG_OK;
}

int fg_probe_fp32_peak(float *tflops)
{
    if (!tflops) return FG_E_INVALID;
    return fg::probe_fp32(tflops);
}

const char *fg_last_error(void) { return fg::g_err.c_str(); }

int fg_selftest_bounded_wait(unsigned int spin_limit, unsigned int *flags)
{
    if (!flags) return FG_E_INVALID;
    *flags = 0;
    if (fg::bounded_wait_selftest(spin_limit, flags) != 0) {
        fg::set_error("fg_selftest_bounded_wait", cudaGetLastError());
        return FG_E_CUDA;
    }
    return FG_OK;
}

const char *fg_version(void) { return "fluidgrid_gb300 0.1 sm_103a"; }

} /* extern "C" */
