/* Headless C++ mirror of FluidGrid's simulation classes (GPUSPHFluid,
 * HeterogeneousSimulator, RigidBodySimulator, RigidBody, BlockEmitter,
 * ApplicationData), implemented on the world C ABI of this library.
 * Declarations and the reference each class follows: include/fluidgrid_sim.hpp. */
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <fstream>
#include <sstream>
#include <vector>
#include "../../include/fluidgrid_sim.hpp"

namespace Simulation {

namespace Application {

ApplicationData::ApplicationData()
{
    memset(&mCommonFluidParams, 0, sizeof(mCommonFluidParams));
    memset(&mKernelsCache, 0, sizeof(mKernelsCache));
    memset(&mCommonRigidBodyParams, 0, sizeof(mCommonRigidBodyParams));
}

ApplicationData *ApplicationData::instance()
{
    static ApplicationData inst;
    return &inst;
}

} // namespace Application

namespace Emitter {

BlockEmitter::BlockEmitter(mc::math::Vec3f block_min, mc::math::Vec3f block_max, float particle_spacing)
    : mBlockSizeMin(block_min), mBlockSizeMax(block_max), mParticleSpacing(particle_spacing)
{
}

/* Emitter.cpp:16-43: rows in x, layers in z, then the next height in y, with
 * float loop counters as there; slots beyond the block are inactive. */
void BlockEmitter::reset(float4 *positions, int count)
{
    int used = 0;
    float y = mBlockSizeMin.y;
    if (mParticleSpacing > 0.0f) {
        while (used < count) {
            int row = 0;
            for (float z = mBlockSizeMin.z; z < mBlockSizeMax.z; z += mParticleSpacing)
                for (float x = mBlockSizeMin.x; x < mBlockSizeMax.x; x += mParticleSpacing) {
                    if (used < count) positions[used++] = make_float4(x, y, z, 1.0f);
                    row++;
                }
            if (!row) break; /* an empty block would never fill */
            y += mParticleSpacing;
        }
    }
    for (; used < count; used++) positions[used] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
}

} // namespace Emitter

namespace Simulators {

/* ------------------------------------------------------------ RigidBody */

RigidBody::RigidBody() : mIsStatic(false), mParticleRadius(0.0f), mMass(0.0f)
{
    memset(&inertiaTensor, 0, sizeof(inertiaTensor));
    memset(&invInertiaTensor, 0, sizeof(invInertiaTensor));
    mPosition = make_float3(0.0f, 0.0f, 0.0f);
    mOrientation = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
}

RigidBody::~RigidBody() {}

/* RigidBody.cpp:55-126: the reference's text format and its fixed inertia
 * (200 m / 12 on the diagonal) and inverse inertia (0.00125). */
RigidBody *RigidBody::loadFromFile(std::string filename)
{
    std::ifstream file(filename.c_str());
    if (!file) return nullptr;
    RigidBody *rb = new RigidBody();
    std::string line;
    std::getline(file, line);
    if (line.compare(0, 6, "static") == 0) {
        rb->mIsStatic = true;
        rb->mMass = 0.0f;
    } else {
        std::getline(file, line);
        rb->mIsStatic = false;
        rb->mMass = (float)atof(line.c_str());
    }
    std::getline(file, line);
    rb->mParticleRadius = (float)atof(line.c_str());
    std::getline(file, line);
    rb->mOriginalMeshFilename = line;
    std::getline(file, line);
    const int n = (int)atof(line.c_str());
    rb->mRelativeParticlePositions.resize(n > 0 ? n : 0);
    for (int i = 0; i < n; i++) {
        std::getline(file, line);
        std::istringstream ls(line);
        std::string a, b, c;
        ls >> a >> b >> c;
        rb->mRelativeParticlePositions[i] = make_float4((float)atof(a.c_str()), (float)atof(b.c_str()),
                                                        (float)atof(c.c_str()), rb->mParticleRadius);
    }
    const float I = 200.0f * (rb->mMass / 12.0f);
    rb->inertiaTensor.Ix = make_float4(I, 0.0f, 0.0f, 0.0f);
    rb->inertiaTensor.Iy = make_float4(0.0f, I, 0.0f, 0.0f);
    rb->inertiaTensor.Iz = make_float4(0.0f, 0.0f, I, 0.0f);
    rb->invInertiaTensor.Ix = make_float4(0.00125f, 0.0f, 0.0f, 0.0f);
    rb->invInertiaTensor.Iy = make_float4(0.0f, 0.00125f, 0.0f, 0.0f);
    rb->invInertiaTensor.Iz = make_float4(0.0f, 0.0f, 0.00125f, 0.0f);
    return rb;
}

/* --------------------------------------------------- RigidBodySimulator */

RigidBodySimulator *RigidBodySimulator::instance()
{
    static RigidBodySimulator inst;
    return &inst;
}

void RigidBodySimulator::addElement(RigidBody *rb)
{
    if (!rb) return;
    (rb->isStatic() ? mStatic : mDynamic).push_back(rb);
}

void RigidBodySimulator::reset()
{
    mDynamic.clear();
    mStatic.clear();
    mCoupled = nullptr;
    mInteractionStarted = false;
}

void RigidBodySimulator::release() { reset(); }

int RigidBodySimulator::getNumStaticParticles()
{
    int n = 0;
    for (auto *b : mStatic) n += b->getNumParticles();
    return n;
}

int RigidBodySimulator::getNumStaticRigidBodies() { return (int)mStatic.size(); }

int RigidBodySimulator::startInteraction()
{
    if (mInteractionStarted) return FG_E_STATE; /* RigidBodySimulator.cpp:313-323 asserts the same */
    mInteractionStarted = true;
    return FG_OK;
}

int RigidBodySimulator::endInteraction()
{
    if (!mInteractionStarted) return FG_E_STATE;
    mInteractionStarted = false;
    return FG_OK;
}

/* One rigid stage on the coupled fluid's world (built, or rebuilt with the
 * current bodies, by HeterogeneousSimulator::prepare). */
int RigidBodySimulator::coupled_stage(int stage)
{
    if (!mInteractionStarted) return FG_E_STATE;
    const int r = HeterogeneousSimulator::instance()->prepare();
    if (r != FG_OK) return r;
    if (!mCoupled || !mCoupled->world()) return FG_E_STATE;
    return fg_world_run_stage(mCoupled->world(), stage, 0);
}

int RigidBodySimulator::generateCollisionData() { return coupled_stage(FG_RUN_RB_GRID); }

int RigidBodySimulator::calculateRigidBodyForcesFromFluid(float4 *pos, float4 *vel, unsigned int *start,
                                                          unsigned int *end)
{
    if (!mInteractionStarted) return FG_E_STATE;
    int r = HeterogeneousSimulator::instance()->prepare();
    if (r != FG_OK) return r;
    Fluid::GPUSPHFluid *f = mCoupled;
    if (!f || !f->world()) return FG_E_STATE;
    const bool pos_ok = pos == f->getOrderedPosition() || pos == f->getPosition();
    const bool vel_ok = vel == f->getOrderedVelocities() || vel == f->getVelocity();
    if (!pos_ok || !vel_ok || start != f->getHashStart() || end != f->getHashEnd()) return FG_E_INVALID;
    return fg_world_run_stage(f->world(), FG_RUN_RB_FROM_FLUID, 0);
}

int RigidBodySimulator::calculateRigidBodyForcesFromRB() { return coupled_stage(FG_RUN_RB_FROM_RB); }
int RigidBodySimulator::applyForces() { return coupled_stage(FG_RUN_BODY_SUMS); }
int RigidBodySimulator::integrate() { return coupled_stage(FG_RUN_BODY_INTEGRATE); }

int RigidBodySimulator::getBodyState(double *x4, double *v4, double *q4, double *L4)
{
    if (!mCoupled || !mCoupled->world()) return FG_E_STATE;
    const int ids[4] = {FG_BUF_BODY_X, FG_BUF_BODY_V, FG_BUF_BODY_Q, FG_BUF_BODY_L};
    double *outs[4] = {x4, v4, q4, L4};
    int r = fg_world_sync(mCoupled->world());
    if (r != FG_OK) return r;
    for (int k = 0; k < 4; k++) {
        if (!outs[k]) continue;
        void *p = nullptr;
        size_t bytes = 0;
        if ((r = fg_world_buffer(mCoupled->world(), ids[k], &p, &bytes)) != FG_OK) return r;
        if ((r = fg_memcpy_d2h(outs[k], p, bytes)) != FG_OK) return r;
    }
    return FG_OK;
}

/* ----------------------------------------------- HeterogeneousSimulator */

HeterogeneousSimulator::HeterogeneousSimulator()
{
    /* KernelsCache, HeterogeneousSimulator.cpp:33-42 (the world computes the
     * same constants per scene; this keeps ApplicationData's copy filled) */
    Application::ApplicationData *ad = Application::ApplicationData::instance();
    const double h = (double)ad->getCommonFluidParams().kernel_radius;
    Application::KernelsCache k;
    k.kPoly6 = (float)(315.0f / ((double)(64.0f * Application::PI) * pow(h, 9)));
    k.kSpikyGradient = (float)(-(45.0f / ((double)Application::PI * pow(h, 6))));
    k.kViscosityLaplacian = (float)(45.0f / ((double)Application::PI * pow(h, 6)));
    ad->setKernelsCache(k);
}

HeterogeneousSimulator *HeterogeneousSimulator::instance()
{
    static HeterogeneousSimulator *inst = new HeterogeneousSimulator();
    return inst;
}

void HeterogeneousSimulator::addSphFluid(Fluid::GPUSPHFluid *fluid)
{
    if (fluid) mFluids.push_back(fluid);
}

int HeterogeneousSimulator::prepare()
{
    RigidBodySimulator *rbs = RigidBodySimulator::instance();
    const bool bodies = !rbs->mDynamic.empty() || !rbs->mStatic.empty();
    for (size_t i = 0; i < mFluids.size(); i++) {
        Fluid::GPUSPHFluid *f = mFluids[i];
        /* the bodies couple to the first fluid, as the reference's single
         * collision data set (RigidBodySimulator::getFluidCollisionData) */
        const bool want = bodies && i == 0;
        if (want != f->mHasBodies || !f->mWorld) {
            const int r = f->rebuild(want);
            if (r != FG_OK) return r;
            if (want) rbs->mCoupled = f;
        }
    }
    return FG_OK;
}

int HeterogeneousSimulator::fluid_stage(Fluid::GPUSPHFluid *fluid, int stage, int flags)
{
    if (!fluid) return FG_E_INVALID;
    const int r = prepare();
    if (r != FG_OK) return r;
    if (!fluid->mWorld) return FG_E_STATE;
    return fg_world_run_stage(fluid->mWorld, stage, flags);
}

int HeterogeneousSimulator::findFluidNeighbourhood(Fluid::GPUSPHFluid *f)
{
    return fluid_stage(f, FG_RUN_NEIGHBOURHOOD, 0);
}

int HeterogeneousSimulator::calculateFluidDensity(Fluid::GPUSPHFluid *f) { return fluid_stage(f, FG_RUN_DENSITY, 0); }

int HeterogeneousSimulator::calculateFluidForces(Fluid::GPUSPHFluid *f, bool useStaticRB, bool useDynamicRB)
{
    int flags = 0;
    if (f && f->mHasBodies) {
        RigidBodySimulator *rbs = RigidBodySimulator::instance();
        const bool has_s = !rbs->mStatic.empty(), has_d = !rbs->mDynamic.empty();
        const bool any = (has_s && useStaticRB) || (has_d && useDynamicRB);
        const bool all = (!has_s || useStaticRB) && (!has_d || useDynamicRB);
        if (any && !all) return FG_E_UNSUPPORTED;
        if (any) flags = FG_RUN_WITH_CONTACT;
    }
    return fluid_stage(f, FG_RUN_FORCES, flags);
}

int HeterogeneousSimulator::integrateFluidForces(Fluid::GPUSPHFluid *f) { return fluid_stage(f, FG_RUN_INTEGRATE, 0); }

int HeterogeneousSimulator::doTimeStep()
{
    int r0 = prepare();
    if (r0 != FG_OK) return r0;
    for (size_t i = 0; i < mFluids.size(); i++) {
        const int r = fg_world_step(mFluids[i]->mWorld, 1);
        if (r != FG_OK) return r;
    }
    for (auto *f : mFluids) {
        const int r = fg_world_sync(f->mWorld);
        if (r != FG_OK) return r;
    }
    return FG_OK;
}

} // namespace Simulators

namespace Fluid {

GPUSPHFluid::GPUSPHFluid(Application::FluidParams fp, Emitter::IEmitter *emitter)
    : mId(0), mFluidParams(fp), mEmitter(emitter), mWorld(nullptr), mHasBodies(false), mForces(nullptr)
{
    rebuild(false);
}

GPUSPHFluid::~GPUSPHFluid()
{
    if (mWorld) fg_world_destroy(mWorld);
    if (mForces) cudaFree(mForces);
}

/* Build (or rebuild, keeping positions and velocities) the fluid's world from
 * ApplicationData's common parameters, the fluid's parameters and -- when
 * coupled -- the RigidBodySimulator's bodies. */
int GPUSPHFluid::rebuild(bool with_bodies)
{
    using namespace Application;
    const CommonFluidParams &c = ApplicationData::instance()->getCommonFluidParams();
    const CommonRigidBodyParams &rp = ApplicationData::instance()->getCommonRigidBodyParams();
    const int n = mFluidParams.max_particles > 0 ? mFluidParams.max_particles : 0;
    std::vector<float4> pos(n), vel(n);
    if (mWorld) {
        int r = fg_world_download(mWorld, (float *)pos.data(), (float *)vel.data());
        if (r == FG_OK) r = fg_world_sync(mWorld);
        if (r != FG_OK) return r;
    } else {
        if (mEmitter && n) mEmitter->reset(pos.data(), n);
        for (auto &v : vel) v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    fg_scene_desc d;
    fg_scene_desc_defaults(&d);
    d.n_particles = (uint32_t)n;
    d.positions = (const float *)pos.data();
    d.velocities = (const float *)vel.data();
    d.cell_size[0] = c.cell_size.x; d.cell_size[1] = c.cell_size.y; d.cell_size[2] = c.cell_size.z;
    d.bucket_size[0] = c.bucket_size.x; d.bucket_size[1] = c.bucket_size.y; d.bucket_size[2] = c.bucket_size.z;
    d.kernel_radius = c.kernel_radius;
    d.velocity_limit = c.velocity_limit;
    d.volume_min[0] = c.volume_min.x; d.volume_min[1] = c.volume_min.y; d.volume_min[2] = c.volume_min.z;
    d.volume_max[0] = c.volume_max.x; d.volume_max[1] = c.volume_max.y; d.volume_max[2] = c.volume_max.z;
    d.gravity[0] = c.global_external_force.x;
    d.gravity[1] = c.global_external_force.y;
    d.gravity[2] = c.global_external_force.z;
    d.simulation_scale = c.simulation_scale;
    d.dt = c.deltaTimeIntegration;
    d.mass = mFluidParams.mass;
    d.rest_density = mFluidParams.restDensity;
    d.gas_constant = mFluidParams.gasConstant;
    d.viscosity = mFluidParams.viscosity;
    std::vector<fg_body_desc> bd;
    std::vector<std::vector<float>> loc;
    if (with_bodies) {
        Simulators::RigidBodySimulator *rbs = Simulators::RigidBodySimulator::instance();
        std::vector<Simulators::RigidBody *> all(rbs->mDynamic);
        all.insert(all.end(), rbs->mStatic.begin(), rbs->mStatic.end());
        for (auto *b : all) {
            fg_body_desc e;
            memset(&e, 0, sizeof(e));
            std::vector<float> l(4 * (size_t)b->getNumParticles());
            memcpy(l.data(), b->getRelativeParticlePositions(), l.size() * sizeof(float));
            loc.push_back(std::move(l));
            e.n_spheres = (uint32_t)b->getNumParticles();
            e.mass = b->isStatic() ? 0.0f : b->getMass();
            const float3 p = b->getPosition();
            const float4 q = b->getOrientation();
            e.position[0] = p.x; e.position[1] = p.y; e.position[2] = p.z;
            e.orientation[0] = q.x; e.orientation[1] = q.y; e.orientation[2] = q.z; e.orientation[3] = q.w;
            const Simulators::sInertiaTensor I = b->getInvInertiaTensor();
            const float m[9] = {I.Ix.x, I.Ix.y, I.Ix.z, I.Iy.x, I.Iy.y, I.Iy.z, I.Iz.x, I.Iz.y, I.Iz.z};
            memcpy(e.inv_inertia, m, sizeof(m));
            bd.push_back(e);
        }
        for (size_t k = 0; k < bd.size(); k++) bd[k].local_spheres = loc[k].data();
        d.n_bodies = (uint32_t)bd.size();
        d.bodies = bd.empty() ? nullptr : bd.data();
        if (!all.empty()) {
            d.fluid_radius = mFluidParams.particle_radius > 0.0f ? mFluidParams.particle_radius : c.pointRadius;
            d.rb_radius = all[0]->getParticleRadius() > 0.0f ? all[0]->getParticleRadius() : rp.particleRadius;
        }
        d.rb_bucket_size[0] = rp.dn_bucket_size.x;
        d.rb_bucket_size[1] = rp.dn_bucket_size.y;
        d.rb_bucket_size[2] = rp.dn_bucket_size.z;
        d.fluid_to_rb_relation[0] = c.fluid_to_srb_relation.x;
        d.fluid_to_rb_relation[1] = c.fluid_to_srb_relation.y;
        d.fluid_to_rb_relation[2] = c.fluid_to_srb_relation.z;
        d.rb_to_fluid_relation[0] = rp.rb_to_fluid_relation.x;
        d.rb_to_fluid_relation[1] = rp.rb_to_fluid_relation.y;
        d.rb_to_fluid_relation[2] = rp.rb_to_fluid_relation.z;
        d.rb_gravity[0] = rp.global_external_force.x;
        d.rb_gravity[1] = rp.global_external_force.y;
        d.rb_gravity[2] = rp.global_external_force.z;
        d.rb_gravity[3] = rp.global_external_force.w;
        d.rb_velocity_limit = rp.velocity_limit;
        d.rb_dt = rp.deltaTimeIntegration > 0.0f ? rp.deltaTimeIntegration : c.deltaTimeIntegration;
        d.rb_volume_min[0] = rp.volume_min.x; d.rb_volume_min[1] = rp.volume_min.y; d.rb_volume_min[2] = rp.volume_min.z;
        d.rb_volume_max[0] = rp.volume_max.x; d.rb_volume_max[1] = rp.volume_max.y; d.rb_volume_max[2] = rp.volume_max.z;
        d.rb_rb_contact = rbs->mDynamic.size() + rbs->mStatic.size() > 1 ? 1 : 0;
    }
    fg_world *w = nullptr;
    const int r = fg_world_create(&d, 1, nullptr, &w);
    if (r != FG_OK) return r;
    if (mWorld) fg_world_destroy(mWorld);
    mWorld = w;
    mHasBodies = with_bodies;
    return FG_OK;
}

void *GPUSPHFluid::buffer(int id)
{
    void *p = nullptr;
    size_t b = 0;
    if (!mWorld || fg_world_buffer(mWorld, id, &p, &b) != FG_OK) return nullptr;
    return p;
}

unsigned int *GPUSPHFluid::getHashKey() { return (unsigned int *)buffer(FG_BUF_KEYS); }
unsigned int *GPUSPHFluid::getParticleID() { return (unsigned int *)buffer(FG_BUF_IDS); }
unsigned int *GPUSPHFluid::getHashStart() { return (unsigned int *)buffer(FG_BUF_START); }
unsigned int *GPUSPHFluid::getHashEnd() { return (unsigned int *)buffer(FG_BUF_END); }
float4 *GPUSPHFluid::getPosition() { return (float4 *)buffer(FG_BUF_POS); }
float4 *GPUSPHFluid::getOrderedPosition() { return (float4 *)buffer(FG_BUF_SPOS); }
float4 *GPUSPHFluid::getOrderedVelocities() { return (float4 *)buffer(FG_BUF_SVEL); }
float4 *GPUSPHFluid::getVelocity() { return (float4 *)buffer(FG_BUF_VEL); }
float2 *GPUSPHFluid::getDensityField() { return (float2 *)buffer(FG_BUF_DP); }

/* The reference allocates d_forces and never fills it (GPUSPHFluid.cpp:17-25;
 * SPHIntegrateK takes it unused); forces go straight into the velocity here
 * too, so this is a zeroed device array of n float4, allocated on first use. */
float4 *GPUSPHFluid::getForces()
{
    if (!mForces && mFluidParams.max_particles > 0) {
        const size_t b = 16 * (size_t)mFluidParams.max_particles;
        if (cudaMalloc(&mForces, b) != cudaSuccess || cudaMemset(mForces, 0, b) != cudaSuccess) {
            cudaGetLastError();
            if (mForces) cudaFree(mForces);
            mForces = nullptr;
        }
    }
    return mForces;
}

/* GPUSPHFluid.cpp:94-95 copies max_particles bytes; this copies the whole
 * n x float4 array. */
int GPUSPHFluid::copyPositionToCPU(float4 **out)
{
    if (!out || !mWorld) return 0;
    const int n = getNumParticles();
    if (!*out) *out = new float4[n > 0 ? n : 1];
    if (fg_world_download(mWorld, (float *)*out, nullptr) != FG_OK || fg_world_sync(mWorld) != FG_OK) return 0;
    return n;
}

} // namespace Fluid
} // namespace Simulation
