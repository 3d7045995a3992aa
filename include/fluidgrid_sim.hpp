// fluidgrid_gb300 -- headless C++ mirror of FluidGrid's simulation classes.
//
// The class and method names of the reference's host API, in its
// namespaces, so host code written against it builds unchanged:
//   Simulation::Fluid::GPUSPHFluid            (GPUSPHFluid.h:30-131)
//   Simulation::Simulators::HeterogeneousSimulator (HeterogeneousSimulator.h:41-45)
//   Simulation::Simulators::RigidBodySimulator (Simulators/RigidBodySimulator.h:136-165)
//   Simulation::Simulators::RigidBody::loadFromFile (Simulators/RigidBody.cpp:55-126)
//   Simulation::Emitter::IEmitter / BlockEmitter (Emitter.h, Emitter.cpp:16-43)
//   Simulation::Application::FluidParams / CommonFluidParams /
//   CommonRigidBodyParams / KernelsCache / ApplicationData (ApplicationData.cuh)
//
// Headless: beginUpdate()/endUpdate() do nothing, getPosition() returns a
// device buffer (no GL interop), render() does not exist.  Every fluid is a
// one-scene world of libfluidgrid_gb300.so; doTimeStep() runs the whole step
// (hash, sort, ranges, density, forces, walls, integration -- and the
// two-way coupling with the RigidBodySimulator's bodies, the reference's
// commented block HeterogeneousSimulator.cpp:57-126) as one captured graph.
// Device pointers returned by the getters are owned by the fluid and stay
// valid until it is destroyed, except that the first doTimeStep() (or stage
// call) after bodies were added rebuilds the fluid's world (and its buffers).
//
// Host code that sequences the step itself, as the reference's commented
// two-way block does, calls the stage methods instead of doTimeStep():
//   RigidBodySimulator::startInteraction();
//   HeterogeneousSimulator::findFluidNeighbourhood(f);
//   HeterogeneousSimulator::calculateFluidDensity(f);
//   RigidBodySimulator::generateCollisionData();
//   RigidBodySimulator::calculateRigidBodyForcesFromFluid(...);
//   RigidBodySimulator::calculateRigidBodyForcesFromRB();   (bodies that touch)
//   HeterogeneousSimulator::calculateFluidForces(f, useStaticRB, useDynamicRB);
//   RigidBodySimulator::applyForces();
//   RigidBodySimulator::integrate();
//   HeterogeneousSimulator::integrateFluidForces(f);
//   RigidBodySimulator::endInteraction();
// Each enqueues one stage of the coupled world (fg_world_run_stage) and
// returns 0 or an fg_status: FG_E_STATE when a stage's inputs were not made
// earlier in the same step.  The stages run the kernels of doTimeStep(), so
// the result is the same bits.  The reference's methods return void; these
// return the status, which callers may ignore.
#ifndef FLUIDGRID_SIM_HPP
#define FLUIDGRID_SIM_HPP

#include <string>
#include <vector>
#include <vector_functions.h> /* make_float3/make_float4/make_int3 for host code */
#include <vector_types.h>
#include "fluidgrid_gb300.h"
#include "fluidgrid_reference.h"

namespace mc {
namespace math {
// the jrfxgl vector the reference's BlockEmitter takes
struct Vec3f {
    float x, y, z;
    Vec3f() : x(0), y(0), z(0) {}
    Vec3f(float a, float b, float c) : x(a), y(b), z(c) {}
};
} // namespace math
} // namespace mc

namespace Simulation {

namespace Application {

const float PI = 3.14159265f;

struct FluidParams {
    float mass;
    float restDensity;
    float viscosity;
    float stiffness;
    float particle_radius; // contact radius against rigid-body spheres
    float gasConstant;
    int max_particles;
};

struct CommonFluidParams : fgr_common_fluid_params {
    int getNumBuckets() const { return bucket_size.x * bucket_size.y * bucket_size.z; }
};

struct CommonRigidBodyParams {
    int3 rb_to_fluid_relation;
    int3 st_bucket_size;
    int3 dn_bucket_size;
    unsigned int st_keyBits;
    float velocity_limit;
    float3 volume_min;
    float3 volume_max;
    float4 global_external_force;
    float simulation_scale;
    float deltaTimeIntegration;
    float particleRadius;
    int getStNumBuckets() const { return st_bucket_size.x * st_bucket_size.y * st_bucket_size.z; }
    int getDnNumBuckets() const { return dn_bucket_size.x * dn_bucket_size.y * dn_bucket_size.z; }
    float3 getCellSize() const
    {
        float3 c;
        c.x = c.y = c.z = particleRadius;
        return c;
    }
};

typedef fgr_kernels_cache KernelsCache;

class ApplicationData {
public:
    static ApplicationData *instance();
    CommonFluidParams &getCommonFluidParams() { return mCommonFluidParams; }
    KernelsCache &getKernelsCache() { return mKernelsCache; }
    CommonRigidBodyParams &getCommonRigidBodyParams() { return mCommonRigidBodyParams; }
    void setCommonFluidParams(CommonFluidParams p) { mCommonFluidParams = p; }
    void setCommonRigidBodyParams(CommonRigidBodyParams p) { mCommonRigidBodyParams = p; }
    void setKernelsCache(KernelsCache k) { mKernelsCache = k; }

private:
    ApplicationData();
    CommonFluidParams mCommonFluidParams;
    KernelsCache mKernelsCache;
    CommonRigidBodyParams mCommonRigidBodyParams;
};

} // namespace Application

namespace Fluid {
class GPUSPHFluid;
}

namespace Emitter {

class IEmitter {
public:
    virtual ~IEmitter() {}
    virtual void update(Simulation::Fluid::GPUSPHFluid *fluid) = 0;
    virtual void reset(float4 *positions, int count) = 0;
};

// Lattice fill of a block, layer by layer upwards (w = 1); slots left over
// are inactive (w = -1).
class BlockEmitter : public IEmitter {
public:
    BlockEmitter(mc::math::Vec3f block_min, mc::math::Vec3f block_max, float particle_spacing);
    void reset(float4 *positions, int count);
    void update(Simulation::Fluid::GPUSPHFluid *) {}
    void UpdateData() {}

private:
    mc::math::Vec3f mBlockSizeMin, mBlockSizeMax;
    float mParticleSpacing;
};

} // namespace Emitter

namespace Simulators {
class HeterogeneousSimulator;
}

namespace Fluid {

class GPUSPHFluid {
public:
    GPUSPHFluid(Application::FluidParams fluidParams, Emitter::IEmitter *emitter);
    ~GPUSPHFluid();

    void beginUpdate() {}
    void endUpdate() {}

    unsigned int *getHashKey();
    unsigned int *getParticleID();
    unsigned int *getHashStart();
    unsigned int *getHashEnd();
    // Copies the positions to *particlePositions (allocated with new[] when
    // NULL); returns the particle count.
    int copyPositionToCPU(float4 **particlePositions);
    float4 *getPosition();
    float4 *getOrderedPosition();
    float4 *getOrderedVelocities();
    float4 *getVelocity();
    // the reference allocates a force buffer it never fills; forces go
    // straight into the velocity here too: a zeroed device array of n float4
    float4 *getForces();
    float2 *getDensityField();
    int getNumParticles() { return mFluidParams.max_particles; }
    float getGasConstant() { return mFluidParams.gasConstant; }
    float getRestDensity() { return mFluidParams.restDensity; }
    float getMass() { return mFluidParams.mass; }
    float getViscosity() { return mFluidParams.viscosity; }

    fg_world *world() { return mWorld; }

public:
    int mId;
    Application::FluidParams mFluidParams;
    Emitter::IEmitter *mEmitter;

private:
    friend class Simulators::HeterogeneousSimulator;
    void *buffer(int id);
    int rebuild(bool with_bodies);
    fg_world *mWorld;
    bool mHasBodies;
    float4 *mForces;
};

} // namespace Fluid

namespace Simulators {

struct sInertiaTensor {
    float4 Ix, Iy, Iz;
};

class RigidBody {
public:
    RigidBody();
    ~RigidBody();
    // Text format: "static" | "dynamic" then the mass, the sphere radius, the
    // source mesh name, the sphere count, then one "x y z" line per sphere.
    static RigidBody *loadFromFile(std::string filename);

    float4 *getRelativeParticlePositions() { return mRelativeParticlePositions.data(); }
    int getNumParticles() { return (int)mRelativeParticlePositions.size(); }
    float getParticleRadius() { return mParticleRadius; }
    float getMass() { return mMass; }
    bool isStatic() { return mIsStatic; }
    sInertiaTensor getInertiaTensor() { return inertiaTensor; }
    sInertiaTensor getInvInertiaTensor() { return invInertiaTensor; }
    const std::string &getMeshFilename() { return mOriginalMeshFilename; }

    // pose (the scene-graph node of the reference)
    void setPosition(float3 p) { mPosition = p; }
    float3 getPosition() { return mPosition; }
    void setOrientation(float4 q) { mOrientation = q; }
    float4 getOrientation() { return mOrientation; }

private:
    std::vector<float4> mRelativeParticlePositions;
    bool mIsStatic;
    float mParticleRadius;
    float mMass;
    std::string mOriginalMeshFilename;
    sInertiaTensor inertiaTensor;
    sInertiaTensor invInertiaTensor;
    float3 mPosition;
    float4 mOrientation;
};

class RigidBodySimulator {
public:
    static RigidBodySimulator *instance();

    void addElement(RigidBody *rbElement);
    void reset();
    void release();

    int getNumStaticParticles();
    int getNumStaticRigidBodies();
    int getNumDynamicRigidBodies() { return (int)mDynamic.size(); }

    // Stages of the two-way step on the coupled fluid's world (the first
    // fluid added to the HeterogeneousSimulator), in the order of
    // RigidBodySimulator.cpp:313-611.  doTimeStep() runs them all itself.
    //   startInteraction/endInteraction  bracket one step (FG_E_STATE when
    //                                    started twice or ended unstarted)
    //   generateCollisionData            sphere world positions, keys, sort,
    //                                    cell ranges of every body (resident:
    //                                    no host broad phase or upload)
    //   calculateRigidBodyForcesFromFluid  sphere force/torque from the fluid;
    //                                    the arguments must be the coupled
    //                                    fluid's buffers (its sorted or, as
    //                                    the reference's commented call passes
    //                                    them, unsorted positions/velocities
    //                                    and its start/end): the fluid's grid
    //                                    is used either way
    //   calculateRigidBodyForcesFromRB   + contact with the other bodies and
    //                                    with static ones (mass 0)
    //   applyForces                      FP64 per-body force/torque sums
    //   integrate                        FP64 body integration
    int generateCollisionData();
    int startInteraction();
    int endInteraction();
    int calculateRigidBodyForcesFromRB();
    int calculateRigidBodyForcesFromFluid(float4 *dfluidParticlePos, float4 *dfluidParticleVel,
                                          unsigned int *dfluidHashStart, unsigned int *dfluidHashEnd);
    int applyForces();
    int integrate();

    // FP64 body state after the last step of the fluid the bodies are
    // coupled to: x (position), v, q (orientation), L per body, 4 doubles
    // each, so every non-null array holds 4 x (dynamic + static bodies)
    // doubles; dynamic bodies come first, in the order they were added
    int getBodyState(double *x4, double *v4, double *q4, double *L4);

    const std::vector<RigidBody *> &dynamicBodies() { return mDynamic; }
    const std::vector<RigidBody *> &staticBodies() { return mStatic; }

private:
    RigidBodySimulator() {}
    friend class HeterogeneousSimulator;
    friend class Fluid::GPUSPHFluid;
    int coupled_stage(int stage);
    std::vector<RigidBody *> mDynamic, mStatic;
    Fluid::GPUSPHFluid *mCoupled = nullptr;
    bool mInteractionStarted = false;
};

class HeterogeneousSimulator {
public:
    static HeterogeneousSimulator *instance();
    void addSphFluid(Fluid::GPUSPHFluid *fluid);
    // One step of every fluid: findFluidNeighbourhood, calculateFluidDensity,
    // calculateFluidForces, integrateFluidForces (HeterogeneousSimulator.cpp:
    // 54-127), plus the rigid-body coupling of the first fluid when the
    // RigidBodySimulator holds bodies.  Returns 0 or an fg_status.
    int doTimeStep();

    // The fluid stages of doTimeStep (private in the reference, public here
    // for host code that sequences the two-way step itself).  With bodies,
    // calculateFluidForces adds the contact term when the flags ask for every
    // kind of body present (static = mass 0, dynamic); asking for only one of
    // two kinds present returns FG_E_UNSUPPORTED, since both share one grid.
    // integrateFluidForces ends the step.
    int findFluidNeighbourhood(Fluid::GPUSPHFluid *fluid);
    int calculateFluidDensity(Fluid::GPUSPHFluid *fluid);
    int calculateFluidForces(Fluid::GPUSPHFluid *fluid, bool useStaticRB, bool useDynamicRB);
    int integrateFluidForces(Fluid::GPUSPHFluid *fluid);

private:
    HeterogeneousSimulator();
    friend class RigidBodySimulator;
    int prepare(); /* (re)build the fluids' worlds for the current bodies */
    int fluid_stage(Fluid::GPUSPHFluid *fluid, int stage, int flags);
    std::vector<Fluid::GPUSPHFluid *> mFluids;
};

} // namespace Simulators
} // namespace Simulation

#endif
