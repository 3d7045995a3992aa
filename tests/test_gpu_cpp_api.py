"""The headless C++ mirror of the reference's simulation classes on the GPU:
a program written against GPUSPHFluid / HeterogeneousSimulator /
RigidBodySimulator (include/fluidgrid_sim.hpp) steps the same bits as the
world API given the same scene."""
import os
import shutil

import numpy as np
import pytest

import cpp_api
from cpp_api import f32
from fluidgrid_gb300 import World, build
from fluidgrid_gb300.scenes import H, SPACING, SceneSpec, Body
from test_cpp_api_cpu import emitter_reference

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not shutil.which("g++"), reason="needs g++")]

BMIN, BMAX, N = (0.02, 0.02, 0.02), (0.5, 0.6, 0.5), 12000


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


# the reference's commented two-way step (HeterogeneousSimulator.cpp:57-126,
# RigidBodySimulator.cpp:313-611) written against the mirror's stage methods,
# with a call out of order first (applyForces before any sphere force: the
# world refuses it and stays usable)
STAGED_LOOP = r"""
    RigidBodySimulator *rbs = RigidBodySimulator::instance();
    HeterogeneousSimulator *hs = HeterogeneousSimulator::instance();
    if (rbs->applyForces() != FG_E_STATE) return 20;  /* interaction not started */
    for (int s = 0; s < %(steps)d; s++) {
        if (rbs->startInteraction()) return 2;
        if (hs->findFluidNeighbourhood(&fluid)) return 3;
        if (s == 0 && rbs->applyForces() != FG_E_STATE) return 21;  /* no sphere forces yet */
        if (hs->calculateFluidDensity(&fluid)) return 4;
        if (rbs->generateCollisionData()) return 5;
        if (rbs->calculateRigidBodyForcesFromFluid(fluid.getPosition(), fluid.getVelocity(), fluid.getHashStart(),
                                                   fluid.getHashEnd())) return 6;
        if (rbs->calculateRigidBodyForcesFromRB()) return 7;
        if (hs->calculateFluidForces(&fluid, rbs->getNumStaticRigidBodies() > 0, true)) return 8;
        if (rbs->applyForces()) return 9;
        if (rbs->integrate()) return 10;
        if (hs->integrateFluidForces(&fluid)) return 11;
        if (rbs->endInteraction()) return 12;
    }
"""

WHOLE_LOOP = r"""
    for (int s = 0; s < %(steps)d; s++)
        if (HeterogeneousSimulator::instance()->doTimeStep() != 0) return 1;
"""


def _program(steps, body_file=None, body_pos=(0.25, 0.55, 0.25), bodies=None, staged=False):
    spec = SceneSpec(pos=np.zeros((1, 4), np.float32))  # defaults only
    if bodies is None:
        bodies = [(body_file, body_pos)] if body_file else []
    body = "".join(r"""
    {
        RigidBody *rb = RigidBody::loadFromFile("%s");
        rb->setPosition(make_float3(%s, %s, %s));
        RigidBodySimulator::instance()->addElement(rb);
    }""" % ((f,) + tuple(f32(v) for v in p)) for f, p in bodies)
    loop = (STAGED_LOOP if staged else WHOLE_LOOP) % dict(steps=steps)
    return r"""
#include <cstdio>
#include "fluidgrid_sim.hpp"
using namespace Simulation;
using namespace Simulation::Simulators;
int main() {
    Application::CommonFluidParams &c = Application::ApplicationData::instance()->getCommonFluidParams();
    c.cell_size = make_float3(%(h)s, %(h)s, %(h)s);
    c.bucket_size = make_int3(64, 64, 64);
    c.kernel_radius = %(h)s;
    c.velocity_limit = %(vl)s;
    c.volume_min = make_float3(0.0f, 0.0f, 0.0f);
    c.volume_max = make_float3(1.0f, 1.0f, 1.0f);
    c.global_external_force = make_float3(0.0f, %(g)s, 0.0f);
    c.simulation_scale = 1.0f;
    c.deltaTimeIntegration = %(dt)s;
    c.fluid_to_srb_relation = make_int3(2, 2, 2);
    Application::CommonRigidBodyParams &r = Application::ApplicationData::instance()->getCommonRigidBodyParams();
    r.rb_to_fluid_relation = make_int3(1, 1, 1);
    r.dn_bucket_size = make_int3(32, 32, 32);
    r.velocity_limit = %(vl)s;
    r.volume_min = make_float3(0.0f, 0.0f, 0.0f);
    r.volume_max = make_float3(1.0f, 1.0f, 1.0f);
    r.global_external_force = make_float4(0.0f, %(g)s, 0.0f, 0.0f);
    r.deltaTimeIntegration = %(dt)s;
    r.particleRadius = %(rr)s;
    Emitter::BlockEmitter em(mc::math::Vec3f(%(b0)s, %(b1)s, %(b2)s), mc::math::Vec3f(%(e0)s, %(e1)s, %(e2)s), %(sp)s);
    Application::FluidParams fp = {%(m)s, %(rho)s, %(mu)s, 0.0f, %(fr)s, %(k)s, %(n)d};
    Fluid::GPUSPHFluid fluid(fp, &em);
    %(body)s
    HeterogeneousSimulator::instance()->addSphFluid(&fluid);
    %(loop)s
    float4 *p = nullptr;
    const int n = fluid.copyPositionToCPU(&p);
    for (int i = 0; i < n; i++) printf("%%a %%a %%a %%a\n", p[i].x, p[i].y, p[i].z, p[i].w);
    double bx[4 * 8] = {0};  /* 4 doubles per body */
    if (RigidBodySimulator::instance()->getBodyState(bx, nullptr, nullptr, nullptr) == 0)
        printf("body %%a %%a %%a\n", bx[0], bx[1], bx[2]);
    delete[] p;
    return 0;
}
""" % dict(h=f32(H), vl=f32(spec.vlimit), g=f32(-9.8), dt=f32(spec.dt), rr=f32(spec.rb_radius),
           b0=f32(BMIN[0]), b1=f32(BMIN[1]), b2=f32(BMIN[2]), e0=f32(BMAX[0]), e1=f32(BMAX[1]), e2=f32(BMAX[2]),
           sp=f32(SPACING), m=f32(spec.mass), rho=f32(spec.rest), mu=f32(spec.visc), fr=f32(spec.fluid_radius),
           k=f32(spec.gas), n=N, body=body, loop=loop)


def _parse(out):
    lines = out.splitlines()
    pos = np.array([[float.fromhex(t) for t in ln.split()] for ln in lines if not ln.startswith("body")], np.float32)
    body = [ln for ln in lines if ln.startswith("body")]
    return pos, ([float.fromhex(t) for t in body[0].split()[1:]] if body else None)


def _world_run(steps, bodies=(), rb_rb=False):
    pos0 = emitter_reference(BMIN, BMAX, SPACING, N)
    spec = SceneSpec(pos=pos0, box_min=(0, 0, 0), box_max=(1, 1, 1), buckets=(64, 64, 64), bodies=list(bodies),
                     rb_buckets=(32, 32, 32), rb_rb=rb_rb)
    w = World([spec])
    w.step(steps)
    p, _ = w.download()
    bx = w.read("BODY_X")[0, :3] if bodies else None
    w.close()
    return p, bx


def test_cpp_fluid_steps_equal_world(tmp_path):
    out = cpp_api.build_and_run(_program(6), cwd=str(tmp_path))
    got, _ = _parse(out)
    ref, _ = _world_run(6)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_cpp_fluid_with_rigid_body_equals_world(tmp_path):
    rng = np.random.default_rng(2)
    pts = rng.uniform(-0.06, 0.06, (300, 3))
    f = tmp_path / "cube.rb"
    f.write_text("dynamic\n2.0\n%.17g\ncube.obj\n300\n" % float(np.float32(0.5 * H)) +
                 "".join("%.17g %.17g %.17g\n" % tuple(p) for p in pts))
    out = cpp_api.build_and_run(_program(4, body_file="cube.rb"), cwd=str(tmp_path))
    got, bx = _parse(out)
    loc = np.zeros((300, 4), np.float32)
    loc[:, :3] = pts.astype(np.float32)
    body = Body(local=loc, mass=2.0, position=(0.25, 0.55, 0.25), orientation=(0.0, 0.0, 0.0, 1.0))
    ref, rbx = _world_run(4, [body])
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert bx is not None and np.array_equal(np.array(bx), rbx)
    assert bx[1] != np.float32(0.55)  # the body moved (it starts inside the block: contact lifts it)


def test_cpp_staged_step_order_equals_world(tmp_path):
    """The stage methods in the reference's commented order, with a dynamic
    cloud of spheres resting on a static plate, give the world's bits."""
    rng = np.random.default_rng(2)
    pts = rng.uniform(-0.06, 0.06, (300, 3))
    r = float(np.float32(0.5 * H))
    (tmp_path / "cube.rb").write_text("dynamic\n2.0\n%.17g\ncube.obj\n300\n" % r +
                                      "".join("%.17g %.17g %.17g\n" % tuple(p) for p in pts))
    g = np.linspace(-0.08, 0.08, 9)
    plate = np.array([(x, 0.0, z) for x in g for z in g])
    # a static body's file has no mass line (RigidBody.cpp:65-79)
    (tmp_path / "plate.rb").write_text("static\n%.17g\nplate.obj\n%d\n" % (r, len(plate)) +
                                       "".join("%.17g %.17g %.17g\n" % tuple(p) for p in plate))
    placed = [("cube.rb", (0.25, 0.55, 0.25)), ("plate.rb", (0.25, 0.48, 0.25))]
    steps = 5
    out = cpp_api.build_and_run(_program(steps, bodies=placed, staged=True), cwd=str(tmp_path))
    got, bx = _parse(out)
    out_whole = cpp_api.build_and_run(_program(steps, bodies=placed), cwd=str(tmp_path))
    whole, bxw = _parse(out_whole)
    # the same scene through the world API: dynamic bodies first, then static
    loc = np.zeros((300, 4), np.float32)
    loc[:, :3] = pts.astype(np.float32)
    ploc = np.zeros((len(plate), 4), np.float32)
    ploc[:, :3] = plate.astype(np.float32)
    cube = Body(local=loc, mass=2.0, position=placed[0][1], orientation=(0.0, 0.0, 0.0, 1.0))
    slab = Body(local=ploc, mass=0.0, position=placed[1][1], orientation=(0.0, 0.0, 0.0, 1.0))
    ref, rbx = _world_run(steps, [cube, slab], rb_rb=True)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(whole.view(np.uint32), ref.view(np.uint32))
    assert bx is not None and np.array_equal(np.array(bx), rbx) and np.array_equal(np.array(bxw), rbx)
    assert bx[1] != np.float32(0.55)
