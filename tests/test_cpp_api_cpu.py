"""The headless C++ mirror's host-only parts, run here without a GPU:
BlockEmitter's lattice fill (Emitter.cpp:16-43) and RigidBody::loadFromFile's
text format (RigidBody.cpp:55-126)."""
import os
import shutil

import numpy as np
import pytest

import cpp_api

pytestmark = pytest.mark.skipif(not shutil.which("g++") or not os.path.exists(
    os.path.join(cpp_api.CUDA_INC, "vector_types.h")) or not os.path.exists(
    os.path.join(cpp_api.LIBDIR, "libfluidgrid_gb300.so")), reason="needs g++, CUDA headers and the built library")


def emitter_reference(bmin, bmax, spacing, count):
    """Emitter.cpp:16-43 restated with float32 loop counters."""
    out = []
    y = np.float32(bmin[1])
    sp = np.float32(spacing)
    while len(out) < count:
        z = np.float32(bmin[2])
        while z < np.float32(bmax[2]):
            x = np.float32(bmin[0])
            while x < np.float32(bmax[0]):
                if len(out) < count:
                    out.append((x, y, z, 1.0))
                x = np.float32(x + sp)
            z = np.float32(z + sp)
        y = np.float32(y + sp)
    return np.array(out, np.float32)


def test_block_emitter_fills_layers_upwards(tmp_path):
    src = r"""
#include <cstdio>
#include "fluidgrid_sim.hpp"
int main() {
    Simulation::Emitter::BlockEmitter e(mc::math::Vec3f(%s, %s, %s), mc::math::Vec3f(%s, %s, %s), %s);
    float4 p[1000];
    e.reset(p, 1000);
    for (int i = 0; i < 1000; i++) printf("%%a %%a %%a %%a\n", p[i].x, p[i].y, p[i].z, p[i].w);
    return 0;
}
""" % tuple(cpp_api.f32(v) for v in (0.1, 0.2, 0.3, 0.3, 0.5, 0.45, 0.02285))
    out = cpp_api.build_and_run(src, cwd=str(tmp_path))
    got = np.array([[float.fromhex(t) for t in ln.split()] for ln in out.splitlines()], np.float32)
    ref = emitter_reference((0.1, 0.2, 0.3), (0.3, 0.5, 0.45), 0.02285, 1000)
    assert np.array_equal(got, ref)


def test_rigid_body_file_format(tmp_path):
    body = tmp_path / "box.rb"
    pts = np.random.default_rng(4).uniform(-0.2, 0.2, (37, 3))
    body.write_text("dynamic\n12.5\n0.02285\nbox.obj\n37\n" + "".join("%.17g %.17g %.17g\n" % tuple(p) for p in pts))
    still = tmp_path / "floor.rb"
    still.write_text("static\n0.04\nfloor.obj\n2\n0 0 0\n1 0 0\n")
    src = r"""
#include <cstdio>
#include "fluidgrid_sim.hpp"
using Simulation::Simulators::RigidBody;
int main() {
    const char *names[2] = {"box.rb", "floor.rb"};
    for (int f = 0; f < 2; f++) {
        RigidBody *b = RigidBody::loadFromFile(names[f]);
        printf("%d %a %a %d %s\n", b->isStatic() ? 1 : 0, b->getMass(), b->getParticleRadius(), b->getNumParticles(),
               b->getMeshFilename().c_str());
        printf("%a %a\n", b->getInertiaTensor().Ix.x, b->getInvInertiaTensor().Iz.z);
        for (int i = 0; i < b->getNumParticles(); i++) {
            float4 p = b->getRelativeParticlePositions()[i];
            printf("%a %a %a %a\n", p.x, p.y, p.z, p.w);
        }
        delete b;
    }
    return 0;
}
"""
    out = cpp_api.build_and_run(src, cwd=str(tmp_path)).splitlines()
    st, mass, rad, n, mesh = out[0].split()
    assert (st, int(n), mesh) == ("0", 37, "box.obj")
    assert float.fromhex(mass) == np.float32(12.5) and float.fromhex(rad) == np.float32(0.02285)
    I, inv = [float.fromhex(t) for t in out[1].split()]
    assert I == np.float32(200.0 * np.float32(np.float32(12.5) / np.float32(12.0)))
    assert inv == np.float32(0.00125)
    got = np.array([[float.fromhex(t) for t in ln.split()] for ln in out[2:2 + 37]], np.float32)
    assert np.array_equal(got[:, :3], pts.astype(np.float32)) and np.all(got[:, 3] == np.float32(0.02285))
    st, mass, rad, n, mesh = out[39].split()
    assert (st, int(n), mesh) == ("1", 2, "floor.obj") and float.fromhex(mass) == 0.0
