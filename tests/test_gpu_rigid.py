"""GPU parity of the two-way fluid/rigid step against the oracle from an
identical state: sphere transform + keys, rigid grid (bit-exact), per-sphere
contact force and torque, fluid-side contact term in the force kernel, FP64
per-body reduction and FP64 body integration.

Tolerances:
  sphere force/torque : |x_gpu - x_ref| <= 1e-4 * max(|x_ref|, median|x_ref|)
  body force/torque   : FP64 sum of the GPU's per-sphere values, rtol 1e-12
  body state (FP64)   : rtol 1e-12 (same arithmetic, reassociation only)
"""
import dataclasses

import numpy as np
import pytest

from fluidgrid_gb300 import World, build
from fluidgrid_gb300.scenes import H, SPACING, SceneSpec, Body, lattice, box_surface, sphere_surface, \
    random_quaternion
from oracle import oracle as O
import helpers as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def rigid_scene(seed=1, nbodies=1, rb_rb=False):
    rng = np.random.default_rng(seed)
    pos = lattice(32, 16, 32, SPACING, (SPACING, SPACING, SPACING), 0.05 * H, rng)
    bodies = []
    for b in range(nbodies):
        c = (0.25 + 0.3 * b, 0.38, 0.37)  # straddles the fluid surface at y ~ 0.37
        loc = box_surface(0.2, 1024, rng) if b % 2 == 0 else sphere_surface(0.12, 700)
        bodies.append(Body(local=loc, mass=10.0, position=c, orientation=random_quaternion(rng)))
    return SceneSpec(pos=pos, box_min=(0, 0, 0), box_max=(1, 1, 1), buckets=(64, 64, 64), bodies=bodies,
                     rb_buckets=(32, 32, 32), rb_rb=rb_rb, name="rigid_small")


def _run(spec, vel0=None):
    w = World([spec])
    pos0 = spec.pos.copy()
    v0 = np.zeros_like(pos0) if vel0 is None else vel0
    w.upload(pos0, v0)
    before = {k: w.read(k) for k in ("RB_LOCAL", "BODY_X", "BODY_V", "BODY_Q", "BODY_L", "BODY_XF", "BODY_VF",
                                     "BODY_QF", "BODY_MASS", "BODY_INV_INERTIA")}
    w.step(1)
    w.sync()
    names = ("SPOS", "SVEL", "START", "END", "IDS", "DP", "VEL", "POS", "RB_WORLD", "RB_KEYS_UNSORTED", "RB_KEYS",
             "RB_IDS", "RB_START", "RB_END", "RB_SPOS", "RB_FORCE", "RB_TORQUE", "BODY_X", "BODY_V", "BODY_Q",
             "BODY_L", "BODY_FSUM", "BODY_TSUM")
    after = {k: w.read(k) for k in names}
    w.close()
    return pos0, v0, before, after


def _rb_grid_ref(spec, before):
    nb = int(np.prod(spec.rb_buckets))
    cell = (spec.rb_radius,) * 3
    keys, ids, world = O.calc_hash_key_with_offset(before["RB_LOCAL"], before["BODY_XF"], before["BODY_QF"], nb, cell)
    sk, si = O.sort_pairs(keys, ids)
    start, end, spos, _ = O.find_cell_offset(sk, si, world, None, nb)
    return dict(keys=keys, world=world, skeys=sk, ids=si, start=start, end=end, spos=spos, nb=nb)


@pytest.mark.parametrize("nbodies", [1, 2])
def test_rigid_grid_bit_exact(nbodies):
    spec = rigid_scene(nbodies=nbodies)
    pos0, v0, before, g = _run(spec)
    r = _rb_grid_ref(spec, before)
    assert np.array_equal(g["RB_WORLD"].view(np.uint32), r["world"].view(np.uint32))
    assert np.array_equal(g["RB_KEYS_UNSORTED"], r["keys"])
    assert np.array_equal(g["RB_KEYS"], r["skeys"])
    assert np.array_equal(g["RB_IDS"], r["ids"])
    T.compare_ranges(g["RB_START"], g["RB_END"], r["start"], r["end"])
    assert np.array_equal(g["RB_SPOS"].view(np.uint32), r["spos"].view(np.uint32))


def _close(a, b, rtol):
    mag = np.linalg.norm(b, axis=1)
    scale = np.maximum(mag, max(np.median(mag), 1e-30))
    return (np.linalg.norm(a - b, axis=1) / scale).max() <= rtol


@pytest.mark.parametrize("nbodies", [1, 2])
def test_sphere_contact_from_fluid(nbodies):
    spec = rigid_scene(nbodies=nbodies)
    pos0, v0, before, g = _run(spec)
    r = _rb_grid_ref(spec, before)
    fl = T.oracle_grid(spec, pos0, v0)
    F, Tq = O.rb_forces_from_fluids(r["spos"], before["BODY_VF"], before["BODY_XF"], spec.rb_radius, fl["spos"],
                                    fl["svel"], fl["start"], fl["end"], spec.fluid_radius, spec.cell_size,
                                    spec.nbuckets, spec.r2f_rel, spec.ck, spec.ckd)
    # GPU writes per-sphere results at the unsorted (body-contiguous) index
    Fg = g["RB_FORCE"][g["RB_IDS"]]
    Tg = g["RB_TORQUE"][g["RB_IDS"]]
    hit = np.linalg.norm(F[:, :3], axis=1) > 0
    assert hit.sum() > 20, "scene must have fluid/rigid contacts"
    assert _close(Fg[:, :3], F[:, :3], 1e-4)
    assert _close(Tg[:, :3], Tq[:, :3], 1e-4)
    assert np.array_equal(Fg[:, 3], F[:, 3]) and np.array_equal(Tg[:, 3], Tq[:, 3])  # w = body index


@pytest.mark.parametrize("rel", [(2, 2, 2), (1, 1, 1), (1, 3, 2), (3, 1, 2)])
def test_fluid_forces_with_rigid_contact(rel):
    """the fluid-side contact term at several search half-widths: the
    row-batched rigid walk (x half-width up to 2) and the bucket-at-a-time
    walk (wider)"""
    spec = dataclasses.replace(rigid_scene(nbodies=2), f2r_rel=rel)
    pos0, v0, before, g = _run(spec)
    r = _rb_grid_ref(spec, before)
    fl = T.oracle_grid(spec, pos0, v0)
    kc = O.kernels_cache(spec.h)
    cp = O.contact_params(spec.fluid_radius, spec.rb_radius, spec.ck, spec.ckd, (spec.rb_radius,) * 3, spec.f2r_rel,
                          0.003)
    dg = O.contact_grid(r["spos"], before["BODY_VF"], r["start"], r["end"], r["nb"])
    nv = O.forces(fl["spos"], fl["svel"], g["DP"], fl["start"], fl["end"], fl["ids"], spec.mass, spec.visc, fl["p"],
                  kc, newvel_init=v0, contact=(cp, None, dg))
    nv0 = O.forces(fl["spos"], fl["svel"], g["DP"], fl["start"], fl["end"], fl["ids"], spec.mass, spec.visc,
                   fl["p"], kc, newvel_init=v0)
    Fg = T.force_from_vel(g["VEL"], v0, spec.dt)
    Fr = T.force_from_vel(nv, v0, spec.dt)
    F0 = T.force_from_vel(nv0, v0, spec.dt)
    touched = np.linalg.norm(Fr - F0, axis=1) > 0
    assert touched.sum() > 20, "contact term must act on some particles"
    mag = np.linalg.norm(Fr, axis=1)
    err = np.linalg.norm(Fg - Fr, axis=1) / np.maximum(mag, np.median(mag))
    assert err.max() <= 2e-4, err.max()


def test_body_reduction_and_fp64_integration():
    spec = rigid_scene(nbodies=2)
    pos0, v0, before, g = _run(spec)
    nb = len(spec.bodies)
    bf, bt = O.rb_reduce(g["RB_FORCE"], g["RB_TORQUE"], nb)
    assert np.allclose(g["BODY_FSUM"], bf, rtol=1e-12, atol=1e-9)
    assert np.allclose(g["BODY_TSUM"], bt, rtol=1e-12, atol=1e-9)
    inv12 = np.zeros((nb, 12))
    for b in range(nb):
        inv12[b, [0, 1, 2, 4, 5, 6, 8, 9, 10]] = before["BODY_INV_INERTIA"][b]
    ext = np.array(spec.rb_gravity, np.float32)
    x, v, L, q = O.integrate_rb(before["BODY_X"], before["BODY_MASS"].astype(np.float32), before["BODY_V"],
                                g["BODY_FSUM"], spec.dt, ext, spec.box_min, spec.box_max, before["BODY_L"],
                                g["BODY_TSUM"], before["BODY_Q"], inv12, spec.rb_vlimit, f64=True)
    for name, ref in (("BODY_X", x), ("BODY_V", v), ("BODY_L", L), ("BODY_Q", q)):
        assert np.allclose(g[name], ref, rtol=1e-12, atol=1e-14), name


def static_dynamic_scene():
    """Three boxes/spheres straddling the fluid surface (y ~ 0.37): body 0 of
    mass 0 (static: the reference's static rigid-body grid,
    RigidBodySimulator.cpp:146-214), bodies 1 and 2 dynamic; body 1 overlaps
    body 0 and body 2.  Rigid/rigid contact on."""
    spec = rigid_scene(nbodies=1, rb_rb=True)
    rng = np.random.default_rng(8)
    ident = (0.0, 0.0, 0.0, 1.0)
    spec.bodies = [Body(local=box_surface(0.2, 1024, rng), mass=0.0, position=(0.25, 0.38, 0.37),
                        orientation=ident),
                   Body(local=box_surface(0.2, 1024, rng), mass=10.0, position=(0.42, 0.40, 0.37),
                        orientation=ident),
                   Body(local=sphere_surface(0.12, 700), mass=8.0, position=(0.63, 0.40, 0.39),
                        orientation=ident)]
    return spec


def test_rigid_rigid_and_static_contact_match_oracle():
    """One world step of a scene with a static body and two touching dynamic
    bodies against the oracle from the identical state:
      - fluid forces with the static-grid term (K_FluidSim.cu:371-377) and the
        dynamic-grid term (:380-386);
      - per-sphere force/torque of the dynamic bodies: fluid contact
        (CalculateRBForcesFromFluidsK) plus sphere/sphere contact with the
        other dynamic body and with the static grid
        (CalculateRigidBodyForcesFromRBK, K_RigidBodySim.cu:18-61);
      - the static body is never moved."""
    spec = static_dynamic_scene()
    pos0, v0, before, g = _run(spec)
    nb_r = int(np.prod(spec.rb_buckets))
    cell = (spec.rb_radius,) * 3
    r = spec.rb_radius
    _, _, world = O.calc_hash_key_with_offset(before["RB_LOCAL"], before["BODY_XF"], before["BODY_QF"], nb_r, cell)
    body = world[:, 3].astype(np.int64)
    grids = {}
    for name, sel in (("static", body == 0), ("dynamic", body > 0)):
        pts = np.ascontiguousarray(world[sel])
        keys, ids = O.calc_hash_key(pts, nb_r, cell)
        sk, si = O.sort_pairs(keys, ids)
        st, en, sp, _ = O.find_cell_offset(sk, si, pts, None, nb_r)
        grids[name] = dict(spos=sp, start=st, end=en, ids=si, first=int(np.flatnonzero(sel)[0]))
    sg, dg = grids["static"], grids["dynamic"]
    bvel = before["BODY_VF"]
    assert not bvel[0].any()
    # fluid side
    fl = T.oracle_grid(spec, pos0, v0)
    kc = O.kernels_cache(spec.h)
    cp = O.contact_params(spec.fluid_radius, r, spec.ck, spec.ckd, cell, spec.f2r_rel, 0.003)
    o_sg = O.contact_grid(sg["spos"], None, sg["start"], sg["end"], nb_r)
    o_dg = O.contact_grid(dg["spos"], bvel, dg["start"], dg["end"], nb_r)
    args = (fl["spos"], fl["svel"], g["DP"], fl["start"], fl["end"], fl["ids"], spec.mass, spec.visc, fl["p"], kc)
    nv = O.forces(*args, newvel_init=v0, contact=(cp, o_sg, o_dg))
    nv_dyn = O.forces(*args, newvel_init=v0, contact=(cp, None, o_dg))
    Fg = T.force_from_vel(g["VEL"], v0, spec.dt)
    Fr = T.force_from_vel(nv, v0, spec.dt)
    touched = np.linalg.norm(Fr - T.force_from_vel(nv_dyn, v0, spec.dt), axis=1) > 0
    assert touched.sum() > 20, "the static body must act on some fluid particles"
    mag = np.linalg.norm(Fr, axis=1)
    assert (np.linalg.norm(Fg - Fr, axis=1) / np.maximum(mag, np.median(mag))).max() <= 2e-4
    # rigid side, dynamic spheres (sorted order of the dynamic grid)
    Ff, Tf = O.rb_forces_from_fluids(dg["spos"], bvel, before["BODY_XF"], r, fl["spos"], fl["svel"], fl["start"],
                                     fl["end"], spec.fluid_radius, spec.cell_size, spec.nbuckets, spec.r2f_rel,
                                     spec.ck, spec.ckd)
    srb = (sg["spos"], sg["start"], sg["end"], nb_r, 1)
    Fr_rb, Tr_rb = O.rb_forces_from_rb(dg["spos"], bvel, before["BODY_XF"], dg["start"], dg["end"], cell, r, nb_r,
                                       spec.rbrb_k, spec.rbrb_kd, srb=srb)
    Fd, _ = O.rb_forces_from_rb(dg["spos"], bvel, before["BODY_XF"], dg["start"], dg["end"], cell, r, nb_r,
                                spec.rbrb_k, spec.rbrb_kd)
    n_dyn = int((np.abs(Fd[:, :3]) > 0).any(1).sum())
    n_sta = int((np.abs(Fr_rb[:, :3] - Fd[:, :3]) > 0).any(1).sum())
    assert n_dyn > 10 and n_sta > 10, (n_dyn, n_sta)
    Fw = (Ff[:, :3] + Fr_rb[:, :3]).astype(np.float32)
    Tw = (Tf[:, :3] + Tr_rb[:, :3]).astype(np.float32)
    # the world writes each sphere's result at its unsorted index
    unsorted = dg["first"] + dg["ids"]
    assert _close(g["RB_FORCE"][unsorted, :3], Fw, 1e-4)
    assert _close(g["RB_TORQUE"][unsorted, :3], Tw, 1e-4)
    assert np.array_equal(g["RB_FORCE"][unsorted, 3], dg["spos"][:, 3])
    # the static body keeps its pose and zero velocity
    assert np.array_equal(g["BODY_X"][0].view(np.uint64), before["BODY_X"][0].view(np.uint64))
    assert np.array_equal(g["BODY_Q"][0].view(np.uint64), before["BODY_Q"][0].view(np.uint64))
    assert not g["BODY_V"][0].any()
    # the dynamic bodies move
    assert not np.array_equal(g["BODY_X"][1:], before["BODY_X"][1:])


def test_rigid_world_multi_step_finite():
    spec = rigid_scene(nbodies=2)
    w = World([spec])
    w.step(30)
    w.check_finite()
    x = w.read("BODY_X")
    assert np.isfinite(x).all()
    w.close()


@pytest.mark.parametrize("pinned", [True, False])
def test_end_to_end_steps_equal_device_steps(pinned):
    """fg_world_e2e_steps (every step uploads the state from host buffers,
    steps and downloads it again) evolves the state bit-identically to
    device-resident steps.  With pinned buffers the copies are captured with
    the step and the velocity upload runs beside the hash and sort; pageable
    buffers are copied around the step."""
    from fluidgrid_gb300.world import PinnedArray
    spec = rigid_scene(nbodies=2)
    K = 12
    a = World([spec])
    a.step(K)
    pa, va = a.download()
    xa = a.read("BODY_X")
    a.close()
    b = World([spec])
    p0, v0 = b.download()
    bufs = [PinnedArray(p0.shape), PinnedArray(v0.shape)] if pinned else []
    hp, hv = (bufs[0].array, bufs[1].array) if pinned else (np.empty_like(p0), np.empty_like(v0))
    hp[:] = p0
    hv[:] = v0
    ms = b.e2e_steps(K, hp, hv, hp, hv)
    pb, vb = b.download()
    xb = b.read("BODY_X")
    b.close()
    for got in (hp, pb):
        assert np.array_equal(got.view(np.uint32), pa.view(np.uint32))
    for got in (hv, vb):
        assert np.array_equal(got.view(np.uint32), va.view(np.uint32))
    assert np.array_equal(xa.view(np.uint64), xb.view(np.uint64))
    assert (ms > 0).all()
    for buf in bufs:
        buf.free()
