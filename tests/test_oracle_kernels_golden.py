"""The oracle's restated SPH kernels against golden vectors recorded from the
reference's own kernels (tests/golden/make_golden_kernels.py runs the
__global__ section of GPU_Kernels/K_FluidSim.cu on the host): density, forces,
forces with the static and dynamic rigid grids, and integration, bit for bit
on the same inputs.  These pin the oracle's kernel loops (27-bucket walk
order, duplicate visits of hash-colliding buckets, self exclusion, inactive
particles, scatter by id), not only the helpers they call."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


def _setup(g):
    h, scale, dt, vlimit, mass, gas, rest, visc, fr, rr, ks, kd = [float(x) for x in g["scalars"]]
    cell = (np.float32(h),) * 3
    p = O.make_common_params(cell, g["buckets"], h, vlimit, g["box"][0], g["box"][1], g["gravity"], scale, dt,
                             relation=g["rel"], point_radius=fr)
    kc = O.kernels_cache(h)
    return p, kc, dict(h=h, mass=mass, gas=gas, rest=rest, visc=visc, fr=fr, rr=rr, ks=ks, kd=kd)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_scene_exercises_the_loops(g):
    """hash collisions (several cells per bucket), inactive particles and
    rigid contacts are present in the recorded scene"""
    n = g["spos"].shape[0]
    occ = g["start"] != 0xFFFFFFFF
    assert occ.sum() < 4096 and (g["end"][occ].astype(np.int64) - g["start"][occ]).max() > 8
    assert (g["spos"][:, 3] <= 0).sum() > n // 40
    for tag in ("srb_static", "srb_dynamic", "srb_both"):
        assert (g[tag] != g["newvel"]).any(axis=1).sum() > 20, tag


def test_density_kernel_bit_exact(g):
    p, kc, s = _setup(g)
    dp, _ = O.density(g["spos"], g["start"], g["end"], p, kc, s["gas"], s["rest"], s["mass"])
    assert np.array_equal(_bits(dp), _bits(g["dp"]))


def test_forces_kernel_bit_exact(g):
    p, kc, s = _setup(g)
    n = g["spos"].shape[0]
    nv = O.forces(g["spos"], g["svel"], g["dp"], g["start"], g["end"], g["ids"], s["mass"], s["visc"], p, kc,
                  newvel_init=np.zeros((n, 4), np.float32))
    assert np.array_equal(_bits(nv), _bits(g["newvel"]))


@pytest.mark.parametrize("case", ["static", "dynamic", "both"])
def test_forces_with_rigid_grids_bit_exact(g, case):
    p, kc, s = _setup(g)
    n = g["spos"].shape[0]
    rb_nb = int(np.prod(g["rb_buckets"]))
    cp = O.contact_params(s["fr"], s["rr"], s["ks"], s["kd"], g["rb_cell"], g["rel"], 0.003)
    sg = O.contact_grid(g["s_pos"], None, g["s_start"], g["s_end"], rb_nb, use=case in ("static", "both"))
    dg = O.contact_grid(g["d_pos"], g["d_vel"], g["d_start"], g["d_end"], rb_nb, use=case in ("dynamic", "both"))
    nv = O.forces(g["spos"], g["svel"], g["dp"], g["start"], g["end"], g["ids"], s["mass"], s["visc"], p, kc,
                  newvel_init=np.zeros((n, 4), np.float32), contact=(cp, sg, dg))
    assert np.array_equal(_bits(nv), _bits(g["srb_" + case]))


def test_integrate_kernel_bit_exact(g):
    p, _, _ = _setup(g)
    out = O.integrate(g["pos"], g["newvel"], p)
    assert np.array_equal(_bits(out), _bits(g["integrated"]))


def _sorted(keys, ids):
    order = np.argsort(keys, kind="stable")
    return np.ascontiguousarray(keys[order]), np.ascontiguousarray(ids[order])


def test_hash_and_ranges_kernels_bit_exact(g):
    """CalcHashKeyK and FindCellOffsetOrderinPosVelK (128-thread blocks with
    their shared-memory neighbour hash and barrier)"""
    h = float(g["scalars"][0])
    nb = int(np.prod(g["buckets"]))
    keys, ids = O.calc_hash_key(g["pos"], nb, (np.float32(h),) * 3)
    assert np.array_equal(keys, g["hash_key"]) and np.array_equal(ids, g["hash_ids"])
    sk, si = O.sort_pairs(keys, ids)
    rk, ri = _sorted(g["hash_key"], g["hash_ids"])
    assert np.array_equal(sk, rk) and np.array_equal(si, ri)  # a stable key sort, as thrust's
    start, end, spos, svel = O.find_cell_offset(sk, si, g["pos"], g["vel"], nb,
                                                end_init=np.zeros(nb, np.uint32))
    assert np.array_equal(start, g["grid_start"]) and np.array_equal(end, g["grid_end"])
    assert np.array_equal(_bits(spos), _bits(g["grid_spos"])) and np.array_equal(_bits(svel), _bits(g["grid_svel"]))


def test_offset_hash_and_position_ranges_kernels_bit_exact(g):
    """CalcHashKeyWithOffsetK (sphere world positions from body centres and
    orientations) and FindCellOffsetOrderingPosK"""
    rb_nb = int(np.prod(g["rb_buckets"]))
    assert set(np.unique(g["rb_local"][:, 3])) == {0.0, 1.0}
    keys, ids, world = O.calc_hash_key_with_offset(g["rb_local"], g["rb_cm"], g["rb_q"], rb_nb, g["rb_cell"])
    assert np.array_equal(keys, g["rb_key"]) and np.array_equal(ids, g["rb_ids"])
    assert np.array_equal(_bits(world), _bits(g["rb_world"]))
    sk, si = O.sort_pairs(keys, ids)
    start, end, spos, _ = O.find_cell_offset(sk, si, world, None, rb_nb, end_init=np.zeros(rb_nb, np.uint32))
    assert np.array_equal(start, g["rb_start"]) and np.array_equal(end, g["rb_end"])
    assert np.array_equal(_bits(spos), _bits(g["rb_spos"]))


@pytest.mark.parametrize("nsrb", [0, 1])
def test_rigid_rigid_contact_kernel_bit_exact(g, nsrb):
    """CalculateRigidBodyForcesFromRBK on two overlapping bodies, without and
    with the static plane"""
    _, _, s = _setup(g)
    rb_nb = int(np.prod(g["rb_buckets"]))
    F_, T_ = O.rb_forces_from_rb(g["rb_spos"], g["rb_bvel"], g["rb_cm"], g["rb_start"], g["rb_end"], g["rb_cell"],
                                 s["rr"], rb_nb, s["ks"], s["kd"],
                                 srb=(g["s_pos"], g["s_start"], g["s_end"], rb_nb, nsrb))
    tag = "rbrbs" if nsrb else "rbrb"
    assert (np.abs(g[tag + "_force"][:, :3]).sum(axis=1) > 0).sum() > 10
    assert np.array_equal(_bits(F_), _bits(g[tag + "_force"]))
    assert np.array_equal(_bits(T_), _bits(g[tag + "_torque"]))


def test_rigid_from_fluid_kernel_bit_exact(g):
    """CalculateRBForcesFromFluidsK: the fluid's contact on each sphere"""
    _, _, s = _setup(g)
    rb_nb = int(np.prod(g["rb_buckets"]))
    nb = int(np.prod(g["buckets"]))
    h = s["h"]
    F_, T_ = O.rb_forces_from_fluids(g["rb_spos"], g["rb_bvel"], g["rb_cm"], s["rr"], g["spos"], g["svel"],
                                     g["start"], g["end"], s["fr"], np.array([h, h, h], np.float32), nb, g["rel"],
                                     s["ks"], s["kd"])
    assert np.array_equal(_bits(F_), _bits(g["rbfl_force"]))
    assert np.array_equal(_bits(T_), _bits(g["rbfl_torque"]))


def test_rigid_integrate_kernel_bit_exact(g):
    """IntegrateRBK in FP32: force clamp, damped angular momentum,
    quaternion update and normalisation, box bounce"""
    h, scale, dt, vlimit = [float(x) for x in g["scalars"][:4]]
    i = g["int_in"]
    x, v, f, L, t, q = (np.ascontiguousarray(i[:, 4 * k:4 * k + 4]) for k in range(6))
    xo, vo, Lo, qo = O.integrate_rb(x, g["int_mass"], v, f, dt, g["int_ext"], g["box"][0], g["box"][1], L, t, q,
                                    g["int_inv"], vlimit)
    out = np.concatenate([xo, vo, Lo, qo], 1)
    assert np.array_equal(_bits(out), _bits(g["int_out"]))
