"""The oracle's restated helpers against golden vectors recorded from the
reference's own helper source files (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_helpers.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


def test_hash_key_bit_exact(g):
    pos, cell, nb, key = g["hash_pos"], g["hash_cell"], g["hash_nb"], g["hash_key"]
    got = np.array([O.hash_key(pos[i], cell[i], int(nb[i])) for i in range(len(pos))], np.uint32)
    assert np.array_equal(got, key)


def test_hash_key_int32_wrap_cases(g):
    # positions far from the origin make the int32 products wrap
    pos = g["hash_pos"]
    assert np.abs(pos).max() > 1e4
    test_hash_key_bit_exact(g)


def test_walls_no_penetration_bit_exact(g):
    f = O.lib()
    import ctypes
    for i in range(len(g["walls_pos"])):
        o = np.zeros(3, np.float32)
        f.fgo_walls_no_penetration(O._f(g["walls_pos"][i].copy()), O._f(g["walls_vel"][i].copy()),
                                   O._f(g["walls_min"].copy()), O._f(g["walls_max"].copy()),
                                   np.float32(0.003043174), np.float32(20000), np.float32(256),
                                   g["walls_scale"][i], O._f(o))
        assert np.array_equal(o.view(np.uint32), g["walls_np"][i].view(np.uint32)), i


def test_walls_no_slip_bit_exact(g):
    f = O.lib()
    mn = np.array([-11.0, -40.0, -11.0], np.float32)
    mx = np.array([11.0, 200.0, 11.0], np.float32)
    nz = 0
    for i in range(len(g["noslip_pos"])):
        o = np.zeros(3, np.float32)
        f.fgo_walls_no_slip(O._f(g["noslip_pos"][i].copy()), O._f(g["walls_vel"][i].copy()),
                            O._f(g["walls_force"][i].copy()), O._f(mn), O._f(mx), np.float32(0.003043174),
                            g["noslip_fkin"][i], g["noslip_fstatic"][i], np.float32(1.0), O._f(o))
        ref = g["walls_ns"][i]
        nz += int(np.any(ref != 0))
        assert np.array_equal(o, ref), i
    assert nz > 100  # the fixture exercises the friction branch


@pytest.mark.parametrize("case", [0, 1, 2, 3])
def test_process_collision_forces_bit_exact(g, case):
    pre = "coll%d_" % case
    cpos, cvel, st, en = g[pre + "cpos"], g[pre + "cvel"], g[pre + "start"], g[pre + "end"]
    cell, nb, rel = g[pre + "cell"], int(g[pre + "nb"]), g[pre + "rel"]
    w_rb, check = [int(x) for x in g[pre + "flags"]]
    eps = np.float32(g[pre + "eps"])
    qpos, qvel, ref = g[pre + "qpos"], g[pre + "qvel"], g[pre + "out"]
    f = O.lib()
    hits = 0
    for i in range(len(qpos)):
        o = np.zeros(3, np.float32)
        f.fgo_process_collision_forces(O._f(qpos[i].copy()), O._f(qvel[i].copy()), np.float32(0.02285),
                                       O._f(cpos), O._f(cvel), np.float32(0.0114), np.float32(-10.0),
                                       np.float32(-5.0), O._i(rel.astype(np.int32)), O._u(st), O._u(en),
                                       O._f(cell), nb, w_rb, check, int(qpos[i, 3]), eps, O._f(o))
        hits += int(np.any(ref[i] != 0))
        assert np.array_equal(o, ref[i]), (case, i, o, ref[i])
    assert hits > 20


def _quat(g, name, fn, a, b=None):
    f = getattr(O.lib(), fn)
    for i in range(len(g[a])):
        o = np.zeros(4, np.float32)
        if b is None:
            f(O._f(g[a][i].copy()), O._f(o))
        else:
            f(O._f(g[a][i].copy()), O._f(g[b][i].copy()), O._f(o))
        assert np.array_equal(o, g[name][i]), (name, i)


def test_quaternion_helpers_bit_exact(g):
    _quat(g, "q_prod", "fgo_quat_product", "q_a", "q_b")
    _quat(g, "q_transform", "fgo_quat_transform_point", "q_point", "q_unit")
    _quat(g, "q_normalize", "fgo_quat_normalize", "q_a")
    _quat(g, "q_cross", "fgo_vec3_cross", "q_a", "q_b")


def test_angular_velocity_bit_exact(g):
    f = O.lib().fgo_angular_velocity
    for i in range(len(g["q_inv"])):
        o = np.zeros(4, np.float32)
        f(O._f(g["q_inv"][i].copy()), O._f(g["q_L"][i].copy()), O._f(g["q_unit"][i].copy()), O._f(o))
        assert np.array_equal(o, g["q_angvel"][i]), i


def test_kernels_cache_values():
    # HeterogeneousSimulator.cpp:33-42 with h = 0.0457
    kc = O.kernels_cache(0.0457)
    h = 0.0457
    pi = float(np.float32(3.14159265))
    assert kc.kPoly6 == pytest.approx(315.0 / (64.0 * pi * h ** 9), rel=1e-6)
    assert kc.kSpikyGradient == pytest.approx(-45.0 / (pi * h ** 6), rel=1e-6)
    assert kc.kViscosityLaplacian == pytest.approx(45.0 / (pi * h ** 6), rel=1e-6)
