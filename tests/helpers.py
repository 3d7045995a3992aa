"""Shared test helpers: the oracle pipeline for a SceneSpec and comparisons.

The oracle (oracle/) is the checker here; the product under test is
libfluidgrid_gb300.so reached through its C ABI."""
import numpy as np

from oracle import oracle as O

EMPTY = 0xFFFFFFFF


def oracle_params(spec):
    return O.make_common_params(spec.cell_size, spec.buckets, spec.h, spec.vlimit, spec.box_min, spec.box_max,
                                spec.gravity, spec.scale, spec.dt, relation=spec.f2r_rel,
                                point_radius=spec.fluid_radius)


def oracle_grid(spec, pos, vel):
    """hash -> stable sort -> ranges/gather, as the reference's
    findFluidNeighbourhood (HeterogeneousSimulator.cpp:131-150)."""
    p = oracle_params(spec)
    nb = spec.nbuckets
    keys, ids = O.calc_hash_key(pos, nb, spec.cell_size)
    sk, si = O.sort_pairs(keys, ids)
    start, end, spos, svel = O.find_cell_offset(sk, si, pos, vel, nb)
    return dict(p=p, keys=keys, skeys=sk, ids=si, start=start, end=end, spos=spos, svel=svel)


def compare_ranges(start_gpu, end_gpu, start_ref, end_ref, base=0):
    """start everywhere, end where the bucket is occupied (the reference
    leaves `end` of empty buckets untouched)."""
    s = start_gpu.astype(np.int64)
    occ = start_ref != EMPTY
    s_adj = np.where(start_gpu == EMPTY, EMPTY, s - base)
    assert np.array_equal(s_adj.astype(np.uint32), start_ref), "start differs"
    e_adj = (end_gpu.astype(np.int64) - base)[occ]
    assert np.array_equal(e_adj, end_ref[occ].astype(np.int64)), "end differs"


def rel_err(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def force_from_vel(vnew, vold, dt):
    return (vnew[:, :3].astype(np.float64) - vold[:, :3].astype(np.float64)) / dt


BEFORE_STEP = ("RB_LOCAL", "BODY_X", "BODY_V", "BODY_Q", "BODY_L", "BODY_XF", "BODY_VF", "BODY_QF", "BODY_MASS",
               "BODY_INV_INERTIA")
AFTER_STEP = ("KEYS_UNSORTED", "KEYS", "IDS", "START", "END", "SPOS", "SVEL", "DP", "VEL", "POS", "RB_FORCE",
              "RB_TORQUE", "RB_IDS", "BODY_FSUM", "BODY_TSUM", "BODY_X", "BODY_V", "BODY_Q", "BODY_L")


def check_grid(g, ref):
    """Hash keys, sort order, cell ranges and sorted gathers bit-exact."""
    assert np.array_equal(g["KEYS_UNSORTED"], ref["keys"]), "hash keys differ"
    assert np.array_equal(g["KEYS"], ref["skeys"]), "sorted keys differ"
    assert np.array_equal(g["IDS"], ref["ids"]), "sort order differs"
    compare_ranges(g["START"], g["END"], ref["start"], ref["end"])
    assert np.array_equal(g["SPOS"].view(np.uint32), ref["spos"].view(np.uint32))
    assert np.array_equal(g["SVEL"].view(np.uint32), ref["svel"].view(np.uint32))


def _body_sums(F, T_, nb):
    bf = np.zeros((nb, 3))
    bt = np.zeros((nb, 3))
    b = F[:, 3].astype(np.int64)
    np.add.at(bf, b, F[:, :3].astype(np.float64))
    np.add.at(bt, b, T_[:, :3].astype(np.float64))
    return bf, bt


def _per_row_rel(a, b):
    """|a - b| per row over max(|b|, 1e-3 max |b|) (0 when b is all zero)."""
    mag = np.linalg.norm(b, axis=1)
    top = mag.max() if mag.size else 0.0
    if top == 0.0:
        return np.zeros(len(b)) if not np.abs(a).any() else np.full(len(b), np.inf)
    return np.linalg.norm(a - b, axis=1) / np.maximum(mag, 1e-3 * top)


def two_way_step_errors(spec, pos0, v0, before, g, fl=None):
    """Errors of one GPU two-way step that started from (pos0, v0, before)
    against the oracle from the identical state, in the reference's step
    order (HeterogeneousSimulator.cpp:57-126): density (FP64 oracle), fluid
    forces with the rigid contact term (FP64), per-sphere contact force and
    torque (FP32 oracle; FP64 reported), FP64 per-body sums and the FP64 body
    integration.  `g` holds the buffers of AFTER_STEP read after the step."""
    if fl is None:
        fl = oracle_grid(spec, pos0, v0)
    kc = O.kernels_cache(spec.h)
    d64, pairs = O.density(fl["spos"], fl["start"], fl["end"], fl["p"], kc, spec.gas, spec.rest, spec.mass,
                           f64=True)
    act = fl["spos"][:, 3] > 0
    e_rho = np.abs(g["DP"][act, 0].astype(np.float64) - d64[act, 0]) / d64[act, 0]
    out = {"density_rel_max": float(e_rho.max()), "density_rel_median": float(np.median(e_rho)),
           "pairs_per_particle": float(pairs) / len(pos0)}
    nbod = len(spec.bodies)
    contact = None
    if nbod:
        nb_r = int(np.prod(spec.rb_buckets))
        cell = (spec.rb_radius,) * 3
        keys, ids, world = O.calc_hash_key_with_offset(before["RB_LOCAL"], before["BODY_XF"], before["BODY_QF"],
                                                       nb_r, cell)
        sk, si = O.sort_pairs(keys, ids)
        rst, ren, rsp, _ = O.find_cell_offset(sk, si, world, None, nb_r)
        args = (rsp, before["BODY_VF"], before["BODY_XF"], spec.rb_radius, fl["spos"], fl["svel"], fl["start"],
                fl["end"], spec.fluid_radius, spec.cell_size, spec.nbuckets, spec.r2f_rel, spec.ck, spec.ckd)
        F64, T64 = O.rb_forces_from_fluids(*args, f64=True)
        F32, T32 = O.rb_forces_from_fluids(*args)
        if spec.rb_rb:
            Frr, Trr = O.rb_forces_from_rb(rsp, before["BODY_VF"], before["BODY_XF"], rst, ren, cell,
                                           spec.rb_radius, nb_r, spec.rbrb_k, spec.rbrb_kd)
            F64[:, :3] += Frr[:, :3]
            T64[:, :3] += Trr[:, :3]
            F32[:, :3] += Frr[:, :3]
            T32[:, :3] += Trr[:, :3]
            out["rb_rb_contact_spheres"] = int((np.abs(Frr[:, :3]) > 0).any(1).sum())
        # the GPU writes each sphere's result at its unsorted (body-contiguous) index
        Fg = g["RB_FORCE"][g["RB_IDS"]]
        Tg = g["RB_TORQUE"][g["RB_IDS"]]
        out["sphere_force_rel_max"] = float(_per_row_rel(Fg[:, :3], F32[:, :3]).max())
        out["sphere_torque_rel_max"] = float(_per_row_rel(Tg[:, :3], T32[:, :3]).max())
        out["sphere_force_rel_max_fp64"] = float(_per_row_rel(Fg[:, :3].astype(np.float64), F64[:, :3]).max())
        out["contact_spheres"] = int((np.abs(F64[:, :3]) > 0).any(1).sum())
        bf64, bt64 = _body_sums(F64, T64, nbod)
        scale_f = max(np.abs(bf64).max(), 1e-30)
        scale_t = max(np.abs(bt64).max(), 1e-30)
        e_bf = np.abs(g["BODY_FSUM"][:, :3] - bf64) / np.maximum(np.abs(bf64), 1e-3 * scale_f)
        e_bt = np.abs(g["BODY_TSUM"][:, :3] - bt64) / np.maximum(np.abs(bt64), 1e-3 * scale_t)
        out["body_force_rel_max"] = float(e_bf.max())
        out["body_torque_rel_max"] = float(e_bt.max())
        cp = O.contact_params(spec.fluid_radius, spec.rb_radius, spec.ck, spec.ckd, cell, spec.f2r_rel, 0.003)
        dg = O.contact_grid(rsp, before["BODY_VF"], rst, ren, nb_r)
        contact = (cp, None, dg)
    # fluid forces in FP64 with the FP64 density, contact with the body velocities
    nv64 = O.forces(fl["spos"], fl["svel"], d64.astype(np.float32), fl["start"], fl["end"], fl["ids"], spec.mass,
                    spec.visc, fl["p"], kc, f64=True, newvel_init=v0, contact=contact)
    Fg_f = force_from_vel(g["VEL"], v0, spec.dt)
    Fr = (nv64[:, :3] - v0[:, :3].astype(np.float64)) / spec.dt
    mag = np.linalg.norm(Fr, axis=1)
    pact = pos0[:, 3] > 0
    e_f = (np.linalg.norm(Fg_f - Fr, axis=1) / np.maximum(mag, np.median(mag)))[pact]
    out["force_rel_max"] = float(e_f.max())
    out["force_rel_median"] = float(np.median(e_f))
    if nbod:
        # FP64 body integration from the FP64 sums
        inv12 = np.zeros((nbod, 12))
        for b in range(nbod):
            inv12[b, [0, 1, 2, 4, 5, 6, 8, 9, 10]] = before["BODY_INV_INERTIA"][b]
        bf4 = np.c_[bf64, np.zeros(nbod)]
        bt4 = np.c_[bt64, np.zeros(nbod)]
        x, v, L, q = O.integrate_rb(before["BODY_X"], before["BODY_MASS"].astype(np.float32), before["BODY_V"], bf4,
                                    spec.dt, np.array(spec.rb_gravity, np.float32), spec.box_min, spec.box_max,
                                    before["BODY_L"], bt4, before["BODY_Q"], inv12, spec.rb_vlimit, f64=True)
        out["body_pos_abs_max_m"] = float(np.abs(g["BODY_X"][:, :3] - x[:, :3]).max())
        out["body_quat_abs_max"] = float(np.abs(g["BODY_Q"] - q).max())
        out["body_vel_abs_max"] = float(np.abs(g["BODY_V"][:, :3] - v[:, :3]).max())
    return out
