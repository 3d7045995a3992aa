"""Precision form (4,194,304 particles, a 10% gaussian jet, eight bodies with
rigid/rigid contact): FP32 forces with Kahan density sums, FP64 body
force/torque reduction and integration on the GPU, compared at steps 1, 10
and 100 with the FP64 oracle from the identical state the GPU started that
step from.  Each step's per-quantity errors are checked against the stated
bounds and written as JSON to $FG_PRECISION_REPORT when that is set.

Bounds (per step, from an identical state):
  density   max |rho - rho64| / rho64                        <= 1e-5
  forces    max |F - F64| / max(|F64|, median |F64|)          <= 2e-4
  body F/T  max |S - S64| / max(|S64|, 1e-3 * max |S64|)      <= 1e-4
  body x,q  max |x - x64| (m, unitless)                       <= 1e-6
            (the GPU integrates FP64 sums of FP32 per-sphere forces, the
            oracle FP64 sums of FP64 per-sphere forces; ~1e-5 relative in the
            force moves a body ~1e-7 m in one step)
"""
import json
import os

import numpy as np
import pytest

from fluidgrid_gb300 import World, build, scenes
from oracle import oracle as O
import helpers as T

pytestmark = pytest.mark.gpu

BEFORE = ("RB_LOCAL", "BODY_X", "BODY_V", "BODY_Q", "BODY_L", "BODY_XF", "BODY_VF", "BODY_QF", "BODY_MASS",
          "BODY_INV_INERTIA")
AFTER = ("DP", "VEL", "POS", "RB_FORCE", "RB_TORQUE", "RB_IDS", "BODY_FSUM", "BODY_TSUM", "BODY_X", "BODY_V",
         "BODY_Q", "BODY_L")


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _body_sums(F, T_, nb):
    bf = np.zeros((nb, 3))
    bt = np.zeros((nb, 3))
    b = F[:, 3].astype(np.int64)
    np.add.at(bf, b, F[:, :3].astype(np.float64))
    np.add.at(bt, b, T_[:, :3].astype(np.float64))
    return bf, bt


def _one_step_errors(spec, pos0, v0, before, g):
    """GPU step from (pos0, v0, before) against the FP64 oracle step."""
    fl = T.oracle_grid(spec, pos0, v0)
    kc = O.kernels_cache(spec.h)
    d64, pairs = O.density(fl["spos"], fl["start"], fl["end"], fl["p"], kc, spec.gas, spec.rest, spec.mass,
                           f64=True)
    act = fl["spos"][:, 3] > 0
    e_rho = np.abs(g["DP"][act, 0].astype(np.float64) - d64[act, 0]) / d64[act, 0]
    # rigid sphere grid from the bodies' FP32 mirrors (bit-exact with the GPU's)
    nb_r = int(np.prod(spec.rb_buckets))
    cell = (spec.rb_radius,) * 3
    keys, ids, world = O.calc_hash_key_with_offset(before["RB_LOCAL"], before["BODY_XF"], before["BODY_QF"], nb_r,
                                                   cell)
    sk, si = O.sort_pairs(keys, ids)
    rst, ren, rsp, _ = O.find_cell_offset(sk, si, world, None, nb_r)
    F64, T64 = O.rb_forces_from_fluids(rsp, before["BODY_VF"], before["BODY_XF"], spec.rb_radius, fl["spos"],
                                       fl["svel"], fl["start"], fl["end"], spec.fluid_radius, spec.cell_size,
                                       spec.nbuckets, spec.r2f_rel, spec.ck, spec.ckd, f64=True)
    if spec.rb_rb:
        Frr, Trr = O.rb_forces_from_rb(rsp, before["BODY_VF"], before["BODY_XF"], rst, ren, cell, spec.rb_radius,
                                       nb_r, spec.rbrb_k, spec.rbrb_kd)
        F64[:, :3] += Frr[:, :3]
        T64[:, :3] += Trr[:, :3]
    nbod = len(spec.bodies)
    bf64, bt64 = _body_sums(F64, T64, nbod)
    scale_f = max(np.abs(bf64).max(), 1e-30)
    scale_t = max(np.abs(bt64).max(), 1e-30)
    e_bf = np.abs(g["BODY_FSUM"][:, :3] - bf64) / np.maximum(np.abs(bf64), 1e-3 * scale_f)
    e_bt = np.abs(g["BODY_TSUM"][:, :3] - bt64) / np.maximum(np.abs(bt64), 1e-3 * scale_t)
    # fluid forces in FP64 with the FP64 density, contact with the body velocities
    cp = O.contact_params(spec.fluid_radius, spec.rb_radius, spec.ck, spec.ckd, cell, spec.f2r_rel, 0.003)
    dg = O.contact_grid(rsp, before["BODY_VF"], rst, ren, nb_r)
    nv64 = O.forces(fl["spos"], fl["svel"], d64.astype(np.float32), fl["start"], fl["end"], fl["ids"], spec.mass,
                    spec.visc, fl["p"], kc, f64=True, newvel_init=v0, contact=(cp, None, dg))
    Fg = T.force_from_vel(g["VEL"], v0, spec.dt)
    Fr = (nv64[:, :3] - v0[:, :3].astype(np.float64)) / spec.dt
    mag = np.linalg.norm(Fr, axis=1)
    pact = pos0[:, 3] > 0
    e_f = (np.linalg.norm(Fg - Fr, axis=1) / np.maximum(mag, np.median(mag)))[pact]
    # FP64 body integration from the FP64 sums
    inv12 = np.zeros((nbod, 12))
    for b in range(nbod):
        inv12[b, [0, 1, 2, 4, 5, 6, 8, 9, 10]] = before["BODY_INV_INERTIA"][b]
    bf4 = np.c_[bf64, np.zeros(nbod)]
    bt4 = np.c_[bt64, np.zeros(nbod)]
    x, v, L, q = O.integrate_rb(before["BODY_X"], before["BODY_MASS"].astype(np.float32), before["BODY_V"], bf4,
                                spec.dt, np.array(spec.rb_gravity, np.float32), spec.box_min, spec.box_max,
                                before["BODY_L"], bt4, before["BODY_Q"], inv12, spec.rb_vlimit, f64=True)
    e_x = np.abs(g["BODY_X"][:, :3] - x[:, :3]).max()
    e_q = np.abs(g["BODY_Q"] - q).max()
    e_v = np.abs(g["BODY_V"][:, :3] - v[:, :3]).max()
    return {"density_rel_max": float(e_rho.max()), "density_rel_median": float(np.median(e_rho)),
            "force_rel_max": float(e_f.max()), "force_rel_median": float(np.median(e_f)),
            "body_force_rel_max": float(e_bf.max()), "body_torque_rel_max": float(e_bt.max()),
            "body_pos_abs_max_m": float(e_x), "body_quat_abs_max": float(e_q), "body_vel_abs_max": float(e_v),
            "pairs_per_particle": float(pairs) / len(pos0), "contact_spheres": int((np.abs(F64[:, :3]) > 0).any(1).sum())}


def test_precision_form_against_fp64_oracle():
    spec = scenes.precision_jet()
    w = World([spec])
    report = {"workload": spec.name, "particles": spec.n, "bodies": len(spec.bodies),
              "rigid_spheres": spec.nspheres, "steps": {}}
    done = 0
    for k in (1, 10, 100):
        if k - 1 > done:
            w.step(k - 1 - done)
            done = k - 1
        pos0, v0 = w.download()
        before = {n: w.read(n) for n in BEFORE}
        diag0 = w.diagnostics()[0]
        w.step(1)
        done += 1
        g = {n: w.read(n) for n in AFTER}
        e = _one_step_errors(spec, pos0, v0, before, g)
        diag1 = w.diagnostics()[0]
        e["fp64_momentum_change"] = [diag1[c] - diag0[c] for c in ("px", "py", "pz")]
        e["fp64_mass"] = diag1["mass"]
        report["steps"][str(k)] = e
        assert e["density_rel_max"] <= 1e-5, (k, e)
        assert e["force_rel_max"] <= 2e-4, (k, e)
        assert e["body_force_rel_max"] <= 1e-4 and e["body_torque_rel_max"] <= 1e-4, (k, e)
        assert e["body_pos_abs_max_m"] <= 1e-6 and e["body_quat_abs_max"] <= 1e-6, (k, e)
        assert diag1["mass"] == diag0["mass"]  # no particle is created or lost
    w.close()
    out = os.environ.get("FG_PRECISION_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)
