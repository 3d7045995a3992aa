"""Generate golden vectors from the reference's own SPH kernels.

Runs only where the reference sources are present: it builds
oracle/_ref/libfgrefk_fluid.so (oracle Makefile target `refk`: the __global__
section of the reference's GPU_Kernels/K_FluidSim.cu compiled as host C++
through the self-written oracle/ref_shim/kernel_host.h, driven once per
particle index by oracle/ref_kernels_fluid.cpp), runs CalculateMassDensityK,
SPHCalculateForcesK, SPHCalculateForcesWithSRBK (static grid, dynamic grid,
both) and SPHIntegrateK on a small seeded scene, and records inputs and outputs
into tests/golden/ref_kernels.npz.  The CPU test suite checks the oracle's
restatement of these kernels against the file bit for bit; nothing at test
time needs the reference sources.

It also builds oracle/_ref/libfgrefk_grid.so and libfgrefk_rigid.so from
K_HashGrid.cu and K_RigidBodySim.cu the same way and records CalcHashKeyK,
FindCellOffsetOrderinPosVelK (its 128-thread blocks run as host thread groups
with a barrier), CalcHashKeyWithOffsetK, FindCellOffsetOrderingPosK,
CalculateRigidBodyForcesFromRBK (without and with the static plane),
CalculateRBForcesFromFluidsK and IntegrateRBK on two overlapping bodies.

The scene: 2,560 jittered lattice particles (5% inactive) with random
velocities in a hashed grid of 16^3 buckets (several cells share a bucket), a
static plane of spheres under the block and one dynamic box of spheres
straddling its surface, each in a 16^3-bucket rigid grid.

    python tests/golden/make_golden_kernels.py [--reference-dir DIR]
"""
import argparse
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from fluidgrid_gb300.scenes import H, SPACING, MASS, REST, GAS, VISC, DT, lattice, box_surface  # noqa: E402

F = ctypes.POINTER(ctypes.c_float)
U = ctypes.POINTER(ctypes.c_uint32)
I = ctypes.POINTER(ctypes.c_int)
P = ctypes.c_void_p

# scene constants (recorded in the file)
BUCKETS = (16, 16, 16)
RB_BUCKETS = (16, 16, 16)
FLUID_RADIUS = 0.25 * H
RB_RADIUS = 0.5 * H
REL = (2, 2, 2)
KSPRING, KDAMP = -10.0, -5.0
SCALE = 0.004
VLIMIT = 200.0
GRAVITY = (0.0, -9.8, 0.0)
BOX_MIN, BOX_MAX = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)


def fp(a):
    return a.ctypes.data_as(F)


def up(a):
    return a.ctypes.data_as(U)


def load_refk(reference_dir):
    subprocess.check_call(["make", "-s", "refk", "REFERENCE_DIR=" + reference_dir], cwd=ORACLE)
    grid = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libfgrefk_grid.so"))
    grid.refk_calc_hash_key.argtypes = [U, U, F, ctypes.c_uint32, ctypes.c_uint32, F]
    grid.refk_calc_hash_key_with_offset.argtypes = [U, U, F, F, F, F, ctypes.c_uint32, F, ctypes.c_int]
    grid.refk_find_cell_offset_pos_vel.argtypes = [U, U, U, U, F, F, F, F, ctypes.c_uint32, ctypes.c_uint32]
    grid.refk_find_cell_offset_pos.argtypes = [U, U, U, U, F, F, ctypes.c_uint32, ctypes.c_uint32]
    rigid = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libfgrefk_rigid.so"))
    rigid.refk_rb_forces_from_rb.argtypes = [F, F, F, F, F, U, U, ctypes.c_uint32, F, ctypes.c_float, ctypes.c_int,
                                             ctypes.c_int, F, U, U, ctypes.c_float, ctypes.c_float, ctypes.c_int]
    rigid.refk_rb_forces_from_fluids.argtypes = [F, F, F, F, F, U, U, ctypes.c_uint32, F, ctypes.c_float,
                                                 ctypes.c_int, F, F, U, U, ctypes.c_float, F, ctypes.c_uint32, I,
                                                 ctypes.c_float, ctypes.c_float]
    rigid.refk_integrate_rb.argtypes = [F, F, F, F, ctypes.c_uint32, ctypes.c_float, F, F, F, F, F, F, F, F,
                                        ctypes.c_float]
    lib = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libfgrefk_fluid.so"))
    lib.grid, lib.rigid = grid, rigid
    lib.refk_params_size.restype = ctypes.c_uint32
    lib.refk_kernels_cache_size.restype = ctypes.c_uint32
    lib.refk_set_params.argtypes = [P, P]
    lib.refk_density.argtypes = [F, F, U, U, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    lib.refk_forces.argtypes = [F, F, F, U, U, F, U, ctypes.c_float, ctypes.c_uint32, ctypes.c_float]
    lib.refk_forces_srb.argtypes = [F, F, F, F, U, U, U, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, F, I,
                                    F, U, U, ctypes.c_uint32, F, F, U, U, ctypes.c_uint32, ctypes.c_int,
                                    ctypes.c_int]
    lib.refk_integrate.argtypes = [F, F, ctypes.c_uint32]
    return lib


def grid(pos4, vel4, cell, nb):
    """hash -> stable sort -> ranges/gather (the oracle's grid build)"""
    keys, ids = O.calc_hash_key(pos4, nb, cell)
    sk, si = O.sort_pairs(keys, ids)
    start, end, spos, svel = O.find_cell_offset(sk, si, pos4, vel4, nb)
    return spos, svel, start, end, si


def main():
    ap = argparse.ArgumentParser()
    default = os.environ.get("FLUIDGRID_REFERENCE_DIR") or os.path.join(ROOT, "..", "reference")
    ap.add_argument("--reference-dir", default=os.path.abspath(default),
                    help="FluidGrid checkout ($FLUIDGRID_REFERENCE_DIR, else `reference` beside this repository)")
    args = ap.parse_args()
    if not os.path.isdir(os.path.join(args.reference_dir, "GPU_Kernels")):
        print("reference sources not found; nothing generated", file=sys.stderr)
        return 1
    lib = load_refk(args.reference_dir)
    rng = np.random.default_rng(0x6B5EED)

    cell = (np.float32(H),) * 3
    p = O.make_common_params(cell, BUCKETS, H, VLIMIT, BOX_MIN, BOX_MAX, GRAVITY, SCALE, DT, relation=REL,
                             point_radius=FLUID_RADIUS)
    kc = O.kernels_cache(H)
    assert lib.refk_params_size() == ctypes.sizeof(p), "CommonFluidParams layout"
    assert lib.refk_kernels_cache_size() == ctypes.sizeof(kc), "KernelsCache layout"
    lib.refk_set_params(ctypes.addressof(p), ctypes.addressof(kc))
    nb = int(np.prod(BUCKETS))

    # fluid: jittered block, 5% inactive, random velocities
    pos = lattice(16, 10, 16, SPACING, (SPACING, SPACING, SPACING), 0.05 * H, rng)
    n = pos.shape[0]
    pos[rng.random(n) < 0.05, 3] = -1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.normal(0, 0.5, (n, 3))
    spos, svel, start, end, ids = grid(pos, vel, cell, nb)

    dp = np.zeros((n, 2), np.float32)
    lib.refk_density(fp(spos), fp(dp), up(start), up(end), n, np.float32(GAS), np.float32(REST), np.float32(MASS))
    nv = np.zeros((n, 4), np.float32)
    lib.refk_forces(fp(spos), fp(svel), fp(dp), up(start), up(end), fp(nv), up(ids), np.float32(MASS), n,
                    np.float32(VISC))

    # rigid grids: a static plane under the block, a dynamic box across its top
    rb_cell = np.array([RB_RADIUS] * 3, np.float32)
    rb_nb = int(np.prod(RB_BUCKETS))
    g = np.arange(0.0, 0.42, RB_RADIUS)
    gx, gz = np.meshgrid(g, g, indexing="ij")
    spl = np.zeros((gx.size, 4), np.float32)
    spl[:, 0], spl[:, 1], spl[:, 2] = gx.ravel(), 0.012, gz.ravel()
    s_pos, _, s_start, s_end, _ = grid(spl, None, rb_cell, rb_nb)
    loc = box_surface(0.12, 384, rng)
    dyn = np.zeros((loc.shape[0], 4), np.float32)
    dyn[:, :3] = loc[:, :3] + np.array([0.2, 0.24, 0.2], np.float32)
    dyn[:, 3] = 0.0  # body index
    d_vel = rng.normal(0, 0.3, (1, 4)).astype(np.float32)  # per-body velocity
    d_pos, _, d_start, d_end, _ = grid(dyn, None, rb_cell, rb_nb)
    rel = np.array(REL, np.int32)
    srb = {}
    for tag, us, ud in (("static", 1, 0), ("dynamic", 0, 1), ("both", 1, 1)):
        o = np.zeros((n, 4), np.float32)
        lib.refk_forces_srb(fp(spos), fp(svel), fp(o), fp(dp), up(ids), up(start), up(end), n, np.float32(MASS),
                            np.float32(VISC), np.float32(FLUID_RADIUS), np.float32(RB_RADIUS),
                            np.float32(KSPRING), np.float32(KDAMP), fp(rb_cell), rel.ctypes.data_as(I), fp(s_pos),
                            up(s_start), up(s_end), rb_nb, fp(d_pos), fp(d_vel), up(d_start), up(d_end), rb_nb,
                            us, ud)
        srb[tag] = o
    # the rigid terms act on some particles in each case
    for tag in srb:
        assert (srb[tag] != nv).any(axis=1).sum() > 20, tag

    ipos = pos.copy()
    lib.refk_integrate(fp(ipos), fp(nv), n)

    # --- grid build through the reference's hash and range kernels; the sort
    # between them is thrust::sort_by_key in the reference (K_FluidSim.cu:685-691),
    # a stable key sort here
    G = lib.grid
    ckey = np.zeros(n, np.uint32)
    cids = np.zeros(n, np.uint32)
    G.refk_calc_hash_key(up(ckey), up(cids), fp(pos), n, nb, fp(np.array(cell, np.float32)))
    order = np.argsort(ckey, kind="stable")
    sk = np.ascontiguousarray(ckey[order])
    si = np.ascontiguousarray(cids[order])
    g_start = np.zeros(nb, np.uint32)
    g_end = np.zeros(nb, np.uint32)
    g_spos = np.zeros((n, 4), np.float32)
    g_svel = np.zeros((n, 4), np.float32)
    G.refk_find_cell_offset_pos_vel(up(g_start), up(g_end), up(sk), up(si), fp(pos), fp(g_spos), fp(vel),
                                    fp(g_svel), n, nb)
    # two bodies' spheres placed by their centres and orientations
    loc_a = box_surface(0.12, 300, rng)
    loc_b = box_surface(0.08, 200, rng)
    loc_b[:, 3] = 1.0
    local = np.ascontiguousarray(np.concatenate([loc_a, loc_b]).astype(np.float32))
    m = local.shape[0]
    cm = np.array([[0.20, 0.24, 0.20, 0.0], [0.29, 0.25, 0.22, 0.0]], np.float32)
    q = rng.normal(0, 1, (2, 4)).astype(np.float32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q = q.astype(np.float32)
    okey = np.zeros(m, np.uint32)
    oids = np.zeros(m, np.uint32)
    world = np.zeros((m, 4), np.float32)
    G.refk_calc_hash_key_with_offset(up(okey), up(oids), fp(cm), fp(q), fp(local), fp(world), m, fp(rb_cell),
                                     rb_nb)
    order = np.argsort(okey, kind="stable")
    rk = np.ascontiguousarray(okey[order])
    ri = np.ascontiguousarray(oids[order])
    r_start = np.zeros(rb_nb, np.uint32)
    r_end = np.zeros(rb_nb, np.uint32)
    r_spos = np.zeros((m, 4), np.float32)
    G.refk_find_cell_offset_pos(up(r_start), up(r_end), up(rk), up(ri), fp(world), fp(r_spos), m, rb_nb)

    # --- rigid kernels on the two bodies: sphere-sphere contact (with and
    # without the static plane), contact from the fluid, FP32 integration
    R = lib.rigid
    bvel = rng.normal(0, 0.3, (2, 4)).astype(np.float32)
    rbrb = {}
    for tag, nsrb in (("rbrb", 0), ("rbrb_static", 1)):
        T_ = np.zeros((m, 4), np.float32)
        F_ = np.zeros((m, 4), np.float32)
        R.refk_rb_forces_from_rb(fp(r_spos), fp(bvel), fp(cm), fp(T_), fp(F_), up(r_start), up(r_end), m,
                                 fp(rb_cell), np.float32(RB_RADIUS), rb_nb, rb_nb, fp(s_pos), up(s_start), up(s_end),
                                 np.float32(KSPRING), np.float32(KDAMP), nsrb)
        rbrb[tag] = (F_, T_)
    assert (np.abs(rbrb["rbrb"][0][:, :3]).sum(axis=1) > 0).sum() > 10, "bodies touch"
    ff = np.zeros((m, 4), np.float32)
    ft = np.zeros((m, 4), np.float32)
    R.refk_rb_forces_from_fluids(fp(r_spos), fp(bvel), fp(cm), fp(ff), fp(ft), up(r_start), up(r_end), m,
                                 fp(rb_cell), np.float32(RB_RADIUS), rb_nb, fp(spos), fp(svel), up(start), up(end),
                                 np.float32(FLUID_RADIUS), fp(np.array(cell, np.float32)), nb, rel.ctypes.data_as(I),
                                 np.float32(KSPRING), np.float32(KDAMP))
    assert (np.abs(ff[:, :3]).sum(axis=1) > 0).sum() > 10, "fluid touches the spheres"
    bx = cm.copy()
    bmass = np.array([10.0, 4.0], np.float32)
    bv = bvel.copy()
    bf = rng.normal(0, 50, (2, 4)).astype(np.float32)
    bL = rng.normal(0, 0.5, (2, 4)).astype(np.float32)
    bt = rng.normal(0, 2, (2, 4)).astype(np.float32)
    bI = np.zeros((2, 12), np.float32)
    binv = np.zeros((2, 12), np.float32)
    binv[:, 0] = binv[:, 5] = binv[:, 10] = 0.00125
    binv[1] += rng.normal(0, 1e-4, 12).astype(np.float32)
    bq = q.copy()
    ext = np.array([0.0, -9.8, 0.0, 0.0], np.float32)
    ix, iv, iL, iq = bx.copy(), bv.copy(), bL.copy(), bq.copy()
    R.refk_integrate_rb(fp(ix), fp(bmass), fp(iv), fp(bf), 2, np.float32(DT), fp(ext), fp(np.array(BOX_MIN, np.float32)),
                        fp(np.array(BOX_MAX, np.float32)), fp(iL), fp(bt), fp(bI), fp(iq), fp(binv), np.float32(VLIMIT))

    out = dict(pos=pos, vel=vel, spos=spos, svel=svel, start=start, end=end, ids=ids, dp=dp, newvel=nv,
               s_pos=s_pos, s_start=s_start, s_end=s_end, d_pos=d_pos, d_vel=d_vel, d_start=d_start, d_end=d_end,
               srb_static=srb["static"], srb_dynamic=srb["dynamic"], srb_both=srb["both"], integrated=ipos,
               buckets=np.array(BUCKETS, np.int64), rb_buckets=np.array(RB_BUCKETS, np.int64),
               rel=rel, rb_cell=rb_cell,
               scalars=np.array([H, SCALE, DT, VLIMIT, MASS, GAS, REST, VISC, FLUID_RADIUS, RB_RADIUS, KSPRING,
                                 KDAMP], np.float64),
               box=np.array([BOX_MIN, BOX_MAX], np.float32), gravity=np.array(GRAVITY, np.float32),
               hash_key=ckey, hash_ids=cids, grid_start=g_start, grid_end=g_end, grid_spos=g_spos,
               grid_svel=g_svel, rb_local=local, rb_cm=cm, rb_q=q, rb_world=world, rb_key=okey, rb_ids=oids,
               rb_start=r_start, rb_end=r_end, rb_spos=r_spos, rb_bvel=bvel,
               rbrb_force=rbrb["rbrb"][0], rbrb_torque=rbrb["rbrb"][1],
               rbrbs_force=rbrb["rbrb_static"][0], rbrbs_torque=rbrb["rbrb_static"][1],
               rbfl_force=ff, rbfl_torque=ft,
               int_in=np.concatenate([bx, bv, bf, bL, bt, bq], 1), int_mass=bmass, int_inv=binv, int_ext=ext,
               int_out=np.concatenate([ix, iv, iL, iq], 1))
    path = os.path.join(HERE, "ref_kernels.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
