"""Generate golden vectors from the reference's own helper source files.

Runs only where the reference sources are present: it builds
oracle/_ref/libfgref.so (oracle/ref_wrap.cpp compiled with the reference's
GPU_Kernels/K_DeviceFunctions.cu, K_Boundaries_*.cu and K_MathUtils.cu through
the self-written headers in oracle/ref_shim) and records inputs and outputs of
those helpers into tests/golden/ref_helpers.npz.  The CPU test suite checks the
oracle's restatement against this file; nothing at test time needs the
reference sources.

    python tests/golden/make_golden.py [--reference-dir DIR]
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

F = ctypes.POINTER(ctypes.c_float)
U = ctypes.POINTER(ctypes.c_uint32)
I = ctypes.POINTER(ctypes.c_int)


def fp(a):
    return a.ctypes.data_as(F)


def load_ref(reference_dir):
    subprocess.check_call(["make", "-s", "ref", "REFERENCE_DIR=" + reference_dir], cwd=ORACLE)
    lib = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libfgref.so"))
    lib.ref_hash_key.restype = ctypes.c_uint32
    lib.ref_hash_key.argtypes = [F, F, ctypes.c_int]
    lib.ref_walls_no_penetration.argtypes = [F, F, F, F] + [ctypes.c_float] * 4 + [F]
    lib.ref_walls_no_slip.argtypes = [F, F, F, F, F] + [ctypes.c_float] * 4 + [F]
    lib.ref_process_collision_forces.argtypes = [
        F, F, ctypes.c_float, F, F, ctypes.c_float, ctypes.c_float, ctypes.c_float, I, U, U, F,
        ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, F]
    for n in ("ref_quat_product", "ref_quat_transform_point", "ref_vec3_cross"):
        getattr(lib, n).argtypes = [F, F, F]
    lib.ref_quat_normalize.argtypes = [F, F]
    lib.ref_angular_velocity.argtypes = [F, F, F, F]
    return lib


def build_grid(lib, pos4, cell, nb):
    """Bucket grid of a sphere collection with the reference hash: stable sort
    by key, start/end by key boundaries, empty buckets start = 0xffffffff."""
    keys = np.array([lib.ref_hash_key(fp(np.ascontiguousarray(p[:3])), fp(cell), nb) for p in pos4],
                    dtype=np.uint32)
    order = np.argsort(keys, kind="stable")
    sk = keys[order]
    start = np.full(nb, 0xFFFFFFFF, dtype=np.uint32)
    end = np.zeros(nb, dtype=np.uint32)
    for i, k in enumerate(sk):
        if i == 0 or k != sk[i - 1]:
            start[k] = i
            if i > 0:
                end[sk[i - 1]] = i
    if len(sk):
        end[sk[-1]] = len(sk)
    return np.ascontiguousarray(pos4[order]), start, end, order


def main():
    ap = argparse.ArgumentParser()
    here = os.path.dirname(os.path.abspath(__file__))
    default = os.environ.get("FLUIDGRID_REFERENCE_DIR") or os.path.join(here, "..", "..", "..", "reference")
    ap.add_argument("--reference-dir", default=os.path.abspath(default),
                    help="FluidGrid checkout ($FLUIDGRID_REFERENCE_DIR, else `reference` beside this repository)")
    args = ap.parse_args()
    if not os.path.isdir(os.path.join(args.reference_dir, "GPU_Kernels")):
        print("reference sources not found; nothing generated", file=sys.stderr)
        return 1
    lib = load_ref(args.reference_dir)
    rng = np.random.default_rng(0x5EED)
    out = {}

    # --- HashKeyD: random, crafted (int32 wrap, negative, exact cell edges)
    h = np.float32(0.0457)
    cells = [np.array([h, h, h], np.float32), np.array([0.5 * h] * 3, np.float32),
             np.array([1.0, 0.75, 2.5], np.float32), np.array([0.02285, 0.02285, 0.02285], np.float32)]
    nbs = [262144, 2097152, 4093, 65536, 1000003]
    pos = np.concatenate([
        rng.uniform(-3, 5, (3000, 3)),
        rng.uniform(-5000, 5000, (500, 3)),
        rng.uniform(1e4, 1e5, (200, 3)),
        np.array([[0, 0, 0], [-0.0, 0.0457, 0.0914], [1e-8, -1e-8, 4.0]]),
    ]).astype(np.float32)
    # positions exactly on cell boundaries of the first cell size
    k = rng.integers(-50, 200, (300, 3)).astype(np.float32)
    pos = np.concatenate([pos, (k * h).astype(np.float32)]).astype(np.float32)
    hk_pos, hk_cell, hk_nb, hk_out = [], [], [], []
    for ci, c in enumerate(cells):
        for nb in nbs:
            sel = pos[rng.choice(len(pos), 400, replace=False)]
            for p in sel:
                hk_pos.append(p)
                hk_cell.append(c)
                hk_nb.append(nb)
                hk_out.append(lib.ref_hash_key(fp(np.ascontiguousarray(p)), fp(c), nb))
    out["hash_pos"] = np.array(hk_pos, np.float32)
    out["hash_cell"] = np.array(hk_cell, np.float32)
    out["hash_nb"] = np.array(hk_nb, np.int64)
    out["hash_key"] = np.array(hk_out, np.uint32)

    # --- walls (no-penetration against a box, no-slip against the literal box)
    n = 2000
    vmin = np.array([0.0, 0.0, 0.0], np.float32)
    vmax = np.array([1.0, 1.0, 1.0], np.float32)
    wp = rng.uniform(-0.01, 1.01, (n, 3)).astype(np.float32)
    wp[: n // 2] = np.where(rng.random((n // 2, 3)) < 0.5, rng.uniform(-0.004, 0.004, (n // 2, 3)),
                            rng.uniform(0.996, 1.004, (n // 2, 3))).astype(np.float32)
    wv = rng.normal(0, 2, (n, 3)).astype(np.float32)
    wf = rng.normal(0, 50, (n, 3)).astype(np.float32)
    scales = rng.choice(np.array([1.0, 0.009, 0.5], np.float32), n)
    np_out = np.zeros((n, 3), np.float32)
    ns_out = np.zeros((n, 3), np.float32)
    nsmin = np.array([-11.0, -40.0, -11.0], np.float32)
    nsmax = np.array([11.0, 200.0, 11.0], np.float32)
    # no-slip inputs near the literal box walls
    sp = rng.uniform(-12, 12, (n, 3)).astype(np.float32)
    sp[:, 1] = rng.uniform(-41, 201, n)
    sel = rng.random((n, 3)) < 0.5
    edge = np.where(rng.random((n, 3)) < 0.5, nsmin + rng.uniform(-0.002, 0.004, (n, 3)),
                    nsmax + rng.uniform(-0.004, 0.002, (n, 3)))
    sp = np.where(sel, edge, sp).astype(np.float32)
    fk = rng.choice(np.array([0.0, 0.3], np.float32), n)
    fs = rng.choice(np.array([0.0, -0.5, 0.5], np.float32), n)
    for i in range(n):
        o = np.zeros(3, np.float32)
        lib.ref_walls_no_penetration(fp(wp[i]), fp(wv[i]), fp(vmin), fp(vmax), np.float32(0.003043174),
                                     np.float32(20000), np.float32(256), scales[i], fp(o))
        np_out[i] = o
        o2 = np.zeros(3, np.float32)
        lib.ref_walls_no_slip(fp(sp[i]), fp(wv[i]), fp(wf[i]), fp(nsmin), fp(nsmax), np.float32(0.003043174),
                              fk[i], fs[i], np.float32(1.0), fp(o2))
        ns_out[i] = o2
    out.update(walls_pos=wp, walls_vel=wv, walls_force=wf, walls_scale=scales, walls_np=np_out,
               walls_min=vmin, walls_max=vmax, noslip_pos=sp, noslip_fkin=fk, noslip_fstatic=fs,
               walls_ns=ns_out)

    # --- ProcessCollisionForcesD over small sphere collections
    cases = []
    for ci, (rel, cell_s, nb, w_rb, check, eps) in enumerate([
            ((1, 1, 1), 0.0457, 4096, 0, 0, 0.0001),
            ((2, 2, 2), 0.02285, 4093, 1, 0, 0.003),
            ((1, 1, 1), 0.02285, 1024, 1, 1, 0.001),
            ((1, 2, 1), 0.03, 512, 0, 0, 0.003)]):
        m = 600
        cpos = np.zeros((m, 4), np.float32)
        cpos[:, :3] = rng.uniform(0.3, 0.6, (m, 3))
        cpos[:, 3] = rng.integers(0, 3, m)
        cell = np.array([cell_s] * 3, np.float32)
        spos, start, end, order = build_grid(lib, cpos, cell, nb)
        if w_rb:
            cvel = rng.normal(0, 1, (3, 4)).astype(np.float32)
        else:
            cvel = rng.normal(0, 1, (m, 4)).astype(np.float32)
        q = 200
        qpos = np.zeros((q, 4), np.float32)
        qpos[:, :3] = rng.uniform(0.28, 0.62, (q, 3))
        qpos[:, 3] = rng.integers(0, 3, q)
        qvel = rng.normal(0, 1, (q, 4)).astype(np.float32)
        res = np.zeros((q, 3), np.float32)
        rel_a = np.array(rel, np.int32)
        for i in range(q):
            o = np.zeros(3, np.float32)
            lib.ref_process_collision_forces(
                fp(qpos[i]), fp(qvel[i]), np.float32(0.02285), fp(spos), fp(cvel), np.float32(0.0114),
                np.float32(-10.0), np.float32(-5.0), rel_a.ctypes.data_as(I), start.ctypes.data_as(U),
                end.ctypes.data_as(U), fp(cell), nb, w_rb, check, int(qpos[i, 3]), np.float32(eps), fp(o))
            res[i] = o
        pre = "coll%d_" % ci
        out.update({pre + "cpos": spos, pre + "cvel": cvel, pre + "start": start, pre + "end": end,
                    pre + "cell": cell, pre + "nb": np.int64(nb), pre + "rel": rel_a,
                    pre + "flags": np.array([w_rb, check], np.int32), pre + "eps": np.float32(eps),
                    pre + "qpos": qpos, pre + "qvel": qvel, pre + "out": res})
        cases.append(ci)
    out["coll_cases"] = np.array(cases, np.int32)

    # --- quaternion / matrix helpers
    nq = 1000
    qa = rng.normal(0, 1, (nq, 4)).astype(np.float32)
    qb = rng.normal(0, 1, (nq, 4)).astype(np.float32)
    qu = (qb / np.linalg.norm(qb, axis=1, keepdims=True)).astype(np.float32)
    pp = rng.uniform(-0.3, 0.3, (nq, 4)).astype(np.float32)
    pp[:, 3] = rng.integers(0, 8, nq)
    inv = np.zeros((nq, 12), np.float32)
    inv[:, 0] = inv[:, 5] = inv[:, 10] = 0.00125
    inv[nq // 2:, :] = rng.normal(0, 0.01, (nq - nq // 2, 12)).astype(np.float32)
    Lm = rng.normal(0, 50, (nq, 4)).astype(np.float32)
    prod = np.zeros((nq, 4), np.float32)
    tr = np.zeros((nq, 4), np.float32)
    nrm = np.zeros((nq, 4), np.float32)
    crs = np.zeros((nq, 4), np.float32)
    angv = np.zeros((nq, 4), np.float32)
    for i in range(nq):
        for fn, a, b, dst in ((lib.ref_quat_product, qa[i], qb[i], prod), (lib.ref_quat_transform_point, pp[i], qu[i], tr),
                              (lib.ref_vec3_cross, qa[i], qb[i], crs)):
            o = np.zeros(4, np.float32)
            fn(fp(np.ascontiguousarray(a)), fp(np.ascontiguousarray(b)), fp(o))
            dst[i] = o
        o = np.zeros(4, np.float32)
        lib.ref_quat_normalize(fp(np.ascontiguousarray(qa[i])), fp(o))
        nrm[i] = o
        o = np.zeros(4, np.float32)
        lib.ref_angular_velocity(fp(np.ascontiguousarray(inv[i])), fp(np.ascontiguousarray(Lm[i])),
                                 fp(np.ascontiguousarray(qu[i])), fp(o))
        angv[i] = o
    out.update(q_a=qa, q_b=qb, q_unit=qu, q_point=pp, q_inv=inv, q_L=Lm, q_prod=prod, q_transform=tr,
               q_normalize=nrm, q_cross=crs, q_angvel=angv)

    path = os.path.join(HERE, "ref_helpers.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
