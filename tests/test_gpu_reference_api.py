"""The reference-named launchers (include/fluidgrid_reference.h) driven in the
order of the reference's own host code, against the oracle:

  HeterogeneousSimulator::doTimeStep (HeterogeneousSimulator.cpp:54-127):
    gCalcHashKey -> gSort -> gFindCellOffsetOrderingPosVel -> gCalcMassDensity
    -> gSPHCalculateForces -> gSPHIntegrate
  two-way coupling (HeterogeneousSimulator.cpp:57-126, RigidBodySimulator.cpp:
  334-611): gCalcHashKeyWithOffset -> sort -> gFindCellOffsetOrderingPos ->
  gCalculateRigidBodyForcesFromFluids -> gSPHCalculateForcesWithSRB ->
  gCopyRBDataToParticle -> sort -> gReorderForceTorque -> segmented scan ->
  gAddForceTorque -> gIntegrateRB

Device memory comes from torch (plumbing only); every computation runs in
libfluidgrid_gb300.so.  Tolerances as in test_gpu_fluid / test_gpu_rigid;
gIntegrateRB is bit-exact against the FP32 oracle.
"""
import ctypes

import numpy as np
import pytest

from fluidgrid_gb300 import _ffi, build, scenes
from fluidgrid_gb300._ffi import float3, float4, int3, fgr_kernels_cache
from oracle import oracle as O
import helpers as T
import test_gpu_rigid as R

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def L():
    build.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _ffi.load()


def dev(a):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    torch.cuda.synchronize()
    return t


def p(t):
    return ctypes.c_void_p(t.data_ptr())


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def u32(n):
    return torch.zeros(n, dtype=torch.int32, device="cuda")


def f4(n):
    return torch.zeros((n, 4), dtype=torch.float32, device="cuda")


def kcache(h):
    k = O.kernels_cache(h)
    return fgr_kernels_cache(k.kPoly6, k.kSpikyGradient, k.kViscosityLaplacian)


def test_do_time_step_through_reference_launchers(L):
    spec = scenes.dam_break_small(seed=99)
    n, nb = spec.n, spec.nbuckets
    rng = np.random.default_rng(4)
    vel0 = np.zeros((n, 4), np.float32)
    vel0[:, :3] = rng.normal(0, 0.3, (n, 3))
    L.gInitializeCommonFluidParams(spec.common_params())
    L.gInitializeKernelParams(kcache(spec.h))
    pos, vel = dev(spec.pos), dev(vel0)
    key, pid, start, end = u32(n), u32(n), u32(nb), u32(nb)
    opos, ovel, forces = f4(n), f4(n), f4(n)
    dp = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    cs = float3(*spec.cell_size)
    L.gCalcHashKey(p(key), p(pid), p(pos), n, nb, cs)
    assert L.fgc_last_status() == 0
    ref = T.oracle_grid(spec, spec.pos, vel0)
    assert np.array_equal(host(key).view(np.uint32), ref["keys"])
    assert np.array_equal(host(pid).view(np.uint32), np.arange(n, dtype=np.uint32))
    L.gSort(p(key), p(pid), n)
    assert L.fgc_last_status() == 0
    assert np.array_equal(host(key).view(np.uint32), ref["skeys"])
    assert np.array_equal(host(pid).view(np.uint32), ref["ids"])
    L.gFindCellOffsetOrderingPosVel(p(start), p(end), p(key), p(pid), p(pos), p(opos), p(vel), p(ovel), n, nb)
    T.compare_ranges(host(start).view(np.uint32), host(end).view(np.uint32), ref["start"], ref["end"])
    assert np.array_equal(host(opos), ref["spos"]) and np.array_equal(host(ovel), ref["svel"])
    L.gCalcMassDensity(p(opos), p(dp), p(key), p(start), p(end), n, spec.gas, spec.rest, spec.mass)
    assert L.fgc_last_status() == 0
    kc = O.kernels_cache(spec.h)
    d64, _ = O.density(ref["spos"], ref["start"], ref["end"], ref["p"], kc, spec.gas, spec.rest, spec.mass, f64=True)
    dpg = host(dp)
    assert (np.abs(dpg[:, 0] - d64[:, 0]) / d64[:, 0]).max() <= 1e-5
    L.gSPHCalculateForces(p(opos), p(ovel), p(forces), p(dp), p(start), p(end), p(vel), p(pid), n, spec.mass,
                          spec.visc)
    assert L.fgc_last_status() == 0
    nv = O.forces(ref["spos"], ref["svel"], dpg, ref["start"], ref["end"], ref["ids"], spec.mass, spec.visc,
                  ref["p"], kc, newvel_init=vel0)
    vg = host(vel)
    Fg, Fr = T.force_from_vel(vg, vel0, spec.dt), T.force_from_vel(nv, vel0, spec.dt)
    mag = np.linalg.norm(Fr, axis=1)
    assert (np.linalg.norm(Fg - Fr, axis=1) / np.maximum(mag, np.median(mag))).max() <= 2e-4
    L.gSPHIntegrate(p(pos), p(vel), p(forces), n, p(dp), p(start), p(end))
    assert L.fgc_last_status() == 0
    pi = O.integrate(spec.pos, vg, ref["p"])
    assert np.array_equal(host(pos).view(np.uint32), pi.view(np.uint32))


def test_gsort_full_32bit_keys(L):
    rng = np.random.default_rng(17)
    for n in (1, 5, 4096, 4097, 100003):
        k = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
        k[: n // 3] = k[n // 2]  # many ties
        v = np.arange(n, dtype=np.uint32)
        kt, vt = dev(k.view(np.int32)), dev(v.view(np.int32))
        L.gSort(p(kt), p(vt), n)
        ko, vo = O.sort_pairs(k, v)
        assert np.array_equal(host(kt).view(np.uint32), ko)
        assert np.array_equal(host(vt).view(np.uint32), vo)


def test_two_way_coupling_through_reference_launchers(L):
    spec = R.rigid_scene(nbodies=2)
    n, nb = spec.n, spec.nbuckets
    L.gInitializeCommonFluidParams(spec.common_params())
    L.gInitializeKernelParams(kcache(spec.h))
    vel0 = np.zeros((n, 4), np.float32)
    ref = T.oracle_grid(spec, spec.pos, vel0)
    # fluid grid from the oracle (already pinned above): upload sorted state
    opos, ovel = dev(ref["spos"]), dev(ref["svel"])
    start, end = dev(ref["start"].view(np.int32)), dev(ref["end"].view(np.int32))
    pid = dev(ref["ids"].view(np.int32))
    dp = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    key = dev(ref["skeys"].view(np.int32))
    L.gCalcMassDensity(p(opos), p(dp), p(key), p(start), p(end), n, spec.gas, spec.rest, spec.mass)
    # rigid spheres: body-major local offsets, w = body index (addElement, RigidBodySimulator.cpp:120-130)
    loc = np.concatenate([np.c_[b.local[:, :3], np.full(len(b.local), i, np.float32)]
                          for i, b in enumerate(spec.bodies)]).astype(np.float32)
    cm = np.array([list(b.position) + [0.0] for b in spec.bodies], np.float32)
    q = np.array([b.orientation for b in spec.bodies], np.float32)
    bvel = np.array([[0.1, -0.2, 0.05, 0.0], [-0.1, 0.0, 0.3, 0.0]], np.float32)
    m = loc.shape[0]
    rnb = int(np.prod(spec.rb_buckets))
    rcell = float3(spec.rb_radius, spec.rb_radius, spec.rb_radius)
    t_loc, t_cm, t_q, t_bv = dev(loc), dev(cm), dev(q), dev(bvel)
    rkey, rid, rworld, rsorted = u32(m), u32(m), f4(m), f4(m)
    rstart, rend = u32(rnb), u32(rnb)
    L.gCalcHashKeyWithOffset(p(rkey), p(rid), p(t_cm), p(t_q), p(t_loc), p(rworld), m, rcell, rnb)
    rk, ri, rw = O.calc_hash_key_with_offset(loc, cm, q, rnb, (spec.rb_radius,) * 3)
    assert np.array_equal(host(rkey).view(np.uint32), rk)
    assert np.array_equal(host(rworld).view(np.uint32), rw.view(np.uint32))
    bits = int(np.ceil(np.log2(rnb)))
    L.fgc_sort_pairs(p(rkey), p(rid), bits, m)
    rsk, rsi = O.sort_pairs(rk, ri)
    assert np.array_equal(host(rid).view(np.uint32), rsi)
    L.gFindCellOffsetOrderingPos(p(rstart), p(rend), p(rkey), p(rid), p(rworld), p(rsorted), m, rnb)
    rs0, re0, rsp, _ = O.find_cell_offset(rsk, rsi, rw, None, rnb)
    T.compare_ranges(host(rstart).view(np.uint32), host(rend).view(np.uint32), rs0, re0)
    assert np.array_equal(host(rsorted), rsp)
    # rigid side: CalculateRBForcesFromFluidsK
    Fo, To = f4(m), f4(m)
    rel = int3(*spec.r2f_rel)
    L.gCalculateRigidBodyForcesFromFluids(p(rsorted), p(t_bv), p(t_cm), p(Fo), p(To), p(rstart), p(rend), m, rcell,
                                          spec.rb_radius, rnb, p(opos), p(ovel), p(start), p(end),
                                          spec.fluid_radius, float3(*spec.cell_size), nb, rel, spec.ck, spec.ckd)
    Fr, Tr = O.rb_forces_from_fluids(rsp, bvel, cm, spec.rb_radius, ref["spos"], ref["svel"], ref["start"],
                                     ref["end"], spec.fluid_radius, spec.cell_size, nb, spec.r2f_rel, spec.ck,
                                     spec.ckd)
    Fg, Tg = host(Fo), host(To)
    assert R._close(Fg[:, :3], Fr[:, :3], 1e-4) and R._close(Tg[:, :3], Tr[:, :3], 1e-4)
    assert np.array_equal(Fg[:, 3], Fr[:, 3])
    # fluid side: SPHCalculateForcesWithSRBK with the dynamic grid
    newvel = dev(vel0)
    dummy_u = u32(8)
    L.gSPHCalculateForcesWithSRB(p(opos), p(ovel), p(f4(1)), p(newvel), p(dp), p(pid), p(start), p(end), n,
                                 spec.mass, spec.visc, spec.fluid_radius, int3(*spec.f2r_rel), spec.rb_radius, rcell,
                                 spec.ck, spec.ckd, p(f4(1)), p(dummy_u), p(dummy_u), 8, p(rsorted), p(t_bv),
                                 p(rstart), p(rend), rnb, False, True)
    assert L.fgc_last_status() == 0
    kc = O.kernels_cache(spec.h)
    cp = O.contact_params(spec.fluid_radius, spec.rb_radius, spec.ck, spec.ckd, (spec.rb_radius,) * 3,
                          spec.f2r_rel, 0.003)
    dg = O.contact_grid(rsp, bvel, rs0, re0, rnb)
    dpg = host(dp)
    nv = O.forces(ref["spos"], ref["svel"], dpg, ref["start"], ref["end"], ref["ids"], spec.mass, spec.visc,
                  ref["p"], kc, newvel_init=vel0, contact=(cp, None, dg))
    Fv, Fvr = T.force_from_vel(host(newvel), vel0, spec.dt), T.force_from_vel(nv, vel0, spec.dt)
    mag = np.linalg.norm(Fvr, axis=1)
    assert (np.linalg.norm(Fv - Fvr, axis=1) / np.maximum(mag, np.median(mag))).max() <= 2e-4
    # applyForces (RigidBodySimulator.cpp:522-566)
    bkey, bidx = u32(m), u32(m)
    L.gCopyRBDataToParticle(p(bkey), p(bidx), p(Fo), m)
    L.fgc_sort_pairs(p(bkey), p(bidx), 8, m)
    Fs, Ts = f4(m), f4(m)
    L.gReorderForceTorque(p(Fs), p(Ts), p(Fo), p(To), p(bidx), m)
    flags = np.zeros(m, np.uint32)
    counts = [len(b.local) for b in spec.bodies]
    offs = np.cumsum([0] + counts)
    flags[offs[:-1]] = 1
    tf = dev(flags.view(np.int32))
    Fscan, Tscan = f4(m), f4(m)
    L.fgc_segmented_scan_float4(p(Fscan), p(Fs), p(tf), m)
    L.fgc_segmented_scan_float4(p(Tscan), p(Ts), p(tf), m)
    last = dev((offs[1:] - 1).astype(np.int32))
    bF, bT = f4(2), f4(2)
    L.gAddForceTorque(p(Fscan), p(Tscan), p(Fs), p(bF), p(bT), p(last), 2)
    assert L.fgc_last_status() == 0
    sF, sT = O.rb_reduce(Fg, Tg, 2)
    gbF, gbT = host(bF).astype(np.float64), host(bT).astype(np.float64)
    assert np.allclose(gbF, sF, rtol=1e-5, atol=1e-5 * np.abs(sF).max())
    assert np.allclose(gbT, sT, rtol=1e-5, atol=1e-5 * np.abs(sT).max())
    # IntegrateRBK in FP32, bit-exact against the FP32 oracle
    mass = np.array([b.mass for b in spec.bodies], np.float32)
    L4 = np.zeros((2, 4), np.float32)
    inv = np.zeros((2, 12), np.float32)
    inv[:, [0, 5, 10]] = 0.00125
    inertia = np.zeros((2, 12), np.float32)
    ext = np.array([0.0, -9.8, 0.0, 0.0], np.float32)
    tx, tm, tv, tL, tqq = dev(cm), dev(mass), dev(bvel), dev(L4), dev(q)
    L.gIntegrateRB(p(tx), p(tm), p(tv), p(bF), 2, spec.dt, float4(*ext), float3(*spec.box_min),
                   float3(*spec.box_max), p(tL), p(bT), p(dev(inertia)), p(tqq), p(dev(inv)), spec.rb_vlimit)
    assert L.fgc_last_status() == 0
    x, v, Lr, qr = O.integrate_rb(cm, mass, bvel, host(bF), spec.dt, ext, spec.box_min, spec.box_max, L4,
                                  host(bT), q, inv, spec.rb_vlimit)
    for got, want in ((host(tx), x), (host(tv), v), (host(tL), Lr), (host(tqq), qr)):
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _sphere_grid(L, loc, cm, q, rnb, radius):
    """gCalcHashKeyWithOffset -> stable sort -> gFindCellOffsetOrderingPos on
    the GPU (bit-exact against the oracle), as RigidBodySimulator.cpp:146-214
    builds the static grid and :464-474 the dynamic one."""
    m = loc.shape[0]
    rcell = float3(radius, radius, radius)
    t_loc, t_cm, t_q = dev(loc), dev(cm), dev(q)
    rkey, rid, rworld, rsorted = u32(m), u32(m), f4(m), f4(m)
    rstart, rend = u32(rnb), u32(rnb)
    L.gCalcHashKeyWithOffset(p(rkey), p(rid), p(t_cm), p(t_q), p(t_loc), p(rworld), m, rcell, rnb)
    rk, ri, rw = O.calc_hash_key_with_offset(loc, cm, q, rnb, (radius,) * 3)
    assert np.array_equal(host(rkey).view(np.uint32), rk)
    L.fgc_sort_pairs(p(rkey), p(rid), int(np.ceil(np.log2(rnb))), m)
    rsk, rsi = O.sort_pairs(rk, ri)
    assert np.array_equal(host(rid).view(np.uint32), rsi)
    L.gFindCellOffsetOrderingPos(p(rstart), p(rend), p(rkey), p(rid), p(rworld), p(rsorted), m, rnb)
    rs0, re0, rsp, _ = O.find_cell_offset(rsk, rsi, rw, None, rnb)
    T.compare_ranges(host(rstart).view(np.uint32), host(rend).view(np.uint32), rs0, re0)
    assert np.array_equal(host(rsorted), rsp)
    return dict(pos=rsorted, start=rstart, end=rend, ref_pos=rsp, ref_start=rs0, ref_end=re0, ids=rsi)


def test_static_and_dynamic_grids_through_reference_launchers(L):
    """SPHCalculateForcesWithSRBK with both the static grid (useStaticRB,
    K_FluidSim.cu:371-377) and the dynamic grid (:380-386), and
    CalculateRigidBodyForcesFromRBK (K_RigidBodySim.cu:18-61) with its
    static-grid term (numSRB > 0), each against the oracle."""
    spec = R.static_dynamic_scene()
    n, nb = spec.n, spec.nbuckets
    L.gInitializeCommonFluidParams(spec.common_params())
    L.gInitializeKernelParams(kcache(spec.h))
    vel0 = np.zeros((n, 4), np.float32)
    vel0[:, :3] = np.random.default_rng(9).normal(0, 0.2, (n, 3))
    ref = T.oracle_grid(spec, spec.pos, vel0)
    opos, ovel = dev(ref["spos"]), dev(ref["svel"])
    start, end = dev(ref["start"].view(np.int32)), dev(ref["end"].view(np.int32))
    pid = dev(ref["ids"].view(np.int32))
    key = dev(ref["skeys"].view(np.int32))
    dp = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    L.gCalcMassDensity(p(opos), p(dp), p(key), p(start), p(end), n, spec.gas, spec.rest, spec.mass)
    rnb = int(np.prod(spec.rb_buckets))
    r = spec.rb_radius
    # static grid: body 0's spheres in world space (RigidBodySimulator.cpp:146-214)
    b0 = spec.bodies[0]
    sloc = np.c_[b0.local[:, :3], np.zeros(len(b0.local), np.float32)].astype(np.float32)
    scm = np.array([list(b0.position) + [0.0]], np.float32)
    sq = np.array([b0.orientation], np.float32)
    sg = _sphere_grid(L, sloc, scm, sq, rnb, r)
    # dynamic grid: bodies 1 and 2, w = dynamic body index
    dyn = spec.bodies[1:]
    dloc = np.concatenate([np.c_[b.local[:, :3], np.full(len(b.local), i, np.float32)]
                           for i, b in enumerate(dyn)]).astype(np.float32)
    dcm = np.array([list(b.position) + [0.0] for b in dyn], np.float32)
    dq = np.array([b.orientation for b in dyn], np.float32)
    bvel = np.array([[0.2, -0.1, 0.0, 0.0], [-0.3, 0.05, 0.1, 0.0]], np.float32)
    dg = _sphere_grid(L, dloc, dcm, dq, rnb, r)
    t_bv, t_cm = dev(bvel), dev(dcm)
    rcell = float3(r, r, r)
    # fluid side: both grids
    newvel = dev(vel0)
    L.gSPHCalculateForcesWithSRB(p(opos), p(ovel), p(f4(1)), p(newvel), p(dp), p(pid), p(start), p(end), n,
                                 spec.mass, spec.visc, spec.fluid_radius, int3(*spec.f2r_rel), r, rcell, spec.ck,
                                 spec.ckd, p(sg["pos"]), p(sg["start"]), p(sg["end"]), rnb, p(dg["pos"]), p(t_bv),
                                 p(dg["start"]), p(dg["end"]), rnb, True, True)
    assert L.fgc_last_status() == 0
    kc = O.kernels_cache(spec.h)
    cp = O.contact_params(spec.fluid_radius, r, spec.ck, spec.ckd, (r,) * 3, spec.f2r_rel, 0.003)
    o_sg = O.contact_grid(sg["ref_pos"], None, sg["ref_start"], sg["ref_end"], rnb)
    o_dg = O.contact_grid(dg["ref_pos"], bvel, dg["ref_start"], dg["ref_end"], rnb)
    dpg = host(dp)
    args = (ref["spos"], ref["svel"], dpg, ref["start"], ref["end"], ref["ids"], spec.mass, spec.visc, ref["p"], kc)
    nv = O.forces(*args, newvel_init=vel0, contact=(cp, o_sg, o_dg))
    nv_dyn = O.forces(*args, newvel_init=vel0, contact=(cp, None, o_dg))
    Fv, Fvr = T.force_from_vel(host(newvel), vel0, spec.dt), T.force_from_vel(nv, vel0, spec.dt)
    touched = np.linalg.norm(Fvr - T.force_from_vel(nv_dyn, vel0, spec.dt), axis=1) > 0
    assert touched.sum() > 20, "the static-grid term must act on some fluid particles"
    mag = np.linalg.norm(Fvr, axis=1)
    assert (np.linalg.norm(Fv - Fvr, axis=1) / np.maximum(mag, np.median(mag))).max() <= 2e-4
    # rigid side: dynamic spheres against the other dynamic body and the static grid
    m = dloc.shape[0]
    Fo, To = f4(m), f4(m)
    L.gCalculateRigidBodyForcesFromRB(p(dg["pos"]), p(t_bv), p(t_cm), p(To), p(Fo), p(dg["start"]), p(dg["end"]),
                                      m, rcell, r, rnb, rnb, p(sg["pos"]), p(sg["start"]), p(sg["end"]),
                                      spec.rbrb_k, spec.rbrb_kd, 1)
    assert L.fgc_last_status() == 0
    srb = (sg["ref_pos"], sg["ref_start"], sg["ref_end"], rnb, 1)
    Fr, Tr = O.rb_forces_from_rb(dg["ref_pos"], bvel, dcm, dg["ref_start"], dg["ref_end"], (r,) * 3, r, rnb,
                                 spec.rbrb_k, spec.rbrb_kd, srb=srb)
    Fd, _ = O.rb_forces_from_rb(dg["ref_pos"], bvel, dcm, dg["ref_start"], dg["ref_end"], (r,) * 3, r, rnb,
                                spec.rbrb_k, spec.rbrb_kd)
    n_dyn = int((np.abs(Fd[:, :3]) > 0).any(1).sum())
    n_sta = int((np.abs(Fr[:, :3] - Fd[:, :3]) > 0).any(1).sum())
    assert n_dyn > 10 and n_sta > 10, (n_dyn, n_sta)
    Fg, Tg = host(Fo), host(To)
    assert R._close(Fg[:, :3], Fr[:, :3], 1e-4) and R._close(Tg[:, :3], Tr[:, :3], 1e-4)
    assert np.array_equal(Fg[:, 3], Fr[:, 3]) and np.array_equal(Tg[:, 3], Tr[:, 3])
