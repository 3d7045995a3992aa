"""ctypes binding of the CPU oracle (oracle/fg_oracle.cpp).

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, the smoke check in
__graft_entry__.py and the CPU-baseline leg of bench.py import this module,
and only as the checker or as the timed CPU restatement of the reference.

`step()` restates the reference's per-step orchestration
(HeterogeneousSimulator.cpp:54-212 for the fluid; the reconstructed two-way
order of the commented block HeterogeneousSimulator.cpp:57-126 with
RigidBodySimulator.cpp:334-611 for the rigid bodies).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfgoracle.so")

F = ctypes.POINTER(ctypes.c_float)
D = ctypes.POINTER(ctypes.c_double)
U = ctypes.POINTER(ctypes.c_uint32)
I = ctypes.POINTER(ctypes.c_int)
LL = ctypes.POINTER(ctypes.c_longlong)


class Float3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


class Int3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int), ("y", ctypes.c_int), ("z", ctypes.c_int)]


class CommonFluidParams(ctypes.Structure):
    """Layout of Simulation::Application::CommonFluidParams (ApplicationData.cuh:46-67)."""
    _fields_ = [("cell_size", Float3), ("bucket_size", Int3), ("keyBits", ctypes.c_uint32),
                ("kernel_radius", ctypes.c_float), ("kernel_radius_squared", ctypes.c_float),
                ("pointRadius", ctypes.c_float), ("pointScale", ctypes.c_float),
                ("velocity_limit", ctypes.c_float), ("volume_min", Float3), ("volume_max", Float3),
                ("global_external_force", Float3), ("simulation_scale", ctypes.c_float),
                ("deltaTimeIntegration", ctypes.c_float), ("fluid_to_srb_relation", Int3)]


class KernelsCache(ctypes.Structure):
    _fields_ = [("kPoly6", ctypes.c_float), ("kSpikyGradient", ctypes.c_float),
                ("kViscosityLaplacian", ctypes.c_float)]


class ContactGrid(ctypes.Structure):
    _fields_ = [("pos4", F), ("vel4", F), ("start", U), ("end", U), ("nbuckets", ctypes.c_uint32),
                ("use", ctypes.c_int)]


class ContactParams(ctypes.Structure):
    _fields_ = [("fluid_radius", ctypes.c_float), ("rb_radius", ctypes.c_float),
                ("kspring", ctypes.c_float), ("kdamping", ctypes.c_float),
                ("cell", ctypes.c_float * 3), ("rel", ctypes.c_int * 3), ("eps", ctypes.c_float)]


_lib = None


def build():
    """Compile the oracle library (oracle/Makefile)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "fg_oracle.cpp")):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        L.fgo_hash_key.restype = ctypes.c_uint32
        L.fgo_hash_key.argtypes = [F, F, ctypes.c_int]
        L.fgo_walls_no_penetration.argtypes = [F, F, F, F] + [ctypes.c_float] * 4 + [F]
        L.fgo_walls_no_slip.argtypes = [F, F, F, F, F] + [ctypes.c_float] * 4 + [F]
        L.fgo_process_collision_forces.argtypes = [
            F, F, ctypes.c_float, F, F, ctypes.c_float, ctypes.c_float, ctypes.c_float, I, U, U, F,
            ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, F]
        for n in ("fgo_quat_product", "fgo_quat_transform_point", "fgo_vec3_cross"):
            getattr(L, n).argtypes = [F, F, F]
        L.fgo_quat_normalize.argtypes = [F, F]
        L.fgo_angular_velocity.argtypes = [F, F, F, F]
        L.fgo_compute_kernels_cache.argtypes = [ctypes.c_float, P(KernelsCache)]
        L.fgo_calc_hash_key.argtypes = [U, U, F, ctypes.c_int, ctypes.c_uint32, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_float]
        L.fgo_calc_hash_key_with_offset.argtypes = [U, U, F, F, F, F, ctypes.c_int, ctypes.c_float,
                                                    ctypes.c_float, ctypes.c_float, ctypes.c_int]
        L.fgo_sort_pairs.argtypes = [U, U, ctypes.c_int]
        L.fgo_find_cell_offset.argtypes = [U, U, U, U, F, F, F, F, ctypes.c_int, ctypes.c_uint32]
        cfp = P(CommonFluidParams)
        kcp = P(KernelsCache)
        L.fgo_density_f32.argtypes = [F, F, U, U, ctypes.c_int, cfp, kcp, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, LL]
        L.fgo_density_f64.argtypes = [F, D, U, U, ctypes.c_int, cfp, kcp, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, LL]
        L.fgo_forces_f32.argtypes = [F, F, F, U, U, F, U, ctypes.c_float, ctypes.c_int, ctypes.c_float, cfp, kcp]
        L.fgo_forces_f64.argtypes = [F, F, D, U, U, D, U, ctypes.c_float, ctypes.c_int, ctypes.c_float, cfp, kcp]
        cpp = P(ContactParams)
        cgp = P(ContactGrid)
        L.fgo_forces_f64_fdp.argtypes = [F, F, F, U, U, D, U, ctypes.c_float, ctypes.c_int, ctypes.c_float, cfp,
                                         kcp, cpp, cgp, cgp]
        L.fgo_forces_srb_f32.argtypes = [F, F, F, U, U, F, U, ctypes.c_float, ctypes.c_int, ctypes.c_float, cfp,
                                         kcp, cpp, cgp, cgp]
        L.fgo_integrate_f32.argtypes = [F, F, ctypes.c_int, cfp]
        L.fgo_rb_forces_from_fluids_f32.argtypes = [F, F, F, F, F, ctypes.c_int, ctypes.c_float, F, F, U, U,
                                                    ctypes.c_float, F, ctypes.c_uint32, I, ctypes.c_float,
                                                    ctypes.c_float]
        L.fgo_rb_forces_from_fluids_f64.argtypes = [F, F, F, D, D, ctypes.c_int, ctypes.c_float, F, F, U, U,
                                                    ctypes.c_float, F, ctypes.c_uint32, I, ctypes.c_float,
                                                    ctypes.c_float]
        L.fgo_rb_forces_from_rb_f32.argtypes = [F, F, F, F, F, U, U, ctypes.c_int, F, ctypes.c_float,
                                                ctypes.c_int, ctypes.c_int, F, U, U, ctypes.c_float,
                                                ctypes.c_float, ctypes.c_int]
        L.fgo_rb_reduce_f64.argtypes = [F, F, ctypes.c_int, ctypes.c_int, D, D]
        L.fgo_integrate_rb_f32.argtypes = [F, F, F, F, ctypes.c_int, ctypes.c_float, F, F, F, F, F, F, F,
                                           ctypes.c_float]
        L.fgo_integrate_rb_f64.argtypes = [D, F, D, D, ctypes.c_int, ctypes.c_float, F, F, F, D, D, D, D,
                                           ctypes.c_float]
        L.fgo_rb_collision_gather.restype = ctypes.c_int
        L.fgo_rb_collision_gather.argtypes = [F, U, U, I, ctypes.c_int, F, U, I]
        L.fgo_max_threads.restype = ctypes.c_int
        L.fgo_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _f(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(F)


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def _u(a):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(U)


def _i(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(I)


def _nullf():
    return ctypes.cast(None, F)


def max_threads():
    return lib().fgo_max_threads()


def set_threads(n):
    lib().fgo_set_threads(int(n))


# ------------------------------------------------------------------ params

def make_common_params(cell, buckets, h, vlimit, vmin, vmax, gravity, scale, dt, relation=(1, 1, 1),
                       key_bits=0, point_radius=0.0):
    p = CommonFluidParams()
    p.cell_size = Float3(*[float(c) for c in cell])
    p.bucket_size = Int3(*[int(b) for b in buckets])
    p.keyBits = int(key_bits)
    p.kernel_radius = float(h)
    p.kernel_radius_squared = float(np.float32(h) * np.float32(h))
    p.pointRadius = float(point_radius)
    p.pointScale = 0.0
    p.velocity_limit = float(vlimit)
    p.volume_min = Float3(*[float(v) for v in vmin])
    p.volume_max = Float3(*[float(v) for v in vmax])
    p.global_external_force = Float3(*[float(g) for g in gravity])
    p.simulation_scale = float(scale)
    p.deltaTimeIntegration = float(dt)
    p.fluid_to_srb_relation = Int3(*[int(r) for r in relation])
    return p


def kernels_cache(h):
    kc = KernelsCache()
    lib().fgo_compute_kernels_cache(float(h), ctypes.byref(kc))
    return kc


def nbuckets(p):
    return int(p.bucket_size.x) * int(p.bucket_size.y) * int(p.bucket_size.z)


# ------------------------------------------------------------------ stages

def hash_key(pos3, cell3, nb):
    return lib().fgo_hash_key(_f(np.ascontiguousarray(pos3, np.float32)),
                              _f(np.ascontiguousarray(cell3, np.float32)), int(nb))


def calc_hash_key(pos4, nb, cell):
    n = pos4.shape[0]
    keys = np.zeros(n, np.uint32)
    ids = np.zeros(n, np.uint32)
    lib().fgo_calc_hash_key(_u(keys), _u(ids), _f(pos4), n, nb, *[float(c) for c in cell])
    return keys, ids


def calc_hash_key_with_offset(local4, cm4, q4, nb, cell):
    n = local4.shape[0]
    keys = np.zeros(n, np.uint32)
    ids = np.zeros(n, np.uint32)
    world = np.zeros((n, 4), np.float32)
    lib().fgo_calc_hash_key_with_offset(_u(keys), _u(ids), _f(cm4), _f(q4), _f(local4), _f(world), n,
                                        *[float(c) for c in cell], int(nb))
    return keys, ids, world


def sort_pairs(keys, vals):
    k = keys.copy()
    v = vals.copy()
    lib().fgo_sort_pairs(_u(k), _u(v), k.shape[0])
    return k, v


def find_cell_offset(keys, ids, pos4, vel4, nb, end_init=None):
    n = keys.shape[0]
    start = np.zeros(nb, np.uint32)
    end = np.zeros(nb, np.uint32) if end_init is None else end_init.copy()
    spos = np.zeros((n, 4), np.float32)
    svel = np.zeros((n, 4), np.float32) if vel4 is not None else None
    lib().fgo_find_cell_offset(_u(start), _u(end), _u(keys), _u(ids), _f(pos4), _f(spos),
                               _f(vel4) if vel4 is not None else _nullf(),
                               _f(svel) if svel is not None else _nullf(), n, nb)
    return start, end, spos, svel


def density(spos, start, end, p, kc, gas, rest, mass, f64=False, dp_init=None):
    n = spos.shape[0]
    pairs = np.zeros(1, np.int64)
    pp = pairs.ctypes.data_as(LL)
    if f64:
        dp = np.zeros((n, 2), np.float64) if dp_init is None else dp_init.astype(np.float64).copy()
        lib().fgo_density_f64(_f(spos), _d(dp), _u(start), _u(end), n, ctypes.byref(p), ctypes.byref(kc),
                              gas, rest, mass, pp)
    else:
        dp = np.zeros((n, 2), np.float32) if dp_init is None else dp_init.astype(np.float32).copy()
        lib().fgo_density_f32(_f(spos), _f(dp), _u(start), _u(end), n, ctypes.byref(p), ctypes.byref(kc),
                              gas, rest, mass, pp)
    return dp, int(pairs[0])


def forces(spos, svel, dp, start, end, ids, mass, visc, p, kc, f64=False, newvel_init=None, contact=None):
    """contact = (ContactParams, static ContactGrid or None, dynamic ContactGrid or None)."""
    n = spos.shape[0]
    cp = sg = dg = None
    if contact is not None:
        cp, sg, dg = contact
    if f64:
        nv = np.zeros((n, 4), np.float64) if newvel_init is None else newvel_init.astype(np.float64).copy()
        dpf = np.ascontiguousarray(dp, np.float32)
        lib().fgo_forces_f64_fdp(_f(spos), _f(svel), _f(dpf), _u(start), _u(end), _d(nv), _u(ids), mass, n, visc,
                                 ctypes.byref(p), ctypes.byref(kc),
                                 ctypes.byref(cp) if cp is not None else None,
                                 ctypes.byref(sg) if sg is not None else None,
                                 ctypes.byref(dg) if dg is not None else None)
    else:
        nv = np.zeros((n, 4), np.float32) if newvel_init is None else newvel_init.astype(np.float32).copy()
        if cp is None:
            lib().fgo_forces_f32(_f(spos), _f(svel), _f(dp), _u(start), _u(end), _f(nv), _u(ids), mass, n, visc,
                                 ctypes.byref(p), ctypes.byref(kc))
        else:
            lib().fgo_forces_srb_f32(_f(spos), _f(svel), _f(dp), _u(start), _u(end), _f(nv), _u(ids), mass, n,
                                     visc, ctypes.byref(p), ctypes.byref(kc), ctypes.byref(cp),
                                     ctypes.byref(sg) if sg is not None else None,
                                     ctypes.byref(dg) if dg is not None else None)
    return nv


def integrate(pos4, vel4, p):
    out = pos4.copy()
    lib().fgo_integrate_f32(_f(out), _f(vel4), out.shape[0], ctypes.byref(p))
    return out


def contact_grid(pos4, vel4, start, end, nb, use=True):
    g = ContactGrid()
    g.pos4 = _f(pos4)
    g.vel4 = _f(vel4) if vel4 is not None else _nullf()
    g.start = _u(start)
    g.end = _u(end)
    g.nbuckets = int(nb)
    g.use = 1 if use else 0
    g._keep = (pos4, vel4, start, end)
    return g


def contact_params(fluid_radius, rb_radius, k, kd, cell, rel, eps):
    c = ContactParams()
    c.fluid_radius = fluid_radius
    c.rb_radius = rb_radius
    c.kspring = k
    c.kdamping = kd
    c.cell[:] = [float(x) for x in cell]
    c.rel[:] = [int(r) for r in rel]
    c.eps = eps
    return c


def rb_forces_from_fluids(rbpos, body_vel, body_cm, radius, sph_pos, sph_vel, sph_start, sph_end, sph_radius,
                          sph_cell, sph_nb, rel, k, kd, f64=False):
    n = rbpos.shape[0]
    dt = np.float64 if f64 else np.float32
    F_ = np.zeros((n, 4), dt)
    T_ = np.zeros((n, 4), dt)
    fn = lib().fgo_rb_forces_from_fluids_f64 if f64 else lib().fgo_rb_forces_from_fluids_f32
    cv = (_d if f64 else _f)
    fn(_f(rbpos), _f(body_vel), _f(body_cm), cv(F_), cv(T_), n, radius, _f(sph_pos), _f(sph_vel), _u(sph_start),
       _u(sph_end), sph_radius, _f(np.asarray(sph_cell, np.float32)), int(sph_nb),
       _i(np.asarray(rel, np.int32)), k, kd)
    return F_, T_


def rb_forces_from_rb(rbpos, body_vel, body_cm, rb_start, rb_end, cell, radius, rb_nb, k, kd, srb=None):
    n = rbpos.shape[0]
    F_ = np.zeros((n, 4), np.float32)
    T_ = np.zeros((n, 4), np.float32)
    if srb is None:
        z4 = np.zeros((1, 4), np.float32)
        zu = np.zeros(1, np.uint32)
        srb = (z4, zu, zu, 1, 0)
    spos, sst, sen, snb, nsrb = srb
    lib().fgo_rb_forces_from_rb_f32(_f(rbpos), _f(body_vel), _f(body_cm), _f(T_), _f(F_), _u(rb_start), _u(rb_end),
                                    n, _f(np.asarray(cell, np.float32)), radius, int(rb_nb), int(snb), _f(spos),
                                    _u(sst), _u(sen), k, kd, int(nsrb))
    return F_, T_


def rb_reduce(force4, torque4, nbodies):
    bf = np.zeros((nbodies, 4), np.float64)
    bt = np.zeros((nbodies, 4), np.float64)
    lib().fgo_rb_reduce_f64(_f(np.ascontiguousarray(force4, np.float32)), _f(np.ascontiguousarray(torque4, np.float32)),
                            force4.shape[0], nbodies, _d(bf), _d(bt))
    return bf, bt


def integrate_rb(x4, mass, v4, f4, dt, ext4, vmin, vmax, L4, t4, q4, inv12, vlimit, f64=False):
    """Returns updated (x4, v4, L4, q4); inputs are not modified."""
    dtp = np.float64 if f64 else np.float32
    x = np.ascontiguousarray(x4, dtp).copy()
    v = np.ascontiguousarray(v4, dtp).copy()
    L = np.ascontiguousarray(L4, dtp).copy()
    q = np.ascontiguousarray(q4, dtp).copy()
    f = np.ascontiguousarray(f4, dtp)
    t = np.ascontiguousarray(t4, dtp)
    inv = np.ascontiguousarray(inv12, dtp)
    cv = _d if f64 else _f
    fn = lib().fgo_integrate_rb_f64 if f64 else lib().fgo_integrate_rb_f32
    fn(cv(x), _f(np.asarray(mass, np.float32)), cv(v), cv(f), x.shape[0], dt, _f(np.asarray(ext4, np.float32)),
       _f(np.asarray(vmin, np.float32)), _f(np.asarray(vmax, np.float32)), cv(L), cv(t), cv(q), cv(inv), vlimit)
    return x, v, L, q


class Stepper:
    """CPU restatement of one full step of a scene (FP32 reference arithmetic).

    Fluid: HeterogeneousSimulator::doTimeStep (HeterogeneousSimulator.cpp:54-127):
      findFluidNeighbourhood (:131-150), calculateFluidDensity (:153-159),
      calculateFluidForces (:161-205), integrateFluidForces (:207-212).
    Rigid bodies, in the order of the commented two-way block (:57-126):
      RigidBodySimulator::generateCollisionData (RigidBodySimulator.cpp:334-477:
      OpenMP broad phase + host gather, then transform+hash, sort, ranges),
      calculateRigidBodyForcesFromFluid (:503-520), forces with the dynamic
      grid (SPHCalculateForcesWithSRBK), applyForces (:522-566), integrate
      (:568-611).

    `scene` is a duck-typed description with the attributes of
    fluidgrid_gb300.scenes.SceneSpec (pos, vel, cell_size, buckets, h, ...)."""

    def __init__(self, scene):
        s = scene
        self.s = s
        self.pos = np.ascontiguousarray(s.pos, np.float32).copy()
        self.vel = (np.zeros_like(self.pos) if s.vel is None else np.ascontiguousarray(s.vel, np.float32).copy())
        self.nb = int(np.prod(s.buckets))
        self.p = make_common_params(s.cell_size, s.buckets, s.h, s.vlimit, s.box_min, s.box_max, s.gravity, s.scale,
                                    s.dt, relation=s.f2r_rel, point_radius=s.fluid_radius)
        self.kc = kernels_cache(s.h)
        self.pairs = 0
        nbod = len(s.bodies)
        self.nbod = nbod
        if nbod:
            self.local = np.concatenate([np.c_[b.local[:, :3], np.full(len(b.local), i, np.float32)]
                                         for i, b in enumerate(s.bodies)]).astype(np.float32)
            self.first = np.cumsum([0] + [len(b.local) for b in s.bodies])[:-1].astype(np.uint32)
            self.count = np.array([len(b.local) for b in s.bodies], np.uint32)
            self.cm = np.array([list(b.position) + [0.0] for b in s.bodies], np.float32)
            self.q = np.array([b.orientation for b in s.bodies], np.float32)
            self.bv = np.zeros((nbod, 4), np.float32)
            self.L = np.zeros((nbod, 4), np.float32)
            self.mass = np.array([b.mass for b in s.bodies], np.float32)
            self.inv = np.zeros((nbod, 12), np.float32)
            for i, b in enumerate(s.bodies):
                self.inv[i, [0, 1, 2, 4, 5, 6, 8, 9, 10]] = np.asarray(b.inv_inertia, np.float32)
            self.rnb = int(np.prod(s.rb_buckets))
            self.rcell = (s.rb_radius,) * 3

    def step(self):
        s = self.s
        keys, ids = calc_hash_key(self.pos, self.nb, s.cell_size)
        sk, si = sort_pairs(keys, ids)
        start, end, spos, svel = find_cell_offset(sk, si, self.pos, self.vel, self.nb)
        dp, pairs = density(spos, start, end, self.p, self.kc, s.gas, s.rest, s.mass)
        self.pairs = pairs
        contact = None
        if self.nbod:
            partner = [1] * self.nbod  # every body meets the fluid (fluid AABB test passes)
            loc, flags, last = rb_collision_gather(self.local, self.first, self.count, partner)
            rk, ri, rw = calc_hash_key_with_offset(loc, self.cm, self.q, self.rnb, self.rcell)
            rsk, rsi = sort_pairs(rk, ri)
            rst, ren, rsp, _ = find_cell_offset(rsk, rsi, rw, None, self.rnb)
            F, T = rb_forces_from_fluids(rsp, self.bv, self.cm, s.rb_radius, spos, svel, start, end,
                                         s.fluid_radius, s.cell_size, self.nb, s.r2f_rel, s.ck, s.ckd)
            cp = contact_params(s.fluid_radius, s.rb_radius, s.ck, s.ckd, self.rcell, s.f2r_rel, 0.003)
            dg = contact_grid(rsp, self.bv, rst, ren, self.rnb)
            contact = (cp, None, dg)
        self.vel = forces(spos, svel, dp, start, end, si, s.mass, s.visc, self.p, self.kc, newvel_init=self.vel,
                          contact=contact)
        if self.nbod:
            bf, bt = rb_reduce(F, T, self.nbod)
            x, v, L, q = integrate_rb(self.cm, self.mass, self.bv, bf.astype(np.float32), s.dt,
                                      np.array(s.rb_gravity, np.float32), s.box_min, s.box_max, self.L,
                                      bt.astype(np.float32), self.q, self.inv, s.rb_vlimit)
            self.cm, self.bv, self.L, self.q = x, v, L, q
        self.pos = integrate(self.pos, self.vel, self.p)


def rb_collision_gather(local4, body_first, body_count, partner):
    nb = len(body_first)
    out = np.zeros_like(local4)
    flags = np.zeros(local4.shape[0], np.uint32)
    last = np.zeros(max(nb, 1), np.int32)
    m = lib().fgo_rb_collision_gather(_f(local4), _u(np.asarray(body_first, np.uint32)),
                                      _u(np.asarray(body_count, np.uint32)), _i(np.asarray(partner, np.int32)), nb,
                                      _f(out), _u(flags), _i(last))
    return out[:m], flags[:m], last
