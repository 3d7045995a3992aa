"""Seeded synthetic scenes for the five benchmark workloads.

No dataset is involved: every scene is generated from a seed (numpy PCG64).
Positions are in metres with simulation_scale = 1, vertical axis y (the
reference's gravity axis, AppMain.cpp:86; rigid floor clamp on y,
K_RigidBodySim.cu:230), cell size = kernel radius h, lattice spacing 0.5h.
Fluid constants: h = 0.0457 m, particle mass 0.02 kg, rest density 998.29,
gas constant 3, viscosity 3.5, dt = 0.003 s, gravity (0, -9.8, 0).  The wall
and friction constants default to the reference's kernel literals
(K_FluidSim.cu:289-293); rigid contact spring/damping -10/-5 are the values
of the reference's commented two-way call (HeterogeneousSimulator.cpp:180).
"""
import ctypes
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

H = 0.0457
SPACING = 0.5 * H
MASS = 0.02
REST = 998.29
GAS = 3.0
VISC = 3.5
DT = 0.003
INV_INERTIA_DIAG = 0.00125  # hard-coded inverse inertia of RigidBody::loadFromFile (RigidBody.cpp:120-122)


@dataclass
class Body:
    local: np.ndarray          # float32 [n, 4] surface spheres in body coordinates (w unused)
    mass: float
    position: tuple
    orientation: tuple         # quaternion x, y, z, w
    inv_inertia: tuple = (INV_INERTIA_DIAG, 0, 0, 0, INV_INERTIA_DIAG, 0, 0, 0, INV_INERTIA_DIAG)


@dataclass
class SceneSpec:
    pos: np.ndarray                        # float32 [n, 4], w = 1 active
    vel: Optional[np.ndarray] = None       # float32 [n, 4] or None
    box_min: tuple = (0.0, 0.0, 0.0)
    box_max: tuple = (1.0, 1.0, 1.0)
    buckets: tuple = (64, 64, 64)
    h: float = H
    cell: Optional[tuple] = None
    mass: float = MASS
    rest: float = REST
    gas: float = GAS
    visc: float = VISC
    dt: float = DT
    scale: float = 1.0
    vlimit: float = 600.0
    gravity: tuple = (0.0, -9.8, 0.0)
    bodies: List[Body] = field(default_factory=list)
    fluid_radius: float = 0.25 * H
    rb_radius: float = 0.5 * H
    rb_buckets: tuple = (32, 32, 32)
    f2r_rel: tuple = (2, 2, 2)
    r2f_rel: tuple = (1, 1, 1)
    ck: float = -10.0
    ckd: float = -5.0
    rb_rb: bool = False
    rbrb_k: float = -10.0    # rigid/rigid contact spring and damping (the fluid/rigid values)
    rbrb_kd: float = -5.0
    rb_gravity: tuple = (0.0, -9.8, 0.0, 0.0)
    rb_vlimit: float = 600.0
    name: str = "scene"

    @property
    def n(self):
        return int(self.pos.shape[0])

    @property
    def nbuckets(self):
        return int(self.buckets[0]) * int(self.buckets[1]) * int(self.buckets[2])

    @property
    def cell_size(self):
        return self.cell if self.cell is not None else (self.h, self.h, self.h)

    @property
    def nspheres(self):
        return sum(int(b.local.shape[0]) for b in self.bodies)

    def fill_desc(self, d, keep):
        from ._ffi import fg_body_desc, load
        load().fg_scene_desc_defaults(ctypes.byref(d))
        pos = np.ascontiguousarray(self.pos, np.float32)
        keep.append(pos)
        d.n_particles = self.n
        d.positions = pos.ctypes.data if self.n else None
        if self.vel is not None:
            vel = np.ascontiguousarray(self.vel, np.float32)
            keep.append(vel)
            d.velocities = vel.ctypes.data
        d.cell_size[:] = [float(c) for c in self.cell_size]
        d.bucket_size[:] = [int(b) for b in self.buckets]
        d.kernel_radius = self.h
        d.velocity_limit = self.vlimit
        d.volume_min[:] = list(self.box_min)
        d.volume_max[:] = list(self.box_max)
        d.gravity[:] = list(self.gravity)
        d.simulation_scale = self.scale
        d.dt = self.dt
        d.mass, d.rest_density, d.gas_constant, d.viscosity = self.mass, self.rest, self.gas, self.visc
        d.fluid_radius = self.fluid_radius
        d.rb_radius = self.rb_radius
        d.rb_bucket_size[:] = [int(b) for b in self.rb_buckets]
        d.fluid_to_rb_relation[:] = list(self.f2r_rel)
        d.rb_to_fluid_relation[:] = list(self.r2f_rel)
        d.contact_kspring, d.contact_kdamping = self.ck, self.ckd
        d.rb_rb_contact = 1 if self.rb_rb else 0
        d.rbrb_kspring, d.rbrb_kdamping = self.rbrb_k, self.rbrb_kd
        d.rb_gravity[:] = list(self.rb_gravity)
        d.rb_velocity_limit = self.rb_vlimit
        d.rb_dt = self.dt
        d.rb_volume_min[:] = list(self.box_min)
        d.rb_volume_max[:] = list(self.box_max)
        if self.bodies:
            arr = (fg_body_desc * len(self.bodies))()
            for i, b in enumerate(self.bodies):
                loc = np.ascontiguousarray(b.local, np.float32)
                keep.append(loc)
                arr[i].n_spheres = loc.shape[0]
                arr[i].local_spheres = loc.ctypes.data
                arr[i].mass = b.mass
                arr[i].position[:] = [float(x) for x in b.position]
                arr[i].orientation[:] = [float(x) for x in b.orientation]
                arr[i].inv_inertia[:] = [float(x) for x in b.inv_inertia]
            keep.append(arr)
            d.n_bodies = len(self.bodies)
            d.bodies = ctypes.cast(arr, ctypes.POINTER(fg_body_desc))

    def common_params(self):
        """The reference's CommonFluidParams for this scene."""
        from ._ffi import fgr_common_fluid_params, float3, int3
        p = fgr_common_fluid_params()
        p.cell_size = float3(*[float(c) for c in self.cell_size])
        p.bucket_size = int3(*[int(b) for b in self.buckets])
        p.keyBits = 0
        p.kernel_radius = self.h
        p.kernel_radius_squared = float(np.float32(self.h) * np.float32(self.h))
        p.pointRadius = self.fluid_radius
        p.pointScale = 0.0
        p.velocity_limit = self.vlimit
        p.volume_min = float3(*self.box_min)
        p.volume_max = float3(*self.box_max)
        p.global_external_force = float3(*self.gravity)
        p.simulation_scale = self.scale
        p.deltaTimeIntegration = self.dt
        p.fluid_to_srb_relation = int3(*self.f2r_rel)
        return p


# ------------------------------------------------------------------ builders

def lattice(nx, ny, nz, spacing, origin, jitter, rng):
    """Jittered lattice, x fastest then z then y (layers in y like the
    reference's BlockEmitter, Emitter.cpp:16-43); w = 1 (active)."""
    iy, iz, ix = np.meshgrid(np.arange(ny), np.arange(nz), np.arange(nx), indexing="ij")
    p = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], 1).astype(np.float64) * spacing + np.asarray(origin)
    p += rng.uniform(-jitter, jitter, p.shape)
    out = np.ones((p.shape[0], 4), np.float32)
    out[:, :3] = p.astype(np.float32)
    return out


def random_quaternion(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    return tuple(float(x) for x in q)  # x, y, z, w


def box_surface(side, count, rng):
    """Regular grid over the six faces of a cube (shared edges once), the
    smallest grid with >= count points, trimmed to exactly `count` by a
    seeded choice."""
    m = 2
    while 6 * m * m - 12 * m + 8 < count:
        m += 1
    g = np.linspace(-side / 2, side / 2, m)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    on = (np.abs(X) >= side / 2 - 1e-9) | (np.abs(Y) >= side / 2 - 1e-9) | (np.abs(Z) >= side / 2 - 1e-9)
    pts = np.stack([X[on], Y[on], Z[on]], 1)
    sel = np.sort(rng.choice(len(pts), count, replace=False))
    out = np.zeros((count, 4), np.float32)
    out[:, :3] = pts[sel]
    return out


def sphere_surface(radius, count):
    """Fibonacci-sphere placement of `count` points."""
    i = np.arange(count) + 0.5
    phi = np.arccos(1 - 2 * i / count)
    th = math.pi * (1 + 5 ** 0.5) * i
    out = np.zeros((count, 4), np.float32)
    out[:, 0] = radius * np.cos(th) * np.sin(phi)
    out[:, 1] = radius * np.cos(phi)
    out[:, 2] = radius * np.sin(th) * np.sin(phi)
    return out


def next_pow2(v):
    p = 1
    while p < v:
        p <<= 1
    return p


# ------------------------------------------------------------------ workloads

def dam_break_small(seed=0x5EED):
    """16,384 particles: 32x16x32 (x, y, z) lattice at 0.5h, jitter +-0.05h,
    in the corner of a 1 m walled box; 262,144 buckets (64^3); no body."""
    rng = np.random.default_rng(seed)
    pos = lattice(32, 16, 32, SPACING, (SPACING, SPACING, SPACING), 0.05 * H, rng)
    return SceneSpec(pos=pos, box_min=(0, 0, 0), box_max=(1, 1, 1), buckets=(64, 64, 64),
                     name="dam_break_16k")


def dam_break_rigid(seed=0x5EED, nx=128, ny=64, nz=128, spheres=4096, box=(4.0, 2.0, 4.0), buckets=(128, 128, 128)):
    """1,048,576 particles (128x64x128 lattice) in a 4x2x4 m box, 2^21
    buckets, one 0.4 m box body of 50 kg with 4,096 surface spheres of radius
    0.5h, centre at height 1.5 m over the block, seeded orientation."""
    rng = np.random.default_rng(seed)
    pos = lattice(nx, ny, nz, SPACING, (SPACING, SPACING, SPACING), 0.05 * H, rng)
    ext = np.array([nx, ny, nz]) * SPACING
    centre = (float(ext[0] / 2 + SPACING), 1.5, float(ext[2] / 2 + SPACING))
    body = Body(local=box_surface(0.4, spheres, rng), mass=50.0, position=centre, orientation=random_quaternion(rng))
    return SceneSpec(pos=pos, box_min=(0, 0, 0), box_max=box, buckets=buckets, bodies=[body],
                     rb_buckets=(32, 32, 32), name="dam_break_rigid_1m")


def precision_jet(seed=0x5EED, nx=256, ny=64, nz=256, nbodies=8):
    """4,194,304 particles, a random 10% with N(0, 1 m/s) velocities, eight
    bodies (boxes and spheres, radius 0.15-0.4 m, 1,024-8,192 spheres)."""
    rng = np.random.default_rng(seed)
    pos = lattice(nx, ny, nz, SPACING, (SPACING, SPACING, SPACING), 0.05 * H, rng)
    n = pos.shape[0]
    vel = np.zeros((n, 4), np.float32)
    jet = rng.choice(n, n // 10, replace=False)
    vel[jet, :3] = rng.normal(0, 1.0, (len(jet), 3)).astype(np.float32)
    ext = np.array([nx, ny, nz]) * SPACING
    box = (float(ext[0] + 0.5), 2.5, float(ext[2] + 0.5))
    bodies = []
    for b in range(nbodies):
        r = float(rng.uniform(0.15, 0.4))
        cnt = int(rng.integers(1024, 8193))
        c = (float(rng.uniform(0.5, ext[0] - 0.5)), float(rng.uniform(1.2, 2.0)), float(rng.uniform(0.5, ext[2] - 0.5)))
        loc = box_surface(2 * r, cnt, rng) if b % 2 == 0 else sphere_surface(r, cnt)
        bodies.append(Body(local=loc, mass=float(50.0 * (r / 0.2) ** 3), position=c, orientation=random_quaternion(rng)))
    return SceneSpec(pos=pos, vel=vel, box_min=(0, 0, 0), box_max=box, buckets=(256, 128, 128), bodies=bodies,
                     rb_buckets=(64, 64, 64), rb_rb=True, name="precision_jet_4m")


def batched_scenes(seed=0x5EED, count=256, nmin=2048, nmax=65536):
    """`count` scenes, fluid counts log-uniform in [nmin, nmax], each a
    jittered block at 0.5h in its own box of twice the block volume; odd
    scenes carry one rigid sphere of radius 0.1 m with 512 surface spheres."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        nx = max(4, int(round((n / 2) ** (1 / 3) * 2 ** (1 / 3))))
        nz = nx
        ny = max(2, int(math.ceil(n / (nx * nz))))
        pos = lattice(nx, ny, nz, SPACING, (SPACING, SPACING, SPACING), 0.05 * H, rng)[:n]
        ext = np.array([nx, ny, nz], np.float64) * SPACING + 2 * SPACING
        box = (float(ext[0] * 2 ** (1 / 3)), float(ext[1] * 2 ** (1 / 3)), float(ext[2] * 2 ** (1 / 3)))
        nb = next_pow2(max(n, 4096))
        bk = (nb, 1, 1)
        bodies = []
        if s % 2 == 1:
            c = (box[0] / 2, float(ext[1] + 0.15), box[2] / 2)
            bodies.append(Body(local=sphere_surface(0.1, 512), mass=5.0, position=c,
                               orientation=random_quaternion(rng)))
        out.append(SceneSpec(pos=pos, box_min=(0, 0, 0), box_max=box, buckets=bk, bodies=bodies,
                             rb_buckets=(4096, 1, 1), name="batched_%d" % s))
    return out


def dam_break_request(n, nboxes, rng, name="request"):
    """A served-form request: a dam-break block of n particles (jittered
    lattice at 0.5h) in a walled box of twice the block's footprint, with
    `nboxes` rigid boxes of side 0.2 m (1,024 surface spheres, 10 kg each)
    dropped from above the block at seeded poses."""
    nx = max(4, int(round((n / 2.0) ** (1.0 / 3.0) * 1.26)))
    nz = nx
    ny = max(2, int(math.ceil(n / (nx * nz))))
    pos = lattice(nx, ny, nz, SPACING, (SPACING, SPACING, SPACING), 0.05 * H, rng)[:n]
    ext = np.array([nx, ny, nz], np.float64) * SPACING + 2 * SPACING
    box = (float(ext[0] * 1.4142), float(max(ext[1] * 2.0, 0.8)), float(ext[2] * 1.4142))
    bodies = []
    for b in range(nboxes):
        c = (float(rng.uniform(0.15, box[0] - 0.15)), float(ext[1] + 0.2 + 0.25 * b),
             float(rng.uniform(0.15, box[2] - 0.15)))
        bodies.append(Body(local=box_surface(0.2, 1024, rng), mass=10.0, position=c,
                           orientation=random_quaternion(rng)))
    nb = next_pow2(max(n, 4096))
    return SceneSpec(pos=pos, box_min=(0, 0, 0), box_max=box, buckets=(nb, 1, 1), bodies=bodies,
                     rb_buckets=(8192, 1, 1), name=name)


def served_templates(seed=0x5EED, count=24, nmin=4096, nmax=524288):
    """Scene pool of the served workload: fluid counts log-uniform in
    [nmin, nmax], 0-4 rigid boxes each.  Requests draw from this pool (with
    their own step counts) so that generating scenes on the host does not
    pace the arrival process."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        out.append(dam_break_request(n, int(rng.integers(0, 5)), rng, name="served_%d" % s))
    return out


WORKLOADS = {
    "dam_break_16k": dam_break_small,
    "dam_break_rigid_1m": dam_break_rigid,
    "precision_jet_4m": precision_jet,
}
