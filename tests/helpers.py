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
