"""GPU parity of the fluid step against the oracle, stage by stage from an
identical input state (the reference's own method: hash keys, sort order and
cell ranges bit-exact; density and forces within stated tolerances;
integration bit-exact given the same velocity).

Tolerances (FP32 GPU vs oracle):
  density  : |rho_gpu - rho_ref64| <= 1e-5 * rho_ref64 (FP64 oracle), and
             <= 2e-5 relative to the FP32 restatement
  forces   : |F_gpu - F_ref| <= 2e-4 * max(|F_ref|, F_med) per particle,
             F = (v_new - v_old) / dt, F_med the median |F_ref| of the scene
"""
import numpy as np
import pytest

from fluidgrid_gb300 import World, scenes, build
from fluidgrid_gb300.scenes import H, SceneSpec, lattice, SPACING
from oracle import oracle as O
import helpers as T

pytestmark = pytest.mark.gpu

RTOL_RHO64 = 1e-5
RTOL_RHO32 = 2e-5
RTOL_F = 2e-4


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _variants():
    out = {"dam_break_16k": scenes.dam_break_small()}
    s = scenes.dam_break_small(seed=11)
    s.buckets = (61, 67, 64)  # non power of two: unsigned modulo path
    out["odd_buckets"] = s
    rng = np.random.default_rng(3)
    pos = lattice(24, 12, 24, SPACING, (1000.0, 2.0, -800.0), 0.05 * H, rng)
    out["far_origin"] = SceneSpec(pos=pos, box_min=(999.9, 1.9, -800.1), box_max=(1001.0, 3.0, -799.0),
                                  buckets=(64, 64, 64), name="far_origin")  # int32 products wrap
    rng = np.random.default_rng(5)
    for n in (1, 7, 129, 4097):
        p = np.ones((n, 4), np.float32)
        p[:, :3] = rng.uniform(0.1, 0.3, (n, 3))
        out["ragged_%d" % n] = SceneSpec(pos=p, buckets=(16, 16, 16), name="ragged_%d" % n)
    return out


VARIANTS = _variants()


def _step(spec, fused=True, vel0=None, digit_bits=None, graphs=True, kernel=None):
    w = World([spec])
    if kernel is not None:
        w.set_option("autotune_period", 0)
        w.set_option("kernel", kernel)
    w.set_fused_integrate(fused)
    w.set_graphs(graphs)
    if digit_bits:
        w.set_digit_bits(digit_bits)
    pos0 = spec.pos.copy()
    v0 = np.zeros_like(pos0) if vel0 is None else vel0.astype(np.float32)
    w.upload(pos0, v0)
    w.step(1)
    w.sync()
    out = {k: w.read(k) for k in ("KEYS_UNSORTED", "KEYS", "IDS", "START", "END", "SPOS", "SVEL", "DP", "POS", "VEL")}
    w.close()
    return pos0, v0, out


@pytest.mark.parametrize("name", sorted(VARIANTS))
def test_grid_build_bit_exact(name):
    spec = VARIANTS[name]
    pos0, v0, g = _step(spec)
    ref = T.oracle_grid(spec, pos0, v0)
    assert np.array_equal(g["KEYS_UNSORTED"], ref["keys"]), "hash keys differ"
    assert np.array_equal(g["KEYS"], ref["skeys"]), "sorted keys differ"
    assert np.array_equal(g["IDS"], ref["ids"]), "sort order differs"
    T.compare_ranges(g["START"], g["END"], ref["start"], ref["end"])
    assert np.array_equal(g["SPOS"].view(np.uint32), ref["spos"].view(np.uint32))
    assert np.array_equal(g["SVEL"].view(np.uint32), ref["svel"].view(np.uint32))


@pytest.mark.parametrize("bits", [1, 3, 5, 6, 7, 8])
def test_sort_digit_widths_identical(bits):
    spec = VARIANTS["dam_break_16k"]
    pos0, v0, g = _step(spec, digit_bits=bits)
    ref = T.oracle_grid(spec, pos0, v0)
    assert np.array_equal(g["IDS"], ref["ids"])
    assert np.array_equal(g["KEYS"], ref["skeys"])


@pytest.mark.parametrize("name", ["dam_break_16k", "odd_buckets", "far_origin", "ragged_129", "ragged_4097"])
def test_density_matches_oracle(name):
    spec = VARIANTS[name]
    pos0, v0, g = _step(spec)
    ref = T.oracle_grid(spec, pos0, v0)
    kc = O.kernels_cache(spec.h)
    d32, pairs = O.density(ref["spos"], ref["start"], ref["end"], ref["p"], kc, spec.gas, spec.rest, spec.mass)
    d64, _ = O.density(ref["spos"], ref["start"], ref["end"], ref["p"], kc, spec.gas, spec.rest, spec.mass,
                       f64=True)
    rho = g["DP"][:, 0].astype(np.float64)
    e64 = np.abs(rho - d64[:, 0]) / d64[:, 0]
    e32 = np.abs(rho - d32[:, 0]) / d32[:, 0]
    assert pairs > 0
    assert e64.max() <= RTOL_RHO64, e64.max()
    assert e32.max() <= RTOL_RHO32, e32.max()
    # pressure k*(rho - rho0) follows; absolute check scaled by k*rho
    pe = np.abs(g["DP"][:, 1] - d64[:, 1]) / (spec.gas * d64[:, 0])
    assert pe.max() <= 2 * RTOL_RHO64


def _forces_check(spec, pos0, v0, g, contact=None):
    ref = T.oracle_grid(spec, pos0, v0)
    kc = O.kernels_cache(spec.h)
    dp = g["DP"]  # identical input state: the GPU's own density field
    nv = O.forces(ref["spos"], ref["svel"], dp, ref["start"], ref["end"], ref["ids"], spec.mass, spec.visc,
                  ref["p"], kc, newvel_init=v0, contact=contact)
    nv64 = O.forces(ref["spos"], ref["svel"], dp, ref["start"], ref["end"], ref["ids"], spec.mass, spec.visc,
                    ref["p"], kc, f64=True, newvel_init=v0, contact=contact)
    Fg = T.force_from_vel(g["VEL"], v0, spec.dt)
    Fr = T.force_from_vel(nv, v0, spec.dt)
    F64 = T.force_from_vel(nv64, v0, spec.dt)
    mag = np.linalg.norm(Fr, axis=1)
    scale = np.maximum(mag, np.median(mag))
    err = np.linalg.norm(Fg - Fr, axis=1) / scale
    err64 = np.linalg.norm(Fg - F64, axis=1) / scale
    assert err.max() <= RTOL_F, (err.max(), int(err.argmax()))
    assert err64.max() <= RTOL_F, err64.max()
    assert np.array_equal(g["VEL"][:, 3], v0[:, 3])  # w untouched (vel.w + 0)
    return err.max(), err64.max()


@pytest.mark.parametrize("name", ["dam_break_16k", "odd_buckets", "far_origin", "ragged_129", "ragged_4097"])
def test_forces_match_oracle(name):
    spec = VARIANTS[name]
    rng = np.random.default_rng(9)
    v0 = np.zeros((spec.n, 4), np.float32)
    v0[:, :3] = rng.normal(0, 0.5, (spec.n, 3))
    pos0, v0, g = _step(spec, vel0=v0)
    _forces_check(spec, pos0, v0, g)


def test_integrate_bit_exact_given_velocity():
    spec = VARIANTS["dam_break_16k"]
    for fused in (True, False):
        pos0, v0, g = _step(spec, fused=fused)
        p = T.oracle_params(spec)
        ref = O.integrate(pos0, g["VEL"], p)
        assert np.array_equal(g["POS"].view(np.uint32), ref.view(np.uint32)), fused


def test_kernel_launch_count():
    """The world counts the kernels it enqueues or replays: each step's
    launches, the target-order refreshes and the timed steps' L2 flushes."""
    spec = VARIANTS["dam_break_16k"]
    w = World([spec])
    w.set_option("autotune_period", 0)
    w.set_option("target_order", 0)
    lps = w.launches_per_step()
    k0 = w.kernel_launches()
    w.step(7)
    assert w.kernel_launches() - k0 == 7 * lps
    k0 = w.kernel_launches()
    w.timed_steps(3, 1 << 20)
    assert w.kernel_launches() - k0 == 3 * (lps + 1)
    w.close()
    w = World([spec])
    w.set_option("autotune_period", 0)
    w.set_option("target_order", 2)
    w.set_option("order_period", 16)
    k0 = w.kernel_launches()
    w.step(16)  # one refresh, at the first step
    d16 = w.kernel_launches() - k0
    w.step(16)  # one more
    assert d16 > 16 * w.launches_per_step()
    assert w.kernel_launches() - k0 == 2 * d16
    w.close()


def test_fused_equals_separate_and_graph_equals_direct():
    spec = VARIANTS["dam_break_16k"]
    a = _step(spec, fused=True)[2]
    b = _step(spec, fused=False)[2]
    c = _step(spec, fused=True, graphs=False)[2]
    for k in ("POS", "VEL", "DP", "IDS"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k


@pytest.mark.parametrize("name", ["dam_break_16k", "far_origin"])
def test_tunables_do_not_change_results(name):
    """The per-particle kernels (walk or neighbour lists, bucket or Morton
    target order in both passes or in the force pass only) only change how
    the work is scheduled: every setting evolves the state bit-identically."""
    spec = VARIANTS[name]
    outs = {}
    for kernel in (0, 1):
        for order in (0, 1, 2):
            for period in ((1, 16) if order else (16,)):
                w = World([spec])
                w.set_option("autotune_period", 0)
                w.set_option("kernel", kernel)
                w.set_option("target_order", order)
                w.set_option("order_period", period)
                w.step(4)
                p, v = w.download()
                outs[(kernel, order, period)] = (p, v, w.read("DP"))
                w.close()
    base = outs[(1, 1, 16)]
    for k, o in outs.items():
        for a, b in zip(o, base):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), k


@pytest.mark.parametrize("name", ["dam_break_16k", "odd_buckets"])
def test_launch_shape_does_not_change_results(name):
    """CTAs per SM and threads per CTA of the density/force grids and the
    radix digit width change no bit of the evolved state."""
    spec = VARIANTS[name]
    outs = {}
    for ctas, bits, block in ((0, 7, 128), (8, 8, 64), (64, 6, 256), (1, 5, 64), (3, 8, 256), (17, 3, 128),
                              (16, 7, 64), (32, 7, 256)):
        w = World([spec])
        w.set_option("autotune_period", 0)
        w.set_option("ctas_per_sm", ctas)
        w.set_option("digit_bits", bits)
        w.set_option("block_size", block)
        assert w.get_option("block_size") == block
        w.step(4)
        p, v = w.download()
        outs[(ctas, bits, block)] = (p, v, w.read("DP"))
        w.close()
    base = outs[(0, 7, 128)]
    for k, o in outs.items():
        for a, b in zip(o, base):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), k


def test_autotuner_keeps_results_and_reports():
    """The autotuner varies the CTAs per SM and the digit width along the
    trajectory; the results do not depend on them, so a tuned run equals an
    untuned one bit for bit."""
    spec = VARIANTS["dam_break_16k"]
    res = []
    for period in (0, 2):
        w = World([spec])
        w.set_option("autotune_period", period)
        w.step(12)
        p, v = w.download()
        st = w.tuning_stats()
        w_ctas = w.get_option("ctas_per_sm")
        res.append((p, v))
        w.close()
    assert st["steps_per_kernel"][1] == 12
    assert w_ctas in (16, 32, 64) and 6 <= st["digit_bits"] <= 8 and st["one_pass_sort"] in (0, 1, 2)
    assert st["block_size"] in (64, 128, 256)
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_list_overflow_falls_back_to_bucket_walk():
    """A neighbour-list capacity below the in-range count sends those
    particles through the bucket walk in the force pass; results stay within
    the oracle tolerances and the overflow counter sees them."""
    spec = VARIANTS["dam_break_16k"]
    rng = np.random.default_rng(13)
    v0 = np.zeros((spec.n, 4), np.float32)
    v0[:, :3] = rng.normal(0, 0.5, (spec.n, 3))
    w = World([spec])
    w.set_option("kernel", 1)
    w.set_option("list_cap", 12)
    assert w.get_option("list_cap") == 12
    w.list_overflows(reset=True)
    w.upload(spec.pos.copy(), v0)
    w.step(1)
    g = {k: w.read(k) for k in ("DP", "VEL", "POS")}
    assert w.list_overflows() > spec.n // 2
    w.close()
    _forces_check(spec, spec.pos, v0, g)


@pytest.mark.parametrize("cap", [1, 12, 40])
def test_list_capacity_never_changes_kernel1_results(cap):
    """Kernel 1's lists hold the bucket walk's order, so a particle that
    overflows its list (and walks the buckets in the force pass) gets the
    same bits as one that does not."""
    spec = VARIANTS["dam_break_16k"]
    outs = []
    for c in (None, cap):
        w = World([spec])
        w.set_option("kernel", 1)
        if c:
            w.set_option("list_cap", c)
        w.step(3)
        outs.append(w.download())
        w.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_list_capacity_grows():
    spec = VARIANTS["dam_break_16k"]
    w = World([spec])
    w.step(1)
    w.set_option("list_cap", 301)  # reallocates the lists, drops captured graphs
    assert w.get_option("list_cap") == 304  # rounded up to a multiple of 4
    w.step(2)
    w.check_finite()
    assert w.list_overflows() == 0
    w.close()


def test_list_capacity_autogrows():
    """With autogrow on, the capacity check every 25 steps raises a too-small
    capacity above the largest in-range count, after which no particle takes
    the bucket-walk fallback."""
    spec = VARIANTS["dam_break_16k"]
    w = World([spec])
    w.set_option("list_cap", 8)
    assert w.get_option("list_autogrow") == 0
    w.set_option("list_autogrow", 1)
    w.step(26)
    assert w.get_option("list_cap") > 8
    w.list_overflows(reset=True)
    w.step(3)
    assert w.list_overflows() == 0
    w.check_finite()
    w.close()


def test_multi_step_graphs_equal_single_steps():
    """Ten steps per captured graph evolve the state bit-identically to one
    step per launch, across autotuning rounds and list capacity checks."""
    spec = VARIANTS["dam_break_16k"]
    outs = []
    for g in (1, 10):
        w = World([spec])
        w.set_option("graph_steps", g)
        w.step(63)
        outs.append(w.download())
        w.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_fp64_diagnostics_match_host_sums():
    """GPU FP64 conservation sums against FP64 sums of the downloaded state,
    and reproducible bit for bit."""
    ss = scenes.batched_scenes(count=3, nmin=3000, nmax=9000)
    w = World(ss)
    w.step(5)
    d = w.diagnostics()
    assert w.diagnostics() == d
    pos, vel = w.download()
    for s, spec in enumerate(ss):
        lo = w.layout(s)
        p = pos[lo["pbase"]:lo["pbase"] + lo["n"]].astype(np.float64)
        v = vel[lo["pbase"]:lo["pbase"] + lo["n"]].astype(np.float64)
        act = p[:, 3] > 0
        m = np.float64(np.float32(spec.mass))
        assert d[s]["active"] == act.sum()
        assert d[s]["mass"] == pytest.approx(m * act.sum(), rel=1e-12)
        for c, k in enumerate(("px", "py", "pz")):
            assert d[s][k] == pytest.approx((m * v[act, c]).sum(), rel=1e-9, abs=1e-12)
        assert d[s]["kinetic"] == pytest.approx((0.5 * m * (v[act, :3] ** 2).sum(1)).sum(), rel=1e-9)
        if spec.bodies:
            bv = w.read("BODY_V")[lo["body_base"]:lo["body_base"] + lo["nbodies"]]
            bm = w.read("BODY_MASS")[lo["body_base"]:lo["body_base"] + lo["nbodies"]]
            assert d[s]["body_py"] == pytest.approx((bm * bv[:, 1]).sum(), rel=1e-12)
    w.close()


@pytest.mark.parametrize("kernel", [0, 1, 2])
def test_each_kernel_matches_oracle(kernel):
    """Every density/force kernel variant against the oracle from an
    identical state (tolerances of this file)."""
    spec = VARIANTS["dam_break_16k"]
    rng = np.random.default_rng(12)
    v0 = np.zeros((spec.n, 4), np.float32)
    v0[:, :3] = rng.normal(0, 0.5, (spec.n, 3))
    w = World([spec])
    w.set_option("kernel", kernel)
    assert w.get_option("kernel") == kernel
    w.upload(spec.pos.copy(), v0)
    w.step(1)
    g = {k: w.read(k) for k in ("DP", "VEL", "POS")}
    w.close()
    ref = T.oracle_grid(spec, spec.pos, v0)
    kc = O.kernels_cache(spec.h)
    d64, _ = O.density(ref["spos"], ref["start"], ref["end"], ref["p"], kc, spec.gas, spec.rest, spec.mass,
                       f64=True)
    assert (np.abs(g["DP"][:, 0] - d64[:, 0]) / d64[:, 0]).max() <= RTOL_RHO64
    _forces_check(spec, spec.pos, v0, g)


def test_runs_per_cta_do_not_change_kernel2_results():
    """Kernel 2 with 1, 2 or 4 bucket runs (warps) per CTA: the same bits."""
    spec = VARIANTS["dam_break_16k"]
    outs = {}
    for runs in (1, 2, 4):
        w = World([spec])
        w.set_option("autotune_period", 0)
        w.set_option("kernel", 2)
        w.set_option("runs_per_cta", runs)
        w.step(3)
        outs[runs] = w.download()
        w.close()
    for r in (1, 2):
        for a, b in zip(outs[r], outs[4]):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), r


def test_autotuner_rounds_over_runs_per_cta_keep_kernel2_results():
    """Autotuning rounds over kernel 2's runs per CTA (one real step per
    candidate) evolve the state as an untuned run does."""
    spec = VARIANTS["dam_break_16k"]
    res = []
    for period in (0, 1):
        w = World([spec])
        w.set_option("kernel", 2)
        w.set_option("autotune_period", period)
        w.set_option("autotune_tiles", 16)  # runs per CTA only
        w.step(9)
        w.check_finite()
        assert w.get_option("runs_per_cta") in (1, 2, 4)
        res.append(w.download())
        w.close()
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("kernel", [1, 2])
def test_dense_runs(kernel):
    """Runs longer than a warp (dense buckets) and candidate sets larger than
    the shared-memory stage: a compressed block with 4x the lattice density."""
    rng = np.random.default_rng(8)
    pos = lattice(24, 12, 24, SPACING * 0.5, (0.2, 0.2, 0.2), 0.02 * H, rng)
    spec = SceneSpec(pos=pos, buckets=(32, 32, 32), name="dense")
    pos0, v0, g = _step(spec, kernel=kernel)
    ref = T.oracle_grid(spec, pos0, v0)
    occ = ref["start"] != 0xFFFFFFFF
    assert (ref["end"][occ].astype(np.int64) - ref["start"][occ]).max() > 32
    kc = O.kernels_cache(spec.h)
    d64, _ = O.density(ref["spos"], ref["start"], ref["end"], ref["p"], kc, spec.gas, spec.rest, spec.mass,
                       f64=True)
    assert (np.abs(g["DP"][:, 0] - d64[:, 0]) / d64[:, 0]).max() <= RTOL_RHO64
    _forces_check(spec, pos0, v0, g)


def test_inactive_particles_are_skipped():
    spec = scenes.dam_break_small(seed=21)
    spec.pos[::5, 3] = -1.0  # BlockEmitter marks unused slots with w = -1 (Emitter.cpp:35-38)
    pos0, v0, g = _step(spec)
    ref = T.oracle_grid(spec, pos0, v0)
    assert np.array_equal(g["IDS"], ref["ids"])
    inactive = ref["spos"][:, 3] <= 0
    assert np.array_equal(g["POS"][::5], pos0[::5])  # not integrated
    assert np.all(g["DP"][inactive] == 0)  # density not written (buffer starts zeroed)
    kc = O.kernels_cache(spec.h)
    d64, _ = O.density(ref["spos"], ref["start"], ref["end"], ref["p"], kc, spec.gas, spec.rest, spec.mass,
                       f64=True)
    act = ~inactive
    e = np.abs(g["DP"][act, 0] - d64[act, 0]) / d64[act, 0]
    assert e.max() <= RTOL_RHO64


def test_multi_step_stays_finite_and_in_box():
    spec = scenes.dam_break_small()
    w = World([spec])
    w.step(50)
    w.check_finite()
    pos, vel = w.download()
    assert np.isfinite(pos).all() and np.isfinite(vel).all()
    assert pos[:, 1].min() > -0.05 and pos[:, :3].max() < 1.05
    w.close()


def test_batched_alone_equals_mixed():
    """Each scene of a packed multi-scene world evolves bit-identically to the
    same scene stepped alone."""
    ss = scenes.batched_scenes(count=6, nmin=2048, nmax=8192)
    for s in ss:
        s.bodies = []
    mixed = World(ss)
    mixed.step(3)
    pm, vm = mixed.download()
    for i, s in enumerate(ss):
        lay = mixed.layout(i)
        alone = World([s])
        alone.step(3)
        pa, va = alone.download()
        sl = slice(lay["pbase"], lay["pbase"] + lay["n"])
        assert np.array_equal(pm[sl], pa), i
        assert np.array_equal(vm[sl], va), i
        alone.close()
    mixed.close()


def test_empty_scene_in_world():
    a = scenes.dam_break_small()
    e = SceneSpec(pos=np.zeros((0, 4), np.float32), buckets=(8, 8, 8), name="empty")
    w = World([e, a, e])
    w.step(2)
    w.check_finite()
    w.close()


@pytest.mark.parametrize("name", ["dam_break_16k", "odd_buckets", "ragged_4097", "ragged_1", "ragged_7",
                                  "far_origin", "one_bucket"])
def test_sort_variants_equal(name):
    """The three sort variants produce the same sorted keys, order and cell
    ranges, so the evolved state is bit-identical: the upsweep / scan /
    downsweep radix passes (0), one kernel per pass with decoupled look-back
    (1) and the counting sort by bucket (2), which writes start/end itself.
    `one_bucket` puts 4,097 particles in a single bucket (one run)."""
    if name == "one_bucket":
        p = np.ones((4097, 4), np.float32)
        p[:, :3] = np.random.default_rng(9).uniform(0.1, 0.3, (4097, 3))
        spec = SceneSpec(pos=p, buckets=(1, 1, 1), name="one_bucket")
    else:
        spec = VARIANTS[name]
    outs = []
    for variant in (0, 1, 2):
        w = World([spec])
        w.set_option("autotune_period", 0)
        w.set_option("one_pass_sort", variant)
        assert w.get_option("one_pass_sort") == variant
        w.step(3)
        st, en = w.read("START"), w.read("END")
        occ = st != 0xFFFFFFFF
        outs.append([w.read(k) for k in ("KEYS", "IDS", "SPOS")] + [st, en[occ]] + list(w.download()))
        w.close()
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_counting_sort_is_the_default_for_dense_bucket_tables():
    """A world with at most 64 buckets per particle counts its keys; one
    with more sorts them by digits."""
    w = World([VARIANTS["dam_break_16k"]])  # 2^18 buckets, 16,384 particles
    assert w.get_option("one_pass_sort") == 2
    w.close()
    w = World([VARIANTS["ragged_7"]])  # 4,096 buckets, 7 particles
    assert w.get_option("one_pass_sort") in (0, 1)
    w.close()


@pytest.mark.parametrize("variant", [1, 2])
def test_sort_large_against_numpy(variant):
    """3M particles in 2^21 buckets.  One pass per kernel: 1,465 tiles, more
    than the GPU holds at once, so tiles look back across tiles that ran
    earlier and left.  Counting: 1,024 bucket tiles, 3M atomics.  Keys and
    order equal a stable numpy sort of the hash keys; the counting sort's
    cell ranges equal numpy's."""
    rng = np.random.default_rng(21)
    n = 3 * 1024 * 1024
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.05, 3.95, (n, 3)).astype(np.float32)
    spec = SceneSpec(pos=pos, box_min=(0, 0, 0), box_max=(4, 4, 4), buckets=(128, 128, 128), name="cloud_3m")
    w = World([spec])
    w.set_option("autotune_period", 0)
    w.set_option("one_pass_sort", variant)
    w.set_stages(1 | 2)  # hash and sort only
    w.step(1)
    ku, ks, ids = w.read("KEYS_UNSORTED"), w.read("KEYS"), w.read("IDS")
    st, en = w.read("START"), w.read("END")
    w.sync()
    w.close()
    order = np.argsort(ku, kind="stable")
    assert np.array_equal(ids, order.astype(np.uint32))
    assert np.array_equal(ks, ku[order])
    if variant == 2:
        nb = 128 ** 3
        cnt = np.bincount(ku, minlength=nb)
        first = np.concatenate([[0], np.cumsum(cnt)[:-1]])
        occ = cnt > 0
        assert np.array_equal(st[occ], first[occ].astype(np.uint32))
        assert (st[~occ] == 0xFFFFFFFF).all()
        assert np.array_equal(en[occ], (first + cnt)[occ].astype(np.uint32))


def test_sort_lookback_wait_is_bounded():
    """The one-pass sort's look-back waits are bounded: a tile whose
    predecessor never publishes gives up after the given number of rounds,
    sets the timeout bit (2) that fg_world_sync reports as FG_E_TIMEOUT, and
    the GPU context stays usable."""
    import ctypes
    from fluidgrid_gb300 import _ffi
    L = _ffi.load()
    flags = ctypes.c_uint32(0)
    _ffi.check(L.fg_selftest_bounded_wait(1 << 16, ctypes.byref(flags)), "fg_selftest_bounded_wait")
    assert flags.value == 2
    w = World([VARIANTS["ragged_129"]])
    w.step(2)
    w.check_finite()
    w.close()
