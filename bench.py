"""Benchmark of the GB300 SPH step (particle-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload dam_break_rigid_1m|dam_break_16k|precision_jet_4m]
                    [--no-cpu-baseline]

A step is one full two-way step of the scene (hash, stable radix sort, cell
ranges + sorted gather, density, rigid-sphere grid and fluid->sphere
contact, pressure+viscosity+walls+contact forces with fused integration,
FP64 per-body reduction and body integration) -- the reference's
HeterogeneousSimulator::doTimeStep with its rigid-body coupling.  Default
workload: 1,048,576 fluid particles + one rigid box of 4,096 surface spheres
(seeded synthetic scene, no dataset).

`value` times K steps with inputs resident in HBM, each step bracketed by
CUDA events on the engine's stream and preceded by a 256 MiB write that
evicts L2 (126 MB).  `e2e` times the same steps through the C ABI with the
particle state copied from pinned host memory to the device and back inside
every step.  Under torchrun (N > 1) every rank runs an independent replica
(the scene does not shard: replicas only), timing is the max over ranks and
`value` sums all ranks' particle-steps.

--impl reference times the CPU restatement of the reference's path (the
oracle: the reference's kernel math as OpenMP host loops plus
RigidBodySimulator's CPU step) on the host cores, rank 0 only.
"""
import argparse
import glob
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLUSH_BYTES = 256 << 20
BYTES_FORCES = 76   # per particle: sorted pos 16 + sorted vel 16 + density/pressure 8 + id 4 + vel 16 + pos 16
BYTES_DENSITY = 24  # sorted pos 16 + density/pressure 8
FLOPS_FORCE_PAIR = 38   # pressure ~17 + viscosity ~15 + accumulate 6, per in-range pair
FLOPS_DENSITY_PAIR = 11
REF_BUDGET_S = 150.0  # CPU time bound of the reference arm's timed sample


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max/sum over ranks (gloo on host tensors; no data-path
    collective exists in this workload)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def reduce(self, v, op):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_value(key, kernel):
    """A figure of `kernel` from the committed ncu summaries (lines
    `<key> <kernel> <value>` in profiles/*.txt), or None."""
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.txt"))):
        with open(path) as f:
            for ln in f:
                t = ln.split()
                if len(t) == 3 and t[0] == key and t[1] == kernel:
                    return float(t[2])
    return None


def profile_traffic(kernel, phase):
    """DRAM bytes per particle of `kernel` in the trajectory phase `phase`
    ("sparse": the opening steps, "dense": the compressed middle) from the
    committed ncu summary, or None."""
    return profile_value("traffic_bytes_per_particle_" + phase, kernel)


def window_phase(first_step, last_step):
    """The trajectory phase a timed window of the 1M dam break lies in: the
    block stays near its lattice density for the first ~60 steps and then
    compresses (in-range neighbours ~29 -> ~110 by step ~150)."""
    mid = 0.5 * (first_step + last_step)
    return "sparse" if mid <= 60 else "dense"


def cpu_model():
    """The host CPU's model name (lscpu or /proc/cpuinfo), or None."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Model"):
                v = ln.split(":", 1)[1].strip()
                if v and not v.isdigit():
                    return v
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu part", "hardware")):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def make_scene(name):
    from fluidgrid_gb300 import scenes
    return scenes.WORKLOADS[name]()


def cpu_baseline(spec, budget_s=15.0, max_steps=60):
    """The oracle's FP32 restatement of the reference step on all host cores,
    on a bounded sample (whole steps of the same workload until ~budget_s)."""
    from oracle import oracle as O
    st = O.Stepper(spec)
    cores = O.max_threads()
    t0 = time.perf_counter()
    st.step()
    done = 1
    while time.perf_counter() - t0 < budget_s and done < max_steps:
        st.step()
        done += 1
    dt = time.perf_counter() - t0
    return {"value": spec.n * done / dt, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": "%d full steps of %s (%d particles, %d rigid spheres) in %.1f s" % (
                done, spec.name, spec.n, spec.nspheres, dt), "pairs_per_step": st.pairs}


def parity_of_step(spec, state):
    """Errors of one GPU step of the benched scene against the FP64 oracle
    from the identical state (the oracle is the checker here): grid order and
    ranges, density relative to FP64, fluid force per particle relative to
    max(|F64|, median |F64|) with the rigid contact term, and the FP64 body
    force sums.  `state` holds the GPU's state before the step and its
    buffers after it."""
    from oracle import oracle as O
    pos0, v0, before, g = state["pos0"], state["vel0"], state["before"], state["after"]
    p = O.make_common_params(spec.cell_size, spec.buckets, spec.h, spec.vlimit, spec.box_min, spec.box_max,
                             spec.gravity, spec.scale, spec.dt, relation=spec.f2r_rel, point_radius=spec.fluid_radius)
    keys, ids = O.calc_hash_key(pos0, spec.nbuckets, spec.cell_size)
    sk, si = O.sort_pairs(keys, ids)
    start, end, spos, svel = O.find_cell_offset(sk, si, pos0, v0, spec.nbuckets)
    grid_exact = bool(np.array_equal(g["IDS"], si) and np.array_equal(g["START"], start))
    kc = O.kernels_cache(spec.h)
    d64, pairs = O.density(spos, start, end, p, kc, spec.gas, spec.rest, spec.mass, f64=True)
    act = spos[:, 3] > 0
    e_rho = np.abs(g["DP"][act, 0].astype(np.float64) - d64[act, 0]) / d64[act, 0]
    contact = None
    out = {}
    if spec.bodies:
        nb_r = int(np.prod(spec.rb_buckets))
        cell = (spec.rb_radius,) * 3
        rk, ri, rw = O.calc_hash_key_with_offset(before["RB_LOCAL"], before["BODY_XF"], before["BODY_QF"], nb_r, cell)
        rsk, rsi = O.sort_pairs(rk, ri)
        rst, ren, rsp, _ = O.find_cell_offset(rsk, rsi, rw, None, nb_r)
        F64, _ = O.rb_forces_from_fluids(rsp, before["BODY_VF"], before["BODY_XF"], spec.rb_radius, spos, svel, start,
                                         end, spec.fluid_radius, spec.cell_size, spec.nbuckets, spec.r2f_rel, spec.ck,
                                         spec.ckd, f64=True)
        bf = np.zeros((len(spec.bodies), 3))
        np.add.at(bf, F64[:, 3].astype(np.int64), F64[:, :3])
        scale_f = max(np.abs(bf).max(), 1e-30)
        out["body_force_rel_max_vs_fp64"] = float((np.abs(g["BODY_FSUM"][:, :3] - bf) /
                                                   np.maximum(np.abs(bf), 1e-3 * scale_f)).max())
        cp = O.contact_params(spec.fluid_radius, spec.rb_radius, spec.ck, spec.ckd, cell, spec.f2r_rel, 0.003)
        contact = (cp, None, O.contact_grid(rsp, before["BODY_VF"], rst, ren, nb_r))
    nv64 = O.forces(spos, svel, d64.astype(np.float32), start, end, si, spec.mass, spec.visc, p, kc, f64=True,
                    newvel_init=v0, contact=contact)
    Fg = (g["VEL"][:, :3].astype(np.float64) - v0[:, :3]) / spec.dt
    Fr = (nv64[:, :3] - v0[:, :3].astype(np.float64)) / spec.dt
    mag = np.linalg.norm(Fr, axis=1)
    e_f = (np.linalg.norm(Fg - Fr, axis=1) / np.maximum(mag, np.median(mag)))[pos0[:, 3] > 0]
    out.update({"step": state["step"], "grid_bit_exact": grid_exact,
                "density_rel_max_vs_fp64": float(e_rho.max()), "force_rel_max_vs_fp64": float(e_f.max()),
                "pairs_per_particle": float(pairs) / len(pos0),
                "bars": {"density": 1e-5, "force": 2e-4, "body_force": 1e-4}})
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    spec = make_scene(args.workload)
    from oracle import oracle as O
    st = O.Stepper(spec)
    for _ in range(args.warmup):
        st.step()
    times = []
    # bounded sample: the first steps of the same trajectory, stopping after
    # REF_BUDGET_S of CPU time (the trajectory's later, denser steps cost more,
    # so a truncated sample overstates the CPU rate, never understates it)
    t_start = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st.step()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > REF_BUDGET_S:
            break
    tot = sum(times)
    done = len(times)
    v = spec.n * done / tot
    line = {"metric": "particle-steps/s", "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * tot / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": spec.name, "particles": spec.n, "buckets": spec.nbuckets,
                       "rigid_spheres": spec.nspheres, "bodies": len(spec.bodies)},
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": O.max_threads(), "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "%d timed full steps (of %d requested, %.0f s budget) after %d warm-up "
                                       "steps" % (done, args.steps, REF_BUDGET_S, args.warmup)},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def pct(a, q):
    return float(np.percentile(np.asarray(a, np.float64), q)) if len(a) else None


def run_batched(steps=1000, warmup=10, plain_sample=64):
    """Batched form: 256 uneven scenes (2,048-65,536 particles, half with a
    rigid sphere) in one world -- one segment-aware launch per stage, ten
    steps per captured graph -- against the plain path that steps each scene
    in its own one-scene world, one scene after another (timed on every
    4th scene, the rest by the same per-particle rate)."""
    from fluidgrid_gb300 import scenes
    from fluidgrid_gb300.world import World
    ss = scenes.batched_scenes(count=256)
    N = sum(s.n for s in ss)
    w = World(ss)
    w.set_option("graph_steps", 10)
    w.step(warmup)
    w.sync()
    blocks = w.timed_blocks(steps // 10, 10)
    w.check_finite()
    per_step = w.timed_steps(50)  # one step per graph: per-step latency of every scene in the batch
    tuning = w.tuning_stats()
    diag = w.diagnostics()
    w.close()
    total_ms = float(blocks.sum())
    value = N * (steps // 10) * 10 / (total_ms * 1e-3)
    bounded = run_batched_groups(ss, steps=steps, warmup=warmup)
    # plain path: each scene alone, sequentially
    sample = ss[::max(1, len(ss) // plain_sample)]
    t_plain, n_plain = 0.0, 0
    for sp in sample:
        ws = World([sp])
        ws.step(3)
        ms = ws.timed_steps(10)
        ws.close()
        t_plain += float(np.mean(ms))
        n_plain += sp.n
    plain = n_plain / (t_plain * 1e-3)
    return {"workload": "batched_256", "scenes": len(ss), "particles": N,
            "rigid_spheres": sum(s.nspheres for s in ss), "steps": (steps // 10) * 10,
            "value": value, "unit": "particle-steps/s", "ms_per_step": total_ms / ((steps // 10) * 10),
            "graph_steps": 10, "scene_step_latency_ms": {"p50": pct(per_step, 50), "p99": pct(per_step, 99)},
            "plain_sequential": {"value": plain, "unit": "particle-steps/s", "scenes_timed": len(sample)},
            "speedup_vs_plain": value / plain,
            "fp64_mass_total": float(sum(d["mass"] for d in diag)),
            "l2": "inputs larger than L2 (%.0f MB of particle state)" % (N * 32 / 1e6),
            "autotune": tuning, "latency_bounded": bounded}


def run_batched_groups(ss, steps=1000, warmup=10, max_group_particles=2_500_000):
    """The batched form with a bound on every scene's step latency: the
    scenes split into the fewest groups of at most `max_group_particles`
    (balanced greedily by particle count), each group one world; the groups
    step in turn, ten steps per graph, so a scene's step latency is its
    group's step time and the GPU never runs two groups at once."""
    from fluidgrid_gb300.world import World
    N = sum(s.n for s in ss)
    G = max(1, -(-N // max_group_particles))
    groups = [[] for _ in range(G)]
    load = [0] * G
    for s in sorted(ss, key=lambda s: -s.n):
        g = int(np.argmin(load))
        groups[g].append(s)
        load[g] += s.n
    worlds = []
    for grp in groups:
        w = World(grp)
        w.set_option("graph_steps", 10)
        w.step(warmup)
        w.sync()
        worlds.append(w)
    total_ms = 0.0
    for w in worlds:  # in turn: one group's blocks at a time
        total_ms += float(w.timed_blocks(steps // 10, 10).sum())
        w.check_finite()
    lat = []
    for w, grp in zip(worlds, groups):
        ms = w.timed_steps(50)  # one step per graph: the step latency of every scene of the group
        lat.extend(np.repeat(ms, len(grp)))
    for w in worlds:
        w.close()
    return {"groups": G, "group_particles": load, "value": N * (steps // 10) * 10 / (total_ms * 1e-3),
            "unit": "particle-steps/s", "scene_step_latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
            "max_group_particles": max_group_particles}


SIZE_CLASSES = (("<=65536", 0, 65536), ("65537-262144", 65537, 262144), (">262144", 262145, 1 << 40))


def size_class(n):
    for name, lo, hi in SIZE_CLASSES:
        if lo <= n <= hi:
            return name
    return SIZE_CLASSES[-1][0]


def run_served(duration=60.0, rate=200.0, budget=120 << 30, seed=0x5EED, pipeline_depth=2):
    """Served form (the C5 workload): Poisson arrivals at `rate` per second of
    dam-break requests (fluid counts log-uniform in [4,096, 524,288], 0-4
    rigid boxes of 1,024 spheres, step counts uniform in [100, 2000]) for
    `duration` seconds of wall time into a continuous-batching server with
    its default admission policy: the HBM budget, a per-step work budget that
    bounds every resident scene's step latency, and reservations with
    backfilling for the oldest request.  Every server step advances every
    resident scene; up to `pipeline_depth` steps stay in flight while the
    host prepares the next.  Step latency is recorded for every resident
    scene and reported per size class."""
    import ctypes
    from fluidgrid_gb300 import _ffi, scenes
    from fluidgrid_gb300.server import Server
    pool = scenes.served_templates(seed=seed)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, int(rate * duration * 1.5) + 16))
    arrivals = arrivals[arrivals < duration]
    picks = rng.integers(0, len(pool), len(arrivals))
    nsteps = rng.integers(100, 2001, len(arrivals))
    cfg = _ffi.fg_server_config()
    _ffi.load().fg_server_config_defaults(ctypes.byref(cfg))
    policy = {"hbm_budget_bytes": budget, "max_particles_per_step": int(cfg.max_particles),
              "target_step_ms": round(float(cfg.target_step_ms), 3), "head_wait_s": round(float(cfg.head_wait_s), 3),
              "autotune_period": int(cfg.autotune_period)}
    srv = Server(budget_bytes=budget, pipeline_depth=pipeline_depth)
    ids = []
    infos = []
    by_class = {name: [] for name, _, _ in SIZE_CLASSES}
    t0 = time.perf_counter()
    k = 0
    while True:
        now = time.perf_counter() - t0
        if now >= duration:
            break
        while k < len(arrivals) and arrivals[k] <= now:
            ids.append(srv.submit(pool[picks[k]], int(nsteps[k])))
            k += 1
        resident = srv.active()
        info = srv.step()
        infos.append(info)
        if info["step_ms"] > 0:
            for cls in {size_class(srv.n_of[r]) for r in resident}:
                by_class[cls].append(info["step_ms"])
    elapsed = time.perf_counter() - t0
    st = srv.stats()
    reqs = [(srv.request(i), srv.n_of[i]) for i in ids]
    srv.close()
    done = [(r, n) for r, n in reqs if r["state"] == 2]
    admitted = [(r, n) for r, n in reqs if r["state"] >= 1]
    step_ms = [i["step_ms"] for i in infos if i["active_particles"] and i["step_ms"] > 0]
    wall_ms = [i["wall_ms"] for i in infos if i["active_particles"]]
    lat_cls = {}
    for name, _, _ in SIZE_CLASSES:
        d = by_class[name]
        rl = [r["done_s"] - r["submit_s"] for r, n in done if size_class(n) == name]
        lat_cls[name] = {"step_samples": len(d), "p50": pct(d, 50), "p99": pct(d, 99),
                         "completed": len(rl), "request_latency_s_p50": pct(rl, 50),
                         "request_latency_s_p99": pct(rl, 99)}
    return {"workload": "served_c5", "duration_s": duration, "arrival_rate_per_s": rate, "policy": policy,
            "pipeline_depth": pipeline_depth, "submitted": len(ids), "admitted": len(admitted),
            "completed": len(done), "queued_at_end": st["queued"], "server_steps": st["steps"],
            "value": st["particle_steps"] / elapsed, "unit": "particle-steps/s",
            "step_latency_ms": {"p50": pct(step_ms, 50), "p99": pct(step_ms, 99)},
            "step_latency_ms_by_size_class": lat_cls,
            "server_step_wall_ms": {"p50": pct(wall_ms, 50), "p99": pct(wall_ms, 99)},
            "request_latency_s": {"p50": pct([r["done_s"] - r["submit_s"] for r, _ in done], 50),
                                  "p99": pct([r["done_s"] - r["submit_s"] for r, _ in done], 99)},
            "admission_wait_s": {"p50": pct([r["admit_s"] - r["submit_s"] for r, _ in admitted], 50),
                                 "p99": pct([r["admit_s"] - r["submit_s"] for r, _ in admitted], 99)},
            "max_resident_particles": int(max([i["active_particles"] for i in infos] + [0])),
            "max_resident_bytes": int(max([i["resident_bytes"] for i in infos] + [0])),
            "device_bytes": st["device_bytes"],
            "note": "arrivals ask ~2e10 particle-steps/s, ~20x the GPU: the queue grows and the admission "
                    "policy decides what runs"}


TRAJECTORY_STEPS = 500  # the configured dam-break trajectory (3 warm-up + 497 timed)
STATE_NAMES = ("RB_LOCAL", "BODY_X", "BODY_V", "BODY_Q", "BODY_L", "BODY_XF", "BODY_VF", "BODY_QF")
AFTER_NAMES = ("IDS", "START", "DP", "VEL", "BODY_FSUM")


def stage_means(prof):
    return {key: float(np.mean([p[key] for p in prof])) for key in prof[0]} if prof else {}


def run_ours(args, rank, world, local):
    import fluidgrid_gb300 as fgm
    from fluidgrid_gb300.world import World, PinnedArray, fp32_peak_tflops
    from fluidgrid_gb300 import _ffi
    L = fgm.load()
    _ffi.check(L.fg_set_device(local), "fg_set_device")
    dist = Dist(world)
    spec = make_scene(args.workload)
    n = spec.n
    W, K = args.warmup, args.steps
    # 1. timed run: W warm-up steps, then K steps each preceded by an L2 flush
    w = World([spec])
    w.step(W)
    w.sync()
    w.counters(reset=True)
    clocks = ClockSampler(local)
    dist.barrier()
    w.sync()
    clocks.start()
    k0 = w.kernel_launches()
    ms = w.timed_steps(K, FLUSH_BYTES)
    launches = w.kernel_launches() - k0  # the steps', the order refreshes' and the L2 flushes'
    w.sync()
    clk = clocks.stop()
    dist.barrier()
    total_ms = dist.reduce(float(ms.sum()), "max")
    pair_visits, counted = w.counters(reset=True)
    w.check_finite()
    tuning = w.tuning_stats()
    tuning["list_overflow_particle_steps"] = w.list_overflows(reset=True)
    # the state at the end of the window and one more step from it: the
    # parity check's input (compared with the oracle in the CPU-baseline leg)
    pstate = None
    if rank == 0 and not args.no_cpu_baseline:
        pos0, vel0 = w.download()
        before = {k: w.read(k) for k in STATE_NAMES} if spec.bodies else {}
        w.step(1)
        pstate = {"step": W + K + 1, "pos0": pos0, "vel0": vel0, "before": before,
                  "after": {k: w.read(k) for k in AFTER_NAMES}}
    w.close()
    # 2. end to end on the same window: every step uploads the particle state
    #    from pinned host memory and downloads it again
    w = World([spec])
    w.step(W)
    pos, vel = w.download()
    hp, hv = PinnedArray((n, 4)), PinnedArray((n, 4))
    hp.array[:] = pos
    hv.array[:] = vel
    dist.barrier()
    ems = w.e2e_steps(K, hp.array, hv.array, hp.array, hv.array)
    dist.barrier()
    e2e_ms = dist.reduce(float(ems.sum()), "max")
    hp.free()
    hv.free()
    w.close()
    # 3. per-stage breakdown over the same window (about 20 profiled steps)
    every = max(1, K // 20)
    w = World([spec])
    w.step(W)
    prof = []
    for k in range(K):
        if k % every == every // 2:
            prof.append(w.stage_profile(FLUSH_BYTES))
        else:
            w.step(1)
    w.close()
    stages = stage_means(prof)
    # 4. the whole configured trajectory, unless the window already is it
    traj = None
    if W + K < TRAJECTORY_STEPS:
        w = World([spec])
        w.step(3)
        tms = w.timed_steps(TRAJECTORY_STEPS - 3, FLUSH_BYTES)
        w.close()
        w = World([spec])
        tprof = []
        for k in range(TRAJECTORY_STEPS):
            if k % 25 == 12:
                tprof.append(w.stage_profile(FLUSH_BYTES))
            else:
                w.step(1)
        w.close()
        traj = {"steps": TRAJECTORY_STEPS - 3, "warmup": 3, "ms_per_step": float(tms.mean()),
                "value": world * n / (float(tms.mean()) * 1e-3), "unit": "particle-steps/s",
                "step_ms": {"p50": pct(tms, 50), "p99": pct(tms, 99)}, "stages_ms": stage_means(tprof)}
    value = world * n * K / (total_ms * 1e-3)
    e2e_value = world * n * K / (e2e_ms * 1e-3)
    # 5. the batched and served forms (one GPU each rank, replicas)
    forms = {}
    if "batched" in args.forms:
        forms["batched"] = run_batched()
    if "served" in args.forms:
        forms["served"] = run_served(duration=args.served_seconds)
    if rank == 0:
        peak, peak_kind = measured_peaks()
        phase = window_phase(W, W + K)

        def hbm(kernel, stage, per_p):
            a = per_p * n / (stages[stage] * 1e-3) / 1e9
            t = profile_traffic(kernel, phase)
            return {"kernel": kernel, "achieved": a, "peak": peak, "unit": "GB/s", "frac": a / peak,
                    "bytes_per_particle": per_p, "traffic": (t * n) if t else None, "traffic_phase": phase,
                    "ms": stages[stage]}
        dom = max(("forces", "density"), key=lambda k: stages.get(k, 0.0))
        dom_kernel = "k_forces" if dom == "forces" else "k_density"
        roof = hbm(dom_kernel, dom, BYTES_FORCES if dom == "forces" else BYTES_DENSITY)
        cpu = None if args.no_cpu_baseline else cpu_baseline(spec)
        fp32_peak = fp32_peak_tflops()
        pairs_per_step = pair_visits / max(counted, 1)
        flops = (FLOPS_FORCE_PAIR * (pairs_per_step - n)) if dom == "forces" else FLOPS_DENSITY_PAIR * pairs_per_step
        ach = flops / (stages[dom] * 1e-3) / 1e12
        roof.update({"bound": "hbm", "peak_kind": peak_kind,
                     "issue_active_pct": profile_value("issue_active_pct_" + phase, dom_kernel),
                     "fp32": {"achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                              "pairs_per_step": pairs_per_step, "peak_kind": "measured (FMA probe)"},
                     "force_kernel": hbm("k_forces", "forces", BYTES_FORCES),
                     "density_kernel": hbm("k_density", "density", BYTES_DENSITY)})
        parity = parity_of_step(spec, pstate) if pstate is not None else None
        ms_sorted = np.sort(ms)
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": K, "warmup": W, "ms_per_step": total_ms / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded jittered lattice + rigid box, seed 0x5EED)",
            "config": {"workload": spec.name, "particles": n, "buckets": spec.nbuckets,
                       "rigid_spheres": spec.nspheres, "bodies": len(spec.bodies),
                       "trajectory_steps": [W, W + K], "trajectory_phase": phase,
                       "l2": "flushed before every timed step (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "single",
                       "autotune": tuning},
            "latency_ms": {"p50": float(np.percentile(ms_sorted, 50)), "p99": float(np.percentile(ms_sorted, 99)),
                           "max": float(ms_sorted[-1]), "slowest_steps": [int(W + k) for k in np.argsort(-ms)[:5]]},
            "stages_ms": stages,
            "trajectory_mean": traj,
            "roofline": roof,
            "cpu_baseline": ({k: v for k, v in cpu.items() if k != "pairs_per_step"} if cpu else None),
            "parity": parity,
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": 32 * n,
                    "d2h_bytes_per_step": 32 * n, "ms_per_step": e2e_ms / K,
                    "step_ms": {"p50": float(np.percentile(ems, 50)), "p99": float(np.percentile(ems, 99)),
                                "max": float(ems.max()), "slowest_steps": [int(W + k) for k in np.argsort(-ems)[:5]]}},
            "gpu_launches": launches,
            "clocks": clk,
            "forms": forms,
        }
        print(json.dumps(line))
    dist.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: the configured 500-step trajectory (3 warm-up + 497 timed steps)
    ap.add_argument("--steps", type=int, default=497)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam_break_rigid_1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--forms", default="batched,served",
                    help="comma list of extra forms to measure after the plain path: batched, served")
    ap.add_argument("--served-seconds", type=float, default=60.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_info()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
