"""Python handle on the C ABI world (include/fluidgrid_gb300.h).

A World is a packed set of scenes stepped together on one GPU; a one-scene
world is the plain drop-in step of HeterogeneousSimulator::doTimeStep
(HeterogeneousSimulator.cpp:54-127).  All compute runs in
libfluidgrid_gb300.so; this module only marshals host arrays.
"""
import ctypes

import numpy as np

from . import _ffi
from ._ffi import BUF, check


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class PinnedArray:
    """numpy view of pinned host memory from fg_host_alloc."""

    def __init__(self, shape, dtype=np.float32):
        self.L = _ffi.load()
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.p = self.L.fg_host_alloc(max(nbytes, 16))
        if not self.p:
            raise _ffi.FluidGridError("fg_host_alloc(%d) failed" % nbytes)
        buf = (ctypes.c_char * max(nbytes, 16)).from_address(self.p)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self.p:
            self.array = None
            self.L.fg_host_free(ctypes.c_void_p(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def fp32_peak_tflops():
    v = ctypes.c_float()
    check(_ffi.load().fg_probe_fp32_peak(ctypes.byref(v)), "fg_probe_fp32_peak")
    return float(v.value)


class World:
    def __init__(self, specs, stream=None):
        if not isinstance(specs, (list, tuple)):
            specs = [specs]
        self.L = _ffi.load()
        self.specs = list(specs)
        n = len(self.specs)
        self._descs = (_ffi.fg_scene_desc * n)()
        self._keep = []
        for i, sp in enumerate(self.specs):
            sp.fill_desc(self._descs[i], self._keep)
        h = ctypes.c_void_p()
        st = ctypes.c_void_p(stream) if stream else None
        check(self.L.fg_world_create(self._descs, n, st, ctypes.byref(h)), "fg_world_create")
        self.h = h
        self.n = self.L.fg_world_particles(h)
        self.nscenes = n
        self.nspheres = self.L.fg_world_spheres(h)
        self.nbodies = self.L.fg_world_bodies(h)

    # ---------------------------------------------------------------- lifecycle
    def close(self):
        if getattr(self, "h", None):
            self.L.fg_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- stepping
    def step(self, nsteps=1):
        check(self.L.fg_world_step(self.h, int(nsteps)), "fg_world_step")

    def sync(self):
        check(self.L.fg_world_sync(self.h), "fg_world_sync")

    def check_finite(self):
        check(self.L.fg_world_check(self.h), "fg_world_check")
        self.sync()

    def set_stages(self, mask):
        check(self.L.fg_world_set_stages(self.h, int(mask)), "fg_world_set_stages")

    def set_fused_integrate(self, fused):
        check(self.L.fg_world_set_fused_integrate(self.h, 1 if fused else 0), "set_fused_integrate")

    def set_digit_bits(self, bits):
        check(self.L.fg_world_set_sort_digit_bits(self.h, int(bits)), "set_sort_digit_bits")

    def set_graphs(self, on):
        check(self.L.fg_world_set_graphs(self.h, 1 if on else 0), "set_graphs")

    def set_option(self, name, value):
        check(self.L.fg_world_set_option(self.h, _ffi.OPTIONS[name], int(value)), "fg_world_set_option")

    def get_option(self, name):
        v = ctypes.c_int()
        check(self.L.fg_world_get_option(self.h, _ffi.OPTIONS[name], ctypes.byref(v)), "fg_world_get_option")
        return int(v.value)

    def options(self):
        return {k: self.get_option(k) for k in _ffi.OPTIONS}

    def counters(self, reset=False):
        """(in-range pair visits, steps) counted since the last reset."""
        pv = ctypes.c_uint64()
        st = ctypes.c_uint64()
        check(self.L.fg_world_counters(self.h, 1 if reset else 0, ctypes.byref(pv), ctypes.byref(st)),
              "fg_world_counters")
        return int(pv.value), int(st.value)

    def list_overflows(self, reset=False):
        """Particles (summed over steps) whose in-range visits exceeded the
        neighbour-list capacity since the last reset."""
        v = ctypes.c_uint64()
        check(self.L.fg_world_list_overflows(self.h, 1 if reset else 0, ctypes.byref(v)), "fg_world_list_overflows")
        return int(v.value)

    def tuning_stats(self):
        """Steps run with each density/force kernel, the last kernel trial
        times and the tunables in use."""
        cnt = (ctypes.c_uint32 * _ffi.NUM_KERNELS)()
        ms = (ctypes.c_float * _ffi.NUM_KERNELS)()
        check(self.L.fg_world_tuning_stats(self.h, cnt, ms), "fg_world_tuning_stats")
        return {"steps_per_kernel": list(cnt), "last_trial_ms": [round(x, 4) for x in ms],
                "kernel": self.get_option("kernel"), "ctas_per_sm": self.get_option("ctas_per_sm"),
                "digit_bits": self.get_option("digit_bits"), "one_pass_sort": self.get_option("one_pass_sort"),
                "block_size": self.get_option("block_size"), "runs_per_cta": self.get_option("runs_per_cta"),
                "list_cap": self.get_option("list_cap")}

    def launches_per_step(self):
        return int(self.L.fg_world_launches_per_step(self.h))

    def kernel_launches(self):
        """Kernel launches this world has enqueued or replayed so far."""
        c = ctypes.c_uint64(0)
        check(self.L.fg_world_kernel_launches(self.h, ctypes.byref(c)), "fg_world_kernel_launches")
        return int(c.value)

    # ---------------------------------------------------------------- timing
    STAGES = ["hash", "sort", "ranges", "density", "rb_grid", "rb_contact", "forces", "bodies"]

    def stage_profile(self, flush_bytes=256 << 20):
        """One step with CUDA events around each stage (after an L2 flush);
        returns {stage: ms}."""
        ms = (ctypes.c_float * 8)()
        check(self.L.fg_world_stage_profile(self.h, int(flush_bytes), ms), "fg_world_stage_profile")
        return dict(zip(self.STAGES, list(ms)))

    def timed_steps(self, nsteps, flush_bytes=256 << 20):
        ms = (ctypes.c_float * max(1, nsteps))()
        check(self.L.fg_world_timed_steps(self.h, int(nsteps), int(flush_bytes), ms), "fg_world_timed_steps")
        return np.array(ms[:nsteps], np.float64)

    DIAG = ["active", "mass", "px", "py", "pz", "kinetic", "mx", "my", "mz", "body_px", "body_py", "body_pz",
            "body_Lx", "body_Ly", "body_Lz", "body_kinetic"]

    def diagnostics(self):
        """FP64 conservation diagnostics computed on the GPU: one dict per
        scene (fluid mass, momentum, kinetic energy, first moment; body
        momentum, angular momentum, kinetic energy)."""
        out = (ctypes.c_double * (16 * max(1, self.nscenes)))()
        check(self.L.fg_world_diagnostics(self.h, out), "fg_world_diagnostics")
        return [dict(zip(self.DIAG, out[16 * s:16 * s + 16])) for s in range(self.nscenes)]

    def timed_blocks(self, nblocks, steps_per_block, flush_bytes=0):
        """nblocks blocks of steps_per_block steps, each bracketed by CUDA
        events; returns the block durations in ms."""
        ms = (ctypes.c_float * max(1, nblocks))()
        check(self.L.fg_world_timed_blocks(self.h, int(nblocks), int(steps_per_block), int(flush_bytes), ms),
              "fg_world_timed_blocks")
        return np.array(ms[:nblocks], np.float64)

    def e2e_steps(self, nsteps, host_pos, host_vel, out_pos, out_vel):
        ms = (ctypes.c_float * max(1, nsteps))()
        check(self.L.fg_world_e2e_steps(self.h, int(nsteps), _ptr(host_pos), _ptr(host_vel), _ptr(out_pos),
                                        _ptr(out_vel), ms), "fg_world_e2e_steps")
        return np.array(ms[:nsteps], np.float64)

    # ---------------------------------------------------------------- state
    def upload(self, pos4, vel4=None):
        pos4 = np.ascontiguousarray(pos4, np.float32)
        vel4 = None if vel4 is None else np.ascontiguousarray(vel4, np.float32)
        check(self.L.fg_world_upload(self.h, _ptr(pos4), _ptr(vel4)), "fg_world_upload")
        self.sync()

    def download(self):
        pos = np.empty((self.n, 4), np.float32)
        vel = np.empty((self.n, 4), np.float32)
        check(self.L.fg_world_download(self.h, _ptr(pos), _ptr(vel)), "fg_world_download")
        self.sync()
        return pos, vel

    def layout(self, scene):
        out = (ctypes.c_uint32 * 8)()
        check(self.L.fg_world_scene_layout(self.h, int(scene), out), "fg_world_scene_layout")
        keys = ("pbase", "n", "bucket_base", "nb", "sph_base", "nsph", "body_base", "nbodies")
        return dict(zip(keys, list(out)))

    def buffer(self, name):
        p = ctypes.c_void_p()
        b = ctypes.c_size_t()
        check(self.L.fg_world_buffer(self.h, BUF[name], ctypes.byref(p), ctypes.byref(b)), "fg_world_buffer")
        return p.value, b.value

    _DT = {"POS": (np.float32, 4), "VEL": (np.float32, 4), "KEYS_UNSORTED": (np.uint32, 0),
           "KEYS": (np.uint32, 0), "IDS": (np.uint32, 0), "START": (np.uint32, 0), "END": (np.uint32, 0),
           "SPOS": (np.float32, 4), "SVEL": (np.float32, 4), "DP": (np.float32, 2),
           "RB_LOCAL": (np.float32, 4), "RB_WORLD": (np.float32, 4), "RB_KEYS_UNSORTED": (np.uint32, 0),
           "RB_KEYS": (np.uint32, 0), "RB_IDS": (np.uint32, 0), "RB_START": (np.uint32, 0),
           "RB_END": (np.uint32, 0), "RB_SPOS": (np.float32, 4), "RB_FORCE": (np.float32, 4),
           "RB_TORQUE": (np.float32, 4), "BODY_X": (np.float64, 4), "BODY_V": (np.float64, 4),
           "BODY_Q": (np.float64, 4), "BODY_L": (np.float64, 4), "BODY_FSUM": (np.float64, 4),
           "BODY_TSUM": (np.float64, 4), "BODY_XF": (np.float32, 4), "BODY_VF": (np.float32, 4),
           "BODY_QF": (np.float32, 4), "BODY_MASS": (np.float64, 0), "BODY_INV_INERTIA": (np.float64, 9)}

    def read(self, name):
        """Copy a device buffer to a new numpy array (synchronises)."""
        self.sync()
        p, b = self.buffer(name)
        dt, w = self._DT[name]
        count = b // np.dtype(dt).itemsize
        out = np.empty(count, dt)
        if b:
            check(self.L.fg_memcpy_d2h(_ptr(out), ctypes.c_void_p(p), b), "fg_memcpy_d2h")
        return out.reshape(-1, w) if w else out

    def write(self, name, arr):
        self.sync()
        p, b = self.buffer(name)
        dt, _ = self._DT[name]
        a = np.ascontiguousarray(arr, dt)
        if a.nbytes != b:
            raise ValueError("buffer %s holds %d bytes, got %d" % (name, b, a.nbytes))
        if b:
            check(self.L.fg_memcpy_h2d(ctypes.c_void_p(p), _ptr(a), b), "fg_memcpy_h2d")
