"""Python handle on the served form (fg_server_* in include/fluidgrid_gb300.h):
continuous batching of independent scenes under an HBM budget.  All work runs
in libfluidgrid_gb300.so; this module marshals scenes and results."""
import ctypes

import numpy as np

from . import _ffi
from ._ffi import check


class Server:
    def __init__(self, budget_bytes=120 << 30, max_particles=None, max_admit_per_step=0, use_graphs=True,
                 grow_via_host=False, stream=None, pipeline_depth=0, target_step_ms=None, head_wait_s=None):
        """None keeps the library default of a setting (fg_server_config_defaults)."""
        self.L = _ffi.load()
        cfg = _ffi.fg_server_config()
        self.L.fg_server_config_defaults(ctypes.byref(cfg))
        cfg.hbm_budget_bytes = int(budget_bytes)
        if max_particles is not None:
            cfg.max_particles = int(max_particles)
        cfg.max_admit_per_step = int(max_admit_per_step)
        cfg.use_graphs = 1 if use_graphs else 0
        cfg.grow_via_host = 1 if grow_via_host else 0
        cfg.pipeline_depth = int(pipeline_depth)
        if target_step_ms is not None:
            cfg.target_step_ms = float(target_step_ms)
        if head_wait_s is not None:
            cfg.head_wait_s = float(head_wait_s)
        h = ctypes.c_void_p()
        check(self.L.fg_server_create(ctypes.byref(cfg), ctypes.c_void_p(stream) if stream else None,
                                      ctypes.byref(h)), "fg_server_create")
        self.h = h
        self.n_of = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.fg_server_destroy(self.h)
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

    def submit(self, spec, steps):
        """Queue `spec` for `steps` steps; returns the request id."""
        d = _ffi.fg_scene_desc()
        keep = []
        spec.fill_desc(d, keep)
        rid = ctypes.c_uint64()
        check(self.L.fg_server_submit(self.h, ctypes.byref(d), int(steps), ctypes.byref(rid)), "fg_server_submit")
        self.n_of[rid.value] = spec.n
        return int(rid.value)

    def step(self):
        info = _ffi.fg_server_step_info()
        check(self.L.fg_server_step(self.h, ctypes.byref(info)), "fg_server_step")
        return {k: getattr(info, k) for k, _ in info._fields_ if k != "pad_"}

    def request(self, rid):
        info = _ffi.fg_request_info()
        check(self.L.fg_server_request(self.h, int(rid), ctypes.byref(info)), "fg_server_request")
        return {k: getattr(info, k) for k, _ in info._fields_}

    def done(self, rid):
        return self.request(rid)["state"] == _ffi.REQ_DONE

    def result(self, rid, release=True):
        """Final (positions, velocities) of a finished request."""
        n = self.n_of[rid]
        pos = np.empty((n, 4), np.float32)
        vel = np.empty((n, 4), np.float32)
        check(self.L.fg_server_result(self.h, int(rid), ctypes.c_void_p(pos.ctypes.data),
                                      ctypes.c_void_p(vel.ctypes.data), 1 if release else 0), "fg_server_result")
        if release:
            del self.n_of[rid]
        return pos, vel

    def active(self):
        """Request ids of the resident scenes (the ones the next step advances)."""
        n = ctypes.c_uint32()
        check(self.L.fg_server_active(self.h, None, 0, ctypes.byref(n)), "fg_server_active")
        ids = (ctypes.c_uint64 * max(1, n.value))()
        check(self.L.fg_server_active(self.h, ids, n.value, ctypes.byref(n)), "fg_server_active")
        return list(ids[:n.value])

    def stats(self):
        st = _ffi.fg_server_stats_info()
        check(self.L.fg_server_stats(self.h, ctypes.byref(st)), "fg_server_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}
