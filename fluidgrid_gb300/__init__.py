"""fluidgrid_gb300 -- GB300-native (sm_103a) SPH step of FluidGrid.

The hot path (hash grid build, density/pressure, pressure+viscosity forces,
walls, integration, fluid/rigid contact with per-body force/torque
reduction) runs in hand-written CUDA kernels inside
fluidgrid_gb300/_lib/libfluidgrid_gb300.so, reached through the C ABI of
include/fluidgrid_gb300.h (worlds of scenes, the continuous-batching server)
and the reference's own launcher
names in include/fluidgrid_reference.h.  This package marshals host arrays
and generates seeded synthetic scenes; it computes nothing itself.
"""
from ._ffi import FluidGridError, load, lib_path  # noqa: F401
from .world import World  # noqa: F401
from .server import Server  # noqa: F401
from . import scenes  # noqa: F401

__all__ = ["World", "Server", "FluidGridError", "load", "lib_path", "scenes"]
