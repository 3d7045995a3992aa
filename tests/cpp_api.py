"""Compiles small C++ programs against include/fluidgrid_sim.hpp and the
library (the headless mirror of the reference's simulation classes)."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "fluidgrid_gb300", "_lib")
CUDA_INC = "/usr/local/cuda/include"


def f32(x):
    """A C++ hex float literal of the float32 value of x."""
    import numpy as np
    return float(np.float32(x)).hex() + "f"


def build_and_run(src, args=(), cwd=None):
    d = cwd or tempfile.mkdtemp()
    cpp = os.path.join(d, "prog.cpp")
    exe = os.path.join(d, "prog")
    with open(cpp, "w") as f:
        f.write(src)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", INC, "-I", CUDA_INC, cpp, "-o", exe, "-L", LIBDIR,
                           "-lfluidgrid_gb300", "-Wl,-rpath," + LIBDIR])
    r = subprocess.run([exe] + list(args), cwd=d, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("program exited with %d; stderr:\n%s" % (r.returncode, r.stderr[-4000:]))
    return r.stdout
