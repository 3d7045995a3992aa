"""Build libfluidgrid_gb300.so in-tree for sm_103a (GB300).

    python -m fluidgrid_gb300.build [--force] [--verbose-ptxas]

Each .cu under csrc/ is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a -lineinfo -O3) and linked into
fluidgrid_gb300/_lib/libfluidgrid_gb300.so.  No fast-math: the bucket hash
needs IEEE division and the kernels use explicit rounding intrinsics where the
reference's results must be reproduced bit for bit.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libfluidgrid_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers_mtime():
    ts = [os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC)
          if f.endswith((".h", ".cuh"))]
    inc = os.path.join(os.path.dirname(HERE), "include")
    ts += [os.path.getmtime(os.path.join(inc, f)) for f in os.listdir(inc) if f.endswith(".h")]
    return max(ts) if ts else 0.0


def _compile(src, force, extra):
    obj = os.path.join(OBJ_DIR, src[:-3] + ".o")
    s = os.path.join(CSRC, src)
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(s), headers_mtime()):
        return obj, ""
    cmd = [nvcc()] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                             "-diag-suppress", "1444", "-c", s, "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stdout + r.stderr


def build(force=False, verbose_ptxas=False, quiet=True):
    os.makedirs(OBJ_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, force or verbose_ptxas, extra), srcs))
    objs = [o for o, _ in results]
    logs = "".join(l for _, l in results)
    if verbose_ptxas or not quiet:
        sys.stdout.write(logs)
    newest = max(os.path.getmtime(o) for o in objs)
    if force or verbose_ptxas or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose_ptxas=a.verbose_ptxas, quiet=False))


if __name__ == "__main__":
    main()
