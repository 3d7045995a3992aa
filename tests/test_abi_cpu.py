"""CPU checks of the drop-in boundary: the C-ABI library loads, exports every
symbol the public headers declare, its struct layouts match the ctypes
mirrors, and argument validation works without a GPU."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import fluidgrid_gb300 as fg
from fluidgrid_gb300 import _ffi, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def lib():
    from fluidgrid_gb300 import build
    build.build()
    return fg.load()


def declared_functions(header):
    text = open(os.path.join(INC, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M)
    return sorted(set(n for n in names if not n.startswith("__")))


@pytest.mark.parametrize("header", ["fluidgrid_gb300.h", "fluidgrid_reference.h"])
def test_library_exports_every_declared_symbol(lib, header):
    names = declared_functions(header)
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_launcher_names_complete(lib):
    # every extern "C" launcher of K_HashGrid.cuh, K_FluidSim.cuh, K_RigidBodySim.cuh
    for n in _ffi.REFERENCE_SYMBOLS + _ffi.C_ABI_SYMBOLS:
        assert hasattr(lib, n), n


C_LAYOUT = r"""
#include <stdio.h>
#include <stddef.h>
#include "fluidgrid_gb300.h"
#include "fluidgrid_reference.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(fg_scene_desc), offsetof(fg_scene_desc, bodies),
         offsetof(fg_scene_desc, rb_volume_max), sizeof(fg_body_desc), offsetof(fg_body_desc, inv_inertia),
         sizeof(fgr_common_fluid_params), offsetof(fgr_common_fluid_params, fluid_to_srb_relation));
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(fg_server_config),
         offsetof(fg_server_config, use_graphs), offsetof(fg_server_config, pipeline_depth),
         offsetof(fg_server_config, target_step_ms), offsetof(fg_server_config, head_wait_s),
         sizeof(fg_server_step_info),
         offsetof(fg_server_step_info, wall_ms), offsetof(fg_server_step_info, resident_bytes),
         sizeof(fg_request_info), offsetof(fg_request_info, submit_s), offsetof(fg_request_info, resident_bytes),
         sizeof(fg_server_stats_info), offsetof(fg_server_stats_info, device_bytes));
  return 0;
}
"""


def test_struct_layouts_match_ctypes():
    cuda_inc = "/usr/local/cuda/include"
    if not os.path.exists(os.path.join(cuda_inc, "vector_types.h")):
        pytest.skip("CUDA headers not found")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "l.c")
        open(src, "w").write(C_LAYOUT)
        exe = os.path.join(d, "l")
        subprocess.check_call(["gcc", "-I", INC, "-I", cuda_inc, src, "-o", exe])
        got = [int(x) for x in subprocess.check_output([exe]).split()]
    D, B, C = _ffi.fg_scene_desc, _ffi.fg_body_desc, _ffi.fgr_common_fluid_params
    want = [ctypes.sizeof(D), D.bodies.offset, D.rb_volume_max.offset, ctypes.sizeof(B), B.inv_inertia.offset,
            ctypes.sizeof(C), C.fluid_to_srb_relation.offset]
    SC, SI, RI, ST = (_ffi.fg_server_config, _ffi.fg_server_step_info, _ffi.fg_request_info,
                      _ffi.fg_server_stats_info)
    want += [ctypes.sizeof(SC), SC.use_graphs.offset, SC.pipeline_depth.offset, SC.target_step_ms.offset,
             SC.head_wait_s.offset, ctypes.sizeof(SI), SI.wall_ms.offset,
             SI.resident_bytes.offset, ctypes.sizeof(RI), RI.submit_s.offset, RI.resident_bytes.offset,
             ctypes.sizeof(ST), ST.device_bytes.offset]
    assert got == want
    # CommonFluidParams of the reference: 26 four-byte fields, 4-byte alignment
    assert ctypes.sizeof(C) == 104


def test_defaults_are_reference_literals(lib):
    d = _ffi.fg_scene_desc()
    lib.fg_scene_desc_defaults(ctypes.byref(d))
    assert d.wall_distance == pytest.approx(0.003043174)
    assert (d.wall_stiffness, d.wall_damping) == (20000.0, 256.0)
    assert list(d.noslip_min) == [-11.0, -40.0, -11.0] and list(d.noslip_max) == [11.0, 200.0, 11.0]
    assert d.fluid_contact_eps == pytest.approx(0.003) and d.rb_contact_eps == pytest.approx(0.0001)
    assert d.rbrb_eps == pytest.approx(0.001)
    assert (d.contact_kspring, d.contact_kdamping) == (-10.0, -5.0)


def _create(lib, spec):
    descs = (_ffi.fg_scene_desc * 1)()
    keep = []
    spec.fill_desc(descs[0], keep)
    h = ctypes.c_void_p()
    return lib.fg_world_create(descs, 1, None, ctypes.byref(h)), descs, keep


def test_invalid_scene_rejected_without_gpu(lib):
    spec = scenes.dam_break_small()
    spec.buckets = (0, 64, 64)
    st, _, _ = _create(lib, spec)
    assert _ffi.STATUS[st] == "FG_E_INVALID"
    spec = scenes.dam_break_small()
    spec.cell = (0.0, 0.1, 0.1)
    st, _, _ = _create(lib, spec)
    assert _ffi.STATUS[st] == "FG_E_INVALID"
    spec = scenes.dam_break_rigid(nx=8, ny=4, nz=8, spheres=64)
    spec.bodies[0].mass = -1.0  # 0 is a static body; negative is invalid
    st, _, _ = _create(lib, spec)
    assert _ffi.STATUS[st] == "FG_E_INVALID"


def test_null_arguments_rejected(lib):
    assert lib.fg_world_create(None, 1, None, None) == 1
    assert lib.fg_world_step(None, 1) == 1
    assert lib.fg_world_sync(None) == 1


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_ffi, "_lib", None)
    monkeypatch.setattr(_ffi, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(fg.FluidGridError):
        _ffi.load()


def test_scene_generators_are_seeded():
    a = scenes.dam_break_small(seed=7)
    b = scenes.dam_break_small(seed=7)
    c = scenes.dam_break_small(seed=8)
    assert a.n == 16384 and np.array_equal(a.pos, b.pos) and not np.array_equal(a.pos, c.pos)
    r = scenes.dam_break_rigid(nx=16, ny=8, nz=16)
    assert r.bodies[0].local.shape == (4096, 4)
    q = np.array(r.bodies[0].orientation)
    assert abs(np.linalg.norm(q) - 1) < 1e-6
    # spheres lie on the cube surface
    loc = r.bodies[0].local[:, :3]
    assert np.allclose(np.abs(loc).max(axis=1), 0.2, atol=1e-6)


def test_full_size_generators_shapes():
    r = scenes.dam_break_rigid()
    assert r.n == 1048576 and r.nbuckets == 2 ** 21 and r.nspheres == 4096
    assert r.pos[:, :3].min() > 0 and (r.pos[:, :3].max(axis=0) < np.array(r.box_max)).all()


def test_batched_generator():
    ss = scenes.batched_scenes(count=16)
    ns = [s.n for s in ss]
    assert min(ns) >= 2048 and max(ns) <= 65536
    assert all(len(s.bodies) == (i % 2) for i, s in enumerate(ss))
    assert all(s.bodies[0].local.shape[0] == 512 for s in ss if s.bodies)


def _header_enum(prefix):
    text = open(os.path.join(INC, "fluidgrid_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(%s\w*)\s*=\s*(\d+)" % prefix, text)}


def test_option_and_status_codes_match_header():
    opts = _header_enum("FG_OPT_")
    assert opts, "no FG_OPT_ enumerators found"
    assert {"FG_OPT_" + k.upper(): v for k, v in _ffi.OPTIONS.items()} == opts
    status = _header_enum("FG_E_")
    status["FG_OK"] = _header_enum("FG_OK")["FG_OK"]
    assert {v: k for k, v in _ffi.STATUS.items()} == status


def test_run_stage_codes_match_header():
    run = _header_enum("FG_RUN_")
    contact = run.pop("FG_RUN_WITH_CONTACT")
    assert {"FG_RUN_" + k.upper(): v for k, v in _ffi.RUN.items()} == run
    assert contact == _ffi.RUN_WITH_CONTACT
    # the stages are numbered in step order, from 1
    assert sorted(run.values()) == list(range(1, len(run) + 1))


def test_server_config_defaults(lib):
    """The served form admits by HBM budget and by a per-step work budget
    (particles and predicted time), with reservations for the oldest
    request."""
    c = _ffi.fg_server_config()
    lib.fg_server_config_defaults(ctypes.byref(c))
    assert c.hbm_budget_bytes == 120 << 30 and c.use_graphs == 1
    assert c.max_particles == 1200000 and c.target_step_ms == pytest.approx(1.1)
    assert c.head_wait_s == 0.0 and c.pipeline_depth == 0
