"""Precision form (4,194,304 particles, a 10% gaussian jet, eight bodies with
rigid/rigid contact): FP32 forces with Kahan density sums, FP64 body
force/torque reduction and integration on the GPU, compared at steps 1, 10
and 100 with the FP64 oracle from the identical state the GPU started that
step from.  Each step's per-quantity errors are checked against the stated
bounds and written as JSON to $FG_PRECISION_REPORT when that is set.

Bounds (per step, from an identical state):
  density   max |rho - rho64| / rho64                        <= 1e-5
  forces    max |F - F64| / max(|F64|, median |F64|)          <= 2e-4
  body F/T  max |S - S64| / max(|S64|, 1e-3 * max |S64|)      <= 1e-4
  sphere F/T per sphere against the FP32 oracle, same scaling <= 1e-4
  body x,q  max |x - x64| (m, unitless)                       <= 1e-6
            (the GPU integrates FP64 sums of FP32 per-sphere forces, the
            oracle FP64 sums of FP64 per-sphere forces; ~1e-5 relative in the
            force moves a body ~1e-7 m in one step)
"""
import json
import os

import numpy as np
import pytest

from fluidgrid_gb300 import World, build, scenes
import helpers as T

pytestmark = pytest.mark.gpu

BEFORE = T.BEFORE_STEP
AFTER = T.AFTER_STEP


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def test_precision_form_against_fp64_oracle():
    spec = scenes.precision_jet()
    w = World([spec])
    report = {"workload": spec.name, "particles": spec.n, "bodies": len(spec.bodies),
              "rigid_spheres": spec.nspheres, "steps": {}}
    done = 0
    for k in (1, 10, 100):
        if k - 1 > done:
            w.step(k - 1 - done)
            done = k - 1
        pos0, v0 = w.download()
        before = {n: w.read(n) for n in BEFORE}
        diag0 = w.diagnostics()[0]
        w.step(1)
        done += 1
        g = {n: w.read(n) for n in AFTER}
        e = T.two_way_step_errors(spec, pos0, v0, before, g)
        diag1 = w.diagnostics()[0]
        e["fp64_momentum_change"] = [diag1[c] - diag0[c] for c in ("px", "py", "pz")]
        e["fp64_mass"] = diag1["mass"]
        report["steps"][str(k)] = e
        assert e["density_rel_max"] <= 1e-5, (k, e)
        assert e["force_rel_max"] <= 2e-4, (k, e)
        assert e["body_force_rel_max"] <= 1e-4 and e["body_torque_rel_max"] <= 1e-4, (k, e)
        assert e["sphere_force_rel_max"] <= 1e-4 and e["sphere_torque_rel_max"] <= 1e-4, (k, e)
        assert e["body_pos_abs_max_m"] <= 1e-6 and e["body_quat_abs_max"] <= 1e-6, (k, e)
        assert diag1["mass"] == diag0["mass"]  # no particle is created or lost
    w.close()
    out = os.environ.get("FG_PRECISION_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)
