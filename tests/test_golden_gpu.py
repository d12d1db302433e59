"""The CUDA engine against the reference's own kernels (tests/golden/*.npz).

Prediction: the engine is put in the golden's pre-step state (positions,
previous positions, velocities, running vertex normals, triangle order) with
the case's gravity, damping and wind, and steps once.  Its predicted
positions and velocities must agree with the reference's PBDStepExternal
kernels within golden_cases.PRED_ATOL_X (1e-5 m; 1e-5 m / dt on
velocities) and its running vertex normals with the reference's
UpdateVertexNormals within golden_cases.VN_ATOL.

Collision stages and solver: the engine is put in the golden's
collision-stage input state (the reference's prediction): gravity, damping
and wind are switched off so that its prediction x = x_prev + dt v
reproduces the golden's predicted positions bit for bit, and the triangle
order is set to the golden's pre-sort order.  One step later its Morton
codes, sorted order, hierarchy, refit boxes, rightmost leaves, pairs and
VF / EE contacts must equal the reference's bit for bit, and its positions
and velocities after the solver, the velocity update and the world clamp
must agree with what the reference's solver kernels computed from the same
state within golden_cases.SOLVER_ATOL_X (1e-5 m; 1e-5 m / dt on velocities)
on every state whose bends stay away from the reference's d -> 1
singularity (golden_cases.bend_conditioning).  With useFriction the
velocities are compared with the reference's friction kernels' output.
"""
from __future__ import annotations

import numpy as np
import pytest

import golden_cases
from licenta_gb300 import ClothBatch

pytestmark = pytest.mark.gpu

FILES = golden_cases.golden_files()


@pytest.mark.parametrize("friction", [False, True], ids=["plain", "friction"])
@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_engine_matches_reference_kernels(path, friction):
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    p = spec.params
    p.useFriction = 1 if friction else 0
    p.gravity[:] = (0.0, 0.0, 0.0)
    p.kDamp = 0.0
    p.globalVelDamp = 0.0
    p.windOn = 0
    b = ClothBatch([spec], debug_capture=True)
    try:
        assert np.array_equal(b.debug(0, "FEATURES"), d["features"])
        b.set_state(0, x=d["x_prev"], x_prev=d["x_prev"], v=d["v"])
        b.set_triangle_order(0, d["perm_before"])
        b.step(1)
        b.sync()
        assert np.array_equal(b.debug(0, "PRED_X").view(np.uint32), d["x"].view(np.uint32))
        assert np.array_equal(b.debug(0, "PERM_BEFORE"), d["perm_before"].astype(np.uint32))
        assert golden_cases.diff(lambda name: b.debug(0, name), d) == []
        st = b.get_state(0)
        assert np.isfinite(st["x"]).all() and np.isfinite(st["v"]).all()
        if not golden_cases.well_conditioned(spec, d):
            return
        dt = float(d["dt"])
        dx = np.abs(st["x"] - d["ref_solve_x_end"]).max()
        dv = np.abs(st["v"] - d["ref_friction_v" if friction else "ref_solve_v"]).max()
        assert dx <= golden_cases.SOLVER_ATOL_X, dx
        assert dv <= golden_cases.SOLVER_ATOL_X / dt, dv
    finally:
        b.close()


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_engine_prediction_matches_reference_kernels(path):
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    p = spec.params
    # the engine's wind state starts at startWindDir: the goldens use a
    # constant wind (zero variation) or none
    assert not p.windOn or (p.windMinVariation == 0.0 and p.windMaxVariation == 0.0)
    b = ClothBatch([spec], debug_capture=True)
    try:
        b.set_state(0, x=d["pre_x"], x_prev=d["pre_x_prev"], v=d["pre_v"], vn=d["pre_vn"])
        b.set_triangle_order(0, d["perm_before"])
        b.step(1)
        b.sync()
        dt = float(d["dt"])
        dx = np.abs(b.debug(0, "PRED_X") - d["x"]).max()
        dv = np.abs(b.debug(0, "PRED_V") - d["v"]).max()
        dvn = np.abs(b.get_state(0)["vn"] - d["ref_vn"]).max()
        assert np.array_equal(b.debug(0, "PRED_XPREV"), d["x_prev"])
        assert dx <= golden_cases.PRED_ATOL_X, dx
        assert dv <= golden_cases.PRED_ATOL_X / dt, dv
        assert dvn <= golden_cases.VN_ATOL, dvn
    finally:
        b.close()
