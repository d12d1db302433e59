"""The oracle against the reference's own kernels (tests/golden/*.npz).

Each golden file holds a collision-stage input state and the outputs of the
reference's collision kernels, compiled from its sources and run on a GPU
(tests/golden/make_golden.py, oracle/ref_pin/).  The FP32 oracle must
reproduce every stage bit for bit: Morton codes, the stable sort, the Karras
hierarchy, the refit boxes and rightmost leaves, the broadphase pairs and the
VF / EE contacts (vertex ids and weights).  The golden files also hold what
the reference's solver kernels (PBDStepSolver, _FinalUpdate) computed from
the same state with those contacts.  The FP32 oracle's solver, which
evaluates the reference's formulas in the reference's order, must agree with
it within golden_cases.SOLVER_ATOL_X on every state.  (Bit equality is not
asked of the solver: the reference's kernels call CUDA's powf and acosf,
whose last-place rounding differs from the host library's.)  The FP64 oracle,
run with the FP32 oracle's discrete decisions, must agree within the same
tolerance on every state whose bends stay away from the reference's d -> 1
singularity (golden_cases.bend_conditioning); windy20_mesh_h_step40 passes
within 1.7e-8 of it and is the case that shows the singularity.
"""
from __future__ import annotations

import numpy as np
import pytest

import golden_cases

FILES = golden_cases.golden_files()


def test_golden_vectors_exist():
    assert len(FILES) >= len(golden_cases.CASES), "tests/golden holds no reference vectors"


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_oracle_matches_reference_kernels(path):
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    assert golden_cases.compare_oracle(spec, d) == []


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_golden_inputs_are_in_reference_layout(path):
    d = golden_cases.load(path)
    T = len(d["perm_before"])
    assert d["ref_node_min"].shape == (2 * T - 1, 3)
    assert d["ref_lefts"].shape == (T - 1,)
    assert np.all(np.diff(d["ref_morton"].astype(np.uint64).astype(object)) >= 0)
    assert sorted(d["ref_order"].tolist()) == list(range(T))


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_oracle_solver_matches_reference_kernels(path):
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    dt = float(d["dt"])
    r = golden_cases.compare_oracle_solver(spec, d)
    tags = ("fp32", "fp64") if golden_cases.well_conditioned(spec, d) else ("fp32",)
    for tag in tags:
        assert r[f"{tag}_dx"] <= golden_cases.SOLVER_ATOL_X, r
        assert r[f"{tag}_dxp"] <= golden_cases.SOLVER_ATOL_X, r
        assert r[f"{tag}_dv"] <= golden_cases.SOLVER_ATOL_X / dt, r
    # most vertices come out bit-identical to the reference's kernels
    assert r["fp32_bitexact"] >= 0.8, r


def test_bend_singularity_is_the_only_excluded_case():
    """Exactly one golden state is excluded from the FP64 comparison, and it
    is excluded because a bend passes within the bound of d = 1."""
    excluded = []
    for path in FILES:
        d = golden_cases.load(path)
        spec = golden_cases.make_spec(d["case"])
        worst, bound = golden_cases.bend_conditioning(spec, d)
        if worst < bound:
            excluded.append((path.stem, worst, bound))
    assert [e[0] for e in excluded] == ["windy20_mesh_h_step40"], excluded
    assert excluded[0][1] < 0.2 * excluded[0][2]


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_oracle_friction_matches_reference_kernels(path):
    """CudaPBD::ApplyFriction: the oracle's restatement (FP32 and FP64) against
    the reference's friction kernels on the same velocities, ground flags and
    VF contacts."""
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    r = golden_cases.compare_oracle_friction(spec, d)
    assert r["fp32_dv"] <= golden_cases.FRICTION_ATOL_V, r
    assert r["fp64_dv"] <= golden_cases.FRICTION_ATOL_V, r


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_oracle_prediction_matches_reference_kernels(path):
    """PBDStepExternal (ApplyExternalForces with gravity and wind,
    DampVelocities' global and rigid-mode damping, ExplicitEuler) and
    UpdateVertexNormals: the oracle (FP32 and FP64) from the golden's
    pre-step state against what the reference's kernels computed from it."""
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    r = golden_cases.compare_oracle_prediction(spec, d)
    dt = float(d["dt"])
    for tag in ("fp32", "fp64"):
        assert r[f"{tag}_dx"] <= golden_cases.PRED_ATOL_X, r
        assert r[f"{tag}_dv"] <= golden_cases.PRED_ATOL_X / dt, r
        assert r[f"{tag}_dvn"] <= golden_cases.VN_ATOL, r
    # the step did change the velocities (gravity alone adds 9.81 / 60 m/s)
    assert r["changed_dv"] > 0.1, r


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_golden_prediction_is_the_collision_input(path):
    """The collision stages' input of every golden is the reference's own
    prediction: x = x_prev + dt v as ExplicitEuler rounds it (no fused
    multiply-add), from the pre-step state with gravity and damping on."""
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    p = spec.params
    assert p.kDamp > 0 and p.globalVelDamp > 0 and p.gravity[1] < 0
    dt = np.float32(d["dt"])
    want = (d["x_prev"] + (dt * d["v"]).astype(np.float32)).astype(np.float32)
    assert np.array_equal(want.view(np.uint32), d["x"].view(np.uint32))
    assert np.array_equal(d["x_prev"], d["pre_x_prev"])


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_oracle_contact_records_and_response_match_reference_kernels(path):
    """The oracle's full PrimitiveContact records (ids, weights, time, normal)
    from the continuous tests (CCDTriangleTests) and the discrete tests
    (DCDTriangleTests of HandleCollisionsDiscrete) on the reference's pairs,
    and its impulse response (SolveCollisions: CreateImpulses +
    ApplyImpulses) on the reference's contacts, against the reference's
    kernels, bit for bit."""
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    r = golden_cases.compare_oracle_response(spec, d)
    assert r["ccd_records_equal"] and r["dcd_records_equal"], r
    assert r["impulse_dx"] == 0.0 and r["impulse_dv"] == 0.0, r
