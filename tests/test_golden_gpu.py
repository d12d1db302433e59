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


def _narrowphase_inputs(torch, d):
    """The golden's collision-stage state as the narrowphase entry takes it:
    the triangles and ownership bytes in the sorted slot order the
    reference's pairs index, on the device."""
    spec = golden_cases.make_spec(d["case"])
    slot = d["perm_before"].astype(np.int64)[d["ref_order"].astype(np.int64)]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return dict(spec=spec, x=dev(d["x"]), xp=dev(d["x_prev"]), v=dev(d["v"]),
                tris=dev(spec.indices.astype(np.uint32)[slot]), feats=dev(d["features"].astype(np.uint8)[slot]),
                pairs=dev(d["ref_pairs"].astype(np.uint32).reshape(-1, 2)))


@pytest.mark.parametrize("mode", ["ccd", "dcd"])
@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_narrowphase_entry_matches_reference_kernels(cuda, path, mode):
    """lc_narrowphase_run on the reference's pairs of each golden state:
    CreateTriangleTests + CCDTriangleTests (mode ccd) or + DCDTriangleTests
    (mode dcd, the discrete tests of HandleCollisionsDiscrete at x_prev).
    Its VF and EE contacts must be the reference kernels' PrimitiveContact
    records (ids, weights, time, normal) bit for bit, in the same order."""
    torch = cuda
    from licenta_gb300 import Narrowphase, _ffi
    d = golden_cases.load(path)
    a = _narrowphase_inputs(torch, d)
    V, T, P = a["spec"].num_vertices, a["spec"].num_triangles, len(a["pairs"])
    np_ = Narrowphase(V, T, max(P, 1))
    cap = 15 * max(P, 1)
    vf = torch.zeros((cap, 12), dtype=torch.int32, device="cuda")
    ee = torch.zeros((cap, 12), dtype=torch.int32, device="cuda")
    ccd = mode == "ccd"
    try:
        rc, nvf, nee = np_.run(a["x"].data_ptr() if ccd else None, a["xp"].data_ptr(),
                               a["v"].data_ptr() if ccd else None, V, a["tris"].data_ptr(), a["feats"].data_ptr(),
                               T, a["pairs"].data_ptr(), P, float(d["thickness"]), float(d["dt"]), vf.data_ptr(), cap,
                               ee.data_ptr(), cap, mode=_ffi.LC_NARROW_CCD if ccd else _ffi.LC_NARROW_DCD)
        assert rc == 0
        refs = (d["ref_vf"], d["ref_ee"]) if ccd else (d["ref_dcd_vf"], d["ref_dcd_ee"])
        for got, n, ref in ((vf, nvf, refs[0]), (ee, nee, refs[1])):
            assert n == len(ref)
            assert np.array_equal(got[:n].cpu().numpy(), ref.astype(np.int32))
    finally:
        np_.close()


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_impulse_response_entry_matches_reference_kernels(cuda, path):
    """lc_solve_collisions (SolveCollisions: CreateImpulses + ApplyImpulses)
    on each golden state's continuous contacts: positions and velocities
    bit for bit against the reference's kernels."""
    torch = cuda
    import ctypes as C
    from licenta_gb300 import _ffi
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    dev = lambda arr, dt=np.float32: torch.from_numpy(np.ascontiguousarray(arr, dt)).cuda()
    x, xp, v = dev(d["x"]), dev(d["x_prev"]), dev(d["v"])
    fixed = dev(spec.pinned, np.uint8)
    vf = dev(d["ref_vf"].reshape(-1, 12), np.int32)
    ee = dev(d["ref_ee"].reshape(-1, 12), np.int32)
    prm = golden_cases.impulse_params(spec, float(d["thickness"]))
    vp = lambda t: C.c_void_p(t.data_ptr())
    rc = _ffi.lib().lc_solve_collisions(vp(x), vp(xp), vp(v), vp(fixed), spec.num_vertices, vp(vf), len(d["ref_vf"]),
                                        vp(ee), len(d["ref_ee"]), prm["stiffness"], prm["vertex_mass"], prm["dt"],
                                        prm["thickness"], None)
    torch.cuda.synchronize()
    assert rc == 0, _ffi.lib().lc_last_error_string()
    assert np.array_equal(x.cpu().numpy().view(np.uint32), d["ref_impulse_x"].view(np.uint32))
    assert np.array_equal(v.cpu().numpy().view(np.uint32), d["ref_impulse_v"].view(np.uint32))


def test_narrowphase_entry_reports_capacity_and_bad_indices(cuda):
    torch = cuda
    from licenta_gb300 import Narrowphase, _ffi
    d = golden_cases.load(golden_cases.GOLDEN / "cloth48_k06_step45.npz")
    a = _narrowphase_inputs(torch, d)
    V, T, P = a["spec"].num_vertices, a["spec"].num_triangles, len(a["pairs"])
    np_ = Narrowphase(V, T, P)
    n_ee = len(d["ref_ee"])
    assert n_ee > 4
    vf = torch.zeros((len(d["ref_vf"]) + 1, 12), dtype=torch.int32, device="cuda")
    ee = torch.full((n_ee, 12), -3, dtype=torch.int32, device="cuda")
    try:
        # room for half the EE contacts: the first half written, the rest untouched, full count reported
        half = n_ee // 2
        rc, nvf, nee = np_.run(a["x"].data_ptr(), a["xp"].data_ptr(), a["v"].data_ptr(), V, a["tris"].data_ptr(),
                               a["feats"].data_ptr(), T, a["pairs"].data_ptr(), P, float(d["thickness"]),
                               float(d["dt"]), vf.data_ptr(), len(vf), ee.data_ptr(), half)
        assert rc == 3 and nee == n_ee and nvf == len(d["ref_vf"])
        g = ee.cpu().numpy()
        assert np.array_equal(g[:half], d["ref_ee"][:half].astype(np.int32))
        assert np.all(g[half:] == -3)
        # a pair index past the triangle count is reported, not followed
        bad = a["pairs"].clone()
        bad[P // 2, 1] = T
        rc, _, _ = np_.run(a["x"].data_ptr(), a["xp"].data_ptr(), a["v"].data_ptr(), V, a["tris"].data_ptr(),
                           a["feats"].data_ptr(), T, bad.data_ptr(), P, float(d["thickness"]), float(d["dt"]),
                           vf.data_ptr(), len(vf), ee.data_ptr(), n_ee)
        assert rc == 1 and b"out of range" in _ffi.lib().lc_last_error_string()
    finally:
        np_.close()
