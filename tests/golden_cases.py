"""Cases of the golden vectors (tests/golden/*.npz) and the comparisons the
tests make against them.

Each golden holds a state before one step and what the reference's own
kernels computed from it (tests/golden/make_golden.py): the prediction
(predicted positions and velocities, which are also the collision stages'
input), the running vertex normals, the collision stages, the solver and
friction.  The layouts follow
the reference: node arrays of 2T-1 entries with the leaves at T-1+slot
(Collision/CudaBVH.cu:128-149), pairs as (leaf slot, leaf slot)
(Collision/CudaBVH.cu:71,85), contacts as PrimitiveContact {v1..v4,
w1..w4, t, n} (Physics/Structs.h:106-129).
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from licenta_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"

# name, scene, scene kwargs, oracle steps before the captured step, extras
CASES = [
    dict(name="small32_step0", scene="small_cloth", kw=dict(seed=0), steps=0),
    dict(name="small32_step58", scene="small_cloth", kw=dict(seed=0), steps=58),
    dict(name="small32_step80", scene="small_cloth", kw=dict(seed=0), steps=80),
    dict(name="windy20_mesh_h_step40", scene="small_cloth", kw=dict(seed=5, n=20), steps=40,
         wind=(1.5, 0.0, -1.0), mesh_thickness=True),
    dict(name="cloth48_k06_step45", scene="small_cloth", kw=dict(seed=9, n=48, stiffness=0.6), steps=45,
         wind=(-1.2, 0.0, 0.8)),
    # an unpinned cloth that has landed on the ground (ground constraints)
    dict(name="ground24_step16", scene="small_cloth", kw=dict(seed=3, n=24), steps=16, unpin=True,
         world_min_y=0.9),
    # an unpinned cloth draped over the analytic sphere
    dict(name="sphere24_step22", scene="small_cloth", kw=dict(seed=4, n=24), steps=22, unpin=True,
         sphere=((0.5, 0.7, 0.5), 0.2)),
    # triangle bending instead of the dihedral bends, folded onto itself
    dict(name="tribend28_step139", scene="small_cloth", kw=dict(seed=12, n=28), steps=139, tri_bend=True),
]


def make_spec(case: dict):
    spec = getattr(scenes, case["scene"])(**case["kw"])
    if case.get("wind"):
        scenes.set_constant_wind(spec.params, tuple(case["wind"]))
    if case.get("mesh_thickness"):
        spec.params.thicknessFromMesh = 1
    if case.get("tri_bend"):
        spec.params.useTriangleBending = 1
    if case.get("unpin"):
        spec.pinned[:] = 0
    if case.get("world_min_y") is not None:
        spec.params.worldMin[1] = case["world_min_y"]
    if case.get("sphere"):
        centre, radius = case["sphere"]
        spec.params.sphereOn = 1
        spec.params.spherePos[:] = centre
        spec.params.sphereRadius = radius
    return spec


def load(path: Path) -> dict:
    with np.load(path) as z:
        d = {k: z[k] for k in z.files}
    d["case"] = json.loads(str(d["meta"]))
    return d


def golden_files():
    return sorted(GOLDEN.glob("*.npz"))


def masses(spec) -> np.ndarray:
    """Per-vertex masses as the reference's body sets them
    (Physics/CudaDeformableBody.cpp:52,80-82): objectMass over the vertex
    count, 1000 for a pinned vertex."""
    p = spec.params
    m = np.full(spec.num_vertices, np.float32(p.objectMass) / np.float32(spec.num_vertices), np.float32)
    m[np.asarray(spec.pinned) != 0] = np.float32(1000.0)
    return m


# Tolerances of the prediction comparisons: 1e-5 m on positions (the parity
# bar), 1e-5 m / dt on velocities (a position difference over one timestep)
# and 1e-5 on the unit running vertex normals, which the reference sums with
# float atomics in the GPU's order.
PRED_ATOL_X = 1e-5
VN_ATOL = 1e-5


def compare_oracle_prediction(spec, d: dict) -> dict:
    """Largest differences between the oracle's prediction (PBDStepExternal:
    external forces, damping, explicit Euler; FP32 and FP64) and the
    reference kernels' from the same pre-step state, and between the
    oracle's running vertex normals and the reference's on the reference's
    predicted positions."""
    from oracle.oracle_ffi import Oracle
    out = {}
    for fp64 in (False, True):
        tag = "fp64" if fp64 else "fp32"
        o = Oracle([spec], fp64=fp64)
        try:
            o.set_state(0, x=d["pre_x"], x_prev=d["pre_x_prev"], v=d["pre_v"], vn=d["pre_vn"])
            o.set_wind(0, d["pre_wind"], int(d["pre_rng"]))
            o.external(0)
            st = o.get_state(0)
            out[f"{tag}_dx"] = float(np.abs(st["x"] - d["x"]).max())
            out[f"{tag}_dv"] = float(np.abs(st["v"] - d["v"]).max())
            o.set_state(0, x=d["x"], x_prev=d["x_prev"], v=d["v"], vn=d["pre_vn"])
            o.set_perm(0, d["perm_before"])
            o.collide(0)
            out[f"{tag}_dvn"] = float(np.abs(o.get_state(0)["vn"] - d["ref_vn"]).max())
        finally:
            o.close()
    out["changed_dv"] = float(np.abs(d["v"] - d["pre_v"]).max())
    return out


def impulse_params(spec, h: float) -> dict:
    """The arguments SolveCollisions passes (Physics/CudaDeformableBody.cpp:
    527-535): stiffness kStretch, the vertex mass objectMass / (dims.x
    dims.y), the timestep and the thickness."""
    p = spec.params
    return dict(stiffness=float(p.kStretch),
                vertex_mass=float(np.float32(p.objectMass) / np.float32(int(p.dims[0]) * int(p.dims[1]))),
                dt=float(p.timestep), thickness=float(h))


def slot_order(d: dict) -> np.ndarray:
    """Original triangle of each sorted slot: the triangle order the
    reference's pairs index."""
    return d["perm_before"].astype(np.int64)[d["ref_order"].astype(np.int64)]


def compare_oracle_response(spec, d: dict) -> dict:
    """The oracle's impulse response (SolveCollisions) and its full contact
    records (continuous and discrete tests on the golden's pairs) against
    the reference's: largest position / velocity differences and whether
    every record (ids, weights, time, normal) is identical."""
    from oracle.oracle_ffi import narrow_contacts, solve_collisions
    h = float(d["thickness"])
    x, v = solve_collisions(d["x"], d["x_prev"], d["v"], spec.pinned, d["ref_vf"], d["ref_ee"],
                            **impulse_params(spec, h))
    slot = slot_order(d)
    tris, feats = spec.indices[slot], d["features"][slot]
    out = dict(impulse_dx=float(np.abs(x - d["ref_impulse_x"]).max()),
               impulse_dv=float(np.abs(v - d["ref_impulse_v"]).max()))
    for mode, tag, kv, ke in ((0, "ccd", "ref_vf", "ref_ee"), (1, "dcd", "ref_dcd_vf", "ref_dcd_ee")):
        vf, ee = narrow_contacts(mode, d["x"], d["x_prev"], d["v"], tris, feats, d["ref_pairs"], h, float(d["dt"]))
        out[f"{tag}_records_equal"] = bool(np.array_equal(vf, d[kv].astype(np.int32))
                                            and np.array_equal(ee, d[ke].astype(np.int32)))
    return out


def solver_inputs(spec, d: dict, oracle) -> dict:
    """Arguments of the reference's solver chain (refchain.RefKernels.solve)
    for the golden's state: the oracle's topology and the cloth's parameters."""
    p = spec.params
    sphere = ((tuple(p.spherePos), float(p.sphereRadius)) if p.sphereOn else None)
    return dict(topo=oracle.topology(0), iterations=int(p.solverIterations), k_stretch=float(p.kStretch),
                k_bend=float(p.kBend), thickness=float(d["thickness"]), ground_y=float(p.worldMin[1]),
                dt=float(p.timestep), sphere=sphere, world=(tuple(p.worldMin), tuple(p.worldMax)))


def expected(d: dict) -> dict:
    """The reference's outputs in the engine's debug layouts."""
    perm = d["perm_before"].astype(np.int64)
    order = d["ref_order"].astype(np.int64)
    nodes = np.concatenate([d["ref_node_min"], d["ref_node_max"]], axis=1)
    vf, ee = d["ref_vf"].astype(np.int32), d["ref_ee"].astype(np.int32)
    return dict(
        MORTON=d["ref_morton"].astype(np.uint64),
        PERM=perm[order].astype(np.uint32),
        LEFTS=d["ref_lefts"].astype(np.int32),
        RIGHTS=d["ref_rights"].astype(np.int32),
        # the root's entry is never written by the reference (zero there)
        PARENTS=d["ref_parents"].astype(np.int32)[1:],
        RML=np.stack([d["ref_rmll"], d["ref_rmlr"]], axis=1).astype(np.int32),
        NODE_AABB=nodes.astype(np.float32),
        PAIRS=d["ref_pairs"].astype(np.uint32),
        VF=(vf[:, :4], vf[:, 4:8].view(np.float32)),
        EE=(ee[:, :4], ee[:, 4:8].view(np.float32)),
    )


def _as(name, a):
    a = np.asarray(a)
    if name == "PARENTS":
        return a.astype(np.int32)[1:]
    if name == "RML":
        return a.reshape(-1, 2).astype(np.int32)
    if name == "NODE_AABB":
        return a.reshape(-1, 6).astype(np.float32)
    if name == "PAIRS":
        return a.reshape(-1, 2).astype(np.uint32)
    if name == "MORTON":
        return a.astype(np.uint64)
    if name == "PERM":
        return a.astype(np.uint32)
    return a.astype(np.int32)


def diff(get, d: dict) -> list[str]:
    """Names of the stages where `get(name)` differs from the golden."""
    exp = expected(d)
    out = []
    for name, want in exp.items():
        got = get(name)
        if name in ("VF", "EE"):
            gv, gw = got
            wv, ww = want
            gv = np.asarray(gv).reshape(-1, 4).astype(np.int32)
            gw = np.asarray(gw).reshape(-1, 4).astype(np.float32)
            if gv.shape != wv.shape or not np.array_equal(gv, wv) or not np.array_equal(gw.view(np.uint32),
                                                                                         ww.view(np.uint32)):
                out.append(f"{name}({len(gv)} vs {len(wv)})")
            continue
        got = _as(name, got)
        if name == "NODE_AABB":
            same = got.shape == want.shape and np.array_equal(got.view(np.uint32), want.view(np.uint32))
        else:
            same = got.shape == want.shape and np.array_equal(got, want)
        if not same:
            out.append(name)
    return out


def oracle_refit(spec, d: dict) -> dict:
    """The FP32 oracle's internal-node boxes and rightmost leaves on the
    golden input (the seed of the reference's refit, see refchain.collide)."""
    from oracle.oracle_ffi import Oracle
    o = Oracle([spec], fp64=False)
    try:
        o.set_state(0, x=d["x"], x_prev=d["x_prev"], v=d["v"])
        o.set_perm(0, d["perm_before"])
        o.collide(0)
        na = o.debug(0, "NODE_AABB").reshape(-1, 6)
        rml = o.debug(0, "RML").reshape(-1, 2)
        return dict(node_min=na[:, :3].copy(), node_max=na[:, 3:].copy(), rmll=rml[:, 0].copy(),
                    rmlr=rml[:, 1].copy())
    finally:
        o.close()


def compare_oracle(spec, d: dict) -> list[str]:
    """Run the FP32 oracle's collision stages on the golden input."""
    from oracle.oracle_ffi import Oracle
    o = Oracle([spec], fp64=False)
    try:
        feats = o.debug(0, "FEATURES")
        if not np.array_equal(feats, d["features"]):
            return ["FEATURES"]
        o.set_state(0, x=d["x"], x_prev=d["x_prev"], v=d["v"])
        o.set_perm(0, d["perm_before"])
        o.collide(0)
        return diff(lambda name: o.debug(0, name), d)
    finally:
        o.close()


# Tolerance of the solver comparisons: 1e-5 m on positions (the parity bar of
# the solver against the FP64 restatement); velocities are position
# differences over one timestep, so theirs is 1e-5 m / dt.
SOLVER_ATOL_X = 1e-5


def oracle_solve(spec, d: dict, fp64: bool, forced: dict | None = None):
    """The oracle's solver iterations and velocity update on the golden's
    predicted state with the reference's contacts, optionally with imposed
    decisions: (x, v, x_prev, the decisions taken)."""
    from oracle.oracle_ffi import Oracle
    o = Oracle([spec], fp64=fp64)
    try:
        vf = (d["ref_vf"][:, :4], d["ref_vf"][:, 4:8].view(np.float32))
        ee = (d["ref_ee"][:, :4], d["ref_ee"][:, 4:8].view(np.float32))
        x, v, xp = o.solve_on(0, d["x"], d["x_prev"], vf, ee, forced=forced)
        return x, v, xp, o.solve_decisions(0)
    finally:
        o.close()


DECISIONS = ("ground", "ground_it", "lra", "dyn", "sphere")


def decision_diff(a: dict, b: dict) -> int:
    """How many discrete decisions differ between two solves of one state."""
    n = 0
    for k in DECISIONS:
        x, y = np.asarray(a[k]).ravel(), np.asarray(b[k]).ravel()
        if x.shape != y.shape:
            return -1
        if k == "ground_it":
            n += int(np.unpackbits((x ^ y).view(np.uint8)).sum())
        else:
            n += int(np.count_nonzero(x != y))
    return n


def bend_conditioning(spec, d: dict) -> tuple[float, float]:
    """(smallest 1 - d over every bend and solver iterate, the smallest value
    at which positions are still comparable within SOLVER_ATOL_X).

    d = n1 . n2 is the cosine of the reference's bend angle on the raw
    positions (Physics/CudaPBD.cu:1035-1058).  As d -> 1 its correction is
    0 * inf: sqrt(1 - d^2) (phi - phi0) over a scale factor that vanishes like
    1 - d, applied along vectors of size sqrt(1 - d).  A float rounding of the
    unit normals (eps = 2^-24) then moves the correction by about
    L eps / sqrt(1 - d) for edges of length L, so two correct FP32
    implementations, or FP32 and FP64, agree within the tolerance only while
    1 - d >= (L eps / tol)^2.  The iterates are the FP32 oracle's, which
    follow the reference's formulas."""
    from oracle.oracle_ffi import Oracle
    o = Oracle([spec], fp64=False)
    try:
        vf = (d["ref_vf"][:, :4], d["ref_vf"][:, 4:8].view(np.float32))
        ee = (d["ref_ee"][:, :4], d["ref_ee"][:, 4:8].view(np.float32))
        o.solve_on(0, d["x"], d["x_prev"], vf, ee)
        t = o.topology(0)
        b = t["b"]
        worst = np.inf
        # triangle bends have no dihedral angle, hence no such singularity
        for k in range(0 if t["tri_bend"] else int(spec.params.solverIterations)):
            x = o.solve_iterate(0, k).astype(np.float64)
            c23 = np.cross(x[b[:, 1]], x[b[:, 2]])
            c24 = np.cross(x[b[:, 1]], x[b[:, 3]])
            n1 = c23 / np.linalg.norm(c23, axis=1, keepdims=True)
            n2 = c24 / np.linalg.norm(c24, axis=1, keepdims=True)
            worst = min(worst, float((1.0 - (n1 * n2).sum(axis=1)).min()))
        edge = float(np.max(t["sl0"]))
        return worst, (edge * 2.0 ** -24 / SOLVER_ATOL_X) ** 2
    finally:
        o.close()


def well_conditioned(spec, d: dict) -> bool:
    worst, bound = bend_conditioning(spec, d)
    return worst >= bound


def compare_oracle_solver(spec, d: dict) -> dict:
    """Largest differences between the oracle's solver and the reference's,
    on positions after the iterations and on velocities.

    The FP32 oracle runs on its own decisions; the share of vertices on which
    it agrees with the reference bit for bit is reported.  The FP64 oracle
    runs with the FP32 oracle's decisions imposed: the Jacobi update divides
    by the number of non-zero corrections, so a threshold that FP32 and FP64
    decide differently (a contact or a ground plane the previous step left at
    exactly the thickness) moves a vertex by a finite amount."""
    out = {}
    x, v, xp, dec32 = oracle_solve(spec, d, False)
    for fp64 in (False, True):
        if fp64:
            x, v, xp, _ = oracle_solve(spec, d, True, forced=dec32)
        tag = "fp64" if fp64 else "fp32"
        out[f"{tag}_dx"] = float(np.abs(x - d["ref_solve_x"]).max())
        out[f"{tag}_dv"] = float(np.abs(v - d["ref_solve_v"]).max())
        out[f"{tag}_dxp"] = float(np.abs(xp - d["ref_solve_x_prev"]).max())
        if not fp64:
            same = np.all(x.view(np.uint32) == d["ref_solve_x"].view(np.uint32), axis=1)
            out["fp32_bitexact"] = float(same.mean())
    return out


# Friction changes velocities only; from the same inputs the oracle and the
# reference's kernels differ by roundings (CUDA's powf against the host's).
FRICTION_ATOL_V = 1e-5


def compare_oracle_friction(spec, d: dict) -> dict:
    """Largest velocity differences between the oracle's friction (FP32, FP64)
    and the reference's friction kernels, on the reference solver's
    velocities, ground flags and VF contacts (with their normals)."""
    from oracle.oracle_ffi import Oracle
    vf = d["ref_vf"]
    ids, w = vf[:, :4], vf[:, 4:8].view(np.float32)
    normals = np.ascontiguousarray(vf[:, 9:12]).view(np.float32)
    out = {}
    for fp64 in (False, True):
        o = Oracle([spec], fp64=fp64)
        try:
            v = o.friction_on(0, d["ref_solve_v"], d["ref_ground"], (ids, w), normals)
        finally:
            o.close()
        out["fp64_dv" if fp64 else "fp32_dv"] = float(np.abs(v - d["ref_friction_v"]).max())
    out["changed"] = float(np.abs(d["ref_friction_v"] - d["ref_solve_v"]).max())
    return out
