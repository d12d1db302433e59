"""Cases of the collision-stage golden vectors (tests/golden/*.npz) and the
comparisons the tests make against them.

Each golden holds a collision-stage input state and what the reference's own
kernels computed from it (tests/golden/make_golden.py).  The layouts follow
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
]


def make_spec(case: dict):
    spec = getattr(scenes, case["scene"])(**case["kw"])
    if case.get("wind"):
        scenes.set_constant_wind(spec.params, tuple(case["wind"]))
    if case.get("mesh_thickness"):
        spec.params.thicknessFromMesh = 1
    return spec


def load(path: Path) -> dict:
    with np.load(path) as z:
        d = {k: z[k] for k in z.files}
    d["case"] = json.loads(str(d["meta"]))
    return d


def golden_files():
    return sorted(GOLDEN.glob("*.npz"))


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
