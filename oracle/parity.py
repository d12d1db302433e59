"""Teacher-forced parity of the CUDA engine against the oracle.

TEST INFRASTRUCTURE ONLY (used by tests/ and __graft_entry__.smoke()).

One step of one cloth is checked in two ways:

* collision stages, bit-exact: the FP32 mirror re-runs the collision pipeline
  on the GPU's own predicted positions and must reproduce the GPU's Morton
  codes, sorted order, hierarchy, refit boxes, pairs and VF/EE contacts;
* positions, within a tolerance: the FP64 oracle starts from the GPU's
  pre-step state and replays the GPU's discrete decisions for the step (the
  contact set, ground / LRA / sphere activation and which terms were counted
  in each Jacobi iteration), so the comparison measures the continuous
  arithmetic only.  The reference's update divides by the number of non-zero
  corrections, so a decision taken differently by FP32 and FP64 near a
  threshold would otherwise move a vertex by a finite amount.
"""
from __future__ import annotations

import numpy as np

COLLISION_ARRAYS = ("MORTON", "PERM", "LEFTS", "RIGHTS", "PARENTS", "RML", "NODE_AABB", "PAIRS")


# A step's solve is near a singularity of the reference's raw-position bend
# formula when a hinge comes within 1 - n1.n2 < SINGULAR_FWD of d = 1 (the
# correction is 0 * inf there, in the forward step as in its derivative) or
# within 1 + n1.n2 < SINGULAR_NEG of d = -1 (the correction is a 0 / 0 ratio
# whose derivative grows like (1 + d)^-1/2).  Reverse-pass comparisons excuse
# such steps.
SINGULAR_FWD = 1e-7
SINGULAR_NEG = 1e-11


def capture_pre(batch, c):
    st = batch.get_state(c)
    return st, batch.triangle_order(c)


def check_collision(batch, c, o32, pre_vn, tag=""):
    """FP32 mirror on the GPU's predicted state; raises on the first mismatch."""
    o32.set_state(0, x=batch.debug(c, "PRED_X"), x_prev=batch.debug(c, "PRED_XPREV"), v=batch.debug(c, "PRED_V"),
                  vn=pre_vn)
    o32.set_perm(0, batch.debug(c, "PERM_BEFORE"))
    o32.collide(0)
    for what in COLLISION_ARRAYS:
        g, r = batch.debug(c, what), o32.debug(0, what)
        if g.shape != r.shape or not np.array_equal(g, r):
            raise AssertionError(f"{tag}: {what} differs")
    n = 0
    for what in ("VF", "EE"):
        (gv, gw), (rv, rw) = batch.debug(c, what), o32.debug(0, what)
        if not (np.array_equal(gv, rv) and np.array_equal(gw, rw)):
            raise AssertionError(f"{tag}: {what} contacts differ ({len(gv)} vs {len(rv)})")
        n += len(gv)
    if getattr(batch.specs[c], "collider", None) is not None:
        (gv, gw), (rv, rw) = batch.debug(c, "COLLIDER"), o32.debug(0, "COLLIDER")
        if not (np.array_equal(gv, rv) and np.array_equal(gw, rw)):
            raise AssertionError(f"{tag}: collider contacts differ ({int((gv[:, 1] >= 0).sum())} vs "
                                 f"{int((rv[:, 1] >= 0).sum())})")
        n += int((gv[:, 1] >= 0).sum())
    return n


def fp64_step_error(batch, c, o64, pre, perm, sphere: bool, friction: bool = False):
    """Max |x_gpu - x_fp64| (metres) after the step the batch just took."""
    o64.set_state(0, **{k: v.astype(np.float64) for k, v in pre.items()})
    o64.set_perm(0, perm)
    vf, ee = batch.debug(c, "VF"), batch.debug(c, "EE")
    o64.freeze_contacts(0, vf, ee, batch.debug(c, "VF_NORMAL") if friction else None)
    o64.force_decisions(0, batch.debug(c, "GROUND"), batch.debug(c, "GROUND_ACTIVE"), batch.debug(c, "LRA"),
                        batch.debug(c, "DYN_ACTIVE"), batch.debug(c, "SPHERE") if sphere else None)
    if getattr(batch.specs[c], "collider", None) is not None:
        o64.freeze_collider(0, batch.debug(c, "COLLIDER"))
    o64.step_one(0)
    g = batch.get_state(c)
    r = o64.get_state(0)
    for k in ("x", "x_prev", "v"):
        if not np.isfinite(g[k]).all():
            raise AssertionError(f"non-finite {k}")
    return float(np.abs(g["x"] - r["x"]).max()), float(np.abs(g["v"] - r["v"]).max())


def conditioning_bound(spec, tol: float) -> float:
    """The smallest 1 - n1.n2 of a bend at which the reference's bend
    correction is still determined within `tol` by FP32 arithmetic: near
    d = 1 it is 0 * inf, and one rounding of the unit normals moves it by
    about L 2^-24 / sqrt(1 - d) for edges of length L."""
    p = np.asarray(spec.positions, np.float64)
    idx = np.asarray(spec.indices, np.int64).reshape(-1, 3)
    L = max(float(np.linalg.norm(p[idx[:, a]] - p[idx[:, b]], axis=1).max()) for a, b in ((0, 1), (1, 2), (2, 0)))
    return (L * 2.0 ** -24 / tol) ** 2


def run_parity(specs, steps, check_every=1, variant=0, friction=False, contact_gather=0, tol=1e-5):
    """Steps `specs` as one batch for `steps` steps, checking every step of
    every cloth against the oracle: collision stages bit-exact (every
    `check_every` steps) and positions within `tol` of the FP64 oracle,
    teacher-forced.  A step that misses `tol` is excused only if a bend of
    it passed within rounding of the reference's d -> 1 singularity, and at
    most one step in twenty may be.  Returns (worst position error,
    contacts checked, excused steps, steps checked)."""
    from licenta_gb300 import ClothBatch
    from oracle.oracle_ffi import Oracle
    batch = ClothBatch(specs, debug_capture=True, solver_variant=variant)
    if contact_gather:
        from licenta_gb300 import autotune
        cfg = autotune.get_tuning(batch)
        cfg["contact_gather"] = contact_gather
        assert autotune.set_tuning(batch, cfg)
    o32 = [Oracle([s], fp64=False) for s in specs]
    o64 = [Oracle([s], fp64=True) for s in specs]
    for o in o64:
        o.track_bend(0)
    bound = [conditioning_bound(s, tol) for s in specs]
    worst = 0.0
    contacts = 0
    singular = 0
    try:
        for step in range(steps):
            pre = [capture_pre(batch, c) for c in range(len(specs))]
            batch.step(1)
            batch.sync()
            for c, s in enumerate(specs):
                if step % check_every == 0:
                    contacts += check_collision(batch, c, o32[c], pre[c][0]["vn"], tag=f"cloth {c} step {step}")
                err, err_v = fp64_step_error(batch, c, o64[c], pre[c][0], pre[c][1], bool(s.params.sphereOn),
                                             friction)
                if err > tol and o64[c].bend_conditioning(0) < bound[c]:
                    # a bend passed the reference's d -> 1 singularity: the
                    # step's result is set by rounding, not by the scheme
                    singular += 1
                    continue
                worst = max(worst, err)
                assert err <= tol, f"cloth {c} step {step}: |x - x_fp64| = {err:.3e}"
                if friction:  # friction changes velocities only
                    assert err_v <= tol / s.params.timestep, f"cloth {c} step {step}: |v - v_fp64| = {err_v:.3e}"
    finally:
        batch.close()
        for o in o32 + o64:
            o.close()
    assert singular <= max(1, steps * len(specs) // 20), f"{singular} steps near the bend singularity"
    return worst, contacts, singular, steps * len(specs)


def check_all_cloths(batch, specs, o32, o64, pre, tol=1e-5):
    """One step of every cloth of a batch that was just stepped, against the
    oracle: collision stages bit-exact (the FP32 mirror on the GPU's
    predicted state, all cloths in parallel) and positions teacher-forced
    against the FP64 oracle (the GPU's pre-step state, contacts and
    decisions, all cloths in parallel).  pre: capture_pre of every cloth
    before the step; o32, o64: oracles over the same specs, o64 with
    track_bend on.  Returns dict(worst, excused, contacts, pairs); raises on
    a collision mismatch or a position error above tol on a step that no bend
    singularity excuses."""
    n = len(specs)
    for c in range(n):
        o32.set_state(c, x=batch.debug(c, "PRED_X"), x_prev=batch.debug(c, "PRED_XPREV"),
                      v=batch.debug(c, "PRED_V"), vn=pre[c][0]["vn"])
        o32.set_perm(c, batch.debug(c, "PERM_BEFORE"))
    o32.collide_all()
    contacts = pairs = 0
    for c in range(n):
        for what in COLLISION_ARRAYS:
            g, r = batch.debug(c, what), o32.debug(c, what)
            if g.shape != r.shape or not np.array_equal(g, r):
                raise AssertionError(f"cloth {c}: {what} differs")
        pairs += len(batch.debug(c, "PAIRS"))
        for what in ("VF", "EE"):
            (gv, gw), (rv, rw) = batch.debug(c, what), o32.debug(c, what)
            if not (np.array_equal(gv, rv) and np.array_equal(gw, rw)):
                raise AssertionError(f"cloth {c}: {what} contacts differ ({len(gv)} vs {len(rv)})")
            contacts += len(gv)
        if getattr(specs[c], "collider", None) is not None:
            (gv, gw), (rv, rw) = batch.debug(c, "COLLIDER"), o32.debug(c, "COLLIDER")
            if not (np.array_equal(gv, rv) and np.array_equal(gw, rw)):
                raise AssertionError(f"cloth {c}: collider contacts differ ({int((gv[:, 1] >= 0).sum())} vs "
                                     f"{int((rv[:, 1] >= 0).sum())})")
            contacts += int((gv[:, 1] >= 0).sum())
    for c, s in enumerate(specs):
        st, perm = pre[c]
        o64.set_state(c, **{k: v.astype(np.float64) for k, v in st.items()})
        o64.set_perm(c, perm)
        o64.freeze_contacts(c, batch.debug(c, "VF"), batch.debug(c, "EE"))
        o64.force_decisions(c, batch.debug(c, "GROUND"), batch.debug(c, "GROUND_ACTIVE"), batch.debug(c, "LRA"),
                            batch.debug(c, "DYN_ACTIVE"), batch.debug(c, "SPHERE") if s.params.sphereOn else None)
        if getattr(s, "collider", None) is not None:
            o64.freeze_collider(c, batch.debug(c, "COLLIDER"))
    o64.step_frozen_all()
    worst, excused = 0.0, 0
    for c, s in enumerate(specs):
        g = batch.get_state(c)
        if not np.isfinite(g["x"]).all():
            raise AssertionError(f"cloth {c}: non-finite positions")
        err = float(np.abs(g["x"] - o64.get_state(c)["x"]).max())
        if err > tol and o64.bend_conditioning(c) < conditioning_bound(s, tol):
            excused += 1
            continue
        if err > tol:
            raise AssertionError(f"cloth {c}: |x - x_fp64| = {err:.3e}")
        worst = max(worst, err)
    return dict(worst=worst, excused=excused, contacts=contacts, pairs=pairs)
