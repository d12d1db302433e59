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
    return n


def fp64_step_error(batch, c, o64, pre, perm, sphere: bool, friction: bool = False):
    """Max |x_gpu - x_fp64| (metres) after the step the batch just took."""
    o64.set_state(0, **{k: v.astype(np.float64) for k, v in pre.items()})
    o64.set_perm(0, perm)
    vf, ee = batch.debug(c, "VF"), batch.debug(c, "EE")
    o64.freeze_contacts(0, vf, ee, batch.debug(c, "VF_NORMAL") if friction else None)
    o64.force_decisions(0, batch.debug(c, "GROUND"), batch.debug(c, "GROUND_ACTIVE"), batch.debug(c, "LRA"),
                        batch.debug(c, "DYN_ACTIVE"), batch.debug(c, "SPHERE") if sphere else None)
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
