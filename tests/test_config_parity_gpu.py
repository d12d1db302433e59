"""Parity at the sizes of the workloads the engine is measured on, through the
C ABI, against the oracle:

* the plain small cloth (32 x 32, 10 iterations) over its whole 120-step
  rollout, every step;
* the batched workload (256 cloths, sides 16..192, 3.68 M vertices, the
  bench's seed) on sampled steps of its rollout: every cloth's collision
  stages bit-exact and its positions teacher-forced within 1e-5 m of the FP64
  oracle;
* the large cloth (512 x 512 onto the analytic sphere, 20 iterations) on
  steps before and after it reaches the sphere;
* the LBVH microbenchmark's 1 M random triangles: Morton codes, sorted order,
  hierarchy, node boxes, rightmost leaves and pairs bit-exact against the
  oracle, in both Morton modes.

Every figure (largest position error, steps excused by the bend singularity,
pairs and contacts checked) goes to the parity report printed at the end of
the run.
"""
from __future__ import annotations

import numpy as np
import pytest

from licenta_gb300 import ClothBatch, Lbvh, _ffi, scenes
from oracle import parity
from oracle.oracle_ffi import Oracle, lbvh_boxes

pytestmark = pytest.mark.gpu

POS_TOL = 1e-5  # metres on a 1 m cloth: the 1e-5 relative bound


def test_plain_small_cloth_whole_rollout(parity_report):
    worst, contacts, excused, checked = parity.run_parity([scenes.small_cloth(seed=0)], steps=120, tol=POS_TOL)
    parity_report(steps=checked, worst_m=f"{worst:.2e}", excused=excused, contacts=contacts)
    assert contacts > 0


def _sampled_steps(specs, samples, variant=0):
    """Steps one batch of `specs` and checks every cloth on the steps listed
    (1-based) in `samples`; returns the per-sample figures."""
    batch = ClothBatch(specs, debug_capture=True, solver_variant=variant)
    o32 = Oracle(specs, fp64=False)
    o64 = Oracle(specs, fp64=True)
    for c in range(len(specs)):
        o64.track_bend(c)
    out = []
    done = 0
    try:
        for k in samples:
            if k - 1 > done:
                batch.step(k - 1 - done)
            pre = [parity.capture_pre(batch, c) for c in range(len(specs))]
            batch.step(1)
            batch.sync()
            done = k
            r = parity.check_all_cloths(batch, specs, o32, o64, pre, tol=POS_TOL)
            out.append((k, r))
    finally:
        batch.close()
        o32.close()
        o64.close()
    return out


def test_batched_workload_sampled_steps(parity_report):
    """All 256 cloths of the batched workload on steps 6 (the cloths falling),
    25 (the pinned cloths swinging through their lowest point, the most pairs
    and contacts of the rollout) and 100."""
    specs = scenes.batched_cloths(seed=0)
    res = _sampled_steps(specs, (6, 25, 100))
    for k, r in res:
        parity_report(step=k, cloths=len(specs), worst_m=f"{r['worst']:.2e}", excused=r["excused"],
                      pairs=r["pairs"], contacts=r["contacts"])
    assert max(r["pairs"] for _, r in res) > 10_000_000
    assert max(r["contacts"] for _, r in res) > 100_000
    # at most one cloth-step in twenty near the bend singularity
    assert sum(r["excused"] for _, r in res) <= len(specs) * len(res) // 20


def test_large_cloth_sampled_steps(parity_report):
    """The 512 x 512 cloth (262,144 vertices, 522,242 triangles) dropped onto
    the analytic sphere: steps 1 and 2, then 40 and 41, when it lies on the
    sphere (sphere projection and self-contact)."""
    spec = scenes.large_cloth(seed=0)
    res = _sampled_steps([spec], (1, 2, 40, 41))
    for k, r in res:
        parity_report(step=k, worst_m=f"{r['worst']:.2e}", excused=r["excused"], pairs=r["pairs"],
                      contacts=r["contacts"])
    assert res[-1][1]["pairs"] > 1_000_000


@pytest.mark.parametrize("mode", [_ffi.LC_MORTON_REF63, _ffi.LC_MORTON_K30], ids=["ref63", "k30"])
def test_lbvh_one_million_triangles_bit_exact(cuda, parity_report, mode):
    torch = cuda
    count = 1_000_000
    lo, hi = scenes.random_triangle_boxes(count, seed=0)
    lo_t, hi_t = torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda()  # held until the build has read them
    h = Lbvh(count, chunk_size=64, morton_mode=mode)
    try:
        h.build(lo_t.data_ptr(), hi_t.data_ptr(), count)
        n = h.pairs(None, 0)
        want = lbvh_boxes(lo, hi, chunk=64, mode=mode)
        for what in ("MORTON", "PERM", "LEFTS", "RIGHTS", "PARENTS", "RML", "NODE_AABB", "PAIRS"):
            got = h.debug(what)
            exp = want[what]
            if what == "NODE_AABB":
                got, exp = got.view(np.uint32), exp.view(np.uint32)
            assert got.shape == exp.shape and np.array_equal(got, exp), what
        assert n == len(want["PAIRS"])
        codes = want["MORTON"]
        parity_report(triangles=count, pairs=n, distinct_codes=int(np.unique(codes).size))
    finally:
        h.close()


def test_lbvh_awkward_sizes_bit_exact(cuda):
    """One handle built at awkward sizes in turn, largest first (the tile
    table is rebuilt when the count changes): a single key, one tile exactly,
    one key past a tile, a last tile of one key, counts that are not a
    multiple of the refit's 256-leaf blocks.  Codes, order, hierarchy, boxes
    and pairs must equal the oracle's for each (one-sweep sort over 1 to 49
    tiles, two-pass refit)."""
    torch = cuda
    sizes = [100_001, 32_769, 4_097, 2_049, 2_048, 2_047, 257, 2]
    h = Lbvh(max(sizes), chunk_size=64)
    try:
        for count in sizes:
            lo, hi = scenes.random_triangle_boxes(count, seed=count)
            lo_t, hi_t = torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda()
            h.build(lo_t.data_ptr(), hi_t.data_ptr(), count)
            n = h.pairs(None, 0)
            want = lbvh_boxes(lo, hi, chunk=64, mode=_ffi.LC_MORTON_REF63)
            for what in ("MORTON", "PERM", "LEFTS", "RIGHTS", "PARENTS", "RML", "NODE_AABB", "PAIRS"):
                got, exp = h.debug(what), want[what]
                if what == "NODE_AABB":
                    got, exp = got.view(np.uint32), exp.view(np.uint32)
                assert got.shape == exp.shape and np.array_equal(got, exp), (count, what)
            assert n == len(want["PAIRS"]), count
    finally:
        h.close()


def test_free_rollout_drift_report(parity_report):
    """The untethered drift of the plain small cloth: the engine (FP32) and
    the FP64 oracle each run the 120-step rollout on their own, with no
    teacher forcing.  The scheme is chaotic once the cloth touches itself
    (a contact one implementation finds and the other misses moves vertices
    by a finite amount), so no bound is asserted past the first contact;
    the report gives the drift at a few steps and the first step where the
    two contact sets differ.  Before that step the drift must stay within
    the per-step bound times the steps taken."""
    spec = scenes.small_cloth(seed=0)
    batch = ClothBatch([spec], debug_capture=True)
    o64 = Oracle([spec], fp64=True)
    drift, first_split = {}, None
    try:
        for step in range(1, 121):
            batch.step(1)
            batch.sync()
            o64.step_one(0)
            d = float(np.abs(batch.get_state(0)["x"] - o64.get_state(0)["x"]).max())
            if first_split is None:
                gv, ov = batch.debug(0, "VF")[0], o64.debug(0, "VF")[0]
                ge, oe = batch.debug(0, "EE")[0], o64.debug(0, "EE")[0]
                if not (np.array_equal(gv, ov) and np.array_equal(ge, oe)):
                    first_split = step
                else:
                    assert d <= POS_TOL * step, f"step {step}: drift {d:.2e} before the contact sets split"
            if step in (1, 10, 30, 60, 90, 120):
                drift[f"drift_m_step{step}"] = f"{d:.2e}"
            assert np.isfinite(d)
    finally:
        batch.close()
        o64.close()
    parity_report(first_contact_split_step=first_split, **drift)
