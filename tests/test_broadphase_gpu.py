"""The object-level broadphase family (lc_broadphase_*) on the GPU against
the oracle's brute-force pair set: every method must return exactly the
pairs of overlapping boxes, for scattered boxes, coincident boxes (equal
centres), boxes spanning many grid cells, a hash table small enough that
cells share buckets, and the empty and one-object cases; the capacity
errors; and the ICollisionMethod-shaped adapter over a sequence of adds,
moves and removals."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from licenta_gb300 import _ffi
from licenta_gb300.broadphase import Broadphase, CollisionMethod
from oracle.broadphase import box_pairs

pytestmark = pytest.mark.gpu

METHODS = ["brute", "sap", "grid", "hash", "bvh"]


def scattered(n, seed, size=(0.005, 0.05)):
    rng = np.random.default_rng(seed)
    lo = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    return lo, lo + rng.uniform(*size, (n, 3)).astype(np.float32)


def run(method, lo, hi, **kw):
    kw.setdefault("cells_per_axis", 24)
    kw.setdefault("cell_size", 0.04)
    kw.setdefault("table_size", 1 << 14)
    bp = Broadphase(method, max(len(lo), 1), **kw)
    try:
        bp.update(torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda())
        p = bp.test().cpu().numpy()
        crit = bp.criteria()
    finally:
        bp.close()
    return p[np.lexsort((p[:, 1], p[:, 0]))] if len(p) else p.reshape(0, 2), crit


@pytest.mark.parametrize("method", METHODS)
def test_scattered_boxes(method, parity_report):
    lo, hi = scattered(6000, seed=1)
    want = box_pairs(lo, hi)
    got, crit = run(method, lo, hi)
    parity_report(method=method, objects=len(lo), pairs=len(want), tests=crit["intersection_tests"],
                  collision_ms=f"{crit['collision_ms']:.3f}")
    assert len(want) > 1000
    assert np.array_equal(got, want)


def test_methods_agree_at_scale(parity_report):
    """200,000 boxes (sorts of about a hundred tiles and more, the one-sweep
    look-back across many of them): the four sublinear methods return the
    same pair set, and the pairs of its first 20,000 boxes are the oracle's
    brute-force pairs of those boxes."""
    lo, hi = scattered(200_000, seed=11, size=(0.001, 0.01))
    kw = dict(cells_per_axis=128, cell_size=0.01, table_size=1 << 20, max_entries=8 * len(lo))
    got = {m: run(m, lo, hi, **kw)[0] for m in ("sap", "grid", "hash", "bvh")}
    ref = got["bvh"]
    for m, g in got.items():
        assert np.array_equal(g, ref), m
    k = 20_000
    sub = ref[(ref[:, 0] < k) & (ref[:, 1] < k)]
    assert np.array_equal(sub, box_pairs(lo[:k], hi[:k]))
    parity_report(objects=len(lo), pairs=len(ref), checked_subset=k, subset_pairs=len(sub))


@pytest.mark.parametrize("method", METHODS)
def test_coincident_and_large_boxes(method):
    lo, hi = scattered(1500, seed=2)
    # 40 copies of one box (equal centres), and 30 boxes spanning a quarter of the world
    lo = np.concatenate([lo, np.tile(lo[:1], (40, 1))])
    hi = np.concatenate([hi, np.tile(hi[:1], (40, 1))])
    rng = np.random.default_rng(3)
    big = rng.uniform(0.0, 0.7, (30, 3)).astype(np.float32)
    lo = np.concatenate([lo, big])
    hi = np.concatenate([hi, big + np.float32(0.3)])
    got, _ = run(method, lo, hi, max_entries=200_000)
    assert np.array_equal(got, box_pairs(lo, hi))


def test_hash_buckets_shared_by_many_cells():
    lo, hi = scattered(3000, seed=4)
    got, _ = run("hash", lo, hi, table_size=16, cell_size=0.03)
    assert np.array_equal(got, box_pairs(lo, hi))


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("n", [0, 1, 2])
def test_tiny_inputs(method, n):
    lo = np.zeros((n, 3), np.float32)
    hi = np.ones((n, 3), np.float32)  # each box covers the whole 24^3 grid
    got, _ = run(method, lo, hi, max_entries=60_000)
    assert np.array_equal(got, box_pairs(lo, hi))


def test_capacity_errors():
    lo, hi = scattered(2000, seed=5)
    want = box_pairs(lo, hi)
    bp = Broadphase("bvh", len(lo))
    try:
        bp.update(torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda())
        with pytest.raises(_ffi.LcError) as e:
            bp.test(cap=len(want) // 2)
        assert e.value.status == _ffi.LC_ERR_CAPACITY_OVERFLOW
    finally:
        bp.close()
    g = Broadphase("grid", len(lo), cells_per_axis=200, max_entries=len(lo))
    try:
        with pytest.raises(_ffi.LcError) as e:
            g.update(torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda())
        assert e.value.status == _ffi.LC_ERR_CAPACITY_OVERFLOW
    finally:
        g.close()


@pytest.mark.parametrize("method", METHODS)
def test_collision_method_object_lifecycle(method):
    """ObjectAdded / ObjectMoved / ObjectRemoved between frames, as a scene
    of moving objects drives ICollisionMethod, against the oracle each frame."""
    rng = np.random.default_rng(6)
    m = CollisionMethod(method, max_objects=800, cells_per_axis=16, cell_size=0.05, table_size=4096)
    boxes = {}
    try:
        for k in range(600):
            lo = rng.uniform(0, 1, 3).astype(np.float32)
            boxes[k] = (lo, lo + rng.uniform(0.01, 0.06, 3).astype(np.float32))
            m.ObjectAdded(k, *boxes[k])
        for frame in range(4):
            for k in rng.choice(sorted(boxes), 50, replace=False):
                lo = np.clip(boxes[k][0] + rng.normal(0, 0.02, 3), 0, 1).astype(np.float32)
                boxes[k] = (lo, lo + (boxes[k][1] - boxes[k][0]))
                m.ObjectMoved(k, *boxes[k])
            for k in rng.choice(sorted(boxes), 20, replace=False):
                m.ObjectRemoved(k)
                del boxes[k]
            for k in range(1000 + 30 * frame, 1000 + 30 * frame + 30):
                lo = rng.uniform(0, 1, 3).astype(np.float32)
                boxes[k] = (lo, lo + np.float32(0.04))
                m.ObjectAdded(k, *boxes[k])
            m.Update()
            got = {tuple(sorted(p)) for p in m.TestCollision()}
            keys = sorted(boxes)
            want = {(keys[a], keys[b]) for a, b in box_pairs(np.array([boxes[k][0] for k in keys]),
                                                            np.array([boxes[k][1] for k in keys]))}
            assert got == want, f"frame {frame}"
            assert m.GetLastFrameCriteria()["Memory Used (KB)"] > 0
    finally:
        m.close()
