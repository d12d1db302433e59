"""The host side of the object-level broadphase (licenta_gb300.broadphase):
the ICollisionMethod-shaped adapter's object bookkeeping, run over a
stand-in that computes the oracle's pair set, and the oracle's own pair
rule."""
from __future__ import annotations

import numpy as np

from licenta_gb300 import broadphase
from oracle.broadphase import box_pairs


class _OracleBroadphase:
    """Stands in for the CUDA Broadphase: the oracle's pairs of the boxes
    of the last update."""

    def update(self, lo, hi):
        self.lo, self.hi = lo.numpy(), hi.numpy()

    def test(self):
        import torch
        return torch.from_numpy(box_pairs(self.lo, self.hi))

    def criteria(self):
        return dict(collision_ms=0.0, structure_ms=0.0, intersection_tests=0, pairs=0, memory_bytes=0)


def _adapter():
    m = broadphase.CollisionMethod.__new__(broadphase.CollisionMethod)
    m.bp = _OracleBroadphase()
    m.max_objects = 100
    m._ids, m._slot = [], {}
    m._lo = np.zeros((0, 3), np.float32)
    m._hi = np.zeros((0, 3), np.float32)
    m._criteria = {}
    m.device = "cpu"
    return m


def test_box_pairs_closed_overlap():
    lo = np.array([[0, 0, 0], [1, 0, 0], [1.0001, 0, 0], [0.5, 0.5, 0.5]], np.float32)
    hi = lo + np.float32(1.0)
    hi[3] = lo[3] + np.float32(0.1)
    got = {tuple(p) for p in box_pairs(lo, hi)}
    # boxes touching at x = 1 overlap (closed intervals); 0 and 2 are apart
    assert got == {(0, 1), (0, 3), (1, 2)}


def test_adapter_keeps_ids_through_add_move_remove():
    m = _adapter()
    rng = np.random.default_rng(0)
    boxes = {}
    for k in range(12):
        lo = rng.uniform(0, 1, 3).astype(np.float32)
        boxes[f"obj{k}"] = (lo, lo + np.float32(0.3))
        m.ObjectAdded(f"obj{k}", *boxes[f"obj{k}"])
    for k in (3, 0, 11):
        m.ObjectRemoved(f"obj{k}")
        del boxes[f"obj{k}"]
    lo = np.array([0.5, 0.5, 0.5], np.float32)
    boxes["obj5"] = (lo, lo + np.float32(0.6))
    m.ObjectMoved("obj5", *boxes["obj5"])
    m.Update()
    got = m.TestCollision()
    names = sorted(boxes)
    want = {tuple(sorted((names[a], names[b])))
            for a, b in box_pairs(np.array([boxes[n][0] for n in names]), np.array([boxes[n][1] for n in names]))}
    assert {tuple(sorted(p)) for p in got} == want
    assert set(m.GetLastFrameCriteria()) == {"Time Spent - Collisions", "Time Spent - Structure Update",
                                             "Intersection Tests", "Memory Used (KB)"}
