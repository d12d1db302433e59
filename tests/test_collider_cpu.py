"""The static triangle collider (lc_batch_set_collider) in the oracle's
restatement: a cloth dropped onto an icosphere mesh rests on it and does
not pass through, the contact rule and its winding, and the slot capacity.
The engine's kernels are compared with this restatement in
tests/test_collider_gpu.py."""
from __future__ import annotations

from dataclasses import replace

import numpy as np

from licenta_gb300 import scenes
from oracle.oracle_ffi import Oracle


def face_planes(vertices, indices, winding):
    a, b, c = (np.asarray(vertices, np.float64)[np.asarray(indices)[:, k]] for k in range(3))
    n = np.cross(b - a, c - a)
    if winding == "cw":
        n = -n
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return n, (n * a).sum(1)


def depth_inside(x, n, d0):
    """How far each point lies inside the convex polytope of the planes
    (negative: outside, by at least that much from some plane)."""
    return -(np.asarray(x, np.float64) @ n.T - d0).max(axis=1)


def test_cloth_rests_on_the_icosphere_and_falls_through_without_it():
    spec = scenes.icosphere_cloth()
    n, d0 = face_planes(*spec.collider)
    o = Oracle([spec], fp64=False)
    bare = Oracle([replace(spec, collider=None)], fp64=False)
    try:
        h = o.thickness(0)
        worst, contacts, fell = -np.inf, 0, False
        for _ in range(40):
            o.step(1, threads=1)
            bare.step(1, threads=1)
            worst = max(worst, float(depth_inside(o.get_state(0)["x"], n, d0).max()))
            ids, _ = o.debug(0, "COLLIDER")
            contacts += int((ids[:, 1] >= 0).sum())
            assert not o.counters(0)["collider_overflow"]
            fell |= bool((depth_inside(bare.get_state(0)["x"], n, d0) > 0.05).any())
    finally:
        o.close()
        bare.close()
    assert contacts > 0
    assert worst <= -0.5 * h, f"a vertex came within {-worst:.4f} m of the inside"
    assert fell, "without the collider the cloth should pass through the sphere"


def one_face_cloth(winding="ccw", height=0.05, speed=-3.0, n=4):
    """A small cloth over one large horizontal triangle at y = 0 moving down
    at `speed` m/s; the triangle's free side is up for "ccw"."""
    spec = scenes.icosphere_cloth(n=n, height=height, span=0.1)
    # (b - a) x (c - a) points up: counter-clockwise seen from above
    tri_v = np.array([[-1.0, 0.0, -1.0], [0.0, 0.0, 1.0], [1.0, 0.0, -1.0]], np.float32)
    spec = replace(spec, collider=(tri_v, np.array([[0, 1, 2]], np.uint32), winding))
    spec.params.gravity[:] = (0.0, 0.0, 0.0)
    return spec, speed


def test_fast_vertices_stop_on_the_free_side_of_a_face():
    """Vertices that cross the face within one step (5 cm at 3 m/s and
    60 Hz, more than the thickness) end it on the free side, at h."""
    spec, speed = one_face_cloth("ccw", height=0.03)
    o = Oracle([spec], fp64=False)
    try:
        h = o.thickness(0)
        o.set_state(0, v=np.tile(np.array([0.0, speed, 0.0], np.float32), (spec.num_vertices, 1)))
        o.step(1, threads=1)
        y = o.get_state(0)["x"][:, 1]
        ids, w = o.debug(0, "COLLIDER")
    finally:
        o.close()
    assert (ids[:, 1] >= 0).reshape(-1, 8).any(axis=1).all(), "every vertex should touch the face"
    assert np.allclose(w[ids[:, 1] >= 0][:, :3], [0.0, 1.0, 0.0], atol=1e-6)
    assert y.min() >= h - 1e-6, f"a vertex ended at y = {y.min():.5f} below h = {h:.5f}"


def test_the_winding_names_the_free_side():
    """The same face wound the other way has its free side below: a cloth
    coming down from above starts behind it, beyond the reach, and passes."""
    spec, speed = one_face_cloth("cw", height=0.3)
    o = Oracle([spec], fp64=False)
    try:
        o.set_state(0, v=np.tile(np.array([0.0, speed, 0.0], np.float32), (spec.num_vertices, 1)))
        for _ in range(12):
            o.step(1, threads=1)
        y = o.get_state(0)["x"][:, 1]
    finally:
        o.close()
    assert y.max() < 0.0, "the cloth should pass through a face seen from its back"


def test_more_contacts_than_slots_is_reported():
    """Nine copies of one face under a vertex are nine contacts, one more
    than a vertex keeps: the oracle reports it (the engine's lc_batch_sync
    returns LC_ERR_CAPACITY_OVERFLOW)."""
    spec, _ = one_face_cloth("ccw", height=0.005)
    v, i, wnd = spec.collider
    spec = replace(spec, collider=(np.tile(v, (9, 1)), (np.arange(27, dtype=np.uint32)).reshape(9, 3), wnd))
    o = Oracle([spec], fp64=False)
    try:
        o.step(1, threads=1)
        assert o.counters(0)["collider_overflow"]
        ids, _ = o.debug(0, "COLLIDER")
        assert np.array_equal(ids[:8, 1], np.arange(8)), "the lowest faces are kept"
    finally:
        o.close()
