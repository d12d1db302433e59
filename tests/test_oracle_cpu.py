"""The oracle on its own (CPU): structural invariants of every stage of the
collision pipeline, FP32-mirror vs FP64 agreement of the PBD step, and the
reference's quirks it must keep."""
from __future__ import annotations

import numpy as np
import pytest

from licenta_gb300 import _ffi, scenes
from oracle.oracle_ffi import Oracle


def stepped(spec, steps, fp64=False):
    o = Oracle([spec], fp64=fp64)
    o.step(steps)
    return o


def overlap(a, b):
    return not (np.any(a[3:] < b[:3]) or np.any(a[:3] > b[3:]))


@pytest.fixture(scope="module")
def hanging():
    return stepped(scenes.small_cloth(seed=3, n=20), 40)


def test_sort_is_stable_and_ordered(hanging):
    m = hanging.debug(0, "MORTON")
    assert np.all(m[1:] >= m[:-1])
    perm = hanging.debug(0, "PERM")
    assert sorted(perm.tolist()) == list(range(len(perm)))


def test_tree_topology_is_consistent(hanging):
    T = hanging.T[0]
    L, R, P = hanging.debug(0, "LEFTS"), hanging.debug(0, "RIGHTS"), hanging.debug(0, "PARENTS")
    assert len(L) == T - 1 and len(P) == 2 * T - 1
    children = np.concatenate([L, R])
    assert sorted(children.tolist()) == list(range(1, 2 * T - 1)), "every node except the root has one parent"
    for i in range(T - 1):
        assert P[L[i]] == i and P[R[i]] == i


def test_refit_boxes_contain_children(hanging):
    T = hanging.T[0]
    L, R = hanging.debug(0, "LEFTS"), hanging.debug(0, "RIGHTS")
    box = hanging.debug(0, "NODE_AABB")
    for i in range(T - 1):
        for c in (L[i], R[i]):
            assert np.all(box[i, :3] <= box[c, :3]) and np.all(box[i, 3:] >= box[c, 3:])


def test_pairs_equal_brute_force_when_no_chunk_overflow(hanging):
    T = hanging.T[0]
    c = hanging.counters(0)
    assert c["dropped"] == 0
    box = hanging.debug(0, "NODE_AABB")[T - 1:]
    pairs = hanging.debug(0, "PAIRS")
    got = set(map(tuple, pairs.tolist()))
    assert len(got) == len(pairs), "no duplicate pairs"
    lo, hi = box[:, :3], box[:, 3:]
    ov = ~((hi[:, None, :] < lo[None, :, :]) | (lo[:, None, :] > hi[None, :, :])).any(-1)
    iu = np.triu_indices(T, 1)
    want = set(zip(iu[0][ov[iu]].tolist(), iu[1][ov[iu]].tolist()))
    assert got == want


def test_pairs_are_in_leaf_then_dfs_order(hanging):
    pairs = hanging.debug(0, "PAIRS")
    assert np.all(np.diff(pairs[:, 0].astype(np.int64)) >= 0)
    assert np.all(pairs[:, 0] < pairs[:, 1])


def test_chunk_cap_drops_pairs_like_the_reference():
    s = scenes.small_cloth(seed=3, n=20)
    s.params.BVHChunkSize = 3
    o = stepped(s, 5)
    c = o.counters(0)
    pairs = o.debug(0, "PAIRS")
    assert c["dropped"] > 0
    assert np.bincount(pairs[:, 0]).max() <= 3


def test_contacts_respect_feature_ownership_and_sanity(hanging):
    vf_v, vf_w = hanging.debug(0, "VF")
    ee_v, ee_w = hanging.debug(0, "EE")
    assert len(vf_v) + len(ee_v) > 0
    for v in vf_v:
        assert v[0] not in v[1:]
    for v in ee_v:
        assert not ({v[0], v[1]} & {v[2], v[3]})
    assert np.all(vf_w[:, 0] == 1.0)
    assert np.all(vf_w[:, 1:] <= 0.0)


def test_feature_ownership_covers_each_vertex_and_edge_once():
    s = scenes.small_cloth(seed=0, n=9)
    o = Oracle([s])
    f = o.debug(0, "FEATURES")
    idx = s.indices
    owned_v = {}
    owned_e = {}
    for t, (a, b, c) in enumerate(idx):
        for bit, v in zip((5, 4, 3), (a, b, c)):
            if f[t] >> bit & 1:
                assert v not in owned_v
                owned_v[v] = t
        for bit, e in zip((2, 1, 0), ((a, b), (b, c), (c, a))):
            if f[t] >> bit & 1:
                k = tuple(sorted(e))
                assert k not in owned_e
                owned_e[k] = t
    assert len(owned_v) == s.num_vertices
    edges = {tuple(sorted(e)) for a, b, c in idx for e in ((a, b), (b, c), (c, a))}
    assert set(owned_e) == edges


def test_fp32_mirror_tracks_fp64_before_contacts():
    s = scenes.small_cloth(seed=2, n=24)
    a, b = Oracle([s], fp64=False), Oracle([s], fp64=True)
    for _ in range(12):
        a.step(1)
        b.step(1)
    xa, xb = a.get_state(0)["x"], b.get_state(0)["x"]
    assert np.abs(xa - xb).max() < 2e-5


def test_pinned_vertices_keep_their_previous_positions():
    s = scenes.small_cloth(seed=4, n=12)
    o = stepped(s, 10, fp64=True)
    st = o.get_state(0)
    pins = np.flatnonzero(s.pinned)
    assert np.allclose(st["x_prev"][pins], s.positions[pins].astype(np.float64))
    assert np.all(st["v"][pins] == 0.0)


def test_world_clamp_and_ground():
    s = scenes.small_cloth(seed=4, n=12)
    o = stepped(s, 60, fp64=True)
    x = o.get_state(0)["x"]
    assert np.all(x >= 0.0) and np.all(x <= 1.0)
    assert np.isfinite(x).all()


def test_wind_moves_the_cloth_along_the_normals():
    base = scenes.small_cloth(seed=4, n=12)
    windy = scenes.small_cloth(seed=4, n=12)
    scenes.set_constant_wind(windy.params, (0.0, 3.0, 0.0))
    a, b = stepped(base, 5, fp64=True), stepped(windy, 5, fp64=True)
    assert np.abs(a.get_state(0)["x"] - b.get_state(0)["x"]).max() > 1e-5


def _swept_boxes(o, spec, order):
    x, xp = o.debug(0, "PRED_X"), o.debug(0, "PRED_XPREV")
    h = np.float32(o.thickness(0))
    tri = spec.indices[order]
    lo = np.minimum(x[tri].min(1) - h, xp[tri].min(1) - h)
    hi = np.maximum(x[tri].max(1) + h, xp[tri].max(1) + h)
    return np.concatenate([lo, hi], axis=1)


def test_leaf_boxes_follow_presort_slots_with_the_quirk():
    """Collision/CudaBVH + Physics/CudaDeformableUtils.cu:146-149, 346-349:
    leaf k keeps the box of pre-sort slot k; the fixed mode gathers it."""
    for quirk in (1, 0):
        s = scenes.small_cloth(seed=3, n=16)
        s.params.refLeafAabbQuirk = quirk
        o = stepped(s, 3)
        T = o.T[0]
        leaf = o.debug(0, "NODE_AABB")[T - 1:]
        order = o.debug(0, "PERM_BEFORE") if quirk else o.debug(0, "PERM")
        assert np.array_equal(leaf, _swept_boxes(o, s, order))
        other = o.debug(0, "PERM") if quirk else o.debug(0, "PERM_BEFORE")
        assert not np.array_equal(leaf, _swept_boxes(o, s, other))


def test_k30_mode_runs_and_sorts():
    s = scenes.small_cloth(seed=3, n=16)
    s.params.mortonMode = _ffi.LC_MORTON_K30
    o = stepped(s, 3)
    m = o.debug(0, "MORTON")
    assert m.max() < (1 << 30) and np.all(m[1:] >= m[:-1])


def test_equal_code_scene_leaves_nodes_unreached():
    """The scene of the malformed-hierarchy GPU test: runs of equal Morton
    codes leave internal nodes, the root among them, unreached by the refit
    (zero boxes, zero rightmost leaves), while the same mesh with its loose
    triangles spread apart builds a well-formed hierarchy."""
    bad = scenes.equal_code_cloth()
    good = scenes.equal_code_cloth(offset=(0.0, 0.0, 0.0))
    n0 = good.num_vertices - 12
    good.positions[n0:] += np.repeat(np.arange(4, dtype=np.float32) * 0.01, 3)[:, None] * np.float32([1, 0, 0])
    for spec, broken in ((bad, True), (good, False)):
        o = Oracle([spec], fp64=False)
        o.external(0)
        o.collide(0)
        T = o.T[0]
        box, rml = o.debug(0, "NODE_AABB")[:T - 1], o.debug(0, "RML")
        unreached = np.flatnonzero(np.all(box == 0, axis=1) & np.all(rml == 0, axis=1))
        o.close()
        assert (0 in unreached) == broken and (len(unreached) > 0) == broken
