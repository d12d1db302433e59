"""Test infrastructure: the pair set every lc_broadphase method must
return, computed by brute force on the CPU — all pairs (a, b), a < b, of
boxes whose closed extents overlap on every axis, as
Collision::DataStructures::BoundingBox::Collides tests two boxes (the
criterion of the reference's BVH and SpatialGrid members,
Collision/BVH.cpp:243, Collision/SpatialGrid.cpp:143)."""
from __future__ import annotations

import numpy as np


def box_pairs(lo, hi, block: int = 2048) -> np.ndarray:
    """(k, 2) int64 pairs, sorted, of the boxes lo[i]..hi[i] ((n, 3) arrays)."""
    lo = np.asarray(lo, np.float32).reshape(-1, 3)
    hi = np.asarray(hi, np.float32).reshape(-1, 3)
    n = lo.shape[0]
    out = []
    for a0 in range(0, n, block):
        a1 = min(n, a0 + block)
        ok = np.ones((a1 - a0, n), bool)
        for ax in range(3):
            ok &= (lo[a0:a1, ax][:, None] <= hi[None, :, ax]) & (hi[a0:a1, ax][:, None] >= lo[None, :, ax])
        ia, ib = np.nonzero(ok)
        ia = ia + a0
        keep = ib > ia
        out.append(np.stack([ia[keep], ib[keep]], axis=1))
    if not out:
        return np.zeros((0, 2), np.int64)
    p = np.concatenate(out).astype(np.int64)
    return p[np.lexsort((p[:, 1], p[:, 0]))]
