"""Concurrent batches (lc_group_*): one workload cut into member batches that
are stepped at the same time on the group's own streams must evolve exactly
as the same cloths stepped in one batch.  Each cloth's step depends only on
that cloth (its sort segment, hierarchy, contacts and on-chip solve), and the
solver's fixed-point sums do not depend on how the work is partitioned, so
the states agree bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from licenta_gb300 import ClothBatch, ClothBatchGroup, scenes

pytestmark = pytest.mark.gpu


def test_group_matches_single_batch(cuda):
    torch = cuda
    specs = scenes.batched_cloths(seed=7, count=9, n_min=12, n_max=40)
    one = ClothBatch(specs)
    grp = ClothBatchGroup(specs, lanes=3)
    try:
        assert len(grp.batches) == 3 and grp.ranges[0][0] == 0 and grp.ranges[-1][1] == len(specs)
        s = torch.cuda.Stream()
        one.step(25, s)
        grp.step(25, s)
        one.sync()
        grp.sync()
        for c in range(len(specs)):
            a, b = one.get_state(c), grp.get_state(c)
            for k in ("x", "x_prev", "v"):
                assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (c, k)
        # whole-state copies through the group's slices
        V = sum(sp.num_vertices for sp in specs)
        host = [np.empty((V, 3), np.float32) for _ in range(3)]
        grp.read_state(*(h.ctypes.data for h in host), True, s)
        grp.sync()
        off = 0
        for c, sp in enumerate(specs):
            st = one.get_state(c)
            assert np.array_equal(host[0][off:off + sp.num_vertices], st["x"])
            off += sp.num_vertices
        assert grp.counters()["pairs"] == one.counters()["pairs"]
    finally:
        grp.close()
        one.close()


def test_size_ordered_group_matches_single_batch(cuda):
    """order="size": the group holds the cloths largest first, its lanes are
    ranges of that order (each tuned on its own), and group cloth c evolves
    exactly as cloth order[c] of the caller's list stepped in one batch."""
    torch = cuda
    from licenta_gb300 import autotune
    specs = scenes.batched_cloths(seed=8, count=10, n_min=10, n_max=44)
    one = ClothBatch(specs)
    grp = ClothBatchGroup(specs, lanes=2, order="size")
    try:
        assert sorted(grp.order) == list(range(len(specs)))
        sizes = [specs[i].num_vertices for i in grp.order]
        assert sizes == sorted(sizes, reverse=True)
        # a smaller cluster on the small cloths' lane changes launch shapes only
        cfg = autotune.get_tuning(grp.batches[1])
        cfg["cluster_size"] = 8
        assert autotune.set_tuning(grp.batches[1], cfg)
        s = torch.cuda.Stream()
        one.step(25, s)
        grp.step(25, s)
        one.sync()
        grp.sync()
        for c, i in enumerate(grp.order):
            a, b = one.get_state(i), grp.get_state(c)
            for k in ("x", "x_prev", "v"):
                assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (c, i, k)
    finally:
        grp.close()
        one.close()


def test_step_io_matches_write_step_read(cuda):
    """lc_group_step_io (each member's copies and steps on its own stream,
    joined at the end) gives the same states, bit for bit, as
    lc_batch_write_state + lc_group_step + lc_batch_read_state on the caller's
    stream, step after step: one call of one step, then one of five."""
    torch = cuda
    specs = scenes.batched_cloths(seed=9, count=8, n_min=12, n_max=36)
    a = ClothBatchGroup(specs, lanes=2, order="size")
    b = ClothBatchGroup(specs, lanes=2, order="size")
    try:
        s = torch.cuda.Stream()
        V = sum(sp.num_vertices for sp in specs)
        ha = [torch.empty((V, 3), dtype=torch.float32, pin_memory=True) for _ in range(3)]
        hb = [torch.empty((V, 3), dtype=torch.float32, pin_memory=True) for _ in range(3)]
        a.read_state(*(h.data_ptr() for h in ha), True, s)
        b.read_state(*(h.data_ptr() for h in hb), True, s)
        for _ in range(6):
            a.write_state(*(h.data_ptr() for h in ha), True, s)
            a.step(1, s)
            a.read_state(*(h.data_ptr() for h in ha), True, s)
        b.step_io(*(h.data_ptr() for h in hb), *(h.data_ptr() for h in hb), True, s)
        b.step_io(*(h.data_ptr() for h in hb), *(h.data_ptr() for h in hb), True, s, nsteps=5)
        torch.cuda.synchronize()
        for x, y in zip(ha, hb):
            assert torch.equal(x.view(torch.int32), y.view(torch.int32))
        assert a.counters()["pairs"] == b.counters()["pairs"]
    finally:
        a.close()
        b.close()
