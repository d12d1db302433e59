"""The two-pass refit's locality rule, on a CPU model of the kernels.

k_refit_local (licenta_gb300/csrc/lc_lbvh.cu) keeps a node's arrival counter
in its block's shared memory when the node's leaf range [min(i, j), max(i,
j)] lies inside one 256-leaf block, and leaves every other arrival to
k_refit_upper's device-scope counter.  That is only sound if every arrival at
such a node comes from a thread of the same block.  The model builds the
hierarchy the way k_karras does (index-tiebroken prefix for the ranges,
code-only split with the midpoint for equal codes, "largest parent wins"),
then runs the per-leaf climbs in random interleavings with the block rule and
with the single global counter, and checks that (a) no node is reached by
both counters or from two blocks, and (b) boxes and rightmost leaves equal
the single-counter refit, including runs of equal codes where two nodes
claim one child."""
import random

import numpy as np
import pytest


def _clz64(x: int) -> int:
    return 64 if x == 0 else 64 - x.bit_length()


def _karras(keys):
    T = len(keys)
    In = T - 1
    child, parent, nend = [None] * In, [-1] * (2 * T - 1), [0] * In

    def delta(i, j):
        if j < 0 or j > In:
            return -1
        x = keys[i] ^ keys[j]
        return _clz64(x) if x else _clz64(i ^ j) + 64

    for i in range(In):
        d = -1 if delta(i, i + 1) - delta(i, i - 1) < 0 else 1
        dmin = delta(i, i - d)
        lmax = 2
        while delta(i, i + lmax * d) > dmin:
            lmax <<= 1
        l, t = 0, lmax // 2
        while t >= 1:
            if delta(i, i + (l + t) * d) > dmin:
                l += t
            t //= 2
        j = i + l * d
        first, last = min(i, j), max(i, j)
        if keys[first] == keys[last]:
            split = (first + last) >> 1
        else:
            com = _clz64(keys[first] ^ keys[last])
            split, step = first, last - first
            while True:
                step = (step + 1) >> 1
                ns = split + step
                if ns < last and _clz64(keys[first] ^ keys[ns]) > com:
                    split = ns
                if step <= 1:
                    break
        left = In + split if split == first else split
        right = In + split + 1 if split + 1 == last else split + 1
        child[i], nend[i] = (left, right), j
        parent[left] = max(parent[left], i)
        parent[right] = max(parent[right], i)
    return child, parent, nend


def _refit(keys, child, parent, nend, leaf, block, rng):
    """block=None: one device counter per node; else the two-pass rule."""
    T = len(keys)
    In = T - 1
    box = {In + k: leaf[k] for k in range(T)}
    box.update({i: 0.0 for i in range(In)})
    rml = {i: (0, 0) for i in range(In)}
    visits, seen = {}, {}

    def climb(s):
        b = None if block is None else s // block
        pid = parent[In + s]
        for _ in range(T + 1):
            if pid < 0 or pid >= In:
                return
            if block is None:
                kind = "g"
            else:
                lo, hi = min(pid, nend[pid]), max(pid, nend[pid])
                kind = "s" if lo // block == b and hi // block == b else "g"
            seen.setdefault(pid, set()).add((kind, b if kind == "s" else None))
            key = (kind, pid)
            first = visits.get(key, 0) == 0  # the atomic's old value decides
            visits[key] = visits.get(key, 0) + 1
            yield
            if first:
                return
            a, c = child[pid]
            box[pid] = min(box[a], box[c])
            rml[pid] = (a if a >= In else max(rml[a]), c if c >= In else max(rml[c]))
            if pid == 0:
                return
            pid = parent[pid]

    live = [climb(s) for s in range(T)]
    while live:
        k = rng.randrange(len(live))
        try:
            next(live[k])
        except StopIteration:
            live[k] = live[-1]
            live.pop()
    for pid, kinds in seen.items():
        assert len(kinds) == 1, f"node {pid} reached as {kinds}"
    return box, rml


@pytest.mark.parametrize("mode", ["distinct", "dups", "manydups"])
def test_block_local_refit_matches_single_counter(mode):
    rng = random.Random(7 if mode == "distinct" else (8 if mode == "dups" else 9))
    for trial in range(40):
        T = rng.choice([2, 3, 5, 17, 64, 200, 700])
        if mode == "distinct":
            keys = sorted(rng.sample(range(1 << 20), T))
        elif mode == "dups":
            keys = sorted(rng.randrange(1 << 9) for _ in range(T))
        else:
            keys = sorted(rng.randrange(8) for _ in range(T))
        child, parent, nend = _karras(keys)
        leaf = [rng.random() for _ in range(T)]
        block = rng.choice([4, 8, 32, 256])
        ref = _refit(keys, child, parent, nend, leaf, None, random.Random(trial))
        got = _refit(keys, child, parent, nend, leaf, block, random.Random(trial + 1000))
        assert ref == got, (trial, T, block)
