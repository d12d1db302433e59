"""The allocation-free LBVH query, lc_lbvh_pairs_static, against the
allocating entry points (lc_lbvh_create / lc_lbvh_build / lc_lbvh_pairs /
lc_lbvh_sorted_ids), through the C ABI.

lc_lbvh_pairs_static serves callers that cannot call cudaMalloc: code under a
custom allocator or a fixed memory pool, plugins in a process that owns the
device memory, real-time loops that must not allocate.  It keeps every
intermediate buffer in one scratch array built into the library, shared by
all calls.  Two calls in a row, on different inputs, must each return exactly
the pairs and the sorted order of the allocating path (pairs and ids are
integers, so the comparison is exact); the second call shows that nothing the
first call left in the shared scratch leaks into the next result.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from licenta_gb300 import Lbvh, _ffi, scenes

pytestmark = pytest.mark.gpu


def dense_boxes(n: int, seed: int, side: float, grow: float):
    """Triangle boxes whose centres are packed into a cube of the given side
    and whose extents are scaled by `grow`, so that many of them overlap."""
    lo, hi = scenes.random_triangle_boxes(n, seed=seed)
    centre, half = (lo + hi) * 0.5 * np.float32(side), (hi - lo) * 0.5 * np.float32(grow)
    return (centre - half).astype(np.float32), (centre + half).astype(np.float32)


def allocating_query(torch, lo_t, hi_t, n, chunk, mode):
    h = Lbvh(n, chunk_size=chunk, morton_mode=mode)
    h.build(lo_t.data_ptr(), hi_t.data_ptr(), n)
    cap = n * chunk
    pairs = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    count = h.pairs(pairs.data_ptr(), cap)
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    h.sorted_ids(ids.data_ptr())
    torch.cuda.synchronize()
    h.close()
    return pairs[:count].clone(), ids, count


def test_static_lbvh_matches_allocating_entry_point_twice(cuda):
    torch = cuda
    L = _ffi.lib()
    # (triangles, seed, side, grow, pairs per leaf, Morton mode, pairs expected
    # at least).  The 30-bit codes get a sparser cloud so that no two centres
    # share a code; chunk 8 on the dense cloud drops pairs past the cap.
    cases = [(1999, 3, 0.03, 1.0, 64, _ffi.LC_MORTON_REF63, 8000),
             (2048, 4, 0.2, 3.0, 32, _ffi.LC_MORTON_K30, 900),
             (1500, 5, 0.03, 1.0, 8, _ffi.LC_MORTON_REF63, 1500)]
    for n, seed, side, grow, chunk, mode, least in cases:
        lo, hi = dense_boxes(n, seed, side, grow)
        lo_t = torch.from_numpy(lo).cuda()
        hi_t = torch.from_numpy(hi).cuda()
        want_pairs, want_ids, want_count = allocating_query(torch, lo_t, hi_t, n, chunk, mode)
        assert want_count >= least, "the test boxes should overlap a lot"
        cap = n * chunk
        pairs = torch.full((cap, 2), -1, dtype=torch.int32, device="cuda")
        ids = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        count = C.c_uint64()
        rc = L.lc_lbvh_pairs_static(C.c_void_p(lo_t.data_ptr()), C.c_void_p(hi_t.data_ptr()), n, chunk, mode,
                                    C.c_void_p(pairs.data_ptr()), cap, C.byref(count), C.c_void_p(ids.data_ptr()),
                                    None)
        assert rc == 0, L.lc_last_error_string()
        assert count.value == want_count
        assert torch.equal(pairs[:want_count], want_pairs)
        assert torch.equal(ids, want_ids)


def test_static_lbvh_capacity_overflow_keeps_to_the_buffer(cuda):
    """cap below the pair count: the call reports LC_ERR_CAPACITY_OVERFLOW with
    the full count, writes exactly the first cap pairs of the allocating
    path's list and nothing past them; run on a non-default stream."""
    torch = cuda
    L = _ffi.lib()
    n, chunk = 1999, 64
    lo, hi = dense_boxes(n, 3, 0.03, 1.0)
    lo_t = torch.from_numpy(lo).cuda()
    hi_t = torch.from_numpy(hi).cuda()
    want_pairs, _, want_count = allocating_query(torch, lo_t, hi_t, n, chunk, _ffi.LC_MORTON_REF63)
    cap = want_count // 2
    buf = torch.full((want_count, 2), -7, dtype=torch.int32, device="cuda")
    count = C.c_uint64()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    rc = L.lc_lbvh_pairs_static(C.c_void_p(lo_t.data_ptr()), C.c_void_p(hi_t.data_ptr()), n, chunk,
                                _ffi.LC_MORTON_REF63, C.c_void_p(buf.data_ptr()), cap, C.byref(count), None,
                                C.c_void_p(s.cuda_stream))
    torch.cuda.synchronize()
    assert rc == 3, L.lc_last_error_string()
    assert count.value == want_count
    assert torch.equal(buf[:cap], want_pairs[:cap])
    assert bool((buf[cap:] == -7).all()), "a pair was written past cap"


def test_static_lbvh_rejects_sizes_beyond_its_scratch(cuda):
    torch = cuda
    L = _ffi.lib()
    n = 2049
    buf = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    count = C.c_uint64()
    rc = L.lc_lbvh_pairs_static(C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), n, 64, 0, None, 0,
                                C.byref(count), None, None)
    assert rc == 1 and b"2048" in L.lc_last_error_string()
    rc = L.lc_lbvh_pairs_static(C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), 100, 65, 0, None, 0,
                                C.byref(count), None, None)
    assert rc == 1
