"""The object-level broadphase family (lc_broadphase_*, the reference's
Collision::ICollisionMethod, Collision/ICollisionMethod.h:15-87).

``Broadphase`` is the thin binding: boxes in device memory in, overlapping
pairs out.  ``CollisionMethod`` keeps the reference interface's shape for
hosts that move objects one at a time: ObjectAdded / ObjectMoved /
ObjectRemoved edit a host box table, Update() sends it to the device and
builds the method's structure, TestCollision() returns the set of pairs of
object ids whose boxes overlap, and GetLastFrameCriteria() the reference's
per-frame criteria (collision time, structure time, intersection tests,
memory in KB).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _ffi

METHODS = {"brute": _ffi.LC_BP_BRUTE, "sap": _ffi.LC_BP_SAP, "grid": _ffi.LC_BP_GRID, "hash": _ffi.LC_BP_HASH,
           "bvh": _ffi.LC_BP_BVH}


def _p(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr() if t is not None else 0)


class Broadphase:
    """lc_broadphase over one method.  grid: world_min / world_max /
    cells_per_axis; hash: cell_size / table_size; max_entries bounds the
    (object, cell) entries of the two grids (0: 8 per object)."""

    def __init__(self, method: str, max_objects: int, *, world_min=(0.0, 0.0, 0.0), world_max=(1.0, 1.0, 1.0),
                 cells_per_axis: int = 32, cell_size: float = 0.05, table_size: int = 1 << 20,
                 max_entries: int = 0):
        d = _ffi.BroadphaseDesc()
        d.method = METHODS[method]
        d.max_objects = int(max_objects)
        d.max_entries = int(max_entries)
        d.world_min[:] = [float(v) for v in world_min]
        d.world_max[:] = [float(v) for v in world_max]
        d.cells_per_axis = int(cells_per_axis)
        d.cell_size = float(cell_size)
        d.table_size = int(table_size)
        h = C.c_void_p()
        _ffi.check(_ffi.lib().lc_broadphase_create(C.byref(d), C.byref(h)), "lc_broadphase_create")
        self._h = h
        self.method = method
        self._boxes = None

    def close(self) -> None:
        if getattr(self, "_h", None):
            _ffi.lib().lc_broadphase_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, box_min: torch.Tensor, box_max: torch.Tensor) -> None:
        """Boxes (n, 3) float32 on the GPU; kept referenced until the next update."""
        lo = box_min.detach().to(torch.float32).contiguous()
        hi = box_max.detach().to(torch.float32).contiguous()
        self._boxes = (lo, hi)
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        _ffi.check(_ffi.lib().lc_broadphase_update(self._h, _p(lo), _p(hi), lo.shape[0], stream),
                   "lc_broadphase_update")

    def test(self, cap: int | None = None) -> torch.Tensor:
        """The pairs (k, 2) int64 on the GPU, lower index first."""
        L = _ffi.lib()
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        n = C.c_uint64()
        if cap is None:
            _ffi.check(L.lc_broadphase_test(self._h, None, 0, C.byref(n), stream), "lc_broadphase_test")
            cap = n.value
        out = torch.empty((max(int(cap), 1), 2), dtype=torch.int32, device="cuda")
        _ffi.check(L.lc_broadphase_test(self._h, _p(out), int(cap), C.byref(n), stream), "lc_broadphase_test")
        return out[:n.value].to(torch.int64)

    def criteria(self) -> dict:
        c = _ffi.BroadphaseCriteria()
        _ffi.check(_ffi.lib().lc_broadphase_get_criteria(self._h, C.byref(c)), "lc_broadphase_get_criteria")
        return dict(structure_ms=c.structure_ms, collision_ms=c.collision_ms,
                    intersection_tests=c.intersection_tests, pairs=c.pairs, memory_bytes=c.memory_bytes)


class CollisionMethod:
    """Collision::ICollisionMethod over a Broadphase: objects are any
    hashable ids with a box each."""

    def __init__(self, method: str = "bvh", max_objects: int = 1 << 16, **kw):
        self.bp = Broadphase(method, max_objects, **kw)
        self.max_objects = int(max_objects)
        self._ids: list = []                 # slot -> object id
        self._slot: dict = {}                # object id -> slot
        self._lo = np.zeros((0, 3), np.float32)
        self._hi = np.zeros((0, 3), np.float32)
        self._criteria: dict = {}
        self.device = "cuda"

    def ObjectAdded(self, obj, box_min, box_max) -> None:
        if obj in self._slot:
            raise ValueError(f"object {obj!r} already added")
        if len(self._ids) >= self.max_objects:
            raise ValueError("more objects than max_objects")
        self._slot[obj] = len(self._ids)
        self._ids.append(obj)
        self._lo = np.vstack([self._lo, np.asarray(box_min, np.float32).reshape(1, 3)])
        self._hi = np.vstack([self._hi, np.asarray(box_max, np.float32).reshape(1, 3)])

    def ObjectMoved(self, obj, box_min, box_max) -> None:
        s = self._slot[obj]
        self._lo[s] = np.asarray(box_min, np.float32)
        self._hi[s] = np.asarray(box_max, np.float32)

    def ObjectRemoved(self, obj) -> None:
        s = self._slot.pop(obj)
        last = len(self._ids) - 1
        if s != last:  # the last object takes the freed slot
            moved = self._ids[last]
            self._ids[s] = moved
            self._slot[moved] = s
            self._lo[s], self._hi[s] = self._lo[last], self._hi[last]
        self._ids.pop()
        self._lo, self._hi = self._lo[:last], self._hi[:last]

    def Update(self) -> None:
        lo = torch.from_numpy(np.ascontiguousarray(self._lo)).to(self.device)
        hi = torch.from_numpy(np.ascontiguousarray(self._hi)).to(self.device)
        self.bp.update(lo, hi)

    def TestCollision(self) -> set:
        pairs = self.bp.test().cpu().numpy()
        ids = self._ids
        c = self.bp.criteria()
        # the keys of Core/Utils.hpp:42-46
        self._criteria = {"Time Spent - Collisions": c["collision_ms"],
                          "Time Spent - Structure Update": c["structure_ms"],
                          "Intersection Tests": float(c["intersection_tests"]),
                          "Memory Used (KB)": c["memory_bytes"] / 1024.0}
        return {(ids[a], ids[b]) for a, b in pairs}

    def GetLastFrameCriteria(self) -> dict:
        return dict(self._criteria)

    def close(self) -> None:
        self.bp.close()
