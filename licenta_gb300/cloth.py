"""Python side of the engine: a batch of cloths, the reference's body
interface on top of it, and the standalone LBVH.

``CudaDeformableBody`` mirrors Physics::CudaDeformableBody
(Physics/CudaDeformableBody.h:18-28): constructed from the vertex array, the
index array, the parameters and the pinned flags; ``FixedUpdate`` runs one
step (Physics/CudaDeformableBody.cpp:550-627) and ``Update`` writes the
positions back into the caller's vertex array as FinalVertUpdate does
(:473-495).  Every call goes through the C ABI of include/lc/lc.h; there is no
CPU path.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Sequence

import numpy as np

from . import _ffi
from .scenes import ClothSpec


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _stream_handle(stream) -> C.c_void_p | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return C.c_void_p(stream)
    h = getattr(stream, "cuda_stream", None)  # torch.cuda.Stream
    return C.c_void_p(h) if h is not None else None


class ClothBatch:
    """Many independent cloths stepped together (one launch sequence per step)."""

    def __init__(self, specs: Sequence[ClothSpec], *, use_graph: bool = True, debug_capture: bool = False,
                 vf_capacity: int = 0, ee_capacity: int = 0, block_size: int = 0, solver_variant: int = 0,
                 adjoint: bool = False, cand_capacity: int = 0):
        L = _ffi.lib()
        self.specs = list(specs)
        self._keep = []
        descs = (_ffi.ClothDesc * len(self.specs))()
        for k, s in enumerate(self.specs):
            pos = np.ascontiguousarray(s.positions, dtype=np.float32)
            idx = np.ascontiguousarray(s.indices, dtype=np.uint32)
            pin = np.ascontiguousarray(s.pinned, dtype=np.uint8)
            self._keep += [pos, idx, pin]
            descs[k].num_vertices = pos.shape[0]
            descs[k].num_triangles = idx.shape[0]
            descs[k].positions = pos.ctypes.data_as(C.POINTER(C.c_float))
            descs[k].indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
            descs[k].pinned = pin.ctypes.data_as(C.POINTER(C.c_uint8))
            descs[k].params = s.params
        opt = _ffi.default_options()
        opt.use_graph = 1 if use_graph else 0
        opt.debug_capture = 1 if debug_capture else 0
        opt.vf_capacity = vf_capacity
        opt.ee_capacity = ee_capacity
        opt.block_size = block_size
        opt.solver_variant = solver_variant
        opt.adjoint = 1 if adjoint else 0
        opt.cand_capacity = cand_capacity
        h = C.c_void_p()
        _ffi.check(L.lc_batch_create(descs, len(self.specs), C.byref(opt), C.byref(h)), "lc_batch_create")
        self._h = h
        self._keep.clear()
        self.num_vertices = [s.num_vertices for s in self.specs]
        self.num_triangles = [s.num_triangles for s in self.specs]
        for k, s in enumerate(self.specs):
            if getattr(s, "collider", None) is not None:
                self.set_collider(k, *s.collider)

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            _ffi.lib().lc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- stepping -----------------------------------------------------------
    def step(self, nsteps: int = 1, stream=None) -> None:
        _ffi.check(_ffi.lib().lc_batch_step(self._h, nsteps, _stream_handle(stream)), "lc_batch_step")

    def sync(self) -> None:
        _ffi.check(_ffi.lib().lc_batch_sync(self._h), "lc_batch_sync")

    # -- state --------------------------------------------------------------
    def get_state(self, cloth: int) -> dict:
        V = self.num_vertices[cloth]
        out = {k: np.empty((V, 3), dtype=np.float32) for k in ("x", "x_prev", "v", "vn")}
        _ffi.check(_ffi.lib().lc_batch_get_state(self._h, cloth, _ptr(out["x"]), _ptr(out["x_prev"]), _ptr(out["v"]),
                                                 _ptr(out["vn"]), 1), "lc_batch_get_state")
        return out

    def set_state(self, cloth: int, x=None, x_prev=None, v=None, vn=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32) for a in (x, x_prev, v, vn)]
        _ffi.check(_ffi.lib().lc_batch_set_state(self._h, cloth, *[_ptr(a) for a in arrs], 1), "lc_batch_set_state")

    def triangle_order(self, cloth: int) -> np.ndarray:
        out = np.empty(self.num_triangles[cloth], dtype=np.uint32)
        _ffi.check(_ffi.lib().lc_batch_get_triangle_order(self._h, cloth, _ptr(out)), "get_triangle_order")
        return out

    def set_triangle_order(self, cloth: int, perm) -> None:
        p = np.ascontiguousarray(perm, dtype=np.uint32)
        _ffi.check(_ffi.lib().lc_batch_set_triangle_order(self._h, cloth, _ptr(p)), "set_triangle_order")

    def read_positions(self, out: np.ndarray | None = None, stream=None) -> np.ndarray:
        """Positions of every cloth, packed in cloth order (the Update() copy-out)."""
        if out is None:
            out = np.empty((sum(self.num_vertices), 3), dtype=np.float32)
        _ffi.check(_ffi.lib().lc_batch_read_positions(self._h, _ptr(out), 1, _stream_handle(stream)),
                   "lc_batch_read_positions")
        return out

    def read_positions_to(self, dst_ptr: int, is_host: bool, stream=None) -> None:
        _ffi.check(_ffi.lib().lc_batch_read_positions(self._h, C.c_void_p(dst_ptr), 1 if is_host else 0,
                                                      _stream_handle(stream)), "lc_batch_read_positions")

    def write_vertex_records(self, dst_ptr: int, stride: int = 48, pos_offset: int = 0, normal_offset: int = 28,
                             stream=None) -> None:
        """Positions (x_prev) and running normals into interleaved device
        records, Rendering::VertexFormat by default (48 B: position at 0,
        normal at 28); other bytes of the records are left as they are."""
        _ffi.check(_ffi.lib().lc_batch_write_vertex_records(self._h, C.c_void_p(dst_ptr), stride, pos_offset,
                                                            normal_offset, _stream_handle(stream)),
                   "lc_batch_write_vertex_records")

    def write_state(self, x: int | None, x_prev: int | None, v: int | None, is_host: bool, stream=None) -> None:
        """Upload the whole batch state from packed float3 arrays (raw pointers)."""
        vp = lambda a: None if a is None else C.c_void_p(a)
        _ffi.check(_ffi.lib().lc_batch_write_state(self._h, vp(x), vp(x_prev), vp(v), 1 if is_host else 0,
                                                   _stream_handle(stream)), "lc_batch_write_state")

    def read_state(self, x: int | None, x_prev: int | None, v: int | None, is_host: bool, stream=None) -> None:
        vp = lambda a: None if a is None else C.c_void_p(a)
        _ffi.check(_ffi.lib().lc_batch_read_state(self._h, vp(x), vp(x_prev), vp(v), 1 if is_host else 0,
                                                  _stream_handle(stream)), "lc_batch_read_state")

    def profile(self, nsteps: int = 1, stream=None) -> dict:
        p = _ffi.Profile()
        _ffi.check(_ffi.lib().lc_batch_profile(self._h, nsteps, _stream_handle(stream), C.byref(p)),
                   "lc_batch_profile")
        return dict(phases=dict(zip(_ffi.PHASES, list(p.phase_ms))), jacobi_ms=p.jacobi_ms,
                    traverse_ms=p.traverse_ms, narrow_ms=p.narrow_ms, sort_ms=p.sort_ms, step_ms=p.step_ms,
                    kernels_per_step=p.kernels_per_step, solver_ms=p.solver_ms, solver_variant=p.solver_variant,
                    cluster_size=p.cluster_size, ccd_vf_ms=p.ccd_vf_ms, ccd_ee_ms=p.ccd_ee_ms)

    def set_sphere(self, cloth: int, pos, radius: float) -> None:
        p = (C.c_float * 3)(*[float(v) for v in pos])
        _ffi.check(_ffi.lib().lc_batch_set_sphere(self._h, cloth, p, float(radius)), "lc_batch_set_sphere")

    def set_collider(self, cloth: int, vertices, indices, winding: str = "ccw") -> None:
        """A static triangle collider for one cloth (lc_batch_set_collider);
        an empty index array removes it.  winding: "ccw" when the faces turn
        counter-clockwise seen from the free side, "cw" for the opposite
        (scenes.icosphere)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        w = {"ccw": _ffi.LC_WINDING_CCW, "cw": _ffi.LC_WINDING_CW}[winding]
        _ffi.check(_ffi.lib().lc_batch_set_collider(self._h, cloth, _ptr(v), len(v), _ptr(i), len(i), w),
                   "lc_batch_set_collider")

    def constraint_counts(self, cloth: int) -> tuple[int, int]:
        a, b = C.c_int32(), C.c_int32()
        _ffi.check(_ffi.lib().lc_batch_constraint_counts(self._h, cloth, C.byref(a), C.byref(b)), "constraint_counts")
        return a.value, b.value

    def set_stiffness(self, cloth: int, k_stretch=None, k_bend=None) -> None:
        ks = None if k_stretch is None else np.ascontiguousarray(k_stretch, dtype=np.float32)
        kb = None if k_bend is None else np.ascontiguousarray(k_bend, dtype=np.float32)
        _ffi.check(_ffi.lib().lc_batch_set_stiffness(self._h, cloth, _ptr(ks), _ptr(kb)), "lc_batch_set_stiffness")

    def counters(self) -> dict:
        out = (C.c_uint64 * 4)()
        _ffi.check(_ffi.lib().lc_batch_counters(self._h, out), "lc_batch_counters")
        return dict(pairs=out[0], vf=out[1], ee=out[2], dropped=out[3])

    # -- debug dumps ----------------------------------------------------------
    _DT = {1: (np.float32, 3), 2: (np.float32, 3), 3: (np.float32, 3), 4: (np.uint32, 1), 5: (np.uint64, 1),
           6: (np.uint32, 1), 7: (np.int32, 1), 8: (np.int32, 1), 9: (np.int32, 1), 10: (np.int32, 2),
           11: (np.float32, 6), 12: (np.uint32, 2), 15: (np.uint8, 1), 16: (np.uint8, 1), 17: (np.uint32, 1),
           18: (np.uint8, 1), 19: (np.uint8, 1), 20: (np.int8, 1), 21: (np.float32, 3)}

    def debug(self, cloth: int, what: str) -> np.ndarray:
        sel = _ffi.DBG[what]
        L = _ffi.lib()
        n = C.c_uint64()
        _ffi.check(L.lc_batch_debug_get(self._h, cloth, sel, None, 0, C.byref(n)), "lc_batch_debug_get")
        if sel in (13, 14, 22):
            # lc_contact records: 4 int32 ids then 4 float32 weights (collider: plane)
            raw = np.empty((max(n.value, 1), 8), dtype=np.int32)
            _ffi.check(L.lc_batch_debug_get(self._h, cloth, sel, _ptr(raw), n.value, C.byref(n)), "lc_batch_debug_get")
            raw = raw[:n.value]
            return raw[:, :4].copy(), raw[:, 4:].copy().view(np.float32)
        dt, width = self._DT[sel]
        out = np.empty((n.value, width) if width > 1 else (n.value,), dtype=dt)
        _ffi.check(L.lc_batch_debug_get(self._h, cloth, sel, _ptr(out), n.value, C.byref(n)), "lc_batch_debug_get")
        return out


class ClothBatchGroup:
    """One workload stepped as several concurrent batches (lc_group_*).

    The group's cloths are cut into ``lanes`` contiguous ranges of about equal
    vertex count; each range is its own ClothBatch and the group steps them on
    streams of its own, so one batch's latency-bound kernels overlap with the
    others'.  Whole-state copies take the same packed arrays as ClothBatch
    (group order), each lane reading or writing its slice.

    ``order="given"`` keeps the caller's cloth order.  ``order="size"`` orders
    the cloths by vertex count, largest first, so each lane holds cloths of
    like size and can take its own launch shapes (the small cloths' lane
    picks smaller solver clusters); group cloth c is then specs[order[c]],
    and every per-cloth call and packed array of the group is in that order.
    """

    @staticmethod
    def group_order(specs: Sequence[ClothSpec], order: str = "given") -> list[int]:
        """Indices into specs, in the group's cloth order."""
        if order == "given":
            return list(range(len(specs)))
        if order == "size":
            return sorted(range(len(specs)), key=lambda i: (-specs[i].num_vertices, i))
        raise ValueError("order must be 'given' or 'size'")

    def __init__(self, specs: Sequence[ClothSpec], lanes: int = 2, order: str = "given", **kw):
        specs = list(specs)
        if lanes < 1 or lanes > len(specs):
            raise ValueError("lanes must lie in 1..number of cloths")
        self.order = self.group_order(specs, order)
        specs = [specs[i] for i in self.order]
        cum = np.cumsum([s.num_vertices for s in specs])
        cuts = [0] + [int(np.searchsorted(cum, cum[-1] * k / lanes)) + 1 for k in range(1, lanes)] + [len(specs)]
        cuts = sorted(set(min(max(c, 1), len(specs)) for c in cuts[1:-1]) | {0, len(specs)})
        self.ranges = list(zip(cuts[:-1], cuts[1:]))
        self.batches = [ClothBatch(specs[a:b], **kw) for a, b in self.ranges]
        self.specs = specs
        self.num_vertices = [s.num_vertices for s in specs]
        self._voff = [int(sum(self.num_vertices[:a])) for a, _ in self.ranges]
        arr = (C.c_void_p * len(self.batches))(*[b._h.value for b in self.batches])
        h = C.c_void_p()
        _ffi.check(_ffi.lib().lc_group_create(arr, len(self.batches), C.byref(h)), "lc_group_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            _ffi.lib().lc_group_destroy(self._h)
            self._h = None
        for b in getattr(self, "batches", []):
            b.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, nsteps: int = 1, stream=None) -> None:
        _ffi.check(_ffi.lib().lc_group_step(self._h, nsteps, _stream_handle(stream)), "lc_group_step")

    def step_io(self, x_in, x_prev_in, v_in, x_out, x_prev_out, v_out, is_host: bool, stream=None,
                nsteps: int = 1) -> None:
        """nsteps steps, the whole state moved in and out at each (pointers to
        packed 3-float arrays in group order, None to skip): each member batch
        copies its slice in, steps and copies it out on its own stream, and
        the members are joined only at the end, so one batch's copies overlap
        the others' steps."""
        p = [None if a is None else C.c_void_p(a) for a in (x_in, x_prev_in, v_in, x_out, x_prev_out, v_out)]
        _ffi.check(_ffi.lib().lc_group_step_io(self._h, nsteps, *p, 1 if is_host else 0, _stream_handle(stream)),
                   "lc_group_step_io")

    def sync(self) -> None:
        for b in self.batches:
            b.sync()

    def locate(self, cloth: int) -> tuple[ClothBatch, int]:
        """The member batch holding a cloth and the cloth's index there."""
        for (a, e), b in zip(self.ranges, self.batches):
            if a <= cloth < e:
                return b, cloth - a
        raise IndexError(cloth)

    def get_state(self, cloth: int) -> dict:
        b, k = self.locate(cloth)
        return b.get_state(k)

    def _slices(self, ptrs, stride: int):
        for off, b in zip(self._voff, self.batches):
            yield b, [None if p is None else p + off * stride for p in ptrs]

    def write_state(self, x, x_prev, v, is_host: bool, stream=None) -> None:
        for b, (px, pp, pv) in self._slices((x, x_prev, v), 12):
            b.write_state(px, pp, pv, is_host, stream)

    def read_state(self, x, x_prev, v, is_host: bool, stream=None) -> None:
        for b, (px, pp, pv) in self._slices((x, x_prev, v), 12):
            b.read_state(px, pp, pv, is_host, stream)

    def counters(self) -> dict:
        out = dict(pairs=0, vf=0, ee=0, dropped=0)
        for b in self.batches:
            for k, v in b.counters().items():
                out[k] += v
        return out

    def constraint_counts(self, cloth: int) -> tuple[int, int]:
        b, k = self.locate(cloth)
        return b.constraint_counts(k)


class CudaDeformableBody:
    """Physics::CudaDeformableBody on the GB300 engine (one-cloth batch).

    verts: (V, 3) float array that ``Update`` writes the published positions
    into (the reference writes m_dPrevPositions into its VertexFormat array).
    """

    def __init__(self, verts: np.ndarray, indices: np.ndarray, params: _ffi.ClothParams,
                 fixed_verts: Iterable[bool], **batch_kw):
        self.m_verts = verts
        self.m_indices = np.asarray(indices, dtype=np.uint32).reshape(-1, 3)
        pinned = np.asarray(list(fixed_verts), dtype=np.uint8)
        spec = ClothSpec(np.asarray(verts, dtype=np.float32).reshape(-1, 3), self.m_indices, pinned, params)
        self._batch = ClothBatch([spec], **batch_kw)

    def FixedUpdate(self, stream=None) -> None:
        self._batch.step(1, stream)

    def Update(self) -> None:
        self._batch.read_positions(self.m_verts.reshape(-1, 3) if self.m_verts.dtype == np.float32 else None)
        self._batch.sync()

    def SetSpherePos(self, pos, radius: float) -> None:
        self._batch.set_sphere(0, pos, radius)

    @property
    def batch(self) -> ClothBatch:
        return self._batch


class Lbvh:
    """Standalone LBVH over caller boxes (Collision/CudaBVH.cu chain)."""

    def __init__(self, max_triangles: int, chunk_size: int = 64, morton_mode: int = _ffi.LC_MORTON_REF63):
        h = C.c_void_p()
        _ffi.check(_ffi.lib().lc_lbvh_create(max_triangles, chunk_size, morton_mode, C.byref(h)), "lc_lbvh_create")
        self._h = h

    def build(self, bmin_ptr: int, bmax_ptr: int, count: int, stream=None) -> None:
        _ffi.check(_ffi.lib().lc_lbvh_build(self._h, C.c_void_p(bmin_ptr), C.c_void_p(bmax_ptr), count,
                                            _stream_handle(stream)), "lc_lbvh_build")

    def pairs(self, out_ptr: int | None, cap: int, stream=None) -> int:
        n = C.c_uint64()
        _ffi.check(_ffi.lib().lc_lbvh_pairs(self._h, None if out_ptr is None else C.c_void_p(out_ptr), cap,
                                            C.byref(n), _stream_handle(stream)), "lc_lbvh_pairs")
        return n.value

    def sorted_ids(self, out_ptr: int, stream=None) -> None:
        _ffi.check(_ffi.lib().lc_lbvh_sorted_ids(self._h, C.c_void_p(out_ptr), _stream_handle(stream)),
                   "lc_lbvh_sorted_ids")

    _DT = {"MORTON": (np.uint64, 1), "PERM": (np.uint32, 1), "LEFTS": (np.int32, 1), "RIGHTS": (np.int32, 1),
           "PARENTS": (np.int32, 1), "RML": (np.int32, 2), "NODE_AABB": (np.float32, 6), "PAIRS": (np.uint32, 2)}

    def debug(self, what: str) -> np.ndarray:
        """An array of the last build (lc_lbvh_debug_get), in host memory."""
        dt, width = self._DT[what]
        sel = _ffi.DBG[what]
        n = C.c_uint64()
        L = _ffi.lib()
        _ffi.check(L.lc_lbvh_debug_get(self._h, sel, None, 0, C.byref(n)), "lc_lbvh_debug_get")
        out = np.empty((n.value, width) if width > 1 else (n.value,), dtype=dt)
        _ffi.check(L.lc_lbvh_debug_get(self._h, sel, _ptr(out), n.value, C.byref(n)), "lc_lbvh_debug_get")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            _ffi.lib().lc_lbvh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Narrowphase:
    """DeformableUtils::CreateTriangleTests + CCDTriangleTests on caller data
    (lc_narrowphase_*): VF and EE contacts of broadphase pairs, in the
    reference's order."""

    def __init__(self, max_vertices: int, max_triangles: int, max_pairs: int, candidate_capacity: int = 0,
                 contact_capacity: int = 0):
        h = C.c_void_p()
        _ffi.check(_ffi.lib().lc_narrowphase_create(max_vertices, max_triangles, max_pairs, candidate_capacity,
                                                    contact_capacity, C.byref(h)), "lc_narrowphase_create")
        self._h = h

    def run(self, x_ptr: int | None, x_prev_ptr: int, v_ptr: int | None, num_vertices: int, tri_ptr: int,
            feat_ptr: int | None, num_triangles: int, pair_ptr: int | None, num_pairs: int, thickness: float,
            timestep: float, vf_ptr: int | None, vf_cap: int, ee_ptr: int | None, ee_cap: int, stream=None,
            mode: int = _ffi.LC_NARROW_CCD) -> tuple[int, int, int]:
        """Device pointers in, PrimitiveContact records (12 words) out;
        returns (status, VF count, EE count)."""
        nvf, nee = C.c_uint64(), C.c_uint64()
        vp = lambda p: None if p is None else C.c_void_p(p)
        rc = _ffi.lib().lc_narrowphase_run(self._h, mode, vp(x_ptr), vp(x_prev_ptr), vp(v_ptr), num_vertices, vp(tri_ptr),
                                           vp(feat_ptr), num_triangles, vp(pair_ptr), num_pairs, thickness, timestep,
                                           vp(vf_ptr), vf_cap, vp(ee_ptr), ee_cap, C.byref(nvf), C.byref(nee),
                                           _stream_handle(stream))
        return rc, nvf.value, nee.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            _ffi.lib().lc_narrowphase_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
