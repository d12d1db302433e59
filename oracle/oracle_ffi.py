"""ctypes binding of oracle/liblc_oracle.so.

TEST INFRASTRUCTURE ONLY (see oracle/lc_oracle.hpp): the checker for the CUDA
engine, loaded by tests/, smoke() and bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Sequence

import numpy as np

from licenta_gb300 import _ffi
from licenta_gb300.scenes import ClothSpec

from . import build_oracle

_lib = None
VP = C.c_void_p


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        sig = {
            "lco_create": (VP, [C.POINTER(_ffi.ClothDesc), C.c_int, C.c_int]),
            "lco_destroy": (None, [VP]),
            "lco_num_cloths": (C.c_int, [VP]),
            "lco_step": (C.c_int, [VP, C.c_int, C.c_int]),
            "lco_max_threads": (C.c_int, []),
            "lco_sizes": (C.c_int, [VP, C.c_int, VP, VP, VP, VP]),
            "lco_get_state": (C.c_int, [VP, C.c_int, VP, VP, VP, VP]),
            "lco_set_state": (C.c_int, [VP, C.c_int, VP, VP, VP, VP]),
            "lco_get_perm": (C.c_int, [VP, C.c_int, VP]),
            "lco_set_perm": (C.c_int, [VP, C.c_int, VP]),
            "lco_get_wind": (C.c_int, [VP, C.c_int, VP, VP]),
            "lco_set_wind": (C.c_int, [VP, C.c_int, VP, C.c_uint64]),
            "lco_external": (C.c_int, [VP, C.c_int]),
            "lco_collide": (C.c_int, [VP, C.c_int]),
            "lco_step_one": (C.c_int, [VP, C.c_int]),
            "lco_set_frozen_contacts": (C.c_int, [VP, C.c_int, VP, C.c_uint64, VP, C.c_uint64]),
            "lco_set_collider": (C.c_int, [VP, C.c_int, VP, C.c_int, VP, C.c_int, C.c_int]),
            "lco_set_frozen_collider": (C.c_int, [VP, C.c_int, VP, C.c_uint64]),
            "lco_set_stiffness": (C.c_int, [VP, C.c_int, VP, VP]),
            "lco_set_forced": (C.c_int, [VP, C.c_int, VP, VP, VP, VP, C.c_uint64, VP]),
            "lco_thickness": (C.c_int, [VP, C.c_int, VP]),
            "lco_counters": (C.c_int, [VP, C.c_int, C.c_uint64 * 4]),
            "lco_debug_get": (C.c_int, [VP, C.c_int, C.c_int, VP, C.c_uint64, C.POINTER(C.c_uint64)]),
            "lco_grid_indices": (C.c_int, [C.c_int, C.c_int, VP]),
            "lco_morton": (C.c_uint64, [C.c_float, C.c_float, C.c_float, C.c_int]),
            "lco_adj_record": (C.c_int, [VP, C.c_int, C.c_int]),
            "lco_adj_replay": (C.c_int, [VP, C.c_int, C.c_int, C.c_int]),
            "lco_adj_backward": (C.c_int, [VP, C.c_int, VP, VP, VP, VP, VP]),
            "lco_adj_clear": (C.c_int, [VP, C.c_int]),
            "lco_set_stiffness_d": (C.c_int, [VP, C.c_int, VP, VP]),
            "lco_topology": (C.c_int, [VP, C.c_int] + [VP] * 10),
            "lco_solve_on": (C.c_int, [VP, C.c_int, VP, VP, VP, C.c_uint64, VP, C.c_uint64, VP, VP, VP]),
            "lco_solve_iterate": (C.c_int, [VP, C.c_int, C.c_int, VP]),
            "lco_set_frozen_normals": (C.c_int, [VP, C.c_int, VP, C.c_uint64]),
            "lco_tri_bends": (C.c_int, [VP, C.c_int, VP, VP]),
            "lco_track_bend": (C.c_int, [VP, C.c_int, C.c_int]),
            "lco_bend_conditioning": (C.c_int, [VP, C.c_int, C.POINTER(C.c_double)]),
            "lco_friction_on": (C.c_int, [VP, C.c_int, VP, VP, VP, VP, C.c_uint64, VP]),
            "lco_solve_decisions": (C.c_int, [VP, C.c_int, VP, VP, VP, VP, C.c_uint64, C.POINTER(C.c_uint64), VP]),
            "lco_collide_all": (C.c_int, [VP, C.c_int]),
            "lco_solve_collisions": (C.c_int, [VP, VP, VP, VP, C.c_int, VP, C.c_uint64, VP, C.c_uint64, C.c_float,
                                               C.c_float, C.c_float, C.c_float]),
            "lco_narrow_contacts": (C.c_int, [C.c_int, VP, VP, VP, C.c_int, VP, VP, C.c_int, VP, C.c_uint64,
                                              C.c_float, C.c_float, VP, C.c_uint64, C.POINTER(C.c_uint64), VP,
                                              C.c_uint64, C.POINTER(C.c_uint64)]),
            "lco_step_frozen_all": (C.c_int, [VP, C.c_int]),
            "lco_lbvh_boxes": (C.c_int, [VP, VP, C.c_int, C.c_int, C.c_int] + [VP] * 8 +
                               [C.c_uint64, C.POINTER(C.c_uint64)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _chk(rc: int, where: str) -> None:
    if rc != 0:
        raise RuntimeError(f"oracle {where}: status {rc}")


class Oracle:
    """A batch of oracle cloths (fp64=True: FP64; False: FP32 mirror)."""

    _DT = _ffi_DT = {1: (np.float32, 3), 2: (np.float32, 3), 3: (np.float32, 3), 4: (np.uint32, 1),
                     5: (np.uint64, 1), 6: (np.uint32, 1), 7: (np.int32, 1), 8: (np.int32, 1), 9: (np.int32, 1),
                     10: (np.int32, 2), 11: (np.float32, 6), 12: (np.uint32, 2), 15: (np.uint8, 1)}

    def __init__(self, specs: Sequence[ClothSpec], fp64: bool = True):
        keep = []
        descs = (_ffi.ClothDesc * len(specs))()
        for k, s in enumerate(specs):
            pos = np.ascontiguousarray(s.positions, dtype=np.float32)
            idx = np.ascontiguousarray(s.indices, dtype=np.uint32)
            pin = np.ascontiguousarray(s.pinned, dtype=np.uint8)
            keep += [pos, idx, pin]
            descs[k].num_vertices = pos.shape[0]
            descs[k].num_triangles = idx.shape[0]
            descs[k].positions = pos.ctypes.data_as(C.POINTER(C.c_float))
            descs[k].indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
            descs[k].pinned = pin.ctypes.data_as(C.POINTER(C.c_uint8))
            descs[k].params = s.params
        self._h = lib().lco_create(descs, len(specs), 1 if fp64 else 0)
        if not self._h:
            raise RuntimeError("oracle create failed")
        self.fp64 = fp64
        self.n = len(specs)
        self.V = [s.num_vertices for s in specs]
        self.T = [s.num_triangles for s in specs]
        for k, s in enumerate(specs):
            if getattr(s, "collider", None) is not None:
                self.set_collider(k, *s.collider)

    def close(self):
        if getattr(self, "_h", None):
            lib().lco_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, nsteps: int = 1, threads: int = 0) -> None:
        _chk(lib().lco_step(self._h, nsteps, threads), "step")

    def step_one(self, c: int) -> None:
        _chk(lib().lco_step_one(self._h, c), "step_one")

    def external(self, c: int) -> None:
        _chk(lib().lco_external(self._h, c), "external")

    def collide(self, c: int) -> None:
        _chk(lib().lco_collide(self._h, c), "collide")

    def collide_all(self, threads: int = 0) -> None:
        """The collision stages of every cloth, in parallel over cloths."""
        _chk(lib().lco_collide_all(self._h, threads), "collide_all")

    def step_frozen_all(self, threads: int = 0) -> None:
        """One step of every cloth with its frozen contacts (and any forced
        decisions), the collision stages skipped; in parallel over cloths."""
        _chk(lib().lco_step_frozen_all(self._h, threads), "step_frozen_all")

    def get_state(self, c: int) -> dict:
        V = self.V[c]
        out = {k: np.empty((V, 3), dtype=np.float64) for k in ("x", "x_prev", "v", "vn")}
        _chk(lib().lco_get_state(self._h, c, _p(out["x"]), _p(out["x_prev"]), _p(out["v"]), _p(out["vn"])), "get_state")
        return out

    def set_state(self, c: int, x=None, x_prev=None, v=None, vn=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (x, x_prev, v, vn)]
        _chk(lib().lco_set_state(self._h, c, *[_p(a) for a in arrs]), "set_state")

    def perm(self, c: int) -> np.ndarray:
        out = np.empty(self.T[c], dtype=np.uint32)
        _chk(lib().lco_get_perm(self._h, c, _p(out)), "get_perm")
        return out

    def set_perm(self, c: int, perm) -> None:
        p = np.ascontiguousarray(perm, dtype=np.uint32)
        _chk(lib().lco_set_perm(self._h, c, _p(p)), "set_perm")

    def wind(self, c: int):
        w = np.empty(3, dtype=np.float64)
        r = C.c_uint64()
        _chk(lib().lco_get_wind(self._h, c, _p(w), C.byref(r)), "get_wind")
        return w, r.value

    def set_wind(self, c: int, wind, rng: int) -> None:
        w = np.ascontiguousarray(wind, dtype=np.float64)
        _chk(lib().lco_set_wind(self._h, c, _p(w), rng), "set_wind")

    def set_collider(self, c: int, vertices, indices, winding: str = "ccw") -> None:
        """The static triangle collider of lc_batch_set_collider; winding
        "cw" when the faces turn clockwise seen from the free side."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        cw = {"ccw": 0, "cw": 1}[winding]
        _chk(lib().lco_set_collider(self._h, c, _p(v), len(v), _p(i), len(i), cw), "set_collider")

    def freeze_collider(self, c: int, records) -> None:
        """The next step takes these collider contacts (the engine's
        LC_DBG_COLLIDER records as (ids, planes))."""
        ids, w = records
        rec = np.zeros((len(ids), 8), np.int32)
        rec[:, :4] = np.asarray(ids, np.int32).reshape(-1, 4)
        rec[:, 4:] = np.asarray(w, np.float32).reshape(-1, 4).view(np.int32)
        _chk(lib().lco_set_frozen_collider(self._h, c, _p(rec), len(rec)), "set_frozen_collider")

    def freeze_contacts(self, c: int, vf: tuple, ee: tuple, vf_normals=None) -> None:
        def pack(t):  # lc_contact records: 4 int32 ids then 4 float32 weights
            v, w = t
            v = np.asarray(v, np.int32).reshape(-1, 4)
            w = np.asarray(w, np.float32).reshape(-1, 4)
            rec = np.zeros((max(len(v), 1), 8), np.int32)
            rec[:len(v), :4] = v
            rec[:len(v), 4:] = w.view(np.int32)
            return rec, len(v)
        a, na = pack(vf)
        b, nb = pack(ee)
        _chk(lib().lco_set_frozen_contacts(self._h, c, _p(a), na, _p(b), nb), "set_frozen_contacts")
        if vf_normals is not None:
            nr = np.ascontiguousarray(vf_normals, np.float32).reshape(-1, 3)
            _chk(lib().lco_set_frozen_normals(self._h, c, _p(nr), len(nr)), "set_frozen_normals")

    def force_decisions(self, c: int, ground, ground_it, lra, dyn, sphere=None) -> None:
        """Replay another implementation's discrete decisions in the next step."""
        g = np.ascontiguousarray(ground, dtype=np.uint8)
        gi = np.ascontiguousarray(ground_it, dtype=np.uint32)
        la = np.ascontiguousarray(lra, dtype=np.uint8)
        dy = np.ascontiguousarray(dyn, dtype=np.uint8)
        sp = None if sphere is None else np.ascontiguousarray(sphere, dtype=np.int8)
        _chk(lib().lco_set_forced(self._h, c, _p(g), _p(gi), _p(la), _p(dy), dy.size, _p(sp)), "set_forced")

    def set_stiffness(self, c: int, k_stretch=None, k_bend=None) -> None:
        ks = None if k_stretch is None else np.ascontiguousarray(k_stretch, dtype=np.float32)
        kb = None if k_bend is None else np.ascontiguousarray(k_bend, dtype=np.float32)
        _chk(lib().lco_set_stiffness(self._h, c, _p(ks), _p(kb)), "set_stiffness")

    def sizes(self, c: int):
        """(vertices, triangles, stretch constraints, bend constraints) of cloth c."""
        out = [C.c_int() for _ in range(4)]
        _chk(lib().lco_sizes(self._h, c, *[C.byref(o) for o in out]), "sizes")
        return tuple(o.value for o in out)

    # ---- adjoint (FP64 oracle) ------------------------------------------
    def adj_record(self, c: int, nsteps: int) -> None:
        """Step cloth c, recording each step's decisions for the adjoint."""
        _chk(lib().lco_adj_record(self._h, c, nsteps), "adj_record")

    def adj_replay(self, c: int, first: int, nsteps: int) -> None:
        """Step cloth c with the decisions recorded for steps [first, first + nsteps)."""
        _chk(lib().lco_adj_replay(self._h, c, first, nsteps), "adj_replay")

    def adj_backward(self, c: int, gx, gxp, gv):
        """Reverse over the recorded steps.  Returns dL/d(x, x_prev, v) of the
        state before the first recorded step and dL/dk of every stretch and
        bend constraint, given dL/d(x, x_prev, v) after the last."""
        nv, nt, ne, nb = self.sizes(c)
        arrs = [np.ascontiguousarray(a, np.float64).reshape(nv, 3).copy() for a in (gx, gxp, gv)]
        gks, gkb = np.zeros(ne), np.zeros(nb)
        _chk(lib().lco_adj_backward(self._h, c, *[_p(a) for a in arrs], _p(gks), _p(gkb)), "adj_backward")
        return arrs[0], arrs[1], arrs[2], gks, gkb

    def adj_clear(self, c: int) -> None:
        _chk(lib().lco_adj_clear(self._h, c), "adj_clear")

    def set_stiffness_d(self, c: int, k_stretch=None, k_bend=None) -> None:
        ks = None if k_stretch is None else np.ascontiguousarray(k_stretch, np.float64)
        kb = None if k_bend is None else np.ascontiguousarray(k_bend, np.float64)
        _chk(lib().lco_set_stiffness_d(self._h, c, _p(ks), _p(kb)), "set_stiffness_d")

    # ---- solver pin -------------------------------------------------------
    def topology(self, c: int) -> dict:
        """The static topology of cloth c: stretch ends s12 (E, 2), rest
        lengths sl0 (E), bend vertices b (B, 4), the per-vertex slot CSR soff
        (V+1) and its entries sent (kind << 30 | role << 28 | constraint),
        pinned ids fixed (F), attachment lengths lra_l0 (V, F), inverse masses
        invm (V) and pinned flags (V); with triangle bending (tri_bend), b
        rows are (b0, b1, v, -1) and h0 their rest heights."""
        nv, nt, ne, nb = self.sizes(c)
        counts = np.zeros(2, np.int32)
        _chk(lib().lco_topology(self._h, c, *([None] * 9), _p(counts)), "topology")
        F, S = int(counts[0]), int(counts[1])
        t = dict(s12=np.empty((ne, 2), np.int32), sl0=np.empty(ne), b=np.empty((nb, 4), np.int32),
                 soff=np.empty(nv + 1, np.int32), sent=np.empty(S, np.int32), fixed=np.empty(F, np.int32),
                 lra_l0=np.empty((nv, F)), invm=np.empty(nv, np.float32), pinned=np.empty(nv, np.uint8))
        _chk(lib().lco_topology(self._h, c, *[_p(t[k]) for k in ("s12", "sl0", "b", "soff", "sent", "fixed",
                                                                    "lra_l0", "invm", "pinned")], None), "topology")
        tri = C.c_int()
        _chk(lib().lco_tri_bends(self._h, c, C.byref(tri), None), "tri_bends")
        t["tri_bend"] = bool(tri.value)
        t["h0"] = np.zeros(nb)
        if t["tri_bend"]:
            _chk(lib().lco_tri_bends(self._h, c, None, _p(t["h0"])), "tri_bends")
        return t

    def solve_on(self, c: int, x, x_prev, vf: tuple, ee: tuple, forced: dict | None = None):
        """The solver iterations and the velocity update on a given predicted
        state with given contacts (vf, ee: (vertex ids (N, 4), weights (N, 4))).
        ``forced`` (the keys of ``solve_decisions``) imposes another solve's
        discrete decisions.  Returns (x after the iterations, v, x_prev after
        the update)."""
        nv = self.sizes(c)[0]
        if forced is not None:
            self.force_decisions(c, forced["ground"], forced["ground_it"], forced["lra"], forced["dyn"],
                                 forced.get("sphere"))
        xs = np.ascontiguousarray(x, np.float32).reshape(nv, 3)
        xps = np.ascontiguousarray(x_prev, np.float32).reshape(nv, 3)

        def pack(t):
            v, w = t
            v = np.asarray(v, np.int32).reshape(-1, 4)
            w = np.asarray(w, np.float32).reshape(-1, 4)
            if len(v) and (v.min() < 0 or v.max() >= nv):
                raise ValueError("contact vertex id out of range")
            return np.ascontiguousarray(np.concatenate([v, w.view(np.int32)], axis=1)), len(v)
        a, na = pack(vf)
        b, nb_ = pack(ee)
        out = [np.empty((nv, 3), np.float32) for _ in range(3)]
        _chk(lib().lco_solve_on(self._h, c, _p(xs), _p(xps), _p(a), na, _p(b), nb_, *[_p(o) for o in out]),
             "solve_on")
        return tuple(out)

    def track_bend(self, c: int, on: bool = True) -> None:
        _chk(lib().lco_track_bend(self._h, c, 1 if on else 0), "track_bend")

    def bend_conditioning(self, c: int, reverse: bool = False) -> float:
        """min over bends and solver iterates of 1 - n1.n2 in the last solve
        or step (tracked after track_bend): the forward singularity of the
        reference's bend formula.  reverse=True: min of 1 - |n1.n2|, which
        adds the d -> -1 end where only the derivative is singular."""
        out = (C.c_double * 3)()
        _chk(lib().lco_bend_conditioning(self._h, c, out), "bend_conditioning")
        return min(out[0], out[1]) if reverse else out[0]

    def hinge_conditioning(self, c: int) -> tuple[float, float]:
        """(min 1 - n1.n2, min 1 + n1.n2) over the bends and solver iterates
        of the last solve or step (tracked after track_bend)."""
        out = (C.c_double * 3)()
        _chk(lib().lco_bend_conditioning(self._h, c, out), "bend_conditioning")
        return out[0], out[1]

    def contact_conditioning(self, c: int) -> float:
        """min over the contacts and solver iterates of the last solve or
        step of |n| / h (tracked after track_bend), n the contact vector: the
        contact correction's derivative grows like h / |n|."""
        out = (C.c_double * 3)()
        _chk(lib().lco_bend_conditioning(self._h, c, out), "bend_conditioning")
        return out[2]

    def friction_on(self, c: int, v, ground, vf: tuple, normals) -> np.ndarray:
        """Friction (CudaPBD::ApplyFriction) on given velocities with the given
        ground flags, VF contacts (ids (N, 4), weights (N, 4)) and their face
        normals (N, 3); returns the velocities after it."""
        nv = self.sizes(c)[0]
        vs = np.ascontiguousarray(v, np.float32).reshape(nv, 3)
        g = np.ascontiguousarray(ground, np.uint8).reshape(nv)
        ids = np.asarray(vf[0], np.int32).reshape(-1, 4)
        w = np.asarray(vf[1], np.float32).reshape(-1, 4)
        recs = np.ascontiguousarray(np.concatenate([ids, w.view(np.int32)], axis=1))
        nr = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        out = np.empty((nv, 3), np.float32)
        _chk(lib().lco_friction_on(self._h, c, _p(vs), _p(g), _p(recs), _p(nr), len(ids), _p(out)), "friction_on")
        return out

    def solve_iterate(self, c: int, k: int) -> np.ndarray:
        """Positions after iteration k (0 = before the first) of the last solve_on."""
        out = np.empty((self.sizes(c)[0], 3), np.float32)
        _chk(lib().lco_solve_iterate(self._h, c, k, _p(out)), "solve_iterate")
        return out

    def solve_decisions(self, c: int) -> dict:
        """The discrete decisions of the last solve_on: ground constraints
        created (V), ground terms counted per iteration (V bit masks),
        attachments active (V x F), contact corrections counted (iterations x
        4 x (VF + EE)) and ray-sphere outcomes (V)."""
        nv = self.sizes(c)[0]
        F = self.topology(c)["fixed"].size
        n = C.c_uint64()
        _chk(lib().lco_solve_decisions(self._h, c, None, None, None, None, 0, C.byref(n), None), "solve_decisions")
        out = dict(ground=np.empty(nv, np.uint8), ground_it=np.empty(nv, np.uint32), lra=np.empty(nv * F, np.uint8),
                   dyn=np.empty(n.value, np.uint8), sphere=np.empty(nv, np.int8))
        _chk(lib().lco_solve_decisions(self._h, c, _p(out["ground"]), _p(out["ground_it"]), _p(out["lra"]),
                                       _p(out["dyn"]), n.value, C.byref(n), _p(out["sphere"])), "solve_decisions")
        return out

    def thickness(self, c: int) -> float:
        h = C.c_float()
        _chk(lib().lco_thickness(self._h, c, C.byref(h)), "thickness")
        return h.value

    def counters(self, c: int) -> dict:
        out = (C.c_uint64 * 4)()
        rc = lib().lco_counters(self._h, c, out)
        return dict(pairs=out[0], vf=out[1], ee=out[2], dropped=out[3], stack_overflow=rc == 7,
                    collider_overflow=rc == 3)

    def debug(self, c: int, what: str):
        sel = _ffi.DBG[what]
        n = C.c_uint64()
        _chk(lib().lco_debug_get(self._h, c, sel, None, 0, C.byref(n)), "debug_get")
        if sel in (13, 14, 22):
            raw = np.empty((max(n.value, 1), 8), dtype=np.int32)
            _chk(lib().lco_debug_get(self._h, c, sel, _p(raw), n.value, C.byref(n)), "debug_get")
            raw = raw[:n.value]
            return raw[:, :4].copy(), raw[:, 4:].copy().view(np.float32)
        dt, width = self._DT[sel]
        out = np.empty((n.value, width) if width > 1 else (n.value,), dtype=dt)
        _chk(lib().lco_debug_get(self._h, c, sel, _p(out), n.value, C.byref(n)), "debug_get")
        return out


def lbvh_boxes(bmin, bmax, chunk: int = 64, mode: int = 0) -> dict:
    """The restatement's LBVH over caller boxes ((T, 3) float32 min / max
    corners): sorted Morton codes and order, lefts / rights / parents,
    rightmost leaves, node boxes and pairs, in the layouts of the engine's
    lc_lbvh_debug_get."""
    lo = np.ascontiguousarray(bmin, np.float32).reshape(-1, 3)
    hi = np.ascontiguousarray(bmax, np.float32).reshape(-1, 3)
    T = lo.shape[0]
    out = dict(MORTON=np.empty(T, np.uint64), PERM=np.empty(T, np.uint32), LEFTS=np.empty(T - 1, np.int32),
               RIGHTS=np.empty(T - 1, np.int32), PARENTS=np.empty(2 * T - 1, np.int32),
               RML=np.empty((T - 1, 2), np.int32), NODE_AABB=np.empty((2 * T - 1, 6), np.float32))
    n = C.c_uint64()
    args = [_p(out[k]) for k in ("MORTON", "PERM", "LEFTS", "RIGHTS", "PARENTS", "RML", "NODE_AABB")]
    _chk(lib().lco_lbvh_boxes(_p(lo), _p(hi), T, chunk, mode, *args, None, 0, C.byref(n)), "lbvh_boxes")
    pairs = np.empty((n.value, 2), np.uint32)
    _chk(lib().lco_lbvh_boxes(_p(lo), _p(hi), T, chunk, mode, *([None] * 7), _p(pairs), n.value, C.byref(n)),
         "lbvh_boxes")
    out["PAIRS"] = pairs
    return out


def solve_collisions(x, x_prev, v, fixed, vf, ee, *, stiffness: float, vertex_mass: float, dt: float,
                     thickness: float):
    """CudaDeformableBody::SolveCollisions restated (float): x, x_prev, v
    (V, 3); fixed (V,) flags; vf, ee (N, 12) PrimitiveContact records.
    Returns the new positions and velocities."""
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 3).copy()
    xp = np.ascontiguousarray(x_prev, np.float32).reshape(-1, 3)
    vel = np.ascontiguousarray(v, np.float32).reshape(-1, 3).copy()
    fx = np.ascontiguousarray(fixed, np.uint8).reshape(-1)
    a = np.ascontiguousarray(vf, np.int32).reshape(-1, 12)
    b = np.ascontiguousarray(ee, np.int32).reshape(-1, 12)
    _chk(lib().lco_solve_collisions(_p(x), _p(xp), _p(vel), _p(fx), x.shape[0], _p(a), len(a), _p(b), len(b),
                                    stiffness, vertex_mass, dt, thickness), "solve_collisions")
    return x, vel


def narrow_contacts(mode: int, x, x_prev, v, triangles, features, pairs, thickness: float, dt: float):
    """The narrowphase restated on caller data (mode 0: continuous tests,
    1: discrete tests at x_prev), as (N, 12) PrimitiveContact records."""
    xs = [np.ascontiguousarray(a, np.float32).reshape(-1, 3) for a in (x, x_prev, v)]
    tris = np.ascontiguousarray(triangles, np.uint32).reshape(-1, 3)
    feats = np.ascontiguousarray(features, np.uint8).reshape(-1)
    pr = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
    nvf, nee = C.c_uint64(), C.c_uint64()
    args = lambda a, ca, b, cb: (mode, _p(xs[0]), _p(xs[1]), _p(xs[2]), xs[1].shape[0], _p(tris), _p(feats),
                                 len(tris), _p(pr), len(pr), thickness, dt, a, ca, C.byref(nvf), b, cb, C.byref(nee))
    _chk(lib().lco_narrow_contacts(*args(None, 0, None, 0)), "narrow_contacts")
    vf = np.zeros((nvf.value, 12), np.int32)
    ee = np.zeros((nee.value, 12), np.int32)
    _chk(lib().lco_narrow_contacts(*args(_p(vf), len(vf), _p(ee), len(ee))), "narrow_contacts")
    return vf, ee


def morton(x: float, y: float, z: float, mode: int = 0) -> int:
    return int(lib().lco_morton(x, y, z, mode))


def max_threads() -> int:
    return int(lib().lco_max_threads())
