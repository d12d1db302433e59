"""Autotuner of a batch's launch shapes.

For a given batch it times a small grid of launch shapes (traversal block,
global-memory Jacobi block, narrowphase grid, Jacobi solver variant and the
on-chip solver's cluster size) on the batch's current state and keeps the
fastest.  The timing loop is the library's own (lc_batch_autotune, which C++
hosts call directly): every candidate starts from the same saved state and is
timed with CUDA events over a few steps after a warm-up; the batch is left in
the state it was given, with the winning shapes applied.  This module adds
the search space as a dict and a cache of results.

Block, grid and cluster sizes never change results.  The solver variant does
(the variants sum the Jacobi corrections in different orders, all within the
FP64 tolerance), so it is only searched when ``allow_variants`` is set.

Results are cached per workload signature (cloth count, vertex / triangle
totals, iterations, GPU name) in a JSON file, so a repeated run applies the
stored shapes without timing.
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import torch

from . import _ffi

DEFAULT_SPACE = {
    "traverse_block": (64, 128, 256),
    "jacobi_block": (128, 256, 512),
    "narrow_blocks_per_sm": (4, 8, 16),
    "solver_variant": (1, 2, 3),
    "cluster_size": (4, 8, 16),
    "contact_gather": (0, 1),
}
DEFAULT_CACHE = Path.home() / ".cache" / "licenta_gb300" / "autotune.json"


def get_tuning(batch) -> dict:
    t = _ffi.Tuning()
    _ffi.check(_ffi.lib().lc_batch_get_tuning(batch._h, C.byref(t)), "lc_batch_get_tuning")
    return {k: getattr(t, k) for k, _ in _ffi.Tuning._fields_}


def set_tuning(batch, cfg: dict) -> bool:
    """Applies cfg; False when the batch cannot take it (e.g. a solver
    variant that needs every cloth on chip)."""
    t = _ffi.Tuning(**{k: int(cfg.get(k, 0)) for k, _ in _ffi.Tuning._fields_})
    rc = _ffi.lib().lc_batch_set_tuning(batch._h, C.byref(t))
    if rc == 0:
        return True
    if rc in (1, 6):  # invalid argument / not supported
        return False
    _ffi.check(rc, "lc_batch_set_tuning")
    return False


def signature(batch) -> str:
    specs = batch.specs
    iters = sorted({int(s.params.solverIterations) for s in specs})
    return json.dumps({"cloths": len(specs), "V": sum(batch.num_vertices), "T": sum(batch.num_triangles),
                       "iterations": iters, "gpu": torch.cuda.get_device_name()}, sort_keys=True)


def autotune(batch, *, steps: int = 3, warmup: int = 1, space: dict | None = None, allow_variants: bool = True,
             cache: Path | str | None = DEFAULT_CACHE, refresh: bool = False) -> dict:
    """Tunes `batch` in place and returns {"config": ..., "ms_per_step": ...,
    "tried": [...]} (from the cache when the workload was tuned before)."""
    key = signature(batch)
    store = {}
    if cache is not None and Path(cache).exists():
        try:
            store = json.loads(Path(cache).read_text())
        except ValueError:
            store = {}
    if not refresh and key in store and set_tuning(batch, store[key]["config"]):
        return dict(store[key], cached=True)

    space = dict(DEFAULT_SPACE if space is None else space)
    current = get_tuning(batch)
    sp = _ffi.AutotuneSpace()
    for k in ("traverse_block", "jacobi_block", "narrow_blocks_per_sm", "solver_variant", "cluster_size",
              "contact_gather"):
        # a key the space leaves out is not searched: the cluster size stays
        # automatic, the contact mode off, the others as the batch has them
        held = (0,) if k in ("cluster_size", "contact_gather") else (current[k],)
        vals = [int(v) for v in space.get(k, held)]
        arr = getattr(sp, k)
        if not 1 <= len(vals) <= len(arr):
            raise ValueError(f"autotune space {k}: 1..{len(arr)} values")
        arr[:len(vals)] = vals
        setattr(sp, "n_" + k, len(vals))
    cap = 1
    for k in ("traverse_block", "jacobi_block", "narrow_blocks_per_sm", "solver_variant", "cluster_size",
              "contact_gather"):
        cap *= getattr(sp, "n_" + k)
    trials = (_ffi.AutotuneTrial * cap)()
    best_t, best_ms, n = _ffi.Tuning(), C.c_float(), C.c_int32()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    _ffi.check(_ffi.lib().lc_batch_autotune(batch._h, C.byref(sp), steps, warmup, 1 if allow_variants else 0,
                                            C.c_void_p(stream.cuda_stream), C.byref(best_t), C.byref(best_ms),
                                            trials, cap, C.byref(n)), "lc_batch_autotune")
    torch.cuda.synchronize()
    fields = [k for k, _ in _ffi.Tuning._fields_]
    tried = [{"config": {k: getattr(trials[i].config, k) for k in fields}, "ms_per_step": trials[i].ms_per_step}
             for i in range(min(n.value, cap))]
    best = {"config": {k: getattr(best_t, k) for k in fields}, "ms_per_step": best_ms.value}
    result = {"config": best["config"], "ms_per_step": best["ms_per_step"], "tried": tried}
    if cache is not None and tried:
        store[key] = {"config": best["config"], "ms_per_step": best["ms_per_step"]}
        Path(cache).parent.mkdir(parents=True, exist_ok=True)
        Path(cache).write_text(json.dumps(store, indent=1))
    return dict(result, cached=False)
