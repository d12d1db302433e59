"""Autotuner of a batch's launch shapes.

For a given batch it times a small grid of launch shapes (traversal block,
global-memory Jacobi block, narrowphase grid, Jacobi solver variant and the
on-chip solver's cluster size) on the batch's current state and keeps the
fastest.  Every candidate starts from the
same saved state (lc_batch_save_state / lc_batch_load_state) and is timed
with CUDA events over a few steps after a warm-up; the batch is left in the
state it was given, with the winning shapes applied.

Block, grid and cluster sizes never change results.  The solver variant does
(the variants sum the Jacobi corrections in different orders, all within the
FP64 tolerance), so it is only searched when ``allow_variants`` is set.

Results are cached per workload signature (cloth count, vertex / triangle
totals, iterations, GPU name) in a JSON file, so a repeated run applies the
stored shapes without timing.
"""
from __future__ import annotations

import ctypes as C
import itertools
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


def _time(batch, state, steps: int, warmup: int, stream) -> float:
    L = _ffi.lib()
    sp = C.c_void_p(stream.cuda_stream)
    _ffi.check(L.lc_batch_load_state(batch._h, C.c_void_p(state.data_ptr()), sp), "lc_batch_load_state")
    batch.step(warmup, stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    batch.step(steps, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    batch.sync()
    return e0.elapsed_time(e1) / steps


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
    if not allow_variants:
        space["solver_variant"] = (get_tuning(batch)["solver_variant"],)
    L = _ffi.lib()
    n = C.c_uint64()
    _ffi.check(L.lc_batch_state_size(batch._h, C.byref(n)), "lc_batch_state_size")
    state = torch.empty(n.value, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    _ffi.check(L.lc_batch_save_state(batch._h, C.c_void_p(state.data_ptr()), C.c_void_p(stream.cuda_stream)),
               "lc_batch_save_state")
    original = get_tuning(batch)
    names = list(space)
    tried = []
    for values in itertools.product(*(space[k] for k in names)):
        cfg = dict(zip(names, values))
        cfg.setdefault("cluster_size", 0)
        # the Jacobi block only matters for the global-memory solver, the
        # cluster size only for the on-chip ones
        if cfg["solver_variant"] != 1 and cfg["jacobi_block"] != space["jacobi_block"][0]:
            continue
        if cfg["solver_variant"] == 1 and cfg["cluster_size"] not in (0, space.get("cluster_size", (0,))[0]):
            continue
        if cfg["solver_variant"] == 1:
            cfg["cluster_size"] = 0
        # the contact mode only matters for the scatter solver
        cfg.setdefault("contact_gather", 0)
        if cfg["solver_variant"] != 3 and cfg["contact_gather"] != space.get("contact_gather", (0,))[0]:
            continue
        if cfg["solver_variant"] != 3:
            cfg["contact_gather"] = 0
        if not set_tuning(batch, cfg):
            continue
        tried.append({"config": cfg, "ms_per_step": _time(batch, state, steps, warmup, stream)})
    best = min(tried, key=lambda r: r["ms_per_step"]) if tried else {"config": original, "ms_per_step": None}
    set_tuning(batch, best["config"])
    _ffi.check(L.lc_batch_load_state(batch._h, C.c_void_p(state.data_ptr()), C.c_void_p(stream.cuda_stream)),
               "lc_batch_load_state")
    torch.cuda.synchronize()
    result = {"config": best["config"], "ms_per_step": best["ms_per_step"], "tried": tried}
    if cache is not None and tried:
        store[key] = {"config": best["config"], "ms_per_step": best["ms_per_step"]}
        Path(cache).parent.mkdir(parents=True, exist_ok=True)
        Path(cache).write_text(json.dumps(store, indent=1))
    return dict(result, cached=False)
