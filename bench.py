#!/usr/bin/env python
"""Cloth-step throughput of the GB300 engine.

Workload (the batched forward workload): 256 independent cloths, each a
square grid whose side is drawn from U{16..192} (seeded), per-cloth stiffness
U[0.5, 1.0], constant wind U[-2, 2] m/s^2 on x and z, two pinned corners,
10 solver iterations, dt = 1/60 s, self-collision on.  One "step" advances
every cloth of the batch by one CudaDeformableBody::FixedUpdate.  value =
cloth-steps/s = cloths x steps / device time.  With --gpus N (torchrun, one
rank per GPU) one seeded workload of 256 N cloths is split across the ranks
by licenta_gb300.shard.my_share, about 256 cloths each: weak scaling with no
collective on the data path.

Also reported: the plain path (the same engine stepping one cloth per call,
on a seeded sample of the workload's cloths), e2e through the public API with
the whole state uploaded from and downloaded to pinned host memory every
step, the per-phase profile, the roofline of the dominant kernel, sampled SM
clocks, and the CPU oracle port timed on the host cores.

--impl reference times the reference scheme's CPU restatement (the oracle,
OpenMP over cloths on every host core) on the same workload and window (all
256 cloths, the same warm-up and timed steps): the reference has no CPU
implementation of its GPU cloth step.  It builds the workload without loading
the CUDA library.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cloth-steps/s, 256 uneven cloths (16..192 side) batched, 10 iterations, self-collision"
UNIT = "cloth-steps/s"
NCLOTH = 256
# DRAM bytes of the solver's launches in one step of the 256-cloth workload
# (both lanes, default launch shapes, steps 6 and 7): dram__bytes_read.sum +
# dram__bytes_write.sum of k_solve_cluster_scatter from one single-pass ncu
# capture of `bench.py --steps 2 --warmup 5 --no-plain --no-cpu-baseline
# --no-adjoint --no-lbvh --no-large --no-autotune` (684.1 and 682.6 MB).
SOLVER_DRAM_BYTES_PER_STEP = 683.4e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-lbvh", action="store_true")
    ap.add_argument("--only-lbvh", action="store_true",
                    help="run only the LBVH microbenchmark and print its line (for profiling it alone)")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-next", action="store_true",
                    help="skip the broadphase family, narrowphase entry and impulse response timings")
    ap.add_argument("--rollout-1m", action="store_true",
                    help="also run the million-vertex 300-step checkpointed rollout and report its device memory")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--lanes", type=int, default=2,
                    help="concurrent batches the workload is cut into (lc_group_step)")
    ap.add_argument("--cloths", type=int, default=NCLOTH,
                    help="cloths per GPU (the workload has 256; fewer only for small profiling cases)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(parts)
            except ValueError:
                pass
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_gbs() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def save_state(batch, stream):
    """The batch's dynamic state in a device buffer (lc_batch_save_state)."""
    import ctypes as C
    import torch
    from licenta_gb300 import _ffi
    n = C.c_uint64()
    _ffi.check(_ffi.lib().lc_batch_state_size(batch._h, C.byref(n)), "lc_batch_state_size")
    buf = torch.empty(n.value, dtype=torch.uint8, device="cuda")
    _ffi.check(_ffi.lib().lc_batch_save_state(batch._h, C.c_void_p(buf.data_ptr()), C.c_void_p(stream.cuda_stream)),
               "lc_batch_save_state")
    return buf


def load_state(batch, buf, stream):
    import ctypes as C
    from licenta_gb300 import _ffi
    _ffi.check(_ffi.lib().lc_batch_load_state(batch._h, C.c_void_p(buf.data_ptr()), C.c_void_p(stream.cuda_stream)),
               "lc_batch_load_state")


def sampled_profile(batch, state, steps: int, stream, samples: int = 5) -> dict:
    """Per-kernel times averaged over `samples` steps spread evenly over the
    timed rollout (replayed from its saved starting state), with the
    broadphase pair and contact counts of the same steps."""
    load_state(batch, state, stream)
    gap = max(steps // samples - 1, 0)
    acc, cnts = None, []
    for _ in range(samples):
        if gap:
            batch.step(gap, stream)
        p = batch.profile(1, stream)
        c = batch.counters()
        cnts.append((c["pairs"], c["vf"] + c["ee"]))
        if acc is None:
            acc = {k: (dict(v) if isinstance(v, dict) else v) for k, v in p.items()}
            continue
        for k, v in p.items():
            if isinstance(v, dict):
                for q in v:
                    acc[k][q] += v[q]
            elif isinstance(v, float):
                acc[k] += v
    for k, v in acc.items():
        if isinstance(v, dict):
            for q in v:
                v[q] /= samples
        elif isinstance(v, float):
            acc[k] = v / samples
    acc["pairs"] = float(np.mean([c[0] for c in cnts]))
    acc["contacts"] = float(np.mean([c[1] for c in cnts]))
    acc["samples"] = samples
    return acc


def combined_profile(profs: list) -> dict:
    """The member batches' profiles (each measured alone) as one: per-kernel
    times and pair / contact counts add up, since together they do the
    whole workload's work."""
    out = {k: (dict(v) if isinstance(v, dict) else v) for k, v in profs[0].items()}
    for p in profs[1:]:
        for k, v in p.items():
            if isinstance(v, dict):
                for q in v:
                    out[k][q] += v[q]
            elif isinstance(v, float) and k != "samples":
                out[k] += v
    out["kernels_per_step"] = sum(int(p["kernels_per_step"]) for p in profs)
    out["lanes"] = len(profs)
    return out


def algorithmic_bytes(batch, specs, prof) -> dict:
    """Compulsory DRAM bytes per launch of the hot kernels: each kernel's
    per-unit bytes (below) times the units one launch processes.  Pair and
    contact counts are the profile's (averaged over its sampled steps)."""
    V = sum(s.num_vertices for s in specs)
    T = sum(s.num_triangles for s in specs)
    E = B = 0
    for c in range(len(specs)):
        e, b = batch.constraint_counts(c)
        E += e
        B += b
    P, C = prof["pairs"], prof["contacts"]
    return {
        # one Jacobi launch of the global-memory solver: x read + x write
        # (float4), 2 CSR offsets, one entry per incident constraint, each
        # constraint record once, contact records + entries, x_prev
        "jacobi": 32 * V + 8 * V + 4 * (2 * E + 4 * B) + 16 * E + 20 * B + 16 * 4 * C + 32 * C + 16 * V,
        # one launch of the cluster-resident solver (set-up, every iteration
        # and integration on chip): x and x_prev read, x, x_prev, v written
        # (float4), each stretch (ids + l0, kp) and bend (ids + kp) record
        # once, each contact (ids + weights) once
        "solver": 16 * V + 16 * V + 48 * V + 16 * E + 20 * B + 32 * C,
        # leaf box + pair writes + count, every node record once
        "traverse": 32 * T + 4 * P + 4 * T + 48 * (2 * T - 1),
        # pair read, mask written (candidate counts per 32 pairs), triangle
        # records, per-vertex state once
        "narrow": 10 * P + 20 * T + 48 * V,
        "_sizes": dict(V=V, T=T, E=E, B=B, P=P, C=C),
    }


# ---------------------------------------------------------------------------
def adjoint_timing(seed: int) -> dict:
    """The differentiable-rollout workload: a 64x64 cloth, 60 steps, 10
    iterations, checkpoints every 10 steps, loss = summed squared distance of
    the final positions to a target.  Times the forward rollout and its
    backward pass (re-running each segment from its checkpoint, then the
    reverse of every step) with CUDA events, and the plain forward step of
    the same cloth on the default solver."""
    import torch
    from licenta_gb300 import ClothBatch, scenes
    from licenta_gb300.adjoint import ClothRollout, DiffCloth

    steps, every = 60, 10
    spec = scenes.adjoint_cloth(seed=seed)
    cloth = DiffCloth([spec], checkpoint_every=every)
    ks = torch.full((cloth.E,), 0.9, device="cuda", requires_grad=True)
    kb = torch.full((cloth.B,), 0.9, device="cuda", requires_grad=True)
    x0 = torch.tensor(spec.positions, device="cuda", requires_grad=True)
    v0 = torch.zeros_like(x0, requires_grad=True)
    target = x0.detach() - torch.tensor([0.0, 0.3, 0.0], device="cuda")

    def once():
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        out = ClothRollout.apply(cloth, steps, ks, kb, x0, v0)
        loss = ((out - target) ** 2).sum()
        e[1].record()
        loss.backward()
        e[2].record()
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])

    for _ in range(2):
        once()
    runs = [once() for _ in range(3)]
    fwd = float(np.median([r[0] for r in runs])) / steps
    bwd = float(np.median([r[1] for r in runs])) / steps
    cloth.close()
    b = ClothBatch([spec])
    b.step(3)
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    b.step(steps)
    g1.record()
    torch.cuda.synchronize()
    plain = g0.elapsed_time(g1) / steps
    b.close()
    return {"workload": "differentiable rollout: 64x64 cloth, 60 steps, 10 iterations, checkpoints every 10",
            "forward_ms_per_step": fwd, "backward_ms_per_step": bwd, "adjoint_over_forward": bwd / fwd,
            "forward_default_solver_ms_per_step": plain, "adjoint_over_default_forward": bwd / plain,
            "what": "backward = segment re-run from checkpoints + recorded step + reverse pass, per step"}


def adjoint_batched_timing(seed: int, steps: int = 100, every: int = 20, fit_steps: int = 50,
                           fit_iters: int = 8) -> dict:
    """The batched differentiable rollout: 128 cloths (sides U{32..128}), each
    dropped onto its own icosphere of subdivision 4 (radius U[0.2, 0.4] m) as
    a static collider, 10 iterations, checkpoints every 20 steps.  Times one
    100-step forward rollout and its backward pass (loss = summed squared
    distance of the final positions to a target) after one warm-up pair,
    with CUDA events.  Then recovers each cloth's stiffness by gradient
    descent from 0.9 toward seeded targets U[0.5, 0.8]
    (adjoint.fit_cloth_stiffness, the targets' final positions from forward
    runs) over a `fit_steps` horizon: past about 50 steps the drapes fold
    chaotically and the exact gradient no longer predicts the loss."""
    import torch
    from licenta_gb300 import scenes
    from licenta_gb300.adjoint import ClothRollout, DiffCloth, fit_cloth_stiffness

    specs = scenes.batched_sphere_cloths(seed=seed, mesh=True)
    cloth = DiffCloth(specs, checkpoint_every=every, unscale=False)
    C = len(specs)
    ks = torch.full((cloth.E,), 0.9, device="cuda", requires_grad=True)
    kb = torch.full((cloth.B,), 0.9, device="cuda", requires_grad=True)
    x0 = torch.tensor(np.concatenate([s.positions for s in specs]), device="cuda", requires_grad=True)
    v0 = torch.zeros_like(x0, requires_grad=True)
    target = x0.detach() - torch.tensor([0.0, 0.5, 0.0], device="cuda")

    def once():
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        out = ClothRollout.apply(cloth, steps, ks, kb, x0, v0)
        loss = ((out - target) ** 2).sum()
        e[1].record()
        loss.backward()
        e[2].record()
        torch.cuda.synchronize()
        fin = float(torch.isfinite(ks.grad).float().mean())
        return e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2]), fin, int(cloth.grad_exponent.max())

    once()
    fwd, bwd, finite, exp_max = once()
    V = cloth.V
    # stiffness recovery over the fit horizon
    counts = [cloth.batch.constraint_counts(c) for c in range(C)]
    kstar = torch.tensor(np.random.default_rng(seed + 1).uniform(0.5, 0.8, C), dtype=torch.float32, device="cuda")
    ecl = torch.repeat_interleave(torch.arange(C, device="cuda"), torch.tensor([e for e, _ in counts], device="cuda"))
    bcl = torch.repeat_interleave(torch.arange(C, device="cuda"), torch.tensor([b for _, b in counts], device="cuda"))
    xs = x0.detach()
    vs = torch.zeros_like(xs)
    with torch.no_grad():
        tgt = ClothRollout.apply(cloth, fit_steps, kstar[ecl], kstar[bcl], xs, vs).clone()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    k, hist = fit_cloth_stiffness(cloth, fit_steps, xs, vs, tgt, iters=fit_iters)
    t1.record()
    torch.cuda.synchronize()
    err0 = float((0.9 - kstar).abs().mean())
    err1 = float((k - kstar).abs().mean())
    closer = float(((k - kstar).abs() < (0.9 - kstar).abs()).float().mean())
    cloth.close()
    return {"workload": f"batched differentiable rollout: {C} cloths (sides 32..128, {V} vertices) onto their own "
                        f"icospheres (subdivision 4) as static colliders, {steps} steps, 10 iterations, "
                        f"checkpoints every {every}",
            "forward_ms_per_step": fwd / steps, "backward_ms_per_step": bwd / steps,
            "adjoint_over_forward": bwd / fwd, "cloth_steps_per_s_forward": C * steps / (fwd / 1000.0),
            "dL_dk_stretch_finite_share": finite, "max_gradient_exponent_2pow60": exp_max,
            "stiffness_recovery": {"horizon_steps": fit_steps, "iterations": fit_iters,
                                   "mean_abs_k_error_start": err0, "mean_abs_k_error_end": err1,
                                   "cloths_closer_share": closer, "loss_start": hist[0][0], "loss_end": hist[-1][0],
                                   "seconds": t0.elapsed_time(t1) / 1000.0,
                                   "method": "per-cloth k, sign of dL/dk (scaled reverse pass), step 0.1 halved "
                                             "on sign flips"},
            "note": "gradients are the reverse pass's per-cloth scaled values (x 2^(-60 e)), all finite; the "
                    "exact gradient of a 100-step contact-rich drape reaches 2^60 and beyond"}


def rollout_1m_memory(seed: int, n: int = 1024, steps: int = 300, every: int = 20) -> dict:
    """The checkpointed differentiable rollout at a million vertices: one
    n x n cloth (n = 1024: 1,048,576 vertices, 2,093,058 triangles) hanging
    from its two pinned corners with self-collision, 300 steps, 10
    iterations, checkpoints every 20 steps; loss = summed squared distance of
    the final positions to a target.  Reports the engine's own device
    allocation (the drop in free device memory when the batch is created),
    the peak of the torch-allocated checkpoints, segment states and
    gradients, and the forward / backward times."""
    import torch
    from licenta_gb300 import scenes
    from licenta_gb300.adjoint import ClothRollout, DiffCloth

    spec = scenes.adjoint_cloth(seed=seed, n=n)
    torch.cuda.synchronize()
    free0, total = torch.cuda.mem_get_info()
    cloth = DiffCloth([spec], checkpoint_every=every)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    ks = torch.full((cloth.E,), 0.9, device="cuda", requires_grad=True)
    kb = torch.full((cloth.B,), 0.9, device="cuda", requires_grad=True)
    x0 = torch.tensor(spec.positions, device="cuda", requires_grad=True)
    v0 = torch.zeros_like(x0, requires_grad=True)
    target = x0.detach() - torch.tensor([0.0, 0.3, 0.0], device="cuda")
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record()
    out = ClothRollout.apply(cloth, steps, ks, kb, x0, v0)
    loss = ((out - target) ** 2).sum()
    e[1].record()
    loss.backward()
    e[2].record()
    torch.cuda.synchronize()
    free2, _ = torch.cuda.mem_get_info()
    finite = float(torch.isfinite(ks.grad).float().mean())
    peak_torch = torch.cuda.max_memory_allocated() - base
    engine = free0 - free1
    res = {"workload": f"checkpointed differentiable rollout: one {n}x{n} cloth ({spec.num_vertices} vertices, "
                       f"{spec.num_triangles} triangles), {steps} steps, 10 iterations, checkpoints every {every}",
           "engine_device_bytes": int(engine), "torch_peak_bytes": int(peak_torch),
           "peak_device_bytes": int(engine + peak_torch), "device_total_bytes": int(total),
           "min_free_after_bytes": int(free2),
           "forward_ms_per_step": e[0].elapsed_time(e[1]) / steps,
           "backward_ms_per_step": e[1].elapsed_time(e[2]) / steps,
           "dL_dk_stretch_finite_share": finite}
    cloth.close()
    return res


def large_cloth_timing(seed: int, steps: int = 30, warmup: int = 5, mesh: bool = True) -> dict:
    """The plain large workload: one 512x512 cloth (262,144 vertices) dropped
    from y = 1 m onto a sphere of radius 0.3 m at the origin, 20 iterations,
    dt = 1/60 s, self-collision on.  mesh=True (the workload as configured):
    the sphere is the icosphere of subdivision 5 (20,480 faces) as a static
    triangle collider; mesh=False: the reference's analytic sphere.  The
    cloth is too large to keep on chip, so the global-memory Jacobi solver
    runs.  CUDA events around `steps` steps after `warmup`; the cloth's pair
    slots alone (134 MB) exceed L2."""
    import torch
    from licenta_gb300 import ClothBatch, scenes
    b = ClothBatch([scenes.large_cloth(seed=seed, mesh=mesh)])
    s = torch.cuda.Stream()
    b.step(warmup, s)
    b.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    b.step(steps, s)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    prof = b.profile(1, s)
    cnt = b.counters()
    b.close()
    what = "the icosphere of subdivision 5 (r 0.3 m) as a static collider" if mesh else \
        "the analytic sphere (r 0.3 m)"
    return {"workload": f"512x512 cloth onto {what}, 20 iterations", "steps": steps,
            "warmup": warmup, "ms_per_step": ms, "cloth_steps_per_s": 1000.0 / ms,
            "solver_variant": prof["solver_variant"], "phases_ms": prof["phases"],
            "pairs": cnt["pairs"], "contacts": cnt["vf"] + cnt["ee"]}


def step_bytes(specs, batch, prof) -> float:
    """Compulsory HBM bytes of one step of the whole workload: 68 V (state) +
    16 E + 24 B (constraints) + 13 T (triangles) + 200 T (hierarchy build and
    traversal) + 16 P (pairs) + 96 C (contacts)."""
    V = sum(s.num_vertices for s in specs)
    T = sum(s.num_triangles for s in specs)
    E = B = 0
    for c in range(len(specs)):
        e, b = batch.constraint_counts(c)
        E += e
        B += b
    return 68.0 * V + 16.0 * E + 24.0 * B + 213.0 * T + 16.0 * prof["pairs"] + 96.0 * prof["contacts"]


def lbvh_timing(seed: int, count: int = 1_000_000) -> dict:
    """The LBVH-only microbenchmark: 1M random triangles (first vertex uniform
    in the unit cube, two edges of length U[1e-3, 5e-3]), their boxes resident
    on the device; one build = Morton codes + stable 63-bit radix sort + Karras
    hierarchy + refit (lc_lbvh_build), one query = traversal + compaction
    (lc_lbvh_pairs).  CUDA events on the launching stream; the inputs (24 MB
    of boxes) and the hierarchy (~150 MB) exceed nothing, so L2 is flushed
    between timed builds by a 256 MB write."""
    import torch
    from licenta_gb300 import Lbvh, scenes
    lo, hi = scenes.random_triangle_boxes(count, seed=seed)
    lo_t, hi_t = torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda()
    h = Lbvh(count, chunk_size=64)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(3):
        h.build(lo_t.data_ptr(), hi_t.data_ptr(), count, stream)
    torch.cuda.synchronize()
    b_ms, q_ms = [], []
    npairs = 0
    for _ in range(10):
        flush.fill_(1.0)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        h.build(lo_t.data_ptr(), hi_t.data_ptr(), count, stream)
        e[1].record()
        npairs = h.pairs(None, 0, stream)
        e[2].record()
        torch.cuda.synchronize()
        b_ms.append(e[0].elapsed_time(e[1]))
        q_ms.append(e[1].elapsed_time(e[2]))
    h.close()
    build = float(np.median(b_ms))
    # algorithmic bytes of one build: boxes read + key/slot written (32 T),
    # 8 sort passes of (key, payload) read + written (8 x 24 T), hierarchy
    # written (20 T: children, parents), refit (56 T: node boxes read/written)
    alg = (32 + 8 * 24 + 20 + 56) * count
    peak, kind = measured_peak_gbs()
    return {"workload": f"LBVH build over {count} random triangles (63-bit Morton)", "builds_per_s": 1000.0 / build,
            "build_ms": build, "query_ms": float(np.median(q_ms)), "pairs": int(npairs),
            "roofline": {"bound": "hbm", "achieved": alg / (build / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (build / 1000.0) / 1e9 / peak, "algorithmic_bytes_per_build": alg,
                         "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({kind})"},
            "l2": "flushed by a 256 MB write before each timed build"}


def _cuda_ms(fn, reps: int = 10, warmup: int = 3) -> float:
    """Median CUDA-event time of fn() on the current stream."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def next_rows_timing(seed: int, cpu: bool = True) -> dict:
    """The rows beside the step, each on one GPU, CUDA events on the
    launching stream (median of 10 after 3 warm-up calls):
    - the ICollisionMethod family (lc_broadphase_*): 200,000 random boxes
      (lower corner uniform in the unit cube, sides U[1, 10] mm) resident on
      the device; one call = update (structure build) + test (pair count and
      pairs); the methods' pair sets must agree;
    - friction and triangle bending (batched step time with the option on,
      against off) and the render-format vertex record write, on the first
      32 cloths of the batched workload;
    - the alternative collision pipeline on the 512x512 cloth (262,144
      vertices, 522,242 triangles) 10 steps into its drop onto the analytic
      sphere: its swept triangle boxes (the engine's thickness for this mesh,
      the first edge's length / 3; the world box mapped onto the unit cube) through lc_lbvh_build and lc_lbvh_pairs, then
      lc_narrowphase_run (CCD and DCD) on those pairs
      and lc_solve_collisions (the impulse response) on the CCD contacts.
    cpu: the oracle's restatements on the same inputs, one host thread (the
    narrowphase on the first 200,000 pairs), as a reported baseline."""
    import torch
    from licenta_gb300 import ClothBatch, Lbvh, Narrowphase, _ffi, scenes
    from licenta_gb300.broadphase import Broadphase
    out = {}
    rng = np.random.default_rng(seed + 11)
    N = 200_000
    lo = rng.random((N, 3)).astype(np.float32)
    hi = lo + rng.uniform(1e-3, 1e-2, (N, 3)).astype(np.float32)
    lo_t, hi_t = torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda()
    kw = {"sap": {}, "bvh": {},
          "grid": dict(world_min=(0.0, 0.0, 0.0), world_max=(1.02, 1.02, 1.02), cells_per_axis=128, max_entries=8 * N),
          "hash": dict(cell_size=0.01, table_size=1 << 20, max_entries=8 * N)}
    bp_out, counts = {}, set()
    for name, k in kw.items():
        b = Broadphase(name, N, **k)
        pairs = [None]
        def call():
            b.update(lo_t, hi_t)
            pairs[0] = b.test()
        ms = _cuda_ms(call)
        counts.add(int(pairs[0].shape[0]))
        bp_out[name] = {"ms_per_update_and_test": ms, "pairs": int(pairs[0].shape[0]),
                        "objects_per_s": N / (ms / 1000.0)}
        b.close()
    out["broadphase"] = {"workload": f"{N} random boxes (sides 1..10 mm) in the unit cube", "methods": bp_out,
                         "pair_sets_agree": len(counts) == 1}
    # the alternative pipeline on the large cloth's own pairs
    spec = scenes.large_cloth(seed=seed)
    cb = ClothBatch([spec])
    cb.step(10)
    cb.sync()
    st = cb.get_state(0)
    cb.close()
    # the engine's thickness for this mesh: the first edge's length / 3
    h = float(np.linalg.norm(spec.positions[1].astype(np.float64) - spec.positions[0]) / 3.0)
    dt = float(spec.params.timestep)
    tri = spec.indices.astype(np.int64).reshape(-1, 3)
    T = tri.shape[0]
    P3 = np.stack([st["x"][tri], st["x_prev"][tri]], 1).reshape(T, 6, 3)
    # the world box [-1, 1]^3 mapped onto the unit cube the Morton codes cover
    tlo = ((P3.min(1) - h + 1.0) * 0.5).astype(np.float32)
    thi = ((P3.max(1) + h + 1.0) * 0.5).astype(np.float32)
    lb = Lbvh(T, chunk_size=64)
    tlo_t, thi_t = torch.from_numpy(tlo).cuda(), torch.from_numpy(thi).cuda()
    lb.build(tlo_t.data_ptr(), thi_t.data_ptr(), T)
    npairs = lb.pairs(None, 0)
    pairs_t = torch.empty((max(npairs, 1), 2), dtype=torch.int32, device="cuda")
    lb.pairs(pairs_t.data_ptr(), npairs)
    ids = torch.empty(T, dtype=torch.int32, device="cuda")
    lb.sorted_ids(ids.data_ptr())
    torch.cuda.synchronize()
    lb.close()
    tris_t = torch.from_numpy(tri.astype(np.int32)).cuda()[ids.long()].contiguous()
    x_t, xp_t, v_t = (torch.from_numpy(st[q]).cuda() for q in ("x", "x_prev", "v"))
    cap = 15 * max(npairs, 1)
    vf = torch.zeros((min(cap, 1 << 24), 12), dtype=torch.int32, device="cuda")
    ee = torch.zeros((min(cap, 1 << 24), 12), dtype=torch.int32, device="cuda")
    nph = Narrowphase(spec.num_vertices, T, max(npairs, 1), candidate_capacity=9 * max(npairs, 1),
                      contact_capacity=len(vf))
    res = {}
    for mode, name in ((_ffi.LC_NARROW_CCD, "ccd"), (_ffi.LC_NARROW_DCD, "dcd")):
        got = [0, 0, 0]
        ccd = mode == _ffi.LC_NARROW_CCD
        def call():
            got[:] = nph.run(x_t.data_ptr() if ccd else None, xp_t.data_ptr(), v_t.data_ptr() if ccd else None,
                             spec.num_vertices, tris_t.data_ptr(), None, T, pairs_t.data_ptr(), npairs, h, dt,
                             vf.data_ptr(), len(vf), ee.data_ptr(), len(ee), mode=mode)
        ms = _cuda_ms(call)
        res[name] = {"ms": ms, "pairs_per_s": npairs / (ms / 1000.0), "vf": got[1], "ee": got[2], "status": got[0]}
    # the CCD contacts for the impulse response
    rc, nvf, nee = nph.run(x_t.data_ptr(), xp_t.data_ptr(), v_t.data_ptr(), spec.num_vertices, tris_t.data_ptr(),
                           None, T, pairs_t.data_ptr(), npairs, h, dt, vf.data_ptr(), len(vf), ee.data_ptr(), len(ee))
    nph.close()
    p = spec.params
    vmass = float(np.float32(p.objectMass) / np.float32(int(p.dims[0]) * int(p.dims[1])))
    fixed = torch.zeros(spec.num_vertices, dtype=torch.uint8, device="cuda")
    xw = x_t.clone()
    vw = v_t.clone()
    vp = lambda t: C.c_void_p(t.data_ptr())
    def resp():
        xw.copy_(x_t)
        vw.copy_(v_t)
        _ffi.check(_ffi.lib().lc_solve_collisions(vp(xw), vp(xp_t), vp(vw), vp(fixed), spec.num_vertices, vp(vf),
                                                  nvf, vp(ee), nee, float(p.kStretch), vmass, dt, h, None),
                   "lc_solve_collisions")
    ms_r = _cuda_ms(resp)
    out["collision_pipeline"] = {
        "workload": f"512x512 cloth, step 10 of its drop onto the analytic sphere: {npairs} LBVH pairs of its "
                    f"swept triangle boxes (thickness {h:.3g} m)",
        "narrowphase": res,
        "impulse_response": {"ms": ms_r, "contacts": nvf + nee, "note": "includes re-copying x and v (6 MB)"}}
    # the solver options and the render-format write on the first 32 cloths of
    # the batched workload, steps 6-15 (5 warm-up)
    import dataclasses
    base_specs = scenes.batched_cloths(seed=seed)[:32]
    opts = {}
    for name, fld in (("base", None), ("friction", "useFriction"), ("triangle_bending", "useTriangleBending")):
        sp = [dataclasses.replace(x, params=type(x.params).from_buffer_copy(x.params)) for x in base_specs]
        if fld:
            for x in sp:
                setattr(x.params, fld, 1)
        bb = ClothBatch(sp)
        bb.step(5)
        bb.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        bb.step(10)
        e1.record()
        torch.cuda.synchronize()
        opts[name] = {"ms_per_step": e0.elapsed_time(e1) / 10}
        if name == "base":
            Vb = sum(x.num_vertices for x in sp)
            rec = torch.zeros((Vb, 12), dtype=torch.float32, device="cuda")
            ms_rec = _cuda_ms(lambda: bb.write_vertex_records(rec.data_ptr()))
            opts["vertex_records"] = {"ms": ms_rec, "vertices": Vb, "bytes_written": 48 * Vb,
                                      "gb_per_s": 48 * Vb / (ms_rec / 1000.0) / 1e9}
        bb.close()
    out["solver_options"] = {"workload": "the first 32 cloths of the batched workload, steps 6-15", **opts}
    if cpu:
        from oracle import oracle_ffi
        from oracle.broadphase import box_pairs
        nb = 20_000
        t0 = time.perf_counter()
        box_pairs(lo[:nb], hi[:nb])
        out["broadphase"]["cpu_baseline"] = {"objects_per_s": nb / (time.perf_counter() - t0), "cores": 1,
                                             "kind": "port", "sample": f"brute force over the first {nb} boxes"}
        k = min(npairs, 200_000)
        pr = pairs_t[:k].cpu().numpy()
        tr = tris_t.cpu().numpy()
        t0 = time.perf_counter()
        oracle_ffi.narrow_contacts(0, st["x"], st["x_prev"], st["v"], tr, np.full(T, 0x3F, np.uint8), pr, h, dt)
        out["collision_pipeline"]["cpu_baseline"] = {
            "narrowphase_ccd_pairs_per_s": k / (time.perf_counter() - t0), "cores": 1, "kind": "port",
            "sample": f"the first {k} pairs, the oracle's narrowphase restatement"}
    return out


def cpu_baseline(batch, gspecs, members, state0, stream, warmup: int, steps: int = 4) -> dict:
    """The oracle port (FP32 mirror of the reference GPU scheme), OpenMP over
    cloths on every host core, on a bounded sample of the timed window: every
    cloth of the workload, started from the GPU's state at the window's first
    step (positions, previous positions, velocities, running normals,
    triangle order) and stepped `steps` steps, about 20 s of host work.
    gspecs: the specs in the batch's cloth order."""
    from oracle.oracle_ffi import Oracle, max_threads
    for m, st in zip(members, state0):
        load_state(m, st, stream)
    stream.synchronize()
    o = Oracle(gspecs, fp64=False)
    for c in range(len(gspecs)):
        b, k = batch.locate(c) if hasattr(batch, "locate") else (batch, c)
        st = b.get_state(k)
        o.set_state(c, **{q: st[q].astype(np.float64) for q in ("x", "x_prev", "v", "vn")})
        o.set_perm(c, b.triangle_order(k))
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": len(gspecs) * steps / dt, "unit": UNIT, "cores": max_threads(), "kind": "port",
            "sample": f"all {len(gspecs)} cloths, steps {warmup + 1}..{warmup + steps} (the first {steps} steps of "
                      f"the timed window, from the GPU's state at step {warmup}), FP32 oracle port, OpenMP over "
                      f"cloths", "seconds": dt}


# Longest window the reference arm steps on every cloth: at about 2-5 s of
# host time per 256-cloth step, 40 steps stay within a few minutes.
REF_FULL_WINDOW = 40


def run_reference(args, world, rank):
    """The workload on the reference scheme's CPU restatement, OpenMP over
    cloths on every host core: every cloth, W untimed warm-up steps, then K
    timed steps (the window the GPU arm times).  Windows longer than
    REF_FULL_WINDOW steps time a seeded sample of 32 cloths instead, so that
    the run stays within a few minutes.  The workload is built by
    licenta_gb300.scenes without loading the CUDA library."""
    if rank != 0:
        return
    from licenta_gb300 import scenes
    from oracle.oracle_ffi import Oracle, max_threads
    specs = scenes.batched_cloths(seed=args.seed, count=args.cloths)
    if args.warmup + args.steps <= REF_FULL_WINDOW:
        pick = list(range(len(specs)))
    else:
        rng = np.random.default_rng(args.seed + 11)
        pick = sorted(rng.choice(len(specs), size=min(32, len(specs)), replace=False).tolist())
    o = Oracle([specs[i] for i in pick], fp64=False)
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    o.close()
    sample = len(pick)
    value = sample * args.steps / dt
    cores = max_threads()
    what = (f"all {sample} cloths" if sample == len(specs) else f"{sample} of {len(specs)} cloths (seeded)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched-256-uneven" if args.cloths == NCLOTH else f"batched-{args.cloths}-uneven",
                   "cloths_per_step": sample, "iterations": 10, "dt": 1.0 / 60.0,
                   "window": f"steps {args.warmup + 1}..{args.warmup + args.steps} after {args.warmup} warm-up"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{what}, steps {args.warmup + 1}..{args.warmup + args.steps}, FP32 restatement "
                                   f"of the reference GPU scheme (the reference has no CPU implementation of it), "
                                   f"OpenMP over cloths", "seconds": dt},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args, world, rank, local):
    import torch
    import torch.distributed as dist

    from licenta_gb300 import ClothBatch, ClothBatchGroup, scenes

    torch.cuda.set_device(local)
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # one seeded workload of `cloths` cloths per GPU, split across the ranks
    # by the balancing helper (greedy on the per-step cost), so each rank
    # steps about `cloths` cloths (weak scaling); at one GPU the workload is
    # the 256 cloths themselves
    from licenta_gb300 import shard
    everything = scenes.batched_cloths(seed=args.seed, count=args.cloths * world)
    specs = [everything[i] for i in shard.my_share(everything, rank, world)] if world > 1 else everything
    # the workload as `lanes` concurrent batches: ranges of the cloths ordered
    # by size, so each lane holds cloths of like size and is tuned on its own
    batch = ClothBatchGroup(specs, lanes=args.lanes, order="size") if args.lanes > 1 else ClothBatch(specs)
    members = batch.batches if args.lanes > 1 else [batch]
    stream = torch.cuda.Stream()
    batch.step(args.warmup, stream)
    batch.sync()
    tuning = None
    if not args.no_autotune:
        # launch shapes picked by the project's autotuner on this state, for
        # each member batch (each candidate timed from the same saved state;
        # the state is restored)
        from licenta_gb300 import autotune
        tuning = {"config": [], "candidates": 0}
        with torch.cuda.stream(stream):
            for m in members:
                tuned = autotune.autotune(m, steps=2, warmup=1, cache=None,
                                          space={"traverse_block": (64, 128, 256), "jacobi_block": (256,),
                                                 "narrow_blocks_per_sm": (8, 16), "solver_variant": (1, 3),
                                                 "cluster_size": (4, 8, 16), "contact_gather": (0,)})
                tuning["config"].append(tuned["config"])
                tuning["candidates"] += len(tuned["tried"])

    # start of the timed rollout, for the sampled profile
    state0 = [save_state(m, stream) for m in members]

    # ---- device-timed region ------------------------------------------------
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    batch.step(args.steps, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1))
    batch.sync()
    value = world * args.cloths * args.steps / (ms / 1000.0)

    # ---- e2e through the public API: whole state host -> device -> host -----
    # the same window as `value`: restart from the state at its first step
    V = sum(s.num_vertices for s in specs)
    host = [torch.empty((V, 3), dtype=torch.float32, pin_memory=True) for _ in range(3)]
    for m, st in zip(members, state0):
        load_state(m, st, stream)
    batch.read_state(*(h.data_ptr() for h in host), True, stream)
    torch.cuda.synchronize()
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    if args.lanes > 1:  # every step's copies and step on each lane's own stream
        batch.step_io(*(h.data_ptr() for h in host), *(h.data_ptr() for h in host), True, stream, nsteps=args.steps)
    else:
        for _ in range(args.steps):
            batch.write_state(*(h.data_ptr() for h in host), True, stream)
            batch.step(1, stream)
            batch.read_state(*(h.data_ptr() for h in host), True, stream)
    f1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_e2e = max_over_ranks(f0.elapsed_time(f1))
    batch.sync()
    e2e = {"value": world * args.cloths * args.steps / (ms_e2e / 1000.0), "unit": UNIT,
           "h2d_bytes_per_step": 3 * 12 * V, "d2h_bytes_per_step": 3 * 12 * V,
           "window": f"steps {args.warmup + 1}..{args.warmup + args.steps}, replayed from the saved state at "
                     f"step {args.warmup} (the steps `value` times)",
           "what": ("lc_group_step_io: every step, per lane, lc_batch_write_state (x, x_prev, v from pinned "
                    "host) + lc_batch_step + lc_batch_read_state on the lane's stream" if args.lanes > 1 else
                    "lc_batch_write_state (x, x_prev, v from pinned host) + lc_batch_step + lc_batch_read_state")}

    # ---- profile + roofline: steps sampled over the timed rollout ------------
    prof = combined_profile([sampled_profile(m, st, args.steps, stream) for m, st in zip(members, state0)])
    alg = algorithmic_bytes(batch, specs, prof)
    iters = 10
    if prof["solver_variant"] >= 2:  # cluster-resident solver: one launch per step
        solver = {"solver": (prof["solver_ms"], prof["solver_ms"])}
    else:
        solver = {"jacobi": (prof["jacobi_ms"], prof["jacobi_ms"] * iters)}
    cands = {**solver, "traverse": (prof["traverse_ms"], prof["traverse_ms"]),
             "narrow": (prof["narrow_ms"], prof["narrow_ms"])}
    dom = max(cands, key=lambda k: cands[k][1])
    launch_ms = cands[dom][0]
    peak, peak_kind = measured_peak_gbs()
    sb = step_bytes(specs, batch, prof)
    step_ach = sb / (ms / args.steps / 1000.0) / 1e9 if ms > 0 else 0.0
    step_roof = {"bound": "hbm", "bytes_per_step": sb, "achieved": step_ach, "peak": peak, "unit": "GB/s",
                 "frac": step_ach / peak,
                 "what": "compulsory bytes of one whole step (68V + 16E + 24B + 213T + 16P + 96C, pairs and "
                         "contacts averaged over the sampled steps) / measured time per step"}
    achieved = alg[dom] / (launch_ms / 1000.0) / 1e9 if launch_ms > 0 else 0.0
    measured = dom == "solver" and args.cloths == NCLOTH and args.lanes == 2
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})",
            "traffic": SOLVER_DRAM_BYTES_PER_STEP if measured else None,
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the solver launches of steps 6-7 "
                               "(both lanes), this workload" if measured else "not captured for this configuration"),
            "algorithmic_bytes_per_launch": alg[dom], "launch_ms": launch_ms}

    # ---- plain path: the same engine one cloth per call ---------------------
    plain = None
    if not args.no_plain:
        rng = np.random.default_rng(args.seed + 3)
        pick = rng.choice(len(specs), size=16, replace=False)
        tot_ms = 0.0
        for i in pick:
            b1 = ClothBatch([specs[int(i)]])
            b1.step(args.warmup, stream)
            b1.sync()
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            b1.step(args.steps, stream)
            g1.record(stream)
            torch.cuda.synchronize()
            tot_ms += g0.elapsed_time(g1)
            b1.close()
        plain_value = 16 * args.steps / (tot_ms / 1000.0)
        plain = {"value": plain_value, "unit": UNIT, "sample": "16 of the 256 cloths (seeded), one cloth per step call",
                 "batched_over_plain": (value / world) / plain_value}

    adj = None
    if rank == 0 and not args.no_adjoint:
        adj = adjoint_timing(args.seed)
    lbvh = None
    if rank == 0 and not args.no_lbvh:
        lbvh = lbvh_timing(args.seed)
    large = large_analytic = None
    if rank == 0 and not args.no_large:
        large = large_cloth_timing(args.seed, mesh=True)
        large_analytic = large_cloth_timing(args.seed, mesh=False)
    adj_batched = None
    if rank == 0 and not args.no_adjoint:
        adj_batched = adjoint_batched_timing(args.seed)
    roll_1m = None
    if rank == 0 and args.rollout_1m:
        roll_1m = rollout_1m_memory(args.seed)
    next_rows = None
    if rank == 0 and not args.no_next:
        next_rows = next_rows_timing(args.seed, cpu=world == 1 and not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(batch, batch.specs if args.lanes > 1 else specs, members, state0, stream, args.warmup)

    T = sum(s.num_triangles for s in specs)
    state_mb = (V * 16 * 5) / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded cloths, reference mesh topology)",
        "config": {"workload": "batched-256-uneven" if args.cloths == NCLOTH else f"batched-{args.cloths}-uneven",
                   "global_batch": world * args.cloths, "cloths_per_gpu": args.cloths,
                   "vertices_per_gpu": V, "triangles_per_gpu": T, "iterations": 10, "dt": 1.0 / 60.0,
                   "parallelism": f"shard-by-cloth x{world}",
                   "sharding": f"one seeded workload of {args.cloths * world} cloths split across the ranks by "
                               "licenta_gb300.shard.my_share (greedy per-step cost balance), no collective in the step",
                   "concurrent_batches": args.lanes,
                   "lane_order": "cloths by vertex count, largest first" if args.lanes > 1 else None,
                   "l2": f"inputs larger than L2 (vertex state {state_mb:.0f} MB + constraints + pair buffers)"},
        "roofline": roof, "step_roofline": step_roof, "cpu_baseline": cpu, "clocks": clk, "e2e": e2e,
        "gpu_launches": int(prof["kernels_per_step"]) * args.steps,
        "profile": {"phases_ms": prof["phases"], "jacobi_ms": prof["jacobi_ms"], "traverse_ms": prof["traverse_ms"],
                    "narrow_ms": prof["narrow_ms"], "ccd_vf_ms": prof["ccd_vf_ms"], "ccd_ee_ms": prof["ccd_ee_ms"],
                    "solver_ms": prof["solver_ms"], "sort_ms": prof["sort_ms"],
                    "kernels_per_step": prof["kernels_per_step"], "sizes": alg["_sizes"],
                    "sampled_steps": prof["samples"],
                    "what": "per-launch times averaged over steps sampled evenly across the timed rollout; with "
                            "concurrent batches, each kernel's launches of the member batches, timed alone, summed"},
        "plain": plain,
        "adjoint": adj,
        "lbvh": lbvh,
        "large_cloth": large,
        "large_cloth_analytic_sphere": large_analytic,
        "adjoint_batched": adj_batched,
        "rollout_1m": roll_1m,
        "next_rows": next_rows,
        "tuning": tuning,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    batch.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.only_lbvh:
        import torch
        torch.cuda.set_device(local)
        if rank == 0:
            print(json.dumps({"metric": "LBVH builds/s", **lbvh_timing(args.seed)}), flush=True)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
