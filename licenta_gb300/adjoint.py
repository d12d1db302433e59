"""Differentiable cloth rollouts: the engine's reverse pass behind a
torch.autograd.Function.

``ClothRollout`` steps a batch of cloths for a fixed number of steps from
given initial positions and velocities with given per-constraint
stiffnesses, and returns the published positions after the last step (the
x_prev array the reference's Update() copies out).  Its backward pass returns
dL/d(stretch stiffness), dL/d(bend stiffness), dL/d(initial velocities) and
dL/d(initial positions) (for a pinned vertex, the gradient with respect to its
fixed position).

Memory: the forward pass keeps a checkpoint of the full dynamic state every
``checkpoint_every`` steps; the backward pass re-runs each segment from its
checkpoint, keeping the segment's states, and runs the adjoint of every step
(lc_batch_adjoint_step: the step re-run with its solver iterates recorded,
then reversed with its discrete decisions held fixed).  Peak memory is about
(steps / checkpoint_every + checkpoint_every) states plus one step's tape.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np
import torch

from . import _ffi
from .cloth import ClothBatch
from .scenes import ClothSpec


def _p(t: torch.Tensor | None):
    return None if t is None else C.c_void_p(t.data_ptr())


class DiffCloth:
    """A batch prepared for differentiable rollouts (adjoint tape kept)."""

    def __init__(self, specs: Sequence[ClothSpec], checkpoint_every: int = 10, unscale: bool = True, **batch_kw):
        """unscale=False: ClothRollout's backward returns each cloth's
        gradients as the reverse pass kept them, scaled by 2^(-60 e) with e =
        grad_exponent[cloth] after the call.  They stay finite (and their
        direction exact) where the true gradient of a long contact-rich
        rollout is beyond float range, which is what per-cloth normalised
        descent needs; unscale=True multiplies the scale back in (inf where
        the true value exceeds float)."""
        self.batch = ClothBatch(specs, adjoint=True, use_graph=True, **batch_kw)
        self.h = self.batch._h
        self.every = max(1, int(checkpoint_every))
        self.unscale = unscale
        self.grad_exponent = torch.zeros(len(specs), dtype=torch.int32, device="cuda")
        L = _ffi.lib()
        n = C.c_uint64()
        _ffi.check(L.lc_batch_state_size(self.h, C.byref(n)), "lc_batch_state_size")
        self.state_bytes = n.value
        self.V = sum(self.batch.num_vertices)
        counts = [self.batch.constraint_counts(c) for c in range(len(specs))]
        self.E = sum(e for e, _ in counts)
        self.B = sum(b for _, b in counts)
        self.initial = self.new_state()
        self.save(self.initial)
        torch.cuda.synchronize()

    # -- state buffers ---------------------------------------------------------
    def new_state(self) -> torch.Tensor:
        return torch.empty(self.state_bytes, dtype=torch.uint8, device="cuda")

    @staticmethod
    def _stream():
        return torch.cuda.current_stream()

    @staticmethod
    def _sp():
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def save(self, buf: torch.Tensor) -> None:
        _ffi.check(_ffi.lib().lc_batch_save_state(self.h, _p(buf), self._sp()), "lc_batch_save_state")

    def load(self, buf: torch.Tensor) -> None:
        _ffi.check(_ffi.lib().lc_batch_load_state(self.h, _p(buf), self._sp()), "lc_batch_load_state")

    def step(self, n: int = 1) -> None:
        self.batch.step(n, self._stream())

    def set_stiffness(self, ks: torch.Tensor, kb: torch.Tensor) -> None:
        ks = ks.detach().to("cuda", torch.float32).contiguous()
        kb = kb.detach().to("cuda", torch.float32).contiguous()
        _ffi.check(_ffi.lib().lc_batch_set_constraint_stiffness(self.h, _p(ks), _p(kb), 0),
                   "lc_batch_set_constraint_stiffness")

    def set_initial(self, x0: torch.Tensor, v0: torch.Tensor) -> None:
        """The initial state with positions x0 (x and x_prev) and velocities v0."""
        self.load(self.initial)
        x0 = x0.detach().to("cuda", torch.float32).contiguous()
        v0 = v0.detach().to("cuda", torch.float32).contiguous()
        self.batch.write_state(x0.data_ptr(), x0.data_ptr(), v0.data_ptr(), False, self._stream())

    def positions(self) -> torch.Tensor:
        out = torch.empty((self.V, 3), dtype=torch.float32, device="cuda")
        self.batch.read_state(None, out.data_ptr(), None, False, self._stream())
        return out

    def adjoint_step(self, gx, gxp, gv, gks, gkb, exponent: torch.Tensor | None = None) -> None:
        """Reverse pass of one step; with exponent (int32, one per cloth) the
        rescaled form: a cloth's accumulators are scaled by 2^-60 whenever
        its state gradient passes 2^60, and exponent[c] counts the scalings."""
        if exponent is None:
            _ffi.check(_ffi.lib().lc_batch_adjoint_step(self.h, _p(gx), _p(gxp), _p(gv), _p(gks), _p(gkb),
                                                        self._sp()), "lc_batch_adjoint_step")
        else:
            _ffi.check(_ffi.lib().lc_batch_adjoint_step_rescaled(self.h, _p(gx), _p(gxp), _p(gv), _p(gks), _p(gkb),
                                                                 _p(exponent), self._sp()),
                       "lc_batch_adjoint_step_rescaled")

    def close(self) -> None:
        self.batch.close()


class ClothRollout(torch.autograd.Function):
    """final_positions = ClothRollout.apply(cloth, steps, k_stretch, k_bend, x0, v0)"""

    @staticmethod
    def forward(ctx, cloth: DiffCloth, steps: int, ks, kb, x0, v0):
        cloth.set_stiffness(ks, kb)
        cloth.set_initial(x0, v0)
        ckpts = []
        for n in range(steps):
            if n % cloth.every == 0:
                buf = cloth.new_state()
                cloth.save(buf)
                ckpts.append(buf)
            cloth.step(1)
        ctx.cloth, ctx.steps, ctx.ckpts = cloth, steps, ckpts
        ctx.params = (ks.detach().clone(), kb.detach().clone())
        return cloth.positions()

    @staticmethod
    def backward(ctx, g_out):
        cloth, steps = ctx.cloth, ctx.steps
        cloth.set_stiffness(*ctx.params)
        V = cloth.V
        gx = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        gxp = g_out.detach().to(torch.float32).contiguous().clone()
        gv = torch.zeros_like(gx)
        gks = torch.zeros(cloth.E, dtype=torch.float32, device="cuda")
        gkb = torch.zeros(cloth.B, dtype=torch.float32, device="cuda")
        ncl = len(cloth.batch.num_vertices)
        vcl = torch.repeat_interleave(torch.arange(ncl, device="cuda"),
                                      torch.tensor(cloth.batch.num_vertices, device="cuda"))
        counts = [cloth.batch.constraint_counts(c) for c in range(ncl)]
        ecl = torch.repeat_interleave(torch.arange(ncl, device="cuda"), torch.tensor([e for e, _ in counts], device="cuda"))
        bcl = torch.repeat_interleave(torch.arange(ncl, device="cuda"), torch.tensor([b for _, b in counts], device="cuda"))
        exp60 = torch.zeros(ncl, dtype=torch.int32, device="cuda")
        for seg in range(len(ctx.ckpts) - 1, -1, -1):
            first = seg * cloth.every
            last = min(steps, first + cloth.every)
            states = [ctx.ckpts[seg]]
            cloth.load(ctx.ckpts[seg])
            for _ in range(first, last - 1):
                cloth.step(1)
                buf = cloth.new_state()
                cloth.save(buf)
                states.append(buf)
            for n in range(last - 1, first - 1, -1):
                cloth.load(states[n - first])
                # Each cloth's reverse pass is linear in its seed: when a
                # cloth's state gradient passes 2^60 its accumulators are
                # scaled by 2^-60 on the device and its exponent counted, so
                # no intermediate product overflows in float; the results are
                # rescaled once at the end (to inf where the true gradient is
                # beyond float range).
                cloth.adjoint_step(gx, gxp, gv, gks, gkb, exp60)

        cloth.grad_exponent = exp60.clone()

        def unscale(t, idx):
            if not cloth.unscale:
                return t
            sc = torch.pow(torch.tensor(2.0 ** 60, device="cuda"), exp60.to(torch.float32))[idx]
            if t.dim() == 2:
                sc = sc.unsqueeze(1)
            return torch.where(t == 0, t, t * sc)
        return (None, None, unscale(gks, ecl), unscale(gkb, bcl), unscale(gx + gxp, vcl), unscale(gv, vcl))


def fit_cloth_stiffness(cloth: DiffCloth, steps: int, x0: torch.Tensor, v0: torch.Tensor, target: torch.Tensor,
                        k0: float = 0.9, iters: int = 8, step0: float = 0.1, k_range=(0.3, 0.98)):
    """Per-cloth stiffness recovered by gradient descent: every cloth of the
    batch has one stiffness k_c (its stretch and bend constraints share it),
    starting at k0; the loss is the summed squared distance of the positions
    after `steps` steps to `target`, each cloth's part depending only on its
    own k_c.  Each iteration runs the rollout and its reverse pass and moves
    every k_c by its own step against the sign of dL/dk_c (summed over the
    cloth's constraints), halving the step when the sign flips.  The
    direction comes from the reverse pass's scaled gradients
    (DiffCloth(unscale=False)), so it stays exact where the gradient's
    magnitude is beyond float range.  Returns (k, history) with history a
    list of (total loss, per-cloth losses) before each update."""
    C = len(cloth.batch.num_vertices)
    counts = [cloth.batch.constraint_counts(c) for c in range(C)]
    ecl = torch.repeat_interleave(torch.arange(C, device="cuda"), torch.tensor([e for e, _ in counts], device="cuda"))
    bcl = torch.repeat_interleave(torch.arange(C, device="cuda"), torch.tensor([b for _, b in counts], device="cuda"))
    vcl = torch.repeat_interleave(torch.arange(C, device="cuda"),
                                  torch.tensor(cloth.batch.num_vertices, device="cuda"))
    k = torch.full((C,), float(k0), device="cuda")
    step = torch.full((C,), float(step0), device="cuda")
    prev = torch.zeros(C, device="cuda")
    history = []
    for _ in range(iters):
        ks = k[ecl].clone().requires_grad_(True)
        kb = k[bcl].clone().requires_grad_(True)
        out = ClothRollout.apply(cloth, steps, ks, kb, x0, v0)
        per = torch.zeros(C, device="cuda").index_add_(0, vcl, ((out - target) ** 2).sum(dim=1))
        per.sum().backward()
        history.append((float(per.sum().detach()), per.detach().cpu().numpy()))
        with torch.no_grad():
            g = torch.zeros(C, device="cuda").index_add_(0, ecl, ks.grad).index_add_(0, bcl, kb.grad)
            sgn = torch.sign(g)
            step = torch.where(sgn * prev < 0, step * 0.5, step)
            k = torch.clamp(k - step * sgn, *k_range)
            prev = sgn
    return k, history
