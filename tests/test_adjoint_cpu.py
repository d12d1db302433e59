"""The FP64 adjoint of the cloth step (oracle/lc_oracle.hpp, Cloth::backward)
against central finite differences of the FP64 oracle.

The step is piecewise smooth: contacts, ground / LRA activation and which
contact terms count change discretely.  The rollout is recorded once and every
finite-difference evaluation replays its decisions (Oracle.adj_replay), so
both sides differentiate the same branch.  The loss is the summed squared
distance of the final positions (x_prev after the last step, the positions the
reference publishes) to a target.
"""
from __future__ import annotations

import numpy as np
import pytest

from licenta_gb300 import scenes
from oracle.oracle_ffi import Oracle
from oracle.parity import SINGULAR_FWD, SINGULAR_NEG


class Rollout:
    def __init__(self, spec, warm_steps=0, seed=0, v_scale=0.0):
        self.o = Oracle([spec], fp64=True)
        self.nv, _, self.ne, self.nb = self.o.sizes(0)
        if warm_steps:
            self.o.step(warm_steps, threads=1)
        self.st0 = self.o.get_state(0)
        self.perm0 = self.o.perm(0)
        rng = np.random.default_rng(seed)
        self.v0 = self.st0["v"] + rng.normal(scale=v_scale, size=(self.nv, 3)) * (spec.pinned == 0)[:, None]
        self.ks0 = 0.9 + rng.uniform(-0.1, 0.05, self.ne)
        self.kb0 = 0.9 + rng.uniform(-0.1, 0.05, self.nb)
        self.target = self.st0["x_prev"] + rng.normal(scale=0.05, size=(self.nv, 3))

    def reset(self, x=None, xp=None, v=None, ks=None, kb=None):
        st = self.st0
        self.o.set_state(0, x=st["x"] if x is None else x, x_prev=st["x_prev"] if xp is None else xp,
                         v=self.v0 if v is None else v, vn=st["vn"])
        self.o.set_perm(0, self.perm0)
        self.o.set_stiffness_d(0, self.ks0 if ks is None else ks, self.kb0 if kb is None else kb)

    def loss(self):
        return float(((self.o.get_state(0)["x_prev"] - self.target) ** 2).sum())

    def record(self, steps):
        self.steps = steps
        self.reset()
        self.o.adj_clear(0)
        self.o.adj_record(0, steps)
        xp = self.o.get_state(0)["x_prev"]
        z = np.zeros((self.nv, 3))
        return self.o.adj_backward(0, z, 2 * (xp - self.target), z)

    def fd(self, **perturbed):
        vals = []
        for sgn in (1, -1):
            self.reset(**{k: f(sgn) for k, f in perturbed.items()})
            self.o.adj_replay(0, 0, self.steps)
            vals.append(self.loss())
        self.reset()
        return vals


def check(ad, fd_vals, eps, rtol=1e-3, atol=1e-6):
    """Relative 1e-3, with an absolute floor: a folded rollout amplifies the
    loss's rounding, which puts about 1e-7..1e-6 of noise on a difference
    quotient (the gradients checked are 1e-4..1e-1)."""
    fd = (fd_vals[0] - fd_vals[1]) / (2 * eps)
    assert abs(ad - fd) <= rtol * abs(fd) + atol, f"adjoint {ad:.8g} vs finite difference {fd:.8g}"


def test_adjoint_matches_finite_differences_hanging_cloth():
    spec = scenes.small_cloth(seed=1, n=10)
    r = Rollout(spec, v_scale=0.3)
    gx, gxp, gv, gks, gkb = r.record(8)
    rng = np.random.default_rng(5)
    eps = 1e-3
    for c in rng.choice(r.ne, 4, replace=False):
        check(gks[c], r.fd(ks=lambda s, c=c: r.ks0 + s * eps * (np.arange(r.ne) == c)), eps)
    for c in rng.choice(r.nb, 4, replace=False):
        check(gkb[c], r.fd(kb=lambda s, c=c: r.kb0 + s * eps * (np.arange(r.nb) == c)), eps)
    free = np.where(spec.pinned == 0)[0]
    for i in rng.choice(free, 3, replace=False):
        for d in range(3):
            e = np.zeros((r.nv, 3)); e[i, d] = eps
            check(gv[i, d], r.fd(v=lambda s, e=e: r.v0 + s * e), eps)
    # a pinned vertex: its position enters x and x_prev (kept off the world
    # clamp at z = 0 by a step smaller than its jitter)
    p = int(np.where(spec.pinned)[0][0])
    for d, e_d in ((0, 1e-3), (1, 1e-3), (2, 1e-6)):
        e = np.zeros((r.nv, 3)); e[p, d] = e_d
        x0 = r.st0["x"]
        vals = r.fd(x=lambda s, e=e: x0 + s * e, xp=lambda s, e=e: x0 + s * e)
        check(gx[p, d] + gxp[p, d], vals, e_d)


def test_adjoint_matches_finite_differences_through_contacts():
    spec = scenes.small_cloth(seed=0, n=20)
    r = Rollout(spec, warm_steps=55, seed=1)
    gx, gxp, gv, gks, gkb = r.record(6)
    rng = np.random.default_rng(2)
    eps = 1e-3
    for c in rng.choice(r.ne, 5, replace=False):
        check(gks[c], r.fd(ks=lambda s, c=c: r.ks0 + s * eps * (np.arange(r.ne) == c)), eps)
    for c in rng.choice(r.nb, 5, replace=False):
        check(gkb[c], r.fd(kb=lambda s, c=c: r.kb0 + s * eps * (np.arange(r.nb) == c)), eps)
    free = np.where(spec.pinned == 0)[0]
    for i in rng.choice(free, 3, replace=False):
        for d in range(3):
            e = np.zeros((r.nv, 3)); e[i, d] = eps
            check(gv[i, d], r.fd(v=lambda s, e=e: r.v0 + s * e), eps)
            # positions: a step well below a millimetre, so that no vertex
            # crosses the world clamp (many lie outside the unit box here)
            e = np.zeros((r.nv, 3)); e[i, d] = 1e-6
            check(gxp[i, d], r.fd(xp=lambda s, e=e: r.st0["x_prev"] + s * e), 1e-6)


def test_adjoint_at_the_workload_size_matches_finite_differences():
    """The differentiable-rollout workload's cloth (64 x 64, 10 iterations,
    stiffness 0.9, zero initial velocities; the target is the final state of
    a forward run with stiffness 0.7 and wind (1.5, 0, 0.5) m/s^2): the FP64
    adjoint's directional derivatives along a random direction of the
    per-constraint stiffnesses and one of the initial velocities against
    central finite differences of the rollout replaying the recorded
    decisions, over 50 steps.

    The cloth folds onto itself and the rollout is chaotic: its gradient
    grows from 6e-4 (10 steps) to 2e2 (50) and 8e5 (60) in the largest
    stiffness entry, so a central difference with eps 1e-3 is far outside
    the linear range past about 20 steps.  At 50 steps the difference
    quotients converge to the adjoint as eps shrinks (eps 1e-7: 3e-5
    relative); at 60 they scatter by 15% between eps 1e-8 and 1e-11 (the
    curvature, then FP64 rounding of the loss, dominates), so no finite
    difference resolves the 60-step gradient.  The engine's reverse pass is
    compared with this adjoint step by step over all 60 steps
    (tests/test_adjoint_gpu.py)."""
    spec = scenes.adjoint_cloth(seed=0)
    tgt = scenes.adjoint_cloth(seed=0, stiffness=0.7, wind=(1.5, 0.0, 0.5))
    steps = 50
    t = Oracle([tgt], fp64=True)
    t.step(steps, threads=1)
    target = t.get_state(0)["x_prev"]
    t.close()
    r = Rollout(spec)
    r.ks0[:] = 0.9
    r.kb0[:] = 0.9
    r.v0 = np.zeros_like(r.v0)
    r.target = target
    gx, gxp, gv, gks, gkb = r.record(steps)
    rng = np.random.default_rng(3)
    eps = 1e-7
    dk, db = rng.normal(size=r.ne), rng.normal(size=r.nb)
    norm = np.sqrt((dk ** 2).sum() + (db ** 2).sum())
    dk, db = dk / norm, db / norm
    check(float(gks @ dk + gkb @ db), r.fd(ks=lambda s: r.ks0 + s * eps * dk, kb=lambda s: r.kb0 + s * eps * db), eps)
    dv = rng.normal(size=(r.nv, 3)) * (spec.pinned == 0)[:, None]
    dv /= np.linalg.norm(dv)
    check(float((gv * dv).sum()), r.fd(v=lambda s: r.v0 + s * eps * dv), eps)


def test_fp32_reverse_steps_differ_from_fp64_only_at_singular_hinges():
    """The FP32 restatement, stepped freely through the 64 x 64 workload (60
    steps), reversed one step at a time against the FP64 adjoint taught the
    same state, contacts and decisions.  Every step whose gradients differ
    by more than 2e-3 (relative L2, the state gradients taken as one vector)
    has a bend hinge near a singularity of the reference's raw-position bend
    formula during its solve (oracle.parity.SINGULAR_FWD / SINGULAR_NEG); some of them
    differ by more than 10%, in FP32 arithmetic alone (no GPU involved).
    The engine's per-step reverse comparison excuses the same steps."""
    def rel(a, b):
        a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))

    spec = scenes.adjoint_cloth(seed=0)
    V = spec.num_vertices
    o32, o64 = Oracle([spec], fp64=False), Oracle([spec], fp64=True)
    try:
        _, _, ne, nb = o64.sizes(0)
        for o in (o32, o64):
            o.set_stiffness_d(0, np.full(ne, 0.9), np.full(nb, 0.9))
        o64.track_bend(0, True)
        rng = np.random.default_rng(7)
        worst, unexplained, contacts = 0.0, [], 0
        for n in range(60):
            st, perm = o32.get_state(0), o32.perm(0)
            seeds = [rng.normal(size=(V, 3)) for _ in range(3)]
            o32.adj_clear(0)
            o32.adj_record(0, 1)
            g = o32.adj_backward(0, *seeds)
            vf, ee = o32.debug(0, "VF"), o32.debug(0, "EE")
            contacts += len(vf[0]) + len(ee[0])
            dd = o32.solve_decisions(0)
            o64.set_state(0, **{k: a.astype(np.float64) for k, a in st.items()})
            o64.set_perm(0, perm)
            o64.freeze_contacts(0, vf, ee)
            o64.force_decisions(0, dd["ground"], dd["ground_it"], dd["lra"], dd["dyn"])
            o64.adj_clear(0)
            o64.adj_record(0, 1)
            r = o64.adj_backward(0, *seeds)
            assert all(np.isfinite(a).all() for a in g)
            e = max(rel(np.concatenate([a.ravel() for a in g[:3]]), np.concatenate([a.ravel() for a in r[:3]])),
                    rel(g[3], r[3]), rel(g[4], r[4]))
            worst = max(worst, e)
            fwd, neg = o64.hinge_conditioning(0)
            if e > 2e-3 and fwd >= SINGULAR_FWD and neg >= SINGULAR_NEG:
                unexplained.append((n, e))
    finally:
        o32.close()
        o64.close()
    assert contacts > 0
    assert not unexplained, f"steps differing at well-conditioned hinges: {unexplained}"
    assert worst > 1e-1, "the singular hinges should show in FP32"


def test_adjoint_matches_finite_differences_on_a_static_collider():
    """A 12 x 12 cloth warmed for 14 steps until it lies on an icosphere
    collider (lc_batch_set_collider), then 6 recorded steps: the reverse of
    the collider's projections (the contact planes held as recorded) against
    finite differences that replay the recorded contacts."""
    spec = scenes.icosphere_cloth(seed=4, n=12, depth=2, radius=0.3, height=0.45, span=0.6)
    r = Rollout(spec, warm_steps=14, seed=3)
    r.record(1)
    ids, _ = r.o.debug(0, "COLLIDER")
    assert (ids[:, 1] >= 0).sum() > 10, "the cloth should touch the collider"
    gx, gxp, gv, gks, gkb = r.record(6)
    rng = np.random.default_rng(8)
    eps = 1e-4
    for c in rng.choice(r.ne, 5, replace=False):
        check(gks[c], r.fd(ks=lambda s, c=c: r.ks0 + s * eps * (np.arange(r.ne) == c)), eps)
    for c in rng.choice(r.nb, 3, replace=False):
        check(gkb[c], r.fd(kb=lambda s, c=c: r.kb0 + s * eps * (np.arange(r.nb) == c)), eps)
    touching = np.unique(ids[ids[:, 1] >= 0][:, 0])
    for i in rng.choice(touching, 3, replace=False):
        for d in range(3):
            e = np.zeros((r.nv, 3)); e[i, d] = eps
            check(gv[i, d], r.fd(v=lambda s, e=e: r.v0 + s * e), eps)
            e = np.zeros((r.nv, 3)); e[i, d] = 1e-6
            check(gxp[i, d], r.fd(xp=lambda s, e=e: r.st0["x_prev"] + s * e), 1e-6)
