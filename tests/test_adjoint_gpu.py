"""The engine's reverse pass (lc_batch_adjoint_step / ClothRollout) against
the FP64 adjoint of the oracle, whose own gradients are checked by finite
differences in tests/test_adjoint_cpu.py.

Both sides differentiate the same rollout: the engine in FP32 on its own
trajectory, the oracle in FP64 on its own; the rollouts are short and the
comparisons are on the whole gradient vector (relative L2 error), so that
the FP32 / FP64 difference of the trajectories stays well inside the bound.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from licenta_gb300 import scenes
from licenta_gb300.adjoint import ClothRollout, DiffCloth
from oracle.oracle_ffi import Oracle

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def engine_grads(spec, steps, ks, kb, v0, target, every):
    cloth = DiffCloth([spec], checkpoint_every=every)
    ks_t = torch.tensor(ks, dtype=torch.float32, device="cuda", requires_grad=True)
    kb_t = torch.tensor(kb, dtype=torch.float32, device="cuda", requires_grad=True)
    x0 = torch.tensor(spec.positions, dtype=torch.float32, device="cuda", requires_grad=True)
    v0_t = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    out = ClothRollout.apply(cloth, steps, ks_t, kb_t, x0, v0_t)
    loss = ((out - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    res = dict(loss=float(loss.detach()), ks=ks_t.grad.cpu().numpy(), kb=kb_t.grad.cpu().numpy(),
               x0=x0.grad.cpu().numpy(), v0=v0_t.grad.cpu().numpy(), final=out.detach().cpu().numpy())
    cloth.close()
    return res


def oracle_grads(spec, steps, ks, kb, v0, target):
    o = Oracle([spec], fp64=True)
    st = o.get_state(0)
    o.set_state(0, x=st["x"], x_prev=st["x"], v=v0, vn=st["vn"])
    o.set_stiffness_d(0, ks, kb)
    o.adj_record(0, steps)
    xp = o.get_state(0)["x_prev"]
    z = np.zeros_like(xp)
    gx, gxp, gv, gks, gkb = o.adj_backward(0, z, 2 * (xp - target), z)
    o.close()
    return dict(loss=float(((xp - target) ** 2).sum()), ks=gks, kb=gkb, x0=gx + gxp, v0=gv, final=xp)


def case(seed, n, steps, v_scale, iterations=10):
    spec = scenes.small_cloth(seed=seed, n=n, iterations=iterations)
    o = Oracle([spec], fp64=True)
    _, _, ne, nb = o.sizes(0)
    o.close()
    rng = np.random.default_rng(seed)
    ks = 0.9 + rng.uniform(-0.1, 0.05, ne)
    kb = 0.9 + rng.uniform(-0.1, 0.05, nb)
    v0 = rng.normal(scale=v_scale, size=(spec.num_vertices, 3)) * (spec.pinned == 0)[:, None]
    target = spec.positions + rng.normal(scale=0.05, size=(spec.num_vertices, 3)) - np.array([0.0, 0.2, 0.0])
    return spec, ks, kb, v0, target


def test_engine_adjoint_matches_fp64_adjoint():
    spec, ks, kb, v0, target = case(1, 12, 10, 0.3)
    g = engine_grads(spec, 10, ks, kb, v0, target, every=4)
    r = oracle_grads(spec, 10, ks, kb, v0, target)
    assert np.abs(g["final"] - r["final"]).max() < 1e-5
    for k in ("ks", "kb", "v0", "x0"):
        assert rel_l2(g[k], r[k]) < 2e-3, f"{k}: relative error {rel_l2(g[k], r[k]):.2e}"


def test_batch_of_unequal_iteration_counts_matches_fp64():
    """Two cloths in one differentiable batch, with 10 and 6 solver
    iterations: the recorded step runs on the batch's solver and, for the
    shorter cloth, repeats its last iterate in the tape for the iterations it
    does not run.  Each cloth's gradients must match the FP64 adjoint of that
    cloth alone (the cloths are independent)."""
    a = case(1, 12, 10, 0.3)
    b = case(5, 10, 10, 0.3, iterations=6)
    specs = [a[0], b[0]]
    cloth = DiffCloth(specs, checkpoint_every=4)
    cat = lambda i: np.concatenate([a[i], b[i]]).astype(np.float32)
    ks_t = torch.tensor(cat(1), device="cuda", requires_grad=True)
    kb_t = torch.tensor(cat(2), device="cuda", requires_grad=True)
    x0 = torch.tensor(np.concatenate([x.positions for x in specs]), device="cuda", requires_grad=True)
    v0_t = torch.tensor(cat(3), device="cuda", requires_grad=True)
    out = ClothRollout.apply(cloth, 10, ks_t, kb_t, x0, v0_t)
    loss = ((out - torch.tensor(cat(4), device="cuda")) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    got = dict(ks=ks_t.grad.cpu().numpy(), kb=kb_t.grad.cpu().numpy(), x0=x0.grad.cpu().numpy(),
               v0=v0_t.grad.cpu().numpy(), final=out.detach().cpu().numpy())
    cloth.close()
    off = dict(ks=0, kb=0, x0=0, v0=0, final=0)
    for spec, (sp, ks, kb, v0, target) in zip(specs, (a, b)):
        r = oracle_grads(sp, 10, ks, kb, v0, target)
        size = dict(ks=len(ks), kb=len(kb), x0=sp.num_vertices, v0=sp.num_vertices, final=sp.num_vertices)
        part = {k: got[k][off[k]:off[k] + size[k]] for k in size}
        assert np.abs(part["final"] - r["final"]).max() < 1e-5
        for k in ("ks", "kb", "v0", "x0"):
            assert rel_l2(part[k], r[k]) < 2e-3, f"{sp.params.solverIterations} iterations, {k}"
        for k in size:
            off[k] += size[k]


def test_checkpointing_does_not_change_gradients():
    spec, ks, kb, v0, target = case(3, 14, 12, 0.2)
    a = engine_grads(spec, 12, ks, kb, v0, target, every=12)
    b = engine_grads(spec, 12, ks, kb, v0, target, every=5)
    for k in ("ks", "kb", "v0", "x0"):
        assert rel_l2(b[k], a[k]) < 1e-6, k


def test_stiffness_recovered_by_gradient_descent():
    """The differentiable-rollout workload in small: the target comes from a
    rollout with stiffness 0.7 and wind; starting from 0.9, a few steps of
    gradient descent on the per-constraint stiffness lower the loss."""
    spec = scenes.small_cloth(seed=6, n=16)
    tgt_spec = scenes.small_cloth(seed=6, n=16, stiffness=0.7)
    scenes.set_constant_wind(tgt_spec.params, (1.5, 0.0, 0.5))
    steps = 20
    o = Oracle([tgt_spec], fp64=False)
    o.step(steps, threads=1)
    target = torch.tensor(o.get_state(0)["x_prev"], dtype=torch.float32, device="cuda")
    o.close()
    cloth = DiffCloth([spec], checkpoint_every=5)
    ks = torch.full((cloth.E,), 0.9, device="cuda", requires_grad=True)
    kb = torch.full((cloth.B,), 0.9, device="cuda", requires_grad=True)
    x0 = torch.tensor(spec.positions, device="cuda")
    v0 = torch.zeros_like(x0)
    losses = []
    for _ in range(4):
        out = ClothRollout.apply(cloth, steps, ks, kb, x0, v0)
        loss = ((out - target) ** 2).sum()
        losses.append(float(loss))
        ks.grad = kb.grad = None
        loss.backward()
        with torch.no_grad():
            for p in (ks, kb):
                p -= 0.5 * p.grad / (p.grad.abs().max() + 1e-12) * 0.02
                p.clamp_(0.05, 0.99)
    cloth.close()
    assert losses[-1] < losses[0], losses


def test_rescaled_reverse_pass_is_exact():
    """Contact-rich rollouts amplify the reverse pass by up to ~1e14 per 20
    steps; ClothRollout.backward scales a cloth's accumulators by 2^-60 when
    they pass 2^60 and rescales at the end.  The reverse pass is linear in its
    seed and a power-of-two scaling is exact in floating point, so a seed
    2^70 times larger on one cloth (which triggers its scaling) must give that
    cloth's gradients 2^70 times larger and leave the other cloth's alone."""
    specs = [scenes.small_cloth(seed=21, n=12), scenes.small_cloth(seed=22, n=10)]
    cloth = DiffCloth(specs, checkpoint_every=4)
    x0 = torch.tensor(np.concatenate([s.positions for s in specs]), device="cuda")
    n0 = specs[0].num_vertices
    grads = []
    for big in (False, True):
        ks = torch.full((cloth.E,), 0.9, device="cuda", requires_grad=True)
        kb = torch.full((cloth.B,), 0.9, device="cuda", requires_grad=True)
        xi = x0.clone().requires_grad_(True)
        v0 = torch.zeros_like(x0, requires_grad=True)
        out = ClothRollout.apply(cloth, 10, ks, kb, xi, v0)
        seed = torch.ones_like(out)
        if big:
            seed[:n0] *= 2.0 ** 70  # only the first cloth's seed is large
        out.backward(seed)
        grads.append([t.grad.clone() for t in (ks, kb, xi, v0)])
    cloth.close()
    small, large = grads
    from licenta_gb300 import ClothBatch
    b = ClothBatch(specs)
    ce, cb = b.constraint_counts(0)
    b.close()
    s = 2.0 ** 70
    for g_s, g_l, k in zip(small, large, (ce, cb, n0, n0)):
        # first cloth: scaled by 2^70 (exact up to subnormals of the small run)
        a, b_ = g_s[:k] * s, g_l[:k]
        assert torch.allclose(a, b_, rtol=1e-6, atol=float(b_.abs().max()) * 1e-9)
        assert torch.equal(g_s[k:], g_l[k:])  # second cloth: untouched
    assert torch.isfinite(large[0]).all()


def test_rescaled_entry_matches_plain_entry():
    """lc_batch_adjoint_step_rescaled against lc_batch_adjoint_step on the same
    state and seeds: a cloth whose state gradient passes 2^60 comes back
    scaled by exactly 2^-60 with its exponent counted, the other comes back
    bit-identical with exponent 0.  The calls alternate two flag buffers, so
    the sequence (plain, large, plain, plain) checks that a raised flag is
    cleared before either buffer is used again."""
    specs = [scenes.small_cloth(seed=31, n=12), scenes.small_cloth(seed=32, n=10)]
    cloth = DiffCloth(specs, checkpoint_every=4)
    x0 = torch.tensor(np.concatenate([s.positions for s in specs]), device="cuda")
    cloth.set_stiffness(torch.full((cloth.E,), 0.9, device="cuda"), torch.full((cloth.B,), 0.9, device="cuda"))
    cloth.set_initial(x0, torch.zeros_like(x0))
    cloth.step(3)
    state = cloth.new_state()
    cloth.save(state)
    n0, V = specs[0].num_vertices, cloth.V
    ce, cb = cloth.batch.constraint_counts(0)
    gen = torch.Generator(device="cuda")
    for k, scale in enumerate((1.0, 2.0 ** 70, 1.0, 1.0)):
        gen.manual_seed(5 + k)
        seeds = [torch.randn((V, 3), device="cuda", generator=gen) for _ in range(3)]
        for t in seeds:
            t[:n0] *= scale
        runs = []
        for rescaled in (False, True):
            g = [t.clone() for t in seeds] + [torch.zeros(cloth.E, device="cuda"), torch.zeros(cloth.B, device="cuda")]
            exponent = torch.zeros(2, dtype=torch.int32, device="cuda")
            cloth.load(state)
            cloth.adjoint_step(*g, exponent if rescaled else None)
            runs.append((g, exponent))
        torch.cuda.synchronize()
        (plain, _), (scaled, exponent) = runs
        assert exponent.tolist() == ([1, 0] if scale > 1.0 else [0, 0])
        f = 2.0 ** (60 * int(exponent[0]))
        for a, b, n in zip(plain, scaled, (n0, n0, n0, ce, cb)):
            want, got = a[:n], b[:n] * f
            normal = want.abs() >= 2.0 ** -60  # normal after the 2^-60 scaling: exact
            assert torch.equal(got[normal], want[normal])
            assert float((got - want).abs().max()) <= 2.0 ** -80
            assert torch.equal(a[n:], b[n:])
    cloth.close()


def test_engine_reverse_steps_at_the_workload_size(parity_report):
    """The reverse pass of every step of the differentiable-rollout workload
    (a 64 x 64 cloth, 60 steps, 10 iterations, stiffness 0.9, zero initial
    velocities) against the FP64 adjoint of the same step: before each step
    the oracle takes the engine's state, and after it the engine's contacts
    and discrete decisions, so both differentiate the same piecewise-smooth
    branch from the same point; both reverse the step with the same random
    seed gradients.  (Run freely, the FP32 and FP64 rollouts of this cloth
    find different self-contacts after a few dozen steps and end centimetres
    apart, so their whole-rollout gradients are gradients of different
    trajectories; the whole-rollout comparison is the small case above.)

    The reference's bend formula takes raw positions and is singular where
    a hinge reaches n1.n2 = +-1 (a cloth lying on the ground plane y = 0, a
    plane through the origin, puts hinges there).  A step whose solve brings
    a hinge within 1 - n1.n2 < 1e-7 or 1 + n1.n2 < 1e-11 is excused
    (test_adjoint_cpu.py shows the FP32 restatement failing at such steps
    and only there); every other step must agree to 2e-3 (relative L2, the
    state gradients (x, x_prev, v) as one vector, so that a part that
    cancels to nothing in FP64 is measured on the scale of the others).  On
    the excused steps the engine's error is set beside the FP32
    restatement's, taught the same state: it must be finite and not
    systematically larger (median ratio <= 3)."""
    from oracle import parity
    from oracle.parity import SINGULAR_FWD, SINGULAR_NEG
    spec = scenes.adjoint_cloth(seed=0)
    steps = 60
    cloth = DiffCloth([spec], checkpoint_every=10, debug_capture=True)
    b = cloth.batch
    V = spec.num_vertices
    o64, o32 = Oracle([spec], fp64=True), Oracle([spec], fp64=False)
    _, _, ne, nb = o64.sizes(0)
    for o in (o64, o32):
        o.set_stiffness_d(0, np.full(ne, 0.9), np.full(nb, 0.9))
    o64.track_bend(0, True)
    cloth.set_stiffness(torch.full((cloth.E,), 0.9, device="cuda"), torch.full((cloth.B,), 0.9, device="cuda"))
    x0 = torch.tensor(spec.positions, device="cuda")
    cloth.set_initial(x0, torch.zeros_like(x0))
    rng = np.random.default_rng(7)

    def err(got, want):
        return max(rel_l2(np.concatenate([a.ravel() for a in got[:3]]), np.concatenate([a.ravel() for a in want[:3]])),
                   rel_l2(got[3], want[3]), rel_l2(got[4], want[4]))

    worst_x, worst_ok, ratios = 0.0, 0.0, []
    contacts, ok_contacts, ok_steps = 0, 0, 0
    try:
        for n in range(steps):
            st, perm = parity.capture_pre(b, 0)
            seeds = [rng.normal(size=(V, 3)).astype(np.float32) for _ in range(3)]
            g = [torch.tensor(a, device="cuda") for a in seeds] + [torch.zeros(cloth.E, device="cuda"),
                                                                   torch.zeros(cloth.B, device="cuda")]
            cloth.adjoint_step(*g)
            torch.cuda.synchronize()
            got = [t.cpu().numpy() for t in g]
            assert all(np.isfinite(a).all() for a in got), f"step {n}: non-finite gradient"
            vf, ee = b.debug(0, "VF"), b.debug(0, "EE")
            nc = len(vf[0]) + len(ee[0])
            contacts += nc
            dec = (b.debug(0, "GROUND"), b.debug(0, "GROUND_ACTIVE"), b.debug(0, "LRA"), b.debug(0, "DYN_ACTIVE"))
            want = {}
            for tag, o in (("64", o64), ("32", o32)):
                o.set_state(0, **{k: a.astype(np.float64) for k, a in st.items()})
                o.set_perm(0, perm)
                o.freeze_contacts(0, vf, ee)
                o.force_decisions(0, *dec)
                o.adj_clear(0)
                o.adj_record(0, 1)
                want[tag] = o.adj_backward(0, *seeds)
            worst_x = max(worst_x, float(np.abs(b.get_state(0)["x"] - o64.get_state(0)["x"]).max()))
            fwd, neg = o64.hinge_conditioning(0)
            e_engine = err(got, want["64"])
            if fwd >= SINGULAR_FWD and neg >= SINGULAR_NEG:
                ok_steps += 1
                ok_contacts += nc
                worst_ok = max(worst_ok, e_engine)
            else:
                ratios.append(e_engine / max(err(want["32"], want["64"]), 1e-30))
    finally:
        cloth.close()
        o64.close()
        o32.close()
    med = float(np.median(ratios)) if ratios else 0.0
    parity_report(steps=steps, contacts=contacts, well_conditioned_steps=ok_steps, ok_contacts=ok_contacts,
                  max_rel_well_conditioned=f"{worst_ok:.2e}", singular_steps=len(ratios),
                  median_engine_over_fp32_singular=f"{med:.2f}", max_x=f"{worst_x:.2e}")
    assert ok_contacts > 0, "the well-conditioned steps should include self-contact"
    assert ok_steps >= steps // 2, f"only {ok_steps} steps clear of the bend singularities"
    assert worst_x <= 1e-5
    assert worst_ok < 2e-3, f"well-conditioned step: relative error {worst_ok:.2e}"
    assert med <= 3.0, f"engine error {med:.2f} x the FP32 restatement's on the singular steps"
