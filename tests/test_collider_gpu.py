"""Static triangle colliders (lc_batch_set_collider) on the GPU against the
oracle, through the C ABI: every step's collider contacts (face and plane
of each slot) bit-exact against the FP32 restatement run on the engine's
predicted state, together with the self-collision stages, and positions
within 1e-5 m of the FP64 oracle taught the engine's contacts, in each
solver variant; a batch mixing cloths with and without colliders; the slot
capacity error; and the adjoint batch's refusal."""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from licenta_gb300 import ClothBatch, _ffi, scenes
from oracle import parity

pytestmark = pytest.mark.gpu

POS_TOL = 1e-5  # metres, on a 1 m cloth


@pytest.mark.parametrize("variant", [1, 2, 3], ids=["gather", "cluster", "scatter"])
def test_cloth_dropped_on_an_icosphere(parity_report, variant):
    """A 32 x 32 cloth dropped onto an icosphere of subdivision 3 (1,280
    faces, r 0.3 m): it lands at step 11 and slides off after step 30."""
    spec = scenes.icosphere_cloth(seed=0)
    worst, contacts, excused, checked = parity.run_parity([spec], steps=40, variant=variant, tol=POS_TOL)
    parity_report(steps=checked, worst_m=f"{worst:.2e}", excused=excused, contacts=contacts)
    assert contacts > 1000


def test_batch_mixing_colliders_and_none(parity_report):
    specs = [scenes.icosphere_cloth(seed=1, n=24),
             scenes.small_cloth(seed=2, n=16),
             scenes.icosphere_cloth(seed=3, n=20, depth=2, radius=0.25, height=0.4)]
    worst, contacts, excused, checked = parity.run_parity(specs, steps=30, tol=POS_TOL)
    parity_report(steps=checked, worst_m=f"{worst:.2e}", excused=excused, contacts=contacts)
    assert contacts > 0


def test_removing_the_collider_clears_its_contacts():
    spec = scenes.icosphere_cloth(seed=0, n=16)
    b = ClothBatch([spec], debug_capture=True)
    try:
        b.step(15)
        b.sync()
        ids, _ = b.debug(0, "COLLIDER")
        assert (ids[:, 1] >= 0).any()
        b.set_collider(0, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
        b.step(1)
        b.sync()
        ids, _ = b.debug(0, "COLLIDER")
        assert (ids[:, 1] < 0).all()
    finally:
        b.close()


def test_more_contacts_than_slots_is_a_capacity_error():
    """Nine copies of one face under every vertex: nine contacts where a
    vertex keeps LC_COLLIDER_SLOTS = 8; lc_batch_sync reports it, and the
    eight lowest faces are the ones kept (as the oracle keeps them)."""
    spec = scenes.icosphere_cloth(n=4, height=0.005, span=0.1)
    spec.params.gravity[:] = (0.0, 0.0, 0.0)
    tri_v = np.array([[-1.0, 0.0, -1.0], [0.0, 0.0, 1.0], [1.0, 0.0, -1.0]], np.float32)
    spec = replace(spec, collider=(np.tile(tri_v, (9, 1)), np.arange(27, dtype=np.uint32).reshape(9, 3), "ccw"))
    b = ClothBatch([spec], debug_capture=True)
    try:
        b.step(1)
        with pytest.raises(_ffi.LcError) as e:
            b.sync()
        assert e.value.status == _ffi.LC_ERR_CAPACITY_OVERFLOW
        ids, _ = b.debug(0, "COLLIDER")
        assert np.array_equal(ids[:8, 1], np.arange(8))
    finally:
        b.close()


def test_reverse_pass_through_the_collider_matches_the_fp64_adjoint():
    """A 12 x 12 cloth dropped onto an icosphere collider over 14 steps
    (collider contacts from step 3): the engine's gradients of the loss on the final
    positions with respect to the per-constraint stiffness, the initial
    positions and velocities, against the FP64 adjoint of the oracle, whose
    reverse of the collider projections is checked by finite differences in
    tests/test_adjoint_cpu.py."""
    import torch
    from licenta_gb300.adjoint import ClothRollout, DiffCloth
    from oracle.oracle_ffi import Oracle

    spec = scenes.icosphere_cloth(seed=4, n=12, depth=2, radius=0.3, height=0.4, span=0.6)
    steps = 14
    o = Oracle([spec], fp64=True)
    _, _, ne, nb = o.sizes(0)
    rng = np.random.default_rng(4)
    ks, kb = 0.9 + rng.uniform(-0.1, 0.05, ne), 0.9 + rng.uniform(-0.1, 0.05, nb)
    v0 = rng.normal(scale=0.2, size=(spec.num_vertices, 3))
    target = spec.positions + rng.normal(scale=0.05, size=(spec.num_vertices, 3)) - np.array([0.0, 0.3, 0.0])
    st = o.get_state(0)
    o.set_state(0, x=st["x"], x_prev=st["x"], v=v0, vn=st["vn"])
    o.set_stiffness_d(0, ks, kb)
    o.adj_record(0, steps)
    ids, _ = o.debug(0, "COLLIDER")
    xp = o.get_state(0)["x_prev"]
    z = np.zeros_like(xp)
    gx, gxp, gv, gks, gkb = o.adj_backward(0, z, 2 * (xp - target), z)
    o.close()
    want = dict(ks=gks, kb=gkb, x0=gx + gxp, v0=gv)

    cloth = DiffCloth([spec], checkpoint_every=5)
    try:
        t = dict(ks=torch.tensor(ks, dtype=torch.float32, device="cuda", requires_grad=True),
                 kb=torch.tensor(kb, dtype=torch.float32, device="cuda", requires_grad=True),
                 x0=torch.tensor(spec.positions, dtype=torch.float32, device="cuda", requires_grad=True),
                 v0=torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True))
        out = ClothRollout.apply(cloth, steps, t["ks"], t["kb"], t["x0"], t["v0"])
        loss = ((out - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
        loss.backward()
        torch.cuda.synchronize()
        final = out.detach().cpu().numpy()
        got = {k: v.grad.cpu().numpy() for k, v in t.items()}
    finally:
        cloth.close()
    assert (ids[:, 1] >= 0).sum() > 20, "the cloth should lie on the collider at the end"
    assert np.abs(final - xp).max() < 1e-5
    for k in ("ks", "kb", "v0", "x0"):
        e = float(np.linalg.norm(got[k] - want[k]) / np.linalg.norm(want[k]))
        assert e < 2e-3, f"{k}: relative error {e:.2e}"


def test_per_cloth_stiffness_recovered_on_icosphere_colliders(parity_report):
    """The batched differentiable workload in small (16 cloths, sides 32..128,
    each dropped onto its own icosphere of subdivision 4, radius 0.2..0.4 m):
    per-cloth stiffness recovered by gradient descent from 0.9 toward seeded
    targets in [0.5, 0.8] over a 30-step horizon (landing and drape), from
    the final positions of forward runs with the targets."""
    import torch
    from licenta_gb300.adjoint import ClothRollout, DiffCloth, fit_cloth_stiffness

    specs = scenes.batched_sphere_cloths(seed=0, count=16, mesh=True)
    steps = 30
    cloth = DiffCloth(specs, checkpoint_every=10, unscale=False)
    try:
        C = len(specs)
        counts = [cloth.batch.constraint_counts(c) for c in range(C)]
        kstar = torch.tensor(np.random.default_rng(1).uniform(0.5, 0.8, C), dtype=torch.float32, device="cuda")
        ecl = torch.repeat_interleave(torch.arange(C, device="cuda"), torch.tensor([e for e, _ in counts], device="cuda"))
        bcl = torch.repeat_interleave(torch.arange(C, device="cuda"), torch.tensor([b for _, b in counts], device="cuda"))
        x0 = torch.tensor(np.concatenate([s.positions for s in specs]), device="cuda")
        v0 = torch.zeros_like(x0)
        with torch.no_grad():
            target = ClothRollout.apply(cloth, steps, kstar[ecl], kstar[bcl], x0, v0).clone()
        k, hist = fit_cloth_stiffness(cloth, steps, x0, v0, target, iters=8)
    finally:
        cloth.close()
    e0 = float((0.9 - kstar).abs().mean())
    e1 = float((k - kstar).abs().mean())
    closer = float(((k - kstar).abs() < (0.9 - kstar).abs()).float().mean())
    parity_report(cloths=C, horizon=steps, mean_abs_k_error_start=f"{e0:.4f}", end=f"{e1:.4f}",
                  loss_start=f"{hist[0][0]:.3e}", loss_end=f"{hist[-1][0]:.3e}", closer_share=f"{closer:.2f}")
    assert e1 < 0.2 * e0
    assert closer >= 0.9
    assert hist[-1][0] < 0.1 * hist[0][0]
