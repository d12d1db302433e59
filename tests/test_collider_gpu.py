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


def test_adjoint_batches_refuse_colliders():
    spec = scenes.adjoint_cloth(seed=0, n=8)
    b = ClothBatch([spec], adjoint=True)
    try:
        v, i = scenes.icosphere(2, 0.3)
        with pytest.raises(_ffi.LcError) as e:
            b.set_collider(0, v, i, "cw")
        assert e.value.status == _ffi.LC_ERR_NOT_SUPPORTED
    finally:
        b.close()
