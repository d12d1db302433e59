"""The launch-shape autotuner (licenta_gb300/autotune.py).

Block and grid sizes must not change results: a batch stepped with tuned
shapes (solver variant held) equals, bit for bit, the same batch stepped with
the default shapes.  The tuner must leave the batch's state as it found it,
and a second run must take the cached shapes.
"""
from __future__ import annotations

import numpy as np
import pytest

from licenta_gb300 import ClothBatch, autotune, scenes

pytestmark = pytest.mark.gpu


def test_tuned_shapes_give_identical_steps(tmp_path):
    specs = scenes.batched_cloths(seed=13, count=6, n_min=10, n_max=40)
    ref = ClothBatch(specs)
    ref.step(8)
    ref.sync()
    want = ref.read_positions()
    ref.close()

    b = ClothBatch(specs)
    space = {"traverse_block": (64, 256), "jacobi_block": (128,), "narrow_blocks_per_sm": (4, 16),
             "solver_variant": (3,)}
    before = b.read_positions()
    r = autotune.autotune(b, steps=2, warmup=1, space=space, cache=tmp_path / "tune.json")
    assert not r["cached"] and len(r["tried"]) == 4
    assert np.array_equal(b.read_positions(), before), "the tuner must restore the state"
    b.step(8)
    b.sync()
    assert np.array_equal(b.read_positions(), want)
    r2 = autotune.autotune(b, space=space, cache=tmp_path / "tune.json")
    assert r2["cached"] and r2["config"] == r["config"]
    b.close()


def test_variant_search_stays_within_tolerance(tmp_path):
    specs = scenes.batched_cloths(seed=14, count=4, n_min=12, n_max=30)
    b = ClothBatch(specs)
    r = autotune.autotune(b, steps=1, warmup=1, space={"traverse_block": (128,), "jacobi_block": (256,),
                                                        "narrow_blocks_per_sm": (8,), "solver_variant": (1, 2, 3)},
                          cache=None)
    assert {t["config"]["solver_variant"] for t in r["tried"]} == {1, 2, 3}
    b.step(3)
    b.sync()
    b.close()
