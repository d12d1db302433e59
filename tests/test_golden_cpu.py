"""The oracle against the reference's own kernels (tests/golden/*.npz).

Each golden file holds a collision-stage input state and the outputs of the
reference's collision kernels, compiled from its sources and run on a GPU
(tests/golden/make_golden.py, oracle/ref_pin/).  The FP32 oracle must
reproduce every stage bit for bit: Morton codes, the stable sort, the Karras
hierarchy, the refit boxes and rightmost leaves, the broadphase pairs and the
VF / EE contacts (vertex ids and weights).
"""
from __future__ import annotations

import numpy as np
import pytest

import golden_cases

FILES = golden_cases.golden_files()


def test_golden_vectors_exist():
    assert len(FILES) >= len(golden_cases.CASES), "tests/golden holds no reference vectors"


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_oracle_matches_reference_kernels(path):
    d = golden_cases.load(path)
    spec = golden_cases.make_spec(d["case"])
    assert golden_cases.compare_oracle(spec, d) == []


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_golden_inputs_are_in_reference_layout(path):
    d = golden_cases.load(path)
    T = len(d["perm_before"])
    assert d["ref_node_min"].shape == (2 * T - 1, 3)
    assert d["ref_lefts"].shape == (T - 1,)
    assert np.all(np.diff(d["ref_morton"].astype(np.uint64).astype(object)) >= 0)
    assert sorted(d["ref_order"].tolist()) == list(range(T))
