"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, carries the reference defaults, and its host-side helpers
(mesh generators, Morton encoder) agree with the oracle."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from licenta_gb300 import _ffi, scenes

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = []
    for h in (ROOT / "include").rglob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(lc_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = _ffi.lib()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"
    # and the Python binding types every one of them
    untyped = [n for n in names if n not in _ffi.SIGNATURES]
    assert not untyped, f"not in _ffi.SIGNATURES: {untyped}"


def test_struct_layout_matches_header():
    # lc_cloth_params: 11 floats, 4 float3, 2 floats + int, 2 float3, int2, 3 ints,
    # u64, 3 ints, then the extension block
    assert C.sizeof(_ffi.Contact) == 32
    # lc_broadphase_desc: int, int, u64, 2 float3, int, float, int (+ tail padding to 8)
    assert _ffi.BroadphaseDesc.max_entries.offset == 8 and _ffi.BroadphaseDesc.table_size.offset == 48
    assert C.sizeof(_ffi.BroadphaseDesc) == 56 and C.sizeof(_ffi.BroadphaseCriteria) == 32
    assert _ffi.ClothParams.benchmarkSample.offset % 8 == 0
    assert _ffi.ClothDesc.params.offset % 8 == 0


def test_default_params_are_the_reference_defaults():
    p = _ffi.default_params()
    # Managers/MastersSimulationManager.cpp:33-62, Core/Utils.hpp:18-19
    assert p.BVHChunkSize == 64 and p.solverIterations == 6
    assert abs(p.kStretch - 0.99) < 1e-7 and abs(p.kBend - 0.1) < 1e-7
    assert abs(p.kDamp - 0.05) < 1e-7 and abs(p.globalVelDamp - 0.01) < 1e-7
    assert abs(p.strainLimit - 0.15) < 1e-7 and abs(p.objectMass - 0.525) < 1e-7
    assert abs(p.timestep - 1.0 / 60.0) < 1e-7
    assert tuple(p.worldMin) == (0, 0, 0) and tuple(p.worldMax) == (1, 1, 1)
    assert p.refLeafAabbQuirk == 1 and p.mortonMode == _ffi.LC_MORTON_REF63
    assert p.thicknessFromMesh == 1


def test_workload_generators_match_the_library():
    """scenes builds grids and default parameters without the library (so the
    CPU reference arm of the bench never loads it); they must be the
    library's lc_mesh_grid and lc_default_params byte for byte."""
    L = _ffi.lib()
    for n in (2, 3, 4, 16, 33, 192):
        t = L.lc_mesh_grid(n, n, None)
        want = np.empty((t, 3), dtype=np.uint32)
        L.lc_mesh_grid(n, n, want.ctypes.data_as(C.c_void_p))
        assert np.array_equal(scenes.grid_indices(n), want), n
    assert bytes(scenes.default_params()) == bytes(_ffi.default_params())


def test_invalid_arguments_are_rejected_before_any_device_work():
    L = _ffi.lib()
    h = C.c_void_p()
    assert L.lc_batch_create(None, 0, None, C.byref(h)) == 1
    assert L.lc_batch_step(None, 1, None) == 1
    assert L.lc_lbvh_create(0, 64, 0, C.byref(h)) == 1
    assert b"bad" in L.lc_last_error_string()
    assert L.lc_status_string(3) == b"contact capacity overflow"
    # a group needs distinct, non-null batches (checked before any device call)
    fake = (C.c_void_p * 2)(0x1000, 0x1000)
    assert L.lc_group_create(fake, 2, C.byref(h)) == 1
    assert b"twice" in L.lc_last_error_string()
    assert L.lc_group_create(None, 1, C.byref(h)) == 1
    assert L.lc_group_step(None, 1, None) == 1
    assert L.lc_group_step_io(None, 1, None, None, None, None, None, None, 1, None) == 1
    assert L.lc_batch_adjoint_step_rescaled(None, None, None, None, None, None, None, None) == 1
    assert b"exponent" in L.lc_last_error_string()


def test_grid_generator_matches_reference_topology_and_oracle():
    from oracle.oracle_ffi import lib as olib
    for n in (2, 3, 7, 32):
        idx = scenes.grid_indices(n)
        assert idx.shape == (2 * (n - 1) ** 2, 3)
        ref = np.empty_like(idx)
        olib().lco_grid_indices(n, n, ref.ctypes.data_as(C.c_void_p))
        assert np.array_equal(idx, ref)
    # Rendering/VisualBodyFactory.cpp:365-385 for the first two quads of a 3x3 grid
    idx = scenes.grid_indices(3)
    assert idx[:4].tolist() == [[0, 3, 1], [1, 3, 4], [1, 4, 5], [5, 2, 1]]


def test_icosphere_counts():
    for depth, t in ((1, 80), (4, 5120), (5, 20480)):
        v, idx = scenes.icosphere(depth)
        assert idx.shape == (t, 3) and v.shape == (3 * t // 2, 3)
        r = np.linalg.norm(v, axis=1)
        assert np.allclose(r, 1.0, atol=1e-6)


@pytest.mark.parametrize("mode", [_ffi.LC_MORTON_REF63, _ffi.LC_MORTON_K30])
def test_morton_encoder_matches_oracle(mode):
    from oracle.oracle_ffi import morton
    rng = np.random.default_rng(5)
    pts = np.concatenate([rng.uniform(-0.1, 1.1, size=(3000, 3)),
                          np.array([[0, 0, 0], [1, 1, 1], [0.5, 0.5, 0.5], [1 - 1e-7, 0, 1e-7]])]).astype(np.float32)
    L = _ffi.lib()
    for p in pts:
        a = L.lc_morton3d(float(p[0]), float(p[1]), float(p[2]), mode)
        b = morton(float(p[0]), float(p[1]), float(p[2]), mode)
        assert a == b
    # REF63: x*2^21 clamped; the top bit is never set, (1,1,1) saturates all 63 bits
    if mode == _ffi.LC_MORTON_REF63:
        assert L.lc_morton3d(1.0, 1.0, 1.0, mode) == (1 << 63) - 1
        assert L.lc_morton3d(0.5, 0.0, 0.0, mode) == 1 << 62
    else:
        assert L.lc_morton3d(1.0, 1.0, 1.0, mode) == (1 << 30) - 1


def test_group_orders():
    """ClothBatchGroup's cloth orders: the caller's, or by vertex count
    (largest first, ties in the caller's order), always a permutation."""
    from licenta_gb300 import ClothBatchGroup
    specs = scenes.batched_cloths(seed=3, count=12, n_min=8, n_max=20)
    assert ClothBatchGroup.group_order(specs) == list(range(12))
    o = ClothBatchGroup.group_order(specs, "size")
    assert sorted(o) == list(range(12))
    v = [specs[i].num_vertices for i in o]
    assert v == sorted(v, reverse=True)
    for a, b in zip(o, o[1:]):
        if specs[a].num_vertices == specs[b].num_vertices:
            assert a < b
    with pytest.raises(ValueError):
        ClothBatchGroup.group_order(specs, "random")
