"""The C++ drop-in adapter (include/lc/lc_body.hpp) over the C ABI.

tests/cpp/body_demo.cpp uses lc::CudaDeformableBody as the reference's scene
code uses Physics::CudaDeformableBody (construct from a VertexFormat-shaped
vertex array, FixedUpdate + Update per frame).  The published positions must
equal, bit for bit, those of the Python binding stepping the same cloth.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from licenta_gb300 import ClothBatch, _build, _ffi, scenes

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "body_demo.cpp"
BP_SRC = ROOT / "tests" / "cpp" / "broadphase_demo.cpp"


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not available")
    return g


@pytest.mark.parametrize("src", [SRC, BP_SRC], ids=["body", "collision_method"])
def test_adapter_header_compiles(src):
    r = subprocess.run([_gxx(), "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("tune", [0, 1], ids=["default", "autotuned"])
def test_adapter_steps_like_the_binding(tmp_path, tune):
    lib = _build.build()
    exe = tmp_path / "body_demo"
    r = subprocess.run([_gxx(), "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(SRC), "-o", str(exe),
                        "-L", str(lib.parent), "-llicenta_gb300", f"-Wl,-rpath,{lib.parent}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    spec = scenes.small_cloth(seed=4, n=20)
    steps = 6
    blob = (np.array([spec.num_vertices, spec.num_triangles, steps, tune], np.int32).tobytes()
            + spec.positions.astype(np.float32).tobytes() + spec.indices.astype(np.uint32).tobytes()
            + spec.pinned.astype(np.uint8).tobytes() + bytes(spec.params))
    r = subprocess.run([str(exe)], input=blob, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    got = np.frombuffer(r.stdout, np.float32).reshape(-1, 3)
    b = ClothBatch([spec])
    b.step(steps)
    b.sync()
    want = b.read_positions()
    b.close()
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), np.ascontiguousarray(want, np.float32).view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("method", [_ffi.LC_BP_SAP, _ffi.LC_BP_GRID, _ffi.LC_BP_HASH, _ffi.LC_BP_BVH],
                         ids=["sap", "grid", "hash", "bvh"])
def test_collision_method_adapter_matches_the_oracle(tmp_path, method):
    """lc::CollisionMethod<int> (lc_body.hpp) over three frames of moves and
    removals, each frame's pair set against the oracle's."""
    from oracle.broadphase import box_pairs
    lib = _build.build()
    exe = tmp_path / "broadphase_demo"
    r = subprocess.run([_gxx(), "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(BP_SRC), "-o", str(exe),
                        "-L", str(lib.parent), "-llicenta_gb300", f"-Wl,-rpath,{lib.parent}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rng = np.random.default_rng(9)
    n, frames = 700, 3
    lo = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    hi = lo + rng.uniform(0.01, 0.06, (n, 3)).astype(np.float32)
    blob = np.array([method, n, frames], np.int32).tobytes() + np.concatenate([lo, hi], axis=1).tobytes()
    r = subprocess.run([str(exe)], input=blob, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    out = np.frombuffer(r.stdout, np.int32)
    pos, top = 0, n - 1
    for f in range(frames):
        for i in range(0, n, 3):
            if i > top:
                break
            lo[i, 0] += np.float32(0.01)
            hi[i, 0] += np.float32(0.01)
        top -= 1
        cnt = int(out[pos]); pos += 1
        got = {tuple(p) for p in out[pos:pos + 2 * cnt].reshape(-1, 2)}
        pos += 2 * cnt
        want = {(100 + a, 100 + b) for a, b in box_pairs(lo[:top + 1], hi[:top + 1])}
        assert got == want, f"frame {f}"
