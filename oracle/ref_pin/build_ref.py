"""Build the reference's own CUDA kernels into oracle/_ref/ref_kernels.cubin.

TEST INFRASTRUCTURE ONLY.  The cubin is the "reference as built": the
reference's hot-path translation units, compiled from where they lie in the
reference checkout (never copied), device-linked into one sm_103a image that
oracle/ref_pin/refchain.py loads through the CUDA driver API to produce golden
vectors.  A cubin holds device code only, so the image built here on x86 also
loads on an aarch64 GPU host.

The reference is a Windows / CUDA 9.1 project; these flags (and nothing that
edits its sources) make its kernels compile with nvcc 13:

* ``-Xcudafe --no_alternative_tokens -Xcompiler -fno-operator-names`` —
  Core/CudaUtils.cu:333,343 name a variable ``xor``;
* ``-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP`` — keeps the CUDA
  toolkit's own CUB out of the translation units that include the vendored
  CUB 1.8 (Core/CubWrappers.cuh), whose names would otherwise clash;
* ``-include thrust/host_vector.h -include iostream`` — headers the sources
  rely on being pulled in transitively;
* ``-I oracle/ref_pin/stub`` — a declarations-only <Windows.h> for
  Core/Utils.hpp;
* ``-D__glew_h__ -D__FREEGLUT_H__`` — skips the GL headers that
  Core/Utils.hpp includes for code that is commented out (no GL type or
  function is declared or used);
* ``-include oracle/ref_pin/ref_shim.h`` — routes norm3df to the length the
  restatement uses (the one deliberate substitution);
* ``-rdc=true`` (the project's GenerateRelocatableDeviceCode, LicentaV2.vcxproj
  :107,156) and ``-fmad=false`` (separate roundings, as the restatement);
* ``-DNDEBUG`` — compiles out the device-side ``assert`` calls (Core/CudaUtils.cu
  :74,207,415,424, Physics/CudaPBD.cu:1540,1626); they check values and
  change none, and a failed device assert would stop the GPU context instead
  of reporting a difference.

The reference root (the directory holding Collision/, Core/ and Physics/)
comes from the command line or the LICENTA_REFERENCE environment variable;
there is no built-in default.

Usage: python -m oracle.ref_pin.build_ref REFERENCE_ROOT
"""
from __future__ import annotations

import gzip
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
OUT = REPO / "oracle" / "_ref"
CUBIN = OUT / "ref_kernels.cubin"

# The reference translation units of the cloth step's device code.
SOURCES = [
    "Core/CudaUtils.cu",
    "Collision/CudaBVH.cu",
    "Physics/CudaCubicSolver.cu",
    "Collision/CudaPrimitiveTests.cu",
    "Collision/FeatureList.cu",
    "Collision/CudaCollisionDetection.cu",
    "Collision/CudaCollisionResponse.cu",
    "Physics/CudaDeformableUtils.cu",
    "Physics/CudaPBD.cu",
]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def reference_root(root: str | Path | None = None) -> Path | None:
    """The reference root given, else LICENTA_REFERENCE; None when neither
    names a checkout that holds the cloth step's sources."""
    cand = root if root is not None else os.environ.get("LICENTA_REFERENCE")
    if not cand:
        return None
    cand = Path(cand)
    return cand if (cand / "Collision" / "CudaBVH.cu").exists() else None


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def build(root: Path | None = None, force: bool = False) -> Path | None:
    """Compile the reference kernels; returns the cubin path, or None when the
    reference checkout is not present (the cubin, if built earlier, stays)."""
    root = reference_root(root)
    if root is None:
        return CUBIN if CUBIN.exists() or Path(str(CUBIN) + ".gz").exists() else None
    if CUBIN.exists() and not force:
        newest = max((root / s).stat().st_mtime for s in SOURCES)
        if CUBIN.stat().st_mtime > max(newest, Path(__file__).stat().st_mtime,
                                       (HERE / "ref_shim.h").stat().st_mtime):
            return CUBIN
    obj = OUT / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    flags = [ARCH, "-std=c++17", "-rdc=true", "-fmad=false", "-w", "-DNDEBUG",
             "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP",
             "-Xcudafe", "--no_alternative_tokens", "-Xcompiler", "-fno-operator-names",
             "-I", str(HERE / "stub"), "-include", str(HERE / "ref_shim.h"),
             "-include", "thrust/host_vector.h", "-include", "iostream",
             "-D__glew_h__", "-D__FREEGLUT_H__"]
    jobs, objs = [], []
    for s in SOURCES:
        o = obj / (Path(s).stem + ".o")
        objs.append(str(o))
        jobs.append([_nvcc()] + flags + ["-c", str(root / s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    _run([_nvcc(), ARCH, "-dlink", "-cubin", "-o", str(CUBIN)] + objs)
    shutil.rmtree(obj, ignore_errors=True)  # host objects: not needed past the link
    # A compressed copy as well: tools that move a tree between hosts may drop
    # ELF files they do not recognise as their own; the loader takes either.
    with open(CUBIN, "rb") as f, gzip.open(str(CUBIN) + ".gz", "wb") as g:
        g.write(f.read())
    return CUBIN


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("LICENTA_REFERENCE"):
        sys.exit("usage: python -m oracle.ref_pin.build_ref REFERENCE_ROOT (or set LICENTA_REFERENCE)")
    p = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None, force=True)
    print(p if p else "reference checkout not found")
