"""In-tree build of the CUDA engine (licenta_gb300/_lib/liblicenta_gb300.so).

Compiles every translation unit under licenta_gb300/csrc for sm_103a with
nvcc (in parallel, incrementally by mtime) and links one shared library that
exports the C ABI of include/lc/lc.h.  lc_lbvh.cu is built with -fmad=false so
its float arithmetic keeps the separate roundings the bit-exact stages need.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent
REPO = ROOT.parent
CSRC = ROOT / "csrc"
OUT = ROOT / "_lib"
LIB = OUT / "liblicenta_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

SOURCES = ["lc_api.cu", "lc_lbvh.cu", "lc_step.cu", "lc_scan.cu", "lc_cluster.cu", "lc_static.cu", "lc_adjoint.cu",
           "lc_narrow_api.cu", "lc_response.cu", "lc_broadphase.cu"]
# lc_lbvh.cu carries the bit-exact stages and lc_response.cu the impulse
# response: no FMA contraction, IEEE div/sqrt.
# The solver translation units are compared against FP64 within a tolerance
# and use the approximate (2 ulp) division and square root.
PER_FILE_FLAGS = {
    "lc_lbvh.cu": ["-fmad=false"],
    "lc_response.cu": ["-fmad=false"],
    "lc_step.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "lc_cluster.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "lc_adjoint.cu": ["-prec-div=false", "-prec-sqrt=false"],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA engine cannot be built")
    return cand


def cuda_libdir() -> Path:
    base = Path(nvcc()).resolve().parent.parent
    for sub in ("lib64", "targets/sbsa-linux/lib", "targets/aarch64-linux/lib", "targets/x86_64-linux/lib"):
        p = base / sub
        if (p / "libcudart.so").exists() or list(p.glob("libcudart.so*")):
            return p
    return base / "lib64"


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + [REPO / "include" / "lc" / "lc.h"]
    return max(h.stat().st_mtime for h in hs)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    hdr = _headers_mtime()
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        cmd = [nvcc(), ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
               "--expt-relaxed-constexpr", "-I", str(REPO / "include"), "-c", str(s), "-o", str(o)]
        cmd += PER_FILE_FLAGS.get(src, [])
        stamp = o.with_suffix(".flags")
        if (not force and o.exists() and o.stat().st_mtime > max(s.stat().st_mtime, hdr)
                and stamp.exists() and stamp.read_text() == " ".join(cmd)):
            continue
        jobs.append((cmd, stamp))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j) for j, _ in jobs]:
                f.result()
        for cmd, stamp in jobs:
            stamp.write_text(" ".join(cmd))
    if force or jobs or not LIB.exists():
        libdir = cuda_libdir()
        cmd = [nvcc(), ARCH, "-shared", "-o", str(LIB)] + [str(o) for o in objs] + [
            "-cudart", "shared", "-L", str(libdir), "-Xlinker", "-rpath," + str(libdir)]
        _run(cmd)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
