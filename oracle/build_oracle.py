"""Build recipe of the CPU oracle (oracle/liblc_oracle.so).

TEST INFRASTRUCTURE: the oracle is loaded only by tests/, smoke() and the
CPU-baseline leg of bench.py.  -ffp-contract=off keeps float expressions
unfused on every host (aarch64 GCC contracts by default), which the FP32
mirror needs to stay bit-exact with the GPU's -fmad=false stages.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liblc_oracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "lc_oracle_capi.cpp"
    deps = [src, HERE / "lc_oracle.hpp", HERE.parent / "include" / "lc" / "lc.h"]
    if not force and LIB.exists() and LIB.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return LIB
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared",
           "-o", str(LIB), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build())
