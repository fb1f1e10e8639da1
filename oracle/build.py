"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle.cpp into oracle/liboracle.so with -ffp-contract=off so that
float expressions round exactly as written, and OpenMP for the traversal
loops.  The synthetic scene generator (vulkanwavefrontpathtracer_gb300/
csrc/host.cpp: the benchmark workloads' input data) is compiled in as well,
so that a CPU run generates the same scenes without the product library.
The reference's own sources are built separately (oracle/ref_build.py).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "oracle.cpp"
SCENES = HERE.parent / "vulkanwavefrontpathtracer_gb300" / "csrc" / "host.cpp"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, SCENES.stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", str(SRC), str(SCENES), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
