"""Builds libwfpt.so in-tree: every CUDA/C++ source under csrc/ is compiled
for sm_103a by nvcc (translation units in parallel) and linked into one
shared library next to this file.

Usage: python -m vulkanwavefrontpathtracer_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libwfpt.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-lineinfo"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libwfpt.so")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _compile(src: Path, obj: Path, verbose: bool, ptxas_v: bool) -> tuple[Path, str]:
    cmd = [nvcc(), *ARCH, *COMMON, "-c", str(src), "-o", str(obj), "-I", str(INCLUDE)]
    if src.suffix == ".cpp":
        # Host code rounds every float operation as written (no FMA
        # contraction), so that x86 and Arm hosts compute the same bits.
        cmd += ["-Xcompiler", "-pthread", "-Xcompiler", "-ffp-contract=off"]
    if ptxas_v and src.suffix == ".cu":
        cmd += ["-Xptxas", "-v"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    hdr_mtime = max((h.stat().st_mtime for h in headers()), default=0.0)
    todo = []
    objs = []
    for src in sources():
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_mtime)
        if stale or ptxas_v:
            todo.append((src, obj))
    workers = max(1, min(len(todo), os.cpu_count() or 4))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = [ex.submit(_compile, s, o, verbose, ptxas_v) for s, o in todo]
            for f in futs:
                _, log = f.result()
                if ptxas_v and log:
                    print(log, file=sys.stderr)
    newest = max(o.stat().st_mtime for o in objs)
    if force or todo or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
               "-Xlinker", "-rpath,/usr/local/cuda/lib64", "-Xcompiler", "-pthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true", help="print register/spill/smem use per kernel")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose, ptxas_v=a.ptxas_v))


if __name__ == "__main__":
    main()
