"""Build the in-tree native libraries.

libpgs_gb300.so   frontend (GSInterface re-host) + CUDA backend, sm_103a only.
                  The test-only oracle has its own recipe (oracle/build_oracle.py).

Run ``python parallel-gs_gb300/build.py`` or call ``build_all()``.  Objects
are compiled in parallel; nothing uses cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

GENCODE = "arch=compute_103a,code=sm_103a"
LIB_NAME = "libpgs_gb300.so"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build_product(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "pgs.h"]
    out = BUILD / LIB_NAME
    cu = CSRC / "backend.cu"
    cu_up = CSRC / "upscaler.cu"
    cpp = CSRC / "frontend.cpp"
    o_cu = BUILD / "backend.o"
    o_up = BUILD / "upscaler.o"
    o_cpp = BUILD / "frontend.o"
    stamp = BUILD / "defines.txt"
    defines = os.environ.get("PGS_NVCC_DEFINES", "")
    if _newer(out, headers + [cu, cu_up, cpp, Path(__file__)]) and stamp.exists() and stamp.read_text() == defines:
        return out
    common = ["-I", str(INCLUDE), "-I", str(CSRC)]
    jobs = [
        [nvcc, "-gencode", GENCODE, "-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
         "-Xcompiler", "-fPIC", *common, "-c", str(cu), "-o", str(o_cu)],
        ["g++", "-std=c++17", "-O3", "-fPIC", "-pthread", "-ffp-contract=off", *common, "-c", str(cpp), "-o",
         str(o_cpp)],
        [nvcc, "-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *common, "-c", str(cu_up),
         "-o", str(o_up)],
    ]
    if verbose:
        jobs[0].insert(1, "-Xptxas=-v")
    # Extra compiler definitions for tuning sweeps, e.g. PGS_NVCC_DEFINES="PGS_SHADE_OCC=3".
    for d in os.environ.get("PGS_NVCC_DEFINES", "").split():
        jobs[0].insert(1, "-D" + d)
    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(_run, jobs))
    _run([nvcc, "-shared", "-gencode", GENCODE, "-cudart", "static", str(o_cu), str(o_up), str(o_cpp), "-lpthread",
          "-o", str(out)])
    stamp.write_text(defines)
    return out


def build_all(verbose: bool = False) -> dict:
    return {"product": build_product(verbose)}


if __name__ == "__main__":
    res = build_all(verbose="-v" in sys.argv)
    for k, v in res.items():
        print(k, v)
