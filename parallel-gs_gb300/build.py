"""Build the in-tree native libraries.

libpgs_gb300.so   frontend (GSInterface re-host) + CUDA backend, sm_103a only.
liboracle.so      CPU restatement of the backend, used only by tests and the
                  CPU baseline.
libpgsref.so      the reference's own CPU swizzle path compiled from its
                  sources (only where those sources are present).

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
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"
REF_BUILD = ORACLE / "_ref"
REFERENCE_SRC = Path(os.environ.get("PGS_REFERENCE_DIR", "/root/reference"))

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
        ["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", *common, "-c", str(cpp), "-o", str(o_cpp)],
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
    _run([nvcc, "-shared", "-gencode", GENCODE, "-cudart", "static", str(o_cu), str(o_up), str(o_cpp), "-o", str(out)])
    stamp.write_text(defines)
    return out


def build_oracle() -> Path:
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    src = ORACLE / "oracle_backend.cpp"
    out = ORACLE_BUILD / "liboracle.so"
    if not _newer(out, [src, INCLUDE / "pgs.h", Path(__file__)]):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
              "-I", str(INCLUDE), str(src), "-o", str(out)])
    return out


def build_reference_harness() -> Path | None:
    """Compile the reference's vram_upload/vram_readback where its sources exist."""
    gs = REFERENCE_SRC / "gs"
    if not (gs / "gs_util.hpp").exists():
        return None
    REF_BUILD.mkdir(parents=True, exist_ok=True)
    out = REF_BUILD / "libpgsref.so"
    src = ORACLE / "ref_harness.cpp"
    if not _newer(out, [src, Path(__file__)]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", str(ORACLE / "ref_shim"),
              "-I", str(gs), "-I", str(gs / "shaders"), str(src), "-o", str(out)])
    return out


def build_all(verbose: bool = False) -> dict:
    with ThreadPoolExecutor(max_workers=3) as ex:
        f_prod = ex.submit(build_product, verbose)
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference_harness)
        return {"product": f_prod.result(), "oracle": f_orc.result(), "reference": f_ref.result()}


if __name__ == "__main__":
    res = build_all(verbose="-v" in sys.argv)
    for k, v in res.items():
        print(k, v)
