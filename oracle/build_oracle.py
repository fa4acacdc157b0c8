"""TEST INFRASTRUCTURE ONLY: build recipe for the oracle and the reference harness.

liboracle.so   CPU restatement of the backend (oracle_backend.cpp), used only
               by the tests, the smoke check and the CPU-baseline leg of the
               benchmark.
libpgsref.so   the reference's own CPU swizzle path (gs/gs_util.hpp:50-205)
               compiled from the reference's sources by ref_harness.cpp.
libpgsref_frontend.so
               the reference's own CPU frontend (gs/gs_interface.cpp,
               gs/page_tracker.cpp, gs/gs_util.cpp) compiled unmodified over
               the recording renderer of ref_frontend/ref_frontend.cpp.
The reference's sources are read where the reference is mounted:
$PGS_REFERENCE_DIR, else /root/reference.  Where they are absent these two
are not built and the tests that need them skip.

Outputs go to oracle/_build and oracle/_ref (both git-ignored).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
ROOT = ORACLE.parent
INCLUDE = ROOT / "include"
ORACLE_BUILD = ORACLE / "_build"
REF_BUILD = ORACLE / "_ref"


def reference_dir() -> Path:
    return Path(os.environ.get("PGS_REFERENCE_DIR", "/root/reference"))


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


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
    gs = reference_dir() / "gs"
    if not (gs / "gs_util.hpp").exists():
        print("reference sources not found under %s: libpgsref.so not built" % reference_dir(), file=sys.stderr)
        return None
    REF_BUILD.mkdir(parents=True, exist_ok=True)
    out = REF_BUILD / "libpgsref.so"
    src = ORACLE / "ref_harness.cpp"
    if not _newer(out, [src, Path(__file__)]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", str(ORACLE / "ref_shim"),
              "-I", str(gs), "-I", str(gs / "shaders"), str(src), "-o", str(out)])
    return out


REF_FRONTEND = ORACLE / "ref_frontend"
REF_FRONTEND_SOURCES = ("gs_interface.cpp", "page_tracker.cpp", "gs_util.cpp")


def build_reference_frontend() -> Path | None:
    """Compile the reference's CPU frontend (GSInterface, PageTracker, gs_util)
    from its sources, unmodified, against the stand-in headers under
    ref_frontend/shim and the recording GSRenderer of ref_frontend.cpp."""
    gs = reference_dir() / "gs"
    if not all((gs / f).exists() for f in REF_FRONTEND_SOURCES):
        print("reference sources not found under %s: libpgsref_frontend.so not built" % reference_dir(),
              file=sys.stderr)
        return None
    REF_BUILD.mkdir(parents=True, exist_ok=True)
    out = REF_BUILD / "libpgsref_frontend.so"
    shim = sorted(p for p in (REF_FRONTEND / "shim").rglob("*.hpp"))
    own = REF_FRONTEND / "ref_frontend.cpp"
    srcs = [gs / f for f in REF_FRONTEND_SOURCES] + [own]
    if _newer(out, srcs + shim + [Path(__file__)]):
        return out
    inc = ["-I", str(REF_FRONTEND / "shim"), "-I", str(gs), "-I", str(gs / "shaders")]
    objs = []
    jobs = []
    for src in srcs:
        obj = REF_BUILD / ("frontend_" + src.stem + ".o")
        objs.append(obj)
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-w", *inc, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(_run, jobs))
    _run(["g++", "-shared", "-Wl,--no-undefined", *map(str, objs), "-o", str(out)])
    return out


def build_all() -> dict:
    with ThreadPoolExecutor(max_workers=3) as ex:
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference_harness)
        f_fe = ex.submit(build_reference_frontend)
        return {"oracle": f_orc.result(), "reference": f_ref.result(), "reference_frontend": f_fe.result()}


if __name__ == "__main__":
    for k, v in build_all().items():
        print(k, v)
