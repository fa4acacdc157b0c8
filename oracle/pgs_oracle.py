"""TEST INFRASTRUCTURE ONLY: Python access to the CPU oracle and the reference harness.

liboracle.so (oracle_backend.cpp) restates the reference's GPU backend on the
CPU behind the same pgs_backend_ops table as the CUDA backend; tests plug it
under the product frontend and compare VRAM images.  libpgsref.so is the
reference's own CPU swizzle path (gs/gs_util.hpp:50-205) compiled from its
sources by ref_harness.cpp; it pins the VRAM layout.

Only tests, the smoke check and the CPU-baseline leg of the benchmark import
this module.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
ROOT = ORACLE_DIR.parent
sys.path.insert(0, str(ROOT / "parallel-gs_gb300"))

import pgs  # noqa: E402

ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libpgsref.so"

_oracle = None
_ref = None


def load_oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        if not ORACLE_LIB.exists():
            raise FileNotFoundError("%s missing: run parallel-gs_gb300/build.py" % ORACLE_LIB)
        lib = C.CDLL(str(ORACLE_LIB))
        lib.pgs_oracle_backend_create.argtypes = [C.POINTER(C.c_void_p)]
        lib.pgs_oracle_backend_create.restype = C.c_void_p
        lib.pgs_oracle_fragment_count.argtypes = [C.c_void_p]
        lib.pgs_oracle_fragment_count.restype = C.c_uint64
        lib.pgs_oracle_swizzle.argtypes = [C.c_uint32] * 5
        lib.pgs_oracle_phase_lut.argtypes = [C.c_void_p, C.c_void_p]
        lib.pgs_oracle_phase_lut.restype = None
        lib.pgs_oracle_swizzle.restype = C.c_uint32
        lib.pgs_oracle_state_log.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        lib.pgs_oracle_state_log.restype = C.c_uint32
        lib.pgs_oracle_rcp_fixed.argtypes = [C.c_uint32]
        lib.pgs_oracle_rcp_fixed.restype = C.c_float
        lib.pgs_oracle_rcp_float.argtypes = [C.c_float]
        lib.pgs_oracle_rcp_float.restype = C.c_float
        _oracle = lib
    return _oracle


def load_reference() -> C.CDLL | None:
    """The reference's compiled CPU swizzle, or None when it was not built here."""
    global _ref
    if _ref is None and REF_LIB.exists():
        lib = C.CDLL(str(REF_LIB))
        lib.pgs_ref_swizzle.argtypes = [C.c_uint32] * 6
        lib.pgs_ref_swizzle.restype = C.c_uint32
        args = [C.c_uint32, C.c_void_p, C.c_void_p] + [C.c_uint32] * 7
        lib.pgs_ref_vram_upload.argtypes = args
        lib.pgs_ref_vram_readback.argtypes = args
        _ref = lib
    return _ref


class OracleBackend(pgs.Backend):
    def __init__(self) -> None:
        lib = load_oracle()
        ops = C.c_void_p()
        handle = lib.pgs_oracle_backend_create(C.byref(ops))
        if not handle:
            raise MemoryError("oracle backend")
        self.lib = lib
        super().__init__(ops.value, handle)

    def fragments(self) -> int:
        return int(self.lib.pgs_oracle_fragment_count(self.handle))

    def state_log(self) -> np.ndarray:
        """Primitive states after triangle setup and the single-sample heuristic,
        concatenated over the render passes flushed so far."""
        n = int(self.lib.pgs_oracle_state_log(self.handle, None, 0))
        out = np.zeros(n, dtype=np.uint32)
        self.lib.pgs_oracle_state_log(self.handle, out.ctypes.data, n)
        return out


def render(frame, backend: pgs.Backend | None = None, planes: bool = False):
    """Runs a gsgen.Frame through the product frontend on `backend` (default: oracle).

    Returns the 4 MiB plane-0 image, or all planes when `planes` is set."""
    be = backend or OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=frame.super_sampling, ordered=frame.ordered)
    if frame.meta.get("ssaa_textures"):
        gs.set_super_sampled_textures(True)
    if frame.meta.get("hacks"):
        gs.set_hacks(**frame.meta["hacks"])
    if frame.meta.get("field_aware"):
        # Field-rendered interlaced NTSC (SMODE1 CMOD 2, SMODE2 INT | FFMD) read
        # out at high resolution: the vsync turns field-aware rendering on.
        gs.write_priv_register("SMODE1", (32 << 3) | (2 << 13))
        gs.write_priv_register("SMODE2", 3)
        gs.vsync(0, gs.VSYNC["FORCE_PROGRESSIVE"] | gs.VSYNC["HIGH_RESOLUTION"])
    gs.gif_transfer(0, frame.data)
    vram = gs.read_vram()
    out = vram
    if planes:
        n = 1 if frame.super_sampling == 1 else 2 + frame.super_sampling
        out = np.stack([vram] + [be.read_plane(p) for p in range(1, n)])
    gs.close()
    if backend is None:
        be.close()
    return out
