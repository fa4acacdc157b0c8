"""TEST INFRASTRUCTURE ONLY: the reference's own CPU frontend, run here.

libpgsref_frontend.so is the reference's GSInterface / PageTracker / gs_util
(gs/gs_interface.cpp, gs/page_tracker.cpp, gs/gs_util.cpp) compiled unmodified
over a recording GSRenderer (oracle/ref_frontend/ref_frontend.cpp).  This module
feeds it a GIF stream and parses what the frontend handed its renderer into the
record shapes tests/recording_backend.py produces for the product frontend, so
the two frontends can be compared pass by pass.

Only tests import this module.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "_ref" / "libpgsref_frontend.so"

EV_PASS, EV_TEXTURE, EV_COPY, EV_PALETTE, EV_FLUSH_CACHE, EV_FLUSH_TRANSFER = 1, 2, 3, 4, 5, 6
EV_SUBMIT, EV_COPY_BARRIER, EV_HOST_SYNC, EV_READBACK, EV_REWIND_CLUT, EV_SET_SUPER_SAMPLING = 7, 8, 9, 10, 11, 12
EV_SHADOW_PAGE = 13

# FlushReason (gs/page_tracker.hpp:117-126).
REASONS = ["FBPointer", "Overflow", "TextureHazard", "CopyHazard", "SubmissionFlush", "PressureFlush", "HostAccess"]

POS_DT = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<u4"), ("padding", "<i4")])
ATTR_DT = np.dtype([("s", "<f4"), ("t", "<f4"), ("q", "<f4"), ("rgba", "<u4"), ("fog", "<f4"), ("u", "<u2"),
                    ("v", "<u2")])
PRIM_DT = np.dtype([("bb", "<i2", 4), ("state", "<u4"), ("tex", "<u4"), ("tex2", "<u4"), ("alpha", "<u4"),
                    ("fbmsk", "<u4"), ("fogcol", "<u4")])
STATE_DT = np.dtype([("combiner", "<u4"), ("blend_mode", "<u4"), ("dimx_lo", "<u4"), ("dimx_hi", "<u4")])
TEXINFO_DT = np.dtype([("id", "<u4"), ("sizes", "<f4", 4), ("region", "<f4", 4), ("bias", "<f4", 2),
                       ("arrayed", "<i4"), ("flags", "<i4")])
INST_DT = np.dtype([("frame", "<u8"), ("zbuf", "<u8"), ("base_x", "<u4"), ("base_y", "<u4"),
                    ("coarse_tiles_width", "<u4"), ("coarse_tiles_height", "<u4"), ("opaque_fbmask", "<u4"),
                    ("sampling_rate_x_log2", "<u4"), ("sampling_rate_y_log2", "<u4"), ("z_sensitive", "<u4"),
                    ("z_write", "<u4"), ("channel_shuffle", "<u4")])
TEXDESC_DT = np.dtype([("id", "<u4"), ("tex0", "<u8"), ("tex1", "<u8"), ("miptbp1_3", "<u8"), ("miptbp4_6", "<u8"),
                       ("texa", "<u8"), ("clamp", "<u8"), ("palette_bank", "<u4"), ("samples", "<u4"),
                       ("rect_x", "<u4"), ("rect_y", "<u4"), ("rect_w", "<u4"), ("rect_h", "<u4"),
                       ("rect_levels", "<u4")], align=False)

_lib = None


def available() -> bool:
    return LIB.exists()


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise FileNotFoundError("%s missing: run oracle/build_oracle.py where the reference is mounted" % LIB)
        lib = C.CDLL(str(LIB))
        vp = C.c_void_p
        lib.pgs_ref_frontend_create.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        lib.pgs_ref_frontend_create.restype = vp
        lib.pgs_ref_frontend_destroy.argtypes = [vp]
        lib.pgs_ref_frontend_gif_transfer.argtypes = [vp, C.c_uint32, vp, C.c_size_t]
        lib.pgs_ref_frontend_write_register.argtypes = [vp, C.c_uint32, C.c_uint64]
        lib.pgs_ref_frontend_flush.argtypes = [vp]
        lib.pgs_ref_frontend_set_hacks.argtypes = [vp, C.c_uint32, C.c_uint32]
        lib.pgs_ref_frontend_set_super_sampling_rate.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32]
        lib.pgs_ref_frontend_log_size.argtypes = [vp]
        lib.pgs_ref_frontend_log_size.restype = C.c_size_t
        lib.pgs_ref_frontend_log_data.argtypes = [vp]
        lib.pgs_ref_frontend_log_data.restype = vp
        lib.pgs_ref_frontend_log_clear.argtypes = [vp]
        _lib = lib
    return _lib


def _parse_pass(b: bytes) -> dict:
    hdr = struct.unpack_from("<12I", b, 0)
    reason, n, nstates, ntex, ninst, ts, aa1, scanmsk, demote, fb_mode, fb_psm, fb_cpsm = hdr
    off = 48
    inst = np.frombuffer(b, INST_DT, ninst, off)
    off += INST_DT.itemsize * ninst
    pos = np.frombuffer(b, POS_DT, 3 * n, off)
    off += POS_DT.itemsize * 3 * n
    attr = np.frombuffer(b, ATTR_DT, 3 * n, off)
    off += ATTR_DT.itemsize * 3 * n
    prim = np.frombuffer(b, PRIM_DT, n, off)
    off += PRIM_DT.itemsize * n
    states = np.frombuffer(b, STATE_DT, nstates, off)
    off += STATE_DT.itemsize * nstates
    tex = np.frombuffer(b, TEXINFO_DT, ntex, off)
    off += TEXINFO_DT.itemsize * ntex
    assert off == len(b), (off, len(b))
    return {"flush_reason": REASONS[reason], "num_primitives": n, "coarse_tile_size_log2": ts, "has_aa1": aa1,
            "has_scanmsk": scanmsk, "blend_demote": demote, "feedback_mode": fb_mode, "feedback_psm": fb_psm,
            "feedback_cpsm": fb_cpsm, "instances": inst, "positions": pos, "attributes": attr, "prims": prim,
            "states": states, "textures": tex}


def parse_log(blob: bytes) -> list[dict]:
    """Events in order: {"type": name, ...payload}."""
    out = []
    off = 0
    while off < len(blob):
        typ, size = struct.unpack_from("<II", blob, off)
        off += 8
        b = blob[off:off + size]
        off += size
        if typ == EV_PASS:
            ev = _parse_pass(b)
            ev["type"] = "pass"
        elif typ == EV_TEXTURE:
            ev = {"type": "texture", **{k: np.frombuffer(b, TEXDESC_DT, 1)[0][k].item() for k in TEXDESC_DT.names}}
        elif typ == EV_COPY:
            bb, pos, reg, dirr, size_, offset, required, shadow = struct.unpack_from("<7QI", b, 0)
            ev = {"type": "copy", "bitbltbuf": bb, "trxpos": pos, "trxreg": reg, "trxdir": dirr, "host_size": size_,
                  "offset": offset, "required": required, "needs_shadow_vram": shadow, "data": bytes(b[60:])}
        elif typ == EV_PALETTE:
            tex0, texclut, bias, scale, ref_base, mask, incoming, inst = struct.unpack_from("<QQIfIIII", b, 0)
            ev = {"type": "palette", "tex0": tex0, "texclut": texclut, "csm2_x_bias": bias, "csm2_x_scale": scale,
                  "csm1_reference_base": ref_base, "csm1_mask": mask, "incoming": incoming, "instance": inst}
        else:
            words = struct.unpack_from("<%dI" % (size // 4), b, 0)
            names = {EV_FLUSH_CACHE: "flush_cache", EV_FLUSH_TRANSFER: "flush_transfer", EV_SUBMIT: "submit",
                     EV_COPY_BARRIER: "copy_barrier", EV_HOST_SYNC: "host_sync", EV_READBACK: "readback",
                     EV_REWIND_CLUT: "rewind_clut", EV_SET_SUPER_SAMPLING: "set_super_sampling",
                     EV_SHADOW_PAGE: "shadow_page"}
            ev = {"type": names.get(typ, "unknown%d" % typ), "words": words}
        out.append(ev)
    return out


class RefFrontend:
    """GSInterface of the reference over the recording renderer."""

    def __init__(self, super_sampling: int = 1, ordered: bool = True, super_sampled_textures: bool = False):
        self.lib = load()
        self.h = self.lib.pgs_ref_frontend_create(super_sampling, int(ordered), int(super_sampled_textures))
        if not self.h:
            raise RuntimeError("pgs_ref_frontend_create failed")

    def gif_transfer(self, path: int, data: bytes) -> None:
        buf = np.frombuffer(data, dtype=np.uint8)
        self.lib.pgs_ref_frontend_gif_transfer(self.h, path, buf.ctypes.data, buf.size)

    def write_register(self, addr: int, value: int) -> None:
        self.lib.pgs_ref_frontend_write_register(self.h, addr, value)

    def set_hacks(self, disable_mipmaps: bool = False, allow_blend_demote: bool = False) -> None:
        self.lib.pgs_ref_frontend_set_hacks(self.h, int(disable_mipmaps), int(allow_blend_demote))

    def set_super_sampling_rate(self, super_sampling: int, ordered: bool = True,
                                super_sampled_textures: bool = False) -> None:
        self.lib.pgs_ref_frontend_set_super_sampling_rate(self.h, super_sampling, int(ordered),
                                                          int(super_sampled_textures))

    def flush(self) -> None:
        self.lib.pgs_ref_frontend_flush(self.h)

    def events(self) -> list[dict]:
        n = self.lib.pgs_ref_frontend_log_size(self.h)
        return parse_log(C.string_at(self.lib.pgs_ref_frontend_log_data(self.h), n)) if n else []

    def clear(self) -> None:
        self.lib.pgs_ref_frontend_log_clear(self.h)

    def close(self) -> None:
        if self.h:
            self.lib.pgs_ref_frontend_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
