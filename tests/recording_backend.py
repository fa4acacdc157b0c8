"""A pgs_backend_ops implementation in Python that records what the frontend sends.

Used by the host-logic tests: the product frontend runs unchanged and every
flush_rendering / copy_vram / update_palette_cache call is captured as numpy
records for inspection.  No rendering happens."""
import ctypes as C

import numpy as np

import pgs

MAXP = 64 * 1024


class VertexPosition(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_uint32), ("padding", C.c_int32)]


class VertexAttribute(C.Structure):
    _fields_ = [("s", C.c_float), ("t", C.c_float), ("q", C.c_float), ("rgba", C.c_uint32), ("fog", C.c_float),
                ("u", C.c_uint16), ("v", C.c_uint16)]


class PrimitiveAttribute(C.Structure):
    _fields_ = [("bb", C.c_int16 * 4), ("state", C.c_uint32), ("tex", C.c_uint32), ("tex2", C.c_uint32),
                ("alpha", C.c_uint32), ("fbmsk", C.c_uint32), ("fogcol", C.c_uint32)]


class StateVector(C.Structure):
    _fields_ = [("combiner", C.c_uint32), ("blend_mode", C.c_uint32), ("dimx_lo", C.c_uint32), ("dimx_hi", C.c_uint32)]


class TextureDesc(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("tbp0", "tbw", "psm", "tw_log2", "th_log2", "cpsm", "csa", "clut_instance",
                                          "aem", "ta0", "ta1", "wms", "wmt", "minu", "maxu", "minv", "maxv",
                                          "levels")] + \
               [("mip", C.c_uint32 * 6), ("samples", C.c_uint32), ("mxl", C.c_uint32)]


class RPInstance(C.Structure):
    _fields_ = [("frame", C.c_uint64), ("zbuf", C.c_uint64), ("base_x", C.c_int32), ("base_y", C.c_int32),
                ("coarse_tiles_width", C.c_uint32), ("coarse_tiles_height", C.c_uint32),
                ("sampling_rate_x_log2", C.c_uint32), ("sampling_rate_y_log2", C.c_uint32),
                ("opaque_fbmask", C.c_uint32), ("z_sensitive", C.c_uint32), ("z_write", C.c_uint32),
                ("channel_shuffle", C.c_uint32)]


class RenderPass(C.Structure):
    _fields_ = [("positions", C.POINTER(VertexPosition)), ("attributes", C.POINTER(VertexAttribute)),
                ("prims", C.POINTER(PrimitiveAttribute)), ("num_primitives", C.c_uint32),
                ("states", C.POINTER(StateVector)), ("num_states", C.c_uint32),
                ("textures", C.POINTER(TextureDesc)), ("num_textures", C.c_uint32),
                ("instances", RPInstance * 8), ("num_instances", C.c_uint32),
                ("coarse_tile_size_log2", C.c_uint32), ("has_aa1", C.c_uint32), ("has_scanmsk", C.c_uint32),
                ("flush_reason", C.c_uint32), ("has_mipmap", C.c_uint32), ("has_ss_textures", C.c_uint32),
                ("field_aware", C.c_uint32), ("blend_demote", C.c_uint32), ("num_snapshots", C.c_uint32),
                ("snapshot_textures", C.c_uint32 * 4)]


class CopyDesc(C.Structure):
    _fields_ = [("bitbltbuf", C.c_uint64), ("trxpos", C.c_uint64), ("trxreg", C.c_uint64), ("trxdir", C.c_uint64),
                ("host_data", C.c_void_p), ("host_size", C.c_uint64), ("host_offset", C.c_uint64),
                ("host_required", C.c_uint64)]


class PaletteUpload(C.Structure):
    _fields_ = [("tex0", C.c_uint64), ("texclut", C.c_uint64), ("csm2_x_scale", C.c_float),
                ("csm2_x_bias", C.c_uint32), ("base_instance", C.c_uint32), ("target", C.c_uint32)]


DESTROY = C.CFUNCTYPE(None, C.c_void_p)
RESERVE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint32, C.POINTER(C.POINTER(VertexPosition)),
                      C.POINTER(C.POINTER(VertexAttribute)), C.POINTER(C.POINTER(PrimitiveAttribute)))
FLUSH = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(RenderPass))
COPY = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(CopyDesc))
PALETTE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(PaletteUpload))
SETSS = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint32, C.c_uint32)
SUBMIT = C.CFUNCTYPE(C.c_int, C.c_void_p)
READ = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p)
WRITE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p)
ERROR = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_uint32))
VSYNC = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)


class Ops(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("destroy", DESTROY), ("reserve", RESERVE), ("flush", FLUSH),
                ("copy", COPY), ("palette", PALETTE), ("set_ss", SETSS), ("submit", SUBMIT), ("read", READ),
                ("write", WRITE), ("error", ERROR), ("read_async", C.c_void_p), ("wait_ticket", C.c_void_p),
                ("sample_circuit", C.c_void_p), ("vsync", VSYNC), ("timestamps", C.c_void_p),
                ("snapshot_vram", SUBMIT), ("readback_rect", C.c_void_p)]


def _struct_array(ptr, n, fields):
    return [{k: (list(getattr(ptr[i], k)) if k in ("bb", "mip") else getattr(ptr[i], k)) for k in fields}
            for i in range(n)]


class RecordingBackend(pgs.Backend):
    """Backend that records; `passes`, `copies`, `palettes`, `ss` hold what was sent."""

    def __init__(self, max_samples_log2: int = 4):
        self.max_samples_log2 = max_samples_log2
        self.passes, self.copies, self.palettes, self.ss = [], [], [], []
        # Every call in order: ("pass", i), ("copy", i), ("palette", i).
        self.events = []
        self.vram = np.zeros(pgs.VRAM_SIZE, dtype=np.uint8)
        self.next_clut = 0
        self._pos = (VertexPosition * (3 * MAXP))()
        self._attr = (VertexAttribute * (3 * MAXP))()
        self._prim = (PrimitiveAttribute * MAXP)()
        self.vsyncs = 0
        self._cbs = Ops(6, DESTROY(lambda s: None), RESERVE(self._reserve), FLUSH(self._flush), COPY(self._copy),
                        PALETTE(self._palette), SETSS(self._set_ss), SUBMIT(lambda s: 0), READ(self._read),
                        WRITE(self._write), ERROR(self._error), None, None, None, VSYNC(self._vsync), None,
                        SUBMIT(self._snapshot))
        super().__init__(C.addressof(self._cbs), 1)

    def _reserve(self, s, n, pos, attr, prim):
        pos[0] = C.cast(self._pos, C.POINTER(VertexPosition))
        attr[0] = C.cast(self._attr, C.POINTER(VertexAttribute))
        prim[0] = C.cast(self._prim, C.POINTER(PrimitiveAttribute))
        return 0

    def _flush(self, s, rpp):
        rp = rpp.contents
        n = rp.num_primitives
        rec = {
            "num_primitives": n,
            "positions": [(rp.positions[i].x, rp.positions[i].y, rp.positions[i].z) for i in range(3 * n)],
            "attributes": _struct_array(rp.attributes, 3 * n, ("s", "t", "q", "rgba", "fog", "u", "v")),
            "prims": _struct_array(rp.prims, n, ("bb", "state", "tex", "tex2", "alpha", "fbmsk", "fogcol")),
            "states": _struct_array(rp.states, rp.num_states, ("combiner", "blend_mode", "dimx_lo", "dimx_hi")),
            "textures": _struct_array(rp.textures, rp.num_textures, [f[0] for f in TextureDesc._fields_[:-1]]),
            "instances": [{f[0]: getattr(rp.instances[i], f[0]) for f in RPInstance._fields_}
                          for i in range(rp.num_instances)],
            "coarse_tile_size_log2": rp.coarse_tile_size_log2,
            "has_aa1": rp.has_aa1, "has_scanmsk": rp.has_scanmsk, "flush_reason": rp.flush_reason,
            "has_mipmap": rp.has_mipmap, "has_ss_textures": rp.has_ss_textures,
            "field_aware": rp.field_aware, "blend_demote": rp.blend_demote,
            "snapshot_textures": list(rp.snapshot_textures)[:rp.num_snapshots],
        }
        self.snapshots_taken = 0
        if n == 0:
            return 0
        self.passes.append(rec)
        self.events.append(("pass", len(self.passes) - 1))
        return 0

    def _copy(self, s, dp):
        d = dp.contents
        data = C.string_at(d.host_data, d.host_size) if d.host_data else b""
        self.copies.append({"bitbltbuf": d.bitbltbuf, "trxpos": d.trxpos, "trxreg": d.trxreg, "trxdir": d.trxdir,
                            "data": data, "offset": d.host_offset, "required": d.host_required})
        self.events.append(("copy", len(self.copies) - 1))
        return 0

    def _palette(self, s, up):
        u = up.contents
        self.next_clut = (u.target - 1) % 1024 if u.target else (self.next_clut + 1) % 1024
        self.palettes.append({"tex0": u.tex0, "texclut": u.texclut, "base_instance": u.base_instance,
                              "instance": self.next_clut})
        self.events.append(("palette", len(self.palettes) - 1))
        return self.next_clut

    def _snapshot(self, s):
        self.events.append(("snapshot", len(self.passes)))
        self.snapshots_taken = getattr(self, "snapshots_taken", 0) + 1
        return self.snapshots_taken - 1

    def _set_ss(self, s, x, y):
        # Like a backend created with max_samples_log2 sample planes.
        if x + y > self.max_samples_log2:
            return pgs.STATUS_CODES["PGS_ERROR_UNSUPPORTED"]
        self.ss.append((x, y))
        return 0

    def _read(self, s, plane, off, size, dst):
        C.memmove(dst, self.vram.ctypes.data + off, size)
        return 0

    def _write(self, s, off, size, src):
        C.memmove(self.vram.ctypes.data + off, src, size)
        return 0

    def _vsync(self, s, params, dst):
        # Merging is not recorded: the image stays as the caller allocated it.
        self.vsyncs += 1
        return 0

    def _error(self, s, flags):
        if flags:
            flags[0] = 0
        return 0

    def close(self):
        self.handle = None
