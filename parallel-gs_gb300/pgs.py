"""Python binding of the GS frontend and the CUDA backend (ctypes over include/pgs.h).

The classes mirror the reference's GSInterface API (gs/gs_interface.hpp:251-304):

    backend = CudaBackend(device=0, max_samples_log2=4)
    gs = GSInterface(backend, super_sampling=4)
    gs.gif_transfer(0, packet_bytes)
    vram = gs.read_vram()          # 4 MiB numpy array (flushes and waits)

The product path always runs the CUDA backend from the in-tree
libpgs_gb300.so; it raises if the library or a GPU is missing.  Any other
object exposing ``ops`` (a pgs_backend_ops pointer) and ``handle`` can be
passed to GSInterface in its place.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libpgs_gb300.so"
VRAM_SIZE = 4 * 1024 * 1024

PGS_OK = 0
STATUS_NAMES = {
    0: "PGS_OK", -1: "PGS_ERROR_INVALID_ARGUMENT", -2: "PGS_ERROR_OUT_OF_MEMORY", -3: "PGS_ERROR_CUDA",
    -4: "PGS_ERROR_NO_DEVICE", -5: "PGS_ERROR_UNSUPPORTED", -6: "PGS_ERROR_DEVICE_FLAG", -7: "PGS_ERROR_CAPACITY",
    -8: "PGS_ERROR_IO",
}


STATUS_CODES = {v: k for k, v in STATUS_NAMES.items()}


class PGSError(RuntimeError):
    def __init__(self, status: int, what: str) -> None:
        super().__init__("%s failed: %s (%d)" % (what, STATUS_NAMES.get(status, "?"), status))
        self.status = status


def check(status: int, what: str) -> None:
    if status != PGS_OK:
        raise PGSError(status, what)


class FlushStats(C.Structure):
    _fields_ = [("num_render_passes", C.c_uint64), ("num_primitives", C.c_uint64), ("num_copies", C.c_uint64),
                ("num_palette_updates", C.c_uint64), ("num_copy_barriers", C.c_uint64),
                ("num_flushes_by_reason", C.c_uint64 * 8)]


class GSOptions(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("super_sampling", C.c_uint32), ("ordered_super_sampling", C.c_uint32), ("vram_size", C.c_uint32),
                ("dynamic_super_sampling", C.c_uint32), ("super_sampled_textures", C.c_uint32),
                ("threaded_decode", C.c_uint32)]


# pgs_gs_options.threaded_decode.
THREADED_DECODE_AUTO, THREADED_DECODE_OFF, THREADED_DECODE_ALWAYS = 0, 1, 2


class CudaBackendOptions(C.Structure):
    _fields_ = [("device", C.c_int), ("max_samples_log2", C.c_uint32), ("flags", C.c_uint32),
                ("arena_mib", C.c_uint32)]


class CircuitParams(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("fbp", "fbw", "psm", "dbx", "dby", "phase", "phase_stride", "super_samples",
                                          "width", "height", "valid_width", "valid_height")]


class BatchTuning(C.Structure):
    _fields_ = [("cta_threads", C.c_uint32), ("ctas_per_sm", C.c_uint32), ("largest_first", C.c_uint32),
                ("solo_min_prims", C.c_uint32)]


class BackendStats(C.Structure):
    _fields_ = [("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("render_passes", C.c_uint64)]


# Every C-ABI symbol include/pgs.h declares.
EXPORTED_SYMBOLS = [
    "pgs_cuda_backend_create", "pgs_cuda_backend_begin_record", "pgs_cuda_backend_end_record",
    "pgs_cuda_backend_replay", "pgs_cuda_backend_stream", "pgs_cuda_backend_launches_per_replay",
    "pgs_cuda_backend_last_shade_ms", "pgs_cuda_backend_fragment_count", "pgs_cuda_backend_get_stats",
    "pgs_cuda_backend_set_shade_timing", "pgs_cuda_backend_sample_circuit",
    "pgs_batch_create", "pgs_batch_destroy", "pgs_batch_add", "pgs_batch_replay", "pgs_batch_set_tuning",
    "pgs_batch_get_tuning", "pgs_batch_autotune", "pgs_batch_stream", "pgs_batch_launches_per_replay",
    "pgs_batch_synchronize",
    "pgs_upscaler_create", "pgs_upscaler_destroy", "pgs_upscaler_param_count", "pgs_upscaler_set_params",
    "pgs_upscaler_get_params", "pgs_upscaler_get_gradient", "pgs_upscaler_forward", "pgs_upscaler_backward",
    "pgs_upscaler_adam_step", "pgs_upscaler_stream", "pgs_upscaler_set_stream", "pgs_upscaler_synchronize",
    "pgs_umma_selftest",
    "pgs_upscaler_set_tensor_path", "pgs_upscaler_get_error",
    "pgs_gs_create", "pgs_gs_destroy", "pgs_gs_gif_transfer", "pgs_gs_write_register", "pgs_gs_flush",
    "pgs_gs_read_vram", "pgs_gs_read_vram_async", "pgs_gs_wait",
    "pgs_gs_write_priv_register", "pgs_gs_read_priv_register", "pgs_gs_scanout_circuit", "pgs_gs_vsync",
    "pgs_gs_set_super_sampled_textures", "pgs_gs_vsync_can_skip", "pgs_gs_set_hacks",
    "pgs_gs_reset_context_state", "pgs_gs_clobber_register_state", "pgs_gs_read_register", "pgs_gs_set_register",
    "pgs_gs_get_gif_path", "pgs_gs_set_gif_path", "pgs_gs_set_signal_interface", "pgs_gs_set_debug_mode",
    "pgs_gs_get_accumulated_timestamps",
    "pgs_gs_dump_open", "pgs_gs_dump_next_vsync", "pgs_gs_dump_close", "pgs_gs_dump_record_begin",
    "pgs_gs_dump_record_vsync", "pgs_gs_dump_record_end", "pgs_gs_write_vram", "pgs_gs_read_transfer_fifo", "pgs_gs_consume_flush_stats",
    "pgs_gs_set_super_sampling_rate",
]

_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads the product library (raises FileNotFoundError when it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError("%s is missing: run parallel-gs_gb300/build.py" % p)
    lib = C.CDLL(str(p))
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    lib.pgs_cuda_backend_create.argtypes = [C.POINTER(CudaBackendOptions), C.POINTER(vp), C.POINTER(i32)]
    lib.pgs_cuda_backend_create.restype = vp
    lib.pgs_cuda_backend_begin_record.argtypes = [vp]
    lib.pgs_cuda_backend_end_record.argtypes = [vp]
    lib.pgs_cuda_backend_replay.argtypes = [vp, u32, i32, i32]
    lib.pgs_cuda_backend_stream.argtypes = [vp]
    lib.pgs_cuda_backend_stream.restype = vp
    lib.pgs_cuda_backend_launches_per_replay.argtypes = [vp]
    lib.pgs_cuda_backend_launches_per_replay.restype = u32
    lib.pgs_cuda_backend_last_shade_ms.argtypes = [vp, C.POINTER(C.c_float)]
    lib.pgs_cuda_backend_fragment_count.argtypes = [vp, C.POINTER(u64)]
    lib.pgs_cuda_backend_get_stats.argtypes = [vp, C.POINTER(BackendStats)]
    lib.pgs_cuda_backend_set_shade_timing.argtypes = [vp, i32]
    lib.pgs_cuda_backend_sample_circuit.argtypes = [vp, C.POINTER(CircuitParams), vp]
    lib.pgs_batch_create.argtypes = [C.c_int, C.POINTER(i32)]
    lib.pgs_batch_create.restype = vp
    lib.pgs_batch_destroy.argtypes = [vp]
    lib.pgs_batch_destroy.restype = None
    lib.pgs_batch_add.argtypes = [vp, vp]
    lib.pgs_batch_replay.argtypes = [vp, u32, i32, i32]
    lib.pgs_batch_set_tuning.argtypes = [vp, C.POINTER(BatchTuning)]
    lib.pgs_batch_get_tuning.argtypes = [vp, C.POINTER(BatchTuning)]
    lib.pgs_batch_autotune.argtypes = [vp, u32, i32, C.POINTER(BatchTuning), C.POINTER(C.c_float)]
    lib.pgs_batch_stream.argtypes = [vp]
    lib.pgs_batch_stream.restype = vp
    lib.pgs_batch_launches_per_replay.argtypes = [vp]
    lib.pgs_batch_launches_per_replay.restype = u32
    lib.pgs_batch_synchronize.argtypes = [vp]
    lib.pgs_gs_create.argtypes = [vp, vp, C.POINTER(GSOptions), C.POINTER(i32)]
    lib.pgs_gs_create.restype = vp
    lib.pgs_gs_destroy.argtypes = [vp]
    lib.pgs_gs_destroy.restype = None
    lib.pgs_gs_gif_transfer.argtypes = [vp, u32, vp, C.c_size_t]
    lib.pgs_gs_write_register.argtypes = [vp, u32, u64]
    lib.pgs_gs_flush.argtypes = [vp]
    lib.pgs_gs_read_vram.argtypes = [vp, u64, u64, vp]
    lib.pgs_gs_read_vram_async.argtypes = [vp, u64, u64, vp, C.POINTER(u64)]
    lib.pgs_gs_wait.argtypes = [vp, u64]
    lib.pgs_gs_write_priv_register.argtypes = [vp, u32, u64]
    lib.pgs_gs_dump_open.argtypes = [vp, C.c_char_p]
    lib.pgs_gs_dump_next_vsync.argtypes = [vp, C.POINTER(u32)]
    lib.pgs_gs_dump_close.argtypes = [vp]
    lib.pgs_gs_dump_record_begin.argtypes = [vp, C.c_char_p]
    lib.pgs_gs_dump_record_vsync.argtypes = [vp, u32]
    lib.pgs_gs_dump_record_end.argtypes = [vp]
    lib.pgs_gs_read_priv_register.argtypes = [vp, u32, C.POINTER(u64)]
    lib.pgs_gs_scanout_circuit.argtypes = [vp, u32, u32, u32, vp, u64, C.POINTER(u32), C.POINTER(u32)]
    lib.pgs_gs_vsync.argtypes = [vp, C.POINTER(VsyncInfo), vp, u64, C.POINTER(ScanoutResult)]
    lib.pgs_gs_write_vram.argtypes = [vp, u64, u64, vp]
    lib.pgs_gs_read_transfer_fifo.argtypes = [vp, vp, u32]
    lib.pgs_gs_consume_flush_stats.argtypes = [vp, C.POINTER(FlushStats)]
    lib.pgs_gs_set_super_sampling_rate.argtypes = [vp, u32, u32]
    lib.pgs_gs_set_super_sampled_textures.argtypes = [vp, i32]
    lib.pgs_gs_vsync_can_skip.argtypes = [vp, C.POINTER(VsyncInfo)]
    lib.pgs_gs_set_hacks.argtypes = [vp, C.POINTER(Hacks)]
    lib.pgs_gs_reset_context_state.argtypes = [vp]
    lib.pgs_gs_clobber_register_state.argtypes = [vp]
    lib.pgs_gs_read_register.argtypes = [vp, u32, C.POINTER(u64)]
    lib.pgs_gs_set_register.argtypes = [vp, u32, u64]
    lib.pgs_gs_get_gif_path.argtypes = [vp, u32, C.POINTER(GifPath)]
    lib.pgs_gs_set_gif_path.argtypes = [vp, u32, C.POINTER(GifPath)]
    lib.pgs_gs_set_signal_interface.argtypes = [vp, C.POINTER(SignalInterface)]
    lib.pgs_gs_set_debug_mode.argtypes = [vp, C.POINTER(DebugMode)]
    lib.pgs_gs_get_accumulated_timestamps.argtypes = [vp, u32, C.POINTER(C.c_double)]
    if path is None:
        _lib = lib
    return lib


class BackendOps(C.Structure):
    """pgs_backend_ops; only used to call destroy/read_vram on foreign backends."""
    _fields_ = [("abi_version", C.c_uint32),
                ("destroy", C.CFUNCTYPE(None, C.c_void_p)),
                ("reserve_primitive_buffers", C.c_void_p),
                ("flush_rendering", C.c_void_p),
                ("copy_vram", C.c_void_p),
                ("update_palette_cache", C.c_void_p),
                ("set_super_sampling", C.c_void_p),
                ("flush_submit", C.c_void_p),
                ("read_vram", C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p)),
                ("write_vram", C.c_void_p),
                ("get_error", C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_uint32)))]


class VsyncInfo(C.Structure):
    _fields_ = [("phase", C.c_uint32), ("flags", C.c_uint32)]


SIGNAL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64)


class GifPath(C.Structure):
    """pgs_gif_path (GIFPath, gs/gs_interface.hpp:63-68)."""
    _fields_ = [("tag", C.c_uint64 * 2), ("reg", C.c_uint32), ("loop", C.c_uint32)]


class SignalInterface(C.Structure):
    """pgs_signal_interface (SignalInterface, gs/gs_interface.hpp:238-248)."""
    _fields_ = [("on_signal", SIGNAL_FN), ("on_finish", SIGNAL_FN), ("on_label", SIGNAL_FN), ("user", C.c_void_p)]


class DebugMode(C.Structure):
    """pgs_debug_mode (DebugMode, gs/gs_interface.hpp:137-153)."""
    _fields_ = [(n, C.c_uint32) for n in ("feedback_render_target", "timestamps", "deterministic_timeline_query",
                                          "disable_sampler_feedback", "draw_mode")]


TIMESTAMPS = ["SyncHostToVRAM", "CopyVRAM", "PaletteUpdate", "TextureUpload", "TriangleSetup", "Binning", "Shading",
              "Readback", "VSync"]


class Hacks(C.Structure):
    """pgs_hacks (Hacks, gs/gs_interface.hpp:209-237)."""
    _fields_ = [(n, C.c_uint32) for n in ("disable_mipmaps", "unsynced_readbacks", "backbuffer_promotion",
                                          "allow_blend_demote")]


class ScanoutResult(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("width", "height", "mode_width", "mode_height", "internal_width",
                                          "internal_height", "interlaced", "interlace_phase", "double_strike",
                                          "high_resolution_scanout")] + \
               [("sampling_rate_mhz", C.c_float), ("padding", C.c_uint32)]


class Backend:
    """A backend instance: `ops` is a pgs_backend_ops pointer, `handle` its state."""

    def __init__(self, ops: int, handle: int) -> None:
        self.ops = ops
        self.handle = handle

    def read_plane(self, plane: int, offset: int = 0, size: int = VRAM_SIZE) -> np.ndarray:
        out = np.empty(size, dtype=np.uint8)
        table = C.cast(C.c_void_p(self.ops), C.POINTER(BackendOps)).contents
        check(table.read_vram(self.handle, plane, offset, size, out.ctypes.data), "read_vram")
        return out

    def error_flags(self) -> int:
        table = C.cast(C.c_void_p(self.ops), C.POINTER(BackendOps)).contents
        flags = C.c_uint32(0)
        table.get_error(self.handle, C.byref(flags))
        return flags.value

    def close(self) -> None:
        if self.handle:
            table = C.cast(C.c_void_p(self.ops), C.POINTER(BackendOps)).contents
            table.destroy(self.handle)
            self.handle = None


class CudaBackend(Backend):
    """The sm_103a backend.  Fails loudly when no GPU or library is present."""

    def __init__(self, device: int = 0, max_samples_log2: int = 4, arena_mib: int = 0) -> None:
        self.lib = load_library()
        opts = CudaBackendOptions(device, max_samples_log2, 0, arena_mib)
        ops = C.c_void_p()
        status = C.c_int(0)
        handle = self.lib.pgs_cuda_backend_create(C.byref(opts), C.byref(ops), C.byref(status))
        if not handle:
            raise PGSError(status.value, "pgs_cuda_backend_create")
        super().__init__(ops.value, handle)

    def begin_record(self) -> None:
        check(self.lib.pgs_cuda_backend_begin_record(self.handle), "begin_record")

    def end_record(self) -> None:
        check(self.lib.pgs_cuda_backend_end_record(self.handle), "end_record")

    def replay(self, count: int = 1, reset_vram: bool = True, use_graph: bool = True) -> None:
        check(self.lib.pgs_cuda_backend_replay(self.handle, count, int(reset_vram), int(use_graph)), "replay")

    def stream(self) -> int:
        return self.lib.pgs_cuda_backend_stream(self.handle)

    def sample_circuit(self, d_dst_ptr: int, fbp: int, fbw: int, psm: int, width: int, height: int) -> None:
        """Progressive 1x read-out of a framebuffer rectangle at (0, 0) into device
        memory (RGBA8), queued on the backend's stream."""
        p = CircuitParams(fbp, fbw, psm, 0, 0, 0, 1, 1, width, height, width, height)
        check(self.lib.pgs_cuda_backend_sample_circuit(self.handle, C.byref(p), d_dst_ptr), "sample_circuit")

    def launches_per_replay(self) -> int:
        return int(self.lib.pgs_cuda_backend_launches_per_replay(self.handle))

    def fragments(self) -> int:
        v = C.c_uint64(0)
        check(self.lib.pgs_cuda_backend_fragment_count(self.handle, C.byref(v)), "fragment_count")
        return int(v.value)

    def stats(self) -> dict:
        st = BackendStats()
        check(self.lib.pgs_cuda_backend_get_stats(self.handle, C.byref(st)), "get_stats")
        return {"h2d_bytes": st.h2d_bytes, "d2h_bytes": st.d2h_bytes, "kernel_launches": st.kernel_launches,
                "render_passes": st.render_passes}

    def set_shade_timing(self, enable: bool) -> None:
        check(self.lib.pgs_cuda_backend_set_shade_timing(self.handle, int(enable)), "set_shade_timing")

    def last_shade_ms(self) -> float:
        v = C.c_float(0)
        check(self.lib.pgs_cuda_backend_last_shade_ms(self.handle, C.byref(v)), "last_shade_ms")
        return float(v.value)


class GSInterface:
    """GSInterface (gs/gs_interface.hpp:251-304) over any backend."""

    def __init__(self, backend: Backend, super_sampling: int = 1, ordered: bool = True, lib: C.CDLL | None = None,
                 super_sampled_textures: bool = False, dynamic_super_sampling: bool = False,
                 threaded_decode: int = THREADED_DECODE_AUTO):
        self.lib = lib or load_library()
        self.backend = backend
        opts = GSOptions(C.sizeof(GSOptions), super_sampling, int(ordered), VRAM_SIZE, int(dynamic_super_sampling),
                         int(super_sampled_textures), threaded_decode)
        status = C.c_int(0)
        self.handle = self.lib.pgs_gs_create(C.c_void_p(backend.ops), C.c_void_p(backend.handle), C.byref(opts),
                                             C.byref(status))
        if not self.handle:
            raise PGSError(status.value, "pgs_gs_create")

    def gif_transfer(self, path: int, data) -> None:
        buf = np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray, memoryview)) else \
            np.ascontiguousarray(data).view(np.uint8)
        check(self.lib.pgs_gs_gif_transfer(self.handle, path, buf.ctypes.data, buf.size), "gif_transfer")

    def write_register(self, addr: int, value: int) -> None:
        check(self.lib.pgs_gs_write_register(self.handle, addr, value & 0xFFFFFFFFFFFFFFFF), "write_register")

    def flush(self) -> None:
        check(self.lib.pgs_gs_flush(self.handle), "flush")

    def read_vram(self, offset: int = 0, size: int = VRAM_SIZE, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(size, dtype=np.uint8)
        check(self.lib.pgs_gs_read_vram(self.handle, offset, size, out.ctypes.data), "read_vram")
        return out

    def read_vram_async(self, out: np.ndarray, offset: int = 0, size: int | None = None) -> int:
        """Queues a read of plane 0 into `out` behind everything submitted so far;
        `out` is valid once wait(ticket) returns.  Pinned `out` is written by DMA
        directly, other memory through a pinned staging copy."""
        size = out.nbytes if size is None else size
        ticket = C.c_uint64()
        check(self.lib.pgs_gs_read_vram_async(self.handle, offset, size, out.ctypes.data, C.byref(ticket)),
              "read_vram_async")
        return int(ticket.value)

    def wait(self, ticket: int) -> None:
        check(self.lib.pgs_gs_wait(self.handle, ticket), "wait")

    def dump_open(self, path) -> None:
        """Restores the start state of a GS dump (PCSX2 / GSdx format)."""
        check(self.lib.pgs_gs_dump_open(self.handle, str(path).encode()), "dump_open")

    def dump_next_vsync(self):
        """Replays packets up to the next vsync; returns its field, or None at the end."""
        f = C.c_uint32(0)
        r = self.lib.pgs_gs_dump_next_vsync(self.handle, C.byref(f))
        if r < 0:
            check(r, "dump_next_vsync")
        return int(f.value) if r == 1 else None

    def dump_close(self) -> None:
        check(self.lib.pgs_gs_dump_close(self.handle), "dump_close")

    def dump_record_begin(self, path) -> None:
        check(self.lib.pgs_gs_dump_record_begin(self.handle, str(path).encode()), "dump_record_begin")

    def dump_record_vsync(self, field: int = 0) -> None:
        check(self.lib.pgs_gs_dump_record_vsync(self.handle, field), "dump_record_vsync")

    def dump_record_end(self) -> None:
        check(self.lib.pgs_gs_dump_record_end(self.handle), "dump_record_end")

    PRIV = {"PMODE": 0, "SMODE1": 1, "SMODE2": 2, "SRFSH": 3, "SYNCH1": 4, "SYNCH2": 5, "SYNCV": 6, "DISPFB1": 7,
            "DISPLAY1": 8, "DISPFB2": 9, "DISPLAY2": 10, "EXTBUF": 11, "EXTDATA": 12, "EXTWRITE": 13, "BGCOLOR": 14}
    SCANOUT_FORCE_PROGRESSIVE = 1
    SCANOUT_HIGH_RESOLUTION = 2

    def write_priv_register(self, reg, value: int) -> None:
        index = self.PRIV[reg] if isinstance(reg, str) else int(reg)
        check(self.lib.pgs_gs_write_priv_register(self.handle, index, value), "write_priv_register")

    def read_priv_register(self, reg) -> int:
        index = self.PRIV[reg] if isinstance(reg, str) else int(reg)
        v = C.c_uint64()
        check(self.lib.pgs_gs_read_priv_register(self.handle, index, C.byref(v)), "read_priv_register")
        return int(v.value)

    def scanout_circuit(self, circuit: int, phase: int = 0, flags: int = 0) -> np.ndarray:
        """RGBA8 image (height, width, 4) of CRTC circuit 0 or 1."""
        w, h = C.c_uint32(), C.c_uint32()
        cap = 4096 * 4096 * 4
        out = np.zeros(cap, dtype=np.uint8)
        check(self.lib.pgs_gs_scanout_circuit(self.handle, circuit, phase, flags, out.ctypes.data, cap, C.byref(w),
                                              C.byref(h)), "scanout_circuit")
        return out[: w.value * h.value * 4].reshape(h.value, w.value, 4).copy()

    VSYNC = {"FORCE_PROGRESSIVE": 1, "HIGH_RESOLUTION": 2, "OVERSCAN": 4, "CRTC_OFFSETS": 8, "ANTI_BLUR": 16,
             "ADAPT_HORIZONTAL": 32, "RAW_CIRCUIT": 64, "SKIP_DEINTERLACE": 128}

    def vsync(self, phase: int = 0, flags: int = 0):
        """One vsync: (RGBA8 image (height, width, 4), result dict)."""
        info = VsyncInfo(phase, flags)
        res = ScanoutResult()
        cap = 3840 * 2160 * 4
        out = np.zeros(cap, dtype=np.uint8)
        check(self.lib.pgs_gs_vsync(self.handle, C.byref(info), out.ctypes.data, cap, C.byref(res)), "vsync")
        d = {k: getattr(res, k) for k, _ in ScanoutResult._fields_ if k != "padding"}
        img = out[: res.width * res.height * 4].reshape(res.height, res.width, 4).copy()
        return img, d

    def vsync_can_skip(self, phase: int = 0, flags: int = 0) -> bool:
        """GSInterface::vsync_can_skip: progressive read-out with no recent tall SCANMSK primitive."""
        r = self.lib.pgs_gs_vsync_can_skip(self.handle, C.byref(VsyncInfo(phase, flags)))
        check(min(r, 0), "vsync_can_skip")
        return r == 1

    def set_hacks(self, disable_mipmaps: bool = False, unsynced_readbacks: bool = False,
                  backbuffer_promotion: bool = False, allow_blend_demote: bool = False) -> None:
        """GSInterface::set_hacks; backbuffer_promotion is not supported (PGSError)."""
        h = Hacks(int(disable_mipmaps), int(unsynced_readbacks), int(backbuffer_promotion), int(allow_blend_demote))
        check(self.lib.pgs_gs_set_hacks(self.handle, C.byref(h)), "set_hacks")

    def reset_context_state(self) -> None:
        check(self.lib.pgs_gs_reset_context_state(self.handle), "reset_context_state")

    def clobber_register_state(self) -> None:
        check(self.lib.pgs_gs_clobber_register_state(self.handle), "clobber_register_state")

    def read_register(self, addr: int) -> int:
        v = C.c_uint64()
        check(self.lib.pgs_gs_read_register(self.handle, addr, C.byref(v)), "read_register")
        return v.value

    def set_register(self, addr: int, value: int) -> None:
        check(self.lib.pgs_gs_set_register(self.handle, addr, value), "set_register")

    def get_gif_path(self, path: int) -> dict:
        p = GifPath()
        check(self.lib.pgs_gs_get_gif_path(self.handle, path, C.byref(p)), "get_gif_path")
        return {"tag": (p.tag[0], p.tag[1]), "reg": p.reg, "loop": p.loop}

    def set_gif_path(self, path: int, tag, reg: int = 0, loop: int = 0) -> None:
        p = GifPath((C.c_uint64 * 2)(*tag), reg, loop)
        check(self.lib.pgs_gs_set_gif_path(self.handle, path, C.byref(p)), "set_gif_path")

    def set_signal_interface(self, on_signal=None, on_finish=None, on_label=None) -> None:
        """Python callables taking the register value; a true result flushes."""
        def wrap(fn):
            return SIGNAL_FN(lambda user, payload: int(bool(fn(payload)))) if fn else SIGNAL_FN()
        self._signal = SignalInterface(wrap(on_signal), wrap(on_finish), wrap(on_label), None)
        check(self.lib.pgs_gs_set_signal_interface(self.handle, C.byref(self._signal)), "set_signal_interface")

    def set_debug_mode(self, timestamps: bool = False, feedback_render_target: bool = False,
                       deterministic_timeline_query: bool = False, disable_sampler_feedback: bool = False,
                       draw_mode: int = 0) -> None:
        m = DebugMode(int(feedback_render_target), int(timestamps), int(deterministic_timeline_query),
                      int(disable_sampler_feedback), draw_mode)
        check(self.lib.pgs_gs_set_debug_mode(self.handle, C.byref(m)), "set_debug_mode")

    def get_accumulated_timestamps(self, kind) -> float:
        """Seconds of GPU time in a stage (index or name from TIMESTAMPS)."""
        t = TIMESTAMPS.index(kind) if isinstance(kind, str) else int(kind)
        v = C.c_double()
        check(self.lib.pgs_gs_get_accumulated_timestamps(self.handle, t, C.byref(v)), "get_accumulated_timestamps")
        return v.value

    def write_vram(self, data, offset: int = 0) -> None:
        buf = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if isinstance(data, bytes) else data)
        check(self.lib.pgs_gs_write_vram(self.handle, offset, buf.nbytes, buf.ctypes.data), "write_vram")

    def read_transfer_fifo(self, num_128b_words: int) -> bytes:
        out = np.zeros(num_128b_words * 16, dtype=np.uint8)
        check(self.lib.pgs_gs_read_transfer_fifo(self.handle, out.ctypes.data, num_128b_words), "read_transfer_fifo")
        return out.tobytes()

    def consume_flush_stats(self) -> dict:
        st = FlushStats()
        check(self.lib.pgs_gs_consume_flush_stats(self.handle, C.byref(st)), "consume_flush_stats")
        return {"render_passes": st.num_render_passes, "primitives": st.num_primitives, "copies": st.num_copies,
                "palette_updates": st.num_palette_updates,
                "flush_reasons": list(st.num_flushes_by_reason)}

    def set_super_sampled_textures(self, enable: bool) -> None:
        check(self.lib.pgs_gs_set_super_sampled_textures(self.handle, int(enable)), "set_super_sampled_textures")

    def set_super_sampling_rate(self, super_sampling: int, ordered: bool = True) -> None:
        check(self.lib.pgs_gs_set_super_sampling_rate(self.handle, super_sampling, int(ordered)),
              "set_super_sampling_rate")

    def close(self) -> None:
        if self.handle:
            self.lib.pgs_gs_destroy(self.handle)
            self.handle = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Batched replay of several recorded CudaBackends (pgs_batch_*)."""

    def __init__(self, device: int = 0) -> None:
        self.lib = load_library()
        status = C.c_int(0)
        self.handle = self.lib.pgs_batch_create(device, C.byref(status))
        if not self.handle:
            raise PGSError(status.value, "pgs_batch_create")
        self.backends = []

    def add(self, backend: "CudaBackend") -> None:
        check(self.lib.pgs_batch_add(self.handle, backend.handle), "batch_add")
        self.backends.append(backend)

    def replay(self, count: int = 1, reset_vram: bool = True, use_graph: bool = True) -> None:
        check(self.lib.pgs_batch_replay(self.handle, count, int(reset_vram), int(use_graph)), "batch_replay")

    def set_tuning(self, cta_threads: int, ctas_per_sm: int, largest_first: bool = True, solo_min_prims: int = 0) -> None:
        t = BatchTuning(cta_threads, ctas_per_sm, int(largest_first), solo_min_prims)
        check(self.lib.pgs_batch_set_tuning(self.handle, C.byref(t)), "batch_set_tuning")

    def tuning(self) -> dict:
        t = BatchTuning()
        check(self.lib.pgs_batch_get_tuning(self.handle, C.byref(t)), "batch_get_tuning")
        return {"cta_threads": t.cta_threads, "ctas_per_sm": t.ctas_per_sm, "largest_first": bool(t.largest_first),
                "solo_min_prims": t.solo_min_prims}

    def autotune(self, trials: int = 3, reset_vram: bool = True) -> tuple[dict, float]:
        t = BatchTuning()
        ms = C.c_float(0.0)
        check(self.lib.pgs_batch_autotune(self.handle, trials, int(reset_vram), C.byref(t), C.byref(ms)), "autotune")
        return ({"cta_threads": t.cta_threads, "ctas_per_sm": t.ctas_per_sm, "largest_first": bool(t.largest_first),
                 "solo_min_prims": t.solo_min_prims}, float(ms.value))

    def stream(self) -> int:
        return self.lib.pgs_batch_stream(self.handle)

    def launches_per_replay(self) -> int:
        return int(self.lib.pgs_batch_launches_per_replay(self.handle))

    def synchronize(self) -> None:
        check(self.lib.pgs_batch_synchronize(self.handle), "batch_synchronize")

    def close(self) -> None:
        if self.handle:
            self.lib.pgs_batch_destroy(self.handle)
            self.handle = None


UPSCALER_SHAPES = [(4, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 4)]


def upscaler_init_params(seed: int = 0) -> np.ndarray:
    """He-initialised flat parameter vector (per layer: weights [tap][out][in],
    then biases); the last layer starts small so the network starts near the
    identity through its residual."""
    rng = np.random.default_rng(seed)
    parts = []
    for i, (cin, cout) in enumerate(UPSCALER_SHAPES):
        std = np.sqrt(2.0 / (9 * cin)) * (0.1 if i == len(UPSCALER_SHAPES) - 1 else 1.0)
        parts.append(rng.normal(0.0, std, size=9 * cout * cin).astype(np.float32))
        parts.append(np.zeros(cout, dtype=np.float32))
    return np.concatenate(parts)


class Upscaler:
    """BF16 tensor-core anti-aliasing network (pgs_upscaler_*).  Images are
    device tensors of shape (n, h, w, 4), uint8, contiguous (e.g. torch)."""

    def __init__(self, device: int = 0) -> None:
        self.lib = load_library()
        lib = self.lib
        vp, u32 = C.c_void_p, C.c_uint32
        lib.pgs_upscaler_create.argtypes = [C.c_int, C.POINTER(C.c_int)]
        lib.pgs_upscaler_create.restype = vp
        lib.pgs_upscaler_destroy.argtypes = [vp]
        lib.pgs_upscaler_destroy.restype = None
        lib.pgs_upscaler_param_count.argtypes = [vp]
        lib.pgs_upscaler_param_count.restype = u32
        for name in ("pgs_upscaler_set_params", "pgs_upscaler_get_params", "pgs_upscaler_get_gradient"):
            getattr(lib, name).argtypes = [vp, vp, u32]
        lib.pgs_upscaler_forward.argtypes = [vp, vp, u32, u32, u32, vp]
        lib.pgs_upscaler_backward.argtypes = [vp, vp, vp, u32, u32, u32, C.POINTER(C.c_double)]
        lib.pgs_upscaler_adam_step.argtypes = [vp, C.c_float]
        lib.pgs_upscaler_stream.argtypes = [vp]
        lib.pgs_upscaler_stream.restype = vp
        lib.pgs_upscaler_set_stream.argtypes = [vp, vp]
        lib.pgs_upscaler_synchronize.argtypes = [vp]
        lib.pgs_upscaler_set_tensor_path.argtypes = [vp, C.c_int]
        lib.pgs_upscaler_get_error.argtypes = [vp, C.POINTER(u32)]
        status = C.c_int(0)
        self.handle = lib.pgs_upscaler_create(device, C.byref(status))
        if not self.handle:
            raise PGSError(status.value, "pgs_upscaler_create")
        self.count = int(lib.pgs_upscaler_param_count(self.handle))

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        check(self.lib.pgs_upscaler_set_params(self.handle, p.ctypes.data, p.size), "upscaler_set_params")

    def params(self) -> np.ndarray:
        out = np.empty(self.count, dtype=np.float32)
        check(self.lib.pgs_upscaler_get_params(self.handle, out.ctypes.data, self.count), "upscaler_get_params")
        return out

    def gradient(self) -> np.ndarray:
        out = np.empty(self.count, dtype=np.float32)
        check(self.lib.pgs_upscaler_get_gradient(self.handle, out.ctypes.data, self.count), "upscaler_get_gradient")
        return out

    def forward(self, images, out) -> None:
        n, h, w, _ = images.shape
        check(self.lib.pgs_upscaler_forward(self.handle, images.data_ptr(), n, h, w, out.data_ptr()), "upscaler_forward")

    def backward(self, images, targets, want_loss: bool = True):
        n, h, w, _ = images.shape
        loss = C.c_double(0.0)
        check(self.lib.pgs_upscaler_backward(self.handle, images.data_ptr(), targets.data_ptr(), n, h, w,
                                             C.byref(loss) if want_loss else None), "upscaler_backward")
        return float(loss.value) if want_loss else None

    def set_tensor_path(self, tcgen05) -> None:
        """32->32 layers on tcgen05 (True or 2: two persistent CTAs per SM, 1: one)
        or on the mma.sync path (False / 0)."""
        mode = 2 if tcgen05 is True else int(tcgen05)
        check(self.lib.pgs_upscaler_set_tensor_path(self.handle, mode), "upscaler_set_tensor_path")

    def error_flags(self) -> int:
        v = C.c_uint32(0)
        self.lib.pgs_upscaler_get_error(self.handle, C.byref(v))
        return int(v.value)

    def adam_step(self, lr: float) -> None:
        check(self.lib.pgs_upscaler_adam_step(self.handle, lr), "upscaler_adam_step")

    def stream(self) -> int:
        return self.lib.pgs_upscaler_stream(self.handle)

    def set_stream(self, stream: int | None) -> None:
        """Queues later work on `stream` (a cudaStream_t pointer, e.g. a
        backend's stream()); None returns to the upscaler's own stream."""
        check(self.lib.pgs_upscaler_set_stream(self.handle, stream), "upscaler_set_stream")

    def synchronize(self) -> None:
        check(self.lib.pgs_upscaler_synchronize(self.handle), "upscaler_synchronize")

    def close(self) -> None:
        if self.handle:
            self.lib.pgs_upscaler_destroy(self.handle)
            self.handle = None


def umma_selftest(mode: int, device: int = 0) -> np.ndarray:
    """128x32 result of the tcgen05 self-test (pgs_umma_selftest)."""
    lib = load_library()
    lib.pgs_umma_selftest.argtypes = [C.c_int, C.c_uint32, C.c_void_p]
    out = np.zeros((128, 32), dtype=np.float32)
    check(lib.pgs_umma_selftest(device, mode, out.ctypes.data), "umma_selftest")
    return out
