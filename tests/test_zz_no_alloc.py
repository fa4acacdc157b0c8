"""Allocation-free local->local VRAM copy (pgs_vram_local_copy_noalloc).

Some callers cannot allocate device memory at the point where they need a VRAM
copy: code running under another framework's memory pool or inside a stream
capture, or a latency-critical path with a no-cudaMalloc rule.  They own the
VRAM image and call this entry point, which stages the source rectangle in a
fixed device array of the library instead of allocating.  This test drives the
same copies through the backend's normal path (copy_vram via the frontend's
TRXDIR write) and through the allocation-free entry point on a copy of the same
VRAM, and requires identical bytes after each of several calls in a row.  The
file sorts last so that a run stopping at the first failure has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

import pgs

pytestmark = pytest.mark.gpu

BITBLTBUF, TRXPOS, TRXREG, TRXDIR = 0x50, 0x51, 0x52, 0x53
PSMCT32, PSMCT16, PSMCT16S, PSMT8, PSMT4 = 0x00, 0x02, 0x0A, 0x13, 0x14


class CopyDesc(C.Structure):
    _fields_ = [("bitbltbuf", C.c_uint64), ("trxpos", C.c_uint64), ("trxreg", C.c_uint64),
                ("trxdir", C.c_uint64), ("host_data", C.c_void_p), ("host_size", C.c_uint64),
                ("host_offset", C.c_uint64), ("host_required", C.c_uint64)]


def regs(sbp, sbw, spsm, dbp, dbw, dpsm, ssax, ssay, dsax, dsay, w, h):
    bitbltbuf = sbp | (sbw << 16) | (spsm << 24) | (dbp << 32) | (dbw << 48) | (dpsm << 56)
    trxpos = ssax | (ssay << 16) | (dsax << 32) | (dsay << 48)
    trxreg = w | (h << 32)
    return bitbltbuf, trxpos, trxreg


COPIES = [
    # 32-bit rectangle into another buffer.
    regs(0, 10, PSMCT32, 4096, 4, PSMCT32, 5, 7, 3, 2, 200, 90),
    # 8-bit copy whose source and destination overlap.
    regs(8192, 4, PSMT8, 8192, 4, PSMT8, 10, 5, 40, 20, 128, 64),
    # 16-bit source into a 4-bit destination (nibble writes).
    regs(2048, 2, PSMCT16, 12288, 2, PSMT4, 3, 1, 8, 8, 64, 48),
    # 16S into 16S with wrap-around source coordinates.
    regs(1024, 1, PSMCT16S, 1536, 2, PSMCT16S, 2040, 60, 0, 0, 32, 16),
]


def test_noalloc_copy_matches_copy_vram_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    lib = pgs.load_library()
    fn = lib.pgs_vram_local_copy_noalloc
    fn.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(CopyDesc), C.c_void_p]
    fn.restype = C.c_int

    rng = np.random.default_rng(7)
    init = rng.integers(0, 256, size=pgs.VRAM_SIZE, dtype=np.uint8)
    backend = pgs.CudaBackend(0, max_samples_log2=0)
    gs = pgs.GSInterface(backend, super_sampling=1)
    try:
        gs.write_vram(init)
        device_vram = torch.from_numpy(init.copy()).cuda()
        torch.cuda.synchronize()
        for bitbltbuf, trxpos, trxreg in COPIES:
            gs.write_register(BITBLTBUF, bitbltbuf)
            gs.write_register(TRXPOS, trxpos)
            gs.write_register(TRXREG, trxreg)
            gs.write_register(TRXDIR, 2)
            expected = gs.read_vram()

            desc = CopyDesc(bitbltbuf, trxpos, trxreg, 2, None, 0, 0, 0)
            assert fn(C.c_void_p(device_vram.data_ptr()), 1, C.byref(desc), None) == 0
            torch.cuda.synchronize()
            got = device_vram.cpu().numpy()
            assert np.array_equal(got, expected)
            # The copy changed something, so the comparison is not vacuous.
            assert not np.array_equal(got, init)
    finally:
        gs.close()
        backend.close()


def test_noalloc_copy_rejects_oversized_rectangles():
    torch = pytest.importorskip("torch")
    lib = pgs.load_library()
    fn = lib.pgs_vram_local_copy_noalloc
    fn.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(CopyDesc), C.c_void_p]
    fn.restype = C.c_int
    vram = torch.zeros(pgs.VRAM_SIZE, dtype=torch.uint8, device="cuda")
    bitbltbuf, trxpos, trxreg = regs(0, 16, PSMCT32, 0, 16, PSMCT32, 0, 0, 0, 0, 1024, 512)
    desc = CopyDesc(bitbltbuf, trxpos, trxreg, 2, None, 0, 0, 0)
    assert fn(C.c_void_p(vram.data_ptr()), 1, C.byref(desc), None) == pgs.STATUS_CODES["PGS_ERROR_CAPACITY"]
    desc.trxdir = 0
    assert fn(C.c_void_p(vram.data_ptr()), 1, C.byref(desc), None) == pgs.STATUS_CODES["PGS_ERROR_INVALID_ARGUMENT"]
