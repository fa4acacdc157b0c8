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


# Copies into the rendered colour buffer (FBP 0, 640 wide), so that they clear
# super-sample reference bits a 4x render left there.
SS_COPIES = [
    regs(8192, 4, PSMCT32, 0, 10, PSMCT32, 0, 0, 16, 16, 256, 128),
    regs(9216, 2, PSMCT16, 0, 10, PSMCT16, 4, 4, 300, 40, 96, 64),
    regs(10240, 4, PSMT8, 0, 10, PSMT8, 0, 3, 64, 200, 128, 32),
    regs(0, 10, PSMCT32, 0, 10, PSMCT32, 100, 100, 120, 110, 64, 64),
]


def _entry_point():
    lib = pgs.load_library()
    fn = lib.pgs_vram_local_copy_noalloc
    fn.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(CopyDesc), C.c_void_p]
    fn.restype = C.c_int
    return fn


def test_noalloc_copy_clears_reference_plane_like_copy_vram():
    """On a 4x super-sampled backend copy_vram also clears the destination's
    bits in the super-sample reference plane (plane 1).  The entry point does
    the same when it is given every plane; all six planes must match after each
    of several copies in a row."""
    torch = pytest.importorskip("torch")
    import gsgen

    fn = _entry_point()
    frame = gsgen.frame_c2(seed=3, num_triangles=300, num_sprites=30, super_sampling=4, num_textures=2)
    backend = pgs.CudaBackend(0, max_samples_log2=2)
    gs = pgs.GSInterface(backend, super_sampling=4)
    num_planes = 2 + 4
    try:
        gs.gif_transfer(0, frame.data)
        gs.flush()
        planes = np.stack([backend.read_plane(p) for p in range(num_planes)])
        # The render left reference bits for the copies to clear.
        assert np.count_nonzero(planes[1]) > 0
        device_vram = torch.from_numpy(planes.reshape(-1).copy()).cuda()
        torch.cuda.synchronize()
        for bitbltbuf, trxpos, trxreg in SS_COPIES:
            before = device_vram.cpu().numpy().reshape(num_planes, -1)
            gs.write_register(BITBLTBUF, bitbltbuf)
            gs.write_register(TRXPOS, trxpos)
            gs.write_register(TRXREG, trxreg)
            gs.write_register(TRXDIR, 2)
            gs.flush()
            expected = np.stack([backend.read_plane(p) for p in range(num_planes)])

            desc = CopyDesc(bitbltbuf, trxpos, trxreg, 2, None, 0, 0, 0)
            assert fn(C.c_void_p(device_vram.data_ptr()), num_planes, C.byref(desc), None) == 0
            torch.cuda.synchronize()
            got = device_vram.cpu().numpy().reshape(num_planes, -1)
            for p in range(num_planes):
                assert np.array_equal(got[p], expected[p]), "plane %d differs" % p
            assert not np.array_equal(got[0], before[0])
        # Some reference bits were cleared, so plane 1 was really exercised.
        assert np.count_nonzero(got[1]) < np.count_nonzero(planes[1])
    finally:
        gs.close()
        backend.close()


def test_noalloc_copy_accepts_exactly_the_limit():
    """A rectangle of exactly PGS_NOALLOC_COPY_MAX_PIXELS (512 x 512) is copied
    bit-exactly; one more row is refused with PGS_ERROR_CAPACITY and leaves
    VRAM untouched."""
    torch = pytest.importorskip("torch")
    fn = _entry_point()
    rng = np.random.default_rng(11)
    init = rng.integers(0, 256, size=pgs.VRAM_SIZE, dtype=np.uint8)
    backend = pgs.CudaBackend(0, max_samples_log2=0)
    gs = pgs.GSInterface(backend, super_sampling=1)
    try:
        gs.write_vram(init)
        device_vram = torch.from_numpy(init.copy()).cuda()
        torch.cuda.synchronize()
        bitbltbuf, trxpos, trxreg = regs(0, 8, PSMCT32, 8192, 8, PSMCT32, 0, 0, 0, 0, 512, 512)
        assert 512 * 512 == 256 * 1024
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

        bitbltbuf, trxpos, trxreg = regs(0, 8, PSMCT32, 0, 8, PSMCT32, 0, 0, 0, 1, 512, 513)
        desc = CopyDesc(bitbltbuf, trxpos, trxreg, 2, None, 0, 0, 0)
        assert fn(C.c_void_p(device_vram.data_ptr()), 1, C.byref(desc), None) == \
            pgs.STATUS_CODES["PGS_ERROR_CAPACITY"]
        torch.cuda.synchronize()
        assert np.array_equal(device_vram.cpu().numpy(), expected)
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
