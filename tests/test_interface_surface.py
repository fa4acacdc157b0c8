"""The rest of GSInterface's surface (gs/gs_interface.hpp:251-304):
reset_context_state, clobber_register_state, register file and GIF path
accessors, the signal interface and debug mode / timestamps, on the recording
backend and the CPU oracle."""
import ctypes as C

import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle
from recording_backend import RecordingBackend

SIGNAL, FINISH, LABEL = 0x60, 0x61, 0x62


def qwords(*pairs) -> bytes:
    return np.array(pairs, dtype=np.uint64).tobytes()


def ad_tag(nloop):
    """PACKED GIFtag with one A+D register per loop."""
    return g.gif_tag(nloop, 0, 1, g.D_AD)


def ad(addr, value):
    return (value, addr)


def triangle_stream(fbp=0):
    s = g.GifStream()
    g._frame_setup(s, fbp, 2, g.PSMCT32, 40, g.PSMZ24, 128, 64, g.test_reg(zte=0))
    q = np.zeros((3, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(np.full((3, 4), 90))
    q[:, 1] = g.q_xyz2(np.array([0, 600, 100]), np.array([0, 80, 500]), np.zeros(3, dtype=np.int64))
    s.packed(g.prim_reg(g.PRIM_TRI), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
    return s


def test_reset_context_state_returns_registers_and_paths_to_power_on():
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    gs.gif_transfer(0, triangle_stream().tobytes())
    assert gs.read_register(g.FRAME_1) != 0
    # Leave path 2 inside a PACKED GIFtag of 3 loops.
    gs.gif_transfer(2, qwords(ad_tag(3), ad(g.SCISSOR_1, 5)))
    assert gs.get_gif_path(2)["loop"] == 1
    gs.reset_context_state()
    assert gs.read_register(g.FRAME_1) == 0
    # The reference's power-on file is all zero, PRMODECONT.AC included.
    assert gs.read_register(g.PRMODECONT) == 0
    assert gs.get_gif_path(2) == {"tag": (0, 0), "reg": 0, "loop": 0}
    # The triangle drawn before the reset was flushed by it.
    assert sum(len(p["prims"]) for p in be.passes) == 1
    gs.close()


def test_set_register_and_clobber_rebuild_state():
    """A FRAME stored without side effects takes effect on the next draw after
    clobber_register_state."""
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    s = triangle_stream(fbp=0)
    gs.gif_transfer(0, s.tobytes())
    gs.flush()
    gs.set_register(g.FRAME_1, g.frame_reg(20, 2, g.PSMCT32))
    gs.clobber_register_state()
    q = np.zeros((3, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(np.full((3, 4), 90))
    q[:, 1] = g.q_xyz2(np.array([0, 600, 100]), np.array([0, 80, 500]), np.zeros(3, dtype=np.int64))
    s2 = g.GifStream()
    s2.packed(g.prim_reg(g.PRIM_TRI), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
    gs.gif_transfer(0, s2.tobytes())
    gs.flush()
    assert be.passes[-1]["instances"][0]["frame"] & 0x1FF == 20
    with pytest.raises(pgs.PGSError):
        gs.read_register(128)
    gs.close()


def test_gif_path_set_validates_and_resumes():
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    tag = ad_tag(2)
    with pytest.raises(pgs.PGSError):
        gs.set_gif_path(1, tag, reg=0, loop=3)   # loop > NLOOP
    assert gs.get_gif_path(1)["loop"] == 0
    # Resume a path one loop into its tag: the next qword is its second A+D.
    gs.set_gif_path(1, tag, reg=0, loop=1)
    gs.gif_transfer(1, qwords(ad(g.FOGCOL, 0x123456)))
    assert gs.read_register(g.FOGCOL) == 0x123456
    assert gs.get_gif_path(1)["loop"] == 2
    gs.close()


def test_signal_interface_callbacks_and_flush():
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    seen = []
    gs.set_signal_interface(on_signal=lambda v: seen.append(("signal", v)) or True,
                            on_finish=lambda v: seen.append(("finish", v)) or False,
                            on_label=lambda v: seen.append(("label", v)) or False)
    s = triangle_stream()
    s.ad([(FINISH, 7), (LABEL, 0x55)])
    gs.gif_transfer(0, s.tobytes())
    assert seen == [("finish", 7), ("label", 0x55)]
    assert len(be.passes) == 0          # no flush asked for
    s = g.GifStream()
    s.ad([(SIGNAL, 0x1234)])
    gs.gif_transfer(0, s.tobytes())
    assert seen[-1] == ("signal", 0x1234)
    assert len(be.passes) == 1          # the true result flushed the pending triangle
    gs.set_signal_interface()
    gs.gif_transfer(0, s.tobytes())
    assert len(seen) == 3
    gs.close()


def test_debug_mode_without_backend_timing():
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    gs.set_debug_mode(timestamps=True, draw_mode=2)
    gs.gif_transfer(0, triangle_stream().tobytes())
    gs.flush()
    assert all(gs.get_accumulated_timestamps(k) == 0.0 for k in pgs.TIMESTAMPS)
    with pytest.raises(pgs.PGSError):
        gs.set_debug_mode(draw_mode=3)
    with pytest.raises(pgs.PGSError):
        gs.get_accumulated_timestamps(9)
    gs.close()
    be.close()


def test_super_sampling_rate_is_lowered_to_what_the_backend_supports():
    """set_super_sampling_rate takes min(requested, the backend's maximum)
    (gs/gs_interface.cpp:69-70) instead of failing; 1x turns super-sampled
    textures off (:74-78)."""
    be = RecordingBackend(max_samples_log2=2)
    gs = pgs.GSInterface(be, super_sampling=16, super_sampled_textures=True)
    # 16x (2, 2) and 8x (1, 2) are refused by a 4-plane backend; 4x ordered is taken.
    assert be.ss[-1] == (1, 1)
    gs.set_super_sampling_rate(8)
    assert be.ss[-1] == (1, 1)
    gs.set_super_sampling_rate(2)
    assert be.ss[-1] == (0, 1)
    gs.set_super_sampling_rate(16, ordered=False)
    assert be.ss[-1] == (0, 2)
    gs.close()

    be = RecordingBackend(max_samples_log2=0)
    gs = pgs.GSInterface(be, super_sampling=4, super_sampled_textures=True)
    assert be.ss[-1] == (0, 0)
    gs.close()


def test_options_struct_size_reads_older_layouts():
    """pgs_gs_options.struct_size: fields past it read as zero, so a caller
    built against the three-field layout gets no super-sampled textures."""
    lib = pgs.load_library()
    be = RecordingBackend()
    full = pgs.GSOptions(0, 4, 1, pgs.VRAM_SIZE, 0, 1)
    short = pgs.GSOptions(16, 4, 1, pgs.VRAM_SIZE, 1, 1)
    status = C.c_int(0)
    for opts in (full, short):
        h = lib.pgs_gs_create(C.c_void_p(be.ops), C.c_void_p(be.handle), C.byref(opts), C.byref(status))
        assert h and status.value == 0
        lib.pgs_gs_destroy(C.c_void_p(h))
    assert be.ss[-1] == (1, 1)
    bad = pgs.GSOptions(4, 4, 1, pgs.VRAM_SIZE, 0, 0)
    h = lib.pgs_gs_create(C.c_void_p(be.ops), C.c_void_p(be.handle), C.byref(bad), C.byref(status))
    assert not h and status.value == pgs.STATUS_CODES["PGS_ERROR_INVALID_ARGUMENT"]
