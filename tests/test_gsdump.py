"""GS dumps: the reader restores the start state and replays packets; the
writer's output replays to the same VRAM; a dump written in the reference
layout by an independent writer (gsgen.write_dump) replays the same way."""
import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle


def render(data, vram=None, ss=1):
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=ss)
    if vram is not None:
        gs.write_vram(vram)
    gs.gif_transfer(0, data)
    out = gs.read_vram()
    gs.close()
    be.close()
    return out


def test_recorded_dump_replays_to_same_vram(tmp_path):
    f = g.frame_c2(seed=17, num_triangles=300, num_sprites=30, super_sampling=1, num_textures=2)
    ref = render(f.data)
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    gs.dump_record_begin(tmp_path / "a.gs")
    gs.gif_transfer(0, f.data)
    gs.write_register(g.TEXFLUSH, 0)
    gs.dump_record_vsync(1)
    gs.dump_record_end()
    assert np.array_equal(gs.read_vram(), ref)
    gs.close()
    be.close()

    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    gs.dump_open(tmp_path / "a.gs")
    assert gs.dump_next_vsync() == 1
    assert gs.dump_next_vsync() is None
    assert np.array_equal(gs.read_vram(), ref)
    gs.close()
    be.close()


def test_start_state_is_restored(tmp_path):
    """VRAM and the register file come from the dump header, not from packets."""
    rng = np.random.default_rng(3)
    vram = rng.integers(0, 256, pgs.VRAM_SIZE, dtype=np.uint8).tobytes()
    setup = g.GifStream()
    g._frame_setup(setup, 0, 5, g.PSMCT32, 50, g.PSMZ24, 320, 240, g.test_reg(zte=1, ztst=2))
    draw = g.GifStream()
    x, y = g.random_triangles(rng, 200, 320, 240, 4.0, 2000.0)
    z = rng.integers(0, 1 << 24, size=(200, 3))
    rgba = rng.integers(0, 256, size=(600, 4))
    q = np.zeros((600, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(rgba)
    q[:, 1] = g.q_xyz2(x.reshape(600), y.reshape(600), z.reshape(600))
    draw.packed(g.prim_reg(g.PRIM_TRI, iip=1), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
    ref = render(setup.tobytes() + draw.tobytes(), vram=vram)
    regs = {g.PRMODECONT: 1, g.FRAME_1: g.frame_reg(0, 5, g.PSMCT32), g.ZBUF_1: g.zbuf_reg(50, g.PSMZ24),
            g.SCISSOR_1: g.scissor_reg(0, 319, 0, 239), g.TEST_1: g.test_reg(zte=1, ztst=2)}
    for version, serial in ((9, b""), (8, b"serial-and-screenshot")):
        path = tmp_path / ("b%d.gs" % version)
        g.write_dump(path, [(0, draw.tobytes())], vram=vram, regs=regs, version=version, serial=serial)
        be = pgs_oracle.OracleBackend()
        gs = pgs.GSInterface(be)
        gs.dump_open(path)
        assert gs.dump_next_vsync() == 0
        assert np.array_equal(gs.read_vram(), ref)
        gs.close()
        be.close()


def test_rejects_non_dumps(tmp_path):
    p = tmp_path / "x.gs"
    p.write_bytes(b"\\x00" * 64)
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    with pytest.raises(pgs.PGSError):
        gs.dump_open(p)
    with pytest.raises(pgs.PGSError):
        gs.dump_open(tmp_path / "missing.gs")
    gs.close()
    be.close()


@pytest.mark.gpu
def test_dump_replay_parity_on_cuda(tmp_path):
    """A three-frame dump recorded on the CUDA backend replays bit-exactly on
    both backends at every vsync (4x SSAA)."""
    frames = [g.frame_fuzz(seed=s) for s in (3, 8, 21)]
    be = pgs.CudaBackend(0, max_samples_log2=2)
    gs = pgs.GSInterface(be, super_sampling=4)
    gs.dump_record_begin(tmp_path / "c.gs")
    live = []
    for i, f in enumerate(frames):
        gs.gif_transfer(0, f.data)
        gs.dump_record_vsync(i & 1)
        live.append(gs.read_vram())
    gs.dump_record_end()
    gs.close()
    assert be.error_flags() == 0
    be.close()

    for make in (lambda: pgs.CudaBackend(0, max_samples_log2=2), pgs_oracle.OracleBackend):
        be = make()
        gs = pgs.GSInterface(be, super_sampling=4)
        gs.dump_open(tmp_path / "c.gs")
        for i, want in enumerate(live):
            assert gs.dump_next_vsync() == (i & 1)
            assert np.array_equal(gs.read_vram(), want), "vsync %d" % i
        assert gs.dump_next_vsync() is None
        gs.close()
        be.close()
