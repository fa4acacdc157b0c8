"""Field-aware rendering, the SCANMSK progressive-scan timeout, vsync_can_skip
and the hacks (disable_mipmaps, allow_blend_demote): frontend decisions on a
recording backend and their effect on the CPU oracle.  GPU parity on seeded
frames is in test_gpu_parity.py."""
import copy

import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle
from recording_backend import RecordingBackend

FIELD = pgs.GSInterface.VSYNC["FORCE_PROGRESSIVE"] | pgs.GSInterface.VSYNC["HIGH_RESOLUTION"]
NTSC = (32 << 3) | (2 << 13)
PROGRESSIVE = (32 << 3)


def small_pass(height=64, tall=False):
    """A few flat triangles into a 128 x height CT32 frame (one pass)."""
    s = g.GifStream()
    h = 448 if tall else height
    g._frame_setup(s, 0, 2, g.PSMCT32, 40, g.PSMZ24, 128, h, g.test_reg(zte=1, ztst=1))
    rng = np.random.default_rng(3)
    n = 20
    x, y = g.random_triangles(rng, n, 128, h, 30.0, 2000.0)
    q = np.zeros((3 * n, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(rng.integers(0, 256, size=(3 * n, 4)))
    q[:, 1] = g.q_xyz2(x.reshape(-1), y.reshape(-1), np.zeros(3 * n, dtype=np.int64))
    s.packed(g.prim_reg(g.PRIM_TRI, iip=1), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
    return s.tobytes()


def field_pass(smode1=NTSC, smode2=3, flags=FIELD, ss=4):
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=ss)
    gs.write_priv_register("SMODE1", smode1)
    gs.write_priv_register("SMODE2", smode2)
    gs.vsync(0, flags)
    gs.gif_transfer(0, small_pass())
    gs.flush()
    rp = be.passes[-1]
    gs.close()
    return rp


def test_field_aware_needs_high_resolution_field_rendering_and_ssaa():
    assert field_pass()["field_aware"] == 1
    assert field_pass(flags=pgs.GSInterface.VSYNC["FORCE_PROGRESSIVE"])["field_aware"] == 0
    assert field_pass(smode2=1)["field_aware"] == 0              # INT without FFMD
    assert field_pass(smode2=2)["field_aware"] == 0              # FFMD without INT
    assert field_pass(smode1=PROGRESSIVE)["field_aware"] == 0
    assert field_pass(ss=1)["field_aware"] == 0
    # The raw flag decides, not the read-out that vsync settles on: without
    # FORCE_PROGRESSIVE the read-out is not high resolution, the rendering is
    # still field aware (gs/gs_interface.cpp:4666-4670).
    assert field_pass(flags=pgs.GSInterface.VSYNC["HIGH_RESOLUTION"])["field_aware"] == 1


def test_field_aware_keeps_pass_super_sampled_and_untightened_box():
    """Channel shuffles demote a super-sampled pass to 1x, except under
    field-aware rendering; the instance box is not tightened by the
    top-left rule then."""
    def shuffle_pass(flags):
        be = RecordingBackend()
        gs = pgs.GSInterface(be, super_sampling=4)
        gs.write_priv_register("SMODE1", NTSC)
        gs.write_priv_register("SMODE2", 3)
        gs.vsync(0, flags)
        s = g.GifStream()
        g._frame_setup(s, 0, 2, g.PSMCT16, 40, g.PSMZ24, 128, 64, g.test_reg(zte=0))
        s.ad([(g.FRAME_1, g.frame_reg(0, 2, g.PSMCT16, fbmsk=0x3FFF))])
        q = np.zeros((3, 2, 2), dtype=np.uint64)
        q[:, 0] = g.q_rgbaq(np.full((3, 4), 200))
        q[:, 1] = g.q_xyz2(np.array([8 * 16 + 9, 60 * 16, 30 * 16]), np.array([4 * 16 + 9, 10 * 16, 50 * 16]),
                           np.zeros(3, dtype=np.int64))
        s.packed(g.prim_reg(g.PRIM_TRI), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
        gs.gif_transfer(0, s.tobytes())
        gs.flush()
        rp = be.passes[-1]
        gs.close()
        return rp
    plain, field = shuffle_pass(pgs.GSInterface.VSYNC["FORCE_PROGRESSIVE"]), shuffle_pass(FIELD)
    assert plain["instances"][0]["sampling_rate_y_log2"] == 0
    assert field["instances"][0]["sampling_rate_y_log2"] == 1
    # Vertex 0 at (8 + 9/16, 4 + 9/16): tightened, the box starts at row 5;
    # field aware it starts at row 4.
    assert plain["prims"][0]["bb"][:2] == [9, 5]
    assert field["prims"][0]["bb"][:2] == [8, 4]


def test_field_aware_oracle_rows_snap_for_short_instances_only():
    """Field-aware rendering changes super-sampled output of a frame that ends
    above row 256 and leaves a 448-row frame as it was."""
    for tall, changes in ((False, True), (True, False)):
        f = g.Frame("fa", small_pass(tall=tall), 4, True, 20, {})
        a = pgs_oracle.render(f, planes=True)
        f2 = copy.deepcopy(f)
        f2.meta["field_aware"] = True
        b = pgs_oracle.render(f2, planes=True)
        assert (not np.array_equal(a, b)) == changes


def tall_scanmsk_stream(height):
    s = g.GifStream()
    g._frame_setup(s, 0, 10, g.PSMCT32, 100, g.PSMZ24, 640, 448, g.test_reg(zte=0))
    s.ad([(g.SCANMSK, 2)])
    q = np.zeros((2, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(np.full((2, 4), 100))
    q[:, 1] = g.q_xyz2(np.array([0, 64 * 16]), np.array([0, height * 16]), np.zeros(2, dtype=np.int64))
    s.packed(g.prim_reg(g.PRIM_SPRITE), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
    return s.tobytes()


@pytest.mark.parametrize("height,tall", [(448, True), (300, False)])
def test_complex_scanmsk_timeout(height, tall):
    """A SCANMSK primitive taller than 400 rows switches progressive read-out
    off for 4 vsyncs (gs/gs_interface.cpp:1947-1959, 4631-4637): an
    alternating-field NTSC scan-out reports interlaced meanwhile, and
    vsync_can_skip is false until the countdown ends."""
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=1)
    gs.write_priv_register("SMODE1", NTSC)
    gs.write_priv_register("SMODE2", 1)  # INT, field per frame: progressive when forced
    fp = pgs.GSInterface.VSYNC["FORCE_PROGRESSIVE"]
    assert gs.vsync_can_skip(0, fp)
    gs.gif_transfer(0, tall_scanmsk_stream(height))
    seen = []
    for _ in range(6):
        skip = gs.vsync_can_skip(0, fp)
        _, res = gs.vsync(0, fp)
        seen.append((skip, res["interlaced"]))
    gs.close()
    if tall:
        assert seen == [(False, 1)] * 4 + [(True, 0)] * 2
    else:
        assert seen == [(True, 0)] * 6
    # Without FORCE_PROGRESSIVE the output is interlaced and never skippable.
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=1)
    gs.write_priv_register("SMODE2", 1)
    assert not gs.vsync_can_skip(0, 0)
    gs.close()


def test_hacks_disable_mipmaps_and_blend_demote_flags():
    f = g.frame_mip(3)
    for hack, levels_one in ((False, False), (True, True)):
        be = RecordingBackend()
        gs = pgs.GSInterface(be, super_sampling=f.super_sampling)
        gs.set_hacks(disable_mipmaps=hack, allow_blend_demote=hack)
        gs.gif_transfer(0, f.data)
        gs.flush()
        levels = [t["levels"] for rp in be.passes for t in rp["textures"]]
        assert all(l == 1 for l in levels) == levels_one
        assert all(rp["has_mipmap"] == 0 for rp in be.passes) == levels_one
        assert all(rp["blend_demote"] == int(hack) for rp in be.passes)
        gs.close()


def test_backbuffer_promotion_is_refused():
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    with pytest.raises(pgs.PGSError) as e:
        gs.set_hacks(backbuffer_promotion=True)
    assert e.value.status == pgs.STATUS_CODES["PGS_ERROR_UNSUPPORTED"]
    gs.close()


def test_blend_demote_oracle():
    """Crowded blended tiles without depth writes go single-sampled when every
    state of the pass blends (even seeds); one unblended state keeps the pass
    as it was (odd seeds)."""
    for seed in (0, 1):
        f = g.frame_blend_demote(seed)
        a = pgs_oracle.render(f, planes=True)
        f2 = copy.deepcopy(f)
        f2.meta["hacks"] = {}
        b = pgs_oracle.render(f2, planes=True)
        assert (not np.array_equal(a, b)) == (seed % 2 == 0)
