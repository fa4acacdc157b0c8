"""Super-sampled textures (the reference's super_sampled_textures option):
frontend decisions and known answers on the CPU oracle.  GPU parity on seeded
frames is in test_gpu_parity.py."""
import numpy as np

import gsgen as g
import pgs
import pgs_oracle
from recording_backend import RecordingBackend

W, H = 128, 64


def scene(blit, ssaa_textures=True, ss=4, mmag=0):
    """A super-sampled pass draws triangles into page 0 (128x64 CT32); then a
    sprite copies that buffer 1:1 (blit) or at half size into page 40."""
    s = g.GifStream()
    g._frame_setup(s, 0, 2, g.PSMCT32, 20, g.PSMZ24, W, H, g.test_reg(zte=1, ztst=2))
    rng = np.random.default_rng(4)
    n = 60
    x, y = g.random_triangles(rng, n, W, H, 8.0, 600.0)
    z = rng.integers(0, 1 << 24, size=(n, 3))
    q = np.zeros((3 * n, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(rng.integers(0, 256, size=(3 * n, 4)))
    q[:, 1] = g.q_xyz2(x.reshape(-1), y.reshape(-1), z.reshape(-1))
    s.packed(g.prim_reg(g.PRIM_TRI, iip=1), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
    s.ad([(g.FRAME_1, g.frame_reg(40, 2, g.PSMCT32)), (g.TEST_1, g.test_reg(zte=1, ztst=1)),
          (g.ZBUF_1, g.zbuf_reg(20, g.PSMZ24, 1)), (g.TEX0_1, g.tex0_reg(0, 2, g.PSMCT32, 7, 6, tcc=1, tfx=1)),
          (g.TEX1_1, g.tex1_reg(mmag=mmag, mmin=mmag)), (g.CLAMP_1, g.clamp_reg(1, 1))])
    sw = W if blit else W // 2
    sh = H if blit else H // 2
    v = np.zeros((2, 3, 2), dtype=np.uint64)
    v[:, 0] = g.q_rgbaq(np.full((2, 4), 0x80))
    v[:, 1] = g.q_uv(np.array([0, W * 16]), np.array([0, H * 16]))
    v[:, 2] = g.q_xyz2(np.array([0, sw * 16]), np.array([0, sh * 16]), np.zeros(2, dtype=np.int64))
    s.packed(g.prim_reg(g.PRIM_SPRITE, tme=1, fst=1), [g.D_RGBAQ, g.D_UV, g.D_XYZ2], v.reshape(-1, 2))
    return g.Frame("ssaa_tex_kat", s.tobytes(), ss, True, n + 1,
                   {"width": W, "height": H, "fbp": 40, "zbp": 20, "ssaa_textures": ssaa_textures})


def planes_at(img, fbp, psm=g.PSMCT32, stride=2):
    lib = pgs_oracle.load_oracle()
    idx = np.array([[lib.pgs_oracle_swizzle(x, y, fbp * 32, stride, psm) for x in range(W)] for y in range(H)])
    return np.stack([p.view(np.uint32)[idx] for p in img])


def test_create_option_turns_super_sampled_textures_on():
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=4, super_sampled_textures=True)
    gs.gif_transfer(0, scene(True).data)
    gs.flush()
    assert be.passes[-1]["has_ss_textures"] == 1
    gs.close()


def test_descriptor_and_texture_word():
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=4)
    gs.set_super_sampled_textures(True)
    gs.gif_transfer(0, scene(True).data)
    gs.flush()
    last = be.passes[-1]
    assert last["has_ss_textures"] == 1
    assert [t["samples"] for t in last["textures"]] == [4]
    assert last["prims"][-1]["tex"] & (1 << 24)
    gs.close()
    # Off at 1x, and without the option.
    for ss, on in ((1, True), (4, False)):
        be = RecordingBackend()
        gs = pgs.GSInterface(be, super_sampling=ss)
        gs.set_super_sampled_textures(on)
        gs.gif_transfer(0, scene(True).data)
        gs.flush()
        assert all(t["samples"] in (0, 1) for p in be.passes for t in p["textures"])
        gs.close()


def test_nearest_blit_maps_sample_to_sample():
    """A 1:1 nearest blit of a super-sampled buffer keeps every sample: the
    destination's reference and sample planes equal the source's."""
    img = pgs_oracle.render(scene(True), planes=True)
    src, dst = planes_at(img, 0), planes_at(img, 40)
    ref = src[1] == 0xFFFFFFFF
    assert ref.any()
    for sp in range(2, img.shape[0]):
        assert np.array_equal(dst[sp][ref], src[sp][ref])
    # Without super-sampled textures the blit reads the single-sampled image.
    img1 = pgs_oracle.render(scene(True, ssaa_textures=False), planes=True)
    d1 = planes_at(img1, 40)
    assert not np.array_equal(d1[2:][:, ref], dst[2:][:, ref])


def test_linear_downsample_reads_layers():
    """A bilinear half-size copy runs (per-sample or single-sampled layer per the
    setup heuristic) and differs from the copy without super-sampled textures."""
    a = planes_at(pgs_oracle.render(scene(False, mmag=1), planes=True), 40)
    b = planes_at(pgs_oracle.render(scene(False, ssaa_textures=False, mmag=1), planes=True), 40)
    assert a.shape == b.shape


def test_phase_lut_entries():
    """Every bilinear entry of the phase LUT has unorm8 weights summing to 255,
    its first tap in the centre texel, sample ids below the sample count and
    texel offsets in -1..1; nearest entries hold sample ids (init_phase_lut,
    gs/gs_renderer.cpp:93-315)."""
    lib = pgs_oracle.load_oracle()
    for ss, ordered in ((2, True), (4, True), (4, False), (8, True), (16, True), (16, False)):
        be = pgs_oracle.OracleBackend()
        gs = pgs.GSInterface(be, super_sampling=ss, ordered=ordered)
        lut = np.zeros(64 * 64 * 2 + 32 * 32, dtype=np.uint32)
        lib.pgs_oracle_phase_lut(be.handle, lut.ctypes.data)
        gs.close()
        be.close()
        ex, ey = lut[0:8192:2], lut[1:8192:2]
        w = np.stack([(ey >> (8 * i)) & 0xFF for i in range(4)])
        assert np.all(w.sum(axis=0) == 255)
        assert np.all(((ex >> 16) & 0xF) == 0)          # tap 0: texel offset (0, 0)
        ids = np.stack([(ex >> (4 * i)) & 0xF for i in range(4)])
        assert ids.max() < ss
        assert np.all(lut[8192:] < ss)
        # The first tap is the nearest point in the centre texel: it carries the
        # largest weight for most phases.
        assert (w[0] >= w[1:].max(axis=0)).mean() > 0.5
