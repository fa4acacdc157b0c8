"""Mipmapping: the frontend's texture descriptors (levels, MIPTBP / MTBA bases,
per-level page hazards) and known answers of the oracle's LOD selection and
trilinear blend (sample_texture, gs/shaders/ubershader.comp:1064-1131,
1230-1255).  GPU parity on seeded mip frames is in test_gpu_parity.py."""
import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle
from recording_backend import RecordingBackend

W, H = 64, 32
COLORS = [(200, 16, 40, 128), (30, 220, 60, 128), (90, 100, 250, 128), (12, 34, 56, 128)]


def chain_stream(auto=False, tex1=0, q=1.0, st=(0.5, 0.5), fst=False, uv=(0, 0), mxl_levels=4, upload=True):
    """A 64x64 CT32 texture whose level l is the solid colour COLORS[l], then one
    sprite covering a 64x32 framebuffer with TEX1 = tex1."""
    s = g.GifStream()
    s.ad([(g.PRMODECONT, 1), (g.FRAME_1, g.frame_reg(0, 1, g.PSMCT32)), (g.ZBUF_1, g.zbuf_reg(100, g.PSMZ24)),
          (g.SCISSOR_1, g.scissor_reg(0, W - 1, 0, H - 1)), (g.XYOFFSET_1, 0), (g.TEST_1, g.test_reg(zte=1, ztst=1))])
    tw = th = 6
    levels = []
    if auto:
        base, row, blocks = 32 * 10, 1, 64 * 64 // 64
        for lv in range(4):
            levels.append((base, max(row, 1)))
            base += blocks
            blocks //= 4
            row //= 2
    else:
        levels = [((10 + 2 * lv) * 32, 1) for lv in range(mxl_levels)]
    for lv, (tbp, tbw) in enumerate(levels if upload else []):
        # A transfer shorter than 64 bits writes nothing: the 1x1 level goes up as 2x1.
        n = 64 >> lv
        px = np.tile(np.array(COLORS[lv % 4], dtype=np.uint8), max(n, 2) * n).tobytes()
        s.upload(tbp, tbw, g.PSMCT32, 0, 0, max(n, 2), n, px)
    regs = [(g.TEX1_1, tex1)]
    if not auto:
        regs.append((g.MIPTBP1_1, g.miptbp_reg(levels[1:4])))
        regs.append((g.MIPTBP2_1, g.miptbp_reg(levels[4:7])))
    regs.append((g.TEX0_1, g.tex0_reg(levels[0][0], 1, g.PSMCT32, tw, th, tcc=1, tfx=1)))
    regs.append((g.CLAMP_1, g.clamp_reg(1, 1)))
    s.ad(regs)
    n = 2
    x = np.array([0, W * 16], dtype=np.int64)
    y = np.array([0, H * 16], dtype=np.int64)
    z = np.array([5, 5], dtype=np.int64)
    rgba = np.full((n, 4), 128, dtype=np.int64)
    if fst:
        desc = [g.D_RGBAQ, g.D_UV, g.D_XYZ2]
        cols = [g.q_rgbaq(rgba), g.q_uv(np.array([uv[0]] * n), np.array([uv[1]] * n)), g.q_xyz2(x, y, z)]
    else:
        qq = np.full(n, q, dtype=np.float32)
        desc = [g.D_RGBAQ, g.D_ST, g.D_XYZ2]
        cols = [g.q_rgbaq(rgba), g.q_st(np.full(n, st[0] * q, np.float32), np.full(n, st[1] * q, np.float32), qq),
                g.q_xyz2(x, y, z)]
    s.packed(g.prim_reg(g.PRIM_SPRITE, tme=1, fst=int(fst)), desc, np.stack(cols, axis=1).reshape(-1, 2))
    return s.tobytes()


def pixel(data):
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    gs.gif_transfer(0, data)
    v = gs.read_vram()
    gs.close()
    be.close()
    return tuple(int(c) for c in v[0:4])


def lin(a, b, w):
    out = []
    for ca, cb in zip(a, b):
        acc = (16 - w) * ca + w * cb
        r, f = acc >> 4, acc & 15
        out.append(r + (1 if f > 8 or (f == 8 and r & 1) else 0))
    return tuple(out)


@pytest.mark.parametrize("k,level", [(0, 0), (16, 1), (32, 2), (48, 3), (-16, 0), (112, 3)])
def test_fixed_lod_selects_level(k, level):
    """LCM = 1: LOD = K >> 4 clamped to [0, MXL]; MMIN nearest-mipmap-nearest."""
    tex1 = g.tex1_reg(lcm=1, mxl=3, mmin=2, k=k & 0xFFF)
    assert pixel(chain_stream(tex1=tex1)) == COLORS[level]


@pytest.mark.parametrize("q,k,l,want", [(1.0, 0, 0, 0), (0.5, 0, 0, 1), (0.25, 0, 0, 2), (0.125, 0, 0, 3),
                                         (2.0, 0, 0, 0), (0.5, -16, 0, 0), (0.5, 0, 1, 2), (1.0, 40, 0, 3)])
def test_lod_from_q(q, k, l, want):
    """LCM = 0: LOD = ceil(-log2|Q| * 2^(L+4) + K) / 16, nearest level (MMIN 4 rounds
    LOD + 0.5 down to the level)."""
    tex1 = g.tex1_reg(lcm=0, mxl=3, mmin=4, l=l, k=k & 0xFFF)
    assert pixel(chain_stream(tex1=tex1, q=q)) == COLORS[want]


@pytest.mark.parametrize("k", [8, 24, 4, 36])
def test_trilinear_blends_two_levels(k):
    """MMIN 5 (linear-mipmap-linear): floor(fract * 16) / 16 of the next level."""
    tex1 = g.tex1_reg(lcm=0, mxl=3, mmin=5, k=k)
    lo, w = k // 16, k % 16
    assert pixel(chain_stream(tex1=tex1, q=1.0)) == lin(COLORS[lo], COLORS[lo + 1], w)


def test_non_mipmap_mmin_ignores_mxl():
    """MMIN 0/1 never read levels > 0 (MXL only counts with a mipmap mode)."""
    for mmin in (0, 1):
        tex1 = g.tex1_reg(lcm=1, mxl=3, mmin=mmin, k=32)
        assert pixel(chain_stream(tex1=tex1)) == COLORS[0]


def test_mxl_past_the_chain_reads_last_level():
    """A 64x64 texture has 7 levels; MXL = 7 clamps the sampled level to 6 (the
    reference's sampler clamps to the image's last level)."""
    tex1 = g.tex1_reg(lcm=1, mxl=7, mmin=2, k=7 * 16)
    assert pixel(chain_stream(tex1=tex1, mxl_levels=7)) == COLORS[6 % 4]


def test_mtba_generates_level_bases():
    """TEX1.MTBA: levels 1-3 follow level 0 block by block with halving widths
    (gs/gs_interface.cpp:805-843) -- the same image as explicit MIPTBP1 bases."""
    for k in (16, 32, 48):
        tex1 = g.tex1_reg(lcm=1, mxl=3, mmin=2, mtba=1, k=k)
        assert pixel(chain_stream(auto=True, tex1=tex1)) == COLORS[k // 16]


def test_descriptor_levels_and_bases():
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    gs.gif_transfer(0, chain_stream(tex1=g.tex1_reg(lcm=1, mxl=2, mmin=3, k=16)))
    gs.flush()
    rp = be.passes[-1]
    assert rp["has_mipmap"] == 1
    (t,) = rp["textures"]
    assert t["levels"] == 3
    assert t["mip"][:2] == [(12 * 32) | (1 << 16), (14 * 32) | (1 << 16)]
    assert t["mip"][2:] == [0, 0, 0, 0]
    tex = rp["prims"][0]["tex"]
    assert (tex >> 21) & 7 == 2 and tex & (1 << 18)
    gs.close()

    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    gs.gif_transfer(0, chain_stream(tex1=g.tex1_reg(lcm=1, mxl=2, mmin=1, k=16)))
    gs.flush()
    rp = be.passes[-1]
    assert rp["has_mipmap"] == 0 and rp["textures"][0]["levels"] == 1
    gs.close()


def test_write_to_mip_level_pages_ends_the_pass():
    """A framebuffer write to pages of level 2 followed by a draw sampling the
    chain splits the pass before that draw: texture hazards cover every
    level's pages (texture_page_rects_read_full, gs/gs_interface.cpp:1201-1206).
    The write itself does not end the pass (the chain was read before it).
    The reference frontend gives the same passes where it is built."""
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    data = chain_stream(tex1=g.tex1_reg(lcm=1, mxl=3, mmin=2, k=32))
    s = g.GifStream()
    # Render into the pages of level 2 (page 14), then sample the chain again.
    s.ad([(g.FRAME_1, g.frame_reg(14, 1, g.PSMCT32)), (g.PRIM, g.prim_reg(g.PRIM_SPRITE))])
    verts = np.zeros((2, 2, 2), dtype=np.uint64)
    verts[:, 0] = g.q_rgbaq(np.full((2, 4), 7, dtype=np.int64))
    verts[:, 1] = g.q_xyz2(np.array([0, 64]), np.array([0, 64]), np.array([0, 0]))
    s.packed(g.prim_reg(g.PRIM_SPRITE), [g.D_RGBAQ, g.D_XYZ2], verts.reshape(-1, 2))
    again = chain_stream(tex1=g.tex1_reg(lcm=1, mxl=3, mmin=2, k=32), upload=False)
    gs.gif_transfer(0, data)
    gs.flush()
    first = len(be.passes)
    gs.gif_transfer(0, again + s.tobytes() + again)
    gs.flush()
    # Sampling the chain after the write to its level-2 pages ends the pass.
    assert [p["num_primitives"] for p in be.passes[first:]] == [2, 1]
    assert be.passes[first]["flush_reason"] == 2
    # Without a mip chain the same write does not touch the sampled pages.
    be2 = RecordingBackend()
    gs2 = pgs.GSInterface(be2)
    flat = chain_stream(tex1=g.tex1_reg(lcm=1, mxl=3, mmin=1, k=32), upload=False)
    gs2.gif_transfer(0, data)
    gs2.flush()
    first = len(be2.passes)
    gs2.gif_transfer(0, flat + s.tobytes() + flat)
    gs2.flush()
    assert len(be2.passes) - first == 1
    gs.close()
    gs2.close()
    import pgs_ref_frontend
    if pgs_ref_frontend.available():
        for stream, counts in ((again, [2, 1]), (flat, [3])):
            ref = pgs_ref_frontend.RefFrontend()
            ref.gif_transfer(0, data)
            ref.flush()
            ref.clear()
            ref.gif_transfer(0, stream + s.tobytes() + stream)
            ref.flush()
            assert [e["num_primitives"] for e in ref.events() if e["type"] == "pass"] == counts
            ref.close()
