"""Host logic of the frontend (GSInterface re-host), checked against the rules in
gs/gs_interface.cpp with a backend that only records what it is sent."""
import struct

import numpy as np
import pytest

import gsgen as g
import pgs
from recording_backend import RecordingBackend

Z_TEST, Z_WRITE, OPAQUE, PARALLELOGRAM, MULTISAMPLE = 12, 13, 14, 15, 16
Z_GREATER, PERSPECTIVE, IIP, FIX, SPRITE, LINE = 17, 18, 19, 20, 21, 22
SNAP_RASTER, SNAP_ATTRIBUTE = 25, 26
# pgs_flush_reason (the reference's FlushReason numbering).
FLUSH_FB_POINTER, FLUSH_OVERFLOW, FLUSH_TEXTURE_HAZARD, FLUSH_COPY_HAZARD, FLUSH_SUBMISSION = 0, 1, 2, 3, 4
FLUSH_PRESSURE, FLUSH_HOST_ACCESS = 5, 6


def bit(v, b):
    return (v >> b) & 1


def make(ss=1):
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=ss)
    return be, gs


def setup(s, test=None, extra=()):
    s.ad([(g.PRMODECONT, 1), (g.FRAME_1, g.frame_reg(0, 10, g.PSMCT32)), (g.ZBUF_1, g.zbuf_reg(140, g.PSMZ24)),
          (g.SCISSOR_1, g.scissor_reg(0, 639, 0, 447)), (g.XYOFFSET_1, 0),
          (g.TEST_1, test if test is not None else g.test_reg(zte=1, ztst=2)), *extra])


def verts(s, prim, pts, z=1000, rgba=(10, 20, 30, 40)):
    n = len(pts)
    x = np.array([p[0] for p in pts], dtype=np.int64)
    y = np.array([p[1] for p in pts], dtype=np.int64)
    zz = np.full(n, z, dtype=np.int64)
    col = np.tile(np.array(rgba, dtype=np.int64), (n, 1))
    q = np.zeros((n, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(col)
    q[:, 1] = g.q_xyz2(x, y, zz)
    lo, hi = g.gif_tag(n, 0, 2, g.D_RGBAQ | (g.D_XYZ2 << 4), pre=1, prim=prim)
    s._qwords(np.array([[lo, hi]], dtype=np.uint64))
    s._qwords(q.reshape(-1, 2))


def run(ss=1, build=None):
    be, gs = make(ss)
    s = g.GifStream()
    build(s)
    gs.gif_transfer(0, s.tobytes())
    gs.flush()
    gs.close()
    return be


def test_triangle_record_positions_bbox_and_state():
    pts = [(100 * 16 + 3, 50 * 16 + 8), (140 * 16, 52 * 16 + 15), (120 * 16 + 1, 90 * 16 + 2)]
    be = run(build=lambda s: (setup(s), verts(s, g.prim_reg(g.PRIM_TRI, iip=1), pts)))
    assert len(be.passes) == 1
    rp = be.passes[0]
    assert rp["num_primitives"] == 1
    # pos[i] = vertex_queue[2 - i] (gs/gs_interface.cpp:2503-2510): newest vertex first.
    assert [p[:2] for p in rp["positions"]] == list(reversed(pts))
    xs, ys = [p[0] for p in pts], [p[1] for p in pts]
    lo = ((min(xs) + 15) >> 4, (min(ys) + 15) >> 4)
    hi = ((max(xs) - 1) >> 4, (max(ys) - 1) >> 4)
    assert rp["prims"][0]["bb"] == [lo[0], lo[1], hi[0], hi[1]]
    st = rp["prims"][0]["state"]
    assert bit(st, Z_TEST) and bit(st, Z_WRITE) and bit(st, OPAQUE) and bit(st, IIP) and bit(st, PERSPECTIVE)
    assert not bit(st, Z_GREATER) and not bit(st, SPRITE)
    inst = rp["instances"][0]
    assert inst["z_sensitive"] and inst["z_write"]
    assert (inst["base_x"], inst["base_y"]) == lo


def test_strip_and_fan_vertex_queue():
    p = [(i * 160 + 100, (i % 2) * 400 + 100) for i in range(6)]
    be = run(build=lambda s: (setup(s), verts(s, g.prim_reg(g.PRIM_TRISTRIP), p), verts(s, g.prim_reg(g.PRIM_TRIFAN), p)))
    prims = be.passes[0]["positions"]
    assert be.passes[0]["num_primitives"] == 8
    strip = [tuple(q[:2] for q in prims[3 * i:3 * i + 3]) for i in range(4)]
    assert strip[0] == (p[2], p[1], p[0]) and strip[3] == (p[5], p[4], p[3])
    fan = [tuple(q[:2] for q in prims[3 * i:3 * i + 3]) for i in range(4, 8)]
    # Fans keep vertex 0 in the queue's first slot.
    assert all(f[2] == p[0] for f in fan)
    assert fan[0][:2] == (p[2], p[1]) and fan[3][:2] == (p[5], p[4])


def test_sprite_state_bits():
    be = run(build=lambda s: (setup(s), verts(s, g.prim_reg(g.PRIM_SPRITE), [(160, 160), (800, 640)])))
    st = be.passes[0]["prims"][0]["state"]
    for b in (PARALLELOGRAM, SPRITE, SNAP_RASTER, SNAP_ATTRIBUTE):
        assert bit(st, b)
    assert not bit(st, MULTISAMPLE)


def test_scissor_and_never_tests_cull():
    def build(s):
        setup(s)
        s.ad([(g.SCISSOR_1, g.scissor_reg(0, 63, 0, 63))])
        verts(s, g.prim_reg(g.PRIM_TRI), [(2000, 2000), (3000, 2000), (2500, 2500)])
        s.ad([(g.SCISSOR_1, g.scissor_reg(0, 639, 0, 447)), (g.TEST_1, g.test_reg(zte=1, ztst=0))])
        verts(s, g.prim_reg(g.PRIM_TRI), [(200, 200), (300, 200), (250, 250)])
        s.ad([(g.TEST_1, g.test_reg(ate=1, atst=0, afail=0, zte=1, ztst=1))])
        verts(s, g.prim_reg(g.PRIM_TRI), [(200, 200), (300, 200), (250, 250)])
    be = run(build=build)
    assert be.passes == []


def test_xyoffset_is_subtracted():
    def build(s):
        setup(s, extra=[(g.XYOFFSET_1, 2048 * 16 | ((2048 * 16) << 32))])
        verts(s, g.prim_reg(g.PRIM_TRI), [(2048 * 16 + 160, 2048 * 16 + 160), (2048 * 16 + 480, 2048 * 16 + 160),
                                          (2048 * 16 + 320, 2048 * 16 + 480)])
    be = run(build=build)
    assert [p[:2] for p in be.passes[0]["positions"]] == [(320, 480), (480, 160), (160, 160)]


def test_reglist_packet():
    def build(s):
        setup(s)
        s.ad([(g.PRIM, g.prim_reg(g.PRIM_TRI))])
        regs = [(g.RGBAQ, 0x11223344), (g.XYZ2, 160 | (160 << 16)), (g.XYZ2, 480 | (160 << 16)), (g.XYZ2, 320 | (480 << 16))]
        desc = g.D_RGBAQ | (g.D_XYZ2 << 4) | (g.D_XYZ2 << 8) | (g.D_XYZ2 << 12)
        lo, hi = g.gif_tag(1, 1, 4, desc)
        s._qwords(np.array([[lo, hi], [regs[0][1], regs[1][1]], [regs[2][1], regs[3][1]]], dtype=np.uint64))
    be = run(build=build)
    rp = be.passes[0]
    assert rp["num_primitives"] == 1
    assert rp["attributes"][0]["rgba"] == 0x11223344


def test_frame_pointer_changes_use_instances_then_flush():
    def build(s):
        setup(s)
        for i in range(10):
            s.ad([(g.FRAME_1, g.frame_reg(i * 8, 2, g.PSMCT32))])
            verts(s, g.prim_reg(g.PRIM_TRI), [(160, 160), (480, 160), (320, 480)])
    be = run(build=build)
    # Up to 8 framebuffer instances per pass (MaxRenderPassInstances), then an FBPointer flush.
    assert [p["num_primitives"] for p in be.passes] == [8, 2]
    assert len(be.passes[0]["instances"]) == 8
    insts = [(p["state"] >> 29) & 7 for p in be.passes[0]["prims"]]
    assert insts == list(range(8))


def test_overflow_flush_at_64k_primitives():
    n = 64 * 1024 + 10
    def build(s):
        setup(s)
        nv = 3 * n
        x = np.tile(np.array([160, 480, 320], dtype=np.int64), n)
        y = np.tile(np.array([160, 160, 480], dtype=np.int64), n)
        q = np.zeros((nv, 2, 2), dtype=np.uint64)
        q[:, 0] = g.q_rgbaq(np.full((nv, 4), 9, dtype=np.int64))
        q[:, 1] = g.q_xyz2(x, y, np.full(nv, 5, dtype=np.int64))
        s.packed(g.prim_reg(g.PRIM_TRI), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
    be = run(build=build)
    assert [p["num_primitives"] for p in be.passes] == [64 * 1024, 10]


def test_state_vector_dedup_and_blend_bits():
    def build(s):
        setup(s, extra=[(g.ALPHA_1, g.alpha_reg(0, 1, 0, 1, fix=0x40))])
        verts(s, g.prim_reg(g.PRIM_TRI, abe=1), [(160, 160), (480, 160), (320, 480)])
        verts(s, g.prim_reg(g.PRIM_TRI, abe=1), [(160, 160), (480, 160), (320, 480)])
        verts(s, g.prim_reg(g.PRIM_TRI), [(160, 160), (480, 160), (320, 480)])
    be = run(build=build)
    rp = be.passes[0]
    assert len(rp["states"]) == 2
    s0 = rp["states"][0]["blend_mode"]
    assert s0 & (1 << 9)  # ABE
    assert (s0 >> 11) & 3 == 0 and (s0 >> 13) & 3 == 1 and (s0 >> 15) & 3 == 0 and (s0 >> 17) & 3 == 1
    # Blending with Cd terms is not opaque; the unblended primitive is.
    assert not bit(rp["prims"][0]["state"], OPAQUE) and bit(rp["prims"][2]["state"], OPAQUE)
    assert (rp["prims"][0]["alpha"] >> 8) & 0xFF == 0x40


def test_clut_load_modes():
    """CLD decides which TEX0 writes load the CLUT (handle_clut_upload,
    gs/gs_interface.cpp:563-589).  Loads from distinct sources all reach the
    backend; none is read by a draw in between, so each replaces the last in
    its ring slot, starting from the same palette (update_palette_cache,
    gs/gs_renderer.cpp:3400-3419).  An identical load is reused instead
    (palette memoisation).  The reference frontend makes the same loads."""
    def build(s):
        setup(s)
        def tex0(cbp, cld):
            return g.tex0_reg(0x2000, 4, g.PSMT8, 8, 8, cbp=cbp, cpsm=g.PSMCT32) | (cld << 61)
        s.ad([(g.TEX0_1, tex0(0x3000, 1))])   # CLD=1: load
        s.ad([(g.TEX0_1, tex0(0x3000, 0))])   # CLD=0: no load
        s.ad([(g.TEX0_1, tex0(0x3020, 2))])   # CLD=2: load, CBP0 := CBP
        s.ad([(g.TEX0_1, tex0(0x3020, 4))])   # CLD=4: CBP0 equal -> no load
        s.ad([(g.TEX0_1, tex0(0x3010, 4))])   # CBP differs -> load
        s.ad([(g.TEX0_1, tex0(0x3010, 1))])   # identical to the last load -> reused
    be = run(build=build)
    cbps = [(p["tex0"] >> 37) & 0x3fff for p in be.palettes]
    assert cbps == [0x3000, 0x3020, 0x3010]
    assert [p["instance"] for p in be.palettes] == [1, 1, 1]
    assert [p["base_instance"] for p in be.palettes] == [0, 0, 0]
    import pgs_ref_frontend
    if pgs_ref_frontend.available():
        s = g.GifStream()
        build(s)
        ref = pgs_ref_frontend.RefFrontend()
        ref.gif_transfer(0, s.tobytes())
        ref.flush()
        loads = [e for e in ref.events() if e["type"] == "palette"]
        assert [(e["tex0"] >> 37) & 0x3fff for e in loads] == cbps
        assert [e["instance"] for e in loads] == [1, 1, 1]
        ref.close()


def test_partial_image_transfer_and_texture_read_flush():
    be, gs = make()
    s = g.GifStream()
    setup(s)
    data = bytes(range(256)) * 64  # 128x128 PSMT8 = 16 KiB
    s.ad([(g.BITBLTBUF, g.bitbltbuf_reg(dbp=0x2000, dbw=2, dpsm=g.PSMT8)), (g.TRXPOS, 0),
          (g.TRXREG, g.trxreg_reg(128, 128)), (g.TRXDIR, 0)])
    tag_lo, tag_hi = g.gif_tag(len(data) // 16, 2, 0)
    head = np.array([[tag_lo, tag_hi]], dtype=np.uint64).tobytes()
    gs.gif_transfer(0, s.tobytes() + head + data[:4096])
    assert be.copies == []  # waiting for the rest of the image
    # A textured draw flushes the partial transfer before it reads VRAM.
    t = g.GifStream()
    t.ad([(g.TEX0_1, g.tex0_reg(0x2000, 2, g.PSMT8, 7, 7, cbp=0x3000, cld=1))])
    verts(t, g.prim_reg(g.PRIM_SPRITE, tme=1, fst=1), [(0, 0), (1600, 1600)])
    # The rest of the IMAGE packet still belongs to the open GIF path; send the draw on path 1.
    gs.gif_transfer(1, t.tobytes())
    assert len(be.copies) == 1 and be.copies[0]["offset"] == 0 and len(be.copies[0]["data"]) == 4096
    gs.gif_transfer(0, data[4096:])
    gs.flush()
    gs.close()
    assert len(be.copies) == 2 and be.copies[1]["offset"] == 4096 and len(be.copies[1]["data"]) == len(data)


def _uv_sprite(s, prim, xy0, xy1, uv0, uv1):
    """A sprite with explicit UVs (FST = 1), in 1/16 pixel / texel units."""
    q = np.zeros((2, 3, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(np.array([[10, 20, 30, 40]] * 2))
    for i, (xy, uv) in enumerate(((xy0, uv0), (xy1, uv1))):
        q[i, 1, 0] = uv[0] | (uv[1] << 16)
        q[i, 1, 1] = g.D_UV
        q[i, 2] = g.q_xyz2(np.array([xy[0]]), np.array([xy[1]]), np.array([1000]))[0]
    lo, hi = g.gif_tag(2, 0, 3, g.D_RGBAQ | (0xE << 4) | (g.D_XYZ2 << 8), pre=1, prim=prim)
    s._qwords(np.array([[lo, hi]], dtype=np.uint64))
    s._qwords(q.reshape(-1, 2))


@pytest.mark.parametrize("uv_origin,counts", [(10, [1, 1]), (40, [2])])
def test_texture_read_after_framebuffer_write(uv_origin, counts):
    """A sprite sampling its own framebuffer (TBP0 = FBP * 32) in sliced
    feedback: the reference narrows the texture to the sprite's UV box
    (drawing_kick_update_texture, gs/gs_interface.cpp:1478-1509), so the pass
    ends only when that box covers blocks an earlier primitive wrote
    (mark_texture_read, gs/page_tracker.cpp:327-345).  The triangle covers
    pixels 10..29; UVs from texel 10 overlap it, from texel 40 they do not."""
    def build(s):
        setup(s)
        verts(s, g.prim_reg(g.PRIM_TRI), [(160, 160), (480, 160), (320, 480)])
        s.ad([(g.TEX0_1, g.tex0_reg(0, 10, g.PSMCT32, 6, 6))])
        u = uv_origin * 16
        _uv_sprite(s, g.prim_reg(g.PRIM_SPRITE, tme=1, fst=1), (6400, 6400), (8000, 7000), (u, u), (u + 160, u + 160))
    be = run(build=build)
    assert [p["num_primitives"] for p in be.passes] == counts
    assert be.passes[-1]["flush_reason"] == FLUSH_SUBMISSION
    if len(counts) > 1:
        assert be.passes[0]["flush_reason"] == FLUSH_TEXTURE_HAZARD
    import pgs_ref_frontend
    if pgs_ref_frontend.available():
        s = g.GifStream()
        build(s)
        ref = pgs_ref_frontend.RefFrontend()
        ref.gif_transfer(0, s.tobytes())
        ref.flush()
        assert [e["num_primitives"] for e in ref.events() if e["type"] == "pass"] == counts
        ref.close()


def test_coarse_tile_size_heuristic():
    # binning_cost = tiles8 x prims (gs/gs_interface.cpp:148-169).
    def one(n, ss):
        def build(s):
            setup(s)
            verts(s, g.prim_reg(g.PRIM_TRI), [(0, 0), (639 * 16, 0), (0, 447 * 16)] * n)
        return run(ss, build).passes[0]["coarse_tile_size_log2"]
    assert one(1, 1) == 3          # 80x56 tiles8 x 1 prim = 4480 < 10k
    assert one(3, 1) == 4
    assert one(3000, 1) == 5
    assert one(3000, 4) == 4


def test_super_sampling_rate_sent_to_backend():
    be, gs = make(ss=4)
    gs.set_super_sampling_rate(16, ordered=True)
    gs.set_super_sampling_rate(8)
    gs.close()
    assert be.ss == [(1, 1), (2, 2), (1, 2)]


def test_read_vram_async_falls_back_to_synchronous_copy():
    """Backends without an asynchronous read (ABI 1 tables, the oracle) copy
    before pgs_gs_read_vram_async returns and hand out ticket 0."""
    import gsgen
    import pgs_oracle
    f = gsgen.frame_c1(seed=21, num_triangles=200)
    for be in (pgs_oracle.OracleBackend(), RecordingBackend()):
        gs = pgs.GSInterface(be)
        gs.gif_transfer(0, f.data)
        out = np.zeros(pgs.VRAM_SIZE, dtype=np.uint8)
        ticket = gs.read_vram_async(out)
        assert ticket == 0
        gs.wait(ticket)
        assert np.array_equal(out, gs.read_vram())
        gs.close()
        be.close()


@pytest.mark.parametrize("tex_page,rect", [
    (37, (6, 3, 8, 3)),      # one page row
    (37, (6, 2, 8, 3)),      # two rows
    (37, (6, 1, 8, 5)),      # five rows (general row loop)
    (64, (3, 6, 4, 6)),      # pages 63 and 64: the span crosses a 64-page word
    (63, (0, 6, 3, 7)),      # last page of a word, two rows
])
def test_framebuffer_write_over_sampled_page_keeps_the_pass(tex_page, rect):
    """A draw whose page rectangle (x0, y0, x1, y1 in 64x32 CT32 pages, 10
    pages per row) covers a page sampled earlier in the pass does not end the
    pass: the reference samples a texture-cache image taken before the pass
    renders (gs/page_tracker.cpp:155-190 marks the write without a flush), and
    this backend decodes every texture of a pass before it shades any primitive
    of it.  A new texture over those pages after the write does end the pass
    (mark_texture_read, gs/page_tracker.cpp:327-345); the texture the pass
    already holds would not be checked again until the next TEXFLUSH that
    counts.  The reference frontend gives the same passes where it is built."""
    def build(again):
        def b(s):
            setup(s)
            s.ad([(g.TEX0_1, g.tex0_reg(tex_page * 32, 1, g.PSMCT32, 6, 5))])
            verts(s, g.prim_reg(g.PRIM_SPRITE, tme=1, fst=1), [(0, 0), (16 * 16, 16 * 16)])
            x0, y0, x1, y1 = rect
            verts(s, g.prim_reg(g.PRIM_SPRITE), [(x0 * 64 * 16, y0 * 32 * 16), ((x1 + 1) * 64 * 16 - 16, (y1 + 1) * 32 * 16 - 16)])
            if again:
                s.ad([(g.TEX0_1, g.tex0_reg(tex_page * 32, 1, g.PSMCT32, 6, 4))])
                verts(s, g.prim_reg(g.PRIM_SPRITE, tme=1, fst=1), [(0, 0), (16 * 16, 16 * 16)])
        return b
    be = run(build=build(False))
    assert [p["num_primitives"] for p in be.passes] == [2]
    be = run(build=build(True))
    assert [p["num_primitives"] for p in be.passes] == [2, 1]
    assert be.passes[0]["flush_reason"] == FLUSH_TEXTURE_HAZARD
    import pgs_ref_frontend
    if pgs_ref_frontend.available():
        for again, counts in ((False, [2]), (True, [2, 1])):
            s = g.GifStream()
            build(again)(s)
            ref = pgs_ref_frontend.RefFrontend()
            ref.gif_transfer(0, s.tobytes())
            ref.flush()
            assert [e["num_primitives"] for e in ref.events() if e["type"] == "pass"] == counts
            ref.close()


@pytest.mark.parametrize("maker", ["c2", "c1", "fuzz", "strips"])
def test_records_do_not_depend_on_transfer_chunking(maker):
    """Whole PACKED loops are decoded a tag's worth at a time (with the writes
    spelled out for ST / UV, RGBAQ, XYZ2 and RGBAQ, XYZ2 lists); sent one qword
    per call they take the per-qword path.  Both must give the same records,
    states and passes."""
    if maker == "c2":
        data = g.frame_c2(seed=9, num_triangles=6000, num_sprites=300, super_sampling=1, num_textures=2).data
    elif maker == "c1":
        data = g.frame_c1(seed=4, num_triangles=4000).data
    elif maker == "fuzz":
        data = g.frame_fuzz(5).data
    else:
        # Strips and fans with XYZ3 (no drawing) and XYZF2 kicks, ST/RGBAQ/UV/FOG lists.
        rng = np.random.default_rng(2)
        s = g.GifStream()
        setup(s)
        for prim, desc in ((g.PRIM_TRISTRIP, [g.D_RGBAQ, 0xD, g.D_XYZ2]), (g.PRIM_TRIFAN, [g.D_ST, g.D_RGBAQ, g.D_XYZF2]),
                           (g.PRIM_TRI, [0xA, g.D_UV, g.D_RGBAQ, g.D_XYZ2])):
            n = 3000
            q = np.zeros((n, len(desc), 2), dtype=np.uint64)
            for k, d in enumerate(desc):
                q[:, k, 0] = rng.integers(0, 1 << 63, n, dtype=np.uint64)
                q[:, k, 1] = rng.integers(0, 1 << 63, n, dtype=np.uint64)
                if d in (g.D_XYZ2, 0xD, g.D_XYZF2):
                    q[:, k, 0] = g.q_xyz2(rng.integers(0, 640 * 16, n), rng.integers(0, 448 * 16, n), np.zeros(n))[:, 0]
            s.packed(g.prim_reg(prim, iip=1, tme=int(g.D_ST in desc or g.D_UV in desc), fst=int(g.D_UV in desc),
                                fge=int(0xA in desc or g.D_XYZF2 in desc)), desc, q.reshape(-1, 2))
        data = s.tobytes()
    outs = []
    for chunk in (len(data), 16):
        be, gs = make()
        if chunk == len(data):
            gs.gif_transfer(0, data)
        else:
            for off in range(0, len(data), chunk):
                gs.gif_transfer(0, data[off:off + chunk])
        gs.flush()
        gs.close()
        outs.append(be.passes)
    assert len(outs[0]) == len(outs[1])

    def bits(v):
        # Compare floats by their bits (random ST payloads include NaNs).
        if isinstance(v, float):
            return struct.unpack("<I", struct.pack("<f", v))[0]
        if isinstance(v, dict):
            return {k: bits(x) for k, x in v.items()}
        if isinstance(v, (list, tuple)):
            return [bits(x) for x in v]
        return v
    for a, b in zip(*outs):
        assert bits(a) == bits(b)
