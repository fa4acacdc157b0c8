"""Bit-exact parity of the CUDA backend against the CPU oracle.

Both backends sit under the same product frontend and receive the same seeded
GIF command stream; every VRAM plane (GS memory, super-sample reference flags
and the sample planes) must match byte for byte."""
import numpy as np
import pytest

import gsgen
import pgs
import pgs_oracle

pytestmark = pytest.mark.gpu


def run_both(frame):
    obe = pgs_oracle.OracleBackend()
    ref = pgs_oracle.render(frame, obe, planes=True)
    ofrags = obe.fragments()
    obe.close()
    be = pgs.CudaBackend(0, max_samples_log2=4)
    try:
        out = pgs_oracle.render(frame, be, planes=True)
        assert be.error_flags() == 0
        # Covered samples counted by the shading kernels equal the oracle's.
        assert be.fragments() == ofrags
    finally:
        be.close()
    return ref, out


def assert_same(ref, out):
    assert ref.shape == out.shape
    if not np.array_equal(ref, out):
        diff = np.nonzero(ref.reshape(-1) != out.reshape(-1))[0]
        plane = diff // pgs.VRAM_SIZE
        off = diff % pgs.VRAM_SIZE
        raise AssertionError("%d bytes differ; first at plane %d offset 0x%x (oracle %d, cuda %d)" % (
            diff.size, plane[0], off[0], ref.reshape(-1)[diff[0]], out.reshape(-1)[diff[0]]))


@pytest.mark.parametrize("n", [1, 50, 2000])
def test_c1_gouraud_zbuffer(n):
    ref, out = run_both(gsgen.frame_c1(seed=11, num_triangles=n))
    assert_same(ref, out)


@pytest.mark.parametrize("ss", [1, 4])
def test_c2_textured_blended_small(ss):
    f = gsgen.frame_c2(seed=5, num_triangles=400, num_sprites=40, super_sampling=ss, num_textures=2)
    ref, out = run_both(f)
    assert_same(ref, out)


def test_c1_full_size():
    """Plain method at its benchmark size: 10k triangles, 640x448, 1x."""
    ref, out = run_both(gsgen.frame_c1(seed=1))
    assert_same(ref, out)


def test_c2_full_size():
    """Textured and blended at its benchmark size: 50k triangles + 2k sprites, 4x SSAA."""
    ref, out = run_both(gsgen.frame_c2(seed=2))
    assert_same(ref, out)


def test_record_replay_reproduces_frame():
    """A recorded frame program replayed (plain and as a CUDA graph) from its
    starting VRAM reproduces the recorded result on every plane."""
    f = gsgen.frame_c2(seed=9, num_triangles=3000, num_sprites=100, super_sampling=4, num_textures=3)
    be = pgs.CudaBackend(0, max_samples_log2=4)
    try:
        gs = pgs.GSInterface(be, super_sampling=4)
        be.begin_record()
        gs.gif_transfer(0, f.data)
        gs.flush()
        be.end_record()
        first = np.stack([be.read_plane(p) for p in range(6)])
        be.replay(1, reset_vram=True, use_graph=False)
        again = np.stack([be.read_plane(p) for p in range(6)])
        be.replay(3, reset_vram=True, use_graph=True)
        graph = np.stack([be.read_plane(p) for p in range(6)])
        gs.close()
    finally:
        be.close()
    assert np.array_equal(first, again)
    assert np.array_equal(first, graph)


REPLAY_STREAMS = {
    "c2_8_textures": lambda: gsgen.frame_c2(seed=4, num_triangles=2000, num_sprites=100, num_textures=8),
    "c3_psmt4": lambda: gsgen.stream_c3(3, num_primitives=3000),
    "c3_ct16": lambda: gsgen.stream_c3(6, num_primitives=3000),
    "hazards": lambda: gsgen.frame_hazards(2),
    "fuzz": lambda: gsgen.frame_fuzz(5),
}


@pytest.mark.parametrize("name", sorted(REPLAY_STREAMS))
def test_replay_batches_uploads_and_clut_loads(name):
    """Replays launch consecutive host->local uploads with disjoint pages, and
    chains of CLUT loads, as one kernel each; every plane must still equal the
    recorded run, which executed them one at a time."""
    f = REPLAY_STREAMS[name]()
    be = pgs.CudaBackend(0, max_samples_log2=4)
    try:
        gs = pgs.GSInterface(be, super_sampling=f.super_sampling, ordered=f.ordered)
        be.begin_record()
        gs.gif_transfer(0, f.data)
        gs.flush()
        be.end_record()
        planes = 2 + f.super_sampling if f.super_sampling > 1 else 1
        first = np.stack([be.read_plane(p) for p in range(planes)])
        be.replay(1, reset_vram=True, use_graph=False)
        again = np.stack([be.read_plane(p) for p in range(planes)])
        be.replay(2, reset_vram=True, use_graph=True)
        graph = np.stack([be.read_plane(p) for p in range(planes)])
        gs.close()
    finally:
        be.close()
    assert np.array_equal(first, again)
    assert np.array_equal(first, graph)


@pytest.mark.parametrize("ss,ordered", [(2, True), (4, False), (8, False), (16, True), (16, False)])
def test_c2_small_sampling_rates(ss, ordered):
    """Every sampling grid the frontend offers: 2x, 4x sparse, 8x (2x4), 16x ordered and sparse."""
    f = gsgen.frame_c2(seed=7, num_triangles=400, num_sprites=40, super_sampling=ss, num_textures=2)
    f.ordered = ordered
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("zpsm", [gsgen.PSMZ16, gsgen.PSMZ24, gsgen.PSMZ32])
def test_flat_ui_single_sample_heuristic(zpsm):
    """Flat UI triangles and lines next to a 3D mesh at 4x: the single-sample
    heuristic's demotions must match the oracle's."""
    ref, out = run_both(gsgen.frame_flat_ui(zpsm=zpsm))
    assert_same(ref, out)


@pytest.mark.parametrize("ss", [8, 16])
def test_flat_ui_high_rates(ss):
    ref, out = run_both(gsgen.frame_flat_ui(seed=6, super_sampling=ss))
    assert_same(ref, out)


@pytest.mark.parametrize("ss", [8, 16])
def test_c4_feedback_small(ss):
    """Render-to-texture feedback across 10 passes with texture-hazard flushes."""
    ref, out = run_both(gsgen.frame_c4(seed=12, super_sampling=ss, num_triangles=8000))
    assert_same(ref, out)


@pytest.mark.parametrize("ss", [8, 16])
def test_c4_full_size(ss):
    """8x / 16x at its benchmark size: 100k triangles over 10 feedback passes."""
    ref, out = run_both(gsgen.frame_c4(seed=4, super_sampling=ss))
    assert_same(ref, out)


def test_pipelined_async_readback():
    """Frames decoded back to back with asynchronous readbacks in flight: each
    ticket's buffer holds the VRAM as of its own frame (pinned and pageable
    destinations)."""
    import torch
    frames = [gsgen.frame_c1(seed=30 + k, num_triangles=1500) for k in range(4)]
    obe = pgs_oracle.OracleBackend()
    ogs = pgs.GSInterface(obe)
    expect = []
    for f in frames:
        ogs.gif_transfer(0, f.data)
        expect.append(ogs.read_vram())
    ogs.close()
    obe.close()
    be = pgs.CudaBackend(0, max_samples_log2=4)
    try:
        gs = pgs.GSInterface(be)
        pinned = [torch.empty(pgs.VRAM_SIZE, dtype=torch.uint8, pin_memory=True).numpy() for _ in range(2)]
        pageable = [np.empty(pgs.VRAM_SIZE, dtype=np.uint8) for _ in range(2)]
        outs, tickets = [], []
        for k, f in enumerate(frames):
            gs.gif_transfer(0, f.data)
            buf = pinned[k % 2] if k < 2 else pageable[k % 2]
            tickets.append(gs.read_vram_async(buf))
            outs.append(buf)
        for k in range(len(frames)):
            gs.wait(tickets[k])
            assert np.array_equal(outs[k], expect[k]), "frame %d" % k
        gs.close()
    finally:
        be.close()


def scanout_both(frame, setup, calls):
    outs = []
    for be in (pgs_oracle.OracleBackend(), pgs.CudaBackend(0, max_samples_log2=4)):
        try:
            gs = pgs.GSInterface(be, super_sampling=frame.super_sampling, ordered=frame.ordered)
            gs.gif_transfer(0, frame.data)
            for reg, value in setup:
                gs.write_priv_register(reg, value)
            outs.append([gs.scanout_circuit(*c) for c in calls])
            gs.close()
        finally:
            be.close()
    return outs


@pytest.mark.parametrize("ss,ordered", [(1, True), (4, True), (8, True), (16, True), (16, False)])
def test_scanout_circuit_parity(ss, ordered):
    """CRTC read-out: progressive, high-resolution (2x2 sample resolve) and
    interlaced field reads agree with the oracle byte for byte."""
    f = gsgen.frame_c2(seed=13, num_triangles=600, num_sprites=60, super_sampling=ss, num_textures=2)
    f.ordered = ordered
    prog = pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE
    hires = prog | pgs.GSInterface.SCANOUT_HIGH_RESOLUTION
    setup = [("DISPFB1", gsgen.dispfb_reg(0, 10, gsgen.PSMCT32)),
             ("DISPLAY1", gsgen.display_reg(636, 50, 3, 0, 2559, 447)),
             ("DISPFB2", gsgen.dispfb_reg(0, 10, gsgen.PSMCT24, dbx=3, dby=1)),
             ("DISPLAY2", gsgen.display_reg(636, 51, 3, 0, 2559, 446)),
             ("SMODE2", gsgen.smode2_reg(1, 0))]
    calls = [(0, 0, prog), (0, 0, hires), (1, 1, hires), (0, 0, 0), (1, 1, 0)]
    ref, out = scanout_both(f, setup, calls)
    for r, o in zip(ref, out):
        assert r.shape == o.shape
        assert np.array_equal(r, o)


@pytest.mark.parametrize("seed", range(40))
def test_feature_fuzz(seed):
    """Random state coverage (every primitive type, AA1, fog, blend / alpha /
    depth / destination-alpha modes, masks, scissor, all colour and depth
    formats, every texture format and wrap mode, random sampling rate)."""
    f = gsgen.frame_fuzz(seed)
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(16))
def test_mipmap_parity(seed):
    """Mip chains (MIPTBP1/2 and MTBA bases), every MMIN mode, LOD from Q with L
    and signed K, fixed LOD, trilinear, wrap modes, random sampling rate."""
    f = gsgen.frame_mip(seed)
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(12))
def test_aliased_frame_depth_parity(seed):
    """Frame and depth buffer at one base: per-primitive steps while depth is
    written, snapshot depth for the depth-tested runs after it."""
    f = gsgen.frame_alias(seed)
    ref, out = run_both(f)
    assert_same(ref, out)


def _extremes_frame(kind):
    """Edge cases: the whole 4 MiB as one 1024x1024 CT32 frame (no depth) with
    screen-filling and degenerate primitives; a 2048-wide CT16 frame with
    primitives beyond the 12.4 range edges; an empty draw list."""
    s = gsgen.GifStream()
    rng = np.random.default_rng(77)
    if kind == "full_vram":
        w, h = 1024, 1024
        gsgen._frame_setup(s, 0, 16, gsgen.PSMCT32, 0, gsgen.PSMZ24, w, h, gsgen.test_reg(zte=1, ztst=1))
        s.ad([(gsgen.ZBUF_1, gsgen.zbuf_reg(0, gsgen.PSMZ24, 1))])
        pts = [(0, 0), (w * 16, 0), (0, h * 16), (w * 16, h * 16), (0, h * 16), (w * 16, 0),
               (100, 100), (100, 100), (100, 100),            # zero area
               (0, 0), (w * 16, h * 16 // 2), (w * 16, h * 16 // 2 + 1)]  # sliver
    elif kind == "wide_ct16":
        w, h = 2048, 1024
        gsgen._frame_setup(s, 0, 32, gsgen.PSMCT16, 0, gsgen.PSMZ16, w, h, gsgen.test_reg(zte=1, ztst=1))
        s.ad([(gsgen.ZBUF_1, gsgen.zbuf_reg(0, gsgen.PSMZ16, 1))])
        pts = [(0, 0), (0xFFFF, 0), (0, 0xFFFF), (40000, 100), (65535, 65535), (100, 40000)]
    else:
        w, h = 64, 64
        gsgen._frame_setup(s, 0, 1, gsgen.PSMCT32, 10, gsgen.PSMZ24, w, h, gsgen.test_reg(zte=1, ztst=1))
        return gsgen.Frame("empty", s.tobytes(), 4, True, 0, {"width": w, "height": h, "fbp": 0, "zbp": 10})
    n = len(pts)
    q = np.zeros((n, 2, 2), dtype=np.uint64)
    q[:, 0] = gsgen.q_rgbaq(rng.integers(0, 256, (n, 4)))
    q[:, 1] = gsgen.q_xyz2(np.array([p[0] for p in pts]), np.array([p[1] for p in pts]), np.zeros(n, dtype=np.int64))
    s.packed(gsgen.prim_reg(gsgen.PRIM_TRI, iip=1), [gsgen.D_RGBAQ, gsgen.D_XYZ2], q.reshape(-1, 2))
    return gsgen.Frame(kind, s.tobytes(), 1, True, n // 3, {"width": w, "height": h, "fbp": 0, "zbp": 0})


@pytest.mark.parametrize("kind,ss", [("full_vram", 1), ("full_vram", 16), ("wide_ct16", 1), ("wide_ct16", 4),
                                     ("empty", 4)])
def test_extreme_sizes(kind, ss):
    f = _extremes_frame(kind)
    f = gsgen.Frame(f.name, f.data, ss, True, f.num_primitives, f.meta)
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(12))
def test_super_sampled_textures_parity(seed):
    """Sprites sampling pages a super-sampled pass wrote, with super-sampled
    textures on: sample mapping, resolved and single-sampled layers, phase-LUT
    filtering, blur detection, at 2x / 4x / 8x / 16x."""
    f = gsgen.frame_ssaa_textures(seed)
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(6))
def test_combined_feature_streams(seed):
    """One stream that runs a mipmapped frame, a super-sampled-texture frame, an
    aliased frame/depth frame and a feature-fuzz frame back to back at one
    sampling rate (state, textures and pages carried from one to the next)."""
    parts = [gsgen.frame_ssaa_textures(seed), gsgen.frame_mip(seed), gsgen.frame_alias(seed), gsgen.frame_fuzz(seed)]
    f = gsgen.Frame("combined_%d" % seed, b"".join(p.data for p in parts), parts[0].super_sampling, parts[0].ordered,
                    sum(p.num_primitives for p in parts), dict(parts[0].meta))
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(12))
def test_field_aware_rendering_parity(seed):
    """Frames drawn after a high-resolution vsync of field-rendered output:
    forced super-sampled tiles, rows snapped at half the sample pitch,
    FORCE_LINEAR_SUPER_SAMPLE blur kernels, and 448-row frames that stay as
    they were."""
    ref, out = run_both(gsgen.frame_field_aware(seed))
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(8))
def test_blend_demote_parity(seed):
    """allow_blend_demote: crowded blended tiles without depth writes shade
    single-sampled (per-tile primitive counts from binning)."""
    ref, out = run_both(gsgen.frame_blend_demote(seed))
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(4))
def test_disable_mipmaps_parity(seed):
    f = gsgen.frame_mip(seed)
    f.meta["hacks"] = {"disable_mipmaps": True}
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(8))
def test_fused_rectangles_parity(seed):
    """Triangle pairs fused into parallelograms (provoking vertex 0 and 2),
    flat, FST and STQ textured, lists and strips, 1x and super-sampled, with
    pairs the fusion must leave apart."""
    ref, out = run_both(gsgen.frame_quads(seed))
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(4))
def test_combined_stream_with_fusion_and_hacks(seed):
    """Fused rectangles, a mipmapped frame, the super-sampled-texture frame and
    the blend-demotion frame in one stream at one rate, with blend demotion on
    and field-aware rendering chosen by a vsync first."""
    parts = [gsgen.frame_ssaa_textures(seed), gsgen.frame_quads(seed), gsgen.frame_mip(seed),
             gsgen.frame_blend_demote(seed)]
    meta = dict(parts[0].meta)
    meta["field_aware"] = seed % 2 == 0
    meta["hacks"] = {"allow_blend_demote": True}
    f = gsgen.Frame("combined2_%d" % seed, b"".join(p.data for p in parts), parts[0].super_sampling,
                    parts[0].ordered, 0, meta)
    ref, out = run_both(f)
    assert_same(ref, out)


@pytest.mark.parametrize("seed", range(16))
def test_hazard_stream_parity(seed):
    """Hazard-heavy streams: uploads into textures the open pass samples (VRAM
    snapshots the textures decode from), copies out of framebuffers, CLUT
    reloads and memoised palettes, TEXFLUSH, render to texture and feedback,
    at 1x and 4x.  The same streams match the reference frontend record for
    record (test_frontend_reference.py)."""
    ref, out = run_both(gsgen.frame_hazards(seed))
    assert_same(ref, out)


def test_snapshot_textures_read_the_data_before_the_upload():
    """A texture sampled before an upload overwrites it, in the same pass,
    reads the old texels from a VRAM snapshot; CUDA and the oracle agree
    (test_snapshot.py checks the oracle against an explicit flush)."""
    import snapshot_streams
    ref, out = run_both(snapshot_streams.sample_then_upload())
    assert_same(ref, out)
