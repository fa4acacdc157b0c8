"""vsync output (GSRenderer::vsync, gs/gs_renderer.cpp:4189-5055) through the
product frontend on the CPU oracle: video-mode table, CRTC rectangles, PMODE
merge (replace / ALP / circuit-1 alpha over circuit 2 or BGCOLOR), EXTWRITE
write-back and the FastMAD deinterlacer.  CUDA parity is in test_gpu_vsync.py."""
import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle

NTSC, PAL, PROG = 2, 3, 0
FP = pgs.GSInterface.VSYNC["FORCE_PROGRESSIVE"]


def _swz(x, y, base, stride, psm):
    return pgs_oracle.load_oracle().pgs_oracle_swizzle(x, y, base, stride, psm)
ADAPT = pgs.GSInterface.VSYNC["ADAPT_HORIZONTAL"]


def make(seed=0, ss=1):
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=ss)
    rng = np.random.default_rng(seed)
    gs.write_vram(rng.integers(0, 256, pgs.VRAM_SIZE, dtype=np.uint8))
    return be, gs


def set_priv(gs, regs):
    for i, v in regs.items():
        gs.write_priv_register(i, v)


def prog_frame_regs(pmode, fbp1=0, fbp2=20, bg=0x123456):
    """480p (progressive analog, clock divider 2): both circuits 640x448 at the
    display origin (DX 318, DY 50), MAGH 2."""
    return {0: pmode, 1: g.smode1_reg(PROG, 32), 2: g.smode2_reg(0, 0), 14: bg,
            7: g.dispfb_reg(fbp1, 10, g.PSMCT32), 8: g.display_reg(318, 50, 1, 0, 1279, 447),
            9: g.dispfb_reg(fbp2, 10, g.PSMCT32), 10: g.display_reg(318, 50, 1, 0, 1279, 447)}


def ntsc_field_regs(pmode, fbp1=0):
    """Interlaced NTSC (field mode): circuit 1 640x448 at DX 636, DY 50, MAGH 4."""
    return {0: pmode, 1: g.smode1_reg(NTSC, 32), 2: g.smode2_reg(1, 0), 14: 0,
            7: g.dispfb_reg(fbp1, 10, g.PSMCT32), 8: g.display_reg(636, 50, 3, 0, 2559, 447)}


@pytest.mark.parametrize("cmod,lc,interlace,flags,want", [
    (NTSC, 32, 1, 0, (640, 224)), (NTSC, 32, 1, FP, (640, 448)), (NTSC, 32, 0, FP, (640, 224)),
    (PAL, 32, 1, FP, (640, 512)), (PAL, 32, 1, 0, (640, 256)), (PROG, 32, 0, FP, (640, 448)),
    (PROG, 15, 0, FP, (640, 480)), (PROG, 22, 0, FP, (1280, 1440)),
    (NTSC, 32, 1, FP | pgs.GSInterface.VSYNC["OVERSCAN"], (712, 480))])
def test_video_mode_table(cmod, lc, interlace, flags, want):
    """Mode sizes of GSRenderer::vsync (:4262-4378): analog NTSC/PAL fields,
    doubled when the output is neither interlaced nor double-strike (field-mode
    interlace forced progressive is not interlaced; 240p NTSC is double-strike),
    VGA, HDTV."""
    be, gs = make()
    set_priv(gs, {0: g.pmode_reg(en1=0), 1: g.smode1_reg(cmod, lc), 2: g.smode2_reg(interlace, 0)})
    img, r = gs.vsync(0, flags)
    assert (r["mode_width"], r["mode_height"]) == want
    gs.close()
    be.close()


def test_unknown_mode_gives_no_image():
    be, gs = make()
    set_priv(gs, {1: g.smode1_reg(1, 3)})
    img, r = gs.vsync(0, FP)
    assert img.size == 0 and r["mode_width"] == 0
    gs.close()
    be.close()


def test_single_circuit_is_copied_one_to_one():
    """EN1 only, MMOD=ALP with ALP=0xff: the merged frame is circuit 1 as it is
    (1:1 viewport at the NTSC display origin)."""
    be, gs = make(1)
    set_priv(gs, prog_frame_regs(g.pmode_reg(en1=1, en2=0, mmod=1, alp=0xFF)))
    circ = gs.scanout_circuit(0, 0, pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)
    img, r = gs.vsync(0, FP)
    assert img.shape == (448, 640, 4) and not r["interlaced"]
    assert np.array_equal(img, circ[:448, :640])
    gs.close()
    be.close()


def blend(s, d, a):
    v = s.astype(np.int64) * a + d.astype(np.int64) * (255 - a)
    q, rem = v // 255, v % 255
    return (q + (2 * rem > 255)).astype(np.uint8)


@pytest.mark.parametrize("mmod,alp", [(1, 0x80), (1, 0x20), (0, 0xFF)])
def test_alpha_merge_over_circuit2(mmod, alp):
    be, gs = make(2)
    set_priv(gs, prog_frame_regs(g.pmode_reg(en1=1, en2=1, mmod=mmod, slbg=0, alp=alp)))
    c1 = gs.scanout_circuit(0, 0, pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)[:448, :640]
    c2 = gs.scanout_circuit(1, 0, pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)[:448, :640]
    img, r = gs.vsync(0, FP)
    a = np.full(c1.shape[:2] + (1,), alp, dtype=np.int64) if mmod == 1 else c1[..., 3:4].astype(np.int64)
    want = blend(c1[..., :3], c2[..., :3], a)
    assert np.array_equal(img[..., :3], want)
    assert np.array_equal(img[..., 3], c1[..., 3])
    gs.close()
    be.close()


def test_background_where_no_circuit_covers():
    """SLBG=1 blends circuit 1 over BGCOLOR (alpha 0) and circuit 2 is not drawn;
    outside circuit 1's rectangle the frame is BGCOLOR."""
    be, gs = make(3)
    regs = prog_frame_regs(g.pmode_reg(en1=1, en2=1, mmod=1, slbg=1, alp=0x40), bg=0x00A0B0C0)
    regs[8] = g.display_reg(318 + 2 * 100, 50 + 20, 1, 0, 2 * 200 - 1, 99)  # 200x100 at (100, 20)
    set_priv(gs, regs)
    img, r = gs.vsync(0, FP)
    c1 = gs.scanout_circuit(0, 0, pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)
    # A circuit smaller than the mode keeps its CRTC position (no re-centring).
    bg = np.array([0xC0, 0xB0, 0xA0], dtype=np.uint8)
    inner = blend(c1[:100, :200, :3], np.broadcast_to(bg, (100, 200, 3)), np.int64(0x40))
    assert np.array_equal(img[20:120, 100:300, :3], inner)
    assert np.all(img[20:120, 100:300, 3] == c1[:100, :200, 3])
    for outside in (img[:20], img[120:], img[:, :100], img[:, 300:]):
        assert np.all(outside[..., :3] == bg) and np.all(outside[..., 3] == 0)
    gs.close()
    be.close()


def test_stretch_is_exact_at_1_to_1_and_bilinear_otherwise():
    """MAGH such that the circuit is half the viewport width: every output pixel
    is an 8-bit-weight lerp of two neighbouring circuit texels."""
    be, gs = make(4)
    regs = prog_frame_regs(g.pmode_reg(en1=1, en2=0, mmod=1, alp=0xFF))
    regs[8] = g.display_reg(318, 50, 3, 0, 1279, 447)  # MAGH 4: 320 texels over 640 columns
    set_priv(gs, regs)
    img, r = gs.vsync(0, FP | ADAPT)
    c1 = gs.scanout_circuit(0, 0, pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)
    assert c1.shape[1] == 320
    # ADAPT_HORIZONTAL maps the viewport to the circuit's own resolution.
    assert r["mode_width"] == 320 and img.shape[1] == 320
    assert np.array_equal(img[:448], c1[:448])
    img, r = gs.vsync(0, FP)
    assert img.shape[1] == 640
    x = np.arange(640)
    fx = ((2 * x + 1) * 320 * 256) // 1280 - 128
    x0 = np.clip(fx >> 8, 0, 319)
    x1 = np.clip((fx >> 8) + 1, 0, 319)
    w = (fx & 255)[None, :, None]
    row = c1[:448].astype(np.int64)
    want = ((256 - w) * 256 * row[:, x0] + w * 256 * row[:, x1] + 32768) >> 16
    assert np.array_equal(img[:448].astype(np.int64), want)
    gs.close()
    be.close()


def test_extwrite_writes_merged_frame_back():
    """EXTWRITE with EMODC = EMODA = 0 writes the merged texels into VRAM at
    EXBP as CT32 (one texel per column at SMPH = 1 with clock divider 2)."""
    be, gs = make(5)
    regs = prog_frame_regs(g.pmode_reg(en1=1, en2=0, mmod=1, alp=0xFF))
    exbp = 300 * 32
    regs.update({13: 1, 11: g.extbuf_reg(exbp=exbp, exbw=10, fbin=0, wffmd=1),
                 12: g.extdata_reg(smph=1, smpv=0, ww=639, wh=447)})
    set_priv(gs, regs)
    img, r = gs.vsync(0, FP)
    vram = gs.read_vram()
    got = np.empty((448, 640), dtype=np.uint32)
    ys, xs = np.mgrid[0:448, 0:640]
    addr = np.vectorize(lambda x, y: _swz(int(x), int(y), exbp, 10, g.PSMCT32))(xs, ys)
    got = vram.view(np.uint32)[addr]
    want = img.view(np.uint32).reshape(448, 640)
    assert np.array_equal(got, want)
    gs.close()
    be.close()


def test_extwrite_ycbcr_modes_are_in_range():
    be, gs = make(6)
    regs = prog_frame_regs(g.pmode_reg(en1=1, en2=0, mmod=1, alp=0xFF))
    regs.update({13: 1, 11: g.extbuf_reg(exbp=300 * 32, exbw=4, fbin=1, wffmd=0, emoda=1, emodc=2),
                 12: g.extdata_reg(smph=1, smpv=0, ww=255, wh=63)})
    set_priv(gs, regs)
    gs.vsync(0, FP)
    vram = gs.read_vram().view(np.uint32)
    ys, xs = np.mgrid[0:128, 0:256]
    addr = np.vectorize(lambda x, y: _swz(int(x), int(y), 300 * 32, 4, g.PSMCT32))(xs, ys)
    px = vram[addr]
    Y = px & 0xFF
    # Studio-range luma: 16..235, and the alpha channel carries Y.
    assert Y.min() >= 16 and Y.max() <= 235
    assert np.array_equal((px >> 24) & 0xFF, Y)
    gs.close()
    be.close()


def test_deinterlace_weaves_fields():
    """Interlaced NTSC without forced progressive: the output is two fields
    tall; lines of the current field come from it, and on the first frame
    (history filled with the same field) the other lines repeat it with alpha
    255 (FastMAD's weave of an unchanged field)."""
    be, gs = make(7)
    set_priv(gs, ntsc_field_regs(g.pmode_reg(en1=1, en2=0, mmod=1, alp=0xFF)))
    img, r = gs.vsync(1, 0)
    assert r["interlaced"] and img.shape[0] == 2 * r["mode_height"]
    cur = img[1::2]
    other = img[0::2]
    assert np.array_equal(other[:, :, :3], cur[:, :, :3])
    assert np.all(other[1:, :, 3] == 255)
    img2, r2 = gs.vsync(0, 0)
    assert img2.shape == img.shape
    img3, _ = gs.vsync(0, pgs.GSInterface.VSYNC["SKIP_DEINTERLACE"])
    assert img3.shape[0] == r["mode_height"]
    gs.close()
    be.close()


def test_raw_circuit_passthrough():
    be, gs = make(8)
    set_priv(gs, prog_frame_regs(g.pmode_reg(en1=1, en2=0, mmod=1, alp=0xFF)))
    img, r = gs.vsync(0, FP | ADAPT | pgs.GSInterface.VSYNC["RAW_CIRCUIT"])
    circ = gs.scanout_circuit(0, 0, pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)
    assert np.array_equal(img, circ)
    gs.close()
    be.close()


@pytest.mark.parametrize("seed", range(6))
def test_random_crtc_state_runs(seed):
    """Random register states produce a sized image or a clean 0x0 (oracle only)."""
    be, gs = make(seed)
    rng = np.random.default_rng(100 + seed)
    set_priv(gs, g.random_crtc(rng))
    for phase in (0, 1):
        img, r = gs.vsync(phase, int(rng.integers(0, 256)))
        assert img.shape[:2] == (r["height"], r["width"])
    gs.close()
    be.close()
