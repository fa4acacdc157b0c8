"""CRTC circuit read-out (sample_circuit.frag via compute_circuit_rect /
sample_crtc_circuit) on the oracle: known answers from the swizzled VRAM."""
import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle
from recording_backend import RecordingBackend


def expected_1x(vram, psm, fbp, fbw, dbx, dby, w, h, phase=0, stride=1, valid_h=None):
    lib = pgs_oracle.load_oracle()
    out = np.zeros((h, w, 4), dtype=np.uint8)
    valid_h = h if valid_h is None else valid_h
    v16 = vram.view(np.uint16)
    v32 = vram.view(np.uint32)
    for y in range(valid_h):
        for x in range(w):
            a = lib.pgs_oracle_swizzle(x + dbx, y * stride + dby + phase, fbp * 32, fbw, psm)
            if psm in (g.PSMCT16, g.PSMCT16S):
                c = int(v16[a])
                px = ((c & 0x1F) << 3) | (((c >> 5) & 0x1F) << 11) | (((c >> 10) & 0x1F) << 19) | \
                     ((0xFF if c & 0x8000 else 0) << 24)
            else:
                px = int(v32[a])
                if psm != g.PSMCT32:
                    px = (px & 0xFFFFFF) | 0x80000000
            out[y, x] = [(px >> (8 * k)) & 0xFF for k in range(4)]
    return out


@pytest.mark.parametrize("psm", [g.PSMCT32, g.PSMCT24, g.PSMCT16, g.PSMCT16S])
def test_scanout_progressive_matches_vram(psm):
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    rng = np.random.default_rng(5)
    gs.write_vram(rng.integers(0, 256, pgs.VRAM_SIZE, dtype=np.uint8).tobytes())
    gs.write_priv_register("SMODE2", g.smode2_reg(0, 0))
    gs.write_priv_register("DISPFB1", g.dispfb_reg(40, 3, psm, dbx=5, dby=9))
    gs.write_priv_register("DISPLAY1", g.display_reg(600, 40, 3, 0, 4 * 96 - 1, 50 - 1))
    img = gs.scanout_circuit(0)
    vram = gs.read_vram()
    assert img.shape == (50, 96, 4)
    assert np.array_equal(img, expected_1x(vram, psm, 40, 3, 5, 9, 96, 50))
    gs.close()
    be.close()


def test_scanout_interlaced_field_and_odd_height():
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    rng = np.random.default_rng(6)
    gs.write_vram(rng.integers(0, 256, pgs.VRAM_SIZE, dtype=np.uint8).tobytes())
    vram = gs.read_vram()
    gs.write_priv_register("SMODE2", g.smode2_reg(1, 0))          # interlaced, field mode
    gs.write_priv_register("DISPFB2", g.dispfb_reg(10, 2, g.PSMCT32))
    gs.write_priv_register("DISPLAY2", g.display_reg(0, 1, 0, 0, 64 - 1, 37 - 1))
    for phase in (0, 1):
        img = gs.scanout_circuit(1, phase=phase)
        # DY = 1: the field starting on an odd line begins right away.
        offset = (1 ^ phase) & 1
        h = (37 + 1) >> 1
        valid = (37 - offset + 1) >> 1
        assert img.shape == (h, 64, 4)
        exp = expected_1x(vram, g.PSMCT32, 10, 2, 0, 0, 64, h, phase=offset, stride=2, valid_h=valid)
        assert np.array_equal(img, exp)
    # Forced progressive reads every line at full height, rounded up to even.
    img = gs.scanout_circuit(1, phase=1, flags=pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)
    assert img.shape == (38, 64, 4)
    assert np.array_equal(img, expected_1x(vram, g.PSMCT32, 10, 2, 0, 0, 64, 38, valid_h=37))
    gs.close()
    be.close()


def test_scanout_high_resolution_resolves_samples():
    """4x ordered: the 2x2 read-out returns each sample (plane 2 + quad) where
    the reference plane marks the pixel super-sampled, else plane 0."""
    f = g.frame_c1(seed=9, num_triangles=400, width=128, height=64)
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=4)
    gs.gif_transfer(0, f.data)
    gs.write_priv_register("DISPFB1", g.dispfb_reg(0, 2, g.PSMCT32))
    gs.write_priv_register("DISPLAY1", g.display_reg(0, 0, 0, 0, 128 - 1, 64 - 1))
    img = gs.scanout_circuit(0, flags=pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE | pgs.GSInterface.SCANOUT_HIGH_RESOLUTION)
    assert img.shape == (128, 256, 4)
    planes = [be.read_plane(p) for p in range(6)]
    lib = pgs_oracle.load_oracle()
    hits = 0
    for y in range(0, 128, 7):
        for x in range(0, 256, 5):
            a = lib.pgs_oracle_swizzle(x >> 1, y >> 1, 0, 2, g.PSMCT32)
            ref = int(planes[1].view(np.uint32)[a])
            quad = (y & 1) + (x & 1) * 2
            src = planes[2 + quad] if ref == 0xFFFFFFFF else planes[0]
            hits += ref == 0xFFFFFFFF
            px = int(src.view(np.uint32)[a])
            assert list(img[y, x]) == [(px >> (8 * k)) & 0xFF for k in range(4)], (x, y)
    assert hits > 0
    # Without high resolution the same call samples plane 0 at 1x.
    img1 = gs.scanout_circuit(0, flags=pgs.GSInterface.SCANOUT_FORCE_PROGRESSIVE)
    assert img1.shape == (64, 128, 4)
    gs.close()
    be.close()


def test_scanout_needs_backend_support():
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    with pytest.raises(pgs.PGSError):
        gs.scanout_circuit(0)
    gs.close()
