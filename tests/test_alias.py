"""Frame and depth buffer at the same base page: depth reads see colour
written by earlier primitives of the same pass (the reference's aliased
dispatch order, gs/gs_renderer.cpp:2418-2650).  GPU parity on seeded aliasing
frames is in test_gpu_parity.py."""
import numpy as np

import gsgen as g
import pgs
import pgs_oracle


def swz(x, y, psm, base=0, stride=4):
    return pgs_oracle.load_oracle().pgs_oracle_swizzle(x, y, base, stride, psm)


def partner(qx, qy):
    """Pixel whose CT32 colour word is pixel (qx, qy)'s Z32 depth word."""
    za = swz(qx, qy, g.PSMZ32)
    for y in range(32):
        for x in range(64):
            if swz(x, y, g.PSMCT32) == za:
                return x, y
    raise AssertionError


def sprite(s, x0, y0, x1, y1, z, rgba):
    q = np.zeros((2, 2, 2), dtype=np.uint64)
    q[:, 0] = g.q_rgbaq(np.array([rgba, rgba], dtype=np.int64))
    q[:, 1] = g.q_xyz2(np.array([x0 * 16, x1 * 16]), np.array([y0 * 16, y1 * 16]), np.array([z, z]))
    s.packed(g.prim_reg(g.PRIM_SPRITE), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))


def run(z_probe):
    qx, qy = 3, 2
    px, py = partner(qx, qy)
    assert (px // 8, py // 8) != (qx // 8, qy // 8)
    s = g.GifStream()
    s.ad([(g.PRMODECONT, 1), (g.FRAME_1, g.frame_reg(0, 4, g.PSMCT32)), (g.ZBUF_1, g.zbuf_reg(0, g.PSMZ32, 1)),
          (g.SCISSOR_1, g.scissor_reg(0, 255, 0, 127)), (g.XYOFFSET_1, 0), (g.TEST_1, g.test_reg(zte=1, ztst=1))])
    # 1: colour 0x40302010 at P (no depth test) -- this is Q's depth.
    sprite(s, px, py, px + 1, py + 1, 0, (0x10, 0x20, 0x30, 0x40))
    # 2: depth-tested (GEQUAL, no depth write) sprite over Q with depth z_probe.
    s.ad([(g.TEST_1, g.test_reg(zte=1, ztst=2))])
    sprite(s, qx, qy, qx + 1, qy + 1, z_probe, (0xAA, 0xBB, 0xCC, 0xDD))
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    gs.gif_transfer(0, s.tobytes())
    v = gs.read_vram().view(np.uint32)
    gs.close()
    be.close()
    return v[swz(qx, qy, g.PSMCT32)]


def test_depth_test_reads_aliased_colour():
    assert run(0x40302010) == 0xDDCCBBAA   # z >= depth passes
    assert run(0x4030200F) != 0xDDCCBBAA   # one below the aliased colour fails
