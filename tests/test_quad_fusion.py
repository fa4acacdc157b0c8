"""Triangle-pair fusion (gs/gs_interface.cpp:2569-2602, gs/gs_util.cpp:237-377):
two right triangles that tile an axis-aligned rectangle, drawn back to back
with no state change, become one parallelogram primitive; the result in VRAM
is the same as drawing the two triangles."""
import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle
from recording_backend import RecordingBackend

PARALLELOGRAM = 1 << 15


def rect_stream(split, textured, ss, n=60, seed=7):
    """n rectangles as triangle pairs in one PACKED list each (split: a DIMX
    write between the halves, state the template depends on, which keeps them
    apart; a register that feeds no derived state, such as FOGCOL, would not)."""
    rng = np.random.default_rng(seed)
    s = g.GifStream()
    g._frame_setup(s, 0, 5, g.PSMCT32, 60, g.PSMZ24, 320, 224, g.test_reg(zte=1, ztst=1))
    s.upload(200 * 32, 1, g.PSMCT32, 0, 0, 64, 64, rng.integers(0, 256, size=64 * 64 * 4, dtype=np.uint8).tobytes())
    s.ad([(g.TEX0_1, g.tex0_reg(200 * 32, 1, g.PSMCT32, 6, 6, tcc=1, tfx=1)), (g.TEX1_1, g.tex1_reg(mmag=1, mmin=1))])
    for k in range(n):
        w, h = int(rng.integers(1, 80)), int(rng.integers(1, 60))
        x0, y0 = int(rng.integers(0, 240)), int(rng.integers(0, 160))
        sx, sy = [int(v) for v in rng.integers(0, 16, size=2)]
        X = [x0 * 16 + sx, (x0 + w) * 16 + sx]
        Y = [y0 * 16 + sy, (y0 + h) * 16 + sy]
        C = [(X[0], Y[0]), (X[1], Y[0]), (X[1], Y[1]), (X[0], Y[1])]
        u0, v0 = int(rng.integers(0, 32)) * 16, int(rng.integers(0, 32)) * 16
        du, dv = int(rng.integers(1, 40)) * 16, int(rng.integers(1, 40)) * 16
        UV = [(u0, v0), (u0 + du, v0), (u0 + du, v0 + dv), (u0, v0 + dv)]
        # Right angle at the last or the first vertex sent (the kick stores
        # vertices newest first): provoking vertex 0 or 2.
        tris = [[3, 1, 0], [3, 1, 2]] if k % 2 else [[0, 1, 3], [2, 3, 1]]
        col = [int(c) for c in rng.integers(0, 256, size=4)]
        z = int(rng.integers(0, 1 << 24))
        vs = [c for t in tris for c in t]
        q = np.zeros((6, 3, 2), dtype=np.uint64)
        q[:, 0] = g.q_rgbaq(np.array([col] * 6))
        q[:, 1] = g.q_uv(np.array([UV[c][0] for c in vs]), np.array([UV[c][1] for c in vs]))
        q[:, 2] = g.q_xyz2(np.array([C[c][0] for c in vs]), np.array([C[c][1] for c in vs]), np.array([z] * 6))
        p = g.prim_reg(g.PRIM_TRI, tme=int(textured), fst=1)
        desc = [g.D_RGBAQ, g.D_UV, g.D_XYZ2]
        if split:
            s.packed(p, desc, q[:3].reshape(-1, 2))
            s.ad([(g.DIMX, k + 1)])
            s.packed(p, desc, q[3:].reshape(-1, 2))
        else:
            s.packed(p, desc, q.reshape(-1, 2))
    return g.Frame("rects", s.tobytes(), ss, True, 0, {})


def recorded_prims(frame):
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=frame.super_sampling)
    gs.gif_transfer(0, frame.data)
    gs.flush()
    prims = [p for rp in be.passes for p in rp["prims"]]
    gs.close()
    return prims


def test_pairs_fuse_unless_state_changes():
    fused = recorded_prims(rect_stream(False, True, 1))
    assert len(fused) == 60 and all(p["state"] & PARALLELOGRAM for p in fused)
    assert {(p["state"] >> 27) & 3 for p in fused} == {0, 2}
    split = recorded_prims(rect_stream(True, True, 1))
    assert len(split) == 120 and not any(p["state"] & PARALLELOGRAM for p in split)


def test_only_rectangle_halves_fuse():
    """Different Z or colour, a second triangle off the rectangle, or a right
    angle at the middle vertex (which the reference's angle test rejects)
    leave two triangles."""
    def pair(t0, t1, z1=5, col1=(9, 9, 9, 9)):
        s = g.GifStream()
        g._frame_setup(s, 0, 5, g.PSMCT32, 60, g.PSMZ24, 320, 224, g.test_reg(zte=0))
        C = [(160, 160), (480, 160), (480, 400), (160, 400), (496, 400)]
        q = np.zeros((6, 2, 2), dtype=np.uint64)
        q[:, 0] = g.q_rgbaq(np.array([(9, 9, 9, 9)] * 3 + [col1] * 3))
        q[:, 1] = g.q_xyz2(np.array([C[c][0] for c in t0 + t1]), np.array([C[c][1] for c in t0 + t1]),
                           np.array([5] * 3 + [z1] * 3))
        s.packed(g.prim_reg(g.PRIM_TRI), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))
        return len(recorded_prims(g.Frame("pair", s.tobytes(), 1, True, 0, {})))
    assert pair([0, 1, 3], [2, 3, 1]) == 1
    assert pair([0, 1, 3], [2, 3, 1], z1=6) == 2
    assert pair([0, 1, 3], [2, 3, 1], col1=(9, 9, 9, 8)) == 2
    assert pair([0, 1, 3], [4, 3, 1]) == 2
    assert pair([1, 0, 2], [3, 2, 0]) == 1
    assert pair([0, 1, 2], [0, 2, 3]) == 2   # right angle at B in both halves


@pytest.mark.parametrize("textured,ss", [(False, 1), (True, 1), (False, 4), (True, 4)])
def test_fused_rendering_equals_two_triangles(textured, ss):
    a = pgs_oracle.render(rect_stream(False, textured, ss), planes=True)
    b = pgs_oracle.render(rect_stream(True, textured, ss), planes=True)
    assert np.array_equal(a, b)
