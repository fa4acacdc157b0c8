"""A stream whose textured draw is followed, in the same render pass, by an
upload into that texture: the texture must be read as it was before the
upload (the reference's texture cache holds the image; here a VRAM snapshot).
"""
import numpy as np

import gsgen


def sample_then_upload(parts: bool = False):
    """The frame, or its two halves (draw / upload) when `parts` is set."""
    rng = np.random.default_rng(3)
    head = gsgen.GifStream()
    gsgen._frame_setup(head, 0, 2, gsgen.PSMCT32, 100, gsgen.PSMZ24, 128, 64, gsgen.test_reg(zte=0))
    head.upload(200 * 32, 1, gsgen.PSMCT32, 0, 0, 64, 64, rng.integers(0, 256, 64 * 64 * 4, dtype=np.uint8).tobytes())
    head.ad([(gsgen.TEX0_1, gsgen.tex0_reg(200 * 32, 1, gsgen.PSMCT32, 6, 6))])
    q = np.zeros((2, 3, 2), dtype=np.uint64)
    q[:, 0] = gsgen.q_rgbaq(np.full((2, 4), 128))
    q[:, 1] = gsgen.q_uv(np.array([0, 64 * 16]), np.array([0, 64 * 16]))
    q[:, 2] = gsgen.q_xyz2(np.array([0, 64 * 16]), np.array([0, 64 * 16]), np.array([0, 0]))
    head.packed(gsgen.prim_reg(gsgen.PRIM_SPRITE, tme=1, fst=1), [gsgen.D_RGBAQ, gsgen.D_UV, gsgen.D_XYZ2],
                q.reshape(-1, 2))
    tail = gsgen.GifStream()
    tail.upload(200 * 32, 1, gsgen.PSMCT32, 0, 0, 64, 64, rng.integers(0, 256, 64 * 64 * 4, dtype=np.uint8).tobytes())
    # A second draw after the upload reads the new texels.
    q[:, 2] = gsgen.q_xyz2(np.array([64 * 16, 128 * 16]), np.array([0, 64 * 16]), np.array([0, 0]))
    tail.packed(gsgen.prim_reg(gsgen.PRIM_SPRITE, tme=1, fst=1), [gsgen.D_RGBAQ, gsgen.D_UV, gsgen.D_XYZ2],
                q.reshape(-1, 2))
    if parts:
        return head.tobytes(), tail.tobytes()
    return gsgen.Frame("sample_then_upload", head.tobytes() + tail.tobytes(), 1, True, 2, {})
