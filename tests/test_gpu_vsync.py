"""vsync on the CUDA backend against the CPU oracle: random privileged-register
states (video modes, both circuits, PMODE blends, BGCOLOR, EXTWRITE) over
random and rendered (super-sampled) VRAM; output images and the VRAM after
the EXTWRITE write-back must match byte for byte, across consecutive vsyncs
so the deinterlacer's field history is covered."""
import numpy as np
import pytest

import gsgen as g
import pgs
import pgs_oracle

pytestmark = pytest.mark.gpu


def run(backend, frame, vram, regs_seq, calls):
    gs = pgs.GSInterface(backend, super_sampling=frame.super_sampling if frame else 1,
                         ordered=frame.ordered if frame else True)
    if vram is not None:
        gs.write_vram(vram)
    if frame is not None:
        gs.gif_transfer(0, frame.data)
    outs = []
    for regs, (phase, flags) in zip(regs_seq, calls):
        for i, v in regs.items():
            gs.write_priv_register(i, v)
        img, r = gs.vsync(phase, flags)
        outs.append((img, r))
    outs.append((gs.read_vram(), None))
    gs.close()
    return outs


@pytest.mark.parametrize("seed", range(12))
def test_vsync_parity(seed):
    rng = np.random.default_rng(900 + seed)
    frame = g.frame_fuzz(seed) if seed % 2 else None
    vram = None if frame else rng.integers(0, 256, pgs.VRAM_SIZE, dtype=np.uint8)
    base = g.random_crtc(rng)
    regs_seq, calls = [], []
    for k in range(4):
        regs = dict(base) if k == 0 else {}
        if k == 2:
            regs[0] = g.pmode_reg(en1=1, en2=1, mmod=int(rng.integers(0, 2)), slbg=0, alp=int(rng.integers(0, 256)))
        regs_seq.append(regs)
        calls.append((k & 1, int(rng.integers(0, 256)) & ~pgs.GSInterface.VSYNC["SKIP_DEINTERLACE"]))
    obe = pgs_oracle.OracleBackend()
    ref = run(obe, frame, vram, regs_seq, calls)
    obe.close()
    be = pgs.CudaBackend(0, max_samples_log2=4)
    try:
        out = run(be, frame, vram, regs_seq, calls)
        assert be.error_flags() == 0
    finally:
        be.close()
    for i, ((a, ra), (b, rb)) in enumerate(zip(ref, out)):
        assert ra == rb, i
        assert a.shape == b.shape, i
        if not np.array_equal(a, b):
            diff = np.argwhere(a != b)
            raise AssertionError("call %d: %d values differ, first at %s" % (i, len(diff), diff[0]))
