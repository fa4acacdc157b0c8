"""GS transfers on the CUDA backend against golden vectors produced by the
reference's own code (tests/golden/make_golden.py: vram_upload and
vram_readback of gs/gs_util.hpp:50-205, compiled from the reference).

Host->local uploads run through the upload kernel (live) and through the
batched upload kernel (a replay of the recorded upload next to a second one
on other pages); local->host read-outs run through the device de-swizzle
(pgs_backend_ops.readback_rect)."""
from pathlib import Path

import numpy as np
import pytest

import gsgen
import pgs

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
VRAM = pgs.VRAM_SIZE
PSMS = {"CT32": 0x00, "CT24": 0x01, "CT16": 0x02, "CT16S": 0x0A, "T8": 0x13, "T4": 0x14, "T8H": 0x1B,
        "T4HL": 0x24, "T4HH": 0x2C, "Z32": 0x30, "Z24": 0x31, "Z16": 0x32, "Z16S": 0x3A}


def formula_vram(psm: int) -> np.ndarray:
    i = np.arange(VRAM, dtype=np.uint64)
    return (((i * np.uint64(0x9E3779B1) + np.uint64(psm * 7919)) >> np.uint64(11)) & np.uint64(0xFF)).astype(np.uint8)


@pytest.mark.parametrize("name", sorted(PSMS))
def test_upload_matches_reference_on_gpu(name):
    g = np.load(GOLDEN / "ref_upload.npz")
    base, stride, x, y, w, h = (int(v) for v in g[name])
    data = g[name + "_data"].tobytes()
    psm = PSMS[name]
    init = formula_vram(psm)
    expected = init.copy()
    expected[g[name + "_idx"]] = g[name + "_val"]
    # A second upload far away (last page, a 64 x 32 CT32 rectangle) makes the
    # replay launch both in one batched kernel.
    s = gsgen.GifStream()
    s.upload(base, stride, psm, x, y, w, h, data)
    extra = np.random.default_rng(1).integers(0, 256, 64 * 32 * 4, dtype=np.uint8)
    s.upload(511 * 32, 1, gsgen.PSMCT32, 0, 0, 64, 32, extra.tobytes())

    be = pgs.CudaBackend(0, max_samples_log2=0)
    try:
        gs = pgs.GSInterface(be, super_sampling=1)
        gs.write_vram(init)
        be.begin_record()
        gs.gif_transfer(0, s.tobytes())
        gs.flush()
        be.end_record()
        live = be.read_plane(0)
        be.replay(1, reset_vram=True, use_graph=False)
        replay = be.read_plane(0)
        gs.close()
    finally:
        be.close()
    last_page = slice(VRAM - 8192, VRAM)
    assert np.array_equal(live[:VRAM - 8192], expected[:VRAM - 8192])
    assert np.array_equal(replay, live)
    assert not np.array_equal(live[last_page], init[last_page])


@pytest.mark.parametrize("name", sorted(n for n in PSMS if n not in ("T4", "T4HL", "T4HH")))
def test_readback_matches_reference_on_gpu(name):
    g = np.load(GOLDEN / "ref_readback.npz")
    base, stride, x, y, w, h = (int(v) for v in g[name])
    expected = g[name + "_out"]
    psm = PSMS[name]
    be = pgs.CudaBackend(0, max_samples_log2=0)
    try:
        gs = pgs.GSInterface(be, super_sampling=1)
        gs.write_vram(formula_vram(psm))
        gs.write_register(gsgen.BITBLTBUF, gsgen.bitbltbuf_reg(sbp=base, sbw=stride, spsm=psm))
        gs.write_register(gsgen.TRXPOS, gsgen.trxpos_reg(ssax=x, ssay=y))
        gs.write_register(gsgen.TRXREG, gsgen.trxreg_reg(w, h))
        d2h0 = be.stats()["d2h_bytes"]
        gs.write_register(gsgen.TRXDIR, 1)
        d2h = be.stats()["d2h_bytes"] - d2h0
        n128 = (expected.size + 15) // 16
        got = np.frombuffer(gs.read_transfer_fifo(n128), dtype=np.uint8)[: expected.size]
        gs.close()
    finally:
        be.close()
    whole = (expected.size // 16) * 16
    assert np.array_equal(got[:whole], expected[:whole])
    assert not got[whole:].any()
    # Only the rectangle crossed to the host, not the 4 MiB plane.
    assert d2h == expected.size
