"""The CPU oracle against golden vectors produced by the reference's own code.

tests/golden/make_golden.py compiles the reference's swizzle_PS2 and
vram_upload/vram_readback (gs/gs_util.hpp:49-205) from its sources and records
their outputs; these tests replay the same cases through the oracle (and, for
transfers, through the product frontend on the oracle backend)."""
from pathlib import Path

import numpy as np
import pytest

import gsgen
import pgs
import pgs_oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
VRAM = pgs.VRAM_SIZE
PSMS = {"CT32": 0x00, "CT24": 0x01, "CT16": 0x02, "CT16S": 0x0A, "T8": 0x13, "T4": 0x14, "T8H": 0x1B,
        "T4HL": 0x24, "T4HH": 0x2C, "Z32": 0x30, "Z24": 0x31, "Z16": 0x32, "Z16S": 0x3A}


def formula_vram(psm: int) -> np.ndarray:
    i = np.arange(VRAM, dtype=np.uint64)
    return (((i * np.uint64(0x9E3779B1) + np.uint64(psm * 7919)) >> np.uint64(11)) & np.uint64(0xFF)).astype(np.uint8)


@pytest.mark.parametrize("name", sorted(PSMS))
def test_oracle_swizzle_matches_reference(name):
    data = np.load(GOLDEN / "ref_swizzle.npz")[name]
    lib = pgs_oracle.load_oracle()
    x, y, base, stride, expected = data
    got = np.array([lib.pgs_oracle_swizzle(int(a), int(b), int(c), int(d), PSMS[name])
                    for a, b, c, d in zip(x, y, base, stride)], dtype=np.uint32)
    assert np.array_equal(got, expected)


@pytest.mark.parametrize("name", sorted(PSMS))
def test_host_to_local_upload_matches_reference(name):
    g = np.load(GOLDEN / "ref_upload.npz")
    base, stride, x, y, w, h = (int(v) for v in g[name])
    data = g[name + "_data"].tobytes()
    psm = PSMS[name]
    init = formula_vram(psm)
    expected = init.copy()
    expected[g[name + "_idx"]] = g[name + "_val"]

    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=1)
    gs.write_vram(init)
    s = gsgen.GifStream()
    s.upload(base, stride, psm, x, y, w, h, data)
    gs.gif_transfer(0, s.tobytes())
    got = gs.read_vram()
    gs.close()
    be.close()
    assert np.array_equal(got, expected)


@pytest.mark.parametrize("name", sorted(n for n in PSMS if n not in ("T4", "T4HL", "T4HH")))
def test_local_to_host_readback_matches_reference(name):
    g = np.load(GOLDEN / "ref_readback.npz")
    base, stride, x, y, w, h = (int(v) for v in g[name])
    expected = g[name + "_out"]
    psm = PSMS[name]
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=1)
    gs.write_vram(formula_vram(psm))
    gs.write_register(gsgen.BITBLTBUF, gsgen.bitbltbuf_reg(sbp=base, sbw=stride, spsm=psm))
    gs.write_register(gsgen.TRXPOS, gsgen.trxpos_reg(ssax=x, ssay=y))
    gs.write_register(gsgen.TRXREG, gsgen.trxreg_reg(w, h))
    gs.write_register(gsgen.TRXDIR, 1)
    n128 = (expected.size + 15) // 16
    got = np.frombuffer(gs.read_transfer_fifo(n128), dtype=np.uint8)[: expected.size]
    gs.close()
    be.close()
    # The FIFO holds whole 128-bit words (fifo_readback_128b_size = bytes / 16,
    # gs/gs_interface.cpp:3220); reads past it return zeros (:3155-3157).
    whole = (expected.size // 16) * 16
    assert np.array_equal(got[:whole], expected[:whole])
    assert not got[whole:].any()
