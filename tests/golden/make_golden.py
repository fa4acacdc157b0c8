"""Generates the golden fixtures in this directory from the reference's own code.

Run in a checkout where the reference sources are present (they are compiled by
parallel-gs_gb300/build.py into oracle/_ref/libpgsref.so):

    python tests/golden/make_golden.py

Fixtures (all seeded):
  ref_swizzle.npz   swizzle_PS2 (gs/shaders/swizzle_utils.h:329-522) for every
                    storage format at random coordinates, base pointers and strides.
  ref_upload.npz    vram_upload<PSM> (gs/gs_util.hpp:112-205): a rectangle of random
                    data written into a random VRAM image, stored as the changed
                    bytes.
  ref_readback.npz  vram_readback<PSM> (gs/gs_util.hpp:49-110) of a rectangle of a
                    random VRAM image.
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "parallel-gs_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

import build_oracle  # noqa: E402
import pgs_oracle  # noqa: E402

VRAM = 4 * 1024 * 1024
PSMS = {"CT32": 0x00, "CT24": 0x01, "CT16": 0x02, "CT16S": 0x0A, "T8": 0x13, "T4": 0x14, "T8H": 0x1B,
        "T4HL": 0x24, "T4HH": 0x2C, "Z32": 0x30, "Z24": 0x31, "Z16": 0x32, "Z16S": 0x3A}
BPP = {0x00: 32, 0x01: 24, 0x02: 16, 0x0A: 16, 0x13: 8, 0x14: 4, 0x1B: 8, 0x24: 4, 0x2C: 4, 0x30: 32, 0x31: 24,
       0x32: 16, 0x3A: 16}
# Rectangle per format: (base block, stride, x, y, w, h); odd offsets on purpose, and
# w * h * bpp a multiple of 64 bits so the HWREG payload is whole qwords.
RECTS = {0x00: (1024, 10, 3, 5, 37, 22), 0x01: (2048, 4, 9, 2, 21, 24), 0x02: (4096, 6, 17, 11, 33, 12),
         0x0A: (4160, 3, 1, 30, 40, 7), 0x13: (6144, 4, 5, 3, 50, 20), 0x14: (8192, 4, 8, 6, 64, 30),
         0x1B: (9000, 2, 2, 2, 16, 16), 0x24: (9500, 2, 4, 1, 24, 10), 0x2C: (9600, 2, 0, 0, 32, 12),
         0x30: (10000, 5, 7, 13, 19, 26), 0x31: (11000, 4, 60, 33, 31, 16), 0x32: (12000, 2, 11, 63, 45, 4),
         0x3A: (13000, 1, 62, 1, 20, 20)}


def formula_vram(psm: int) -> np.ndarray:
    """Deterministic VRAM image that does not depend on numpy's generator streams."""
    i = np.arange(VRAM, dtype=np.uint64)
    return (((i * np.uint64(0x9E3779B1) + np.uint64(psm * 7919)) >> np.uint64(11)) & np.uint64(0xFF)).astype(np.uint8)


def main():
    build_oracle.build_reference_harness()
    ref = pgs_oracle.load_reference()
    if ref is None:
        raise SystemExit("reference harness unavailable: reference sources not present")
    rng = np.random.Generator(np.random.PCG64(20261203))

    sw = {}
    for name, psm in PSMS.items():
        n = 512
        x = rng.integers(0, 2048, n, dtype=np.uint32)
        y = rng.integers(0, 2048, n, dtype=np.uint32)
        base = rng.integers(0, 16384, n, dtype=np.uint32)
        stride = rng.integers(0, 64, n, dtype=np.uint32)
        out = np.array([ref.pgs_ref_swizzle(int(a), int(b), int(c), int(d), psm, VRAM - 1)
                        for a, b, c, d in zip(x, y, base, stride)], dtype=np.uint32)
        sw[name] = np.stack([x, y, base, stride, out])
    np.savez_compressed(HERE / "ref_swizzle.npz", **sw)

    up = {}
    for name, psm in PSMS.items():
        base, stride, x, y, w, h = RECTS[psm]
        init = formula_vram(psm)
        nbytes = (w * h * BPP[psm] + 7) // 8
        data = rng.integers(0, 256, nbytes, dtype=np.uint8)
        vram = init.copy()
        rc = ref.pgs_ref_vram_upload(psm, vram.ctypes.data, data.ctypes.data, base, stride, x, y, w, h, VRAM - 1)
        assert rc == 0
        idx = np.nonzero(vram != init)[0].astype(np.uint32)
        up[name] = np.array([base, stride, x, y, w, h], dtype=np.uint32)
        up[name + "_data"] = data
        up[name + "_idx"] = idx
        up[name + "_val"] = vram[idx]
    np.savez_compressed(HERE / "ref_upload.npz", **up)

    rb = {}
    for name, psm in PSMS.items():
        if BPP[psm] == 4:
            continue
        base, stride, x, y, w, h = RECTS[psm]
        vr = formula_vram(psm)
        out = np.zeros(w * h * 4, dtype=np.uint8)
        rc = ref.pgs_ref_vram_readback(psm, out.ctypes.data, vr.ctypes.data, base, stride, x, y, w, h, VRAM - 1)
        assert rc == 0
        nbytes = (w * h * BPP[psm]) // 8
        rb[name] = np.array([base, stride, x, y, w, h], dtype=np.uint32)
        rb[name + "_out"] = out[:nbytes]
    np.savez_compressed(HERE / "ref_readback.npz", **rb)
    for f in ("ref_swizzle.npz", "ref_upload.npz", "ref_readback.npz"):
        print(f, (HERE / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
