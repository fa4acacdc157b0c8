"""Seeded GS command-stream generator.

Builds GIF packet streams (128-bit qwords) that drive the frontend exactly as a
PS2 program would: A+D register setup, BITBLTBUF/TRXPOS/TRXREG/TRXDIR + IMAGE
texture and CLUT uploads, and PACKED vertex data.  The packet layout follows
the GIF tag format decoded by GSInterface::gif_transfer
(gs/gs_interface.cpp:4290-4397) and written by GSDumpGenerator
(dump/gs_dump_generator.cpp:104-185).

Workloads (sizes from the benchmark configurations):
  frame_c1  640x448 PSMCT32 + PSMZ24, 10k Gouraud triangles, 1x.
  frame_c2  640x448 PSMCT32 + PSMZ24, 50k perspective-textured blended
            triangles + 2k sprites over 8 PSMT8 256x256 textures with CT32
            CLUTs, bilinear, ATST GREATER 0x40, FBA, dither, 4x SSAA.
  stream_c3 one of 64 mixed streams (C3), seeded by its stream id.
  frame_c4  640x448 at 8x/16x with render-to-texture feedback draws.
All randomness comes from numpy's PCG64 generator with an explicit seed.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

# A+D register addresses (gs/gs_register_addr.hpp).
PRIM, RGBAQ, ST, UV, XYZF2, XYZ2 = 0x00, 0x01, 0x02, 0x03, 0x04, 0x05
TEX0_1, TEX0_2, CLAMP_1, CLAMP_2, FOG = 0x06, 0x07, 0x08, 0x09, 0x0A
TEX1_1, TEX1_2, TEX2_1 = 0x14, 0x15, 0x16
XYOFFSET_1, XYOFFSET_2, PRMODECONT, PRMODE, TEXCLUT = 0x18, 0x19, 0x1A, 0x1B, 0x1C
SCANMSK, TEXA, FOGCOL, TEXFLUSH = 0x22, 0x3B, 0x3D, 0x3F
SCISSOR_1, SCISSOR_2, ALPHA_1, ALPHA_2, DIMX, DTHE, COLCLAMP = 0x40, 0x41, 0x42, 0x43, 0x44, 0x45, 0x46
TEST_1, TEST_2, PABE, FBA_1, FBA_2 = 0x47, 0x48, 0x49, 0x4A, 0x4B
FRAME_1, FRAME_2, ZBUF_1, ZBUF_2 = 0x4C, 0x4D, 0x4E, 0x4F
BITBLTBUF, TRXPOS, TRXREG, TRXDIR, HWREG = 0x50, 0x51, 0x52, 0x53, 0x54

PSMCT32, PSMCT24, PSMCT16, PSMCT16S = 0x00, 0x01, 0x02, 0x0A
PSMT8, PSMT4, PSMT8H = 0x13, 0x14, 0x1B
PSMZ32, PSMZ24, PSMZ16, PSMZ16S = 0x30, 0x31, 0x32, 0x3A

PRIM_POINT, PRIM_LINE, PRIM_LINESTRIP, PRIM_TRI, PRIM_TRISTRIP, PRIM_TRIFAN, PRIM_SPRITE = range(7)

# GIF PACKED register descriptors.
D_PRIM, D_RGBAQ, D_ST, D_UV, D_XYZF2, D_XYZ2, D_AD = 0x0, 0x1, 0x2, 0x3, 0x4, 0x5, 0xE

PAGE_BYTES = 8192
BLOCKS_PER_PAGE = 32


def f32_bits(x) -> np.ndarray:
    return np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)


def prim_reg(prim, iip=0, tme=0, fge=0, abe=0, aa1=0, fst=0, ctxt=0, fix=0) -> int:
    return (prim | (iip << 3) | (tme << 4) | (fge << 5) | (abe << 6) | (aa1 << 7) | (fst << 8) |
            (ctxt << 9) | (fix << 10))


def frame_reg(fbp, fbw, psm, fbmsk=0) -> int:
    return fbp | (fbw << 16) | (psm << 24) | (fbmsk << 32)


def zbuf_reg(zbp, psm, zmsk=0) -> int:
    return zbp | ((psm & 0xF) << 24) | (zmsk << 32)


def test_reg(ate=0, atst=1, aref=0, afail=0, date=0, datm=0, zte=1, ztst=1) -> int:
    return (ate | (atst << 1) | (aref << 4) | (afail << 12) | (date << 14) | (datm << 15) | (zte << 16) |
            (ztst << 17))


def alpha_reg(a, b, c, d, fix=0) -> int:
    return a | (b << 2) | (c << 4) | (d << 6) | (fix << 32)


def scissor_reg(x0, x1, y0, y1) -> int:
    return x0 | (x1 << 16) | (y0 << 32) | (y1 << 48)


def tex0_reg(tbp0, tbw, psm, tw, th, tcc=1, tfx=0, cbp=0, cpsm=0, csm=0, csa=0, cld=0) -> int:
    return (tbp0 | (tbw << 14) | (psm << 20) | (tw << 26) | (th << 30) | (tcc << 34) | (tfx << 35) |
            (cbp << 37) | (cpsm << 51) | (csm << 55) | (csa << 56) | (cld << 61))


def tex1_reg(lcm=0, mxl=0, mmag=0, mmin=0, mtba=0, l=0, k=0) -> int:
    return lcm | (mxl << 2) | (mmag << 5) | (mmin << 6) | (mtba << 9) | (l << 19) | (k << 32)


def clamp_reg(wms=0, wmt=0, minu=0, maxu=0, minv=0, maxv=0) -> int:
    return wms | (wmt << 2) | (minu << 4) | (maxu << 14) | (minv << 24) | (maxv << 34)


def texa_reg(ta0=0, aem=0, ta1=0x80) -> int:
    return ta0 | (aem << 15) | (ta1 << 32)


def bitbltbuf_reg(sbp=0, sbw=0, spsm=0, dbp=0, dbw=0, dpsm=0) -> int:
    return sbp | (sbw << 16) | (spsm << 24) | (dbp << 32) | (dbw << 48) | (dpsm << 56)


def trxpos_reg(ssax=0, ssay=0, dsax=0, dsay=0, dir_=0) -> int:
    return ssax | (ssay << 16) | (dsax << 32) | (dsay << 48) | (dir_ << 59)


def trxreg_reg(w, h) -> int:
    return w | (h << 32)


def dimx_reg(matrix) -> int:
    """4x4 dither matrix of values in [-4, 3]."""
    v = 0
    for r in range(4):
        for c in range(4):
            v |= (int(matrix[r][c]) & 7) << ((r * 4 + c) * 4)
    return v


DEFAULT_DIMX = [[-4, 2, -3, 3], [0, -2, 1, -1], [-3, 3, -4, 2], [1, -1, 0, -2]]


def gif_tag(nloop, flg, nreg, regs=0, eop=0, pre=0, prim=0) -> tuple[int, int]:
    lo = (nloop & 0x7FFF) | (eop << 15) | (pre << 46) | ((prim & 0x7FF) << 47) | (flg << 58) | ((nreg & 0xF) << 60)
    return lo, regs


class GifStream:
    """Accumulates 128-bit qwords as pairs of uint64."""

    def __init__(self) -> None:
        self.chunks: list[np.ndarray] = []

    def _qwords(self, arr: np.ndarray) -> None:
        self.chunks.append(np.ascontiguousarray(arr, dtype=np.uint64).reshape(-1, 2))

    def ad(self, regs: list[tuple[int, int]]) -> None:
        """One PACKED A+D packet writing (address, value) pairs."""
        n = len(regs)
        lo, hi = gif_tag(n, 0, 1, D_AD)
        q = np.zeros((n + 1, 2), dtype=np.uint64)
        q[0] = (lo, hi)
        for i, (addr, val) in enumerate(regs):
            q[i + 1] = (val & 0xFFFFFFFFFFFFFFFF, addr)
        self._qwords(q)

    def image(self, data: bytes) -> None:
        if len(data) % 16:
            data = data + bytes(16 - len(data) % 16)
        nq = len(data) // 16
        off = 0
        while off < nq:
            n = min(nq - off, 0x7FFF)
            lo, hi = gif_tag(n, 2, 0)
            self._qwords(np.array([[lo, hi]], dtype=np.uint64))
            self._qwords(np.frombuffer(data[off * 16:(off + n) * 16], dtype=np.uint64))
            off += n

    def upload(self, dbp, dbw, dpsm, x, y, w, h, data: bytes) -> None:
        self.ad([(BITBLTBUF, bitbltbuf_reg(dbp=dbp, dbw=dbw, dpsm=dpsm)),
                 (TRXPOS, trxpos_reg(dsax=x, dsay=y)),
                 (TRXREG, trxreg_reg(w, h)),
                 (TRXDIR, 0)])
        self.image(data)

    def packed(self, prim: int, desc: list[int], data: np.ndarray) -> None:
        """PACKED packets with a PRIM preset; data is (n_loops * len(desc), 2) qwords."""
        nreg = len(desc)
        regs = 0
        for i, d in enumerate(desc):
            regs |= d << (4 * i)
        data = np.ascontiguousarray(data, dtype=np.uint64).reshape(-1, nreg, 2)
        nloops = data.shape[0]
        off = 0
        # Keep every packet a whole number of primitives so PRE resets nothing mid-strip.
        step = (0x7FFF // 6) * 6
        while off < nloops:
            n = min(nloops - off, step)
            lo, hi = gif_tag(n, 0, nreg, regs, pre=1, prim=prim)
            self._qwords(np.array([[lo, hi]], dtype=np.uint64))
            self._qwords(data[off:off + n].reshape(-1, 2))
            off += n

    def tobytes(self) -> bytes:
        return np.concatenate(self.chunks).astype("<u8").tobytes()


def q_rgbaq(rgba: np.ndarray) -> np.ndarray:
    rgba = rgba.astype(np.uint64)
    lo = rgba[:, 0] | (rgba[:, 1] << np.uint64(32))
    hi = rgba[:, 2] | (rgba[:, 3] << np.uint64(32))
    return np.stack([lo, hi], axis=1)


def q_xyz2(x: np.ndarray, y: np.ndarray, z: np.ndarray) -> np.ndarray:
    lo = x.astype(np.uint64) | (y.astype(np.uint64) << np.uint64(32))
    hi = z.astype(np.uint64) & np.uint64(0xFFFFFFFF)
    return np.stack([lo, hi], axis=1)


def q_st(s: np.ndarray, t: np.ndarray, q: np.ndarray) -> np.ndarray:
    lo = f32_bits(s) | (f32_bits(t) << np.uint64(32))
    hi = f32_bits(q)
    return np.stack([lo, hi], axis=1)


def q_uv(u: np.ndarray, v: np.ndarray) -> np.ndarray:
    lo = u.astype(np.uint64) | (v.astype(np.uint64) << np.uint64(32))
    return np.stack([lo, np.zeros_like(lo)], axis=1)


def random_triangles(rng, n, width, height, area_lo, area_hi):
    """Triangles with log-uniform area, uniform centroid, random shape, in 12.4."""
    area = np.exp(rng.uniform(np.log(area_lo), np.log(area_hi), n))
    cx = rng.uniform(0, width, n)
    cy = rng.uniform(0, height, n)
    t0 = rng.uniform(0, 2 * np.pi, n)
    t1 = t0 + rng.uniform(np.pi / 3, np.pi, n)
    t2 = t1 + rng.uniform(np.pi / 3, np.pi, n)
    ang = np.stack([t0, t1, t2], axis=1)
    ux, uy = np.cos(ang), np.sin(ang)
    a0 = 0.5 * np.abs((ux[:, 1] - ux[:, 0]) * (uy[:, 2] - uy[:, 0]) - (ux[:, 2] - ux[:, 0]) * (uy[:, 1] - uy[:, 0]))
    r = np.sqrt(area / np.maximum(a0, 1e-3))
    x = cx[:, None] + ux * r[:, None]
    y = cy[:, None] + uy * r[:, None]
    xi = np.clip(np.round(x * 16), 0, width * 16 - 1).astype(np.int64)
    yi = np.clip(np.round(y * 16), 0, height * 16 - 1).astype(np.int64)
    return xi, yi


def random_sprites(rng, n, width, height, area_lo, area_hi):
    area = np.exp(rng.uniform(np.log(area_lo), np.log(area_hi), n))
    aspect = np.exp(rng.uniform(np.log(0.5), np.log(2.0), n))
    w = np.sqrt(area * aspect)
    h = area / w
    x0 = rng.uniform(0, width, n) - w / 2
    y0 = rng.uniform(0, height, n) - h / 2
    xs = np.stack([x0, x0 + w], axis=1)
    ys = np.stack([y0, y0 + h], axis=1)
    xi = np.clip(np.round(xs * 16), 0, width * 16 - 1).astype(np.int64)
    yi = np.clip(np.round(ys * 16), 0, height * 16 - 1).astype(np.int64)
    return xi, yi


@dataclass
class Frame:
    """One seeded command stream plus the options it needs."""
    name: str
    data: bytes
    super_sampling: int = 1
    ordered: bool = True
    num_primitives: int = 0
    meta: dict = field(default_factory=dict)


def _frame_setup(s: GifStream, fbp, fbw, fpsm, zbp, zpsm, width, height, test, alpha=0, extra=()):
    s.ad([(PRMODECONT, 1),
          (FRAME_1, frame_reg(fbp, fbw, fpsm)),
          (ZBUF_1, zbuf_reg(zbp, zpsm)),
          (SCISSOR_1, scissor_reg(0, width - 1, 0, height - 1)),
          (XYOFFSET_1, 0),
          (TEST_1, test),
          (ALPHA_1, alpha),
          *extra])


def frame_c1(seed: int = 1, num_triangles: int = 10000, width: int = 640, height: int = 448) -> Frame:
    """Plain method: untextured Gouraud triangles, Z GEQUAL, 1x."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = GifStream()
    zbp = (width * height * 4 + PAGE_BYTES - 1) // PAGE_BYTES
    _frame_setup(s, 0, width // 64, PSMCT32, zbp, PSMZ24, width, height,
                 test_reg(zte=1, ztst=2), extra=[(COLCLAMP, 1)])
    x, y = random_triangles(rng, num_triangles, width, height, 4.0, 4000.0)
    z = rng.integers(0, 1 << 24, size=(num_triangles, 3), dtype=np.int64)
    rgba = rng.integers(0, 256, size=(num_triangles, 3, 4), dtype=np.int64)
    nv = num_triangles * 3
    q = np.zeros((nv, 2, 2), dtype=np.uint64)
    q[:, 0] = q_rgbaq(rgba.reshape(nv, 4))
    q[:, 1] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
    s.packed(prim_reg(PRIM_TRI, iip=1), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
    return Frame("c1", s.tobytes(), 1, True, num_triangles,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp})


def _texture_set(rng, s: GifStream, base_page: int, count: int, tw: int, th: int, psm: int):
    """Uploads `count` paletted textures and their CT32 CLUTs; returns TEX0 values."""
    tex0s = []
    w, h = 1 << tw, 1 << th
    tbw = max(1, w // 64)
    if psm == PSMT8:
        tex_bytes = w * h
        clut_w, clut_h = 16, 16
    else:
        tex_bytes = w * h // 2
        clut_w, clut_h = 8, 2
    pages_per_tex = max(1, (tex_bytes + PAGE_BYTES - 1) // PAGE_BYTES)
    page = base_page
    clut_page = base_page + count * pages_per_tex
    for i in range(count):
        tbp0 = page * BLOCKS_PER_PAGE
        data = rng.integers(0, 256, size=tex_bytes, dtype=np.uint8).tobytes()
        s.upload(tbp0, tbw, psm, 0, 0, w, h, data)
        cbp = clut_page * BLOCKS_PER_PAGE + i * 4
        clut = rng.integers(0, 1 << 32, size=clut_w * clut_h, dtype=np.uint64).astype(np.uint32).tobytes()
        s.upload(cbp, 1, PSMCT32, 0, 0, clut_w, clut_h, clut)
        tex0s.append(tex0_reg(tbp0, tbw, psm, tw, th, tcc=1, tfx=0, cbp=cbp, cpsm=PSMCT32, csm=0, csa=0, cld=1))
        page += pages_per_tex
    return tex0s, clut_page + 1


def frame_c2(seed: int = 2, num_triangles: int = 50000, num_sprites: int = 2000, super_sampling: int = 4,
             width: int = 640, height: int = 448, num_textures: int = 8) -> Frame:
    """Textured and blended: PSMT8 + CT32 CLUT, perspective STQ, bilinear, alpha blend,
    ATST GREATER 0x40, FBA, dither, 4x SSAA."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = GifStream()
    fb_pages = (width * height * 4 + PAGE_BYTES - 1) // PAGE_BYTES
    zbp = fb_pages
    tex_base = 2 * fb_pages
    test = test_reg(ate=1, atst=6, aref=0x40, afail=0, zte=1, ztst=2)
    _frame_setup(s, 0, width // 64, PSMCT32, zbp, PSMZ24, width, height, test,
                 alpha=alpha_reg(0, 1, 0, 1),
                 extra=[(FBA_1, 1), (DTHE, 1), (DIMX, dimx_reg(DEFAULT_DIMX)), (COLCLAMP, 1),
                        (TEX1_1, tex1_reg(mmag=1, mmin=1)), (CLAMP_1, clamp_reg(0, 0)),
                        (TEXA, texa_reg(0, 0, 0x80)), (PABE, 0)])
    tex0s, _ = _texture_set(rng, s, tex_base, num_textures, 8, 8, PSMT8)
    tris_per = np.full(num_textures, num_triangles // num_textures)
    tris_per[: num_triangles % num_textures] += 1
    spr_per = np.full(num_textures, num_sprites // num_textures)
    spr_per[: num_sprites % num_textures] += 1
    for ti in range(num_textures):
        s.ad([(TEX0_1, tex0s[ti])])
        n = int(tris_per[ti])
        x, y = random_triangles(rng, n, width, height, 4.0, 4000.0)
        z = rng.integers(0, 1 << 24, size=(n, 3), dtype=np.int64)
        rgba = rng.integers(0, 256, size=(n, 3, 4), dtype=np.int64)
        qv = rng.uniform(0.25, 4.0, size=(n, 3)).astype(np.float32)
        sn = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
        tn = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
        nv = n * 3
        q = np.zeros((nv, 3, 2), dtype=np.uint64)
        q[:, 0] = q_st((sn * qv).reshape(nv), (tn * qv).reshape(nv), qv.reshape(nv))
        q[:, 1] = q_rgbaq(rgba.reshape(nv, 4))
        q[:, 2] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
        s.packed(prim_reg(PRIM_TRI, iip=1, tme=1, abe=1), [D_ST, D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
        m = int(spr_per[ti])
        if m:
            sx, sy = random_sprites(rng, m, width, height, 4.0, 4000.0)
            sz = rng.integers(0, 1 << 24, size=(m, 2), dtype=np.int64)
            srgba = rng.integers(0, 256, size=(m, 2, 4), dtype=np.int64)
            sq = rng.uniform(0.25, 4.0, size=(m, 2)).astype(np.float32)
            ss = rng.uniform(0.0, 1.0, size=(m, 2)).astype(np.float32)
            st = rng.uniform(0.0, 1.0, size=(m, 2)).astype(np.float32)
            mv = m * 2
            q = np.zeros((mv, 3, 2), dtype=np.uint64)
            q[:, 0] = q_st((ss * sq).reshape(mv), (st * sq).reshape(mv), sq.reshape(mv))
            q[:, 1] = q_rgbaq(srgba.reshape(mv, 4))
            q[:, 2] = q_xyz2(sx.reshape(mv), sy.reshape(mv), sz.reshape(mv))
            s.packed(prim_reg(PRIM_SPRITE, iip=1, tme=1, abe=1), [D_ST, D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
    return Frame("c2", s.tobytes(), super_sampling, True, num_triangles + num_sprites,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp})


def _mesh(rng, gx, gy, width, height, zlo, zhi):
    """A jittered grid mesh as a triangle list; returns (x, y, z) of shape (n, 3) in 12.4."""
    xs = np.linspace(8, width - 8, gx)
    ys = np.linspace(8, height - 8, gy)
    px = np.round((xs[None, :] + rng.uniform(-3, 3, (gy, gx))) * 16).astype(np.int64)
    py = np.round((ys[:, None] + rng.uniform(-3, 3, (gy, gx))) * 16).astype(np.int64)
    pz = rng.integers(zlo, zhi, size=(gy, gx), dtype=np.int64)
    tris = []
    for j in range(gy - 1):
        for i in range(gx - 1):
            tris.append(((j, i), (j, i + 1), (j + 1, i)))
            tris.append(((j, i + 1), (j + 1, i + 1), (j + 1, i)))
    idx = np.array(tris)
    return px[idx[..., 0], idx[..., 1]], py[idx[..., 0], idx[..., 1]], pz[idx[..., 0], idx[..., 1]]


def frame_flat_ui(seed: int = 5, super_sampling: int = 4, zpsm: int = PSMZ24, width: int = 640,
                  height: int = 448, grid: int = 24, num_flat: int = 400, num_lines: int = 64) -> Frame:
    """Super-sampled pass mixing a 3D mesh with flat (constant-Z) triangles and lines.

    Exercises the single-sample heuristic (triangle_setup.comp:826-871 and
    single_sample_heuristic.comp): flat triangles that share a vertex with the
    3D mesh at a depth the mesh uses, flat triangles at mesh depths without a
    shared vertex, flat UI triangles in front of the mesh, flat lines, and a
    second framebuffer with flat primitives only (every flat line demoted)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = GifStream()
    zbits = {PSMZ16: 16, PSMZ16S: 16, PSMZ24: 24, PSMZ32: 32}[zpsm]
    zmax = (1 << zbits) - 1
    fb_pages = (width * height * 4 + PAGE_BYTES - 1) // PAGE_BYTES
    zbp = fb_pages
    fb2 = 2 * fb_pages
    _frame_setup(s, 0, width // 64, PSMCT32, zbp, zpsm, width, height, test_reg(zte=1, ztst=2),
                 extra=[(COLCLAMP, 1)])

    def emit(prim, x, y, z):
        n = x.shape[0]
        nv = n * x.shape[1]
        rgba = rng.integers(0, 256, size=(nv, 4), dtype=np.int64)
        q = np.zeros((nv, 2, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(rgba)
        q[:, 1] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
        s.packed(prim, [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))

    def flat_tris(n, zvals, lo=2.0, hi=600.0):
        x, y = random_triangles(rng, n, width, height, lo, hi)
        return x, y, np.repeat(np.asarray(zvals, dtype=np.int64)[:, None], 3, axis=1)

    # 3D mesh in the middle of the depth range.
    z3lo, z3hi = zmax // 8, zmax // 2
    mx, my, mz = _mesh(rng, grid, grid * height // width + 2, width, height, z3lo, z3hi)
    emit(prim_reg(PRIM_TRI, iip=1), mx, my, mz)

    nq = num_flat // 4
    # Flat triangles sharing one mesh vertex and its depth.
    pick = rng.integers(0, mx.shape[0], nq)
    corner = rng.integers(0, 3, nq)
    sx, sy, sz = flat_tris(nq, mz[pick, corner])
    sx[:, 0], sy[:, 0] = mx[pick, corner], my[pick, corner]
    emit(prim_reg(PRIM_TRI, iip=1), sx, sy, sz)
    # Flat triangles at mesh depths, no shared vertex.
    pick = rng.integers(0, mx.shape[0], nq)
    emit(prim_reg(PRIM_TRI, iip=1), *flat_tris(nq, mz[pick, 0]))
    # Flat triangles at depths inside the mesh range that the mesh does not use.
    emit(prim_reg(PRIM_TRI, iip=1), *flat_tris(nq, rng.integers(z3lo, z3hi, nq) | 1))
    # UI in front of everything, few distinct depths.
    emit(prim_reg(PRIM_TRI, iip=1), *flat_tris(num_flat - 3 * nq, zmax - rng.integers(0, 4, num_flat - 3 * nq)))
    # Flat lines, in front and at mesh depths.
    lx, ly = random_sprites(rng, num_lines, width, height, 16.0, 4000.0)
    lz = np.where(rng.uniform(size=num_lines) < 0.5, zmax - 1, mz[rng.integers(0, mx.shape[0], num_lines), 0])
    emit(prim_reg(PRIM_LINE, iip=1), lx, ly, np.repeat(lz[:, None], 2, axis=1))

    # Second framebuffer: flat primitives only.
    s.ad([(FRAME_1, frame_reg(fb2, width // 64, PSMCT32))])
    emit(prim_reg(PRIM_TRI, iip=1), *flat_tris(nq, rng.integers(0, zmax, nq)))
    lx, ly = random_sprites(rng, num_lines, width, height, 16.0, 4000.0)
    emit(prim_reg(PRIM_LINE, iip=1), lx, ly, np.repeat(rng.integers(0, zmax, num_lines)[:, None], 2, axis=1))
    nprims = mx.shape[0] + num_flat + num_lines + nq + num_lines
    return Frame("flat_ui", s.tobytes(), super_sampling, True, nprims,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp, "fb2": fb2})


def _textured_draw(rng, n, width, height, area_lo_small, area_hi_small, area_lo_big, area_hi_big, big_frac):
    """n triangles, a `big_frac` share with large areas; returns x, y (n, 3) in 12.4."""
    big = rng.uniform(size=n) < big_frac
    nb = int(big.sum())
    x = np.zeros((n, 3), dtype=np.int64)
    y = np.zeros((n, 3), dtype=np.int64)
    if nb:
        x[big], y[big] = random_triangles(rng, nb, width, height, area_lo_big, area_hi_big)
    if n - nb:
        x[~big], y[~big] = random_triangles(rng, n - nb, width, height, area_lo_small, area_hi_small)
    return x, y


def frame_c4(seed: int = 4, super_sampling: int = 8, num_triangles: int = 100000, passes: int = 10,
             draws_per_pass: int = 50, feedback_frac: float = 0.2, width: int = 640, height: int = 448) -> Frame:
    """High-rate SSAA with render-to-texture feedback.

    640x448 PSMCT32 + PSMZ24 at 8x (2x4) or 16x (4x4).  `passes` passes, each
    opened by TEXFLUSH and a FRAME switch between two framebuffers A and B.
    80% of the triangles have areas log-uniform in [1, 16] px, 20% in
    [16, 4000].  A `feedback_frac` share of the draws samples the framebuffer the
    previous pass rendered (TBP0 on pages written earlier in the frame, CT32,
    bilinear, clamped to its top 512x256 region), so the sampled pages never
    overlap the framebuffer being drawn; the others are Gouraud or PSMT8
    textured.  Z GEQUAL throughout; feedback draws blend Cs over Cd by As."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = GifStream()
    fb_pages = (width * height * 4 + PAGE_BYTES - 1) // PAGE_BYTES
    fbw = width // 64
    fb_a, zbp, fb_b = 0, fb_pages, 2 * fb_pages
    tex_base = 3 * fb_pages
    _frame_setup(s, fb_a, fbw, PSMCT32, zbp, PSMZ24, width, height, test_reg(zte=1, ztst=2),
                 alpha=alpha_reg(0, 1, 0, 1),
                 extra=[(COLCLAMP, 1), (TEX1_1, tex1_reg(mmag=1, mmin=1)), (TEXA, texa_reg(0, 0, 0x80))])
    tex0s, _ = _texture_set(rng, s, tex_base, 4, 7, 7, PSMT8)
    per_pass = np.full(passes, num_triangles // passes)
    per_pass[: num_triangles % passes] += 1
    for p in range(passes):
        fb = fb_a if p % 2 == 0 else fb_b
        other = fb_b if p % 2 == 0 else fb_a
        s.ad([(TEXFLUSH, 0), (FRAME_1, frame_reg(fb, fbw, PSMCT32))])
        per_draw = np.full(draws_per_pass, int(per_pass[p]) // draws_per_pass)
        per_draw[: int(per_pass[p]) % draws_per_pass] += 1
        for d in range(draws_per_pass):
            n = int(per_draw[d])
            if n == 0:
                continue
            kind = rng.uniform()
            x, y = _textured_draw(rng, n, width, height, 1.0, 16.0, 16.0, 4000.0, 0.2)
            z = rng.integers(0, 1 << 24, size=(n, 3), dtype=np.int64)
            rgba = rng.integers(0, 256, size=(n, 3, 4), dtype=np.int64)
            nv = n * 3
            if p > 0 and kind < feedback_frac:
                s.ad([(TEX0_1, tex0_reg(other * BLOCKS_PER_PAGE, fbw, PSMCT32, 9, 8, tcc=1, tfx=0)),
                      (CLAMP_1, clamp_reg(1, 1))])
                u = rng.integers(0, 512 * 16, size=(n, 3), dtype=np.int64)
                v = rng.integers(0, 256 * 16, size=(n, 3), dtype=np.int64)
                q = np.zeros((nv, 3, 2), dtype=np.uint64)
                q[:, 0] = q_uv(u.reshape(nv), v.reshape(nv))
                q[:, 1] = q_rgbaq(rgba.reshape(nv, 4))
                q[:, 2] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
                s.packed(prim_reg(PRIM_TRI, iip=1, tme=1, abe=1, fst=1), [D_UV, D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
            elif kind < 0.6:
                s.ad([(TEX0_1, tex0s[int(rng.integers(0, len(tex0s)))]), (CLAMP_1, clamp_reg(0, 0))])
                sn = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
                tn = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
                qv = np.ones((n, 3), dtype=np.float32)
                q = np.zeros((nv, 3, 2), dtype=np.uint64)
                q[:, 0] = q_st(sn.reshape(nv), tn.reshape(nv), qv.reshape(nv))
                q[:, 1] = q_rgbaq(rgba.reshape(nv, 4))
                q[:, 2] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
                s.packed(prim_reg(PRIM_TRI, iip=1, tme=1), [D_ST, D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
            else:
                q = np.zeros((nv, 2, 2), dtype=np.uint64)
                q[:, 0] = q_rgbaq(rgba.reshape(nv, 4))
                q[:, 1] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
                s.packed(prim_reg(PRIM_TRI, iip=1), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
    return Frame("c4", s.tobytes(), super_sampling, super_sampling != 8, num_triangles,
                 {"width": width, "height": height, "fbp": fb_a, "fb_b": fb_b, "zbp": zbp, "passes": passes})


def _mixed_textures(rng, s: GifStream, base_page: int, page_budget: int):
    """1-4 textures of PSMT4 / PSMT8 / PSMCT32, 64x64 to 512x512, with random CT32
    CLUTs, placed from `base_page` within `page_budget` pages.  Returns TEX0 values."""
    tex0s = []
    page = base_page
    end = base_page + page_budget
    for _ in range(int(rng.integers(1, 5))):
        psm = [PSMT4, PSMT8, PSMCT32][int(rng.integers(0, 3))]
        tw, th = int(rng.integers(6, 10)), int(rng.integers(6, 10))
        w, h = 1 << tw, 1 << th
        bpp = {PSMT4: 4, PSMT8: 8, PSMCT32: 32}[psm]
        # Page geometry (width x height in pixels) per format; TBW in 64-pixel units.
        pw, ph = {PSMT4: (128, 128), PSMT8: (128, 64), PSMCT32: (64, 32)}[psm]
        pages = max(1, -(-w // pw)) * max(1, -(-h // ph))
        clut_pages = 1 if psm != PSMCT32 else 0
        while page + pages + clut_pages > end and (tw > 6 or th > 6):
            if tw >= th:
                tw -= 1
            else:
                th -= 1
            w, h = 1 << tw, 1 << th
            pages = max(1, -(-w // pw)) * max(1, -(-h // ph))
        if page + pages + clut_pages > end:
            break
        tbw = max(1, w // 64)
        if psm in (PSMT4, PSMT8):
            tbw = max(2, tbw + (tbw & 1))
        tbp0 = page * BLOCKS_PER_PAGE
        data = rng.integers(0, 256, size=w * h * bpp // 8, dtype=np.uint8).tobytes()
        s.upload(tbp0, tbw, psm, 0, 0, w, h, data)
        page += pages
        cbp = cpsm = 0
        if psm != PSMCT32:
            cw, ch = (16, 16) if psm == PSMT8 else (8, 2)
            cbp = page * BLOCKS_PER_PAGE
            clut = rng.integers(0, 1 << 32, size=cw * ch, dtype=np.uint64).astype(np.uint32).tobytes()
            s.upload(cbp, 1, PSMCT32, 0, 0, cw, ch, clut)
            page += 1
        tex0s.append(tex0_reg(tbp0, tbw, psm, tw, th, tcc=1, tfx=int(rng.integers(0, 2)), cbp=cbp, cpsm=cpsm,
                              csm=0, csa=0, cld=1 if psm != PSMCT32 else 0))
    return tex0s


def stream_c3(stream_id: int, num_primitives: int | None = None) -> Frame:
    """One of the 64 mixed streams of the batched-replay workload.

    Seeded by the stream id: primitive count log-uniform in 1k-200k, a
    PSMCT16 (+PSMZ16) or PSMCT32 (+PSMZ24) framebuffer from 320x240 to 640x512,
    1-4 PSMT4/PSMT8/PSMCT32 textures of 64x64 to 512x512 with random CLUTs, and
    1x/2x/4x SSAA.  Draws mix perspective-textured triangles, Gouraud
    triangles and sprites with random blend and alpha-test state."""
    rng = np.random.Generator(np.random.PCG64(1000 + stream_id))
    n = int(round(np.exp(rng.uniform(np.log(1000), np.log(200000))))) if num_primitives is None else num_primitives
    fpsm = PSMCT16 if rng.uniform() < 0.5 else PSMCT32
    zpsm = PSMZ16 if fpsm == PSMCT16 else PSMZ24
    width = int(rng.integers(5, 11)) * 64
    height = int(rng.integers(15, 33)) * 16
    ss = [1, 2, 4][int(rng.integers(0, 3))]
    bpp = 2 if fpsm == PSMCT16 else 4
    pw, ph = (64, 64) if fpsm == PSMCT16 else (64, 32)
    fb_pages = -(-width // pw) * -(-height // ph)
    zbp = fb_pages
    tex_base = 2 * fb_pages
    s = GifStream()
    _frame_setup(s, 0, width // 64, fpsm, zbp, zpsm, width, height, test_reg(zte=1, ztst=2),
                 alpha=alpha_reg(0, 1, 0, 1),
                 extra=[(COLCLAMP, 1), (TEX1_1, tex1_reg(mmag=1, mmin=1)), (TEXA, texa_reg(0, 0, 0x80)),
                        (DTHE, int(rng.integers(0, 2))), (DIMX, dimx_reg(DEFAULT_DIMX))])
    tex0s = _mixed_textures(rng, s, tex_base, 512 - tex_base)
    zmax = (1 << (16 if zpsm == PSMZ16 else 24)) - 1
    area_hi = 4000.0 * (width * height) / (640 * 448)
    done = 0
    while done < n:
        m = min(n - done, int(rng.integers(50, 2000)))
        kind = rng.uniform()
        state = [(TEST_1, test_reg(ate=int(rng.uniform() < 0.3), atst=6, aref=int(rng.integers(0, 128)), afail=0,
                                   zte=1, ztst=2))]
        abe = int(rng.uniform() < 0.4)
        if tex0s and kind < 0.7:
            state += [(TEX0_1, tex0s[int(rng.integers(0, len(tex0s)))]), (CLAMP_1, clamp_reg(0, 0))]
        s.ad(state)
        z = rng.integers(0, zmax + 1, size=(m, 3), dtype=np.int64)
        rgba = rng.integers(0, 256, size=(m, 3, 4), dtype=np.int64)
        if kind < 0.6 and tex0s:
            x, y = random_triangles(rng, m, width, height, 4.0, area_hi)
            qv = rng.uniform(0.25, 4.0, size=(m, 3)).astype(np.float32)
            sn = rng.uniform(0.0, 1.0, size=(m, 3)).astype(np.float32)
            tn = rng.uniform(0.0, 1.0, size=(m, 3)).astype(np.float32)
            nv = m * 3
            q = np.zeros((nv, 3, 2), dtype=np.uint64)
            q[:, 0] = q_st((sn * qv).reshape(nv), (tn * qv).reshape(nv), qv.reshape(nv))
            q[:, 1] = q_rgbaq(rgba.reshape(nv, 4))
            q[:, 2] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
            s.packed(prim_reg(PRIM_TRI, iip=1, tme=1, abe=abe), [D_ST, D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
        elif kind < 0.7 and tex0s:
            sx, sy = random_sprites(rng, m, width, height, 4.0, area_hi)
            u = rng.integers(0, 256 * 16, size=(m, 2), dtype=np.int64)
            v = rng.integers(0, 256 * 16, size=(m, 2), dtype=np.int64)
            mv = m * 2
            q = np.zeros((mv, 3, 2), dtype=np.uint64)
            q[:, 0] = q_uv(u.reshape(mv), v.reshape(mv))
            q[:, 1] = q_rgbaq(rgba[:, :2].reshape(mv, 4))
            q[:, 2] = q_xyz2(sx.reshape(mv), sy.reshape(mv), z[:, :2].reshape(mv))
            s.packed(prim_reg(PRIM_SPRITE, iip=1, tme=1, abe=abe, fst=1), [D_UV, D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
        else:
            x, y = random_triangles(rng, m, width, height, 4.0, area_hi)
            nv = m * 3
            q = np.zeros((nv, 2, 2), dtype=np.uint64)
            q[:, 0] = q_rgbaq(rgba.reshape(nv, 4))
            q[:, 1] = q_xyz2(x.reshape(nv), y.reshape(nv), z.reshape(nv))
            s.packed(prim_reg(PRIM_TRI, iip=1, abe=abe), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
        done += m
    return Frame("c3_%02d" % stream_id, s.tobytes(), ss, True, n,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp, "fpsm": fpsm, "stream": stream_id})


def dispfb_reg(fbp, fbw, psm, dbx=0, dby=0) -> int:
    """DISPFB1/2 (gs/gs_registers.hpp:612-621)."""
    return (fbp & 0x1FF) | ((fbw & 0x3F) << 9) | ((psm & 0x1F) << 15) | ((dbx & 0x7FF) << 32) | ((dby & 0x7FF) << 43)


def display_reg(dx, dy, magh, magv, dw, dh) -> int:
    """DISPLAY1/2 (gs/gs_registers.hpp:623-633); dw/dh are the register values (size - 1)."""
    return ((dx & 0xFFF) | ((dy & 0x7FF) << 12) | ((magh & 0xF) << 23) | ((magv & 3) << 27) |
            ((dw & 0xFFF) << 32) | ((dh & 0x7FF) << 44))


def smode2_reg(interlace=0, ffmd=0) -> int:
    return (interlace & 1) | ((ffmd & 1) << 1)



def smode1_reg(cmod=2, lc=32) -> int:
    """SMODE1 (gs/gs_registers.hpp:705-732): CMOD 0 progressive / 2 NTSC / 3 PAL,
    LC 32 analog, 22 HDTV, 15 VGA."""
    return ((lc & 0x7F) << 3) | ((cmod & 3) << 13)


def pmode_reg(en1=1, en2=0, mmod=1, amod=0, slbg=0, alp=0xFF) -> int:
    """PMODE (gs/gs_registers.hpp:562-575)."""
    return en1 | (en2 << 1) | (mmod << 5) | (amod << 6) | (slbg << 7) | ((alp & 0xFF) << 8)


def extbuf_reg(exbp=0, exbw=0, fbin=0, wffmd=0, emoda=0, emodc=0, wdx=0, wdy=0) -> int:
    return ((exbp & 0x3FFF) | ((exbw & 0x3F) << 14) | ((fbin & 3) << 20) | ((wffmd & 1) << 22) |
            ((emoda & 3) << 23) | ((emodc & 3) << 25) | ((wdx & 0x7FF) << 32) | ((wdy & 0x7FF) << 43))


def extdata_reg(sx=0, sy=0, smph=0, smpv=0, ww=0, wh=0) -> int:
    return ((sx & 0xFFF) | ((sy & 0x7FF) << 12) | ((smph & 0xF) << 23) | ((smpv & 3) << 27) |
            ((ww & 0xFFF) << 32) | ((wh & 0x7FF) << 44))


def random_crtc(rng) -> dict:
    """Random privileged-register state for vsync coverage: video mode, both
    circuits (formats, offsets, magnification), PMODE blend modes, BGCOLOR,
    EXTWRITE feedback; returns {priv index: value}."""
    mode = [(2, 32), (3, 32), (0, 32), (0, 15), (0, 22)][int(rng.integers(0, 5))]
    interlace = int(rng.integers(0, 2)) if mode[0] != 0 or mode[1] == 22 else 0
    regs = {0: pmode_reg(en1=int(rng.uniform() < 0.8), en2=int(rng.uniform() < 0.5), mmod=int(rng.integers(0, 2)),
                         slbg=int(rng.integers(0, 2)), alp=int(rng.integers(0, 256)) if rng.uniform() < 0.6 else 0xFF),
            1: smode1_reg(*mode), 2: smode2_reg(interlace, int(rng.integers(0, 2))),
            14: int(rng.integers(0, 1 << 24))}
    for c in range(2):
        psm = [PSMCT32, PSMCT24, PSMCT16, PSMCT16S][int(rng.integers(0, 4))]
        magh = [3, 3, 1, 4, 9][int(rng.integers(0, 5))]
        magv = int(rng.integers(0, 2))
        w = int(rng.integers(64, 641))
        h = int(rng.integers(32, 449))
        regs[7 + 2 * c] = dispfb_reg(int(rng.integers(0, 40)), 10, psm, int(rng.integers(0, 64)), int(rng.integers(0, 64)))
        regs[8 + 2 * c] = display_reg(int(rng.integers(500, 700)), int(rng.integers(20, 60)), magh, magv,
                                      w * (magh + 1) - 1, h * (magv + 1) - 1)
    if rng.uniform() < 0.4:
        regs[13] = 1
        # EXBW wide enough that the written rectangle does not alias itself.
        regs[11] = extbuf_reg(exbp=int(rng.integers(0, 0x3000)), exbw=int(rng.integers(7, 11)),
                              fbin=int(rng.integers(0, 2)), wffmd=int(rng.integers(0, 2)),
                              emoda=int(rng.integers(0, 4)), emodc=int(rng.integers(0, 4)),
                              wdx=int(rng.integers(0, 64)), wdy=int(rng.integers(0, 64)))
        regs[12] = extdata_reg(smph=int(rng.integers(0, 4)), smpv=int(rng.integers(0, 2)),
                               ww=int(rng.integers(16, 320)), wh=int(rng.integers(16, 240)))
    return regs

FUZZ_TEXTURE_PSMS = [PSMT8, PSMT4, PSMT8H, 0x24, 0x2C, PSMCT32, PSMCT24, PSMCT16, PSMCT16S]


def frame_fuzz(seed: int, draws: int = 40, width: int = 256, height: int = 224) -> Frame:
    """Random state coverage: every primitive type, AA1, fog, all blend / alpha
    test / destination alpha / depth test modes, FBMSK, scissor, SCANMSK, XYOFFSET,
    colour formats CT32/CT24/CT16/CT16S with Z32/Z24/Z16/Z16S, textures in PSMT8 /
    PSMT4 / PSMT8H / PSMT4HL / PSMT4HH (CT32 or CT16 CLUTs) and CT32 / CT24 / CT16 /
    CT16S, every wrap mode including region clamp / repeat, TEXA alpha expansion,
    nearest and bilinear filtering; the sampling rate is random too."""
    rng = np.random.Generator(np.random.PCG64(50000 + seed))
    s = GifStream()
    fpsm = [PSMCT32, PSMCT24, PSMCT16, PSMCT16S][int(rng.integers(0, 4))]
    zpsm = [PSMZ32, PSMZ24, PSMZ16, PSMZ16S][int(rng.integers(0, 4))]
    fbw = width // 64
    zbp = 32
    ss, ordered = [(1, True), (2, True), (4, True), (4, False), (8, True), (16, True), (16, False)][int(rng.integers(0, 7))]
    s.ad([(PRMODECONT, 1), (FRAME_1, frame_reg(0, fbw, fpsm)), (ZBUF_1, zbuf_reg(zbp, zpsm)),
          (SCISSOR_1, scissor_reg(0, width - 1, 0, height - 1)), (XYOFFSET_1, 0), (COLCLAMP, 1),
          (DIMX, dimx_reg(DEFAULT_DIMX))])
    # Textures from page 64 on.
    texs = []
    page = 64
    for psm in FUZZ_TEXTURE_PSMS:
        tw, th = int(rng.integers(4, 8)), int(rng.integers(4, 8))
        w, h = 1 << tw, 1 << th
        bpp = {PSMT8: 8, PSMT4: 4, PSMT8H: 32, 0x24: 32, 0x2C: 32, PSMCT32: 32, PSMCT24: 24, PSMCT16: 16,
               PSMCT16S: 16}[psm]
        tbw = max(2, w // 64) if psm in (PSMT8, PSMT4) else max(1, w // 64)
        data = rng.integers(0, 256, size=w * h * bpp // 8, dtype=np.uint8).tobytes()
        tbp0 = page * BLOCKS_PER_PAGE
        s.upload(tbp0, tbw, psm, 0, 0, w, h, data)
        page += 10
        cpsm = cbp = cld = csa = 0
        if psm in (PSMT8, PSMT4, PSMT8H, 0x24, 0x2C):
            cpsm = PSMCT32 if rng.uniform() < 0.5 else PSMCT16
            n = 256 if psm in (PSMT8, PSMT8H) else 16
            cw, ch = (16, 16) if n == 256 else (8, 2)
            cbp = page * BLOCKS_PER_PAGE
            cbytes = 4 if cpsm == PSMCT32 else 2
            clut = rng.integers(0, 256, size=cw * ch * cbytes, dtype=np.uint8).tobytes()
            s.upload(cbp, 1, cpsm, 0, 0, cw, ch, clut)
            page += 1
            cld = 1
            csa = int(rng.integers(0, 16)) if (n == 16 and cpsm == PSMCT16) else 0
        texs.append((psm, tbp0, tbw, tw, th, cbp, cpsm, csa, cld, w, h))
    zmax = {PSMZ32: (1 << 32) - 1, PSMZ24: (1 << 24) - 1, PSMZ16: 0xFFFF, PSMZ16S: 0xFFFF}[zpsm]
    for d in range(draws):
        prim = int(rng.integers(0, 7))
        tme = int(rng.uniform() < 0.5)
        fst = int(tme and rng.uniform() < 0.5)
        fge = int(rng.uniform() < 0.2)
        abe = int(rng.uniform() < 0.4)
        aa1 = int(rng.uniform() < 0.15)
        iip = int(rng.uniform() < 0.8)
        regs = [(TEST_1, test_reg(ate=int(rng.uniform() < 0.3), atst=int(rng.integers(0, 8)),
                                  aref=int(rng.integers(0, 256)), afail=int(rng.integers(0, 4)),
                                  date=int(rng.uniform() < 0.15), datm=int(rng.integers(0, 2)),
                                  zte=1, ztst=int(rng.integers(1, 4)))),
                (ALPHA_1, alpha_reg(int(rng.integers(0, 3)), int(rng.integers(0, 3)), int(rng.integers(0, 3)),
                                    int(rng.integers(0, 3)), int(rng.integers(0, 256)))),
                (FBA_1, int(rng.uniform() < 0.2)), (DTHE, int(rng.uniform() < 0.3)),
                (COLCLAMP, int(rng.uniform() < 0.7)), (PABE, int(rng.uniform() < 0.2)),
                (FOGCOL, int(rng.integers(0, 1 << 24))),
                (SCANMSK, [0, 0, 0, 2, 3][int(rng.integers(0, 5))]),
                (TEXA, texa_reg(int(rng.integers(0, 256)), int(rng.integers(0, 2)), int(rng.integers(0, 256))))]
        if rng.uniform() < 0.3:
            x0, y0 = int(rng.integers(0, width // 2)), int(rng.integers(0, height // 2))
            regs.append((SCISSOR_1, scissor_reg(x0, int(rng.integers(x0, width)), y0, int(rng.integers(y0, height)))))
        else:
            regs.append((SCISSOR_1, scissor_reg(0, width - 1, 0, height - 1)))
        fbmsk = 0 if rng.uniform() < 0.7 else int(rng.integers(0, 1 << 32, dtype=np.uint64))
        regs.append((FRAME_1, frame_reg(0, fbw, fpsm, fbmsk)))
        regs.append((ZBUF_1, zbuf_reg(zbp, zpsm, int(rng.uniform() < 0.2))))
        if tme:
            psm, tbp0, tbw, tw, th, cbp, cpsm, csa, cld, w, h = texs[int(rng.integers(0, len(texs)))]
            regs.append((TEX0_1, tex0_reg(tbp0, tbw, psm, tw, th, tcc=int(rng.integers(0, 2)),
                                          tfx=int(rng.integers(0, 4)), cbp=cbp, cpsm=cpsm, csm=0, csa=csa, cld=cld)))
            regs.append((TEX1_1, tex1_reg(mmag=int(rng.integers(0, 2)), mmin=int(rng.integers(0, 2)))))
            wm = [int(rng.integers(0, 4)), int(rng.integers(0, 4))]
            lo_u, lo_v = int(rng.integers(0, w)), int(rng.integers(0, h))
            regs.append((CLAMP_1, clamp_reg(wm[0], wm[1], lo_u, int(rng.integers(lo_u, w)) if wm[0] == 2 else
                                            int(rng.integers(0, w)), lo_v,
                                            int(rng.integers(lo_v, h)) if wm[1] == 2 else int(rng.integers(0, h)))))
        s.ad(regs)
        s.ad([(PRIM, prim_reg(prim, iip=iip, tme=tme, fge=fge, abe=abe, aa1=aa1, fst=fst))])
        nv = int(rng.integers(3, 48))
        x = np.round(rng.uniform(-16, width + 16, nv) * 16).astype(np.int64) & 0xFFFF
        y = np.round(rng.uniform(-16, height + 16, nv) * 16).astype(np.int64) & 0xFFFF
        z = rng.integers(0, min(zmax, (1 << 32) - 1) + 1, nv, dtype=np.uint64).astype(np.int64)
        rgba = rng.integers(0, 256, size=(nv, 4), dtype=np.int64)
        desc = [D_RGBAQ]
        q = [q_rgbaq(rgba)]
        if tme and fst:
            desc.append(D_UV)
            q.append(q_uv(rng.integers(0, 256 * 16, nv), rng.integers(0, 256 * 16, nv)))
        elif tme:
            qq = rng.uniform(0.5, 2.0, nv).astype(np.float32)
            desc.append(D_ST)
            q.append(q_st((rng.uniform(-0.25, 1.25, nv) * qq).astype(np.float32),
                          (rng.uniform(-0.25, 1.25, nv) * qq).astype(np.float32), qq))
        if fge:
            desc.append(D_XYZF2)
            fog = rng.integers(0, 256, nv, dtype=np.uint64)
            lo = (x.astype(np.uint64) | (y.astype(np.uint64) << np.uint64(32)))
            hi = ((z.astype(np.uint64) & np.uint64(0xFFFFFF)) << np.uint64(4)) | (fog << np.uint64(36))
            q.append(np.stack([lo, hi], axis=1))
        else:
            desc.append(D_XYZ2)
            q.append(q_xyz2(x, y, z))
        data = np.stack(q, axis=1).reshape(-1, 2)
        s.packed(prim_reg(prim, iip=iip, tme=tme, fge=fge, abe=abe, aa1=aa1, fst=fst), desc, data)
    return Frame("fuzz_%d" % seed, s.tobytes(), ss, ordered, draws,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp})


MIPTBP1_1, MIPTBP2_1 = 0x34, 0x36


def miptbp_reg(levels: list[tuple[int, int]]) -> int:
    """MIPTBP1 / MIPTBP2 payload from up to three (TBP, TBW) pairs."""
    v = 0
    for i, (tbp, tbw) in enumerate(levels):
        v |= (tbp & 0x3FFF) << (20 * i) | (tbw & 0x3F) << (20 * i + 14)
    return v


# Page size in pixels (width, height) per format, for laying out mip levels.
_PAGE_DIMS = {PSMCT32: (64, 32), PSMCT16: (64, 64), PSMT8: (128, 64), PSMT4: (128, 128)}
_BLOCK_LOG2 = {PSMCT32: (3, 3), PSMCT16: (4, 3), PSMT8: (4, 4), PSMT4: (5, 4)}


def frame_mip(seed: int, draws: int = 30, width: int = 256, height: int = 224) -> Frame:
    """Mipmapping coverage: mip chains of 2-7 levels in CT32 / CT16 / PSMT8 /
    PSMT4 (CLUT) with level bases from MIPTBP1 / MIPTBP2 or generated by
    TEX1.MTBA; draws with every MMIN mode, MMAG, MXL (also past the chain), L,
    signed K, fixed LOD (LCM), perspective STQ with Q over [1/16, 16] and UV
    addressing, all wrap modes; random sampling rate."""
    rng = np.random.Generator(np.random.PCG64(70000 + seed))
    s = GifStream()
    fpsm = [PSMCT32, PSMCT16][int(rng.integers(0, 2))]
    zpsm = PSMZ24
    fbw = width // 64
    zbp = 32
    ss, ordered = [(1, True), (2, True), (4, True), (4, False), (8, True), (16, True)][int(rng.integers(0, 6))]
    s.ad([(PRMODECONT, 1), (FRAME_1, frame_reg(0, fbw, fpsm)), (ZBUF_1, zbuf_reg(zbp, zpsm)),
          (SCISSOR_1, scissor_reg(0, width - 1, 0, height - 1)), (XYOFFSET_1, 0), (COLCLAMP, 1)])
    texs = []
    page = 64
    for ti in range(4):
        psm = [PSMCT32, PSMCT16, PSMT8, PSMT4][ti]
        auto = ti < 3 and rng.uniform() < 0.5
        tw = 8 if auto else int(rng.integers(2, 9))
        th = int(rng.integers(6, 9)) if auto else int(rng.integers(2, 9))
        bpp = {PSMCT32: 32, PSMCT16: 16, PSMT8: 8, PSMT4: 4}[psm]
        nlev = min(tw, th) + 1
        levels = []
        if auto:
            # TEX1.MTBA layout (gs/gs_interface.cpp:805-843): levels 1-3 follow
            # level 0 block by block, the buffer width halving each level.
            bwl, bhl = _BLOCK_LOG2[psm]
            base = page * BLOCKS_PER_PAGE
            row = (1 << tw) // 64
            blocks = ((1 << tw) >> bwl) * ((1 << th) >> bhl)
            for lv in range(min(nlev, 4)):
                levels.append((base, row))
                base += blocks
                blocks //= 4
                row //= 2
            page = (base + BLOCKS_PER_PAGE - 1) // BLOCKS_PER_PAGE + 1
            nlev = len(levels)
        else:
            pw, ph = _PAGE_DIMS[psm]
            for lv in range(min(nlev, 7)):
                wl, hl = (1 << tw) >> lv, (1 << th) >> lv
                tbw = max(1, wl // 64)
                if psm in (PSMT8, PSMT4):
                    tbw = max(2, tbw)
                levels.append((page * BLOCKS_PER_PAGE, tbw))
                page += max(1, (tbw * 64 + pw - 1) // pw) * ((hl + ph - 1) // ph)
        for lv, (tbp, tbw) in enumerate(levels):
            wl, hl = (1 << tw) >> lv, (1 << th) >> lv
            data = rng.integers(0, 256, size=max(16, wl * hl * bpp // 8), dtype=np.uint8).tobytes()
            s.upload(tbp, tbw, psm, 0, 0, wl, hl, data[:max(1, wl * hl * bpp // 8)])
        cpsm = cbp = cld = 0
        if psm in (PSMT8, PSMT4):
            cpsm = PSMCT32 if rng.uniform() < 0.5 else PSMCT16
            cw, ch = (16, 16) if psm == PSMT8 else (8, 2)
            cbp = page * BLOCKS_PER_PAGE
            clut = rng.integers(0, 256, size=cw * ch * (4 if cpsm == PSMCT32 else 2), dtype=np.uint8).tobytes()
            s.upload(cbp, 1, cpsm, 0, 0, cw, ch, clut)
            page += 1
            cld = 1
        texs.append((psm, tw, th, levels, auto, cbp, cpsm, cld))
    assert page * PAGE_BYTES <= 4 * 1024 * 1024
    for d in range(draws):
        psm, tw, th, levels, auto, cbp, cpsm, cld = texs[int(rng.integers(0, len(texs)))]
        w, h = 1 << tw, 1 << th
        lcm = int(rng.uniform() < 0.25)
        k = int(rng.integers(-32, 113)) if lcm else int(rng.integers(-96, 97))
        tex1 = tex1_reg(lcm=lcm, mxl=int(rng.integers(0, 8)), mmag=int(rng.integers(0, 2)),
                        mmin=int(rng.integers(0, 6)), mtba=int(auto), l=int(rng.integers(0, 4)), k=k & 0xFFF)
        regs = [(TEST_1, test_reg(zte=1, ztst=1)), (ALPHA_1, alpha_reg(0, 1, 0, 1)),
                (TEX1_1, tex1)]
        if not auto:
            regs.append((MIPTBP1_1, miptbp_reg(levels[1:4])))
            regs.append((MIPTBP2_1, miptbp_reg(levels[4:7])))
        regs.append((TEX0_1, tex0_reg(levels[0][0], levels[0][1], psm, tw, th, tcc=1, tfx=int(rng.integers(0, 2)),
                                      cbp=cbp, cpsm=cpsm, cld=cld)))
        wm = [int(rng.integers(0, 4)), int(rng.integers(0, 4))]
        lo_u, lo_v = int(rng.integers(0, w)), int(rng.integers(0, h))
        regs.append((CLAMP_1, clamp_reg(wm[0], wm[1], lo_u, int(rng.integers(lo_u, w)) if wm[0] == 2 else
                                        int(rng.integers(0, w)), lo_v,
                                        int(rng.integers(lo_v, h)) if wm[1] == 2 else int(rng.integers(0, h)))))
        s.ad(regs)
        prim = [PRIM_TRI, PRIM_TRISTRIP, PRIM_SPRITE][int(rng.integers(0, 3))]
        fst = int(rng.uniform() < 0.3)
        nv = int(rng.integers(3, 24)) if prim != PRIM_SPRITE else 2 * int(rng.integers(1, 8))
        x = np.round(rng.uniform(-16, width + 16, nv) * 16).astype(np.int64) & 0xFFFF
        y = np.round(rng.uniform(-16, height + 16, nv) * 16).astype(np.int64) & 0xFFFF
        z = rng.integers(0, 1 << 24, nv, dtype=np.int64)
        rgba = rng.integers(0, 256, size=(nv, 4), dtype=np.int64)
        desc = [D_RGBAQ]
        q = [q_rgbaq(rgba)]
        if fst:
            desc.append(D_UV)
            q.append(q_uv(rng.integers(0, 4 * w * 16, nv) - w * 16 // 2 & 0x3FFF,
                          rng.integers(0, 4 * h * 16, nv) - h * 16 // 2 & 0x3FFF))
        else:
            qq = np.exp2(rng.uniform(-4, 4, nv)).astype(np.float32)
            if rng.uniform() < 0.3:
                qq[:] = qq[0]
            desc.append(D_ST)
            q.append(q_st((rng.uniform(-0.5, 1.5, nv) * qq).astype(np.float32),
                          (rng.uniform(-0.5, 1.5, nv) * qq).astype(np.float32), qq))
        desc.append(D_XYZ2)
        q.append(q_xyz2(x, y, z))
        data = np.stack(q, axis=1).reshape(-1, 2)
        s.packed(prim_reg(prim, iip=1, tme=1, fst=fst, abe=int(rng.uniform() < 0.3)), desc, data)
    return Frame("mip_%d" % seed, s.tobytes(), ss, ordered, draws,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp})



def frame_alias(seed: int, width: int = 256, height: int = 128) -> Frame:
    """Frame and depth buffer at the same base page (the Z-swizzle tricks that
    read colour as depth): draws without depth first, then small depth-writing
    primitives (each inside one 8x8 block, so no primitive reads depth that it
    also writes as colour elsewhere), then depth-tested sprites and triangles
    reading the aliased depth, some overlapping earlier sprites."""
    rng = np.random.Generator(np.random.PCG64(80000 + seed))
    s = GifStream()
    fpsm, zpsm = [(PSMCT32, PSMZ32), (PSMCT32, PSMZ24), (PSMCT24, PSMZ24), (PSMCT16, PSMZ16)][int(rng.integers(0, 4))]
    ss = [1, 2, 4][int(rng.integers(0, 3))]
    fbw = width // 64
    s.ad([(PRMODECONT, 1), (FRAME_1, frame_reg(0, fbw, fpsm)), (ZBUF_1, zbuf_reg(0, zpsm)),
          (SCISSOR_1, scissor_reg(0, width - 1, 0, height - 1)), (XYOFFSET_1, 0), (COLCLAMP, 1)])

    def sprites(n, lo, hi, z_test, z_write, abe=0):
        x0 = rng.integers(0, width - 8, n)
        y0 = rng.integers(0, height - 8, n)
        w = rng.integers(lo, hi + 1, n)
        h = rng.integers(lo, hi + 1, n)
        x = np.stack([x0, np.minimum(x0 + w, width)], 1).reshape(-1) * 16
        y = np.stack([y0, np.minimum(y0 + h, height)], 1).reshape(-1) * 16
        z = rng.integers(0, 1 << 24, 2 * n)
        col = rng.integers(0, 256, (2 * n, 4))
        s.ad([(TEST_1, test_reg(zte=1, ztst=[1, 2, 3][int(rng.integers(0, 3))] if z_test else 1)),
              (ZBUF_1, zbuf_reg(0, zpsm, 0 if z_write else 1)), (ALPHA_1, alpha_reg(0, 1, 0, 1))])
        q = np.zeros((2 * n, 2, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(col)
        q[:, 1] = q_xyz2(x, y, z)
        s.packed(prim_reg(PRIM_SPRITE, abe=abe), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))

    def block_sprites(n):
        # Depth-writing sprites inside one 8x8 block each.
        bx = rng.integers(0, width // 8, n) * 8
        by = rng.integers(0, height // 8, n) * 8
        ox = rng.integers(0, 4, n)
        oy = rng.integers(0, 4, n)
        w = rng.integers(1, 5, n)
        h = rng.integers(1, 5, n)
        x = np.stack([bx + ox, bx + ox + w], 1).reshape(-1) * 16
        y = np.stack([by + oy, by + oy + h], 1).reshape(-1) * 16
        z = rng.integers(0, 1 << 24, 2 * n)
        col = rng.integers(0, 256, (2 * n, 4))
        s.ad([(TEST_1, test_reg(zte=1, ztst=[1, 2][int(rng.integers(0, 2))])), (ZBUF_1, zbuf_reg(0, zpsm, 0))])
        q = np.zeros((2 * n, 2, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(col)
        q[:, 1] = q_xyz2(x, y, z)
        s.packed(prim_reg(PRIM_SPRITE), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))

    sprites(int(rng.integers(5, 30)), 4, 64, z_test=False, z_write=False)
    if rng.uniform() < 0.7:
        block_sprites(int(rng.integers(5, 60)))
    for _ in range(int(rng.integers(1, 4))):
        sprites(int(rng.integers(5, 30)), 4, 96, z_test=True, z_write=False, abe=int(rng.integers(0, 2)))
    return Frame("alias_%d" % seed, s.tobytes(), ss, True, 0, {"width": width, "height": height, "fbp": 0, "zbp": 0})


def frame_ssaa_textures(seed: int) -> Frame:
    """Super-sampled textures: a super-sampled 3D pass into an off-screen
    buffer, then sprites that sample it (its pages were written by a pass):
    nearest and bilinear, 1:1 blits, downsamples, upsamples and in-between
    scales, perspective and UV addressing, CT32 / CT16 / PSMT8 views with region
    clamp and repeat, blur-like groups of a few sprites at different phases
    (ABE Cs * As + Cd), and enough sprites in some passes that the blur
    heuristic stays off.  Needs set_super_sampled_textures."""
    rng = np.random.Generator(np.random.PCG64(90000 + seed))
    s = GifStream()
    ss = [2, 4, 8, 16][seed % 4]
    ordered = bool(rng.uniform() < 0.7)
    ow, oh = 256, 128                       # off-screen buffer at page 0
    width, height = 320, 224                # final frame at page 100
    zbp, fin = 60, 100
    _frame_setup(s, 0, ow // 64, PSMCT32, zbp, PSMZ24, ow, oh, test_reg(zte=1, ztst=2))
    n = 300
    x, y = random_triangles(rng, n, ow, oh, 4.0, 1500.0)
    z = rng.integers(0, 1 << 24, size=(n, 3))
    rgba = rng.integers(0, 256, size=(3 * n, 4))
    q = np.zeros((3 * n, 2, 2), dtype=np.uint64)
    q[:, 0] = q_rgbaq(rgba)
    q[:, 1] = q_xyz2(x.reshape(-1), y.reshape(-1), z.reshape(-1))
    s.packed(prim_reg(PRIM_TRI, iip=1), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
    # Final frame; each group samples the off-screen buffer.
    s.ad([(FRAME_1, frame_reg(fin, width // 64, PSMCT32)), (SCISSOR_1, scissor_reg(0, width - 1, 0, height - 1)),
          (TEST_1, test_reg(zte=1, ztst=1)), (ZBUF_1, zbuf_reg(zbp, PSMZ24, 1))])
    clut_cbp = 200 * BLOCKS_PER_PAGE
    clut = rng.integers(0, 256, size=16 * 16 * 4, dtype=np.uint8).tobytes()
    s.upload(clut_cbp, 1, PSMCT32, 0, 0, 16, 16, clut)
    few = seed % 2 == 0  # at most 64 sprites: the blur heuristic is live
    for g in range(int(rng.integers(3, 6)) if few else int(rng.integers(6, 12))):
        view = [PSMCT32, PSMCT32, PSMCT16, PSMT8][int(rng.integers(0, 4))]
        mmag = int(rng.integers(0, 2))
        fst = int(rng.uniform() < 0.7)
        blur = rng.uniform() < (0.6 if few else 0.3)
        nspr = int(rng.integers(2, 6)) if blur else int(rng.integers(2, 6) if few else rng.integers(3, 40))
        wm = [int(rng.integers(0, 4)), int(rng.integers(0, 4))]
        regs = [(TEX0_1, tex0_reg(0, ow // 64, view, 8, 7, tcc=1, tfx=1, cbp=clut_cbp, cpsm=PSMCT32,
                                  cld=1 if view == PSMT8 else 0)),
                (TEX1_1, tex1_reg(mmag=mmag, mmin=mmag)),
                (CLAMP_1, clamp_reg(wm[0], wm[1], int(rng.integers(0, 64)), int(rng.integers(64, 255)),
                                    int(rng.integers(0, 32)), int(rng.integers(32, 127)))),
                (ALPHA_1, alpha_reg(0, 2, 0, 1) if blur else alpha_reg(0, 1, 0, 1))]
        s.ad(regs)
        scale = [1.0, 1.0, 0.5, 2.0, 0.75, 1.5, 3.0][int(rng.integers(0, 7))]
        pts, uvs, stq = [], [], []
        for k in range(nspr):
            w = int(rng.integers(8, 96))
            h = int(rng.integers(8, 64))
            x0 = int(rng.integers(0, width - w))
            y0 = int(rng.integers(0, height - h))
            u0 = int(rng.integers(0, ow - 8)) * 16 + (int(rng.integers(0, 16)) if not blur else k * 4)
            v0 = int(rng.integers(0, oh - 8)) * 16 + (int(rng.integers(0, 16)) if not blur else k * 2)
            pts += [(x0 * 16, y0 * 16), ((x0 + w) * 16, (y0 + h) * 16)]
            uvs += [(u0, v0), (u0 + int(w * scale * 16), v0 + int(h * scale * 16))]
        nv = len(pts)
        xs = np.array([p_[0] for p_ in pts], dtype=np.int64)
        ys = np.array([p_[1] for p_ in pts], dtype=np.int64)
        col = rng.integers(0, 256, size=(nv, 4))
        col[:, 3] = 0x80
        q = np.zeros((nv, 3, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(col)
        if fst:
            q[:, 1] = q_uv(np.array([u for u, _ in uvs]) & 0x3FFF, np.array([v for _, v in uvs]) & 0x3FFF)
            desc = [D_RGBAQ, D_UV, D_XYZ2]
        else:
            qq = np.full(nv, float(rng.uniform(0.5, 2.0)), dtype=np.float32)
            q[:, 1] = q_st(np.array([u / 16.0 / ow for u, _ in uvs], dtype=np.float32) * qq,
                           np.array([v / 16.0 / 128.0 for _, v in uvs], dtype=np.float32) * qq, qq)
            desc = [D_RGBAQ, D_ST, D_XYZ2]
        q[:, 2] = q_xyz2(xs, ys, np.zeros(nv, dtype=np.int64))
        s.packed(prim_reg(PRIM_SPRITE, tme=1, fst=fst, abe=1), desc, q.reshape(-1, 2))
    return Frame("ssaa_tex_%d" % seed, s.tobytes(), ss, ordered, n,
                 {"width": width, "height": height, "fbp": fin, "zbp": zbp, "ssaa_textures": True})

def frame_field_aware(seed: int) -> Frame:
    """Field-aware rendering: a frame drawn after a high-resolution vsync of
    field-rendered interlaced output.  Even seeds: the super-sampled texture
    scene (blur groups take the FORCE_LINEAR_SUPER_SAMPLE path), with or
    without super-sampled textures; odd seeds: the textured 3D scene at
    320 x 224 (instances that may be fields) or 640 x 448 (too tall to be)."""
    if seed % 2 == 0:
        f = frame_ssaa_textures(seed)
        f.meta["ssaa_textures"] = seed % 4 == 0
    else:
        tall = seed % 4 == 3
        f = frame_c2(seed=seed, num_triangles=600, num_sprites=60, super_sampling=[2, 4, 8, 16][(seed // 2) % 4],
                     num_textures=2, width=640 if tall else 320, height=448 if tall else 224)
    f.meta["field_aware"] = True
    f.name = "field_aware_%d" % seed
    return f


def frame_quads(seed: int) -> Frame:
    """Rectangles drawn as triangle pairs (the frontend fuses them into
    parallelograms): flat colour, FST UV and perspective STQ textures, both
    diagonals, every vertex order, triangle lists and strips, super-sampled for
    odd seeds; some pairs broken by a register change, a Z or colour
    difference or a non-rectangular second triangle."""
    rng = np.random.Generator(np.random.PCG64(92000 + seed))
    s = GifStream()
    ss = 1 if seed % 2 == 0 else [2, 4, 8, 16][(seed // 2) % 4]
    width, height, zbp = 320, 224, 60
    _frame_setup(s, 0, width // 64, PSMCT32, zbp, PSMZ24, width, height, test_reg(zte=1, ztst=1))
    s.upload(200 * BLOCKS_PER_PAGE, 1, PSMCT32, 0, 0, 64, 64, rng.integers(0, 256, size=64 * 64 * 4,
                                                                                  dtype=np.uint8).tobytes())
    s.ad([(TEX0_1, tex0_reg(200 * BLOCKS_PER_PAGE, 1, PSMCT32, 6, 6, tcc=1, tfx=1)),
          (TEX1_1, tex1_reg(mmag=int(seed % 3 == 0), mmin=int(seed % 3 == 0))), (CLAMP_1, clamp_reg(0, 0))])
    for k in range(int(rng.integers(60, 140))):
        w, h = int(rng.integers(1, 80)), int(rng.integers(1, 60))
        x0, y0 = int(rng.integers(0, width - w)), int(rng.integers(0, height - h))
        sub = rng.integers(0, 16, size=2) if rng.uniform() < 0.3 else np.zeros(2, dtype=np.int64)
        X = [x0 * 16 + int(sub[0]), (x0 + w) * 16 + int(sub[0])]
        Y = [y0 * 16 + int(sub[1]), (y0 + h) * 16 + int(sub[1])]
        corners = [(X[0], Y[0]), (X[1], Y[0]), (X[1], Y[1]), (X[0], Y[1])]
        u0, v0 = int(rng.integers(0, 32)) * 16, int(rng.integers(0, 32)) * 16
        du, dv = int(rng.integers(1, 40)) * 16, int(rng.integers(1, 40)) * 16
        uvs = [(u0, v0), (u0 + du, v0), (u0 + du, v0 + dv), (u0, v0 + dv)]
        diag = int(rng.integers(0, 2))
        tri = [[0, 1, 2], [0, 2, 3]] if diag == 0 else [[0, 1, 3], [1, 2, 3]]
        tri = [[t[i] for i in rng.permutation(3)] for t in tri]
        z = int(rng.integers(0, 1 << 24))
        col = [int(c) for c in rng.integers(0, 256, size=4)]
        break_kind = int(rng.integers(0, 8))
        kind = int(rng.integers(0, 3))   # 0 flat, 1 FST UV, 2 STQ
        strip = break_kind == 7 and kind != 2
        verts = []
        for t_i, t in enumerate(tri):
            for c in t:
                zz = z + (1 if break_kind == 1 and t_i == 1 else 0)
                cc = list(col)
                if break_kind == 2 and t_i == 1:
                    cc[0] ^= 1
                x, y = corners[c]
                if break_kind == 3 and t_i == 1 and c == t[0]:
                    x += 16
                verts.append((x, y, zz, cc, uvs[c]))
        if strip:
            # Strip order: a, b, c then d completing the rectangle.
            a, b, c, d = [0, 1, 3, 2] if diag == 0 else [1, 2, 0, 3]
            verts = [(corners[i][0], corners[i][1], z, col, uvs[i]) for i in (a, b, c, d)]
        n = len(verts)
        q = np.zeros((n, 3, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(np.array([v[3] for v in verts]))
        if kind == 2:
            qq = np.full(n, float(rng.uniform(0.5, 2.0)), dtype=np.float32)
            q[:, 1] = q_st(np.array([v[4][0] / 16.0 / 64 for v in verts], dtype=np.float32) * qq,
                           np.array([v[4][1] / 16.0 / 64 for v in verts], dtype=np.float32) * qq, qq)
            desc = [D_RGBAQ, D_ST, D_XYZ2]
        else:
            q[:, 1] = q_uv(np.array([v[4][0] for v in verts]), np.array([v[4][1] for v in verts]))
            desc = [D_RGBAQ, D_UV, D_XYZ2]
        q[:, 2] = q_xyz2(np.array([v[0] for v in verts]), np.array([v[1] for v in verts]),
                         np.array([v[2] for v in verts]))
        prim = PRIM_TRISTRIP if strip else PRIM_TRI
        if break_kind == 4:
            # A state change between the halves keeps them apart.
            s.packed(prim_reg(prim, tme=int(kind > 0), fst=int(kind == 1)), desc, q[:3].reshape(-1, 2))
            s.ad([(FOGCOL, int(rng.integers(0, 1 << 24)))])
            s.packed(prim_reg(prim, tme=int(kind > 0), fst=int(kind == 1)), desc, q[3:].reshape(-1, 2))
        else:
            s.packed(prim_reg(prim, tme=int(kind > 0), fst=int(kind == 1), abe=int(k % 5 == 0)), desc,
                     q.reshape(-1, 2))
    return Frame("quads_%d" % seed, s.tobytes(), ss, True, 0,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp})


def frame_blend_demote(seed: int) -> Frame:
    """Blend demotion hack: many overlapping blended triangles and sprites
    (well over 32 per coarse tile), super-sampled, depth written only in the
    left 96 columns so that tiles on the right qualify; odd seeds add one
    unblended sprite, which turns demotion off for the pass."""
    rng = np.random.Generator(np.random.PCG64(91000 + seed))
    s = GifStream()
    ss = [2, 4, 8, 16][seed % 4]
    width, height, zbp = 256, 224, 60
    _frame_setup(s, 0, width // 64, PSMCT32, zbp, PSMZ24, width, height, test_reg(zte=1, ztst=1))
    for p_ in range(3):
        zmsk = int(p_ != 1)
        s.ad([(ZBUF_1, zbuf_reg(zbp, PSMZ24, zmsk)), (TEST_1, test_reg(zte=1, ztst=[1, 2, 1][p_])),
              (ALPHA_1, alpha_reg(0, 1, 0, 1))])
        n = int(rng.integers(40, 120))
        x, y = random_triangles(rng, n, 96 if p_ == 1 else width, height, 200.0, 30000.0)
        z = rng.integers(0, 1 << 24, size=(n, 3))
        rgba = rng.integers(0, 256, size=(3 * n, 4))
        q = np.zeros((3 * n, 2, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(rgba)
        q[:, 1] = q_xyz2(x.reshape(-1), y.reshape(-1), z.reshape(-1))
        s.packed(prim_reg(PRIM_TRI, iip=1, abe=1), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
        if p_ == 1:
            continue
        m = int(rng.integers(20, 60))
        xs, ys = random_sprites(rng, m, width, height, 400.0, 20000.0)
        col = rng.integers(0, 256, size=(2 * m, 4))
        q = np.zeros((2 * m, 2, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(col)
        q[:, 1] = q_xyz2(xs.reshape(-1), ys.reshape(-1), rng.integers(0, 1 << 24, size=2 * m))
        s.packed(prim_reg(PRIM_SPRITE, abe=1), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
    if seed % 2 == 1:
        q = np.zeros((2, 2, 2), dtype=np.uint64)
        q[:, 0] = q_rgbaq(np.array([[255, 0, 0, 128]] * 2))
        q[:, 1] = q_xyz2(np.array([16 * 16, 48 * 16]), np.array([16 * 16, 40 * 16]), np.array([5, 5]))
        s.packed(prim_reg(PRIM_SPRITE), [D_RGBAQ, D_XYZ2], q.reshape(-1, 2))
    return Frame("blend_demote_%d" % seed, s.tobytes(), ss, True, 0,
                 {"width": width, "height": height, "fbp": 0, "zbp": zbp, "hacks": {"allow_blend_demote": True}})


def write_dump(path, transfers, vram: bytes | None = None, regs: dict | None = None, version: int = 9,
               serial: bytes = b"", vsync_fields=(0,)) -> None:
    """Writes a GS dump in the PCSX2 / GSdx layout (GSDumpGenerator::init,
    dump/gs_dump_generator.cpp:186-237): fake CRC, header (+ serial bytes), the
    register block in its fixed order, VRAM, four GIF paths, internal Q and the
    privileged registers; then one transfer packet per entry of `transfers`
    ((path, bytes) pairs) followed by a vsync packet per field."""
    regs = regs or {}
    vram = vram if vram is not None else bytes(4 * 1024 * 1024)
    out = bytearray()
    u32 = lambda v: struct.pack("<I", v & 0xFFFFFFFF)
    u64 = lambda v: struct.pack("<Q", v & 0xFFFFFFFFFFFFFFFF)
    out += u32(0xFFFFFFFF)
    header = [version, len(vram) + (18 + 24) * 8 + 7 * 4 + 80 + 4, 36, len(serial), 0, 0, 0, 0, 0]
    out += u32(36 + len(serial))
    out += b"".join(u32(v) for v in header) + serial
    out += u32(version)
    for r in (PRIM, PRMODECONT, TEXCLUT, SCANMSK, TEXA, FOGCOL, DIMX, DTHE, COLCLAMP, PABE, BITBLTBUF, TRXDIR,
              TRXPOS, TRXREG):
        out += u64(regs.get(r, 0))
    out += u64(0)
    for ctx in range(2):
        for r in (XYOFFSET_1, TEX0_1, TEX1_1, CLAMP_1, 0x34, 0x36, SCISSOR_1, ALPHA_1, TEST_1, FBA_1, FRAME_1,
                  ZBUF_1):
            out += u64(regs.get(r + ctx, 0))
    out += u64(regs.get(RGBAQ, 0)) + u64(regs.get(ST, 0)) + u32(regs.get(UV, 0)) + u32(regs.get(FOG, 0))
    out += u64(0) + u32(0xFFFFFFFF) + u32(0xFFFFFFFF) + u32(0) + u32(0)
    if version >= 9:
        out += bytes(61)
    out += vram
    for _ in range(4):
        out += u64(0) + u64(0) + u32(0)
    out += struct.pack("<f", 1.0)
    out += bytes(2 * 0x200 * 8)
    for p, data in transfers:
        out += bytes([0, p]) + u32(len(data)) + data
    for f in vsync_fields:
        out += bytes([1, f])
    with open(path, "wb") as fh:
        fh.write(bytes(out))


def frame_hazards(seed: int, ops: int = 60, width: int = 256, height: int = 128) -> Frame:
    """A stream made to hit the hazard rules: two CT32 framebuffers A (page 0)
    and B (page 64) with one depth buffer, textures placed on framebuffer pages
    (render to texture), on top of the framebuffer being drawn (feedback) and
    on free pages, uploads into textures the open pass already samples (some
    split around a draw, so part of the image arrives later), LOCAL->LOCAL
    copies out of the framebuffers, CLUT reloads (repeated loads for palette
    memoisation, CLD compare modes, palettes on written pages), TEXFLUSH, FRAME
    switches and region clamps.  1x or 4x super-sampling."""
    rng = np.random.Generator(np.random.PCG64(90000 + seed))
    s = GifStream()
    ss = [1, 4][int(rng.integers(0, 2))]
    fbw = width // 64
    fb_pages = [0, 64]
    zbp = 160
    s.ad([(PRMODECONT, 1), (FRAME_1, frame_reg(fb_pages[0], fbw, PSMCT32)), (ZBUF_1, zbuf_reg(zbp, PSMZ24)),
          (SCISSOR_1, scissor_reg(0, width - 1, 0, height - 1)), (XYOFFSET_1, 0),
          (TEST_1, test_reg(zte=1, ztst=2)), (ALPHA_1, alpha_reg(0, 1, 0, 1))])
    # Free texture pages from 200 on: CT32 textures and PSMT8 ones with CLUTs.
    free = []
    page = 200
    for _ in range(4):
        tw, th = int(rng.integers(4, 7)), int(rng.integers(4, 7))
        w, h = 1 << tw, 1 << th
        s.upload(page * BLOCKS_PER_PAGE, max(1, w // 64), PSMCT32, 0, 0, w, h,
                 rng.integers(0, 256, size=w * h * 4, dtype=np.uint8).tobytes())
        free.append((page * BLOCKS_PER_PAGE, max(1, w // 64), PSMCT32, tw, th))
        page += 4
    clut_pages = [page, page + 1]
    for cp in clut_pages:
        s.upload(cp * BLOCKS_PER_PAGE, 1, PSMCT32, 0, 0, 16, 16, rng.integers(0, 256, size=16 * 16 * 4, dtype=np.uint8).tobytes())
    t8 = (page + 2) * BLOCKS_PER_PAGE
    s.upload(t8, 2, PSMT8, 0, 0, 64, 64, rng.integers(0, 256, size=64 * 64, dtype=np.uint8).tobytes())
    current_fb = 0
    count = 0
    for _ in range(ops):
        op = rng.uniform()
        if op < 0.45:
            # Draw a few primitives into the current framebuffer.
            n = int(rng.integers(1, 12))
            textured = rng.uniform() < 0.7
            regs = []
            if rng.uniform() < 0.25:
                current_fb ^= 1
                regs.append((FRAME_1, frame_reg(fb_pages[current_fb], fbw, PSMCT32)))
            if textured:
                kind = rng.uniform()
                if kind < 0.3:
                    # Render to texture: sample the other framebuffer.
                    tbp = fb_pages[current_fb ^ 1] * BLOCKS_PER_PAGE
                    tex0 = tex0_reg(tbp, fbw, PSMCT32, 8, 7)
                elif kind < 0.45:
                    # Sample the framebuffer being drawn.
                    tbp = fb_pages[current_fb] * BLOCKS_PER_PAGE
                    tex0 = tex0_reg(tbp, fbw, PSMCT32, 8, 7)
                elif kind < 0.75:
                    tbp, tbw, psm, tw, th = free[int(rng.integers(0, len(free)))]
                    tex0 = tex0_reg(tbp, tbw, psm, tw, th)
                else:
                    cld = [1, 1, 2, 4][int(rng.integers(0, 4))]
                    cbp = clut_pages[int(rng.integers(0, 2))] * BLOCKS_PER_PAGE
                    tex0 = tex0_reg(t8, 2, PSMT8, 6, 6, cbp=cbp, cpsm=PSMCT32, cld=cld)
                regs.append((TEX0_1, tex0))
                wms, wmt = int(rng.integers(0, 3)), int(rng.integers(0, 3))
                regs.append((CLAMP_1, clamp_reg(wms, wmt, int(rng.integers(0, 32)), int(rng.integers(32, 128)),
                                                int(rng.integers(0, 32)), int(rng.integers(32, 128)))))
                regs.append((TEX1_1, tex1_reg(mmag=int(rng.integers(0, 2)), mmin=int(rng.integers(0, 2)))))
            s.ad(regs)
            sprite = rng.uniform() < 0.5
            if sprite:
                xs, ys = random_sprites(rng, n, width, height, 4, 2000)
                nv = 2
            else:
                xs, ys = random_triangles(rng, n, width, height, 4, 2000)
                nv = 3
            q = np.zeros((n * nv, 3, 2), dtype=np.uint64)
            q[:, 0] = q_rgbaq(rng.integers(0, 256, size=(n * nv, 4)))
            q[:, 1] = q_uv(rng.integers(0, width * 16, n * nv), rng.integers(0, height * 16, n * nv))
            q[:, 2] = q_xyz2(xs.reshape(-1), ys.reshape(-1), rng.integers(0, 1 << 24, n * nv))
            prim = prim_reg(PRIM_SPRITE if sprite else PRIM_TRI, iip=1, tme=int(textured), fst=1,
                            abe=int(rng.uniform() < 0.3))
            s.packed(prim, [D_RGBAQ, D_UV, D_XYZ2], q.reshape(-1, 2))
            count += n
        elif op < 0.6:
            # Upload into a texture that may be in use; sometimes split around a draw.
            tbp, tbw, psm, tw, th = free[int(rng.integers(0, len(free)))]
            w, h = 1 << tw, 1 << th
            x, y = int(rng.integers(0, w // 2)), int(rng.integers(0, h // 2))
            uw, uh = int(rng.integers(1, w - x + 1)), int(rng.integers(2, h - y + 1)) & ~1
            uh = max(uh, 2)
            data = rng.integers(0, 256, size=uw * uh * 4, dtype=np.uint8).tobytes()
            if rng.uniform() < 0.3 and len(data) >= 64:
                half = (len(data) // 2) & ~15
                s.ad([(BITBLTBUF, bitbltbuf_reg(dbp=tbp, dbw=tbw, dpsm=psm)), (TRXPOS, trxpos_reg(dsax=x, dsay=y)),
                      (TRXREG, trxreg_reg(uw, uh)), (TRXDIR, 0)])
                s.image(data[:half])
                # A draw sampling the texture before the rest of the image.
                s.ad([(TEX0_1, tex0_reg(tbp, tbw, psm, tw, th))])
                xs, ys = random_sprites(rng, 1, width, height, 16, 400)
                qq = np.zeros((2, 3, 2), dtype=np.uint64)
                qq[:, 0] = q_rgbaq(rng.integers(0, 256, size=(2, 4)))
                qq[:, 1] = q_uv(rng.integers(0, w * 16, 2), rng.integers(0, h * 16, 2))
                qq[:, 2] = q_xyz2(xs.reshape(-1), ys.reshape(-1), np.array([1, 1]))
                s.packed(prim_reg(PRIM_SPRITE, tme=1, fst=1), [D_RGBAQ, D_UV, D_XYZ2], qq.reshape(-1, 2))
                s.image(data[half:])
                count += 1
            else:
                s.upload(tbp, tbw, psm, x, y, uw, uh, data)
        elif op < 0.72:
            # Copy a framebuffer rectangle into a free texture or the other framebuffer.
            src = fb_pages[int(rng.integers(0, 2))] * BLOCKS_PER_PAGE
            if rng.uniform() < 0.5:
                dst, dbw = free[int(rng.integers(0, len(free)))][:2]
            else:
                dst, dbw = fb_pages[int(rng.integers(0, 2))] * BLOCKS_PER_PAGE, fbw
            cw, ch = int(rng.integers(8, 64)), int(rng.integers(8, 64))
            s.ad([(BITBLTBUF, bitbltbuf_reg(sbp=src, sbw=fbw, spsm=PSMCT32, dbp=dst, dbw=dbw, dpsm=PSMCT32)),
                  (TRXPOS, trxpos_reg(ssax=int(rng.integers(0, width - cw)), ssay=int(rng.integers(0, height - ch)),
                                      dsax=int(rng.integers(0, 32)), dsay=int(rng.integers(0, 32)))),
                  (TRXREG, trxreg_reg(cw, ch)), (TRXDIR, 2)])
        elif op < 0.85:
            # CLUT reload, often identical to an earlier one.
            cbp = clut_pages[int(rng.integers(0, 2))] * BLOCKS_PER_PAGE
            cld = [1, 1, 1, 2, 3, 4, 5][int(rng.integers(0, 7))]
            s.ad([(TEX0_1, tex0_reg(t8, 2, PSMT8, 6, 6, cbp=cbp, cpsm=PSMCT32, cld=cld))])
        elif op < 0.93:
            s.ad([(TEXFLUSH, 0)])
        else:
            # A palette page rewritten by the host.
            cp = clut_pages[int(rng.integers(0, 2))]
            s.upload(cp * BLOCKS_PER_PAGE, 1, PSMCT32, 0, 0, 16, 16,
                     rng.integers(0, 256, size=16 * 16 * 4, dtype=np.uint8).tobytes())
    return Frame("hazards_%d" % seed, s.tobytes(), ss, True, count, {})
