"""Compare what the product frontend hands its backend with what the reference's
own frontend hands its renderer, for the same GIF stream.

The reference side is oracle/pgs_ref_frontend.py (gs/gs_interface.cpp,
gs/page_tracker.cpp and gs/gs_util.cpp compiled unmodified over a recording
renderer); the product side is the product frontend over
tests/recording_backend.py.  The comparison covers, pass by pass: the flush
reason, the primitive count, the coarse tile size, every instance (FRAME, ZBUF,
origin, tile counts, sampling rates, opaque mask, depth flags, channel shuffle),
the vertex positions and attributes, the primitive words (box, state, tex, tex2,
alpha, fbmsk, fogcol), the state vectors, and each texture's addressing state
and CLUT slot.  Slots the reference never writes are not compared: the third
vertex of sprites and lines, and the attributes of the second vertex of points.
"""
from __future__ import annotations

import numpy as np

import pgs
import pgs_ref_frontend
from recording_backend import RecordingBackend

REASONS = ["FBPointer", "Overflow", "TextureHazard", "CopyHazard", "SubmissionFlush", "PressureFlush", "HostAccess"]
STATE_FIX, STATE_SPRITE, STATE_LINE = 20, 21, 22
INSTANCE_FIELDS = ("frame", "zbuf", "base_x", "base_y", "coarse_tiles_width", "coarse_tiles_height", "opaque_fbmask",
                   "sampling_rate_x_log2", "sampling_rate_y_log2", "z_sensitive", "z_write", "channel_shuffle")


def _field(v: int, o: int, n: int) -> int:
    return (v >> o) & ((1 << n) - 1)


def run_reference(data: bytes, super_sampling: int = 1, ordered: bool = True) -> list[dict]:
    ref = pgs_ref_frontend.RefFrontend(super_sampling, ordered)
    ref.gif_transfer(0, data)
    ref.flush()
    events = ref.events()
    ref.close()
    return events


def run_product(data: bytes, super_sampling: int = 1, ordered: bool = True,
                threaded_decode: int = pgs.THREADED_DECODE_AUTO) -> RecordingBackend:
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=super_sampling, ordered=ordered, threaded_decode=threaded_decode)
    gs.gif_transfer(0, data)
    gs.flush()
    gs.close()
    return be


def compare(data: bytes, super_sampling: int = 1, ordered: bool = True,
            threaded_decode: int = pgs.THREADED_DECODE_AUTO) -> list[str]:
    """Differences between the two frontends as readable lines (empty: none)."""
    events = run_reference(data, super_sampling, ordered)
    be = run_product(data, super_sampling, ordered, threaded_decode)
    ref_passes = [e for e in events if e["type"] == "pass"]
    tex_desc = {e["id"]: e for e in events if e["type"] == "texture"}
    out: list[str] = []
    ra = [(p["flush_reason"], p["num_primitives"]) for p in ref_passes]
    pa = [(REASONS[p["flush_reason"]], p["num_primitives"]) for p in be.passes]
    if ra != pa:
        return ["passes differ: reference %s product %s" % (ra[:12], pa[:12])]
    for i, (a, b) in enumerate(zip(ref_passes, be.passes)):
        n = a["num_primitives"]
        st = a["prims"]["state"]
        keep = np.ones(3 * n, bool)
        two = ((st >> STATE_SPRITE) & 1) | ((st >> STATE_LINE) & 1)
        keep[np.nonzero(two)[0] * 3 + 2] = False
        px, py = a["positions"]["x"].reshape(n, 3), a["positions"]["y"].reshape(n, 3)
        point = (((st >> STATE_SPRITE) & 1) == 1) & (((st >> STATE_FIX) & 1) == 1) & \
                (px[:, 1] == px[:, 0] + 16) & (py[:, 1] == py[:, 0] + 16)
        akeep = keep.copy()
        akeep[np.nonzero(point)[0] * 3 + 1] = False
        bpos = np.array(b["positions"], dtype=np.int64).reshape(-1, 3)
        apos = np.stack([a["positions"]["x"], a["positions"]["y"], a["positions"]["z"]], 1).astype(np.int64)
        if not np.array_equal(apos[keep], bpos[keep]):
            out.append("pass %d: positions differ" % i)
        for k in ("s", "t", "q", "rgba", "fog", "u", "v"):
            av = np.ascontiguousarray(a["attributes"][k])
            bv = np.array([x[k] for x in b["attributes"]], dtype=av.dtype)
            diff = (av.view(np.uint8).reshape(3 * n, -1) != bv.view(np.uint8).reshape(3 * n, -1)).any(1) & akeep
            if diff.any():
                out.append("pass %d: attribute %s differs at %d vertices" % (i, k, int(diff.sum())))
        for k in ("bb", "state", "tex", "tex2", "alpha", "fbmsk", "fogcol"):
            av = a["prims"][k]
            bv = np.array([x[k] for x in b["prims"]], dtype=av.dtype)
            if not np.array_equal(av, bv):
                out.append("pass %d: primitive %s differs" % (i, k))
        astates = [tuple(int(x[k]) for k in ("combiner", "blend_mode", "dimx_lo", "dimx_hi")) for x in a["states"]]
        bstates = [tuple(x[k] for k in ("combiner", "blend_mode", "dimx_lo", "dimx_hi")) for x in b["states"]]
        if astates != bstates:
            out.append("pass %d: state vectors differ" % i)
        if a["coarse_tile_size_log2"] != b["coarse_tile_size_log2"]:
            out.append("pass %d: coarse tile size %d vs %d" % (i, a["coarse_tile_size_log2"], b["coarse_tile_size_log2"]))
        ai, bi = a["instances"], b["instances"]
        if len(ai) != len(bi):
            out.append("pass %d: %d vs %d instances" % (i, len(ai), len(bi)))
        for j, (x, y) in enumerate(zip(ai, bi)):
            for k in INSTANCE_FIELDS:
                if int(x[k]) != int(y[k]):
                    out.append("pass %d instance %d: %s %d vs %d" % (i, j, k, int(x[k]), int(y[k])))
        if len(a["textures"]) != len(b["textures"]):
            out.append("pass %d: %d vs %d textures" % (i, len(a["textures"]), len(b["textures"])))
        for j, (x, y) in enumerate(zip(a["textures"], b["textures"])):
            d = tex_desc.get(int(x["id"]))
            if d is None:
                out.append("pass %d texture %d: no reference descriptor" % (i, j))
                continue
            t0, cl = d["tex0"], d["clamp"]
            expect = {"tbp0": _field(t0, 0, 14), "tbw": _field(t0, 14, 6), "psm": _field(t0, 20, 6),
                      "tw_log2": min(_field(t0, 26, 4), 10), "th_log2": min(_field(t0, 30, 4), 10),
                      "wms": _field(cl, 0, 2), "wmt": _field(cl, 2, 2), "minu": _field(cl, 4, 10),
                      "maxu": _field(cl, 14, 10), "minv": _field(cl, 24, 10), "maxv": _field(cl, 34, 10),
                      "clut_instance": d["palette_bank"], "levels": d["rect_levels"]}
            for k, v in expect.items():
                if y[k] != v:
                    out.append("pass %d texture %d: %s %d vs %d" % (i, j, k, v, y[k]))
    return out
