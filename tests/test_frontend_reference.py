"""The product frontend against the reference's own frontend, run here.

Every seeded stream generator of the benchmark and the parity suite goes
through both frontends (tests/frontend_reference.py explains what is compared):
pass boundaries and flush reasons, instances, coarse tile sizes, primitive
records, state vectors, texture descriptors and CLUT slots must be the same.
frame_hazards streams are built to hit the hazard rules (uploads into textures
the open pass samples, copies out of framebuffers, CLUT reloads, TEXFLUSH,
render-to-texture and feedback).  The reference frontend is compiled from the
reference's sources, so these tests skip where those are not mounted."""
import pytest

import gsgen as g
import pgs
import pgs_ref_frontend
from frontend_reference import compare

pytestmark = pytest.mark.skipif(not pgs_ref_frontend.available(),
                                reason="reference frontend not built (reference sources absent)")

STREAMS = [
    ("c1", lambda: g.frame_c1()),
    ("c2_full", lambda: g.frame_c2()),
    ("c4_8x", lambda: g.frame_c4(num_triangles=20000, passes=10)),
    ("c4_16x", lambda: g.frame_c4(super_sampling=16, num_triangles=20000, passes=10)),
    ("flat_ui", lambda: g.frame_flat_ui()),
] + [("fuzz_%d" % i, (lambda i=i: g.frame_fuzz(i))) for i in range(12)] \
  + [("mip_%d" % i, (lambda i=i: g.frame_mip(i))) for i in range(6)] \
  + [("alias_%d" % i, (lambda i=i: g.frame_alias(i))) for i in range(4)] \
  + [("ssaa_textures_%d" % i, (lambda i=i: g.frame_ssaa_textures(i))) for i in range(4)] \
  + [("field_aware_%d" % i, (lambda i=i: g.frame_field_aware(i))) for i in range(2)] \
  + [("quads_%d" % i, (lambda i=i: g.frame_quads(i))) for i in range(4)] \
  + [("blend_demote_%d" % i, (lambda i=i: g.frame_blend_demote(i))) for i in range(3)] \
  + [("c3_%d" % i, (lambda i=i: g.stream_c3(i, num_primitives=3000))) for i in range(8)] \
  + [("hazards_%d" % i, (lambda i=i: g.frame_hazards(i))) for i in range(16)]


DECODE_MODES = {"auto": pgs.THREADED_DECODE_AUTO, "direct": pgs.THREADED_DECODE_OFF,
                "threaded": pgs.THREADED_DECODE_ALWAYS}


@pytest.mark.parametrize("mode", sorted(DECODE_MODES))
@pytest.mark.parametrize("name,make", STREAMS, ids=[n for n, _ in STREAMS])
def test_frontend_matches_reference(name, make, mode):
    """Every stream with the GIF decoder on the calling thread, on the worker
    thread, and chosen by transfer size."""
    frame = make()
    diffs = compare(frame.data, frame.super_sampling, frame.ordered, DECODE_MODES[mode])
    assert not diffs, "\n".join(diffs[:20])


def test_hazard_streams_take_snapshots():
    """The hazard streams reach the snapshot path (a transfer into a texture
    the open pass holds), so the test above covers it."""
    from frontend_reference import run_product
    taken = 0
    for i in range(16):
        f = g.frame_hazards(i)
        be = run_product(f.data, f.super_sampling, f.ordered)
        taken += sum(1 for e in be.events if e[0] == "snapshot")
    assert taken > 0
