"""VRAM snapshots for textures of the open pass (pgs_backend_ops.snapshot_vram).

An upload into a texture the open pass already samples keeps the pass going
(the reference's texture cache holds the image, gs/page_tracker.cpp:585-594);
the textures held so far decode from a VRAM snapshot taken before the upload.
The frame must equal the same stream with an explicit flush before the upload.
"""
import numpy as np

import pgs
import pgs_oracle
import snapshot_streams
from recording_backend import RecordingBackend


def test_upload_into_sampled_texture_takes_a_snapshot():
    frame = snapshot_streams.sample_then_upload()
    be = RecordingBackend()
    gs = pgs.GSInterface(be)
    gs.gif_transfer(0, frame.data)
    gs.flush()
    gs.close()
    assert [p["num_primitives"] for p in be.passes] == [2]
    assert ("snapshot", 0) in be.events
    assert be.passes[0]["snapshot_textures"] == [1]


def test_snapshot_frame_equals_flush_before_the_upload():
    frame = snapshot_streams.sample_then_upload()
    one = pgs_oracle.render(frame, planes=True)
    head, tail = snapshot_streams.sample_then_upload(parts=True)
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be)
    gs.gif_transfer(0, head)
    gs.flush()
    gs.gif_transfer(0, tail)
    two = gs.read_vram()
    gs.close()
    be.close()
    assert np.array_equal(one[0], two)
    # Both halves drew something different from the first texture's image.
    assert np.count_nonzero(one[0][:64 * 64 * 4]) > 0
