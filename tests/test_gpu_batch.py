"""Batched replay of many mixed command streams (the 64-stream workload).

Every stream's VRAM planes after a batched replay must equal the oracle's
result for that stream alone, whatever the batch's tuning."""
import numpy as np
import pytest

import gsgen
import pgs
import pgs_oracle

pytestmark = pytest.mark.gpu


def planes_of(frame) -> int:
    return 1 if frame.super_sampling == 1 else 2 + frame.super_sampling


def oracle_planes(frame):
    obe = pgs_oracle.OracleBackend()
    ref = pgs_oracle.render(frame, obe, planes=True)
    frags = obe.fragments()
    obe.close()
    return ref, frags


def recorded_backend(frame):
    ss_log2 = {1: 0, 2: 1, 4: 2, 8: 3, 16: 4}[frame.super_sampling]
    be = pgs.CudaBackend(0, max_samples_log2=ss_log2, arena_mib=16)
    gs = pgs.GSInterface(be, super_sampling=frame.super_sampling, ordered=frame.ordered)
    be.begin_record()
    gs.gif_transfer(0, frame.data)
    gs.flush()
    be.end_record()
    gs.close()
    return be


def read_planes(be, frame):
    return np.stack([be.read_plane(p) for p in range(planes_of(frame))])


def check_batch(frames, tuning=None, use_graph=True, replays=2):
    refs = [oracle_planes(f)[0] for f in frames]
    backends = [recorded_backend(f) for f in frames]
    batch = pgs.Batch(0)
    try:
        for be in backends:
            batch.add(be)
        if tuning:
            batch.set_tuning(*tuning)
        batch.replay(replays, reset_vram=True, use_graph=use_graph)
        batch.synchronize()
        for f, be, ref in zip(frames, backends, refs):
            out = read_planes(be, f)
            assert be.error_flags() == 0
            if not np.array_equal(out, ref):
                diff = np.nonzero(out.reshape(-1) != ref.reshape(-1))[0]
                raise AssertionError("%s: %d bytes differ, first at plane %d offset 0x%x" % (
                    f.name, diff.size, diff[0] // pgs.VRAM_SIZE, diff[0] % pgs.VRAM_SIZE))
    finally:
        batch.close()
        for be in backends:
            be.close()


@pytest.mark.parametrize("stream", range(8))
def test_c3_stream_parity(stream):
    """Each mixed stream (CT16/CT32, PSMT4/PSMT8/CT32 textures, 1x/2x/4x) on its own."""
    f = gsgen.stream_c3(stream, num_primitives=3000)
    ref, frags = oracle_planes(f)
    be = pgs.CudaBackend(0, max_samples_log2=4)
    try:
        out = pgs_oracle.render(f, be, planes=True)
        assert be.fragments() == frags
    finally:
        be.close()
    assert np.array_equal(out, ref)


def test_batched_replay_small_streams():
    check_batch([gsgen.stream_c3(i, num_primitives=2000) for i in range(12)])


@pytest.mark.parametrize("tuning", [(128, 8, True), (512, 2, False)])
def test_batched_replay_tunings(tuning):
    check_batch([gsgen.stream_c3(i, num_primitives=1500) for i in range(20, 26)], tuning=tuning)


def test_batched_replay_eager():
    check_batch([gsgen.stream_c3(i, num_primitives=1500) for i in range(30, 34)], use_graph=False)


def test_batched_replay_multi_pass_and_rates():
    """Streams over 64K primitives (several passes each) next to small ones,
    plus high-rate C4 frames whose shading stays on their own streams."""
    frames = [gsgen.stream_c3(i) for i in (40, 41)]
    frames = [f for f in frames] + [gsgen.stream_c3(42, num_primitives=70000), gsgen.frame_c4(seed=7, super_sampling=8,
                                                                                         num_triangles=5000)]
    check_batch(frames)


def test_autotune_keeps_results():
    frames = [gsgen.stream_c3(i, num_primitives=1000) for i in range(50, 56)]
    refs = [oracle_planes(f)[0] for f in frames]
    backends = [recorded_backend(f) for f in frames]
    batch = pgs.Batch(0)
    try:
        for be in backends:
            batch.add(be)
        best, ms = batch.autotune(trials=2)
        assert ms > 0 and best["cta_threads"] in (128, 256, 512)
        batch.replay(1)
        batch.synchronize()
        for f, be, ref in zip(frames, backends, refs):
            assert np.array_equal(read_planes(be, f), ref)
    finally:
        batch.close()
        for be in backends:
            be.close()


@pytest.mark.parametrize("solo", [1, 2500, 70000])
def test_batched_replay_solo_streams(solo):
    """Streams at or above `solo_min_prims` run as their own graph branches, the
    rest through the batched rounds (all solo, mixed, multi-pass solo)."""
    frames = [gsgen.stream_c3(i, num_primitives=n) for i, n in ((60, 1200), (61, 3000), (62, 800), (63, 70000))]
    check_batch(frames, tuning=(512, 2, True, solo))
