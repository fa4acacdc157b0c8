"""The GIF decoder on a worker thread (pgs_gs_options.threaded_decode).

With threaded decode the worker runs GIF decode and vertex assembly ahead of
the calling thread, which runs the register-file state, hazard tracking and the
backend from the worker's commands.  The records handed to the backend must be
the same as with the decoder on the calling thread, also when a transfer is cut
anywhere into pieces and when a host callback reads and writes registers in the
middle of a transfer."""
import numpy as np
import pytest

import gsgen as g
import pgs
from recording_backend import RecordingBackend

SIGNAL = 0x60
MODES = [pgs.THREADED_DECODE_OFF, pgs.THREADED_DECODE_ALWAYS]


def records(be: RecordingBackend) -> list:
    out = []
    for p in be.passes:
        out.append((p["flush_reason"], p["positions"], [tuple(sorted(a.items())) for a in p["attributes"]],
                    [tuple(sorted((k, tuple(v) if isinstance(v, list) else v) for k, v in x.items()))
                     for x in p["prims"]]))
    return out


def run(chunks, mode, ss=1, on_signal=None):
    be = RecordingBackend()
    gs = pgs.GSInterface(be, super_sampling=ss, threaded_decode=mode)
    if on_signal:
        gs.set_signal_interface(on_signal=lambda v: on_signal(gs, v))
    for c in chunks:
        gs.gif_transfer(0, c)
    gs.flush()
    regs = [gs.read_register(r) for r in (g.PRIM, 0x01, 0x02, 0x03)]
    gs.close()
    return records(be), regs


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_cut_transfers_match_one_transfer(seed):
    """A stream cut at random 16-byte boundaries gives the records of the
    whole stream in one call, on either thread."""
    f = g.frame_fuzz(seed)
    data = f.data
    rng = np.random.default_rng(seed)
    cuts = np.sort(rng.choice(np.arange(1, len(data) // 16), size=min(40, len(data) // 16 - 1), replace=False)) * 16
    chunks = [data[a:b] for a, b in zip([0, *cuts], [*cuts, len(data)])]
    whole, whole_regs = run([data], pgs.THREADED_DECODE_OFF, f.super_sampling)
    for mode in MODES:
        got, regs = run(chunks, mode, f.super_sampling)
        assert got == whole
        assert regs == whole_regs


def test_signal_callback_sees_the_stream_stopped_at_its_register():
    """The callback reads the vertex registers as of the SIGNAL and moves the
    drawing offset for the triangles after it; the worker must not have run
    ahead with the old offset."""
    s = g.GifStream()
    g._frame_setup(s, 0, 10, g.PSMCT32, 640, g.PSMZ24, 640, 448, g.test_reg(zte=0))
    rng = np.random.default_rng(5)

    def tris(n):
        q = np.zeros((3 * n, 2, 2), dtype=np.uint64)
        q[:, 0] = g.q_rgbaq(rng.integers(0, 256, (3 * n, 4)))
        q[:, 1] = g.q_xyz2(rng.integers(0, 600 * 16, 3 * n), rng.integers(0, 400 * 16, 3 * n),
                           np.zeros(3 * n, dtype=np.int64))
        s.packed(g.prim_reg(g.PRIM_TRI), [g.D_RGBAQ, g.D_XYZ2], q.reshape(-1, 2))

    tris(2000)
    s.ad([(SIGNAL, 0x77)])
    tris(2000)
    data = s.tobytes()
    results, calls = [], []
    for mode in MODES:
        seen = []

        def on_signal(gs, v):
            seen.append((v, gs.read_register(0x01)))
            gs.write_register(g.XYOFFSET_1, (16 * 16) | ((8 * 16) << 32))
            return False

        got, regs = run([data], mode, on_signal=on_signal)
        results.append(got)
        calls.append(seen)
    assert results[0] == results[1]
    assert calls[0] == calls[1] and len(calls[0]) == 1 and calls[0][0][0] == 0x77
    # The offset moved the second half of the triangles.
    assert sum(len(r[1]) for r in results[0]) == 3 * 4000


def test_invalid_mode_is_rejected():
    with pytest.raises(pgs.PGSError):
        pgs.GSInterface(RecordingBackend(), threaded_decode=3)
