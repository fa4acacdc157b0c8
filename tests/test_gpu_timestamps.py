"""Stage timestamps of the CUDA backend (set_debug_mode timestamps,
get_accumulated_timestamps): every stage the frame runs accumulates GPU time
while timing is on, and nothing accumulates while it is off."""
import pytest

import gsgen
import pgs

pytestmark = pytest.mark.gpu


def test_stage_timestamps_accumulate_only_while_on():
    be = pgs.CudaBackend(0, max_samples_log2=2)
    try:
        gs = pgs.GSInterface(be, super_sampling=4)
        f = gsgen.frame_c2(seed=5, num_triangles=400, num_sprites=40, super_sampling=4, num_textures=2)
        gs.gif_transfer(0, f.data)
        gs.read_vram()
        assert all(gs.get_accumulated_timestamps(k) == 0.0 for k in pgs.TIMESTAMPS)

        gs.set_debug_mode(timestamps=True)
        gs.gif_transfer(0, f.data)
        gs.read_vram()
        gs.write_vram(bytes(4096), 0)
        t = {k: gs.get_accumulated_timestamps(k) for k in pgs.TIMESTAMPS}
        for k in ("CopyVRAM", "PaletteUpdate", "TextureUpload", "TriangleSetup", "Binning", "Shading", "Readback",
                  "SyncHostToVRAM"):
            assert t[k] > 0.0, k
        assert t["Shading"] < 10.0

        gs.set_debug_mode(timestamps=False)
        gs.gif_transfer(0, f.data)
        gs.read_vram()
        assert {k: gs.get_accumulated_timestamps(k) for k in pgs.TIMESTAMPS} == t
        gs.close()
    finally:
        be.close()
