"""Bit-exact parity of the CUDA backend against the CPU oracle.

Both backends sit under the same product frontend and receive the same seeded
GIF command stream; every VRAM plane (GS memory, super-sample reference flags
and the sample planes) must match byte for byte."""
import numpy as np
import pytest

import gsgen
import pgs
import pgs_oracle

pytestmark = pytest.mark.gpu


def run_both(frame):
    ref = pgs_oracle.render(frame, planes=True)
    be = pgs.CudaBackend(0, max_samples_log2=4)
    try:
        out = pgs_oracle.render(frame, be, planes=True)
        assert be.error_flags() == 0
    finally:
        be.close()
    return ref, out


def assert_same(ref, out):
    assert ref.shape == out.shape
    if not np.array_equal(ref, out):
        diff = np.nonzero(ref.reshape(-1) != out.reshape(-1))[0]
        plane = diff // pgs.VRAM_SIZE
        off = diff % pgs.VRAM_SIZE
        raise AssertionError("%d bytes differ; first at plane %d offset 0x%x (oracle %d, cuda %d)" % (
            diff.size, plane[0], off[0], ref.reshape(-1)[diff[0]], out.reshape(-1)[diff[0]]))


@pytest.mark.parametrize("n", [1, 50, 2000])
def test_c1_gouraud_zbuffer(n):
    ref, out = run_both(gsgen.frame_c1(seed=11, num_triangles=n))
    assert_same(ref, out)


@pytest.mark.parametrize("ss", [1, 4])
def test_c2_textured_blended_small(ss):
    f = gsgen.frame_c2(seed=5, num_triangles=400, num_sprites=40, super_sampling=ss, num_textures=2)
    ref, out = run_both(f)
    assert_same(ref, out)
