"""tcgen05 building blocks: a 128x32x32 BF16 product issued from shared memory
descriptors, accumulated in tensor memory and read back, in both operand
layouts the kernels use."""
import numpy as np
import pytest

import pgs

pytestmark = pytest.mark.gpu


def expected():
    r = np.arange(128)[:, None]
    n = np.arange(32)[:, None]
    k = np.arange(32)[None, :]
    a = (((r * 7 + k * 3) % 17) - 8) / 8.0
    b = (((n * 5 + k * 11) % 13) - 6) / 4.0
    return (a @ b.T).astype(np.float32)


@pytest.mark.parametrize("mode", [0, 1])
def test_tcgen05_product(mode):
    out = pgs.umma_selftest(mode)
    assert np.array_equal(out, expected())


def test_bounded_wait_expiry_is_reported_and_context_survives():
    """Mode 2 waits on an mbarrier nothing arrives at: the kernel gives up after
    its poll limit, frees tensor memory, and the host sees the device flag; the
    context stays usable for the next tcgen05 product."""
    with pytest.raises(pgs.PGSError) as e:
        pgs.umma_selftest(2)
    assert e.value.status == pgs.STATUS_CODES["PGS_ERROR_DEVICE_FLAG"]
    assert np.array_equal(pgs.umma_selftest(1), expected())
