"""Upscaler kernels against the CPU oracle: forward results, the loss, and
every parameter's gradient; and a few Adam steps lower the loss."""
import numpy as np
import pytest

import pgs
import upscaler_ref as U

pytestmark = pytest.mark.gpu


def batch(seed, n=2, h=40, w=56):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, size=(n, h, w, 4), dtype=np.uint8)
    # Targets: a smoothed copy, like an anti-aliased resolve of the input.
    t = img.astype(np.float32)
    t = (t + np.roll(t, 1, 1) + np.roll(t, 1, 2) + np.roll(t, (1, 1), (1, 2))) / 4.0
    return img, np.clip(np.rint(t), 0, 255).astype(np.uint8)


def params(seed):
    p = pgs.upscaler_init_params(seed)
    rng = np.random.default_rng(seed + 100)
    p += rng.normal(0, 0.01, p.size).astype(np.float32)   # non-zero biases too
    return p


@pytest.mark.parametrize("tcgen05", [True, False])
def test_forward_and_loss_match_oracle(tcgen05):
    import torch
    img, tgt = batch(1)
    p = params(1)
    up = pgs.Upscaler(0)
    try:
        up.set_tensor_path(tcgen05)
        up.set_params(p)
        di = torch.from_numpy(img).cuda()
        dt = torch.from_numpy(tgt).cuda()
        out = torch.empty_like(di)
        up.forward(di, out)
        loss = up.backward(di, dt)
        up.synchronize()
        assert up.error_flags() == 0
        got = out.cpu().numpy().astype(np.int32)
    finally:
        up.close()
    ref, _ = U.forward(img, p)
    exp = np.clip(np.rint(np.clip(ref, 0, 1) * 255), 0, 255).astype(np.int32)
    d = np.abs(got - exp)
    assert d.max() <= 2 and np.mean(d == 0) > 0.97
    ref_loss, _ = U.backward(img, tgt, p)
    assert abs(loss - ref_loss) <= 2e-3 * ref_loss


@pytest.mark.parametrize("tcgen05", [True, False])
def test_gradients_match_oracle(tcgen05):
    import torch
    img, tgt = batch(2)
    p = params(2)
    up = pgs.Upscaler(0)
    try:
        up.set_tensor_path(tcgen05)
        up.set_params(p)
        up.backward(torch.from_numpy(img).cuda(), torch.from_numpy(tgt).cuda())
        g = up.gradient()
    finally:
        up.close()
    _, ref = U.backward(img, tgt, p)
    o = 0
    for l, (cin, cout) in enumerate(U.SHAPES):
        for part, n in (("w", 9 * cin * cout), ("b", cout)):
            a, b = g[o:o + n].astype(np.float64), ref[o:o + n].astype(np.float64)
            err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert err < 3e-2, (l, part, err)
            o += n
    assert o == g.size


def test_adam_steps_reduce_loss():
    import torch
    img, tgt = batch(3, n=4, h=64, w=64)
    up = pgs.Upscaler(0)
    try:
        up.set_params(pgs.upscaler_init_params(4))
        di, dt = torch.from_numpy(img).cuda(), torch.from_numpy(tgt).cuda()
        first = up.backward(di, dt)
        for _ in range(30):
            up.backward(di, dt, want_loss=False)
            up.adam_step(2e-3)
        last = up.backward(di, dt)
    finally:
        up.close()
    assert last < 0.7 * first


def test_tcgen05_and_mma_sync_paths_agree_on_full_frames():
    """Both tensor paths on 640x448 frames: identical up to the last bit of
    BF16 rounding (accumulation order differs)."""
    import torch
    rng = np.random.default_rng(9)
    img = torch.from_numpy(rng.integers(0, 256, size=(3, 448, 640, 4), dtype=np.uint8)).cuda()
    outs = []
    up = pgs.Upscaler(0)
    try:
        up.set_params(params(9))
        for tc in (True, False):
            up.set_tensor_path(tc)
            o = torch.empty_like(img)
            up.forward(img, o)
            up.synchronize()
            outs.append(o.cpu().numpy().astype(np.int32))
        assert up.error_flags() == 0
    finally:
        up.close()
    d = np.abs(outs[0] - outs[1])
    assert d.max() <= 2 and np.mean(d == 0) > 0.99


def test_forward_on_a_caller_stream_is_identical():
    """pgs_upscaler_set_stream: the same frames through the upscaler's own
    stream and through a stream the caller owns give the same bytes, and
    None returns to the upscaler's stream."""
    import torch
    rng = np.random.default_rng(11)
    img = torch.from_numpy(rng.integers(0, 256, size=(2, 448, 640, 4), dtype=np.uint8)).cuda()
    side = torch.cuda.Stream()
    up = pgs.Upscaler(0)
    try:
        up.set_params(params(11))
        own = up.stream()
        a = torch.empty_like(img)
        up.forward(img, a)
        up.synchronize()
        up.set_stream(side.cuda_stream)
        assert up.stream() == side.cuda_stream
        b = torch.empty_like(img)
        up.forward(img, b)
        side.synchronize()
        up.set_stream(None)
        assert up.stream() == own
        c = torch.empty_like(img)
        up.forward(img, c)
        up.synchronize()
        assert up.error_flags() == 0
    finally:
        up.close()
    assert torch.equal(a, b) and torch.equal(a, c)
