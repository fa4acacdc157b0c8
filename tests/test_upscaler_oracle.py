"""The upscaler's CPU oracle: analytic gradients against finite differences
of its own loss (in FP64 without BF16 rounding), and the BF16 rounding rule."""
import numpy as np

import pgs
import upscaler_ref as U


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 1e-20, 65504.0], dtype=np.float32)
    r = U.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == np.float32(1.0078125)        # above the tie rounds up
    assert abs(r[3] - -3.140625) < 1e-6
    assert np.all(U.bf16(r) == r)


def test_oracle_gradient_matches_finite_differences(monkeypatch):
    # Without BF16 rounding the oracle is a plain FP64 network.
    monkeypatch.setattr(U, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, size=(1, 6, 7, 4), dtype=np.uint8)
    tgt = rng.integers(0, 256, size=(1, 6, 7, 4), dtype=np.uint8)
    params = pgs.upscaler_init_params(3).astype(np.float64)
    params[-4:] = rng.normal(0, 0.05, 4)
    loss, grad = U.backward(img, tgt, params)
    # Spot-check a spread of parameters in every layer.
    idx = np.linspace(0, params.size - 1, 40).astype(int)
    eps = 1e-6
    for i in idx:
        p1 = params.copy(); p1[i] += eps
        p2 = params.copy(); p2[i] -= eps
        l1, _ = U.backward(img, tgt, p1)
        l2, _ = U.backward(img, tgt, p2)
        num = (l1 - l2) / (2 * eps)
        assert abs(num - grad[i]) <= 1e-5 + 1e-3 * abs(num), (i, num, grad[i])
