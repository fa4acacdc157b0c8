"""The trained upscaler (parallel-gs_gb300/upscaler_weights.npy, produced by
upscaler_train.py) against the method without it: on held-out seeds its
output is closer to the exact 16x SSAA resolve than the 1x render is."""
import numpy as np
import pytest

import pgs

pytestmark = pytest.mark.gpu


def test_trained_network_beats_1x_render_on_held_out_scenes():
    import upscaler_train as T
    r = T.PairRenderer(0)
    try:
        inp, tgt = T.build_dataset(r, range(T.EVAL_SEED0 + 400, T.EVAL_SEED0 + 408))
    finally:
        r.close()
    up = pgs.Upscaler(0)
    try:
        up.set_params(np.load(T.WEIGHTS))
        m = T.evaluate(up, inp, tgt)
    finally:
        up.close()
    assert m["psnr_net_db"] > m["psnr_input_db"] + 3.0
    assert m["max_abs_err_net"] <= m["max_abs_err_input"]
