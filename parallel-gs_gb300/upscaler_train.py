"""Training and evaluation of the learned anti-aliasing upscaler.

Pairs are rendered by the method itself: each seeded scene in the style of the
textured-and-blended workload (PSMT8 textures with CT32 CLUTs, perspective
STQ, bilinear, alpha blending, alpha test, FBA, dither; 12,500 triangles + 500
sprites per 640x448 frame) is drawn once at 1x and once at 16x SSAA (4x4
ordered grid); the CRTC read-out of each framebuffer is the input and the
target.  The network trains on random 128x128 crops with Adam, entirely in the
project's own kernels (pgs_upscaler_*); evaluation runs the full frames of
held-out seeds and reports PSNR and maximum absolute error over RGB against
the exact 16x resolve, next to the same figures for the 1x input.

    python parallel-gs_gb300/upscaler_train.py --out upscaler_out

writes weights.npy (the flat FP32 parameter vector) and metrics.json there.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import gsgen  # noqa: E402
import pgs  # noqa: E402

WIDTH, HEIGHT = 640, 448
TRAIN_SEED0, EVAL_SEED0 = 10000, 20000
WEIGHTS = HERE / "upscaler_weights.npy"


def scene(seed: int) -> gsgen.Frame:
    return gsgen.frame_c2(seed=seed, num_triangles=12500, num_sprites=500, super_sampling=1, num_textures=8)


class PairRenderer:
    """Renders a scene at 1x and at 16x SSAA on two CUDA backends and reads
    both framebuffers out as RGBA8 into device tensors."""

    def __init__(self, device: int = 0) -> None:
        self.b1_device = device
        self.b1 = pgs.CudaBackend(device, max_samples_log2=0, arena_mib=32)
        self.b16 = pgs.CudaBackend(device, max_samples_log2=4, arena_mib=32)
        self.g1 = pgs.GSInterface(self.b1, super_sampling=1)
        self.g16 = pgs.GSInterface(self.b16, super_sampling=16, ordered=True)
        self.zeros = np.zeros(pgs.VRAM_SIZE, dtype=np.uint8)

    def render(self, frame: gsgen.Frame, out1, out16) -> None:
        for gs, be, out in ((self.g1, self.b1, out1), (self.g16, self.b16, out16)):
            if out is None:
                continue
            gs.write_vram(self.zeros)
            gs.gif_transfer(0, frame.data)
            gs.flush()
            be.sample_circuit(out.data_ptr(), frame.meta["fbp"], WIDTH // 64, gsgen.PSMCT32, WIDTH, HEIGHT)
        self.b1_sync()

    def render_rate(self, frame: gsgen.Frame, out, ss: int) -> None:
        """The scene at `ss`x SSAA (ordered grid), read out like the target."""
        if not hasattr(self, "rates"):
            self.rates = {}
        if ss not in self.rates:
            be = pgs.CudaBackend(self.b1_device, max_samples_log2={2: 1, 4: 2, 8: 3, 16: 4}[ss], arena_mib=32)
            self.rates[ss] = (be, pgs.GSInterface(be, super_sampling=ss, ordered=True))
        be, gs = self.rates[ss]
        gs.write_vram(self.zeros)
        gs.gif_transfer(0, frame.data)
        gs.flush()
        be.sample_circuit(out.data_ptr(), frame.meta["fbp"], WIDTH // 64, gsgen.PSMCT32, WIDTH, HEIGHT)
        self.b1_sync()

    def b1_sync(self) -> None:
        import torch
        torch.cuda.synchronize()

    def close(self) -> None:
        self.g1.close()
        self.g16.close()
        for be, gs in getattr(self, "rates", {}).values():
            gs.close()
            be.close()
        self.b1.close()
        self.b16.close()


def build_dataset(renderer: PairRenderer, seeds, log=None):
    import torch
    n = len(seeds)
    inp = torch.empty((n, HEIGHT, WIDTH, 4), dtype=torch.uint8, device="cuda")
    tgt = torch.empty_like(inp)
    t0 = time.perf_counter()
    for i, s in enumerate(seeds):
        renderer.render(scene(s), inp[i], tgt[i])
        if log and (i + 1) % 500 == 0:
            log("rendered %d/%d scenes (%.1fs)" % (i + 1, n, time.perf_counter() - t0))
    return inp, tgt


def train(up: pgs.Upscaler, inp, tgt, steps: int, batch: int = 16, crop: int = 128, lr: float = 1e-3,
          seed: int = 0, log=None, eval_every: int = 0, eval_set=None, curve=None) -> list[float]:
    """Adam on random crops with a cosine learning rate.  With eval_every, the
    held-out PSNR of eval_set (inputs, targets) is logged into `curve` every
    eval_every steps, next to the mean training loss since the last point."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    stream = torch.cuda.ExternalStream(up.stream())
    losses = []
    window = []
    n = inp.shape[0]
    with torch.cuda.stream(stream):
        for step in range(steps):
            if eval_every and eval_set is not None and step and step % eval_every == 0:
                up.synchronize()
                m = evaluate(up, *eval_set)
                tr = float(np.mean(window)) if window else float("nan")
                window = []
                point = {"step": step, "train_loss": tr, "train_psnr_db": psnr(tr * 255.0 ** 2) if tr == tr else None,
                         "heldout_psnr_db": m["psnr_net_db"]}
                if curve is not None:
                    curve.append(point)
                if log:
                    log("curve %s" % json.dumps(point))
            idx = torch.randint(0, n, (batch,), generator=g).tolist()
            ys = torch.randint(0, HEIGHT - crop + 1, (batch,), generator=g).tolist()
            xs = torch.randint(0, WIDTH - crop + 1, (batch,), generator=g).tolist()
            bi = torch.stack([inp[i, y:y + crop, x:x + crop] for i, y, x in zip(idx, ys, xs)]).contiguous()
            bt = torch.stack([tgt[i, y:y + crop, x:x + crop] for i, y, x in zip(idx, ys, xs)]).contiguous()
            want = (step % 200 == 0) or step == steps - 1 or bool(eval_every and step % 50 == 0)
            loss = up.backward(bi, bt, want_loss=want)
            if want:
                window.append(loss)
            cur = lr * (0.02 + 0.98 * 0.5 * (1.0 + math.cos(math.pi * step / steps)))
            up.adam_step(cur)
            if want:
                losses.append(loss)
                if log:
                    log("step %d loss %.3e lr %.2e" % (step, loss, cur))
    up.synchronize()
    return losses


def psnr(mse: float) -> float:
    return float("inf") if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse)


def evaluate(up: pgs.Upscaler, inp, tgt, chunk: int = 4) -> dict:
    """PSNR over RGB (aggregate mean squared error) and maximum absolute error,
    for the network output and for the 1x input, against the 16x targets."""
    import torch
    stream = torch.cuda.ExternalStream(up.stream())
    se_net = se_in = 0.0
    max_net = max_in = 0
    per_net, per_in = [], []
    with torch.cuda.stream(stream):
        for s in range(0, inp.shape[0], chunk):
            a = inp[s:s + chunk].contiguous()
            t = tgt[s:s + chunk]
            out = torch.empty_like(a)
            up.forward(a, out)
            dn = out[..., :3].float() - t[..., :3].float()
            di = a[..., :3].float() - t[..., :3].float()
            se_net += float((dn * dn).sum())
            se_in += float((di * di).sum())
            max_net = max(max_net, int(dn.abs().max()))
            max_in = max(max_in, int(di.abs().max()))
            per_net += [psnr(float(v)) for v in (dn * dn).mean(dim=(1, 2, 3))]
            per_in += [psnr(float(v)) for v in (di * di).mean(dim=(1, 2, 3))]
    up.synchronize()
    count = inp.shape[0] * HEIGHT * WIDTH * 3
    return {"psnr_net_db": psnr(se_net / count), "psnr_input_db": psnr(se_in / count),
            "max_abs_err_net": max_net, "max_abs_err_input": max_in,
            "mean_image_psnr_net_db": float(np.mean(per_net)), "mean_image_psnr_input_db": float(np.mean(per_in)),
            "images": int(inp.shape[0])}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=5000)
    ap.add_argument("--eval", type=int, default=500)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default="upscaler_out")
    ap.add_argument("--eval-every", type=int, default=0, help="log held-out PSNR every this many steps")
    ap.add_argument("--curve-scenes", type=int, default=100, help="held-out scenes used for the curve")
    ap.add_argument("--ceilings", action="store_true",
                    help="also report 2x, 4x and 8x SSAA against the 16x targets on the held-out scenes")
    ap.add_argument("--tensor-path", type=int, default=2,
                    help="32->32 layers: 0 mma.sync, 1 or 2 tcgen05 with that many persistent CTAs per SM")
    args = ap.parse_args()
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    logf = open(out / "train.log", "w")

    def log(msg):
        print(msg, flush=True)
        logf.write(msg + "\n")
        logf.flush()

    import torch
    torch.cuda.init()
    r = PairRenderer(0)
    t0 = time.perf_counter()
    tr_in, tr_tgt = build_dataset(r, range(TRAIN_SEED0, TRAIN_SEED0 + args.train), log)
    ev_in, ev_tgt = build_dataset(r, range(EVAL_SEED0, EVAL_SEED0 + args.eval), log)
    t_data = time.perf_counter() - t0
    ceilings = {}
    if args.ceilings:
        # What more samples per pixel recover, on the same held-out scenes: the
        # 1x input is one sample of what the 16x target averages.
        for ss in (2, 4, 8):
            se, count = 0.0, 0
            img = torch.empty((HEIGHT, WIDTH, 4), dtype=torch.uint8, device="cuda")
            for i, sd in enumerate(range(EVAL_SEED0, EVAL_SEED0 + args.eval)):
                r.render_rate(scene(sd), img, ss)
                d = img[..., :3].float() - ev_tgt[i, ..., :3].float()
                se += float((d * d).sum())
                count += HEIGHT * WIDTH * 3
            ceilings["ssaa%dx_psnr_db" % ss] = psnr(se / count)
            log("%dx SSAA against 16x on %d held-out scenes: %.2f dB" % (ss, args.eval, ceilings["ssaa%dx_psnr_db" % ss]))
    r.close()
    up = pgs.Upscaler(0)
    up.set_tensor_path(args.tensor_path)
    up.set_params(pgs.upscaler_init_params(0))
    before = evaluate(up, ev_in[:64], ev_tgt[:64])
    log("before training: %s" % json.dumps(before))
    t1 = time.perf_counter()
    curve = []
    k = min(args.curve_scenes, args.eval)
    losses = train(up, tr_in, tr_tgt, args.steps, args.batch, lr=args.lr, log=log, eval_every=args.eval_every,
                   eval_set=(ev_in[:k], ev_tgt[:k]), curve=curve)
    t_train = time.perf_counter() - t1
    metrics = evaluate(up, ev_in, ev_tgt)
    metrics.update({"train_scenes": args.train, "eval_scenes": args.eval, "steps": args.steps, "batch": args.batch,
                    "crop": 128, "dataset_seconds": t_data, "train_seconds": t_train, "losses": losses,
                    "curve": curve, "curve_scenes": k, "lr": args.lr, **ceilings,
                    "scene": "frame_c2 style, 12500 triangles + 500 sprites, 640x448, input 1x, target 16x SSAA 4x4"})
    log("held-out: %s" % json.dumps({k: v for k, v in metrics.items() if k != "losses"}))
    np.save(out / "weights.npy", up.params())
    (out / "metrics.json").write_text(json.dumps(metrics, indent=1))
    up.close()


if __name__ == "__main__":
    main()
