"""Benchmark: bit-exact GS frames/s on one GB300 (textured + blended 4x SSAA frame).

Workload (the "textured and blended" configuration): one 640x448 PSMCT32 frame
with PSMZ24 depth, 50,000 perspective-textured alpha-blended triangles and
2,000 sprites over 8 PSMT8 256x256 textures with CT32 CLUTs uploaded through
BITBLTBUF/TRXPOS/TRXREG/TRXDIR, bilinear filtering, ATST GREATER 0x40, FBA,
dither, 4x ordered SSAA.  Seeded synthetic command stream (gsgen.frame_c2).

value   frames/s of the device-resident frame program: the frontend's output
        (primitive records, states, textures, transfer payloads) is recorded
        once into HBM; each step restores the frame's starting VRAM (all six
        planes) and replays transfers, CLUT loads, setup, binning and shading
        as one CUDA graph.  L2 is flushed (256 MiB write) between steps.
e2e     frames/s through the public API (pgs.GSInterface) from host memory:
        GIF decode on the host, host->device copies of the step's records and
        payloads, all kernels, and a device->host read of the 4 MiB GS VRAM.
--impl reference
        times the CPU restatement of the reference's backend (the oracle;
        the reference's own renderer needs Vulkan and cannot run here) with all
        host threads on the same frame.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "parallel-gs_gb300"))

METRIC = "bit-exact GS frames/s + Gfrag/s on 1 GB300; upscaler px/s at PSNR vs 16x SSAA"
WORKLOAD = "textured+blended 640x448 CT32/Z24, 50k STQ tris + 2k sprites, 8x PSMT8 256^2 + CT32 CLUT, bilinear, ATST>0x40, FBA, dither, 4x SSAA"

# Other workloads for --workload (the default line is c2).  Each entry: a
# description and the gsgen call that builds the frame.
WORKLOADS = {
    "c2": (WORKLOAD, "gsgen.frame_c2(num_triangles={triangles}, num_sprites={sprites}, super_sampling={ss})"),
    "c1": ("plain 640x448 CT32/Z24, 10k Gouraud tris, Z GEQUAL, 1x", "gsgen.frame_c1()"),
    "c4x8": ("feedback 640x448 CT32/Z24, 100k tris (80% 1-16 px), 10 passes, 20% draws sample the previous "
             "pass's framebuffer, 8x SSAA (2x4)", "gsgen.frame_c4(super_sampling=8)"),
    "c4x16": ("feedback 640x448 CT32/Z24, 100k tris (80% 1-16 px), 10 passes, 20% draws sample the previous "
              "pass's framebuffer, 16x SSAA (4x4)", "gsgen.frame_c4(super_sampling=16)"),
    "c5": ("learned upscaler: 1x render + 6-layer BF16 conv network vs exact 16x SSAA (4x4), 640x448 scenes in "
           "the textured+blended style (12.5k tris + 500 sprites), held-out seeds",
           "gsgen.frame_c2(seed=20000, num_triangles=12500, num_sprites=500, super_sampling=16)"),
    "c3": ("batched replay: 64 seeded streams, 1k-200k prims (log-uniform), CT16/CT32 320x240-640x512, "
           "PSMT4/PSMT8/CT32 textures 64^2-512^2 with CLUTs, 1x/2x/4x SSAA per stream",
           "[gsgen.stream_c3(i) for i in range(64)]"),
}
# Texture and CLUT bytes uploaded per frame.
TEXTURE_BYTES = {"c2": 8 * (256 * 256 + 16 * 16 * 4), "c1": 0, "c4x8": 4 * (128 * 128 + 16 * 16 * 4),
                 "c4x16": 4 * (128 * 128 + 16 * 16 * 4), "c3": 0, "c5": 8 * (256 * 256 + 16 * 16 * 4)}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gs_gb300", choices=["gs_gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--triangles", type=int, default=50000)
    ap.add_argument("--sprites", type=int, default=2000)
    ap.add_argument("--super-sampling", type=int, default=4)
    ap.add_argument("--no-verify", action="store_true")
    ap.add_argument("--quick", action="store_true", help="skip the CPU baseline and the e2e leg (profiling runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the single-thread oracle timing")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the bounded C1 / C4 / C3 / C5 sub-records of the default line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="pgs_clocks_", suffix=".csv")[1])

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        self.path.unlink(missing_ok=True)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def max_over_ranks(value: float, dist, device: str = "cpu") -> float:
    """Slowest rank's time: every rank renders its own replica, so the job ends
    when the last one does."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(steps: int, world: int, max_ms: float) -> float:
    """Frames/s of the whole job: world replicas x steps frames in the slowest rank's time."""
    return world * steps / (max_ms / 1000.0)


def profiled_traffic(summary: str):
    """DRAM bytes (read + write) per launch of the dominant kernel from the ncu
    summary committed under profiles/ (its `traffic_bytes_per_launch:` line)."""
    try:
        for line in (ROOT / "profiles" / summary).read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    except Exception:
        pass
    return None


def profiled_instructions(summary: str):
    """Warp instructions per launch of the dominant kernel from the committed ncu
    summary (its smsp__inst_executed.sum line)."""
    try:
        for line in (ROOT / "profiles" / summary).read_text().splitlines():
            parts = line.split()
            if len(parts) >= 2 and parts[0] == "smsp__inst_executed.sum":
                return float(parts[1])
    except Exception:
        pass
    return None


def issue_roofline(inst_per_frame, shade_s: float, clk: dict):
    """The shading kernels are bound by instruction issue, not DRAM: warp
    instructions per second against the issue peak of 4 schedulers x SMs x the
    SM clock sampled during the run."""
    if not inst_per_frame or not shade_s:
        return None
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz") or 2070.0
    peak = sms * 4 * mhz * 1e6 / 1e12
    achieved = inst_per_frame / shade_s / 1e12
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Twarp-inst/s", "frac": achieved / peak,
            "instructions_per_frame": inst_per_frame,
            "note": "warp instructions per frame from the committed ncu capture of the shading kernel / the "
                    "live CUDA-event shading time; peak = 4 x %d SMs x %.0f MHz" % (sms, mhz)}


def algorithmic_bytes(frame, ss: int) -> dict:
    """Bytes a frame must move at minimum: prim records in,
    setup records written and read, FB/Z read+write per pixel for plane 0,
    the reference plane and every sample, texture and CLUT bytes, and the
    VRAM read-back."""
    w, h = frame.meta["width"], frame.meta["height"]
    px = w * h
    p = frame.num_primitives
    planes = 1 if ss == 1 else 2 + ss
    passes = frame.meta.get("passes", 1)
    fbz = passes * (2 * (4 + 4) * px * (planes - 1 if ss > 1 else 1) + (2 * 8 * px if ss > 1 else 0))
    setup_rw = (80 + 96 + 32) * p * 2
    records = 152 * p
    textures = frame.meta.get("texture_bytes", 0)
    shade = fbz + (80 + 96 + 32) * p + textures
    return {"frame": records + setup_rw + fbz + textures + 4 * 1024 * 1024, "shade": shade}


def run_reference(args, frame):
    """CPU restatement of the backend on all host threads (the reference arm)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pgs_oracle  # noqa: E402
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    frames = frame if isinstance(frame, list) else [frame]
    for _ in range(max(0, min(args.warmup, 1))):
        for f in frames[:1]:
            pgs_oracle.render(f)
    times = []
    frags = 0
    for _ in range(args.steps):
        frags = 0
        t = time.perf_counter()
        for f in frames:
            be = pgs_oracle.OracleBackend()
            pgs_oracle.render(f, be)
            frags += be.fragments()
            be.close()
        times.append(time.perf_counter() - t)
    total = sum(times)
    fps = len(frames) * args.steps / total
    return {
        "metric": METRIC, "value": fps, "unit": "frames/s", "impl": "reference", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+fp32",
        "data": "synthetic (seeded GS command stream)",
        "config": workload_config(args, frame),
        "gfrag_per_s": frags * fps / 1e9,
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": "full frame, %d steps, oracle_backend.cpp with OpenMP over tiles" % args.steps},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def workload_expr(args) -> str:
    return WORKLOADS[args.workload][1].format(triangles=args.triangles, sprites=args.sprites,
                                              ss=args.super_sampling)


def make_frame(args):
    import gsgen  # noqa: F401,E402
    frame = eval(workload_expr(args), {"gsgen": gsgen})
    if isinstance(frame, list):
        return frame
    frame.meta["texture_bytes"] = TEXTURE_BYTES[args.workload]
    return frame


def workload_config(args, frame) -> dict:
    if isinstance(frame, list):
        return {"workload": WORKLOADS[args.workload][0], "streams": len(frame),
                "primitives": sum(f.num_primitives for f in frame),
                "super_sampling": sorted({f.super_sampling for f in frame})}
    cfg = {"workload": WORKLOADS[args.workload][0], "primitives": frame.num_primitives,
           "super_sampling": frame.super_sampling}
    if args.workload == "c2":
        cfg.update({"triangles": args.triangles, "sprites": args.sprites})
    return cfg


def cpu_baseline_sample(args) -> dict:
    """Oracle on one host thread over one full frame (bounded: ~15-30 s)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    env = dict(os.environ, OMP_NUM_THREADS="1")
    code = ("import sys,time; sys.path.insert(0,%r); sys.path.insert(0,%r);"
            "import gsgen,pgs_oracle;"
            "f=%s;"
            "t=time.perf_counter(); pgs_oracle.render(f); print(time.perf_counter()-t)") % (
        str(ROOT / "parallel-gs_gb300"), str(ROOT / "oracle"), workload_expr(args))
    try:
        out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=240)
        dt = float(out.stdout.strip().splitlines()[-1])
        return {"value": 1.0 / dt, "unit": "frames/s", "cores": 1, "kind": "port",
                "sample": "one full frame on one host thread (oracle_backend.cpp)"}
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": "frames/s", "cores": 1, "kind": "port", "sample": "failed: %s" % e}


def tiny_stream_mix(local, n=64, prims=400):
    """Where the batched rounds pay: many small streams (400 primitives each).
    Frames/s of the per-frame graphs one after another, of the batched rounds
    (solo threshold 0) and of one graph with every stream as its own branch."""
    import torch
    import gsgen
    import pgs
    backends = []
    for i in range(n):
        f = gsgen.stream_c3(1000 + i, num_primitives=prims)
        ss_log2 = {1: 0, 2: 1, 4: 2}[f.super_sampling]
        be = pgs.CudaBackend(local, max_samples_log2=ss_log2, arena_mib=4)
        gs = pgs.GSInterface(be, super_sampling=f.super_sampling, ordered=f.ordered)
        be.begin_record()
        gs.gif_transfer(0, f.data)
        gs.flush()
        be.end_record()
        gs.close()
        backends.append(be)
    out = {"streams": n, "primitives_per_stream": prims}
    try:
        for be in backends:
            be.replay(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            for be in backends:
                be.replay(1)
                torch.cuda.synchronize()
        out["plain_fps"] = 3 * n / (time.perf_counter() - t0)
        for name, tuning in (("batched_rounds_fps", (256, 4, True, 0)), ("graph_branches_fps", (512, 2, True, 1))):
            batch = pgs.Batch(local)
            for be in backends:
                batch.add(be)
            batch.set_tuning(*tuning)
            batch.replay(2)
            batch.synchronize()
            t0 = time.perf_counter()
            batch.replay(10)
            batch.synchronize()
            out[name] = 10 * n / (time.perf_counter() - t0)
            batch.close()
    finally:
        for be in backends:
            be.close()
    return out


def run_c3(args, frames, rank, world, local):
    """64 mixed streams: plain per-frame graphs one after another, the same
    graphs launched concurrently on their own streams, and the batched replay
    (one CUDA graph per round schedule, persistent shading launch), the last
    being `value`."""
    import numpy as np
    import torch
    import pgs
    from concurrent.futures import ThreadPoolExecutor

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    dev = "cuda:%d" % local
    ss_log2 = {1: 0, 2: 1, 4: 2, 8: 3, 16: 4}
    backends, recorded = [], []
    for f in frames:
        be = pgs.CudaBackend(local, max_samples_log2=ss_log2[f.super_sampling], arena_mib=16)
        gs = pgs.GSInterface(be, super_sampling=f.super_sampling, ordered=f.ordered)
        be.begin_record()
        gs.gif_transfer(0, f.data)
        gs.flush()
        be.end_record()
        gs.close()
        recorded.append(be.read_plane(0))
        backends.append(be)
    batch = pgs.Batch(local)
    for be in backends:
        batch.add(be)
    tuning, tune_ms = batch.autotune(trials=3)
    batch.replay(1)
    batch.synchronize()
    verified = all(np.array_equal(be.read_plane(0), r) for be, r in zip(backends, recorded))

    # Plain per-frame path: each stream's frame graph, one frame at a time.
    for be in backends:
        be.replay(1)
    torch.cuda.synchronize()
    plain_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        for be in backends:
            be.replay(1)
            torch.cuda.synchronize()
    plain_fps = len(frames) * plain_steps / (time.perf_counter() - t0)
    # The same graphs issued back to back on the streams' own CUDA streams.
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        for be in backends:
            be.replay(1)
    torch.cuda.synchronize()
    concurrent_fps = len(frames) * plain_steps / (time.perf_counter() - t0)

    # Batched replay, device-timed on the batch's stream.
    bstream = torch.cuda.ExternalStream(batch.stream(), device=local)
    flush_buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        batch.replay(1)
    batch.synchronize()
    frags0 = sum(be.fragments() for be in backends)
    clocks = ClockSampler(local)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(bstream):
        for i in range(args.steps):
            flush_buf.fill_(i & 0xFF)
            ev[i][0].record(bstream)
            batch.replay(1)
            ev[i][1].record(bstream)
    batch.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    frags = (sum(be.fragments() for be in backends) - frags0) // args.steps
    if pg:
        total_ms = max_over_ranks(total_ms, pg, dev)
    fps = replica_throughput(args.steps, world, total_ms) * len(frames)
    t_wall = time.perf_counter()
    batch.replay(args.steps)
    batch.synchronize()
    batched_wall_fps = len(frames) * args.steps / (time.perf_counter() - t_wall)

    launches = batch.launches_per_replay()
    # End to end: every stream decoded on the host by a pool of threads (the
    # frontends are independent), uploaded, rendered, and read back.
    e2e_fps, h2d, d2h = None, 0, 0
    if not args.quick:
        batch.close()
        batch = None
        outs = [torch.empty(pgs.VRAM_SIZE, dtype=torch.uint8, pin_memory=True).numpy() for _ in frames]
        ifaces = [pgs.GSInterface(be, super_sampling=f.super_sampling, ordered=f.ordered)
                  for be, f in zip(backends, frames)]
        e2e_steps = max(2, min(args.steps, 5))

        def one(i):
            gs = ifaces[i]
            gs.gif_transfer(0, frames[i].data)
            gs.wait(gs.read_vram_async(outs[i]))

        with ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 1)) as pool:
            for _ in range(3):
                list(pool.map(one, range(len(frames))))
            st0 = [be.stats() for be in backends]
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                list(pool.map(one, range(len(frames))))
            e2e_dt = time.perf_counter() - t0
        st1 = [be.stats() for be in backends]
        e2e_fps = world * len(frames) * e2e_steps / e2e_dt
        h2d = sum(b["h2d_bytes"] - a["h2d_bytes"] for a, b in zip(st0, st1)) // e2e_steps
        d2h = sum(b["d2h_bytes"] - a["d2h_bytes"] for a, b in zip(st0, st1)) // e2e_steps
        for gs in ifaces:
            gs.close()
    if batch:
        batch.close()
    if rank != 0:
        if pg:
            pg.barrier()
        return
    ab = sum(algorithmic_bytes(f, f.super_sampling)["shade"] for f in frames)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak_gbs = peaks.get("hbm_gbs", 6800.0)
    achieved = ab / (total_ms / args.steps / 1000.0) / 1e9
    cpu = None
    if not (args.quick or args.no_cpu_baseline):
        cpu = cpu_baseline_sample_expr("[gsgen.stream_c3(i) for i in range(4)]", "streams 0-3 of 64, one thread")
    tiny_mix = tiny_stream_mix(local) if rank == 0 and not args.quick else None
    out = {
        "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32+fp32", "data": "synthetic (seeded GS command stream)",
        "config": dict(workload_config(args, frames), l2="flushed (256 MiB write) between steps",
                       parallelism="replicas" if world > 1 else "single"),
        "gfrag_per_s": frags * (fps / len(frames)) / 1e9,
        "fragments_per_step": frags,
        "plain_per_frame_fps": plain_fps,
        "concurrent_per_frame_fps": concurrent_fps,
        "batched_wall_fps": batched_wall_fps,
        "batched_vs_plain": fps / plain_fps,
        "tiny_stream_mix": tiny_mix,
        "autotuned": dict(tuning, ms_per_replay=tune_ms),
        "replay_verified": verified,
        "gpu_launches": launches * args.steps,
        "clocks": clk,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                     "frac": achieved / peak_gbs, "traffic": None, "shade_bytes_per_step": ab,
                     "note": "algorithmic bytes of all streams per replay / batched replay time; "
                             "peak = measured hbm_gbs (of measured)"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
    }
    print(json.dumps(out))
    if pg:
        pg.barrier()


def run_c5(args, rank, world, local):
    """Learned upscaler against exact 16x SSAA: output pixels/s of each path
    (device time of render + CRTC read-out, plus the network for the learned
    path) and PSNR / maximum error over RGB on held-out seeds."""
    import numpy as np
    import torch
    import pgs
    import upscaler_train as T

    torch.cuda.set_device(local)
    dev = "cuda:%d" % local
    up = pgs.Upscaler(local)
    up.set_params(np.load(T.WEIGHTS))
    # Quality on held-out seeds (bounded sample of the 500).
    r = T.PairRenderer(local)
    n_eval = 32 if args.quick else 100
    ev_in, ev_tgt = T.build_dataset(r, range(T.EVAL_SEED0, T.EVAL_SEED0 + n_eval))
    quality = T.evaluate(up, ev_in, ev_tgt)
    r.close()
    del ev_in, ev_tgt

    # Throughput: one recorded scene replayed as CUDA graphs on each path.
    frame = T.scene(T.EVAL_SEED0)
    W, H = T.WIDTH, T.HEIGHT
    paths = {}
    for ss in (1, 16):
        be = pgs.CudaBackend(local, max_samples_log2=0 if ss == 1 else 4, arena_mib=32)
        gs = pgs.GSInterface(be, super_sampling=ss, ordered=True)
        gs.write_vram(np.zeros(pgs.VRAM_SIZE, dtype=np.uint8))
        be.begin_record()
        gs.gif_transfer(0, frame.data)
        gs.flush()
        be.end_record()
        paths[ss] = (be, gs)
    img = torch.empty((1, H, W, 4), dtype=torch.uint8, device=dev)
    out = torch.empty_like(img)
    b1, b16 = paths[1][0], paths[16][0]
    s1 = torch.cuda.ExternalStream(b1.stream(), device=local)
    s16 = torch.cuda.ExternalStream(b16.stream(), device=local)
    su = torch.cuda.ExternalStream(up.stream(), device=local)
    flush_buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    # The network queues on the 1x backend's stream, right behind the frame
    # it upscales.
    def learned_once():
        b1.replay(1, reset_vram=True, use_graph=True)
        b1.sample_circuit(img.data_ptr(), 0, W // 64, 0, W, H)
        up.forward(img, out)

    def exact_once():
        b16.replay(1, reset_vram=True, use_graph=True)
        b16.sample_circuit(img.data_ptr(), 0, W // 64, 0, W, H)

    def timed(fn, start_stream, end_stream):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        total = 0.0
        net_ms = 0.0
        for i in range(args.steps):
            with torch.cuda.stream(start_stream):
                flush_buf.fill_(i & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(start_stream)
            fn()
            b.record(end_stream)
            torch.cuda.synchronize()
            total += a.elapsed_time(b)
        return total / args.steps

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    up.set_stream(b1.stream())
    learned_ms = timed(learned_once, s1, s1)
    up.set_stream(None)
    exact_ms = timed(exact_once, s16, s16)
    # Network alone (the tensor-core part), on the tcgen05 path and on the
    # mma.sync path.
    img_c = img.clone()
    net = {}
    for tc in (0, 1, 2):
        up.set_tensor_path(tc)
        for _ in range(3):
            up.forward(img_c, out)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(su)
        for _ in range(args.steps):
            up.forward(img_c, out)
        b.record(su)
        torch.cuda.synchronize()
        net[tc] = a.elapsed_time(b) / args.steps
    net_ms = min(net[1], net[2])
    clk = clocks.stop()
    for be, gs in paths.values():
        gs.close()
        be.close()
    up.close()
    if rank != 0:
        return
    px = W * H
    flops = 2 * 9 * px * (4 * 32 + 4 * 32 * 32 + 32 * 4)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    achieved = flops / (net_ms / 1000.0) / 1e12
    out_json = {
        "metric": METRIC, "value": px / (learned_ms / 1000.0), "unit": "output px/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": learned_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
        "data": "synthetic (seeded GS command streams)",
        "config": {"workload": WORKLOADS["c5"][0], "width": W, "height": H, "eval_seeds": n_eval,
                   "l2": "flushed (256 MiB write) between steps"},
        "ssaa16_px_per_s": px / (exact_ms / 1000.0),
        "speedup_vs_ssaa16": exact_ms / learned_ms,
        "network_ms_per_frame": net_ms,
        "network_ms_per_frame_mma_sync": net[0],
        "network_ms_per_frame_tcgen05_1cta": net[1],
        "network_ms_per_frame_tcgen05_2cta": net[2],
        "tensor_path": "tcgen05 (TMA + TMEM) for the 32->32 layers, mma.sync for 4->32 and 32->4",
        "psnr_db": quality["psnr_net_db"], "psnr_input_db": quality["psnr_input_db"],
        "max_abs_err": quality["max_abs_err_net"], "max_abs_err_input": quality["max_abs_err_input"],
        "clocks": clk,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "note": "network forward: 2*9*HW*(4*32 + 4*32*32 + 32*4) flops / its CUDA-event time; "
                             "peak = measured bf16_tflops (of measured)"},
        "cpu_baseline": None,
        "e2e": None,
    }
    print(json.dumps(out_json))


def cpu_baseline_sample_expr(expr: str, sample: str) -> dict:
    env = dict(os.environ, OMP_NUM_THREADS="1")
    code = ("import sys,time; sys.path.insert(0,%r); sys.path.insert(0,%r);"
            "import gsgen,pgs_oracle;"
            "fs=%s;"
            "t=time.perf_counter(); [pgs_oracle.render(f) for f in fs]; print(len(fs)/(time.perf_counter()-t))") % (
        str(ROOT / "parallel-gs_gb300"), str(ROOT / "oracle"), expr)
    try:
        out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
        return {"value": float(out.stdout.strip().splitlines()[-1]), "unit": "frames/s", "cores": 1, "kind": "port",
                "sample": sample}
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": "frames/s", "cores": 1, "kind": "port", "sample": "failed: %s" % e}


def measure_frame(frame, local, steps, warmup, e2e_steps, verify=True, pg=None) -> dict:
    """One frame recorded through the public API and replayed as a CUDA graph:
    device-timed frames/s with L2 flushed between steps, the shading kernels'
    CUDA-event time, covered samples, and the end-to-end frames/s through the
    API from host buffers (GIF decode on the host, H2D of records and
    payloads, render, D2H of the 4 MiB GS VRAM into pinned memory, readback of
    frame k waited after frame k+1 is decoded)."""
    import numpy as np
    import torch
    import pgs

    backend = pgs.CudaBackend(device=local, max_samples_log2=4)
    try:
        backend.set_shade_timing(True)
        stream = torch.cuda.ExternalStream(backend.stream(), device=local)
        gs = pgs.GSInterface(backend, super_sampling=frame.super_sampling, ordered=frame.ordered)
        backend.begin_record()
        gs.gif_transfer(0, frame.data)
        gs.flush()
        backend.end_record()
        verified = None
        if verify:
            # One replay from the recorded start state must reproduce the recorded frame.
            first = backend.read_plane(0)
            backend.replay(1, reset_vram=True, use_graph=False)
            verified = bool(np.array_equal(first, backend.read_plane(0)))
        flush_buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda:%d" % local)
        for _ in range(warmup):
            backend.replay(1, reset_vram=True, use_graph=True)
        torch.cuda.synchronize()
        launches = backend.launches_per_replay()
        clocks = ClockSampler(local)
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        clocks.start()
        time.sleep(0.3)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        shade_ms = []
        frags0 = backend.fragments()
        with torch.cuda.stream(stream):
            for i in range(steps):
                flush_buf.fill_(i & 0xFF)
                ev[i][0].record(stream)
                backend.replay(1, reset_vram=True, use_graph=True)
                ev[i][1].record(stream)
                shade_ms.append(backend.last_shade_ms())
        torch.cuda.synchronize()
        clk = clocks.stop()
        frags_per_frame = (backend.fragments() - frags0) // steps
        total_ms = sum(a.elapsed_time(b) for a, b in ev)
        if pg:
            total_ms = max_over_ranks(total_ms, pg, "cuda:%d" % local)
        del flush_buf

        vram = [torch.empty(pgs.VRAM_SIZE, dtype=torch.uint8, pin_memory=True).numpy() for _ in range(2)]
        gs2 = pgs.GSInterface(backend, super_sampling=frame.super_sampling, ordered=frame.ordered)
        for _ in range(max(3, warmup)):
            gs2.gif_transfer(0, frame.data)
            gs2.read_vram(out=vram[0])
        torch.cuda.synchronize()
        st0 = backend.stats()
        t0 = time.perf_counter()
        tickets = []
        host_s = 0.0
        for k in range(e2e_steps):
            a = time.perf_counter()
            gs2.gif_transfer(0, frame.data)
            tickets.append(gs2.read_vram_async(vram[k % 2]))
            host_s += time.perf_counter() - a
            if k >= 1:
                gs2.wait(tickets[k - 1])
        if tickets:
            gs2.wait(tickets[-1])
        e2e_dt = time.perf_counter() - t0
        st1 = backend.stats()
        gs2.close()
        gs.close()
    finally:
        backend.close()
    return {"total_ms": total_ms, "steps": steps, "fps_per_rank": steps / (total_ms / 1000.0),
            "shade_ms": statistics.mean(shade_ms), "frags_per_frame": frags_per_frame, "launches": launches,
            "verified": verified, "clocks": clk,
            "e2e_fps_per_rank": e2e_steps / e2e_dt if e2e_steps else None,
            "e2e_host_ms": host_s * 1e3 / e2e_steps if e2e_steps else None,
            "h2d": (st1["h2d_bytes"] - st0["h2d_bytes"]) // max(e2e_steps, 1),
            "d2h": (st1["d2h_bytes"] - st0["d2h_bytes"]) // max(e2e_steps, 1)}


def extra_workloads(local) -> dict:
    """The other configurations at bounded step counts, for the default line:
    C1 and C4 (8x, 16x) device and end-to-end frames/s, C3 batched against
    plain per-frame replay, C5 quality and speed."""
    import gsgen
    out = {}
    for name, expr, steps in (("c1", "gsgen.frame_c1()", 10),
                              ("c4x8", "gsgen.frame_c4(super_sampling=8)", 5),
                              ("c4x16", "gsgen.frame_c4(super_sampling=16)", 5)):
        try:
            frame = eval(expr, {"gsgen": gsgen})
            m = measure_frame(frame, local, steps=steps, warmup=3, e2e_steps=steps)
            out[name] = {"workload": WORKLOADS[name][0], "value": m["fps_per_rank"], "unit": "frames/s",
                         "steps": steps, "gfrag_per_s": m["frags_per_frame"] * m["fps_per_rank"] / 1e9,
                         "shade_ms_per_frame": m["shade_ms"], "replay_verified": m["verified"],
                         "gpu_launches_per_frame": m["launches"], "clocks": m["clocks"],
                         "e2e": {"value": m["e2e_fps_per_rank"], "unit": "frames/s",
                                 "h2d_bytes_per_step": m["h2d"], "d2h_bytes_per_step": m["d2h"],
                                 "host_ms_per_frame": m["e2e_host_ms"]}}
        except Exception as e:  # noqa: BLE001
            out[name] = {"error": repr(e)}
    try:
        out["c3"] = run_c3_bounded(local)
    except Exception as e:  # noqa: BLE001
        out["c3"] = {"error": repr(e)}
    try:
        out["c5"] = run_c5_bounded(local)
    except Exception as e:  # noqa: BLE001
        out["c5"] = {"error": repr(e)}
    return out


def run_c3_bounded(local, steps=3) -> dict:
    """64 C3 streams: plain per-frame graphs one after another against one
    batched replay (the tuning the autotuner picks on this mix: every stream
    its own graph branch), device-timed, L2 flushed between steps."""
    import numpy as np
    import torch
    import gsgen
    import pgs
    ss_log2 = {1: 0, 2: 1, 4: 2}
    frames = [gsgen.stream_c3(i) for i in range(64)]
    backends, recorded = [], []
    try:
        for f in frames:
            be = pgs.CudaBackend(local, max_samples_log2=ss_log2[f.super_sampling], arena_mib=16)
            gs = pgs.GSInterface(be, super_sampling=f.super_sampling, ordered=f.ordered)
            be.begin_record()
            gs.gif_transfer(0, f.data)
            gs.flush()
            be.end_record()
            gs.close()
            recorded.append(be.read_plane(0))
            backends.append(be)
        for be in backends:
            be.replay(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            for be in backends:
                be.replay(1)
                torch.cuda.synchronize()
        plain_fps = len(frames) * steps / (time.perf_counter() - t0)
        batch = pgs.Batch(local)
        for be in backends:
            batch.add(be)
        batch.set_tuning(512, 2, True, 1)
        batch.replay(1)
        batch.synchronize()
        verified = all(np.array_equal(be.read_plane(0), r) for be, r in zip(backends, recorded))
        bstream = torch.cuda.ExternalStream(batch.stream(), device=local)
        flush_buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda:%d" % local)
        for _ in range(2):
            batch.replay(1)
        batch.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(bstream):
            for i in range(steps):
                flush_buf.fill_(i & 0xFF)
                ev[i][0].record(bstream)
                batch.replay(1)
                ev[i][1].record(bstream)
        batch.synchronize()
        torch.cuda.synchronize()
        total_ms = sum(a.elapsed_time(b) for a, b in ev)
        launches = batch.launches_per_replay()
        batch.close()
    finally:
        for be in backends:
            be.close()
    fps = len(frames) * steps / (total_ms / 1000.0)
    return {"workload": WORKLOADS["c3"][0], "value": fps, "unit": "frames/s", "steps": steps,
            "plain_per_frame_fps": plain_fps, "batched_vs_plain": fps / plain_fps,
            "replay_verified": verified, "gpu_launches_per_replay": launches,
            "tuning": "graph branch per stream (512 threads x 2 CTAs/SM)"}


def run_c5_bounded(local, n_eval=24, steps=10) -> dict:
    """The learned upscaler on held-out seeds: PSNR against 16x SSAA, output
    px/s of 1x render + read-out + network against exact 16x SSAA (device
    time), the network's TFLOP/s, end to end through the API from host
    buffers (GIF decode, render, read-out, network, D2H of the output image),
    and the CPU restatement of the network on one core."""
    import numpy as np
    import torch
    import pgs
    import upscaler_train as T
    dev = "cuda:%d" % local
    up = pgs.Upscaler(local)
    params = np.load(T.WEIGHTS)
    up.set_params(params)
    r = T.PairRenderer(local)
    ev_in, ev_tgt = T.build_dataset(r, range(T.EVAL_SEED0, T.EVAL_SEED0 + n_eval))
    quality = T.evaluate(up, ev_in, ev_tgt)
    r.close()
    del ev_in, ev_tgt
    frame = T.scene(T.EVAL_SEED0)
    W, H = T.WIDTH, T.HEIGHT
    paths = {}
    for ss in (1, 16):
        be = pgs.CudaBackend(local, max_samples_log2=0 if ss == 1 else 4, arena_mib=32)
        gs = pgs.GSInterface(be, super_sampling=ss, ordered=True)
        gs.write_vram(np.zeros(pgs.VRAM_SIZE, dtype=np.uint8))
        be.begin_record()
        gs.gif_transfer(0, frame.data)
        gs.flush()
        be.end_record()
        paths[ss] = (be, gs)
    img = torch.empty((1, H, W, 4), dtype=torch.uint8, device=dev)
    out = torch.empty_like(img)
    b1, b16 = paths[1][0], paths[16][0]
    s1 = torch.cuda.ExternalStream(b1.stream(), device=local)
    s16 = torch.cuda.ExternalStream(b16.stream(), device=local)
    su = torch.cuda.ExternalStream(up.stream(), device=local)
    flush_buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    # The network queues on the 1x backend's stream, right behind the frame
    # it upscales.
    def learned_once():
        b1.replay(1, reset_vram=True, use_graph=True)
        b1.sample_circuit(img.data_ptr(), 0, W // 64, 0, W, H)
        up.forward(img, out)

    def exact_once():
        b16.replay(1, reset_vram=True, use_graph=True)
        b16.sample_circuit(img.data_ptr(), 0, W // 64, 0, W, H)

    def timed(fn, start_stream, end_stream):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        total = 0.0
        for i in range(steps):
            with torch.cuda.stream(start_stream):
                flush_buf.fill_(i & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(start_stream)
            fn()
            b.record(end_stream)
            torch.cuda.synchronize()
            total += a.elapsed_time(b)
        return total / steps

    up.set_stream(b1.stream())
    learned_ms = timed(learned_once, s1, s1)
    up.set_stream(None)
    exact_ms = timed(exact_once, s16, s16)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    img_c = img.clone()
    for _ in range(3):
        up.forward(img_c, out)
    torch.cuda.synchronize()
    a.record(su)
    for _ in range(steps):
        up.forward(img_c, out)
    b.record(su)
    torch.cuda.synchronize()
    net_ms = a.elapsed_time(b) / steps
    for be, gs in paths.values():
        gs.close()
        be.close()
    # End to end from host buffers.
    be = pgs.CudaBackend(local, max_samples_log2=0, arena_mib=32)
    gs = pgs.GSInterface(be, super_sampling=1)
    host = torch.empty((1, H, W, 4), dtype=torch.uint8, pin_memory=True)
    zeros = np.zeros(pgs.VRAM_SIZE, dtype=np.uint8)
    st0 = be.stats()
    e2e_steps = steps
    up.set_stream(be.stream())
    be_stream = torch.cuda.ExternalStream(be.stream(), device=local)
    t0 = time.perf_counter()
    for k in range(e2e_steps + 1):
        if k == 1:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st0 = be.stats()
        gs.write_vram(zeros)
        gs.gif_transfer(0, frame.data)
        gs.flush()
        be.sample_circuit(img.data_ptr(), frame.meta["fbp"], W // 64, 0, W, H)
        up.forward(img, out)
        # The read-out runs on torch's own stream (after the network): the
        # pinned buffer's use is then recorded on a stream that outlives it.
        e = torch.cuda.Event()
        e.record(be_stream)
        torch.cuda.current_stream().wait_event(e)
        host.copy_(out, non_blocking=True)
        torch.cuda.synchronize()
    e2e_dt = time.perf_counter() - t0
    st1 = be.stats()
    up.set_stream(None)
    del host, img, out, img_c, flush_buf
    gs.close()
    be.close()
    up.close()
    px = W * H
    flops = 2 * 9 * px * (4 * 32 + 4 * 32 * 32 + 32 * 4)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    return {"workload": WORKLOADS["c5"][0], "value": px / (learned_ms / 1000.0), "unit": "output px/s",
            "steps": steps, "eval_seeds": n_eval,
            "psnr_db": quality["psnr_net_db"], "psnr_input_db": quality["psnr_input_db"],
            "max_abs_err": quality["max_abs_err_net"],
            "ssaa16_px_per_s": px / (exact_ms / 1000.0), "speedup_vs_ssaa16": exact_ms / learned_ms,
            "network_ms_per_frame": net_ms, "network_tflops": flops / (net_ms / 1000.0) / 1e12,
            "network_frac_of_bf16_peak": flops / (net_ms / 1000.0) / 1e12 / peak,
            "e2e": {"value": px * e2e_steps / e2e_dt, "unit": "output px/s",
                    "h2d_bytes_per_step": (st1["h2d_bytes"] - st0["h2d_bytes"]) // e2e_steps,
                    "d2h_bytes_per_step": px * 4},
            "cpu_baseline": upscaler_cpu_baseline(params)}


def upscaler_cpu_baseline(params) -> dict:
    """The network's CPU restatement (oracle/upscaler_ref.py, numpy, one
    thread) on a 160x112 crop of a frame, as output px/s."""
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
    with tempfile.NamedTemporaryFile(suffix=".npy", delete=False) as f:
        np_path = f.name
    import numpy as np
    np.save(np_path, params)
    code = ("import sys,time; sys.path.insert(0,%r); import numpy as np, upscaler_ref as R;"
            "p=np.load(%r); x=np.random.default_rng(0).integers(0,256,(1,112,160,4),dtype=np.uint8);"
            "t=time.perf_counter(); R.forward(x,p); print(160*112/(time.perf_counter()-t))") % (str(ROOT / "oracle"),
                                                                                              np_path)
    try:
        res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
        val = float(res.stdout.strip().splitlines()[-1])
        return {"value": val, "unit": "output px/s", "cores": 1, "kind": "port",
                "sample": "one 160x112 crop through the 6-layer network (numpy restatement)"}
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": "output px/s", "cores": 1, "kind": "port", "sample": "failed: %s" % e}
    finally:
        os.unlink(np_path)


def main():
    args = parse()
    rank, world, local = dist_env()
    import gsgen  # noqa: E402

    if args.workload == "c5" and args.impl != "reference":
        run_c5(args, rank, world, local)
        return
    frame = make_frame(args)
    if isinstance(frame, list) and args.impl != "reference":
        run_c3(args, frame, rank, world, local)
        return

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, frame)))
        return

    import numpy as np
    import torch
    import pgs

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist

    e2e_steps = 0 if args.quick else max(5, min(2 * args.steps, 40))
    m = measure_frame(frame, local, args.steps, args.warmup, e2e_steps, verify=not args.no_verify and rank == 0,
                      pg=pg)
    total_ms = m["total_ms"]
    fps = replica_throughput(args.steps, world, total_ms)
    e2e_fps = world * m["e2e_fps_per_rank"] if m["e2e_fps_per_rank"] else None
    h2d, d2h = m["h2d"], m["d2h"]
    frags_per_frame = m["frags_per_frame"]
    shade_ms = [m["shade_ms"]]
    verified = m["verified"]
    launches = m["launches"]
    clk = m["clocks"]
    extras = None if (args.quick or args.no_extra or rank != 0) else extra_workloads(local)

    if rank != 0:
        if pg:
            pg.barrier()
        return

    ab = algorithmic_bytes(frame, frame.super_sampling)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak_gbs = peaks.get("hbm_gbs", 6800.0)
    frags = frags_per_frame
    shade_s = statistics.mean(shade_ms) / 1000.0
    achieved = ab["shade"] / shade_s / 1e9
    cpu = None if (args.quick or args.no_cpu_baseline) else cpu_baseline_sample(args)
    out = {
        "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32+fp32", "data": "synthetic (seeded GS command stream)",
        "config": dict(workload_config(args, frame), l2="flushed (256 MiB write) between steps",
                       parallelism="replicas" if world > 1 else "single"),
        "gfrag_per_s": frags * fps / 1e9,
        "fragments_per_frame": frags,
        "shade_ms_per_frame": statistics.mean(shade_ms),
        "replay_verified": verified,
        "gpu_launches": launches * args.steps,
        "clocks": clk,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                     "frac": achieved / peak_gbs,
                     "traffic": profiled_traffic("shade_kernel_c2.md") if args.workload == "c2" else None,
                     "shade_bytes_per_frame": ab["shade"],
                     "note": "algorithmic bytes of the shading kernels per frame / their CUDA-event time "
                             "inside the timed replays; peak = measured hbm_gbs (of measured)"},
        "issue_roofline": issue_roofline(profiled_instructions("shade_kernel_c2.md") if args.workload == "c2"
                                         else None, shade_s, clk),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                # Host time per frame inside the API calls (GIF decode, records,
                # submission), against which the device time per frame runs.
                "host_ms_per_frame": m["e2e_host_ms"]},
        "workloads": extras,
    }
    print(json.dumps(out))
    if pg:
        pg.barrier()


if __name__ == "__main__":
    main()
