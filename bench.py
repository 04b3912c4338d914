"""Benchmark of the GB300 rendering backend (one JSON line on stdout).

Workload (default): the 1024x1024 plain-render scene — 2000 gradient fills
(linear/radial, 2-8 stops, pad/reflect/repeat, affine gradientTransform),
500 stroked open cubics, 20 nested clip groups and 10 luminance masks — from
the seeded generator (resvg_gb300/csrc/host/gen.cpp).  One step = one render of
that scene.

  value  scenes/s of the device path: a prepared scene (records resident in
         HBM) rendered into a device pixmap; every pipeline kernel runs each
         step (edge build, binning, band raster), replayed from a CUDA graph.
         Timed per step with CUDA events; L2 is flushed between steps.
  e2e    scenes/s through the drop-in C ABI call resvg_render with a host
         pixmap: host flattening, record + pixmap upload, kernels, pixmap
         download, all inside the timed region.

With --gpus N under torchrun each rank renders its own scene (replicas; the
units are independent scenes, no collective on the data path).
--impl reference times the CPU restatement of resvg's renderer on all host
cores (resvg itself cannot be built without a Rust toolchain).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIG_DESC = {
    0: "512x512, 200 solid cubic loops (non-zero/even-odd), source-over",
    1: "1024x1024, 2000 gradient fills + 500 strokes + 20 nested clips + 10 luminance masks",
    2: "2048x2048, 500 cubic loops + blur/saturate/morphology/arithmetic filter chain (linearRGB)",
    3: "batched: 4096 scenes, side log-uniform 64-1024, paths log-uniform 10-2000 (config-1 paint mix, "
       "20% strokes, 10% with a clip and a blur)",
    4: "differentiable: 256 scenes of 256x256, 64 closed cubic paths (4-16 segments), solid/4-stop linear "
       "gradient paints, one Gaussian blur (learnable sigma), L2 loss against a perturbed target",
}
# (band rows, pixels per thread); band rows 0 = chosen per stream from its width
TUNING_CANDIDATES = [(0, 8), (0, 16), (1, 4), (2, 4), (4, 4), (2, 8), (4, 8), (8, 8), (4, 16), (8, 16)]
SEED = 2026


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--scenes", type=int, default=4096, help="scenes per step of the batched form (config 3)")
    ap.add_argument("--plain-sample", type=int, default=128,
                    help="scenes rendered one by one through the plain drop-in for the batched comparison")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="path-count scale of the workload (1.0 = the full workload; smaller only for profiling)")
    return ap.parse_args()


def dist_setup(n, backend="nccl"):
    """(rank, world) from the torchrun environment; joins the process group
    when world > 1 (one rank per GPU over NCCL; `gloo` for CPU-only runs)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        if backend == "nccl":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    return rank, world


def max_over_ranks(ms, world, device):
    """The slowest rank's step time: every rank reports the job's time."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def shard(rank, n):
    """Scene indices of a rank in the batched form: disjoint, n per rank."""
    return [rank * n + i for i in range(n)]


def _smi_index():
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if lr < len(ids):
            return ids[lr]
    return str(lr)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", _smi_index(),
                                      "--query-gpu=" + self.Q, "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(config):
    """DRAM bytes per raster launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "raster_traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh).get("config%d" % config)
    except Exception:
        return None


def cpu_baseline(tree, w, h):
    import oracle
    t0 = time.perf_counter()
    oracle.render(tree.view(), (1, 0, 0, 1, 0, 0), w, h)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "scenes/s", "cores": 1, "kind": "port",
            "sample": "one full scene rendered single-threaded by the C++ restatement of resvg+tiny-skia "
                      "(%.1f s)" % dt}


def run_reference(args, rank, world):
    """CPU restatement of resvg's renderer on all host cores."""
    if rank != 0:
        return
    import oracle
    import resvg_gb300 as R
    oracle.lib()
    if args.config in (3, 4):
        run_reference_batched(args)
        return
    tree = R.Tree.generate(args.config, seed=SEED, index=0, scale=1.0)
    w, h = (int(v) for v in tree.size)
    threads = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.render_parallel(tree.view(), (1, 0, 0, 1, 0, 0), w, h, threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    ms = 1e3 * sum(times) / len(times)
    value = 1e3 / ms
    line = {"metric": "scenes/s (plain render, config %d)" % args.config, "value": value, "unit": "scenes/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "config%d: %s" % (args.config, CONFIG_DESC.get(args.config, "")),
                       "mpix_per_scene": w * h / 1e6},
            "mpix_s": value * w * h / 1e6,
            "cpu_baseline": {"value": value, "unit": "scenes/s", "cores": threads, "kind": "port",
                             "sample": "one full scene per step, canvas split into %d row strips rendered on %d "
                                       "threads by the C++ restatement of resvg+tiny-skia" % (threads, threads)},
            "e2e": {"value": value, "unit": "scenes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_batched(args):
    """Reference arm of the batched (config 3) and differentiable (config 4)
    forms: the CPU restatement on a bounded sample per step, all host cores
    for config 3, one core for the FP64 soft reference of config 4."""
    import resvg_gb300 as R
    steps = []
    if args.config == 3:
        trees = [R.Tree.generate(3, seed=SEED, index=i, scale=args.scale) for i in range(args.scenes)]
        sizes = [tuple(int(v) for v in t.size) for t in trees]
        for i in range(args.warmup + args.steps):
            cb = cpu_baseline_batch(trees, sizes, budget_s=5.0)
            if i >= args.warmup:
                steps.append(cb)
        metric = "scenes/s (batched render, config 3)"
    else:
        from resvg_gb300 import soft
        a = soft.make_scenes(seed=SEED, scenes=256, size=256, paths=64)
        t = soft.perturb(a, seed=SEED + 1000)
        for i in range(args.warmup + args.steps):
            cb = cpu_baseline_soft(a, t, scenes=2)
            if i >= args.warmup:
                steps.append(cb)
        metric = "grads/s (scenes x (forward + adjoint) per second, config 4)"
    value = sum(c["value"] for c in steps) / len(steps)
    cb = dict(steps[-1])
    cb["value"] = value
    line = {"metric": metric, "value": value, "unit": "scenes/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8" if args.config == 3 else "f64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "config%d: %s" % (args.config, CONFIG_DESC.get(args.config, ""))},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "scenes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batched(args, rank, world):
    """Config 3: thousands of independent scenes in one prepared submission
    (one persistent raster kernel per stage, CUDA-graph replay), against the
    same scenes rendered one call at a time through the plain GPU drop-in."""
    import torch
    import resvg_gb300 as R
    from resvg_gb300 import build as B
    B.build()
    R.init(0)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    n = args.scenes
    trees = [R.Tree.generate(3, seed=SEED, index=i, scale=args.scale) for i in shard(rank, n)]
    sizes = [tuple(int(v) for v in t.size) for t in trees]
    offs, total = [], 0
    for w, h in sizes:
        offs.append(total)
        total += ((w * h * 4 + 255) // 256) * 256
    buf = torch.zeros(total, dtype=torch.uint8, device=dev)
    base = buf.data_ptr()
    ptrs = [base + o for o in offs]
    ws = [w for w, _ in sizes]
    hs = [h for _, h in sizes]
    ident = [(1, 0, 0, 1, 0, 0)] * n
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    # autotune the raster decomposition on a stratified sample of the scenes
    samp = list(range(0, n, max(1, n // 256)))
    t0 = time.perf_counter()
    best, best_ms = R.autotune([trees[i] for i in samp], [ident[i] for i in samp], [ws[i] for i in samp],
                               [hs[i] for i in samp], [ptrs[i] for i in samp], TUNING_CANDIDATES, reps=2)
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    scene = R.Scene(trees, ident, ws, hs, ptrs)
    prep_s = time.perf_counter() - t0

    def step():
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        scene.render(sh)
        s1.record(stream)
        return s0, s1

    for _ in range(args.warmup):
        step()
        scene.check()
    info = scene.info()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms = []
    with ClockSampler() as clk:
        for _ in range(args.steps):
            s0, s1 = step()
            scene.check()
            step_ms.append(s0.elapsed_time(s1))
        torch.cuda.synchronize()
    ms = max_over_ranks(sum(step_ms) / len(step_ms), world, dev)
    value = world * n * 1e3 / ms
    out_px = sum(w * h for w, h in sizes)
    # plain per-scene drop-in (device pixmap, one call per scene, synchronised)
    psamp = list(range(0, n, max(1, n // max(1, args.plain_sample))))
    for i in psamp[:4]:
        R.render_device(trees[i], ident[i], ws[i], hs[i], ptrs[i], ws[i] * 4, sh)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_raster_ms = 0.0
    for i in psamp:
        R.render_device(trees[i], ident[i], ws[i], hs[i], ptrs[i], ws[i] * 4, sh)
        stream.synchronize()
        plain_raster_ms += R.stats()["raster_ms"]
    plain_s = time.perf_counter() - t0
    plain_value = len(psamp) / plain_s
    # end to end through the public batch call: flatten + upload + render + read back every output
    pinned = torch.empty(total, dtype=torch.uint8, pin_memory=True)
    e2e_t = []
    for _ in range(max(1, args.e2e_steps if args.e2e_steps < 5 else 1)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        R.render_batch(trees, ident, ws, hs, ptrs, sh)
        pinned.copy_(buf, non_blocking=True)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * sum(e2e_t) / len(e2e_t)
    st = R.stats()
    # raster-kernel device time for the roofline (un-captured renders, events
    # around the raster launches of every level)
    scene.set_timing(True)
    raster_ms = []
    for _ in range(2):
        step()
        raster_ms.append(scene.check())
    scene.set_timing(False)
    rms = sum(raster_ms) / len(raster_ms)
    alg_bytes = info["output_pixels"] * 8 + info["binned_edges"] * 16 + info["record_bytes"] + \
        info["layer_pixels"] * 8
    peak, peak_kind = peaks()
    achieved = alg_bytes / (rms * 1e-3) / 1e9
    line = {
        "metric": "scenes/s (batched render, config 3)", "value": value, "unit": "scenes/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded generator, seed %d)" % SEED,
        "config": {"workload": "config3: %s" % CONFIG_DESC[3], "scenes": n, "output_mpix": out_px / 1e6,
                   "draws": info["draws"], "edges": info["edges"], "binned_edges": info["binned_edges"],
                   "work_items": info["work_items"], "tuning": {"band_rows": best[0], "pixels_per_thread": best[1],
                                                                "autotune_ms_on_sample": best_ms,
                                                                "autotune_s": tune_s},
                   "prepare_s": prep_s, "l2": "outputs %.1f GB > L2" % (total / 1e9), "graph_replay": True},
        "mpix_s": value * out_px / n / 1e6 if n else 0.0,
        "plain": {"value": plain_value, "unit": "scenes/s", "sample_scenes": len(psamp),
                  "raster_kernel_share": plain_raster_ms * 1e-3 / plain_s,
                  "how": "rgpu_render_device per scene (host flatten + upload + kernels), synchronised"},
        "batched_vs_plain": value / plain_value,
        "raster_ms": rms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None, "kernel": "k_raster (band VM)",
                     "algorithmic_bytes": alg_bytes},
        "e2e": {"value": n * 1e3 / e2e_ms, "unit": "scenes/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(st["h2d_bytes"]), "d2h_bytes_per_step": int(total)},
        "gpu_launches": int(info["kernel_launches"]) * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_batch(trees, sizes, budget_s=10.0)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline_batch(trees, sizes, budget_s=10.0, threads=None):
    """The C++ restatement over a stratified sample of the batch (every k-th
    scene, until about `budget_s` of CPU time), each scene split into row
    strips over `threads` host threads: scenes/s of the sample."""
    import oracle
    threads = threads or os.cpu_count() or 1
    n = len(trees)
    order = [i for k in range(16) for i in range(k, n, 16)]
    done, pixels, t_all = 0, 0, 0.0
    for i in order:
        w, h = sizes[i]
        t0 = time.perf_counter()
        oracle.render_parallel(trees[i].view(), (1, 0, 0, 1, 0, 0), w, h, threads)
        t_all += time.perf_counter() - t0
        done += 1
        pixels += w * h
        if t_all >= budget_s:
            break
    return {"value": done / t_all, "unit": "scenes/s", "cores": threads, "kind": "port",
            "sample": "%d of %d scenes (every 16th first, %.1f Mpx), each in row strips on %d threads, by the C++ "
                      "restatement of resvg+tiny-skia (%.1f s)" % (done, n, pixels / 1e6, threads, t_all)}


def _soft_slice(arr, scenes):
    """The first `scenes` scenes of a soft-renderer batch (host arrays)."""
    P = int(arr["paths"])
    segs_end = int(arr["seg_offset"][scenes * P])
    out = dict(arr)
    out["scenes"] = scenes
    out["seg_offset"] = np.ascontiguousarray(arr["seg_offset"][:scenes * P + 1])
    out["points"] = np.ascontiguousarray(arr["points"][:3 * segs_end])
    for k in ("paint_kind", "colors", "stop_offsets", "stop_colors", "grad_line"):
        out[k] = np.ascontiguousarray(arr[k][:scenes * P])
    out["sigma"] = np.ascontiguousarray(arr["sigma"][:scenes])
    return out


def cpu_baseline_soft(a, t_arrays, scenes=4):
    """The FP64 C++ reference of the soft renderer on `scenes` scenes, one core:
    forward, loss and one directional derivative per scene (a full gradient by
    forward mode would take one such pass per parameter)."""
    import oracle
    sub = _soft_slice(a, scenes)
    _, target = oracle.soft_forward(_soft_slice(t_arrays, scenes))
    direction = {"colors": np.ones_like(sub["colors"], dtype=np.float64)}
    t0 = time.perf_counter()
    oracle.soft_dloss(sub, target.astype(np.float32), direction)
    dt = time.perf_counter() - t0
    return {"value": scenes / dt, "unit": "scenes/s", "cores": 1, "kind": "port",
            "sample": "%d scenes: FP64 forward + loss + one directional derivative (C++ reference, %.1f s)" %
                      (scenes, dt)}


def run_soft(args, rank, world):
    """Config 4: forward soft-coverage render + hand-written adjoint of an L2
    loss over 256 scenes; one step = forward, loss and all parameter gradients."""
    import torch
    from resvg_gb300 import build as B
    from resvg_gb300 import soft
    import resvg_gb300 as R
    B.build()
    R.init(0)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    a = soft.make_scenes(seed=SEED + rank, scenes=256, size=256, paths=64)
    t = soft.perturb(a, seed=SEED + 1000 + rank)
    sc, tgt = soft.Scenes(a), soft.Scenes(t)
    _, target = soft.forward(tgt)

    def step():
        image, blurred = soft.forward(sc)
        loss, g = soft.mse(blurred, target)
        return loss, soft.backward(sc, image, g)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ms_list = []
    with ClockSampler() as clk:
        for _ in range(args.steps):
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record()
            loss, grads = step()
            s1.record()
            torch.cuda.synchronize()
            ms_list.append(s0.elapsed_time(s1))
    ms = max_over_ranks(sum(ms_list) / len(ms_list), world, dev)
    value = world * 256 * 1e3 / ms
    # end to end: parameters from pinned host memory, gradients back to the host
    host = {k: torch.from_numpy(np.ascontiguousarray(a[k])).pin_memory() for k in soft.PARAMS}
    e2e = []
    for _ in range(max(1, min(args.e2e_steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in soft.PARAMS:
            sc.params[k].copy_(host[k], non_blocking=True)
        loss, grads = step()
        out = {k: grads[k].to("cpu", non_blocking=True) for k in soft.PARAMS}
        torch.cuda.synchronize()
        e2e.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * sum(e2e) / len(e2e)
    h2d = sum(int(host[k].numel()) * 4 for k in soft.PARAMS)
    line = {
        "metric": "grads/s (scenes x (forward + adjoint) per second, config 4)", "value": value,
        "unit": "scenes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, seed %d)" % SEED,
        "config": {"workload": "config4: %s" % CONFIG_DESC[4], "scenes": 256, "canvas": [256, 256], "paths": 64,
                   "segments": int(a["seg_offset"][-1]), "loss": loss},
        "mpix_s": value * 256 * 256 / 1e6,
        "e2e": {"value": 256 * 1e3 / e2e_ms, "unit": "scenes/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d},
        "gpu_launches": 12 * args.steps,
        "clocks": clk.summary(),
    }
    # the soft renderer is FP32-ALU bound; the HBM line is reported for
    # completeness: parameters + target + image + blurred image + gradients
    peak, peak_kind = peaks()
    alg_bytes = 2 * h2d + 3 * 256 * 256 * 256 * 16
    line["roofline"] = {"bound": "hbm", "achieved": alg_bytes / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": alg_bytes / (ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind, "traffic": None,
                        "kernel": "soft forward + adjoint (one step)", "algorithmic_bytes": alg_bytes}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_soft(a, t)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    rank, world = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.config == 3:
        run_batched(args, rank, world)
        return
    if args.config == 4:
        run_soft(args, rank, world)
        return
    import torch
    import resvg_gb300 as R
    from resvg_gb300 import build as B
    B.build()
    R.init(0)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    tree = R.Tree.generate(args.config, seed=SEED, index=rank, scale=args.scale)
    w, h = (int(v) for v in tree.size)
    surface = torch.zeros((h, w, 4), dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    scene = R.Scene([tree], [(1, 0, 0, 1, 0, 0)], [w], [h], [surface.data_ptr()])
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def step():
        surface.zero_()
        flush.zero_()
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        scene.render(sh)
        s1.record(stream)
        return s0, s1

    for _ in range(args.warmup):
        step()
        scene.check()
    info = scene.info()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms = []
    with ClockSampler() as clk:
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            s0, s1 = step()
            scene.check()
            step_ms.append(s0.elapsed_time(s1))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    # raster-kernel device time for the roofline: un-captured renders with
    # events around the kernel (same buffers and inputs)
    scene.set_timing(True)
    raster_ms = []
    for _ in range(max(3, args.steps // 4)):
        step()
        raster_ms.append(scene.check())
    scene.set_timing(False)
    if world > 1:
        torch.distributed.barrier()
    ms = max_over_ranks(sum(step_ms) / len(step_ms), world, dev)
    value = world * 1e3 / ms
    rms = sum(raster_ms) / len(raster_ms)

    # ---- end to end through the drop-in C ABI (host pixmap)
    host = np.zeros((h, w, 4), dtype=np.uint8)
    for _ in range(2):
        R.render(tree, (1, 0, 0, 1, 0, 0), pixmap=host)
    e2e_t = [float("nan")]
    if args.e2e_steps:
        e2e_t = []
    for _ in range(args.e2e_steps):
        host[:] = 0
        t0 = time.perf_counter()
        R.render(tree, (1, 0, 0, 1, 0, 0), pixmap=host)
        e2e_t.append(time.perf_counter() - t0)
    st = R.stats()
    e2e_ms = 1e3 * sum(e2e_t) / len(e2e_t)

    # ---- roofline of the raster kernel (algorithmic bytes per launch)
    out_px = info["output_pixels"]
    alg_bytes = out_px * 8 + info["binned_edges"] * 16 + info["record_bytes"] + info["layer_pixels"] * 8
    peak, peak_kind = peaks()
    achieved = alg_bytes / (rms * 1e-3) / 1e9
    line = {
        "metric": "scenes/s (plain render, config %d)" % args.config,
        "value": value, "unit": "scenes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded generator, seed %d)" % SEED,
        "config": {"workload": "config%d: %s" % (args.config, CONFIG_DESC.get(args.config, "")),
                   "canvas": [w, h], "draws": info["draws"], "edges": info["edges"],
                   "binned_edges": info["binned_edges"], "work_items": info["work_items"],
                   "l2": "flushed between steps (256 MB write)", "graph_replay": True},
        "mpix_s": value * out_px / 1e6,
        "raster_ms": rms,
        "wall_s_timed_region": t_wall,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": profiled_traffic(args.config),
                     "kernel": "k_raster (band VM)", "algorithmic_bytes": alg_bytes},
        "e2e": {"value": 1e3 / e2e_ms, "unit": "scenes/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(st["h2d_bytes"]), "d2h_bytes_per_step": int(st["d2h_bytes"])},
        "gpu_launches": int(info["kernel_launches"]) * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(tree, w, h)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
