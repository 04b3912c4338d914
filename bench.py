"""Benchmark of the GB300 rendering backend (one JSON line on stdout).

Workload (default, --config 3): the batched form.  4096 independent scenes in
one submission, canvas side log-uniform in 64..1024 px, path count
log-uniform in 10..2000, the 1024^2 paint mix (solid, linear and radial
gradient fills, 20% strokes), 10% of scenes with one clip and one Gaussian
blur, from the seeded generator (resvg_gb300/csrc/host/gen.cpp).  One step =
one render of the whole batch.

  value      scenes/s of the device path: the batch prepared once (records
             resident in HBM) and rendered by CUDA-graph replay; every
             pipeline kernel runs each step.  Outputs (3.1 GB) exceed L2.
  plain      scenes/s of the same scenes rendered one call at a time through
             the plain per-scene GPU drop-in (rgpu_render_device), on a
             stratified sample; batched_vs_plain = value / plain.
  e2e        scenes/s through the public batch call rgpu_render_batch: host
             flattening, record upload, kernels, and a device->host read of
             every output pixmap, all inside the timed region.
  parity     the timed output compared with the oracle on every scene the CPU
             baseline renders.

--config 0/1/2 time one plain scene (512^2 cubic loops; 1024^2 gradients,
strokes, 20 nested clips and 10 luminance masks; 2048^2 filter chain) by
graph replay, e2e through resvg_render with a host pixmap.  --config 4 times
the differentiable form.

With --gpus N under torchrun the batch is split over the ranks by estimated
cost (greedy LPT on pixels x paths), with no collective on the data path:
value = the whole batch / the slowest rank's step time (strong scaling).
--impl reference times the CPU restatement of resvg's renderer (the oracle)
on all host cores; resvg itself cannot be built without a Rust toolchain.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
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
    3: "batched: 4096 scenes, side log-uniform 64-1024, paths log-uniform 10-2000 (1024^2 paint mix, "
       "20% strokes, 10% with a clip and a blur)",
    4: "differentiable: 256 scenes of 256x256, 64 closed cubic paths (4-16 segments), solid/4-stop linear "
       "gradient paints, one Gaussian blur (learnable sigma), L2 loss against a perturbed target",
}
SEED = 2026
IDENT = (1, 0, 0, 1, 0, 0)


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--scenes", type=int, default=4096, help="scenes per step of the batched form (config 3)")
    ap.add_argument("--plain-sample", type=int, default=128,
                    help="scenes rendered one by one through the plain drop-in for the batched comparison")
    ap.add_argument("--cpu-budget", type=float, default=12.0,
                    help="seconds of CPU work for the oracle baseline sample")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="path-count scale of configs 0-2 (1.0 = the full workload; smaller only for profiling)")
    ap.add_argument("--profile", action="store_true",
                    help="for ncu captures: prepare the workload, render it twice (the sizing render, then the "
                         "one to capture, k_raster launches 1 + levels onwards) and exit")
    ap.add_argument("--tuning", type=str, default="",
                    help="with --profile: band rows and pixels per thread ('4,8'), the choice the timed run's "
                         "autotuner made (the bench line's config.tuning)")
    return ap.parse_args(argv)


# ---------------------------------------------------------------------------- ranks

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


def batch_shard(rank, world, n, seed=SEED):
    """Scene indices of this rank: one n-scene batch split over `world` ranks
    by estimated cost (greedy LPT on side^2 x paths)."""
    from resvg_gb300 import batch as B
    if world <= 1:
        return list(range(n))
    return B.lpt_partition(B.config3_costs(seed, n), world)[rank]


# ---------------------------------------------------------------------------- records

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
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _raster_profile():
    try:
        with open(os.path.join(ROOT, "profiles", "raster_traffic.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


def profiled_traffic(key):
    """DRAM bytes per raster launch from the committed ncu summary, if any."""
    return _raster_profile().get(key)


def profiled_issue(key):
    """The raster kernel's issue-rate roof from the committed ncu summary:
    warp instructions issued / (elapsed SM cycles x 4 schedulers x SMs)."""
    return _raster_profile().get("issue", {}).get(key)


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def host_info():
    """CPU model, architecture and core count of the host the baseline ran on."""
    model = None
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
    except Exception:
        pass
    if not model:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=5).stdout
            for line in out.splitlines():
                if line.startswith("Model name:"):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return {"cpu_model": model or platform.processor() or "unknown", "arch": platform.machine(),
            "nproc": os.cpu_count(), "affinity": host_threads()}


def parity_record(pairs):
    """{"differing_px", "max_delta", ...} over (gpu image, oracle image) pairs."""
    n = mx = px = 0
    scenes_bad = 0
    for g, o in pairs:
        d = np.abs(g.astype(np.int16) - o.astype(np.int16)).max(axis=-1)
        k = int((d > 0).sum())
        n += k
        mx = max(mx, int(d.max()) if d.size else 0)
        px += d.size
        scenes_bad += k > 0
    return {"differing_px": n, "max_delta": mx, "pixels_compared": px, "scenes_compared": len(pairs),
            "scenes_differing": scenes_bad, "oracle": "C++ restatement of resvg + tiny-skia (oracle/)"}


# ---------------------------------------------------------------------------- CPU oracle legs

def cpu_sample_order(n):
    """Stratified order over a batch: every 16th scene first, then the next offset."""
    return [i for k in range(16) for i in range(k, n, 16)]


def cpu_render_sample(trees, sizes, order, budget_s, threads, start=0):
    """Renders scenes of `order` (from `start`) with the oracle, whole scenes in
    parallel over `threads` host threads, chunk by chunk until about
    `budget_s` of wall time.  Returns (rendered indices, images, seconds,
    next start)."""
    import oracle
    done, images, t_all = [], [], 0.0
    pos = start
    chunk = max(1, 2 * threads)
    while pos < len(order) and t_all < budget_s:
        idx = order[pos:pos + chunk]
        pos += len(idx)
        t0 = time.perf_counter()
        ims = oracle.render_many([trees[i].view() for i in idx], [IDENT] * len(idx), [sizes[i] for i in idx],
                                 threads)
        t_all += time.perf_counter() - t0
        done += idx
        images += ims
    return done, images, t_all, pos


def cpu_baseline_batch(trees, sizes, budget_s, threads=None):
    """The oracle over a stratified sample of the batch, whole scenes in
    parallel over all host threads (resvg renders one tree per call, so a CPU
    batch parallelises over scenes): scenes/s of the sample.  Also returns
    the sample's images for the parity check."""
    threads = threads or host_threads()
    order = cpu_sample_order(len(trees))
    done, images, t_all, _ = cpu_render_sample(trees, sizes, order, budget_s, threads)
    px = sum(sizes[i][0] * sizes[i][1] for i in done)
    cb = {"value": len(done) / t_all, "unit": "scenes/s", "cores": threads, "kind": "port",
          "sample": "%d of %d scenes (every 16th first, %.1f Mpx), whole scenes in parallel on %d threads, by the "
                    "C++ restatement of resvg+tiny-skia (%.1f s)" % (len(done), len(trees), px / 1e6, threads,
                                                                       t_all),
          "host": host_info()}
    return cb, dict(zip(done, images))


def cpu_baseline_single(tree, w, h):
    """One full scene rendered single-threaded by the oracle (resvg renders one
    tree per call on one thread).  Returns (record, image)."""
    import oracle
    t0 = time.perf_counter()
    img = oracle.render(tree.view(), IDENT, w, h)
    dt = time.perf_counter() - t0
    return ({"value": 1.0 / dt, "unit": "scenes/s", "cores": 1, "kind": "port",
             "sample": "one full scene rendered single-threaded by the C++ restatement of resvg+tiny-skia "
                       "(%.1f s)" % dt, "host": host_info()}, img)


# ---------------------------------------------------------------------------- reference arm

def run_reference(args, rank, world):
    """The CPU restatement of resvg's renderer on all host cores, on this
    arm's workload.  Loads only the oracle library (its own copy of the scene
    generator), never the product library."""
    if rank != 0:
        return
    import oracle
    oracle.lib()
    threads = host_threads()
    if args.config == 3:
        trees = [oracle.GeneratedTree(3, SEED, i) for i in range(args.scenes)]
        sizes = [tuple(int(v) for v in t.size) for t in trees]
        order = cpu_sample_order(len(trees))
        pos, scenes, secs = 0, 0, 0.0
        per_step = max(1.0, 120.0 / max(1, args.warmup + args.steps))
        for i in range(args.warmup + args.steps):
            if pos >= len(order):
                pos = 0
            done, _, dt, pos = cpu_render_sample(trees, sizes, order, per_step, threads, start=pos)
            if i >= args.warmup:
                scenes += len(done)
                secs += dt
        value = scenes / secs
        metric = "scenes/s (batched render, 4096-scene workload)"
        sample = ("%d scenes of the %d-scene batch over %d steps (stratified order, ~%.1f s per step), whole "
                  "scenes in parallel on %d threads" % (scenes, len(trees), args.steps, per_step, threads))
        dtype = "u8"
        cfg = {"workload": "config3: %s" % CONFIG_DESC[3], "scenes": args.scenes}
    elif args.config == 4:
        from resvg_gb300 import soft
        a = soft.make_scenes(seed=SEED, scenes=256, size=256, paths=64)
        t = soft.perturb(a, seed=SEED + 1000)
        vals = []
        for i in range(args.warmup + args.steps):
            cb = cpu_baseline_soft(a, t, scenes=2)
            if i >= args.warmup:
                vals.append(cb["value"])
        value = sum(vals) / len(vals)
        metric = "grads/s (scenes x (forward + adjoint) per second, config 4)"
        sample = cb["sample"]
        threads = 1
        dtype = "f64"
        cfg = {"workload": "config4: %s" % CONFIG_DESC[4]}
    else:
        tree = oracle.GeneratedTree(args.config, SEED, 0, args.scale)
        w, h = (int(v) for v in tree.size)
        times = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            oracle.render_parallel(tree.view(), IDENT, w, h, threads)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                times.append(dt)
        value = len(times) / sum(times)
        metric = "scenes/s (plain render, config %d)" % args.config
        sample = ("one full scene per step, canvas split into %d row strips rendered on %d threads by the C++ "
                  "restatement of resvg+tiny-skia" % (threads, threads))
        dtype = "u8"
        cfg = {"workload": "config%d: %s" % (args.config, CONFIG_DESC[args.config]), "canvas": [w, h]}
    line = {"metric": metric, "value": value, "unit": "scenes/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True,
            "scaling": "strong" if args.config == 3 else "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded generator, seed %d)" % SEED, "config": cfg,
            "cpu_baseline": {"value": value, "unit": "scenes/s", "cores": threads, "kind": "port",
                             "sample": sample, "host": host_info()},
            "e2e": {"value": value, "unit": "scenes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------- batched form (default)

def run_batched(args, rank, world):
    """Thousands of independent scenes in one prepared submission (one
    persistent raster kernel per dependency level, CUDA-graph replay), against
    the same scenes rendered one call at a time through the plain drop-in."""
    import torch
    import resvg_gb300 as R
    from resvg_gb300 import build as B
    from resvg_gb300 import batch as BT
    B.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    R.init(0)
    n_total = args.scenes
    mine = batch_shard(rank, world, n_total)
    trees = [R.Tree.generate(3, seed=SEED, index=i) for i in mine]
    n = len(trees)
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
    ident = [IDENT] * n
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    # autotune the raster decomposition on a stratified sample of the scenes:
    # band rows per (canvas-width, draw-count) bucket, then pixels per thread
    samp = list(range(0, n, max(1, n // 256)))
    t0 = time.perf_counter()
    table, best_px, tune_ms = BT.autotune_table([trees[i] for i in samp], [ws[i] for i in samp],
                                                [hs[i] for i in samp], [ptrs[i] for i in samp], reps=2)
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

    stroke = warmup_with_stroke_record(step, scene, args.warmup)
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
    value = n_total * 1e3 / ms
    out_px = sum(w * h for w, h in sizes)

    # one render from cleared pixmaps through the same graph, kept for the parity check
    buf.zero_()
    torch.cuda.synchronize()
    step()
    scene.check()

    def image(i):
        w, h = sizes[i]
        return buf[offs[i]:offs[i] + w * h * 4].cpu().numpy().reshape(h, w, 4)

    line_cb, parity = None, None
    if rank == 0 and not args.no_cpu_baseline:
        cb, ref_images = cpu_baseline_batch(trees, sizes, budget_s=args.cpu_budget)
        parity = parity_record([(image(i), ref_images[i]) for i in sorted(ref_images)])
        if world == 1:
            line_cb = cb

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
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        R.render_batch(trees, ident, ws, hs, ptrs, sh)
        pinned.copy_(buf, non_blocking=True)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    e2e_ms = max_over_ranks(1e3 * sum(e2e_t) / len(e2e_t), world, dev)
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
        "metric": "scenes/s (batched render, 4096-scene workload)", "value": value, "unit": "scenes/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded generator, seed %d)" % SEED,
        "config": {"workload": "config3: %s" % CONFIG_DESC[3], "scenes": n_total, "scenes_this_rank": n,
                   "split": "LPT on side^2 x paths" if world > 1 else "one GPU",
                   "output_mpix": out_px / 1e6, "draws": info["draws"], "edges": info["edges"],
                   "binned_edges": info["binned_edges"], "work_items": info["work_items"],
                   "tuning": {"table": [list(e) for e in table], "pixels_per_thread": best_px,
                              "autotune_ms_on_sample": min(min(v.values()) for v in tune_ms.values()),
                              "autotune_s": tune_s,
                              "buckets": "width <= %s x draws <= %s" % (list(BT.WIDTH_BUCKETS),
                                                                        list(BT.DRAW_BUCKETS))},
                   "prepare_s": prep_s, "stroke": stroke, "l2": "outputs %.1f GB > L2 (129 MB)" % (total / 1e9),
                   "graph_replay": True},
        "mpix_s": value * out_px / n / 1e6 if n else 0.0,
        "plain": {"value": plain_value, "unit": "scenes/s", "sample_scenes": len(psamp),
                  "raster_kernel_share": plain_raster_ms * 1e-3 / plain_s,
                  "how": "rgpu_render_device per scene (host flatten + upload + kernels), synchronised"},
        "batched_vs_plain": value / plain_value / max(1, world),
        "raster_ms": rms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": profiled_traffic("config3"), "kernel": "k_raster (band VM)",
                     "algorithmic_bytes": alg_bytes, "issue_roof": profiled_issue("config3")},
        "e2e": {"value": n_total * 1e3 / e2e_ms, "unit": "scenes/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(st["h2d_bytes"]), "d2h_bytes_per_step": int(total),
                "how": "rgpu_render_batch (host flatten + record upload + kernels) + read-back of every pixmap"},
        "gpu_launches": int(info["kernel_launches"]) * args.steps,
        "clocks": clk.summary(),
        "parity": parity,
    }
    if line_cb is not None:
        line["cpu_baseline"] = line_cb
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------- differentiable form

def _soft_slice(arr, scenes):
    """The first `scenes` scenes of a soft-renderer batch (host arrays)."""
    P = int(arr["paths"])
    segs_end = int(arr["seg_offset"][scenes * P])
    out = dict(arr)
    out["scenes"] = scenes
    out["seg_offset"] = np.ascontiguousarray(arr["seg_offset"][:scenes * P + 1])
    out["points"] = np.ascontiguousarray(arr["points"][:3 * segs_end])
    for k in ("paint_kind", "colors", "stop_offsets", "stop_colors", "grad_line", "opacity"):
        out[k] = np.ascontiguousarray(arr[k][:scenes * P])
    out["sigma"] = np.ascontiguousarray(arr["sigma"][:scenes])
    return out


def cpu_baseline_soft(a, t_arrays, scenes=4):
    """The FP64 C++ reference of the soft renderer on `scenes` scenes, one core:
    forward, loss and one directional derivative per scene.  The reference is
    forward mode, so a full gradient costs one such pass per parameter;
    `value` is the directional rate and `full_gradient_value` the rate of a
    full gradient implied by it."""
    import oracle
    sub = _soft_slice(a, scenes)
    _, target = oracle.soft_forward(_soft_slice(t_arrays, scenes))
    direction = {"colors": np.ones_like(sub["colors"], dtype=np.float64)}
    t0 = time.perf_counter()
    oracle.soft_dloss(sub, target.astype(np.float32), direction)
    dt = time.perf_counter() - t0
    nparams = sum(int(np.asarray(sub[k]).size) for k in ("points", "colors", "stop_offsets", "stop_colors",
                                                             "sigma", "opacity")) // scenes
    return {"value": scenes / dt, "unit": "scenes/s (forward + one directional derivative)", "cores": 1,
            "kind": "port", "full_gradient_value": scenes / dt / max(1, nparams),
            "params_per_scene": nparams,
            "sample": "%d scenes: FP64 forward + loss + one directional derivative (C++ reference, %.1f s)" %
                      (scenes, dt), "host": host_info()}


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
        out = {k: grads[k].to("cpu", non_blocking=True) for k in soft.PARAMS}  # noqa: F841
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
    # FP32-bound work: the flops of one step counted by ncu (profiles/soft_config4.json) over the
    # step time, against the nominal FP32 rate (152 SMs x 128 lanes x 2 x 2.07 GHz; no measured figure)
    try:
        with open(os.path.join(ROOT, "profiles", "soft_config4.json")) as fh:
            flop = float(json.load(fh)["flop_per_step"])
    except Exception:
        flop = None
    peak_f = 152 * 128 * 2 * 2.07e9 / 1e12
    alg_bytes = 2 * h2d + 3 * 256 * 256 * 256 * 16
    achieved_f = flop / (ms * 1e-3) / 1e12 if flop else None
    line["roofline"] = {"bound": "fp32", "achieved": achieved_f, "peak": peak_f, "unit": "TFLOP/s",
                        "frac": achieved_f / peak_f if achieved_f else None, "peak_kind": "nominal",
                        "traffic": None, "kernel": "soft forward + adjoint (one step)",
                        "flop_per_step": flop, "flop_source": "ncu FP32 op counters, profiles/soft_config4.md",
                        "algorithmic_bytes": alg_bytes}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_soft(a, t)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------- plain render (configs 0-2)

def run_plain(args, rank, world):
    import torch
    import resvg_gb300 as R
    from resvg_gb300 import build as B
    B.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    R.init(0)
    from resvg_gb300 import batch as BT
    tree = R.Tree.generate(args.config, seed=SEED, index=rank, scale=args.scale)
    w, h = (int(v) for v in tree.size)
    surface = torch.zeros((h, w, 4), dtype=torch.uint8, device=dev)
    # the product's autotuner (rgpu_autotune) picks band rows and pixels per
    # thread for this scene, on a copy of the tree: the timed tree's own first
    # render is the one that strokes its paths
    t0 = time.perf_counter()
    tune_tree = R.Tree.generate(args.config, seed=SEED, index=rank, scale=args.scale)
    best_tuning, tune_ms = R.autotune([tune_tree], [IDENT], [w], [h], [surface.data_ptr()], BT.TUNING_CANDIDATES,
                                      reps=3)
    tune_s = time.perf_counter() - t0
    del tune_tree
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    scene = R.Scene([tree], [IDENT], [w], [h], [surface.data_ptr()])
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

    stroke = warmup_with_stroke_record(step, scene, args.warmup)
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
    timed_image = surface.cpu().numpy()  # the last timed step's output (rendered from a cleared surface)
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
        R.render(tree, IDENT, pixmap=host)
    e2e_t = []
    for _ in range(max(1, args.e2e_steps)):
        host[:] = 0
        t0 = time.perf_counter()
        R.render(tree, IDENT, pixmap=host)
        e2e_t.append(time.perf_counter() - t0)
    st = R.stats()
    e2e_ms = 1e3 * sum(e2e_t) / len(e2e_t)

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
                   "l2": "flushed between steps (256 MB write)", "graph_replay": True, "stroke": stroke,
                   "tuning": {"band_rows": best_tuning[0], "pixels_per_thread": best_tuning[1],
                              "autotune_ms": tune_ms, "autotune_s": tune_s,
                              "candidates": [list(c) for c in BT.TUNING_CANDIDATES]}},
        "mpix_s": value * out_px / 1e6,
        "raster_ms": rms,
        "wall_s_timed_region": t_wall,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": profiled_traffic("config%d" % args.config),
                     "kernel": "k_raster (band VM)", "algorithmic_bytes": alg_bytes,
                     "issue_roof": profiled_issue("config%d" % args.config)},
        "e2e": {"value": 1e3 / e2e_ms, "unit": "scenes/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(st["h2d_bytes"]), "d2h_bytes_per_step": int(st["d2h_bytes"])},
        "gpu_launches": int(info["kernel_launches"]) * args.steps,
        "clocks": clk.summary(),
        "parity": None,
    }
    if rank == 0 and not args.no_cpu_baseline:
        cb, ref = cpu_baseline_single(tree, w, h)
        line["parity"] = parity_record([(timed_image, ref)])
        if world == 1:
            line["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def warmup_with_stroke_record(step, scene, warmup):
    """Runs the warm-up renders; the first one is the prepared scene's sizing
    render, which strokes every path that has no outline yet on the device
    (kernels/stroke.cu) and keeps the outlines for the renders after it.
    Returns that pass's record: paths stroked and the stroke kernel's time."""
    import resvg_gb300 as R
    rec = None
    s0 = R.stats()
    for k in range(warmup):
        step()
        scene.check()
        if k == 0:
            s1 = R.stats()
            rec = {"jobs": int(s1["stroke_jobs"] - s0["stroke_jobs"]),
                   "device_ms": float(s1["stroke_ms"] - s0["stroke_ms"]),
                   "when": "first (sizing) render; later renders and graph replays reuse the outlines"}
    return rec


def run_profile(args):
    """Two renders of the workload through a prepared scene, nothing else:
    the command ncu captures wrap (`-k regex:k_raster -s <levels> -c 1`)."""
    import torch
    import resvg_gb300 as R
    from resvg_gb300 import build as B
    B.build()
    R.init(0)
    if args.config == 4:
        # forward + loss + adjoint of the 256-scene batch, twice (launches 2 onwards are the second step)
        from resvg_gb300 import soft
        a = soft.make_scenes(seed=SEED, scenes=256, size=256, paths=64)
        sc, tgt = soft.Scenes(a), soft.Scenes(soft.perturb(a, seed=SEED + 1000))
        _, target = soft.forward(tgt)
        for _ in range(2):
            image, blurred = soft.forward(sc)
            loss, g = soft.mse(blurred, target)
            soft.backward(sc, image, g)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "config4", "scenes": 256, "loss": loss}), flush=True)
        return
    if args.tuning:
        band_rows, px = (int(v) for v in args.tuning.split(","))
        R.set_tuning(band_rows, px)
    if args.config == 3:
        trees = [R.Tree.generate(3, seed=SEED, index=i) for i in range(args.scenes)]
    else:
        trees = [R.Tree.generate(args.config, seed=SEED, index=0, scale=args.scale)]
    sizes = [tuple(int(v) for v in t.size) for t in trees]
    offs, total = [], 0
    for w, h in sizes:
        offs.append(total)
        total += ((w * h * 4 + 255) // 256) * 256
    buf = torch.zeros(total, dtype=torch.uint8, device="cuda")
    scene = R.Scene(trees, [IDENT] * len(trees), [w for w, _ in sizes], [h for _, h in sizes],
                    [buf.data_ptr() + o for o in offs])
    scene.set_timing(True)  # un-captured renders: every kernel is a launch of its own
    ms = []
    for _ in range(2):
        scene.render()
        ms.append(scene.check())
    print(json.dumps({"profile": "config%d" % args.config, "scenes": len(trees), "raster_ms": ms,
                      "tuning": R.get_tuning(), "info": scene.info()}), flush=True)


def main():
    args = parse()
    rank, world = dist_setup(args.gpus)
    if args.profile:
        run_profile(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.config == 3:
        run_batched(args, rank, world)
    elif args.config == 4:
        run_soft(args, rank, world)
    else:
        run_plain(args, rank, world)


if __name__ == "__main__":
    main()
