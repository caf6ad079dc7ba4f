"""Benchmark of the wavefront path-tracing hot path on GB300.

Workload (default): the "plain method, large" configuration - a 1024 x 1024
value-noise heightfield (2,093,058 triangles) + 64 emissive triangles
(log-uniform intensity in [1, 1000], alias-table light sampling), 256 Disney
materials on 64 x 64 tiles, 1920 x 1080, 64 samples per pixel, 8 bounces,
Russian roulette from bounce 3, counter-based RNG, fp32. Synthetic, seeded.

One step = all 64 samples per pixel of that image: reset, then one
tr_render_samples call that renders them as one continuous wavefront through
the frame's 1920 x 1080 x ms path slots (ms = 16: 33.2 M paths in flight),
refilled with the next samples as paths end; its iterations (plan, connect,
extend, shade) run as one CUDA graph with a device-driven while loop. The
per-stage figures come from eager frames of the same samples. The metric is the reference's Mrays/s = (extend + shadow rays) /
time (Tracer/GUI/MainGui.cpp:97-100,801-805); samples/s is reported beside it.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

Prints one JSON line. Under torchrun each rank renders its own sample shard
(disjoint sample indices; weak scaling, no collective on the data path) and
rank 0 reports the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

EXTEND_BYTES_PER_RAY = 48      # path state in (O, D, T: 48 B)
EXTEND_BYTES_PER_HIT = 64      # path state (48 B) + hit record (16 B) appended to the hit queue
NODE_BYTES = 80                # per node visit: the fixed algorithmic figure of a compressed 8-wide node
TRI_BYTES = 48                 # one traversal triangle (v0, e1, e2)
SHADE_BYTES_FIXED = 140        # state 48 + hit 16 + triangle record 72 + material index 4
L2_BYTES = 129 * 1024 * 1024


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--grid", type=int, default=1024, help="heightfield vertices per side")
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--spp", type=int, default=64)
    p.add_argument("--ms", type=int, default=16, help="samples per pixel per wavefront frame")
    p.add_argument("--cpu-seconds", type=float, default=20.0, help="target CPU work of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--profile", action="store_true",
                   help="render one eager step of the workload (spp samples as one continuous wavefront) and "
                        "exit (the case the ncu captures use)")
    p.add_argument("--workload", default="plain", choices=["plain", "batch", "adjoint", "large"],
                   help="plain: the heightfield (default); batch: the 64-scene mix in one wavefront against "
                        "per-scene renders; adjoint: forward frame and path-replay adjoint of the "
                        "differentiation scene; large: the 20.5M-triangle displaced-sphere scene at 3840x2160, "
                        "16 spp, 12 bounces, forward frame and adjoint over its 4096 materials")
    p.add_argument("--no-autotune", action="store_true", help="plain workload: keep the default launch shapes")
    p.add_argument("--tune-on", default="samples", choices=["samples", "frames"],
                   help="plain workload: what the autotuner times (continuous renders, as the step, or frames)")
    p.add_argument("--rmse-spp", type=int, default=1024,
                   help="plain workload: also compare a render of this many spp against the FP64 oracle")
    p.add_argument("--batch-count", type=int, default=64)
    p.add_argument("--no-extra", action="store_true",
                   help="plain workload: skip the batched and differentiation measurements after the timed region")
    p.add_argument("--pool-paths", type=int, default=0,
                   help="batched rendering: path slots of the continuous wavefront (0: library default)")
    p.add_argument("--no-ms1", action="store_true",
                   help="batch workload: skip the per-scene baseline at the reference's multi_sample = 1")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [line for line in out.splitlines() if line.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_scene(args):
    import trayracer_gb300 as tr

    return tr.heightfield(n=args.grid, width=args.width, height=args.height, spp=args.spp, max_depth=8,
                          rr_start=3)


def cpu_baseline(scene, args, seconds: float, oracle=None):
    """The oracle port (restated reference path) on all host threads over a bounded pixel sample."""
    import trayracer_gb300 as tr
    from oracle import Oracle

    threads = os.cpu_count() or 1
    o = oracle if oracle is not None else Oracle(scene)
    st = tr.settings_for(scene, multi_sample=4)
    wh = scene.width * scene.height
    # calibrate on a small band, then size the sample to the target time
    first = (wh // 2 // scene.width) * scene.width
    n0 = max(4096, threads * 512)
    t = time.perf_counter()
    _, _, c0 = o.render(scene.camera, st, scene.width, scene.height, frames=1, first_pixel=first, pixel_count=n0,
                        threads=threads)
    dt0 = time.perf_counter() - t
    want = n0 * seconds / max(dt0, 1e-3)  # pixel-frames of work for the target time
    n = int(min(wh - first, max(n0, want)))
    frames = max(1, min(16, int(want / n)))  # more frames once the sample holds the lower half of the image
    t = time.perf_counter()
    _, _, c = o.render(scene.camera, st, scene.width, scene.height, frames=frames, first_pixel=first,
                       pixel_count=n, threads=threads)
    dt = time.perf_counter() - t
    rays = c[0] + c[1]
    return {
        "value": rays / dt / 1e6,
        "unit": "Mrays/s",
        "cores": threads,
        "kind": "port",
        "sample": f"{n} pixels x {4 * frames} spp of the {scene.width}x{scene.height} image (rows from the "
                  f"centre), 8 bounces, {rays} rays in {dt:.1f} s",
        "samples_per_s": n * 4 * frames / dt,
        "traversal": "the oracle's median-split binary BVH (up to 4 triangles per leaf), not the GPU's "
                     "SAH-built 8-wide BVH",
    }


def band_accuracy(r, scene, args, frames, sptr, rows=16, spp_long=1024, rows_long=2):
    """Relative image RMSE of the step's 64-spp image on `rows` image rows spread over the frame,
    against the FP64 oracle and against the fp32 oracle (same sample keys on all sides), the fp32
    oracle against the FP64 one, and the fraction of the last frame's paths whose radiance is
    within 1e-4 of the fp32 oracle's. The difference to FP64 is fp32 against fp64 arithmetic:
    it shows as noise where a path's fp32 and fp64 continuations part (near-specular lobes,
    Russian roulette and lobe choices on a last-bit difference) and falls as 1/sqrt(spp). Then
    the same against FP64 at spp_long samples per pixel on rows_long rows."""
    import trayracer_gb300 as tr
    from oracle import Oracle

    W, H, ms = scene.width, scene.height, args.ms
    st = tr.settings_for(scene, multi_sample=ms)
    threads = os.cpu_count() or 1
    orc = Oracle(scene)
    img = r.ColorBuffer()  # the benchmark step's image (one continuous wavefront of all samples)
    # the same samples frame by frame, for the per-path radiance of the last frame
    r.Reset()
    for _ in range(frames):
        r.RenderFrame(stream=sptr, use_graph=True)
    buf = r.Buffers()
    ys = [(k * H) // rows + H // (2 * rows) for k in range(rows)]
    g_img, o32, o64, ok = [], [], [], []
    for y in ys:
        first = y * W
        a32, p32, _ = orc.render(scene.camera, st, W, H, frames=frames, first_pixel=first, pixel_count=W,
                                 want_paths=True, threads=threads)
        a64, _, _ = orc.render(scene.camera, st, W, H, frames=frames, first_pixel=first, pixel_count=W,
                               use_double=True, threads=threads)
        rad = np.stack([r.read_device(buf["radiance"] + 16 * (first + smp * W * H), np.float32, 4 * W)
                        .reshape(W, 4) for smp in range(ms)])[..., :3].astype(np.float64)
        p = p32[..., :3]
        ok.append((np.abs(rad - p) <= 1e-4 * np.maximum(1.0, np.abs(p)) + 1e-6).all(-1).ravel())
        g_img.append(img.reshape(-1, 4)[first:first + W, :3].astype(np.float64))
        o32.append(a32[:, :3] / a32[:, 3:4])
        o64.append(a64[:, :3] / a64[:, 3:4])
    g, i32, i64 = (np.concatenate(x) for x in (g_img, o32, o64))

    def rel(a, b):
        return float(np.sqrt(np.mean((a - b) ** 2)) / max(1e-12, np.sqrt(np.mean(b ** 2))))

    out = {
        "rows": ys,
        "spp": frames * ms,
        "rmse_gpu_vs_fp64": rel(g, i64),
        "rmse_gpu_vs_fp32_oracle": rel(g, i32),
        "rmse_fp32_oracle_vs_fp64": rel(i32, i64),
        "paths_compared": int(sum(x.size for x in ok)),
        "paths_within_1e-4_of_fp32_oracle": float(np.concatenate(ok).mean()),
    }
    if spp_long > frames * ms:
        long_frames = spp_long // ms
        r.Reset()
        for _ in range(long_frames):
            r.RenderFrame(stream=sptr, use_graph=True)
        img = r.ColorBuffer()
        band0 = (H // 2) * W
        nb = rows_long * W
        a64, _, _ = orc.render(scene.camera, st, W, H, frames=long_frames, first_pixel=band0, pixel_count=nb,
                               use_double=True, threads=threads)
        out[f"rmse_gpu_vs_fp64_spp_{long_frames * ms}"] = rel(img.reshape(-1, 4)[band0:band0 + nb, :3]
                                                              .astype(np.float64), a64[:, :3] / a64[:, 3:4])
        out["rows_long"] = list(range(H // 2, H // 2 + rows_long))
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import Oracle

    scene = build_scene(args)
    oracle = Oracle(scene)  # its host BVH is built once, outside the steps
    per_step = max(1.0, min(args.cpu_seconds, 150.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_baseline(scene, args, per_step / 2, oracle)
    vals = []
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(scene, args, per_step, oracle)
        vals.append(last["value"])
    elapsed = time.perf_counter() - t0
    value = float(statistics.median(vals))
    line = {
        "impl": "reference",
        "metric": "Mrays/s",
        "value": round(value, 4),
        "unit": "Mrays/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1000 * elapsed / max(1, args.steps), 2),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": config_dict(args, scene),
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": last["cores"], "kind": "port",
                         "sample": last["sample"], "traversal": last["traversal"]},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own code path is OptiX/RT-core + Windows only; the timed CPU implementation is "
                "the restated reference path (oracle/), each step a bounded pixel sample",
    }
    print(json.dumps(line), flush=True)


def config_dict(args, scene):
    return {
        "workload": f"heightfield {args.grid}x{args.grid} ({scene.triangle_count} tris, 64 emissive), "
                    f"{args.width}x{args.height}, {args.spp} spp, 8 bounces, RR from 3, 256 Disney materials",
        "width": args.width,
        "height": args.height,
        "spp": args.spp,
        "samples_per_frame": args.ms,
        "triangles": scene.triangle_count,
        "l2": "flushed between steps (256 MiB write); scene + wavefront buffers exceed L2",
        "parallelism": f"sample shards x{dist_env()[0]}",
    }


def measure_batch(args, steps, warmup, with_ms1=True):
    """The batching mix: 64 seeded sphere scenes (1k-500k triangles, 128^2-1024^2, 4/16/64 spp,
    1-16 lights, 6 bounces, RR from bounce 3) rendered by one continuous wavefront (a pool of path
    slots refilled from a device cursor, the iterations a CUDA graph while loop) against the same scenes rendered one after the other through tr_render_frame
    (graph per frame, multi_sample = min(spp, 16), the reference's largest multi-sample)."""
    import torch

    import trayracer_gb300 as tr
    from trayracer_gb300.renderer import KernelSettings

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    t = time.perf_counter()
    scenes = tr.sphere_batch(args.batch_count)
    gen_s = time.perf_counter() - t
    st = KernelSettings(multiSample=1, maxDepth=6, seed=1, rrStart=3)
    samples = sum(s.width * s.height * s.spp for s in scenes)

    def timed_batch(items):
        """Median of `steps` graph-launched renders of a batch of `items` (L2 flushed before each),
        and the batch's build time (BVHs and upload)."""
        t0 = time.perf_counter()
        bb = tr.BatchRenderer(items, pool_paths=args.pool_paths)
        built_s = time.perf_counter() - t0
        for _ in range(warmup):
            bb.Render(st, stream=sptr)
        torch.cuda.synchronize()
        ts = []
        with ClockSampler(0) as clk:
            for _ in range(steps):
                flush.fill_(1.0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                bb.Render(st, stream=sptr)
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
        stats_, info_ = bb.Statistics(), bb.Info()
        assert stats_["device_error"] == 0
        bb.close()
        return float(statistics.median(ts)), stats_, info_, clk.summary(), built_s

    # batched: one continuous wavefront, one graph launch
    if args.profile:
        b = tr.BatchRenderer(scenes, pool_paths=args.pool_paths)
        b.Render(st, stream=sptr, use_graph=False)
        out = {"batch": b.Statistics(), "info": b.Info()}
        b.close()
        return out
    batch_ms, bstats, info, batch_clocks, build_s = timed_batch(scenes)
    rays = bstats["extend_rays"] + bstats["shadow_rays"]

    # per scene: one context, each scene uploaded (untimed) and rendered as spp / ms graph frames,
    # with ms = min(spp, 16) (the reference's largest multi-sample) and with ms = 1 (its default,
    # Renderer.cpp:259)
    r = tr.DeviceRenderer(0)

    per_item_ms = []

    def per_scene(max_ms):
        total_ms, total_rays, n_launch = 0.0, 0, 0
        per_item_ms.clear()
        with ClockSampler(0) as pclocks:
            for s in scenes:
                ms = min(s.spp, max_ms)
                frames = s.spp // ms
                r.UpdateScene(s)
                r.SetCamera(s.camera)
                r.Resize((s.width, s.height))
                r.SetSettings(KernelSettings(**{**st.__dict__, "multiSample": ms}))
                elapsed = None
                for _ in range(2):  # the first pass allocates and captures the graph
                    r.Reset()
                    flush.fill_(1.0)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    for _ in range(frames):
                        r.RenderFrame(stream=sptr, use_graph=True)
                    e1.record(stream)
                    e1.synchronize()
                    elapsed = e0.elapsed_time(e1)
                total_ms += elapsed
                per_item_ms.append(elapsed)
                r.Reset()
                for _ in range(frames):
                    r.RenderFrame(stream=sptr, use_graph=False)
                    total_rays += r.Statistics()["path_count"]
                n_launch += frames * (3 * st.maxDepth + 2)  # kernels: extend, shade, connect per bounce, finalize, advance
        return total_ms, total_rays, n_launch, pclocks.summary()

    plain_ms, plain_rays, launches, plain_clocks = per_scene(16)
    # the mix without its 1024^2 items, whose per-scene frames already fill the GPU: a batch of
    # the smaller items alone against their per-scene frames
    small = [k for k, s in enumerate(scenes) if s.width * s.height < 1024 * 1024]
    small_ms, _, small_info, _, _ = timed_batch([scenes[k] for k in small])
    small_per_scene_ms = float(sum(per_item_ms[k] for k in small))
    out = {
        "iterations": bstats["iterations"],
        "launches": bstats["launches"],
        "samples": samples,
        "batch_ms": batch_ms,
        "batch_rays": int(rays),
        "info": info,
        "clocks": batch_clocks,
        "items_below_1024sq": {"count": len(small), "samples": int(small_info["path_count"]),
                               "batched_ms": round(small_ms, 3), "per_scene_ms": round(small_per_scene_ms, 3),
                               "batched_over_per_scene": round(small_per_scene_ms / small_ms, 3),
                               "per_scene_ms_1024sq_items": round(plain_ms - small_per_scene_ms, 3)},
        "per_scene": {"ms": round(plain_ms, 3), "samples_per_s": round(samples / (plain_ms / 1e3), 1),
                      "mrays_per_s": round(plain_rays / (plain_ms / 1e3) / 1e6, 1), "gpu_launches": launches,
                      "clocks": plain_clocks},
        "rays_per_scene": int(plain_rays),
        "speedup_vs_per_scene": round(plain_ms / batch_ms, 3),
        "scene_generation_s": round(gen_s, 2),
        "batch_build_s": round(build_s, 2),
    }
    if with_ms1:
        ms1_ms, ms1_rays, ms1_launches, ms1_clocks = per_scene(1)
        out["per_scene_ms1"] = {"ms": round(ms1_ms, 3), "samples_per_s": round(samples / (ms1_ms / 1e3), 1),
                                "mrays_per_s": round(ms1_rays / (ms1_ms / 1e3) / 1e6, 1),
                                "gpu_launches": ms1_launches, "clocks": ms1_clocks}
        out["speedup_vs_per_scene_ms1"] = round(ms1_ms / batch_ms, 3)
    r.close()
    return out


def run_batch(args):
    m = measure_batch(args, args.steps, args.warmup, with_ms1=not args.no_ms1)
    if args.profile:
        print(json.dumps(m))
        return
    info, samples, batch_ms = m["info"], m["samples"], m["batch_ms"]
    line = {
        "metric": "samples/s",
        "value": round(samples / (batch_ms / 1e3), 1),
        "unit": "samples/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(batch_ms, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{args.batch_count} sphere scenes, {info['triangle_count']} tris, "
                               f"{info['pixel_count']} pixels, {samples} samples, 6 bounces, RR from 3",
                   "pool_paths": info["pool_paths"], "iterations": m["iterations"],
                   "l2": "flushed before each timed render (256 MiB write)"},
        "mrays_per_s": round(m["batch_rays"] / (batch_ms / 1e3) / 1e6, 1),
        "gpu_launches": m["launches"],
        **{k: m.get(k) for k in ("per_scene", "per_scene_ms1", "speedup_vs_per_scene", "speedup_vs_per_scene_ms1",
                                 "items_below_1024sq", "rays_per_scene", "scene_generation_s", "batch_build_s",
                                 "clocks")},
        "rays_batch": m["batch_rays"],
    }
    print(json.dumps(line), flush=True)


def measure_adjoint(args, steps, warmup):
    """Differentiation: the Cornell box with Disney walls, 512^2, 32 spp, 6 bounces, no RR. One
    forward frame (graph replay) and the path-replay adjoint of the L2 loss 0.5 |img - target|^2
    against a target rendered with the Disney parameters perturbed by N(0, 0.05) (clipped to
    [0, 1]); gradients of all 9 parameters of the 8 materials. CUDA events on the launch stream,
    L2 flushed before the forward frame and before the adjoint."""
    import torch

    import trayracer_gb300 as tr
    from trayracer_gb300.renderer import KernelSettings

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    W = H = 512
    spp = 32
    scene = tr.cornell_box(width=W, height=H, wall_closure=tr.TR_CLOSURE_DISNEY, max_depth=6)
    st = KernelSettings(multiSample=spp, maxDepth=6, seed=1, rrStart=1 << 30)
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((W, H))
    # the target: perturbed parameters, another seed
    r.UpdateMaterials(tr.perturbed_materials(scene.materials))
    r.SetSettings(KernelSettings(**{**st.__dict__, "seed": 7}))
    r.RenderFrame(stream=sptr, use_graph=False)
    target = torch.from_numpy(r.ColorBuffer().copy()).cuda()
    r.UpdateMaterials(scene.materials)
    r.SetSettings(st)
    grad = torch.zeros((scene.materials.shape[0], 9), dtype=torch.float32, device="cuda")
    if args.profile:
        r.RenderFrame(stream=sptr, use_graph=False)
        pg = torch.from_numpy(r.ColorBuffer()).cuda() - target  # dL/dcolor of 0.5 |img - target|^2
        r.AdjointFrame(pg.data_ptr(), 1.0 / spp, grad.data_ptr(), stream=sptr)
        torch.cuda.synchronize()
        r.close()
        return {"grad_norm": float(grad.norm())}
    fwd, adj = [], []
    img = None
    with ClockSampler(0) as clocks:
        for i in range(warmup + steps):
            flush.fill_(1.0)
            e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
            r.Reset()
            e0.record(stream)
            r.RenderFrame(stream=sptr, use_graph=True)
            e1.record(stream)
            if img is None:
                img = torch.from_numpy(r.ColorBuffer()).cuda()
                pg = img - target
            flush.fill_(1.0)
            e2.record(stream)
            r.AdjointFrame(pg.data_ptr(), 1.0 / spp, grad.data_ptr(), stream=sptr)
            e3.record(stream)
            e3.synchronize()
            if i >= warmup:
                fwd.append(e0.elapsed_time(e1))
                adj.append(e2.elapsed_time(e3))
    stats = r.Statistics()
    r.close()
    f_ms, a_ms = float(statistics.median(fwd)), float(statistics.median(adj))
    return {
        "forward_ms": round(f_ms, 3),
        "adjoint_ms": round(a_ms, 3),
        "adjoint_over_forward": round(a_ms / f_ms, 3),
        "forward_mrays_per_s": round(stats["path_count"] / (f_ms / 1e3) / 1e6, 1),
        "samples_per_s": round(W * H * spp / (f_ms / 1e3), 1),
        "adjoint_samples_per_s": round(W * H * spp / (a_ms / 1e3), 1),
        "gradient_norm": float(grad.norm()),
        "clocks": clocks.summary(),
    }


def run_adjoint(args):
    m = measure_adjoint(args, args.steps, args.warmup)
    if args.profile:
        print(json.dumps(m))
        return
    line = {
        "metric": "adjoint/forward time",
        "value": m["adjoint_over_forward"],
        "unit": "ratio",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(m["forward_ms"] + m["adjoint_ms"], 3),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "Cornell box with Disney walls, 512x512, 32 spp, 6 bounces, no RR; L2 loss "
                               "against a target rendered with the Disney parameters + N(0, 0.05); gradients of "
                               "9 parameters for each of the 8 materials",
                   "l2": "flushed before the forward frame and before the adjoint (256 MiB write)"},
        **m,
    }
    print(json.dumps(line), flush=True)


def measure_large(args, steps, warmup):
    """The large configuration: 4096 displaced spheres (20.48 M triangles, 100k emissive), 4096
    materials, 3840x2160, 16 spp in one frame (132.7 M paths in flight), 12 bounces, RR from bounce
    3; a forward frame (graph) and the path-replay adjoint of the L2 loss against a black target
    over all materials."""
    import torch

    import trayracer_gb300 as tr

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    t = time.perf_counter()
    scene = tr.displaced_spheres()
    gen_s = time.perf_counter() - t
    st = tr.settings_for(scene, multi_sample=scene.spp)
    r = tr.DeviceRenderer(0)
    t = time.perf_counter()
    r.UpdateScene(scene)
    upload_s = time.perf_counter() - t
    info = r.SceneInfo()
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    r.SetSettings(st)
    W, H = scene.width, scene.height
    grad = torch.zeros((scene.materials.shape[0], 9), dtype=torch.float32, device="cuda")
    fwd, adj, rays = [], [], 0
    pg = None
    with ClockSampler(0) as clocks:
        for i in range(warmup + steps):
            flush.fill_(1.0)
            e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
            r.Reset()
            e0.record(stream)
            r.RenderFrame(stream=sptr, use_graph=True)
            e1.record(stream)
            if pg is None:
                pg = torch.from_numpy(r.ColorBuffer()).cuda()  # dL/dcolor of 0.5 |img|^2
                rays = r.Statistics()["path_count"]
            flush.fill_(1.0)
            e2.record(stream)
            r.AdjointFrame(pg.data_ptr(), 1.0 / scene.spp, grad.data_ptr(), stream=sptr)
            e3.record(stream)
            e3.synchronize()
            if i >= warmup:
                fwd.append(e0.elapsed_time(e1))
                adj.append(e2.elapsed_time(e3))
    stats = r.Statistics()
    assert stats["device_error"] == 0
    r.close()
    f_ms, a_ms = float(statistics.median(fwd)), float(statistics.median(adj))
    return {
        "workload": f"{info['triangle_count']} triangles (4096 displaced spheres, 100k emissive), "
                    f"4096 materials, {W}x{H}, {scene.spp} spp, 12 bounces, RR from 3",
        "mrays_per_s": round(rays / (f_ms / 1e3) / 1e6, 1),
        "samples_per_s": round(W * H * scene.spp / (f_ms / 1e3), 1),
        "forward_ms": round(f_ms, 3),
        "adjoint_ms": round(a_ms, 3),
        "adjoint_over_forward": round(a_ms / f_ms, 3),
        "rays_per_frame": int(rays),
        "scene_generation_s": round(gen_s, 2),
        "scene_upload_s": round(upload_s, 2),
        "scene_device_bytes": int(info["device_bytes"]),
        "gradient_norm": float(grad.norm()),
        "clocks": clocks.summary(),
    }


def run_large(args):
    m = measure_large(args, args.steps, args.warmup)
    line = {
        "metric": "Mrays/s",
        "value": None,
        "unit": "Mrays/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(m["forward_ms"] + m["adjoint_ms"], 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": m["workload"],
                   "l2": "flushed before the forward frame and before the adjoint (256 MiB write)"},
        **{k: v for k, v in m.items() if k != "workload"},
    }
    line["value"] = m["mrays_per_s"]
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.workload == "large":
        run_large(args)
        return

    import torch

    import trayracer_gb300 as tr
    from trayracer_gb300._abi import TR_FLAG_COUNT_TRAVERSAL
    from trayracer_gb300.shards import max_over_ranks, shard_settings

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    scene = build_scene(args)
    frames_per_step = max(1, args.spp // args.ms)
    st = shard_settings(tr.settings_for(scene, multi_sample=args.ms), rank)  # disjoint sample streams per shard
    r = tr.DeviceRenderer(local)
    t = time.perf_counter()
    r.UpdateScene(scene)
    upload_s = time.perf_counter() - t
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    r.SetSettings(st)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    if args.profile:
        r.RenderSamples(args.spp, stream=sptr, use_graph=False)
        s = r.Statistics()
        print(json.dumps({k: s[k] for k in ("path_count", "primary_path_count", "secondary_path_count",
                                             "shadow_ray_count", "hit_ray_count", "iterations", "launches",
                                             "extend_time_ms", "shade_time_ms", "connect_time_ms",
                                             "device_error")}))
        r.close()
        return
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def step(use_graph=True):
        # all spp samples as one continuous wavefront through the frame's path slots
        r.Reset()
        r.RenderSamples(args.spp, stream=sptr, use_graph=use_graph)

    # --- autotuner (launch shapes, BVH leaf size) on this workload, outside the timed region
    tune = None
    if not args.no_autotune:
        tune = r.Autotune(stream=sptr, samples=args.tune_on == "samples")
        tune["timed"] = args.tune_on
        torch.cuda.synchronize()

    # --- counting pass (rays and traversal work of one step), outside the timed region: the
    # same step rendered eagerly with the traversal counters on
    cnt_settings = tr.settings_for(scene, multi_sample=args.ms)
    cnt_settings.seed = st.seed
    cnt_settings.flags |= TR_FLAG_COUNT_TRAVERSAL
    r.SetSettings(cnt_settings)
    r.Reset()
    r.RenderSamples(args.spp, stream=sptr, use_graph=False)
    cs = r.Statistics()
    r.SetSettings(st)
    assert cs["device_error"] == 0, "traversal bound exceeded"
    ext_rays = cs["primary_path_count"] + cs["secondary_path_count"]
    sh_rays = cs["shadow_ray_count"]
    hit_rays = cs["hit_ray_count"]
    primary_rays = cs["primary_path_count"]

    # --- warm-up
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # --- per-stage timing of one eager step: the same continuous wavefront run from a host loop
    # with the stages in sequence (no connect/extend overlap), CUDA events around every launch
    # on the launch stream, summed over the iterations; "generate" is the plan kernels,
    # "finalize" the round start, finalize and sample-count advance
    r.Reset()
    r.RenderSamples(args.spp, stream=sptr, use_graph=False)
    s = r.Statistics()
    stage_ms = {k: s[f"{k}_time_ms"] for k in ("generate", "extend", "shade", "connect", "finalize")}
    stage_launches = s["iterations"] + 1  # per stage: one per iteration, the last finds nothing

    # --- timed region: K steps, graph replay, L2 flushed between steps
    times = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    total_ms = float(sum(times))
    if ws > 1:
        total_ms = max_over_ranks(total_ms, device=f"cuda:{local}")
    final = r.Statistics()
    assert final["device_error"] == 0
    rays_per_step = final["path_count"]

    # --- end to end through the public API, host buffers: per step the camera
    # and settings are handed over from host structs, the frame set is rendered
    # and the 1920x1080 float4 image is read back into pinned host memory
    host_img = torch.empty((scene.height, scene.width, 4), dtype=torch.float32, pin_memory=True)
    host_np = host_img.numpy()
    e2e_times = []
    for i in range(args.steps + 1):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.SetCamera(scene.camera)
        r.SetSettings(st)
        step()
        r.ColorBuffer(out=host_np, stream=sptr)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e_times[1:]))

    value = rays_per_step * args.steps * ws / (total_ms / 1e3) / 1e6
    samples_per_s = scene.width * scene.height * args.spp * args.steps * ws / (total_ms / 1e3)

    # --- roofline of the dominant kernel (extend): algorithmic bytes / time
    peak, peak_kind = measured_peak()
    ext_bytes = (ext_rays * EXTEND_BYTES_PER_RAY + hit_rays * EXTEND_BYTES_PER_HIT
                 + cs["traversal_extend_nodes"] * NODE_BYTES
                 + cs["traversal_extend_tris"] * TRI_BYTES)
    ext_s = stage_ms["extend"] / 1e3
    launches = stage_launches
    achieved = ext_bytes / ext_s / 1e9
    compulsory = (ext_rays * EXTEND_BYTES_PER_RAY + hit_rays * EXTEND_BYTES_PER_HIT) / ext_s / 1e9
    # DRAM bytes per extend ray measured by ncu over all extend launches of one eager step of
    # this workload (one pass), scaled to this run's average launch by its extend rays; labelled
    # with its source in the line, not measured in this run
    traffic, traffic_source = None, None
    prof = ROOT / "profiles" / "extend_kernel_heightfield_1920x1080_traffic.txt"
    if prof.exists():
        for line in prof.read_text().splitlines():
            if line.strip().startswith("dram_bytes_per_extend_ray:"):
                try:
                    traffic = float(line.split(":", 1)[1]) * ext_rays / launches
                    traffic_source = ("ncu dram__bytes_read.sum + dram__bytes_write.sum over the 15 extend "
                                      "launches of one eager step of this workload, per extend ray, scaled to "
                                      "this run's extend rays per launch")
                except ValueError:
                    traffic = None

    # --- the other stages by the same fixed byte formulas (per step). Shade: 140 B read per
    # shaded hit (state 48 + hit 16 + shading record 72 + material index 4), 48 B per extend
    # and per shadow ray written and 32 B per radiance read-modify-write (emissive hits);
    # connect: 48 B per shadow ray, its traversal bytes and 32 B per radiance
    # read-modify-write (unoccluded shadow rays); finalize: per pixel its spp sample
    # radiances (16 B each), the accumulator read and written and the colour written (16 B
    # each). The radiance updates come from the counting pass.
    secondary = ext_rays - primary_rays
    stage_bytes = {
        "shade": hit_rays * 140 + (secondary + sh_rays) * 48 + cs["radiance_updates_shade"] * 32,
        "connect": sh_rays * 48 + cs["traversal_connect_nodes"] * NODE_BYTES + cs["traversal_connect_tris"] * TRI_BYTES
        + cs["radiance_updates_connect"] * 32,
        "finalize": scene.width * scene.height * (16 * args.spp + 48),
    }
    stage_roofline = {}
    for k, b in stage_bytes.items():
        sec = stage_ms[k] / 1e3
        gbs = b / sec / 1e9 if sec > 0 else None
        stage_roofline[k] = {"bytes_per_step": int(b), "achieved_gbs": None if gbs is None else round(gbs, 1),
                             "frac": None if gbs is None else round(gbs / peak, 4)}

    # --- image accuracy on 16 image rows spread over the frame, against the oracle
    accuracy = None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            accuracy = band_accuracy(r, scene, args, frames_per_step, sptr, spp_long=args.rmse_spp)
            from oracle import Oracle

            cpu = cpu_baseline(scene, args, args.cpu_seconds, Oracle(scene))
        except Exception as e:  # the checker is optional; the GPU numbers stand
            cpu = {"value": None, "unavailable": str(e)}

    # the plain workload's renderer and flush buffer are released before the other
    # configurations, so that their measurements do not run beside its allocations
    r.close()
    del flush
    torch.cuda.empty_cache()

    # --- the batched and differentiation configurations, measured in the same process after
    # the plain timed region (their own timed regions, CUDA events, L2 flushed)
    batch = adjoint = large = None
    if rank == 0 and ws == 1 and not args.no_extra:
        adjoint = measure_adjoint(args, steps=5, warmup=3)
        m = measure_batch(args, steps=3, warmup=3, with_ms1=False)
        batch = {
            "batched_over_per_scene": m["speedup_vs_per_scene"],
            "batched_ms": round(m["batch_ms"], 3),
            "per_scene_ms": m["per_scene"]["ms"],
            "batched_samples_per_s": round(m["samples"] / (m["batch_ms"] / 1e3), 1),
            "per_scene_samples_per_s": m["per_scene"]["samples_per_s"],
            "batched_mrays_per_s": round(m["batch_rays"] / (m["batch_ms"] / 1e3) / 1e6, 1),
            "per_scene_mrays_per_s": m["per_scene"]["mrays_per_s"],
            "samples": m["samples"],
            "iterations": m["iterations"],
            "pool_paths": m["info"]["pool_paths"],
            "gpu_launches": m["launches"],
            "items_below_1024sq": m["items_below_1024sq"],
            "workload": f"{args.batch_count} sphere scenes ({m['info']['triangle_count']} tris, "
                        f"{m['info']['pixel_count']} pixels, 4/16/64 spp, 6 bounces, RR from 3); per scene: "
                        f"tr_render_frame graph frames at multi_sample min(spp, 16)",
            "clocks": m["clocks"],
            "per_scene_clocks": m["per_scene"]["clocks"],
        }
        large = measure_large(args, steps=2, warmup=1)

    if rank == 0:
        line = {
            "metric": "Mrays/s",
            "value": round(value, 2),
            "unit": "Mrays/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(total_ms / args.steps, 3),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": config_dict(args, scene),
            "samples_per_s": round(samples_per_s, 1),
            "rays_per_step": int(rays_per_step),
            "extend_rays_per_step": int(ext_rays),
            "shadow_rays_per_step": int(sh_rays),
            "hit_rays_per_step": int(hit_rays),
            "stage_ms_per_step": {k: round(v, 3) for k, v in stage_ms.items()},
            "accuracy": accuracy,
            "roofline": {
                "kernel": "extend_kernel (8-wide BVH closest hit)",
                "bound": "hbm",
                "achieved": round(achieved, 1),
                "peak": peak,
                "peak_kind": peak_kind,
                "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": traffic,
                "traffic_source": traffic_source,
                "bytes_per_launch": int(ext_bytes / launches),
                "avg_launch_ms": round(stage_ms["extend"] / launches, 4),
                "compulsory_frac": round(compulsory / peak, 4),
                "nodes_per_ray": round(cs["traversal_extend_nodes"] / max(1, ext_rays), 3),
                "tris_per_ray": round(cs["traversal_extend_tris"] / max(1, ext_rays), 3),
                "connect_nodes_per_ray": round(cs["traversal_connect_nodes"] / max(1, sh_rays), 3),
                "connect_tris_per_ray": round(cs["traversal_connect_tris"] / max(1, sh_rays), 3),
            },
            "stage_roofline": stage_roofline,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "e2e": {
                "value": round(rays_per_step / e2e_s / 1e6, 2),
                "unit": "Mrays/s",
                "h2d_bytes_per_step": 72 + 32,
                "d2h_bytes_per_step": scene.width * scene.height * 16,
            },
            # per step: the continuous wavefront's plan, connect, extend and shade per iteration
            # plus its start, finalize and advance
            "gpu_launches": args.steps * final["launches"],
            "iterations_per_step": final["iterations"],
            "stage_source": "one eager step of the same samples (continuous wavefront, stages in sequence, "
                            "CUDA events per launch); the timed steps are graph launches with connect beside "
                            "extend",
            "scene_upload_s": round(upload_s, 2),
            "tuning": tune,
            "adjoint": adjoint,
            "batched": batch,
            "large": large,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
