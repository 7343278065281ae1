"""Benchmark of the per-sample path-tracing hot path on one GB300.

A step is one progressive frame (Renderer::render, render/renderer.rs:224)
of the workload at its full resolution and samples per pixel. Default
workload: the triangle-mesh scene (displaced icosphere of 1,310,720
triangles in a 12-triangle Cornell box, 1024x1024, 64 spp, depth 8).

Prints one JSON line:
  value   Msamples/s over K frames, inputs resident in HBM, device time
          (CUDA events around each frame on the renderer's stream; the L2 is
          flushed with a 512 MB write between frames, outside the events)
  e2e     the same metric through the public API (Renderer.render -> C ABI
          rg_render) with the image copied back to host memory every frame
  roofline, cpu_baseline, clocks, gpu_launches as described in the README of
          the JSON keys below.

--impl reference times the CPU restatement of the reference renderer (the
reference crate cannot be built: no Rust toolchain) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

def rank_max(value: float, dist=None, device=None) -> float:
    """The largest `value` over all ranks (the slowest rank's time); `value`
    itself on a single rank."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds: float, world: int, dist=None, device=None) -> tuple:
    """Whole-job throughput of `world` replicas: every rank's units over the
    slowest rank's time. Returns (units per second, that time)."""
    s = rank_max(seconds, dist, device)
    return units_per_rank * world / s, s


WORKLOADS = {
    "mesh": "triangle-mesh Cornell box: displaced icosphere 1,310,720 tris + 12 box tris, 1024x1024, 64 spp, depth 8",
    "spheres": "random spheres (488 spheres), 400x225, 32 spp, depth 50",
    "sdf": "Mandelbulb + torus SDFs, 2 media, 100 spheres, 1280x720, 128 spp, depth 16",
}


def load_workload(name: str):
    from rayna_gb300 import presets
    if name == "mesh":
        return presets.cornell_mesh(level=8, seed=0)
    if name == "spheres":
        return presets.random_spheres(seed=0)
    if name == "sdf":
        return presets.sdf_volumes(seed=0)
    raise ValueError(name)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]) if parts[3] not in ("[N/A]", "N/A") else 0.0,
                             parts[5], parts[6], parts[7], parts[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [r[0] for r in rows]
        busy = [r for r in rows if r[2] > 200.0] or rows
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, v in zip(names, r[3:]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        return {"sm_mhz": statistics.median(r[0] for r in busy), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "sm_mhz_min": min(sm), "reasons": sorted(reasons)}


def cpu_baseline(name: str, threads: int, target_s: float = 15.0):
    """Times the f64 CPU restatement of the reference renderer on a bounded
    sample of the workload (same scene, camera, depth and spp; reduced
    resolution), scaled to about `target_s` seconds of work."""
    from oracle import binding as ob
    from rayna_gb300.scene import RenderOpts, flatten
    scene, cam, opts = load_workload(name)
    flat = flatten(scene)
    probe = RenderOpts(width=16, height=16, samples=opts.samples, ray_depth=opts.ray_depth)
    st, _, _, secs = ob.render(flat, cam, probe, seed=1, frames=1, policy=ob.POLICY_REF_F64, threads=threads)
    per_px = max(secs, 1e-3) / (16 * 16)
    npx = int(max(256, min(opts.width * opts.height, target_s / per_px)))
    side_w = max(16, int(round((npx * opts.width / opts.height) ** 0.5)))
    side_h = max(16, int(round(npx / side_w)))
    sample = RenderOpts(width=side_w, height=side_h, samples=opts.samples, ray_depth=opts.ray_depth)
    st, _, _, secs = ob.render(flat, cam, sample, seed=2, frames=1, policy=ob.POLICY_REF_F64, threads=threads)
    ns = side_w * side_h * opts.samples
    return {"value": ns / secs / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{side_w}x{side_h} px x {opts.samples} spp of the same scene and camera "
                      f"({ns / 1e6:.2f} M samples, {secs:.1f} s), f64 oracle, {threads} threads"}, secs


def run_adjoint(iters: int = 5, stream=None):
    """Differentiable-rendering workload: 1000 Lambertian spheres (3000 albedo
    parameters) + one medium (3 albedo + 1 density), 512x512, forward and
    backward at 16 spp, depth 8, L2 loss against a 1024-spp target of the
    ground-truth parameters; Adam steps on the host. Each iteration renders the
    forward frame, then takes the adjoint of that frame (rg_backward_frame: its
    image, the paths of an independent frame key replayed). Returns timings."""
    import torch

    from rayna_gb300 import Renderer, presets
    scene, cam, opts = presets.adjoint_scene(n_spheres=1000, ground_truth=False)
    gt, _, _ = presets.adjoint_scene(n_spheres=1000, ground_truth=True)
    s = stream.cuda_stream if stream is not None else None
    topts = type(opts)(width=opts.width, height=opts.height, samples=1024, ray_depth=opts.ray_depth)
    with Renderer.new_from(gt, cam, topts, 0, stream=s) as r:
        target = r.frame(seed=1)
    r = Renderer.new_from(scene, cam, opts, 0, stream=s)
    p = np.array([[m.albedo[c] for c in range(3)] for m in r._flat.materials], np.float64)
    dens = np.array([v.density for v in r._flat.volumes], np.float64)
    theta = np.concatenate([p.ravel(), dens])
    m1, m2 = np.zeros_like(theta), np.zeros_like(theta)
    lr, b1, b2 = 0.02, 0.9, 0.999
    fwd_ms, it_ms, losses = [], [], []
    for k in range(iters + 2):
        t0 = time.perf_counter()
        r.render(seed=10_000 + k)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g = r.backward(seed=20_000 + k, target=target, last_frame=True)
        grad = np.concatenate([g["albedo"].astype(np.float64).ravel(), g["density"].astype(np.float64)])
        m1 = b1 * m1 + (1 - b1) * grad
        m2 = b2 * m2 + (1 - b2) * grad * grad
        theta = theta - lr * (m1 / (1 - b1 ** (k + 1))) / (np.sqrt(m2 / (1 - b2 ** (k + 1))) + 1e-8)
        theta = np.clip(theta, 1e-3, None)
        r.set_parameters(albedo=theta[:p.size].reshape(p.shape).astype(np.float32),
                         density=theta[p.size:].astype(np.float32))
        t2 = time.perf_counter()
        if k >= 2:
            fwd_ms.append((t1 - t0) * 1e3)
            it_ms.append((t2 - t1) * 1e3)
        losses.append(g["loss"])
    r.close()
    f, i = statistics.median(fwd_ms), statistics.median(it_ms)
    return {"workload": "1000 spheres (3000 albedos) + 1 medium (3 albedo + density), 512x512, 16 spp, depth 8, "
                        "L2 vs 1024-spp target, Adam",
            "ms_per_iter": i, "forward_ms": f, "iter_over_forward": i / f, "iters": iters,
            "loss_first": losses[0], "loss_last": losses[-1], "n_params": int(theta.size)}


def run_batch(scale: float, steps: int, stream=None):
    """Batched workload: 64 seeded scenes of uneven size (sphere counts
    log-uniform in [10, 5000], half with a displaced mesh of log-uniform
    [1k, 500k] triangles, 0-2 media, resolutions from {256^2, 640x480,
    1280x720, 1920x1080} scaled by `scale`, 16-64 spp, depth 8). The
    batched form the autotuner picks (batched wavefront or persistent tile
    launch, one CUDA graph per frame), against 64 sequential megakernel
    launches of the same frame; both batched forms are reported."""
    from rayna_gb300 import presets
    from rayna_gb300.autotune import Tuner
    from rayna_gb300.batch import BatchRenderer
    items = presets.batch_scenes(64, seed=0, scale=scale)
    s = stream.cuda_stream if stream is not None else None
    with BatchRenderer(items, stream=s) as b:
        cfg = Tuner().tune_batch(b)
        res = {}

        def timed(fn):
            fn(seed=7)
            return statistics.median(fn(seed=100 + k).kernel_ms for k in range(steps))

        res["tuned"] = timed(b.render)
        b.set_tuning(form="wavefront")
        res["wavefront"] = timed(b.render)
        b.set_tuning(form="tiles")
        res["tiles"] = timed(b.render)
        res["sequential"] = timed(b.render_sequential)
        ns = b.n_samples
    return {"workload": f"64 scenes, resolutions x{scale}, {ns / 1e9:.3f} G samples per frame", "tuning": cfg,
            "batched_msamples_s": ns / res["tuned"] / 1e3,
            "batched_wavefront_msamples_s": ns / res["wavefront"] / 1e3,
            "batched_tiles_msamples_s": ns / res["tiles"] / 1e3,
            "sequential_msamples_s": ns / res["sequential"] / 1e3,
            "speedup": res["sequential"] / res["tuned"]}


def run_reference(args, rank, world):
    if rank != 0:  # rank 0 alone times the CPU reference; the others exit without work
        return
    from oracle import binding as ob
    name = args.workload
    threads = ob.hardware_threads()
    results = []
    for i in range(args.warmup + args.steps):
        res, secs = cpu_baseline(name, threads, target_s=args.ref_seconds)
        if i >= args.warmup:
            results.append(res)
    v = statistics.median(r["value"] for r in results)
    line = {
        "impl": "reference", "metric": "Msamples/s", "value": v, "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[name]},
        "cpu_baseline": {"value": v, "unit": "Msamples/s", "cores": threads, "kind": "port",
                         "sample": results[-1]["sample"]},
        "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference crate unbuildable here (no Rust toolchain); timed arm is its f64 C++ restatement",
    }
    print(json.dumps(line), flush=True)


# DRAM bytes (read + write) per ray segment of the traversal kernels, from an
# ncu capture of every traversal launch of one frame (profiles/), by
# (workload, timed form); scaled to a frame by its ray segments.
DRAM_BYTES_PER_SEGMENT = {
    # 18 k_extend launches of one 512x512x64 frame: 20.76 GB over 86.67 M segments
    ("mesh", "wavefront_sorted"): 239.5,
    # 9 fused k_bounce launches of one 512x512x64 frame: 21.00 GB over 86.67 M segments
    ("mesh", "wavefront"): 242.3,
}

# Kernel configurations timed per workload: (form, material-sorted shading,
# BVH width). "megakernel" is the plain form: one thread per pixel-sample over
# binary node pairs.
FORMS = {
    "megakernel": ("megakernel", False, 2),
    "megakernel_wide": ("megakernel", False, 8),
    "wavefront": ("wavefront", False, 2),
    "wavefront_sorted": ("wavefront", True, 2),
    "wavefront_wide": ("wavefront", False, 8),
    "wavefront_sorted_wide": ("wavefront", True, 8),
}


def run_gpu(args, rank, world):
    import ctypes as C

    import torch

    from rayna_gb300 import Renderer
    from rayna_gb300 import _abi as A

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    scene, cam, opts = load_workload(args.workload)
    if args.width:
        opts.width = args.width
    if args.height:
        opts.height = args.height
    if args.spp:
        opts.samples = args.spp
    # a dedicated stream: the library launches on it, so events on it time its kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    forms = list(FORMS) if args.form == "best" else [args.form]
    results = {}
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    t_setup = time.perf_counter()
    for form in forms:
        kind, sort, width = FORMS[form]
        try:
            r = Renderer.new_from(scene, cam, opts, 0, form=kind, stream=stream.cuda_stream, seed=1000 + rank,
                                  stage_times=True)
            r.set_tuning(sort_materials=sort, bvh_width=width, fetch_budget=args.fetch_budget)
        except A.RaynaError as e:
            results[form] = {"error": str(e)}
            continue
        # counting frame: algorithmic work per frame (node visits, primitive tests)
        rc = Renderer.new_from(scene, cam, opts, 0, form=kind, stream=stream.cuda_stream, seed=99, counters=True)
        rc.set_tuning(sort_materials=sort, bvh_width=width, fetch_budget=args.fetch_budget)
        cst = rc.render().stats
        rc.close()
        lib, h = r._lib, r.handle
        st = A.rg_render_stats()
        for i in range(args.warmup):
            A.check(lib, h, lib.rg_render_async(h, r.next_seed(), None, C.byref(st)))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        rays = 0
        torch.cuda.synchronize()
        traverse_ms = 0.0
        with ClockSampler(dev) as clk:
            w0 = time.perf_counter()
            for k in range(args.steps):
                flush.fill_(float(k))
                starts[k].record(stream)
                A.check(lib, h, lib.rg_render_async(h, r.next_seed(), None, C.byref(st)))
                ends[k].record(stream)
                # the traversal kernels' own event pairs, read back after each frame
                A.check(lib, h, lib.rg_sync_stats(h, C.byref(st)))
                traverse_ms += st.traverse_ms
            torch.cuda.synchronize()
            wall = time.perf_counter() - w0
        if dist:
            dist.barrier()
        ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        dev_s = rank_max(sum(ms) / 1e3, dist, "cuda")
        samples = opts.width * opts.height * opts.samples
        assert st.error_flags == 0, st.error_flags
        # end-to-end: the public call with the image read back to host memory every frame
        e2e_s = float("nan")
        if not args.no_e2e:
            r.clear_accumulation()
            for _ in range(2):
                r.render()
            e0 = time.perf_counter()
            for _ in range(args.steps):
                out = r.render()
            e2e_s = time.perf_counter() - e0
            assert out.stats.error_flags == 0, out.stats.error_flags
        e2e_s = rank_max(e2e_s, dist, "cuda")
        results[form] = {
            "msamples_s": samples * args.steps * world / dev_s / 1e6,
            "ms_per_step": dev_s * 1e3 / args.steps,
            "e2e_msamples_s": samples * args.steps * world / e2e_s / 1e6,
            "mrays_s": cst.rays * args.steps * world / dev_s / 1e6,
            "rays_per_frame": cst.rays, "node_visits": cst.node_visits, "prim_tests": cst.prim_tests,
            "sdf_steps": cst.sdf_steps, "wall_s": wall, "clocks": clk.summary(), "device_ms": ms,
            "launches_per_frame": st.kernel_launches, "bvh_width": width,
            "traverse_ms_per_step": traverse_ms / args.steps,
        }
        r.close()
    if rank != 0:
        return
    ok = {f: v for f, v in results.items() if "error" not in v}
    best = max(ok, key=lambda f: ok[f]["msamples_s"])
    b = ok[best]
    hbm, peak_kind = measured_peaks()
    npx = opts.width * opts.height
    # Roofline of the dominant kernels, the traversal launches of a frame (the
    # megakernel, or the wavefront's extend / bounce kernels), timed live with
    # their own CUDA events: algorithmic bytes = one node fetch per node visit
    # (64 B pair, 80 B wide node) + 48 B per primitive test + the 48-byte path
    # record per ray segment.
    node_bytes = 80 if b["bvh_width"] == 8 else 64
    alg_bytes = node_bytes * b["node_visits"] + 48 * b["prim_tests"] + 48 * b["rays_per_frame"]
    achieved = alg_bytes / (b["traverse_ms_per_step"] / 1e3) / 1e9
    dram_per_segment = DRAM_BYTES_PER_SEGMENT.get((args.workload, best))
    traffic = dram_per_segment * b["rays_per_frame"] if dram_per_segment else None
    line = {
        "metric": "Msamples/s", "value": b["msamples_s"], "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": b["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "form": best, "l2": "flushed (512 MB write) between frames",
                   "parallelism": f"replicas{world}"},
        "e2e": {"value": b["e2e_msamples_s"], "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": npx * 12},
        "mrays_s": b["mrays_s"],
        "forms": {f: {k: v[k] for k in ("msamples_s", "mrays_s", "e2e_msamples_s", "ms_per_step", "rays_per_frame",
                                         "node_visits", "prim_tests", "sdf_steps", "wall_s", "launches_per_frame",
                                         "bvh_width")} if "error" not in v
                  else v for f, v in results.items()},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "traffic": traffic, "per": "frame (all traversal launches of one frame)",
                     "algorithmic_bytes": alg_bytes, "kernel_ms": b["traverse_ms_per_step"],
                     "kernel_share": b["traverse_ms_per_step"] / b["ms_per_step"]},
        "gpu_launches": b["launches_per_frame"] * args.steps,
        "clocks": b["clocks"],
    }
    if world == 1 and not args.no_adjoint:
        line["adjoint"] = run_adjoint(stream=stream)
    if world == 1 and args.batch_scale > 0:
        line["batch"] = run_batch(args.batch_scale, max(2, args.steps), stream=stream)
    if world == 1 and not args.no_cpu_baseline:
        from oracle import binding as ob
        cb, _ = cpu_baseline(args.workload, ob.hardware_threads(), target_s=args.ref_seconds)
        line["cpu_baseline"] = cb
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=list(WORKLOADS), default="mesh")
    ap.add_argument("--form", choices=["best"] + list(FORMS), default="best")
    ap.add_argument("--fetch-budget", type=int, default=0,
                    help="node visits between refills in the persistent wavefront kernels (0: library default)")
    ap.add_argument("--ref-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--width", type=int, default=0, help="override the workload resolution (profiling)")
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="resolution scale of the batched workload (1: the configured resolutions; 0: skip)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus if args.gpus == 1 else 1))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        import __graft_entry__ as g
        g.ensure_built()
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
