"""Benchmark of the per-sample path-tracing hot path on one GB300.

A step is one progressive frame (Renderer::render, render/renderer.rs:224)
of a workload at its full resolution and samples per pixel. The headline
workload is the triangle mesh (displaced icosphere of 1,310,720 triangles in
a 12-triangle Cornell box, 1024x1024, 64 spp, depth 8); by default the run
also times the random-spheres workload (400x225, 32 spp, depth 50) and the
SDF + media workload (1280x720, 128 spp, depth 16), reported under
`workloads` with their own roofline and CPU baseline.

Every workload times the plain megakernel and the wavefront form (fused for
the mesh and the spheres, material-sorted for the SDF scene, the library's
defaults), so the wavefront / megakernel ratio is in the same line.

Prints one JSON line:
  value    Msamples/s of the headline workload's fastest form, over K frames,
           inputs resident in HBM, device time (CUDA events around each frame
           on the renderer's stream; the L2 is flushed with a 512 MB write
           between frames, outside the events)
  e2e      the same metric through the public API (Renderer.render -> C ABI
           rg_render) with the image copied back to host memory every frame
  roofline of the dominant kernels (the traversal launches), see roofline()
  cpu_baseline, clocks, gpu_launches, workloads, adjoint, batch

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
    sample of the workload: a centred window of the full-resolution frame
    (same scene, camera, pixels, depth and spp), sized to about `target_s`
    seconds of work."""
    from oracle import binding as ob
    from rayna_gb300.scene import flatten
    scene, cam, opts = load_workload(name)
    flat = flatten(scene)

    def centred(w, h):
        return ((opts.width - w) // 2, (opts.height - h) // 2, w, h)

    st, _, _, secs = ob.render_window(flat, cam, opts, centred(16, 16), seed=1, policy=ob.POLICY_REF_F64,
                                      threads=threads)
    assert st == 0
    per_px = max(secs, 1e-3) / (16 * 16)
    npx = int(max(256, min(opts.width * opts.height, target_s / per_px)))
    w = min(opts.width, max(16, int(round((npx * opts.width / opts.height) ** 0.5))))
    h = min(opts.height, max(16, int(round(npx / w))))
    st, _, _, secs = ob.render_window(flat, cam, opts, centred(w, h), seed=2, policy=ob.POLICY_REF_F64,
                                      threads=threads)
    assert st == 0
    ns = w * h * opts.samples
    return {"value": ns / secs / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"centred {w}x{h} window of the {opts.width}x{opts.height} frame x {opts.samples} spp "
                      f"({ns / 1e6:.2f} M samples, {secs:.1f} s), f64 oracle, {threads} threads"}, secs


def run_adjoint(iters: int = 5, stream=None, width: int = 512, height: int = 512):
    """Differentiable-rendering workload: 1000 Lambertian spheres (3000 albedo
    parameters) + one medium (3 albedo + 1 density), 512x512, forward and
    backward at 16 spp, depth 8, L2 loss against a 1024-spp target of the
    ground-truth parameters; Adam steps on the host. Each iteration renders the
    forward frame, then takes the adjoint of that frame (rg_backward_frame: its
    image, the paths of an independent frame key replayed). Returns timings.
    `width`, `height`: a smaller image of the same scene (profiling)."""
    import torch

    from rayna_gb300 import Renderer, presets
    scene, cam, opts = presets.adjoint_scene(n_spheres=1000, ground_truth=False, width=width, height=height)
    gt, _, _ = presets.adjoint_scene(n_spheres=1000, ground_truth=True, width=width, height=height)
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
# ncu capture of the traversal launches of one frame (the profile summaries
# beside this file), by (workload, timed form); scaled to a frame by its ray
# segments.
DRAM_BYTES_PER_SEGMENT = {
    # 18 k_extend launches of one 512x512x64 frame: 20.76 GB over 86.67 M segments
    ("mesh", "wavefront_sorted"): 239.5,
    # 9 fused k_bounce launches of one 512x512x64 frame: 21.31 GB over 86.67 M segments
    ("mesh", "wavefront"): 245.9,
}

# Kernel configurations: (form, material-sorted shading, BVH width). The
# megakernel is the plain form: one thread per pixel-sample.
FORMS = {
    "megakernel": ("megakernel", False, 2),
    "megakernel_wide": ("megakernel", False, 8),
    "wavefront": ("wavefront", False, 2),
    "wavefront_sorted": ("wavefront", True, 2),
    "wavefront_wide": ("wavefront", False, 8),
    "wavefront_sorted_wide": ("wavefront", True, 8),
}
# Forms timed by default: the plain megakernel and the wavefront form the
# library picks for the scene (fused, or material-sorted for SDFs and media).
DEFAULT_FORMS = {"mesh": ["megakernel", "wavefront"], "spheres": ["megakernel", "wavefront"],
                 "sdf": ["megakernel", "wavefront_sorted"]}

# Algorithmic work per unit (one node visit, one primitive test, one SDF
# evaluation, one Mandelbulb escape iteration, one hit), fixed by formula:
#   bytes: 64 per binary node pair (80 per 8-wide node), 48 per triangle test
#          (v0, e1, e2), 16 per sphere test (centre, radius), 36 per normal
#          fetch and 32 per material fetch at a hit, 12 per output pixel;
#   FP32:  48 per binary node pair (two slab tests of 12 sub/mul + 12
#          min/max), 184 per 8-wide node, 27 per Moller-Trumbore test, 17 per
#          sphere test, 12 per SDF evaluation outside the escape loop, 55 per
#          Mandelbulb iteration (the z^8 step by three complex squarings);
#   SFU:   1 per triangle test (reciprocal), 1 per sphere test (square root),
#          2 per SDF evaluation (square root, logarithm), 6 per Mandelbulb
#          iteration (two square roots, four divisions).
PRIM_COST = {"mesh": (48, 27, 1), "spheres": (16, 17, 1), "sdf": (16, 17, 1)}  # bytes, FP32, SFU per test


def roofline(workload: str, r: dict, hbm_gbs: float, sm_count: int, sm_mhz: float) -> dict:
    """Roofline of the dominant kernels of one frame (the traversal launches:
    the megakernel, or the wavefront's bounce / extend / march kernels; their
    time is the timed frames' device time times their share of a frame,
    measured with their own CUDA events on separate frames): achieved = the largest of algorithmic bytes / time
    against the measured HBM copy bandwidth, FP32 operations / time against
    SMs x 128 lanes x 2 (FMA) x the sampled SM clock, and SFU operations / time
    against SMs x 16 x the sampled clock."""
    t = r["traverse_ms_per_step"] / 1e3
    wide = r["bvh_width"] == 8
    pb, pf, ps = PRIM_COST[workload]
    npx = r["pixels"]
    alg_bytes = (80 if wide else 64) * r["node_visits"] + pb * r["prim_tests"] + (36 + 32) * r["hits"] + 12 * npx
    flops = (184 if wide else 48) * r["node_visits"] + pf * r["prim_tests"] + 12 * r["sdf_steps"] + 55 * r["sdf_iterations"]
    sfu = ps * r["prim_tests"] + 2 * r["sdf_steps"] + 6 * r["sdf_iterations"]
    fp32_peak = sm_count * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s
    sfu_peak = sm_count * 16 * sm_mhz * 1e6 / 1e12         # Tops/s
    terms = {
        "hbm": {"achieved": alg_bytes / t / 1e9, "peak": hbm_gbs, "unit": "GB/s"},
        "fp32": {"achieved": flops / t / 1e12, "peak": fp32_peak, "unit": "TFLOP/s"},
        "sfu": {"achieved": sfu / t / 1e12, "peak": sfu_peak, "unit": "Tops/s"},
    }
    for v in terms.values():
        v["frac"] = v["achieved"] / v["peak"]
    bound = max(terms, key=lambda k: terms[k]["frac"])
    dram = DRAM_BYTES_PER_SEGMENT.get((workload, r["form"]))
    traffic = dram * r["rays_per_frame"] if dram else None
    b = terms[bound]
    return {"bound": bound, "achieved": b["achieved"], "peak": b["peak"], "unit": b["unit"], "frac": b["frac"],
            "traffic": traffic, "dram_frac": traffic / t / 1e9 / hbm_gbs if traffic else None,
            "terms": terms, "per": "frame (all traversal launches of one frame)",
            "algorithmic_bytes": alg_bytes, "fp32_ops": flops, "sfu_ops": sfu, "kernel_ms": t * 1e3,
            "kernel_share": r["traverse_ms_per_step"] / r["ms_per_step"],
            "peak_kind": "hbm: measured; fp32, sfu: SM count x lanes x sampled SM clock"}


def time_form(name, scene, cam, opts, form, steps, warmup, stream, flush, rank, world, dist, dev, args, e2e=True):
    """Times `steps` frames of one kernel configuration (after `warmup`) and
    a counting frame for the work per frame."""
    import ctypes as C

    import torch

    from rayna_gb300 import Renderer
    from rayna_gb300 import _abi as A
    kind, sort, width = FORMS[form]
    r = Renderer.new_from(scene, cam, opts, 0, form=kind, stream=stream.cuda_stream, seed=1000 + rank)
    r.set_tuning(sort_materials=sort, bvh_width=width, fetch_budget=args.fetch_budget)
    # counting frame: algorithmic work per frame (node visits, primitive tests, SDF steps, hits)
    rc = Renderer.new_from(scene, cam, opts, 0, form=kind, stream=stream.cuda_stream, seed=99, counters=True)
    rc.set_tuning(sort_materials=sort, bvh_width=width, fetch_budget=args.fetch_budget)
    cst = rc.render().stats
    rc.close()
    lib, h = r._lib, r.handle
    st = A.rg_render_stats()
    for _ in range(warmup):
        A.check(lib, h, lib.rg_render_async(h, r.next_seed(), None, C.byref(st)))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    launches = 0
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        w0 = time.perf_counter()
        for k in range(steps):
            flush.fill_(float(k))
            starts[k].record(stream)
            A.check(lib, h, lib.rg_render_async(h, r.next_seed(), None, C.byref(st)))
            ends[k].record(stream)
            launches += st.kernel_launches
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    # The traversal kernels' share of a frame, from their own event pairs
    # (RG_FLAG_STAGE_TIMES) on separate frames: recording those events between
    # launches costs time, so the timed frames above carry none.
    rs = Renderer.new_from(scene, cam, opts, 0, form=kind, stream=stream.cuda_stream, seed=2000 + rank,
                           stage_times=True)
    rs.set_tuning(sort_materials=sort, bvh_width=width, fetch_budget=args.fetch_budget)
    trav, frame = [], []
    for k in range(4):
        flush.fill_(float(k))
        A.check(rs._lib, rs.handle, rs._lib.rg_render_async(rs.handle, rs.next_seed(), None, C.byref(st)))
        A.check(rs._lib, rs.handle, rs._lib.rg_sync_stats(rs.handle, C.byref(st)))
        if k:
            trav.append(st.traverse_ms)
            frame.append(st.kernel_ms)
    rs.close()
    share = sum(trav) / max(sum(frame), 1e-9)
    if dist:
        dist.barrier()
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    dev_s = rank_max(sum(ms) / 1e3, dist, "cuda")
    samples = opts.width * opts.height * opts.samples
    e2e_s = float("nan")
    if e2e:
        # end to end: the public call with the image read back to host memory every frame
        r.clear_accumulation()
        for _ in range(2):
            r.render()
        # short frames are timed over about a quarter of a second of frames, so
        # one host hiccup does not decide the mean
        e2e_frames = max(steps, min(400, int(0.25 / max(dev_s / steps, 1e-6))))
        e0 = time.perf_counter()
        for _ in range(e2e_frames):
            out = r.render()
        e2e_s = (time.perf_counter() - e0) * steps / e2e_frames
        assert out.stats.error_flags == 0, out.stats.error_flags
    e2e_s = rank_max(e2e_s, dist, "cuda")
    r.close()
    return {
        "form": form, "msamples_s": samples * steps * world / dev_s / 1e6, "ms_per_step": dev_s * 1e3 / steps,
        "e2e_msamples_s": samples * steps * world / e2e_s / 1e6 if e2e else None,
        "mrays_s": cst.rays * steps * world / dev_s / 1e6, "rays_per_frame": cst.rays,
        "node_visits": cst.node_visits, "prim_tests": cst.prim_tests, "sdf_steps": cst.sdf_steps,
        "sdf_iterations": cst.sdf_iterations, "hits": cst.hits, "pixels": opts.width * opts.height,
        "wall_s": wall, "clocks": clk.summary(), "launches_per_frame": launches // max(steps, 1),
        "bvh_width": width, "traverse_ms_per_step": dev_s * 1e3 / steps * share, "traverse_share": share,
        "steps": steps,
    }


def run_workload(name, forms, steps, warmup, stream, flush, rank, world, dist, dev, args, e2e_best=True):
    """Every form of one workload; returns (results by form, best form)."""
    scene, cam, opts = load_workload(name)
    if name == args.workload:
        if args.width:
            opts.width = args.width
        if args.height:
            opts.height = args.height
        if args.spp:
            opts.samples = args.spp
    res = {}
    for form in forms:
        from rayna_gb300 import _abi as A
        try:
            res[form] = time_form(name, scene, cam, opts, form, steps, warmup, stream, flush, rank, world, dist,
                                  dev, args, e2e=False)
        except A.RaynaError as e:
            res[form] = {"error": str(e)}
    ok = {f: v for f, v in res.items() if "error" not in v}
    best = max(ok, key=lambda f: ok[f]["msamples_s"])
    if e2e_best and not args.no_e2e:
        # the best form again, end to end through Renderer.render
        res[best] = time_form(name, scene, cam, opts, best, steps, warmup, stream, flush, rank, world, dist, dev,
                              args, e2e=True)
    return res, best


def summarise(name, res, best, hbm, sm_count):
    """The per-workload JSON object: forms, ratio, roofline of the best form."""
    keys = ("msamples_s", "mrays_s", "e2e_msamples_s", "ms_per_step", "rays_per_frame", "node_visits", "prim_tests",
            "sdf_steps", "sdf_iterations", "hits", "wall_s", "launches_per_frame", "bvh_width", "steps",
            "traverse_ms_per_step")
    b = res[best]
    clk = b["clocks"].get("sm_mhz") or 2070.0
    out = {"workload": WORKLOADS[name], "best_form": best, "msamples_s": b["msamples_s"],
           "forms": {f: ({k: v[k] for k in keys} if "error" not in v else v) for f, v in res.items()},
           "roofline": roofline(name, b, hbm, sm_count, clk), "clocks": b["clocks"]}
    if "megakernel" in res and "error" not in res["megakernel"]:
        wf = [f for f in res if f.startswith("wavefront") and "error" not in res[f]]
        if wf:
            w = max(wf, key=lambda f: res[f]["msamples_s"])
            out["wavefront_over_megakernel"] = res[w]["msamples_s"] / res["megakernel"]["msamples_s"]
    return out


def run_gpu(args, rank, world):
    import torch

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    if args.adjoint_only:  # the adjoint workload alone (profiling), at --width x --height when given
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        res = run_adjoint(iters=args.steps, stream=stream, width=args.width or 512, height=args.height or 512)
        print(json.dumps({"adjoint": res}), flush=True)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # a dedicated stream: the library launches on it, so events on it time its kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    hbm, _ = measured_peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    forms = (list(FORMS) if args.form == "all" else
             DEFAULT_FORMS[args.workload] if args.form == "default" else args.form.split(","))
    res, best = run_workload(args.workload, forms, args.steps, args.warmup, stream, flush, rank, world, dist, dev, args)
    if rank != 0 and not (world == 1):
        if dist:
            dist.destroy_process_group()
        return
    head = summarise(args.workload, res, best, hbm, sm_count)
    b = res[best]
    opts_px = b["pixels"]
    gpu_launches = sum(v["launches_per_frame"] * v["steps"] for v in res.values() if "error" not in v)
    line = {
        "metric": "Msamples/s", "value": b["msamples_s"], "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": b["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "form": best, "l2": "flushed (512 MB write) between frames",
                   "parallelism": f"replicas{world}", "build": "performance (-fmad=true)"},
        "e2e": {"value": b["e2e_msamples_s"], "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": opts_px * 12},
        "mrays_s": b["mrays_s"],
        "forms": head["forms"],
        "wavefront_over_megakernel": head.get("wavefront_over_megakernel"),
        "roofline": head["roofline"],
        "gpu_launches": gpu_launches,
        "clocks": b["clocks"],
    }
    if world == 1 and args.all_workloads:
        line["workloads"] = {}
        for name in WORKLOADS:
            if name == args.workload:
                continue
            sub_steps = min(args.steps, args.sub_steps)
            r2, b2 = run_workload(name, DEFAULT_FORMS[name], sub_steps, min(args.warmup, 3), stream, flush, rank,
                                  world, dist, dev, args)
            line["workloads"][name] = summarise(name, r2, b2, hbm, sm_count)
            line["gpu_launches"] += sum(v["launches_per_frame"] * v["steps"] for v in r2.values() if "error" not in v)
    if world == 1 and not args.no_adjoint:
        line["adjoint"] = run_adjoint(stream=stream)
    if world == 1 and args.batch_scale > 0:
        line["batch"] = run_batch(args.batch_scale, max(2, args.steps), stream=stream)
    if world == 1 and not args.no_cpu_baseline:
        from oracle import binding as ob
        threads = ob.hardware_threads()
        cb, _ = cpu_baseline(args.workload, threads, target_s=args.ref_seconds)
        line["cpu_baseline"] = cb
        for name, w in line.get("workloads", {}).items():
            w["cpu_baseline"], _ = cpu_baseline(name, threads, target_s=args.ref_seconds / 2)
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
    ap.add_argument("--form", default="default",
                    help="'default' (megakernel and the library's wavefront form), 'all', or a comma list of " +
                         ", ".join(FORMS))
    ap.add_argument("--fetch-budget", type=int, default=0,
                    help="node visits between refills in the persistent wavefront kernels (0: library default)")
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--width", type=int, default=0, help="override the workload resolution (profiling)")
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--only", action="store_true", help="time the --workload alone (no `workloads` sub-results)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run the adjoint workload alone (iterations = --steps; --width/--height shrink it)")
    ap.add_argument("--sub-steps", type=int, default=5, help="timed frames of the other workloads")
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="resolution scale of the batched workload (1: the configured resolutions; 0: skip)")
    args = ap.parse_args()
    args.all_workloads = not args.only
    if args.form not in ("default", "all"):
        for f in args.form.split(","):
            if f not in FORMS:
                ap.error(f"unknown form {f}")
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
