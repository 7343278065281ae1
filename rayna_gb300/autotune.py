"""Autotuner of the launch shapes, keyed on primitive count and resolution.

The image never depends on these knobs (every form and shape renders the same
bits); only the time does. A key is

    kind : log2 bucket of primitives : log2 bucket of pixels : log2 bucket of spp

and its entry records the best configuration found and the timings of every
candidate. Single renders choose between the megakernel and the wavefront
form; for the megakernel the tree (binary or 8-wide), the traversal stack's
placement (entries per thread in shared memory) and the block size; for the
wavefront the tree, fused or material-sorted shading, the node visits between
refills of the persistent traversal kernels, the path budget per wave (queue
capacity), the stack placement and, for scenes with raymarched SDFs, the
evaluations per lane between refills of the march stages. Each form is searched by coordinate
descent: from the library defaults, one knob at a time over its candidates,
keeping the best, in a fixed order. Batches choose the batched form (wavefront
with its path slots per wave, or tiles with the persistent kernel's block
size, blocks per SM and the work-item granularity of the global queue).
Entries live in a JSON file (RAYNA_GB300_TUNE_CACHE, default
~/.cache/rayna_gb300/tuning_cache.json) and are measured with CUDA events on
the device the first time a key is seen.
"""
from __future__ import annotations

import json
import math
import os
import time

from . import _abi as A

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "rayna_gb300", "tuning_cache.json")

WAVE_PATHS = [1 << 24, 1 << 25, 1 << 26, 1 << 27]
FETCH_BUDGETS = [4, 6, 8, 16]
BVH_WIDTHS = [2, 8]
SHARED_STACKS = [-1, 8, 16]  # -1: the whole traversal stack in local memory
MEGA_BLOCKS = [64, 128, 256]
# Coordinate-descent axes per form, searched in this order.
MEGA_AXES = [("bvh_width", BVH_WIDTHS), ("shared_stack", SHARED_STACKS), ("block", MEGA_BLOCKS)]
MARCH_BUDGETS = [8, 16, 32, 64]
SHADE_LANES = [1, 8, 16, 24]
TAIL_PATHS = [1, 1 << 16, 1 << 22, 1 << 30]  # 1: no continuation; 2^30: every path runs to its end in its first launch
WAVE_AXES = [("sort_materials", [False, True]), ("bvh_width", BVH_WIDTHS), ("shared_stack", SHARED_STACKS),
             ("fetch_budget", FETCH_BUDGETS), ("shade_lanes", SHADE_LANES), ("tail_paths", TAIL_PATHS),
             ("wave_paths", WAVE_PATHS)]
WAVE_SDF_AXES = WAVE_AXES + [("march_budget", MARCH_BUDGETS)]
BATCH_SHAPES = ([dict(form="wavefront", wave_paths=w) for w in (1 << 25, 1 << 26, 1 << 27)] +
                [dict(form="tiles", block=b, blocks_per_sm=0, rounds_per_item=r) for b in (64, 128, 256) for r in (1, 4, 16)])


def _bucket(n: int) -> int:
    return int(math.floor(math.log2(max(int(n), 1))))


def render_key(n_prims: int, width: int, height: int, spp: int) -> str:
    return f"render:p{_bucket(n_prims)}:r{_bucket(width * height)}:s{_bucket(spp)}"


def batch_key(n_items: int, n_prims: int, n_pixels: int, n_samples: int) -> str:
    return f"batch:n{_bucket(n_items)}:p{_bucket(n_prims)}:r{_bucket(n_pixels)}:s{_bucket(n_samples)}"


class Tuner:
    def __init__(self, path: str | None = None):
        self.path = path or os.environ.get("RAYNA_GB300_TUNE_CACHE", DEFAULT_CACHE)
        self.table = {}
        if os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.table = json.load(f)
            except (OSError, ValueError):
                self.table = {}

    def lookup(self, key: str):
        e = self.table.get(key)
        return e["best"] if e else None

    def store(self, key: str, best: dict, timings: list):
        self.table[key] = {"best": best, "timings": timings, "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.table, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    # -- single renders ------------------------------------------------------
    @staticmethod
    def _frame_ms(r, frames: int, seed0: int) -> float:
        import ctypes as C
        ms = []
        st = A.rg_render_stats()
        for k in range(frames + 1):
            A.check(r._lib, r.handle, r._lib.rg_render_async(r.handle, seed0 + k, None, C.byref(st)))
            A.check(r._lib, r.handle, r._lib.rg_sync_stats(r.handle, C.byref(st)))
            if k:
                ms.append(st.kernel_ms)
        return sorted(ms)[len(ms) // 2]

    @classmethod
    def _descend(cls, r, form: str, axes, start: dict, frames: int, seed0: int, timings: list, opts) -> dict:
        """Coordinate descent over `axes` from `start`; returns the best knobs."""
        best = dict(start)
        r.set_tuning(**best)
        best_ms = cls._frame_ms(r, frames, seed0)
        timings.append(dict(best, form=form, ms=best_ms))
        for name, values in axes:
            for v in values:
                if v == best.get(name) or (name == "wave_paths" and v < opts.samples):
                    continue
                cand = dict(best, **{name: v})
                r.set_tuning(**cand)
                ms = cls._frame_ms(r, frames, seed0)
                timings.append(dict(cand, form=form, ms=ms))
                if ms < best_ms:
                    best, best_ms = cand, ms
        r.set_tuning(**best)
        return dict(best, form=form, ms=best_ms)

    def tune_render(self, scene, camera, opts, frames: int = 2, force: bool = False, **renderer_kw) -> dict:
        """Best launch configuration for this scene size; measured once per key."""
        from .renderer import Renderer
        from .scene import flatten
        flat = flatten(scene)
        key = render_key(flat.n_prims, opts.width, opts.height, opts.samples)
        if not force and self.lookup(key):
            return self.lookup(key)
        timings = []
        results = []
        with Renderer.new_from(scene, camera, opts, 0, form="megakernel", **renderer_kw) as r:
            d = r.tuning()
            start = {"bvh_width": d["bvh_width"], "shared_stack": d["shared_stack"], "block": d["block"]}
            results.append(self._descend(r, "megakernel", MEGA_AXES, start, frames, 1000, timings, opts))
        with Renderer.new_from(scene, camera, opts, 0, form="wavefront", **renderer_kw) as r:
            d = r.tuning()
            start = {k: d[k] for k in ("sort_materials", "bvh_width", "shared_stack", "fetch_budget", "shade_lanes",
                                       "tail_paths", "wave_paths")}
            axes = WAVE_AXES
            if flat.desc.n_sdfs:  # the march stages' refill budget
                start["march_budget"] = d["march_budget"]
                axes = WAVE_SDF_AXES
            results.append(self._descend(r, "wavefront", axes, start, frames, 2000, timings, opts))
        best = min(results, key=lambda t: t["ms"])
        cfg = {k: v for k, v in best.items() if k != "ms"}
        self.store(key, cfg, timings)
        return cfg

    # -- batches -------------------------------------------------------------
    def tune_batch(self, batch, frames: int = 1, force: bool = False) -> dict:
        """Best persistent-kernel shape for this batch size; measured once per key."""
        from .scene import flatten
        n_prims = sum(flatten(s).n_prims for s, _, _ in batch.items)
        n_pix = sum(o.width * o.height for _, _, o in batch.items)
        key = batch_key(len(batch.items), n_prims, n_pix, batch.n_samples)
        if not force and self.lookup(key):
            cfg = self.lookup(key)
            batch.set_tuning(**cfg)
            return cfg
        timings = []
        for shape in BATCH_SHAPES:
            try:
                batch.set_tuning(**shape)
            except A.RaynaError:
                continue
            batch.render(seed=1)
            ms = []
            for k in range(frames):
                ms.append(batch.render(seed=2 + k).kernel_ms)
            timings.append(dict(shape, ms=sorted(ms)[len(ms) // 2]))
        best = min(timings, key=lambda t: t["ms"])
        cfg = {k: v for k, v in best.items() if k != "ms"}
        batch.set_tuning(**cfg)
        self.store(key, cfg, timings)
        return cfg
