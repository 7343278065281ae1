"""Renderer — the GPU stand-in for rayna_engine's `Renderer<Obj, Sky, Rng>`.

Mirrors render/renderer.rs: `new_from(scene, camera, options, num_threads)`,
`new_default()`, `render() -> Render`, `set_scene/set_camera/set_options`
(each clears the accumulation), `clear_accumulation()`, `set_thread_count()`
and the `scene/camera/options` getters. Every call goes through the C ABI of
include/rayna_gpu.h; there is no CPU path.

Images are numpy arrays of shape (width, height, 3) — the reference's
`Image` is an ndarray of shape (width, height) of RGB pixels
(core/image.rs:24-25).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A
from .scene import Camera, RenderOpts, Scene, flatten


@dataclass
class RenderStats:
    """render/render.rs:4-15 plus device figures."""
    duration: float = 0.0          # seconds, wall time of render()
    num_threads: int = 0           # 0: the device renders
    opts: RenderOpts = field(default_factory=RenderOpts)
    accum_frames: int = 0
    kernel_ms: float = 0.0
    samples: int = 0
    rays: int = 0
    node_visits: int = 0
    prim_tests: int = 0
    sdf_steps: int = 0
    error_flags: int = 0
    traverse_ms: float = 0.0
    invalid_hits: int = 0          # validate=True: hits / colours breaking shared/validate.rs's invariants
    invalid_mask: int = 0          # which invariants (RG_INVALID_* bits)
    hits: int = 0                  # counters=True: closest-hit queries that found a surface
    sdf_iterations: int = 0        # counters=True: Mandelbulb escape-loop iterations


@dataclass
class Render:
    img: np.ndarray
    stats: RenderStats


def _mix_seed(base: int, frame: int) -> int:
    """SplitMix64 of (base, frame): the per-frame key of the random streams."""
    z = (base + 0x9E3779B97F4A7C15 * (frame + 1)) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


class Renderer:
    """GPU renderer with the reference Renderer's methods."""

    def __init__(self, scene: Scene, camera: Camera, options: RenderOpts, *, device: int = 0,
                 form: str = "wavefront", seed: int = 0, stream: int | None = None, counters: bool = False,
                 stage_times: bool = False, validate: bool = False, exact: bool | None = None):
        """`form`: "wavefront" (the default: persistent extend/bounce kernels
        over waves of path slots, 1.5-2.5x the plain form on the workloads) or
        "megakernel" (one thread per pixel-sample). Both render identical
        images; debug render modes and ray_branching > 1 always run the
        megakernel. `counters`, `stage_times`, `validate`: RG_FLAG_* (work
        counters, traversal timing, the reference's debug invariants).
        `exact`: render with the arithmetic-contract build (fused
        multiply-adds only where the source writes them; bit-exact with the
        oracle's f32 policy) instead of the performance build."""
        self._lib = A.load_library(exact=exact)
        dopts = A.rg_device_opts()
        dopts.device = device
        dopts.stream = stream
        dopts.form = {"megakernel": A.RG_FORM_MEGAKERNEL, "wavefront": A.RG_FORM_WAVEFRONT}[form]
        dopts.flags = ((A.RG_FLAG_COUNTERS if counters else 0) | (A.RG_FLAG_STAGE_TIMES if stage_times else 0) |
                       (A.RG_FLAG_VALIDATE if validate else 0))
        h = C.c_void_p()
        st = self._lib.rg_create(C.byref(dopts), C.byref(h))
        A.check(self._lib, None, st)
        self._h = h
        self._stack_knobs = (0, 0, 0)  # requested shared_stack, block, stack_limit (0: library defaults)
        self.form = form
        self.seed = int(seed)
        self._frame = 0
        self._scene = self._camera = self._options = None
        self._flat = None
        self.set_scene(scene)
        self.set_camera(camera)
        self.set_options(options)

    # -- construction --------------------------------------------------------
    @classmethod
    def new_from(cls, scene: Scene, camera: Camera, options: RenderOpts, num_threads: int = 0, **kw) -> "Renderer":
        """Renderer::new_from (renderer.rs:86-107). `num_threads` is accepted
        for signature parity; the device decides its own parallelism."""
        return cls(scene, camera, options, **kw)

    @classmethod
    def tuned(cls, scene: Scene, camera: Camera, options: RenderOpts, tuner=None, **kw) -> "Renderer":
        """A renderer with the kernel form and launch knobs the autotuner
        picked for this scene size (measured on first sight of the size, then
        cached)."""
        from .autotune import Tuner
        cfg = (tuner or Tuner()).tune_render(scene, camera, options, **kw)
        r = cls(scene, camera, options, form=cfg["form"], **kw)
        r.set_tuning(**{k: v for k, v in cfg.items() if k != "form"})
        return r

    @classmethod
    def new_default(cls, **kw) -> "Renderer":
        return cls(Scene(), Camera(), RenderOpts(), **kw)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- properties ----------------------------------------------------------
    @property
    def scene(self) -> Scene:
        return self._scene

    @property
    def camera(self) -> Camera:
        return self._camera

    @property
    def options(self) -> RenderOpts:
        return self._options

    @property
    def handle(self):
        return self._h

    def _check(self, st: int):
        A.check(self._lib, self._h, st)

    def clear_accumulation(self):
        self._check(self._lib.rg_clear_accumulation(self._h))

    def set_scene(self, scene: Scene):
        flat = flatten(scene)
        self._check(self._lib.rg_set_scene(self._h, C.byref(flat.desc)))
        self._scene, self._flat = scene, flat

    def set_camera(self, camera: Camera):
        self._check(self._lib.rg_set_camera(self._h, C.byref(camera.to_c())))
        self._camera = camera

    def set_options(self, options: RenderOpts):
        self._check(self._lib.rg_set_options(self._h, C.byref(options.to_c())))
        self._options = options

    @property
    def n_materials(self) -> int:
        return int(self._flat.desc.n_materials)

    @property
    def n_volumes(self) -> int:
        return int(self._flat.desc.n_volumes)

    def set_parameters(self, albedo=None, density=None):
        """Replaces material albedos (emissive radiance for lights), shape
        (n_materials, 3), and media densities, shape (n_volumes,), without
        rebuilding the BVH. Clears the accumulation."""
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        a = d = None
        if albedo is not None:
            a = np.ascontiguousarray(albedo, np.float32).reshape(self.n_materials, 3)
        if density is not None:
            d = np.ascontiguousarray(density, np.float32).reshape(self.n_volumes)
        self._check(self._lib.rg_set_parameters(self._h, fp(a) if a is not None else None,
                                                fp(d) if d is not None else None))

    def backward(self, seed: int, target=None, adjoint=None, last_frame: bool = False):
        """Adjoint of frame `seed` (rg_backward). With `target` (w, h, 3) the
        loss is sum (I - target)^2; otherwise `adjoint` is dLoss/dI. With
        `last_frame` (and a target) I is the last render()'s frame instead of
        frame `seed` rendered again (rg_backward_frame). Returns a dict with
        'loss', 'albedo' (n_materials, 3), 'emission' (n_materials, 3) and
        'density' (n_volumes,)."""
        o = self._options
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        t = adj = None
        if target is not None:
            t = np.ascontiguousarray(target, np.float32).reshape(o.width, o.height, 3)
        elif adjoint is not None:
            adj = np.ascontiguousarray(adjoint, np.float32).reshape(o.width, o.height, 3)
        else:
            raise ValueError("give a target or an adjoint image")
        ga = np.zeros((self.n_materials, 3), np.float32)
        ge = np.zeros((self.n_materials, 3), np.float32)
        gd = np.zeros(max(self.n_volumes, 1), np.float32)
        g = A.rg_gradients()
        g.albedo, g.emission, g.density = fp(ga), fp(ge), fp(gd)
        if last_frame:
            if t is None:
                raise ValueError("last_frame needs a target")
            self._check(self._lib.rg_backward_frame(self._h, int(seed), fp(t), C.byref(g)))
        else:
            self._check(self._lib.rg_backward(self._h, int(seed), fp(adj) if adj is not None else None,
                                              fp(t) if t is not None else None, C.byref(g)))
        return {"loss": g.loss, "albedo": ga, "emission": ge, "density": gd[: self.n_volumes]}

    def frame(self, seed: int) -> np.ndarray:
        """The image of frame `seed` alone (mean of its samples), leaving the
        running accumulation where it was."""
        sums, frames = self.get_accumulation()
        self.render(seed=seed)
        m, _ = self.frame_moments()
        self.set_accumulation(sums, frames)
        return m

    def set_tuning(self, wave_paths: int | None = None, sort_materials: bool | None = None,
                   bvh_width: int | None = None, fetch_budget: int | None = None, shared_stack: int | None = None,
                   block: int | None = None, stack_limit: int | None = None, march_budget: int | None = None,
                   shade_lanes: int | None = None, tail_paths: int | None = None):
        """Launch knobs (rg_tuning); None leaves a knob as it is. wave_paths:
        wavefront path slots per wave (0 = library default); sort_materials:
        wavefront shading in material-kind order (True) or one fused bounce
        kernel (False); bvh_width: 2 (binary node pairs) or 8 (compressed
        8-wide nodes), 0 = library default; fetch_budget: node visits a
        wavefront lane traverses between refills (0 = library default);
        shared_stack: traversal stack entries per thread in shared memory
        (0 = library default, -1 = none, else 4, 8 or 16); block: megakernel
        threads per block (0 = 128, else 64 or 256); stack_limit: a test knob
        capping the traversal stack a ray may use (0 = all 64); march_budget:
        SDF evaluations per lane between refills in the material-sorted
        wavefront's march stages (0 = 16); shade_lanes: ready lanes a warp
        of a persistent wavefront kernel finishes together (1-32, 0 = 16);
        tail_paths: a fused bounce whose queue holds at most this many paths
        runs them to their ends in that launch (0 = 2^22, 1 = off)."""
        t = A.rg_tuning()
        self._check(self._lib.rg_get_tuning(self._h, C.byref(t)))
        # the resolved defaults come back from rg_get_tuning; hand the requested knobs back
        t.shared_stack, t.block, t.stack_limit = self._stack_knobs
        if wave_paths is not None:
            t.wave_paths = int(wave_paths)
        if sort_materials is not None:
            t.sort_materials = 1 if sort_materials else 2
        if bvh_width is not None:
            t.bvh_width = int(bvh_width)
        if fetch_budget is not None:
            t.fetch_budget = int(fetch_budget)
        if shared_stack is not None:
            t.shared_stack = A.RG_SHARED_STACK_NONE if shared_stack < 0 else int(shared_stack)
        if block is not None:
            t.block = int(block)
        if stack_limit is not None:
            t.stack_limit = int(stack_limit)
        if march_budget is not None:
            t.march_budget = int(march_budget)
        if shade_lanes is not None:
            t.shade_lanes = int(shade_lanes)
        if tail_paths is not None:
            t.tail_paths = int(tail_paths)
        self._check(self._lib.rg_set_tuning(self._h, C.byref(t)))
        self._stack_knobs = (t.shared_stack, t.block, t.stack_limit)

    def tuning(self) -> dict:
        """The knobs in effect (library defaults resolved; shared_stack -1 = none)."""
        t = A.rg_tuning()
        self._check(self._lib.rg_get_tuning(self._h, C.byref(t)))
        return {"wave_paths": t.wave_paths, "sort_materials": t.sort_materials == 1, "bvh_width": t.bvh_width,
                "fetch_budget": t.fetch_budget,
                "shared_stack": -1 if t.shared_stack == A.RG_SHARED_STACK_NONE else t.shared_stack,
                "block": t.block, "stack_limit": t.stack_limit, "march_budget": t.march_budget,
                "shade_lanes": t.shade_lanes, "tail_paths": t.tail_paths}

    def set_sample_range(self, first: int, count: int):
        """Frames trace samples [first, first + count) of each pixel's
        `samples` and add their sum / samples to the accumulation
        (rg_set_sample_range): disjoint ranges on several devices sum to whole
        frames. count 0 restores whole frames; clears the accumulation."""
        self._check(self._lib.rg_set_sample_range(self._h, int(first), int(count)))

    def set_wave_paths(self, n: int, sort_materials: bool | None = None):
        """Wavefront path slots per wave (0: library default) and, optionally,
        whether shading runs in material-kind order (separate stages)."""
        self.set_tuning(wave_paths=n, sort_materials=sort_materials)

    def set_thread_count(self, num_threads: int):
        """Accepted for API parity (renderer.rs:179-182); the device is not thread-pooled."""
        return None

    # -- rendering -----------------------------------------------------------
    def next_seed(self) -> int:
        s = _mix_seed(self.seed, self._frame)
        self._frame += 1
        return s

    def render(self, seed: int | None = None) -> Render:
        """Renderer::render (renderer.rs:224-264): one progressive frame."""
        o = self._options
        img = np.empty((o.width, o.height, 3), dtype=np.float32)
        stats = A.rg_render_stats()
        t0 = time.perf_counter()
        s = self.next_seed() if seed is None else int(seed)
        st = self._lib.rg_render(self._h, s, img.ctypes.data_as(C.POINTER(C.c_float)), C.byref(stats))
        dt = time.perf_counter() - t0
        if st == A.RG_INVALID_CAMERA:
            # render_failed: the magenta checker of ilog2 dimensions
            img = np.ascontiguousarray(img.reshape(-1)[: stats.img_width * stats.img_height * 3]
                                       .reshape(stats.img_width, stats.img_height, 3))
        else:
            self._check(st)
        rs = RenderStats(duration=dt, num_threads=0, opts=o, accum_frames=stats.accum_frames,
                         kernel_ms=stats.kernel_ms, samples=stats.samples, rays=stats.rays,
                         node_visits=stats.node_visits, prim_tests=stats.prim_tests,
                         sdf_steps=stats.sdf_steps, error_flags=stats.error_flags, traverse_ms=stats.traverse_ms,
                         invalid_hits=stats.invalid_hits, invalid_mask=stats.invalid_mask, hits=stats.hits,
                         sdf_iterations=stats.sdf_iterations)
        return Render(img=img, stats=rs)

    def frame_moments(self):
        """Per-pixel mean and sample variance of the last frame's samples."""
        o = self._options
        m = np.empty((o.width, o.height, 3), np.float32)
        v = np.empty_like(m)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._check(self._lib.rg_frame_moments(self._h, fp(m), fp(v)))
        return m, v

    def get_accumulation(self):
        o = self._options
        s = np.empty((o.width, o.height, 3), np.float32)
        n = C.c_uint32()
        self._check(self._lib.rg_get_accumulation(self._h, s.ctypes.data_as(C.POINTER(C.c_float)), C.byref(n)))
        return s, n.value

    def set_accumulation(self, sums: np.ndarray, frames: int):
        s = np.ascontiguousarray(sums, dtype=np.float32)
        self._check(self._lib.rg_set_accumulation(self._h, s.ctypes.data_as(C.POINTER(C.c_float)), int(frames)))

    def query_rays(self, origins, dirs, tmin=1e-3, tmax=3.4028235e38, volume_u=None) -> np.ndarray:
        """Closest-hit queries against the current scene; returns a structured
        array with the fields of rg_hit."""
        o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        n = o.shape[0]
        t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(tmin, np.float32), (n,)))
        t1 = np.ascontiguousarray(np.broadcast_to(np.asarray(tmax, np.float32), (n,)))
        out = (A.rg_hit * max(1, n))()
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        vu = None
        if volume_u is not None:
            vu_arr = np.ascontiguousarray(volume_u, np.float32)
            vu = fp(vu_arr)
        self._check(self._lib.rg_query_rays(self._h, n, fp(o), fp(d), fp(t0), fp(t1), vu, out))
        return hits_to_numpy(out, n)


HIT_DTYPE = np.dtype([("hit", np.uint32), ("prim", np.uint32), ("t", np.float32), ("normal", np.float32, 3),
                      ("ray_normal", np.float32, 3), ("front_face", np.uint32), ("material", np.uint32),
                      ("side", np.uint32)])
assert HIT_DTYPE.itemsize == 48


def inspect_scene(scene) -> dict:
    """Builds a scene's trees on the host only (rg_inspect_scene) and returns
    their statistics; raises RaynaError when the scene is rejected."""
    from .scene import flatten
    lib = A.load_library()
    flat = flatten(scene)
    info = A.rg_scene_info()
    st = lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info))
    if st != A.RG_OK:
        buf = C.create_string_buffer(1024)
        lib.rg_last_error(None, buf, len(buf))
        raise A.RaynaError(st, buf.value.decode(errors="replace"))
    return {k: getattr(info, k) for k, _ in A.rg_scene_info._fields_}


def hits_to_numpy(buf, n: int) -> np.ndarray:
    raw = np.frombuffer(buf, dtype=HIT_DTYPE, count=n)
    return raw.copy()
