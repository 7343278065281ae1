"""BatchRenderer — many independent renders in one persistent launch.

Wraps rg_batch_* of include/rayna_gpu.h. `render()` adds one frame to every
render: by default as a batched wavefront (the paths of all renders in shared
waves, one persistent work-stealing launch per bounce), or as one persistent
launch over a global (scene, tile) queue; the frame is replayed as a CUDA
graph. `render_sequential()` produces the same frame with one megakernel
launch per render (the comparison form).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .scene import flatten


class BatchRenderer:
    def __init__(self, items, *, device: int = 0, stream: int | None = None, seed: int = 0,
                 exact: bool | None = None):
        """`items`: list of (scene, camera, opts). `exact`: the arithmetic-contract build."""
        self._lib = A.load_library(exact=exact)
        self.items = list(items)
        self._flats = [flatten(s) for s, _, _ in self.items]
        n = len(self.items)
        descs = (C.POINTER(A.rg_scene_desc) * max(n, 1))(*[C.pointer(f.desc) for f in self._flats])
        cams = (A.rg_camera * max(n, 1))(*[c.to_c() for _, c, _ in self.items])
        opts = (A.rg_render_opts * max(n, 1))(*[o.to_c() for _, _, o in self.items])
        d = A.rg_device_opts()
        d.device, d.stream = device, stream
        h = C.c_void_p()
        st = self._lib.rg_batch_create(C.byref(d), n, descs, cams, opts, C.byref(h))
        if st != A.RG_OK:
            raise A.RaynaError(st, "rg_batch_create failed")
        self._h = h
        self.seed = int(seed)
        self._frame = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rg_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != A.RG_OK:
            buf = C.create_string_buffer(1024)
            self._lib.rg_batch_last_error(self._h, buf, len(buf))
            raise A.RaynaError(st, buf.value.decode(errors="replace"))

    @property
    def n_samples(self) -> int:
        return sum(o.width * o.height * o.samples for _, _, o in self.items)

    def set_tuning(self, block: int = 0, blocks_per_sm: int = 0, rounds_per_item: int = 0, bvh_width: int = 0,
                   form="wavefront", wave_paths: int = 0, shade_lanes: int = 0):
        """rg_batch_tuning. form: "wavefront" (shared waves of path slots, the
        default) or "tiles" (a persistent megakernel over (render, tile) work
        items); block / blocks_per_sm / rounds_per_item shape the tile form,
        wave_paths the wavefront's path slots per wave and shade_lanes the
        ready lanes a warp of its bounce kernel shades together (0 = library
        defaults)."""
        t = A.rg_batch_tuning()
        t.block, t.blocks_per_sm, t.rounds_per_item = int(block), int(blocks_per_sm), int(rounds_per_item)
        t.bvh_width = int(bvh_width)
        t.form = {"wavefront": A.RG_BATCH_WAVEFRONT, "tiles": A.RG_BATCH_TILES}.get(form, form)
        t.wave_paths = int(wave_paths)
        t.shade_lanes = int(shade_lanes)
        self._check(self._lib.rg_batch_set_tuning(self._h, C.byref(t)))

    def next_seed(self) -> int:
        from .renderer import _mix_seed
        s = _mix_seed(self.seed, self._frame)
        self._frame += 1
        return s

    def render(self, seed: int | None = None) -> A.rg_render_stats:
        st = A.rg_render_stats()
        self._check(self._lib.rg_batch_render(self._h, self.next_seed() if seed is None else int(seed), C.byref(st)))
        return st

    def render_sequential(self, seed: int | None = None) -> A.rg_render_stats:
        st = A.rg_render_stats()
        self._check(self._lib.rg_batch_render_sequential(self._h, self.next_seed() if seed is None else int(seed),
                                                         C.byref(st)))
        return st

    def image(self, index: int) -> np.ndarray:
        o = self.items[index][2]
        img = np.empty((o.width, o.height, 3), np.float32)
        self._check(self._lib.rg_batch_image(self._h, int(index), img.ctypes.data_as(C.POINTER(C.c_float))))
        return img

    def item_seed(self, seed: int, index: int) -> int:
        return int(self._lib.rg_batch_item_seed(int(seed), int(index)))
