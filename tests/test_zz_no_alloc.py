"""The allocation-free entry point, rg_render_static_scratch, through the C ABI.

It exists for callers that cannot call cudaMalloc (a host that owns all device
memory through its own pool, or a render loop where allocation is not allowed):
the path queues live in a fixed device array inside the library, and the caller
passes its own accumulation and output buffers. Its image must equal the one
the regular entry point (rg_render) produces for the same seeds, frame after
frame. This file is collected last so that a failure here comes after every
other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from rayna_gb300 import Renderer, presets
from rayna_gb300 import _abi as A
from rayna_gb300.scene import RenderOpts

pytestmark = pytest.mark.gpu


def test_static_scratch_matches_rg_render_on_two_calls():
    torch = pytest.importorskip("torch")
    scene, cam, _ = presets.random_spheres(seed=0)
    # 96 x 54 pixels x 32 spp = 165,888 paths: more than the 65,536 static path
    # slots, so the frame runs in several waves.
    opts = RenderOpts(width=96, height=54, samples=32, ray_depth=12)
    seeds = [0x5EED0001, 0x5EED0002]
    with Renderer.new_from(scene, cam, opts, 0, form="megakernel") as ref:
        expected = [ref.render(seed=s).img.copy() for s in seeds]  # running means after 1 and 2 frames
    with Renderer.new_from(scene, cam, opts, 0, form="megakernel") as r:
        lib, h = r._lib, r.handle
        n = opts.width * opts.height * 3
        accum = torch.zeros(n, dtype=torch.float32, device="cuda")
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()  # the buffers are ready before the library's stream uses them
        for k, s in enumerate(seeds):
            st = lib.rg_render_static_scratch(h, s, C.c_void_p(accum.data_ptr()), k + 1, C.c_void_p(out.data_ptr()))
            A.check(lib, h, st)
            stats = A.rg_render_stats()
            A.check(lib, h, lib.rg_sync_stats(h, C.byref(stats)))
            assert stats.error_flags == 0
            # the stats describe this frame, not an earlier rg_render's
            assert stats.samples == opts.width * opts.height * opts.samples
            assert stats.kernel_ms > 0.0 and stats.kernel_launches > 0
            got = out.cpu().numpy().reshape(opts.width, opts.height, 3)
            np.testing.assert_array_equal(got, expected[k])


def test_static_scratch_sdf_scene_matches_rg_render():
    """Scenes with raymarched SDFs: rg_render gives each SDF's march stage a
    queue of its own (allocated with the path state); the allocation-free
    entry, which allocates nothing, sends every path that can reach some SDF
    through each stage. Both give the same image bits."""
    torch = pytest.importorskip("torch")
    scene, cam, _ = presets.sdf_volumes(n_spheres=20)
    opts = RenderOpts(width=64, height=36, samples=8, ray_depth=12)
    with Renderer.new_from(scene, cam, opts, 0, form="wavefront") as ref:
        expected = ref.render(seed=77).img.copy()
    with Renderer.new_from(scene, cam, opts, 0, form="wavefront") as r:
        lib, h = r._lib, r.handle
        n = opts.width * opts.height * 3
        accum = torch.zeros(n, dtype=torch.float32, device="cuda")
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        A.check(lib, h, lib.rg_render_static_scratch(h, 77, C.c_void_p(accum.data_ptr()), 1, C.c_void_p(out.data_ptr())))
        stats = A.rg_render_stats()
        A.check(lib, h, lib.rg_sync_stats(h, C.byref(stats)))
        assert stats.error_flags == 0
        np.testing.assert_array_equal(out.cpu().numpy().reshape(opts.width, opts.height, 3), expected)


def test_static_scratch_frame_stats_with_stage_times():
    """With RG_FLAG_STAGE_TIMES the regular entry times its traversal
    launches; the allocation-free entry does not (its events would be created
    on demand), so after it rg_sync_stats reports traverse_ms 0 and this
    frame's samples, call after call, instead of the earlier frame's figures."""
    torch = pytest.importorskip("torch")
    scene, cam, _ = presets.random_spheres(seed=0)
    opts = RenderOpts(width=64, height=36, samples=8, ray_depth=8)
    with Renderer.new_from(scene, cam, opts, 0, stage_times=True) as r:
        first = r.render(seed=3).stats
        assert first.traverse_ms > 0.0
        lib, h = r._lib, r.handle
        n = opts.width * opts.height * 3
        accum = torch.zeros(n, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        for k in range(4):
            A.check(lib, h, lib.rg_render_static_scratch(h, 100 + k, C.c_void_p(accum.data_ptr()), k + 1, None))
            stats = A.rg_render_stats()
            A.check(lib, h, lib.rg_sync_stats(h, C.byref(stats)))
            assert stats.traverse_ms == 0.0
            assert stats.samples == opts.width * opts.height * opts.samples
            assert stats.error_flags == 0


def test_static_scratch_rejects_sizes_beyond_its_array():
    torch = pytest.importorskip("torch")
    scene = presets.single_sphere((0.5, 0.5, 0.5))
    opts = RenderOpts(width=1, height=1, samples=65536 + 1, ray_depth=2)  # one pixel more than the array holds
    with Renderer.new_from(scene, presets.look_at_camera((0, 0, -3), (0, 0, 0), 40.0), opts, 0) as r:
        lib, h = r._lib, r.handle
        buf = torch.zeros(3, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = lib.rg_render_static_scratch(h, 1, C.c_void_p(buf.data_ptr()), 1, None)
        assert st == A.RG_INVALID_ARG
        assert "65536" in A.last_error(lib, h)
        st = lib.rg_render_static_scratch(h, 1, C.c_void_p(buf.data_ptr()), 0, None)
        assert st == A.RG_INVALID_ARG
