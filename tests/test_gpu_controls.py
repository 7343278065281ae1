"""Launch knobs, failure statuses and sample-range sharding on the GPU,
through the C ABI.

* Stack placement (shared entries per thread), the megakernel's block
  size and the ready lanes a wavefront warp finishes together change only
  the time: every setting renders the same image.
* Device errors are statuses: a traversal stack capped below what a ray
  needs (the rg_tuning.stack_limit test knob) makes the frame return
  RG_QUEUE_OVERFLOW promptly, and the next normal frame returns RG_OK (the
  error bits are cleared per frame). Nothing waits or traps: the kernels set
  a bit and drop the far subtree.
* A forced allocation failure (RAYNA_GPU_FAIL_ALLOC, in a child process)
  returns RG_OOM from rg_set_scene and leaves the handle usable.
* Sample ranges: handles that cover disjoint ranges of every pixel's
  samples hold accumulation sums that add up to the whole frame's, and each
  range equals the f32 oracle's render of the same samples path for path.
"""
import ctypes as C
import os
import subprocess
import sys
import time

import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300 import RaynaError, Renderer, presets
from rayna_gb300 import _abi as A
from rayna_gb300.scene import RenderOpts, flatten

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def small(fn, w, h, spp, depth, **kw):
    scene, cam, _ = fn(**kw)
    return scene, cam, RenderOpts(width=w, height=h, samples=spp, ray_depth=depth)


@pytest.mark.parametrize("case", ["mesh", "spheres"])
def test_stack_placement_and_block_do_not_change_images(case):
    scene, cam, opts = (small(presets.cornell_mesh, 48, 48, 8, 8, level=5) if case == "mesh"
                        else small(presets.random_spheres, 64, 36, 8, 12))
    imgs = {}
    for form, knobs in [("megakernel", dict(shared_stack=sh, block=b)) for sh in (-1, 4, 8, 16) for b in (64, 128, 256)] + \
                       [("wavefront", dict(shared_stack=sh, sort_materials=so)) for sh in (-1, 8, 16) for so in (False, True)] + \
                       [("wavefront", dict(shared_stack=8, sort_materials=so, shade_lanes=sl))
                        for so in (False, True) for sl in (1, 7, 32)] + \
                       [("wavefront", dict(shared_stack=8, sort_materials=False, tail_paths=tp)) for tp in (1, 100, 1 << 30)]:
        with Renderer.new_from(scene, cam, opts, 0, form=form) as r:
            r.set_tuning(**knobs)
            t = r.tuning()
            assert t["shared_stack"] == knobs["shared_stack"]
            if form == "megakernel":
                assert t["block"] == knobs["block"]
            out = r.render(seed=17)
            assert out.stats.error_flags == 0
            imgs[(form, tuple(sorted(knobs.items())))] = out.img
    first = next(iter(imgs.values()))
    for k, v in imgs.items():
        np.testing.assert_array_equal(v, first, err_msg=str(k))


def test_tuning_rejects_unknown_stack_and_block_values():
    scene, cam, opts = small(presets.random_spheres, 8, 8, 1, 2)
    with Renderer.new_from(scene, cam, opts, 0) as r:
        for bad in (dict(shared_stack=3), dict(block=96), dict(stack_limit=65), dict(shade_lanes=33)):
            with pytest.raises(RaynaError) as e:
                r.set_tuning(**bad)
            assert e.value.status == A.RG_INVALID_ARG
        # defaults resolve: 8 shared entries for triangle-only scenes, none otherwise
        assert r.tuning()["shared_stack"] == -1 and r.tuning()["block"] == 128 and r.tuning()["stack_limit"] == 64
        assert r.tuning()["shade_lanes"] == 16 and r.tuning()["tail_paths"] == 1 << 22


@pytest.mark.parametrize("form,width", [("megakernel", 2), ("megakernel", 8), ("wavefront", 2), ("wavefront", 8)])
def test_stack_overflow_is_a_status_and_clears_next_frame(form, width):
    scene, cam, opts = small(presets.cornell_mesh, 32, 32, 4, 6, level=5)
    with Renderer.new_from(scene, cam, opts, 0, form=form) as r:
        r.set_tuning(bvh_width=width, stack_limit=1)
        t0 = time.perf_counter()
        with pytest.raises(RaynaError) as e:
            r.render(seed=1)
        assert e.value.status == A.RG_QUEUE_OVERFLOW
        assert "0x1" in str(e.value)  # RG_DEVICE_STACK_OVERFLOW
        assert time.perf_counter() - t0 < 30.0
        # the same knob on a query
        o = np.full((64, 3), 0.5, np.float32)
        d = np.random.default_rng(0).normal(size=(64, 3)).astype(np.float32)
        with pytest.raises(RaynaError) as e:
            r.query_rays(o, d)
        assert e.value.status == A.RG_QUEUE_OVERFLOW
        r.set_tuning(stack_limit=0)
        out = r.render(seed=2)  # raises unless RG_OK
        assert out.stats.error_flags == 0
        assert r.query_rays(o, d)["hit"].sum() > 0


def test_forced_device_allocation_failure_returns_oom():
    """The first counted allocation of rg_set_scene is the host scene build
    (1); the device uploads follow (2, 3, ...). Failing the second device
    upload returns RG_OOM; the next rg_set_scene succeeds and renders."""
    code = (
        "import ctypes as C, numpy as np\n"
        "from rayna_gb300 import _abi as A, presets\n"
        "from rayna_gb300.scene import flatten, RenderOpts\n"
        "lib = A.load_library()\n"
        "scene, cam, _ = presets.random_spheres(seed=0)\n"
        "flat = flatten(scene)\n"
        "h = C.c_void_p()\n"
        "assert lib.rg_create(None, C.byref(h)) == 0\n"
        "a = lib.rg_set_scene(h, C.byref(flat.desc))\n"
        "msg = A.last_error(lib, h)\n"
        "b = lib.rg_set_scene(h, C.byref(flat.desc))\n"
        "assert lib.rg_set_camera(h, C.byref(cam.to_c())) == 0\n"
        "assert lib.rg_set_options(h, C.byref(RenderOpts(width=16, height=9, samples=2, ray_depth=4).to_c())) == 0\n"
        "img = np.zeros(16 * 9 * 3, np.float32)\n"
        "st = A.rg_render_stats()\n"
        "c = lib.rg_render(h, 7, img.ctypes.data_as(C.POINTER(C.c_float)), C.byref(st))\n"
        "lib.rg_destroy(h)\n"
        "print(a, b, c, 'RAYNA_GPU_FAIL_ALLOC' in msg, float(img.mean()) > 0)\n")
    env = dict(os.environ, RAYNA_GPU_FAIL_ALLOC="3")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().splitlines()[-1] == f"{A.RG_OOM} {A.RG_OK} {A.RG_OK} True True"


def test_sample_ranges_sum_to_the_whole_frame():
    scene, cam, opts = small(presets.random_spheres, 48, 27, 16, 10)
    frames = 3
    with Renderer.new_from(scene, cam, opts, 0, seed=5) as r:
        for _ in range(frames):
            r.render()
        whole, n = r.get_accumulation()
    parts = []
    for first, count, form in ((0, 5, "megakernel"), (5, 11, "wavefront")):
        with Renderer.new_from(scene, cam, opts, 0, seed=5, form=form) as r:
            r.set_sample_range(first, count)
            for _ in range(frames):
                out = r.render()
                assert out.stats.samples == opts.width * opts.height * count
            s, k = r.get_accumulation()
            assert k == n
            parts.append(s.astype(np.float64))
            # a sharded frame is no whole frame to differentiate
            with pytest.raises(RaynaError) as e:
                r.backward(seed=1, target=np.zeros((opts.width, opts.height, 3), np.float32), last_frame=True)
            assert e.value.status == A.RG_NOT_READY
            # set_options restores whole frames
            r.set_options(opts)
            assert r.render().stats.samples == opts.width * opts.height * opts.samples
    np.testing.assert_allclose(parts[0] + parts[1], whole, rtol=2e-5, atol=2e-6)


@pytest.mark.parametrize("form", ["megakernel", "wavefront"])
def test_sample_range_matches_the_oracle_path_by_path(form):
    scene, cam, opts = small(presets.random_spheres, 40, 24, 12, 10)
    flat = flatten(scene)
    seed = 0x5A3
    first, count = 4, 5
    with Renderer.new_from(scene, cam, opts, 0, form=form, exact=True) as r:
        r.set_sample_range(first, count)
        out = r.render(seed=seed)
        gm, _ = r.frame_moments()  # mean over the range's samples
        # the accumulation holds their sum / samples
        np.testing.assert_allclose(out.img, gm * count / opts.samples, rtol=1e-6, atol=1e-7)
        with pytest.raises(RaynaError):
            r.set_sample_range(10, 5)  # beyond the 12 samples
    st, om, _, _ = ob.render_window(flat, cam, opts, (0, 0, opts.width, opts.height), seed=seed,
                                    policy=ob.POLICY_GPU_F32, samples=(first, count))
    assert st == 0
    frac = np.all(np.abs(gm - om) <= 1e-4 * (1 + np.abs(om)), axis=2).mean()
    print(f"sample range [{first}, {first + count}) ({form}): {frac:.4f} of pixels match the f32 oracle path for path")
    assert frac >= 0.97


@pytest.mark.parametrize("exact", [True, False])
def test_march_stages_render_the_megakernel_image(exact):
    """The material-sorted wavefront marches each SDF in its own persistent
    stage, `march_budget` evaluations per lane between refills, and finishes
    `shade_lanes` ended marches of a warp together; every setting, and the
    megakernel's one-call march, give the same image bits."""
    scene, cam, opts = small(presets.sdf_volumes, 64, 36, 8, 12, n_spheres=20)
    with Renderer.new_from(scene, cam, opts, 0, form="megakernel", exact=exact) as r:
        ref = r.render(seed=23).img
    for budget, lanes in [(1, 16), (4, 16), (8, 16), (64, 16), (8, 1), (8, 32), (32, 24)]:
        with Renderer.new_from(scene, cam, opts, 0, form="wavefront", exact=exact) as r:
            r.set_tuning(sort_materials=True, march_budget=budget, shade_lanes=lanes)
            assert r.tuning()["march_budget"] == budget and r.tuning()["shade_lanes"] == lanes
            out = r.render(seed=23)
            assert out.stats.error_flags == 0
            np.testing.assert_array_equal(out.img, ref, err_msg=f"march budget {budget}, shade lanes {lanes}")
    with Renderer.new_from(scene, cam, opts, 0) as r:
        with pytest.raises(RaynaError):
            r.set_tuning(march_budget=5000)
