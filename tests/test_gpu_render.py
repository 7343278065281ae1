"""Image parity and Renderer semantics on the GPU, through the C ABI.

* The reference's known answers (simple_renders.rs:22-142) on the device.
* Path-by-path parity: with the same frame seed, the device's
  arithmetic-contract build and the f32 oracle that mirrors its samplers
  trace the same paths; per-pixel means agree to float rounding except where
  a transcendental's last ulp flips a discrete decision (counted).
* Statistical parity of the performance build (the default) with the
  faithful f64 oracle (the reference's rejection samplers): per-pixel means
  within 3 standard errors, relRMSE reported.
* Accumulation, checkpoint/resume, invalid camera, unsupported variants.
"""
import math

import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300 import RaynaError, Renderer, presets
from rayna_gb300.scene import Angle, Camera, RenderMode, RenderOpts, flatten

from test_oracle_pins import SIMPLE_OPTS, check_known_answers, seeded_colours

pytestmark = pytest.mark.gpu


def test_simple_renders_known_answers_gpu():
    for k, colour in enumerate(seeded_colours(4, seed=99)):
        scene = presets.single_sphere(colour)
        with Renderer.new_from(scene, Camera(), SIMPLE_OPTS, 4, seed=k) as r:
            def render(cam):
                r.set_camera(cam)
                return r.render().img
            check_known_answers(render, colour)


def small(scene_fn, w, h, spp, depth, **kw):
    scene, cam, opts = scene_fn(**kw)
    return scene, cam, RenderOpts(width=w, height=h, samples=spp, ray_depth=depth)


CASES = {
    "random_spheres": lambda: small(presets.random_spheres, 80, 45, 32, 50),
    "cornell_mesh": lambda: small(presets.cornell_mesh, 48, 48, 16, 8, level=4),
    "sdf_volumes": lambda: small(presets.sdf_volumes, 64, 36, 16, 16, n_spheres=30),
    "cornell_quads": lambda: small(presets.cornell_quads, 48, 48, 16, 8),
    "cornell": lambda: small(presets.cornell, 48, 48, 16, 8),  # the preset's rotated boxes
    "textures": lambda: small(presets.textures_demo, 64, 36, 16, 8),  # every texture kind, image sky
    "rtiaw": lambda: small(presets.rtiaw_demo, 64, 36, 8, 12),  # the reference's RTIAW_DEMO preset
    "rttnw": lambda: small(presets.rttnw_demo, 48, 48, 16, 8),  # the reference's RTTNW_DEMO preset
}


@pytest.mark.parametrize("case", list(CASES))
def test_path_by_path_parity_with_f32_oracle(case):
    scene, cam, opts = CASES[case]()
    flat = flatten(scene)
    seed = 0x1234567 + len(case)
    with Renderer.new_from(scene, cam, opts, 0, exact=True) as r:
        r.render(seed=seed)
        gm, gv = r.frame_moments()
    st, om, ov, _ = ob.render(flat, cam, opts, seed=seed, frames=1, policy=ob.POLICY_GPU_F32)
    assert st == 0
    diff = np.abs(gm - om)
    close = np.all(diff <= 1e-4 * (1 + np.abs(om)), axis=2)
    frac = close.mean()
    print(f"{case}: {frac:.4f} of pixels match the f32 oracle path for path")
    assert frac >= {"random_spheres": 0.97, "cornell_mesh": 0.97, "sdf_volumes": 0.9, "cornell_quads": 0.97,
                    "cornell": 0.97, "textures": 0.97, "rtiaw": 0.97, "rttnw": 0.97}[case]


@pytest.mark.parametrize("case", list(CASES))
def test_statistical_parity_with_f64_oracle(case):
    scene, cam, opts = CASES[case]()
    flat = flatten(scene)
    frames = {"random_spheres": 24, "cornell_mesh": 48, "sdf_volumes": 32, "cornell_quads": 48, "cornell": 48,
              "textures": 32, "rtiaw": 32, "rttnw": 32}[case]
    spp = opts.samples
    sq = 0.0
    with Renderer.new_from(scene, cam, opts, 0, seed=7) as r:
        for _ in range(frames):
            out = r.render()
            fm, fv = r.frame_moments()
            sq = sq + (spp - 1) * fv.astype(np.float64) + spp * fm.astype(np.float64) ** 2
        img = out.img.astype(np.float64)
        assert out.stats.accum_frames == frames
        assert out.stats.error_flags == 0
    st, om, ov, _ = ob.render(flat, cam, opts, seed=11, frames=frames, policy=ob.POLICY_REF_F64)
    assert st == 0
    n = frames * spp
    gv = np.maximum(sq / n - img ** 2, 0.0) * n / (n - 1)   # device per-sample variance
    se = np.sqrt((gv + ov) / n)
    z = (img - om) / np.maximum(se, 1e-6)
    beyond = np.mean(np.abs(z) > 3)
    rel_rmse = np.sqrt(np.mean((img - om) ** 2)) / max(np.sqrt(np.mean(om ** 2)), 1e-12)
    print(f"{case}: {beyond:.4f} of pixel channels beyond 3 SE, relRMSE {rel_rmse:.4f}, mean z {np.mean(z):+.4f}")
    assert beyond <= 0.01
    # the image means agree within 4 standard errors of the mean over pixels
    gm_img, om_img = img.mean(), om.mean()
    se_img = math.sqrt(np.mean((gv + ov) / n) / img.size) * 3  # pixels are correlated: allow 3x
    assert abs(gm_img - om_img) <= 4 * se_img + 1e-6, (gm_img, om_img, se_img)


def test_accumulation_is_the_running_mean():
    scene, cam, _ = presets.random_spheres(seed=0)
    opts = RenderOpts(width=32, height=18, samples=4, ray_depth=8)
    with Renderer.new_from(scene, cam, opts, 0, seed=3) as r:
        means = []
        for _ in range(5):
            out = r.render()
            m, _ = r.frame_moments()
            means.append(m.astype(np.float64))
        np.testing.assert_allclose(out.img, np.mean(means, axis=0), rtol=2e-6, atol=1e-7)
        sums, frames = r.get_accumulation()
        assert frames == 5
        # checkpoint / resume
        r.clear_accumulation()
        r.set_accumulation(sums, frames)
        out2 = r.render(seed=12345)
        m6, _ = r.frame_moments()
        np.testing.assert_allclose(out2.img, (np.sum(means, axis=0) + m6) / 6, rtol=2e-6, atol=1e-7)
        # set_camera clears the accumulation (renderer.rs:158-161)
        r.set_camera(cam)
        out3 = r.render(seed=777)
        m7, _ = r.frame_moments()
        assert out3.stats.accum_frames == 1
        np.testing.assert_array_equal(out3.img, m7)


def test_same_seed_is_deterministic():
    scene, cam, _ = presets.sdf_volumes(n_spheres=10)
    opts = RenderOpts(width=32, height=18, samples=8, ray_depth=8)
    with Renderer.new_from(scene, cam, opts, 0) as r:
        a = r.render(seed=42).img
        r.clear_accumulation()
        b = r.render(seed=42).img
    np.testing.assert_array_equal(a, b)


def test_invalid_camera_returns_checker():
    scene = presets.single_sphere((0.5, 0.5, 0.5))
    opts = RenderOpts(width=64, height=32, samples=1)
    with Renderer.new_from(scene, Camera(v_fov=Angle(0.0)), opts, 0) as r:
        out = r.render()
    assert out.img.shape == (6, 5, 3)   # ilog2(64) x ilog2(32)
    for x in range(6):
        for y in range(5):
            exp = [0, 0, 0] if (x + y) % 2 == 0 else [1, 0, 1]
            np.testing.assert_array_equal(out.img[x, y], exp)


def test_oversized_branching_and_zero_sizes_are_rejected():
    scene = presets.single_sphere((0.5, 0.5, 0.5))
    with Renderer.new_from(scene, Camera(), RenderOpts(width=8, height=8), 0) as r:
        with pytest.raises(RaynaError) as e:  # 2^41 tree nodes per sample
            r.set_options(RenderOpts(width=8, height=8, ray_depth=40, ray_branching=2))
        assert e.value.status == 1
        with pytest.raises(ValueError):
            r.set_options(RenderOpts(width=0, height=8))


MODE_CASES = {
    "planar": lambda: small(presets.cornell_quads, 40, 40, 4, 8),
    "transformed": lambda: small(presets.cornell, 40, 40, 4, 8),
    "textures": lambda: small(presets.textures_demo, 48, 27, 4, 8),
    "spheres": lambda: small(presets.random_spheres, 48, 27, 4, 8),
    "sdf_volumes": lambda: small(presets.sdf_volumes, 48, 27, 4, 8, n_spheres=20),
}


@pytest.mark.parametrize("mode", [m for m in RenderMode if m != RenderMode.PBR])
@pytest.mark.parametrize("case", list(MODE_CASES))
def test_debug_modes_path_by_path(case, mode):
    """render_px_once's visualisations (renderer.rs:427-490) against the f32
    oracle with the same streams. Exact except where a transcendental's last
    ulp differs (sphere and cylinder uv, the Mandelbulb, cbrt of the distance)."""
    scene, cam, opts = MODE_CASES[case]()
    opts.mode = mode
    flat = flatten(scene)
    with Renderer.new_from(scene, cam, opts, 0, form="wavefront", exact=True) as r:  # routes to the megakernel
        r.render(seed=41)
        gm, _ = r.frame_moments()
    st, om, _, _ = ob.render(flat, cam, opts, seed=41, frames=1, policy=ob.POLICY_GPU_F32)
    assert st == 0
    close = np.all(np.abs(gm - om) <= 1e-5 * (1 + np.abs(om)), axis=2).mean()
    print(f"{case} {mode.name}: {close:.4f} of pixels match")
    assert close >= (0.95 if case == "sdf_volumes" else 0.99)


def test_branching_path_by_path_and_statistics():
    """ray_branching = 2 (renderer.rs:536-568): the device's tree walk equals the
    f32 oracle's walk path for path, and its mean agrees with the faithful f64
    recursion within 3 standard errors; branching 1 renders the usual image."""
    scene, cam, opts = small(presets.cornell_quads, 24, 24, 4, 4)
    flat = flatten(scene)
    opts.ray_branching = 2
    with Renderer.new_from(scene, cam, opts, 0, exact=True) as r:
        r.render(seed=5)
        gm, _ = r.frame_moments()
    st, om, _, _ = ob.render(flat, cam, opts, seed=5, frames=1, policy=ob.POLICY_GPU_F32)
    close = np.all(np.abs(gm - om) <= 1e-4 * (1 + np.abs(om)), axis=2).mean()
    print(f"branching 2: {close:.4f} of pixels match the f32 oracle")
    assert close >= 0.97
    frames, spp = 24, opts.samples
    sq = 0.0
    with Renderer.new_from(scene, cam, opts, 0, seed=3) as r:
        for _ in range(frames):
            out = r.render()
            fm, fv = r.frame_moments()
            sq = sq + (spp - 1) * fv.astype(np.float64) + spp * fm.astype(np.float64) ** 2
        img = out.img.astype(np.float64)
    st, om, ov, _ = ob.render(flat, cam, opts, seed=9, frames=frames, policy=ob.POLICY_REF_F64)
    n = frames * spp
    gv = np.maximum(sq / n - img ** 2, 0.0) * n / (n - 1)
    z = (img - om) / np.maximum(np.sqrt((gv + ov) / n), 1e-6)
    beyond = np.mean(np.abs(z) > 3)
    print(f"branching 2: {beyond:.4f} of pixel channels beyond 3 SE")
    assert beyond <= 0.01


def test_large_spp_path_and_counters():
    """spp > 256 takes the per-thread sample loop; counters are filled."""
    scene = presets.single_sphere((0.3, 0.6, 0.9))
    cam = Camera(pos=(0, 0, -2.7), v_fov=Angle.from_degrees(45), fwd=(0, 0, 1), focus_dist=1.0)
    opts = RenderOpts(width=8, height=8, samples=300, ray_depth=5)
    flat = flatten(scene)
    with Renderer.new_from(scene, cam, opts, 0, counters=True, exact=True) as r:
        out = r.render(seed=9)
        gm, _ = r.frame_moments()
        assert out.stats.samples == 8 * 8 * 300
        assert out.stats.rays >= out.stats.samples
        assert out.stats.node_visits > 0 and out.stats.prim_tests > 0
    st, om, _, _ = ob.render(flat, cam, opts, seed=9, frames=1, policy=ob.POLICY_GPU_F32)
    np.testing.assert_allclose(gm, om, rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("case", list(CASES) + ["large_spp"])
def test_wavefront_equals_megakernel(case, exact):
    """Both kernel forms run the same per-path code with the same random
    streams and sum samples in the same order: identical images, in either
    arithmetic build."""
    if case == "large_spp":
        scene = presets.single_sphere((0.3, 0.6, 0.9))
        cam = Camera(pos=(0, 0, -2.7), v_fov=Angle.from_degrees(45), fwd=(0, 0, 1), focus_dist=1.0)
        opts = RenderOpts(width=8, height=8, samples=300, ray_depth=5)
    else:
        scene, cam, opts = CASES[case]()
    imgs = {}
    for width in (2, 8):
        for form, sort in (("megakernel", None), ("wavefront", False), ("wavefront", True)):
            with Renderer.new_from(scene, cam, opts, 0, form=form, counters=True, exact=exact) as r:
                r.set_tuning(bvh_width=width, sort_materials=sort)
                assert r.tuning()["bvh_width"] == width
                for k in range(2):
                    out = r.render(seed=500 + k)
                assert out.stats.error_flags == 0
                imgs[(width, form, sort)] = (out.img.copy(), r.frame_moments(), out.stats)
    for width in (2, 8):
        a = imgs[(width, "megakernel", None)]
        for key in ((width, "wavefront", False), (width, "wavefront", True)):
            b = imgs[key]
            np.testing.assert_array_equal(a[0], b[0])
            np.testing.assert_array_equal(a[1][0], b[1][0])
            np.testing.assert_array_equal(a[1][1], b[1][1])
            assert a[2].rays == b[2].rays
            # Node and primitive counts depend slightly on which rays share a
            # warp (the binary traversal postpones leaves by warp occupancy,
            # which changes when the closest distance shrinks and so how many
            # far nodes are culled; the persistent extend kernel regroups rays
            # as lanes refill). They are work counters, not results.
            assert abs(a[2].node_visits - b[2].node_visits) <= 0.06 * a[2].node_visits
            assert abs(a[2].prim_tests - b[2].prim_tests) <= 0.06 * a[2].prim_tests
    # The two trees give the same closest hits except at exact-distance ties
    # between primitives (a shared edge hit exactly), where the traversal
    # order picks the primitive.
    a, b = imgs[(2, "megakernel", None)], imgs[(8, "megakernel", None)]
    same = np.all(a[1][0] == b[1][0], axis=2).mean()
    print(f"{case}: binary and 8-wide trees agree on {same:.5f} of pixels")
    assert same >= 0.999
    assert a[2].rays == b[2].rays or same < 1.0


def test_wavefront_small_waves():
    """A path budget smaller than the frame splits it into many waves."""
    import ctypes as C
    scene, cam, opts = CASES["random_spheres"]()
    with Renderer.new_from(scene, cam, opts, 0, form="megakernel") as r:
        ref = r.render(seed=77).img
    with Renderer.new_from(scene, cam, opts, 0, form="wavefront") as r:
        r.set_wave_paths(1000)
        img = r.render(seed=77).img
    np.testing.assert_array_equal(ref, img)


@pytest.mark.parametrize("form", ["megakernel", "wavefront"])
def test_stage_times_bracket_the_traversal(form):
    """RG_FLAG_STAGE_TIMES: the traversal kernels' time is positive and part
    of the frame's kernel time; the image is unchanged by the timing."""
    scene, cam, opts = CASES["cornell_mesh"]()
    with Renderer.new_from(scene, cam, opts, 0, form=form) as r:
        ref = r.render(seed=31).img
    with Renderer.new_from(scene, cam, opts, 0, form=form, stage_times=True) as r:
        out = r.render(seed=31)
    np.testing.assert_array_equal(ref, out.img)
    assert 0.0 < out.stats.traverse_ms <= out.stats.kernel_ms * 1.001 + 1e-3


@pytest.mark.parametrize("form", ["megakernel", "wavefront"])
@pytest.mark.parametrize("case", list(CASES))
def test_validate_mode_finds_no_broken_invariants(case, form):
    """RG_FLAG_VALIDATE checks every closest hit and path colour against the
    reference's debug invariants (shared/validate.rs: finite values, unit
    normals, the distance inside the interval, the point at that distance
    along the ray, uv in [0, 1]^2, colours finite and non-negative). The
    checks only read: the image equals an unchecked render's."""
    scene, cam, opts = CASES[case]()
    with Renderer.new_from(scene, cam, opts, 0, form=form, validate=True) as r:
        out = r.render(seed=3)
        st = out.stats
    assert st.rays > 0 and st.node_visits > 0  # validation runs the counting variants
    assert st.invalid_hits == 0, (st.invalid_hits, st.invalid_mask)
    with Renderer.new_from(scene, cam, opts, 0, form=form) as r:
        img = r.render(seed=3).img
    np.testing.assert_array_equal(out.img, img)
