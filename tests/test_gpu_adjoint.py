"""The device adjoint (rg_backward) through the C ABI.

* Against the FP64 CPU adjoint with the same random streams (the same
  estimator): albedo gradients within 1% of the gradient norm, per material
  where the gradient is not tiny, and the density gradient within 2%.
* Against central finite differences of the device's own loss (h = 1e-3,
  common random numbers): the largest albedo gradients within 1%.
* The loss returned with a target equals sum (I - target)^2 of the frame.
"""
import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300 import Renderer, presets
from rayna_gb300.scene import RenderOpts, flatten

pytestmark = pytest.mark.gpu


def small_case():
    scene, cam, _ = presets.adjoint_scene(n_spheres=60, ground_truth=False)
    gt, _, _ = presets.adjoint_scene(n_spheres=60, ground_truth=True)
    opts = RenderOpts(width=64, height=48, samples=16, ray_depth=8)
    return scene, gt, cam, opts


def test_backward_matches_fp64_cpu_adjoint():
    scene, gt, cam, opts = small_case()
    with Renderer.new_from(gt, cam, opts, 0) as r:
        target = r.frame(seed=77)
    flat = flatten(scene)
    seed = 4242
    with Renderer.new_from(scene, cam, opts, 0) as r:
        g = r.backward(seed, target=target)
        img = r.frame(seed)
    ref = ob.backward(flat, cam, opts, seed, target=target, policy=ob.POLICY_REF_F64)
    assert abs(g["loss"] - float(np.sum((img.astype(np.float64) - target) ** 2))) <= 1e-4 * g["loss"]
    assert abs(g["loss"] - ref["loss"]) <= 2e-3 * ref["loss"]
    ga, ra = g["albedo"].astype(np.float64), ref["albedo"]
    norm = np.linalg.norm(ra)
    assert norm > 0
    assert np.linalg.norm(ga - ra) <= 0.01 * norm, np.linalg.norm(ga - ra) / norm
    big = np.abs(ra) > 0.05 * np.abs(ra).max()
    rel = np.abs(ga[big] - ra[big]) / np.abs(ra[big])
    assert np.quantile(rel, 0.95) <= 0.01, np.quantile(rel, 0.95)
    gd, rd = float(g["density"][0]), float(ref["density"][0])
    assert abs(gd - rd) <= 0.02 * abs(rd) + 1e-6, (gd, rd)
    print(f"albedo rel err {np.linalg.norm(ga - ra) / norm:.2e}, density {gd:.5g} vs {rd:.5g}")


def test_backward_general_kernel_variant_matches_fp64_cpu_adjoint():
    """Scenes of spheres with media replay in a kernel variant of their own;
    a scene with another primitive kind (here an axis box) takes the general
    variant, whose gradients must match the FP64 CPU adjoint as well."""
    from rayna_gb300.scene import AxisBoxMesh, LambertianMaterial, SimpleObject
    scene, gt, cam, opts = small_case()
    for s in (scene, gt):
        s.objects.insert(1, SimpleObject(AxisBoxMesh((-2.5, 0.0, -1.0), (-1.5, 1.2, 0.0)),
                                         LambertianMaterial((0.6, 0.4, 0.3))))
    with Renderer.new_from(gt, cam, opts, 0) as r:
        target = r.frame(seed=71)
    seed = 515
    with Renderer.new_from(scene, cam, opts, 0) as r:
        g = r.backward(seed, target=target)
    ref = ob.backward(flatten(scene), cam, opts, seed, target=target, policy=ob.POLICY_REF_F64)
    assert abs(g["loss"] - ref["loss"]) <= 2e-3 * ref["loss"]
    ga, ra = g["albedo"].astype(np.float64), ref["albedo"]
    norm = np.linalg.norm(ra)
    assert norm > 0
    assert np.linalg.norm(ga - ra) <= 0.01 * norm, np.linalg.norm(ga - ra) / norm
    gd, rd = float(g["density"][0]), float(ref["density"][0])
    assert abs(gd - rd) <= 0.02 * abs(rd) + 1e-6, (gd, rd)
    print(f"general variant: albedo rel err {np.linalg.norm(ga - ra) / norm:.2e}, density {gd:.5g} vs {rd:.5g}")


def test_backward_albedo_matches_finite_differences():
    scene, gt, cam, opts = small_case()
    with Renderer.new_from(gt, cam, opts, 0) as r:
        target = r.frame(seed=78)
    seed = 99
    with Renderer.new_from(scene, cam, opts, 0) as r:
        base = np.array([[m.albedo[c] for c in range(3)] for m in r._flat.materials], np.float32)
        g = r.backward(seed, target=target)["albedo"]
        order = np.argsort(-np.abs(g).ravel())[:6]
        h = 1e-3
        for flat_i in order:
            m, c = divmod(int(flat_i), 3)
            vals = []
            for sgn in (1, -1):
                p = base.copy()
                p[m, c] += sgn * h
                r.set_parameters(albedo=p)
                vals.append(float(np.sum((r.frame(seed).astype(np.float64) - target) ** 2)))
            r.set_parameters(albedo=base)
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - g[m, c]) <= 0.01 * abs(fd) + 1e-4, (m, c, fd, g[m, c])


def test_backward_with_adjoint_image_and_parameter_updates():
    scene, gt, cam, opts = small_case()
    with Renderer.new_from(scene, cam, opts, 0) as r:
        ones = np.ones((opts.width, opts.height, 3), np.float32)
        g1 = r.backward(5, adjoint=ones)
        assert g1["loss"] == 0.0
        # d(sum I)/d albedo is non-negative for Lambertian scenes
        assert np.all(g1["albedo"] >= -1e-6)
        dens = r.n_volumes
        r.set_parameters(density=np.full(dens, 0.9, np.float32))
        g2 = r.backward(5, adjoint=ones)
        assert g2["density"].shape == (dens,)
        assert np.isfinite(g2["density"]).all()


def test_backward_rejects_textures():
    """The adjoint differentiates solid albedos: a textured scene or an image
    sky is refused with RG_UNSUPPORTED_VARIANT."""
    from rayna_gb300._abi import RaynaError
    scene, cam, _ = presets.textures_demo()
    opts = RenderOpts(width=16, height=9, samples=2, ray_depth=4)
    with Renderer.new_from(scene, cam, opts, 0) as r:
        with pytest.raises(RaynaError) as e:
            r.backward(seed=1, adjoint=np.ones((16, 9, 3), np.float32))
        assert e.value.status == 2


def test_backward_frame_uses_the_last_render():
    """rg_backward_frame takes I from the last render(): its gradients equal
    rg_backward's with the adjoint image 2 (I - target) of that frame, and it
    refuses once the parameters changed."""
    from rayna_gb300._abi import RaynaError
    scene, gt, cam, opts = small_case()
    with Renderer.new_from(gt, cam, opts, 0) as r:
        target = r.frame(seed=77)
    with Renderer.new_from(scene, cam, opts, 0) as r:
        r.render(seed=5)
        image, _ = r.frame_moments()
        g1 = r.backward(seed=9, target=target, last_frame=True)
        g2 = r.backward(seed=9, adjoint=2.0 * (image.astype(np.float32) - target.astype(np.float32)))
        np.testing.assert_allclose(g1["albedo"], g2["albedo"], rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(g1["density"], g2["density"], rtol=1e-5, atol=1e-7)
        want = float(np.sum((image.astype(np.float64) - target.astype(np.float64)) ** 2))
        assert abs(g1["loss"] - want) <= 1e-4 * want
        r.set_parameters(albedo=np.full((r.n_materials, 3), 0.5, np.float32))
        with pytest.raises(RaynaError) as e:
            r.backward(seed=9, target=target, last_frame=True)
        assert e.value.status == 10  # RG_NOT_READY


def test_gradients_on_the_full_adjoint_workload():
    """The differentiable-rendering workload itself: 1000 spheres (3000 albedo
    parameters) and one medium (3 albedo + 1 density), 512x512, 16 spp,
    depth 8, L2 loss against a 1024-spp target of the ground-truth parameters.
    The eight largest albedo gradients against the device's own central
    differences (h = 1e-3, common random numbers: the frame key is fixed, so
    the paths are the same on both sides and I is a polynomial in the
    albedos), within 1%; the whole gradient and the density gradient against
    the FP64 CPU adjoint of the same frame, within 1% of the gradient norm and
    2% respectively."""
    scene, cam, opts = presets.adjoint_scene(n_spheres=1000, ground_truth=False)
    gt, _, _ = presets.adjoint_scene(n_spheres=1000, ground_truth=True)
    topts = RenderOpts(width=opts.width, height=opts.height, samples=1024, ray_depth=opts.ray_depth)
    with Renderer.new_from(gt, cam, topts, 0) as r:
        target = r.frame(seed=1)
    seed = 31337
    with Renderer.new_from(scene, cam, opts, 0) as r:
        assert r.n_materials == 1001 and r.n_volumes == 1  # 1000 spheres + the medium's material
        base = np.array([[m.albedo[c] for c in range(3)] for m in r._flat.materials], np.float32)
        g = r.backward(seed, target=target)
        ga = g["albedo"]
        order = np.argsort(-np.abs(ga).ravel())[:8]
        h = 1e-3
        for flat_i in order:
            m, c = divmod(int(flat_i), 3)
            vals = []
            for sgn in (1, -1):
                p = base.copy()
                p[m, c] += sgn * h
                r.set_parameters(albedo=p)
                vals.append(float(np.sum((r.frame(seed).astype(np.float64) - target) ** 2)))
            r.set_parameters(albedo=base)
            fd = (vals[0] - vals[1]) / (2 * h)
            print(f"albedo ({m}, {c}): adjoint {ga[m, c]:.6g}, central difference {fd:.6g}")
            assert abs(fd - ga[m, c]) <= 0.01 * abs(fd) + 1e-4, (m, c, fd, ga[m, c])
    ref = ob.backward(flatten(scene), cam, opts, seed, target=target, policy=ob.POLICY_REF_F64)
    ra = ref["albedo"]
    rel = np.linalg.norm(ga.astype(np.float64) - ra) / np.linalg.norm(ra)
    gd, rd = float(g["density"][0]), float(ref["density"][0])
    print(f"vs FP64 adjoint: albedo gradient error {rel:.2e} of its norm; density {gd:.6g} vs {rd:.6g}")
    assert rel <= 0.01, rel
    assert abs(gd - rd) <= 0.02 * abs(rd) + 1e-6, (gd, rd)
