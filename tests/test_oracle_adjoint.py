"""The CPU adjoint (oracle) against central finite differences (runs on CPU).

Scattered directions do not depend on albedos, so with common random numbers
the rendered image is a polynomial in the albedos and the path-replay
gradient must equal the central difference (h = 1e-3) to rounding. Emission
gradients likewise. The density gradient is a score-function estimator of the
derivative of the expectation; the finite difference of the same frames
estimates the same derivative, and both are compared on many samples.
"""
import numpy as np

from oracle import binding as ob
from rayna_gb300 import presets
from rayna_gb300.scene import (
    Camera, LambertianMaterial, LightMaterial, RenderOpts, Scene, SimpleObject, SphereMesh, flatten,
)


def loss_of(flat, cam, opts, seed, target, policy=ob.POLICY_REF_F64):
    st, m, _, _ = ob.render(flat, cam, opts, seed=seed, frames=1, policy=policy, gpu_sampling=True)
    assert st == 0
    return float(np.sum((m - target) ** 2))


def test_albedo_gradient_matches_central_differences():
    scene, cam, _ = presets.adjoint_scene(n_spheres=30, ground_truth=False)
    opts = RenderOpts(width=24, height=16, samples=8, ray_depth=6)
    flat = flatten(scene)
    gt_scene, _, _ = presets.adjoint_scene(n_spheres=30, ground_truth=True)
    st, target, _, _ = ob.render(flatten(gt_scene), cam, opts, seed=5, frames=1, policy=ob.POLICY_REF_F64,
                                 gpu_sampling=True)
    seed = 1234
    g = ob.backward(flat, cam, opts, seed, target=target.astype(np.float32))
    assert abs(g["loss"] - loss_of(flat, cam, opts, seed, target.astype(np.float32))) < 1e-9 * max(1.0, g["loss"])
    h = 1e-3
    checked = 0
    for m in [0, 1, 2, 3, 7, 12]:
        for c in range(3):
            base = flat.c_materials[m].albedo[c]
            ob.set_albedo(flat, m, c, base + h)
            lp = loss_of(flat, cam, opts, seed, target.astype(np.float32))
            ob.set_albedo(flat, m, c, base - h)
            lm = loss_of(flat, cam, opts, seed, target.astype(np.float32))
            ob.set_albedo(flat, m, c, base)
            fd = (lp - lm) / (2 * h)
            an = g["albedo"][m, c]
            assert abs(fd - an) <= 1e-3 * max(abs(fd), 1e-4), (m, c, fd, an)
            checked += abs(fd) > 1e-6
    assert checked >= 6


def test_emission_gradient_matches_central_differences():
    objs = [SimpleObject(SphereMesh((0.0, 0.0, 0.0), 1.0), LambertianMaterial((0.6, 0.5, 0.4))),
            SimpleObject(SphereMesh((0.0, 3.0, 0.0), 1.0), LightMaterial((4.0, 3.0, 2.0)))]
    scene = Scene(objects=objs, skybox=None)
    cam = presets.look_at_camera((0.0, 1.0, -6.0), (0.0, 1.0, 0.0), 45.0)
    opts = RenderOpts(width=16, height=16, samples=8, ray_depth=4)
    flat = flatten(scene)
    target = np.full((16, 16, 3), 0.3, np.float32)
    g = ob.backward(flat, cam, opts, 9, target=target)
    h = 1e-3
    for c in range(3):
        base = flat.c_materials[1].albedo[c]
        ob.set_albedo(flat, 1, c, base + h)
        lp = loss_of(flat, cam, opts, 9, target)
        ob.set_albedo(flat, 1, c, base - h)
        lm = loss_of(flat, cam, opts, 9, target)
        ob.set_albedo(flat, 1, c, base)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g["emission"][1, c]) <= 1e-3 * max(abs(fd), 1e-4), (c, fd, g["emission"][1, c])


def test_density_gradient_score_function_vs_finite_differences():
    """Expectation-level check: the score-function gradient and the central
    difference of the loss, both averaged over 24 frames."""
    scene, cam, _ = presets.adjoint_scene(n_spheres=12, ground_truth=False)
    cam = presets.look_at_camera((4.0, 1.5, 3.0), (0.0, 1.0, 0.0), 30.0)
    opts = RenderOpts(width=20, height=14, samples=16, ray_depth=6)
    flat = flatten(scene)
    # adjoint = 1 everywhere: d(sum I)/d density
    ones = np.ones((20, 14, 3), np.float32)
    h = 0.02
    an, fd = [], []
    for k in range(24):
        seed = 100 + k
        an.append(ob.backward(flat, cam, opts, seed, adjoint=ones)["density"][0])
        base = flat.c_volumes[0].density
        ob.set_density(flat, 0, base + h)
        st, mp, _, _ = ob.render(flat, cam, opts, seed=seed, frames=1, policy=ob.POLICY_REF_F64, gpu_sampling=True)
        ob.set_density(flat, 0, base - h)
        st, mm, _, _ = ob.render(flat, cam, opts, seed=seed, frames=1, policy=ob.POLICY_REF_F64, gpu_sampling=True)
        ob.set_density(flat, 0, base)
        fd.append((mp.sum() - mm.sum()) / (2 * h))
    an, fd = np.array(an), np.array(fd)
    se = np.sqrt(an.var() / len(an) + fd.var() / len(fd))
    assert abs(an.mean()) > 3 * np.sqrt(an.var() / len(an)), "gradient should be clearly non-zero"
    assert abs(an.mean() - fd.mean()) <= 4 * se, (an.mean(), fd.mean(), se)
