"""Pins of the CPU oracle (runs on CPU).

The reference's own tests hold four known answers for the render path
(rayna_engine/tests/simple_renders.rs:22-142): a Lambertian unit sphere under
WhiteSkybox, 320x320, 10 spp, depth 5, seen from four camera positions. They
are checked here on the faithful f64 oracle, with seeded colours in the
reference's range (0.11 .. 0.89). Closed-form cases pin the rest: Philox
known-answer vectors, the viewport, and furnace identities.
"""
import math

import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300 import presets
from rayna_gb300.scene import Angle, Camera, RenderOpts, flatten

THRESH = 0.1
SIMPLE_OPTS = RenderOpts(width=320, height=320, samples=10, ray_depth=5)  # tests/common/mod.rs:13-20


def seeded_colours(n, seed=1234):
    rng = np.random.Generator(np.random.PCG64(seed))
    return 0.01 + THRESH + (0.98 - 2 * THRESH) * rng.random((n, 3))


def classify(img, target):
    """simple_renders.rs:55-82: [colour, white, black, other] fractions."""
    px = img.reshape(-1, 3)
    white = np.all(np.abs(1.0 - px) < THRESH, axis=1)
    black = ~white & np.all(np.abs(px) < THRESH, axis=1)
    colour = ~white & ~black & np.all(np.abs(np.asarray(target) - px) < THRESH, axis=1)
    other = ~white & ~black & ~colour
    n = px.shape[0]
    return colour.sum() / n, white.sum() / n, black.sum() / n, other.sum() / n


def simple_camera(z):
    return Camera(pos=(0.0, 0.0, z), v_fov=Angle.from_degrees(45.0), fwd=(0.0, 0.0, 1.0), focus_dist=1.0,
                  defocus_angle=Angle.from_degrees(0.0))


def check_known_answers(render_fn, colour):
    c, w, b, o = classify(render_fn(simple_camera(0.0)), colour)
    assert (c, w, b, o) == (0.0, 0.0, 1.0, 0.0), "inside the sphere: all black"
    c, w, b, o = classify(render_fn(simple_camera(-1.01)), colour)
    assert (c, w, b, o) == (1.0, 0.0, 0.0, 0.0), "next to the sphere: all colour"
    c, w, b, o = classify(render_fn(simple_camera(1.01)), colour)
    assert (c, w, b, o) == (0.0, 1.0, 0.0, 0.0), "looking at the sky: all white"
    c, w, b, o = classify(render_fn(simple_camera(-2.7)), colour)
    assert c >= 0.6 and 0.2 <= w <= 0.4 and o <= 0.05 and b == 0.0, (c, w, b, o)


@pytest.mark.parametrize("policy", [ob.POLICY_REF_F64, ob.POLICY_GPU_F32])
def test_simple_renders_known_answers(policy):
    for k, colour in enumerate(seeded_colours(3)):
        flat = flatten(presets.single_sphere(colour))

        def render(cam):
            st, mean, _, _ = ob.render(flat, cam, SIMPLE_OPTS, seed=100 + k, policy=policy)
            assert st == 0
            return mean

        check_known_answers(render, colour)


def test_philox_known_answers():
    # Random123 known-answer vectors of philox4x32-10
    assert ob.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert ob.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert ob.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_viewport_matches_camera_rs():
    cam = Camera(pos=(13.0, 2.0, 3.0), v_fov=Angle.from_degrees(20.0), fwd=(-13.0, -2.0, -3.0), focus_dist=10.0,
                 defocus_angle=Angle.from_degrees(0.6))
    st, vp = ob.viewport(cam)
    assert st == 0
    fwd = np.array([-13.0, -2.0, -3.0]) / np.linalg.norm([13.0, 2.0, 3.0])
    w = -fwd
    u = np.cross([0, 1, 0], w); u /= np.linalg.norm(u)
    v = np.cross(w, u)
    size = 2 * math.tan(math.radians(10.0)) * 10.0
    rad = 10.0 * math.tan(math.radians(0.3))
    np.testing.assert_allclose(vp[1], np.array([13.0, 2.0, 3.0]) - w * 10.0, rtol=1e-12)
    np.testing.assert_allclose(vp[2], u * size, rtol=1e-12)
    np.testing.assert_allclose(vp[3], -v * size, rtol=1e-12)
    np.testing.assert_allclose(vp[4], u * rad, rtol=1e-12)


@pytest.mark.parametrize("cam", [
    Camera(v_fov=Angle(0.0)),                                   # FovInvalid
    Camera(focus_dist=0.0),                                     # FocalLengthInvalid
    Camera(fwd=(0.0, 0.0, 0.0)),                                # ForwardVectorInvalid
    Camera(fwd=(0.0, 1.0, 0.0)),                                # cross(Y, w) cannot be normalised
])
def test_invalid_cameras(cam):
    st, _ = ob.viewport(cam)
    assert st == 3


def test_furnace_convex_objects():
    """A convex Lambertian or fuzz-0 metal sphere under WhiteSkybox reflects
    exactly its albedo: every scattered ray leaves the sphere for the sky."""
    from rayna_gb300.scene import MetalMaterial, Scene, SimpleObject, SphereMesh, WhiteSkybox
    cam = simple_camera(-1.01)
    opts = RenderOpts(width=16, height=16, samples=4, ray_depth=5)
    for mat, alb in [(None, (0.3, 0.6, 0.9)), ("metal", (0.7, 0.5, 0.2))]:
        if mat is None:
            scene = presets.single_sphere(alb)
        else:
            scene = Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), MetalMaterial(alb, 0.0))], skybox=WhiteSkybox())
        st, mean, var, _ = ob.render(flatten(scene), cam, opts, seed=3)
        assert st == 0
        np.testing.assert_allclose(mean, np.broadcast_to(np.array(alb), mean.shape), rtol=1e-6)


def test_oracle_policies_agree_statistically():
    """The f64 reference samplers and the f32 device samplers estimate the same
    image: per-pixel means agree within 4 combined standard errors."""
    scene, cam, _ = presets.random_spheres(seed=0)
    opts = RenderOpts(width=24, height=16, samples=16, ray_depth=10)
    flat = flatten(scene)
    st, m0, v0, _ = ob.render(flat, cam, opts, seed=1, frames=16, policy=ob.POLICY_REF_F64)
    st1, m1, v1, _ = ob.render(flat, cam, opts, seed=2, frames=16, policy=ob.POLICY_GPU_F32)
    assert st == 0 and st1 == 0
    n = 16 * 16
    se = np.sqrt(v0 / n + v1 / n) + 1e-6
    z = (m0 - m1) / se
    assert np.mean(np.abs(z) > 4) < 0.01
    assert abs(np.mean(m0) - np.mean(m1)) < 4 * np.sqrt(np.mean(v0 + v1) / (n * m0.size))
