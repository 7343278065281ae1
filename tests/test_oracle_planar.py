"""Oracle pins for ParallelogramMesh, InfinitePlaneMesh and CylinderMesh (CPU).

Known answers worked out from the reference's formulas
(mesh/planar/mod.rs:161-194, parallelogram.rs:49-57, infinite_plane.rs:87-92,
mesh/primitive/cylinder.rs:64-183), including its conventions: a plane's
normal is normalize(cross(u, v)) and its front face is the side the normal
faces away from the ray (denominator < 0); the cylinder misses rays parallel
to its axis, takes a cap's face and normal from the side of its body root,
and sets "front face" when the ray leaves along the normal.
Then the f32 oracle (the device's operation order) against the faithful f64
oracle on seeded ray suites.
"""
import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300.scene import (
    CylinderMesh, InfinitePlaneMesh, LambertianMaterial, ParallelogramMesh, Planar, Scene, SimpleObject, flatten,
)

from raysuite import planar_scene, rays_at

POLICIES = [ob.POLICY_REF_F64, ob.POLICY_GPU_F32]


def one(mesh):
    return flatten(Scene(objects=[SimpleObject(mesh, LambertianMaterial((0.5, 0.5, 0.5)))]))


def q(flat, o, d, policy):
    h, t64, n64 = ob.query(flat, np.array([o], np.float32), np.array([d], np.float32), policy=policy, pretest=True)
    return h[0], t64[0], n64[0]


@pytest.mark.parametrize("policy", POLICIES)
def test_parallelogram_known_answers(policy):
    # corner 0, u = X, v = Z: normal = cross(X, Z) = -Y
    flat = one(ParallelogramMesh(Planar.new((0, 0, 0), (1, 0, 0), (0, 0, 1))))
    h, t, _ = q(flat, (0.25, 1.0, 0.75), (0, -1, 0), policy)
    assert h["hit"] == 1 and abs(t - 1.0) < 1e-6
    np.testing.assert_allclose(h["normal"], (0, -1, 0), atol=1e-7)
    assert h["front_face"] == 0  # denominator dot(n, dir) = +1: back face
    np.testing.assert_allclose(h["ray_normal"], (0, 1, 0), atol=1e-7)
    h, t, _ = q(flat, (0.25, -1.0, 0.75), (0, 1, 0), policy)
    assert h["hit"] == 1 and h["front_face"] == 1 and abs(t - 1.0) < 1e-6
    np.testing.assert_allclose(h["ray_normal"], (0, -1, 0), atol=1e-7)
    for x, z in [(1.5, 0.5), (-0.01, 0.5), (0.5, 1.01)]:  # outside uv in [0, 1]^2
        assert q(flat, (x, 1.0, z), (0, -1, 0), policy)[0]["hit"] == 0
    assert q(flat, (0.5, 1.0, 0.5), (1, 0, 0), policy)[0]["hit"] == 0  # parallel


@pytest.mark.parametrize("policy", POLICIES)
def test_parallelogram_from_three_points(policy):
    # From<[P; 3]>: corner b, sides a - b and c - b
    flat = one(ParallelogramMesh(((0, 2, 0), (0, 0, 0), (2, 0, 0))))
    h, t, _ = q(flat, (1.5, 1.5, 5.0), (0, 0, -1), policy)
    assert h["hit"] == 1 and abs(t - 5.0) < 1e-6


@pytest.mark.parametrize("policy", POLICIES)
def test_infinite_plane_known_answer(policy):
    flat = one(InfinitePlaneMesh(Planar.new((0, -1, 0), (1, 0, 0), (0, 0, 1))))
    h, t, _ = q(flat, (300.0, 5.0, -700.0), (0, -1, 0), policy)
    assert h["hit"] == 1 and abs(t - 6.0) < 1e-6
    assert h["prim"] == 0
    assert q(flat, (0, 5, 0), (0, 1, 0), policy)[0]["hit"] == 0  # behind the origin


@pytest.mark.parametrize("policy", POLICIES)
def test_cylinder_known_answers(policy):
    flat = one(CylinderMesh((0, 0, 0), (0, 2, 0), 0.5))
    # body, from outside
    h, t, _ = q(flat, (2.0, 1.0, 0.0), (-1, 0, 0), policy)
    assert h["hit"] == 1 and abs(t - 1.5) < 1e-6 and h["side"] == 0
    np.testing.assert_allclose(h["normal"], (1, 0, 0), atol=1e-6)
    np.testing.assert_allclose(h["ray_normal"], (1, 0, 0), atol=1e-6)
    # from inside, the far wall
    h, t, _ = q(flat, (0.0, 1.0, 0.0), (1, 0, 0), policy)
    assert h["hit"] == 1 and abs(t - 0.5) < 1e-6 and h["side"] == 0
    np.testing.assert_allclose(h["ray_normal"], (-1, 0, 0), atol=1e-6)
    # top cap, entered from above and outside the infinite cylinder: face 2, normal +Y
    o = np.array([2.0, 3.0, 0.0])
    d = np.array([0.2, 2.0, 0.0]) - o
    h, t, _ = q(flat, o, d, policy)
    assert h["hit"] == 1 and h["side"] == 2
    assert abs(t - np.linalg.norm(d)) < 1e-5
    np.testing.assert_allclose(h["normal"], (0, 1, 0), atol=1e-6)
    # top cap by a ray running inside the infinite cylinder: the reference takes
    # the cap's face and normal from the side of its body root (cylinder.rs:
    # `dist_along_norm` is not recomputed for the cap), here beyond p1: face 1, -Y
    d = np.array([0.01, -1.0, 0.0])
    h, t, _ = q(flat, (0.1, 3.0, 0.0), d, policy)
    assert h["hit"] == 1 and h["side"] == 1
    assert abs(t - np.linalg.norm(d)) < 1e-5
    np.testing.assert_allclose(h["normal"], (0, -1, 0), atol=1e-6)
    # exactly parallel to the axis: the reference's quadratic has a = 0 and misses
    assert q(flat, (0.1, 3.0, 0.0), (0, -1, 0), policy)[0]["hit"] == 0


def test_f32_oracle_agrees_with_f64_on_planar_suite():
    rng = np.random.Generator(np.random.PCG64(21))
    flat = flatten(planar_scene())
    o, d = rays_at(rng, 4000, (-3, -3, -3), (3, 3, 3))
    h32, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest="brute")
    h64, t64, _ = ob.query(flat, o, d, policy=ob.POLICY_REF_F64, pretest=True)
    agree = np.mean(h32["hit"] == h64["hit"])
    assert agree >= 0.998, agree
    m = (h32["hit"] == 1) & (h64["hit"] == 1) & (h32["prim"] == h64["prim"])
    assert m.mean() >= 0.99 * (h64["hit"] == 1).mean()
    rel = np.abs(h32["t"][m] - t64[m]) / np.maximum(np.abs(t64[m]), 1e-30)
    print(f"planar suite: hit agreement {agree:.5f}, median rel err {np.median(rel):.2e}, "
          f"{np.mean(rel > 1e-5):.4f} beyond 1e-5")
    assert np.median(rel) < 1e-6
    assert np.mean(rel > 1e-4) < 0.002


def test_structured_oracle_equals_brute_force_on_planar_suite():
    """The reference's BVH (with its padded planar boxes) returns what the
    primitive tests alone return."""
    rng = np.random.Generator(np.random.PCG64(22))
    flat = flatten(planar_scene())
    o, d = rays_at(rng, 3000, (-3, -3, -3), (3, 3, 3))
    a, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest=True)
    b, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest="brute")
    assert np.array_equal(a["hit"], b["hit"])
    m = a["hit"] == 1
    assert np.array_equal(a["t"][m], b["t"][m])
