"""Structure-independence of the f32 oracle's closest hits (runs on CPU).

The device traverses its own binary BVH and skips the reference's
per-object box pre-test; its bit-exactness is checked against brute force.
Here the oracle shows that, with the conservative f32 slab test, the
reference's tree with and without the pre-test gives the brute-force answer.
"""
import numpy as np

from oracle import binding as ob
from rayna_gb300.scene import flatten

from raysuite import rays_at, triangle_scene


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_query_pretest_is_immaterial():
    """The device skips the reference's per-object Aabb pre-test (object/bvh.rs:
    100-106). With the conservative f32 slab test, the f32 oracle's BVH with
    the pre-test, without it, and brute force agree bit for bit, on rays aimed
    at mesh vertices (the points that lie on box boundaries)."""
    rng = np.random.Generator(np.random.PCG64(11))
    scene, verts = triangle_scene(level=3)
    flat = flatten(scene)
    o, d = rays_at(rng, 20000, (0, 0, 0), (1, 1, 1), targets=verts.reshape(-1, 3))
    a, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest=True)
    b, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest=False)
    c, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest="brute")
    for x in (a, b):
        assert np.array_equal(x["hit"], c["hit"]) and np.array_equal(bits(x["t"]), bits(c["t"]))
