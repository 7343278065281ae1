"""The compressed 8-wide tree, built on the host (no GPU).

rg_inspect_scene runs the same build as rg_set_scene, including the
structural check of the 8-wide tree (children after parents, every node and
primitive reached once, every child's quantised grid box containing the
bounds of every primitive below it); a failed check is an error. These cases
cover the shapes that stress the builder and the quantisation: many
primitives, coincident centroids, flat and point-like extents, extreme
coordinate ranges and tiny scenes.
"""
import numpy as np
import pytest

from rayna_gb300 import RaynaError, presets
from rayna_gb300.renderer import inspect_scene
from rayna_gb300.scene import (
    AxisBoxMesh, BvhMesh, IsotropicMaterial, LambertianMaterial, MetalMaterial, RaymarchedIsosurfaceMesh, Scene,
    SdfTorus, SimpleObject, SphereMesh, Triangle, VolumetricObject,
)

MAX_WIDE_DEPTH = 60


def check(scene, n_prims):
    info = inspect_scene(scene)
    assert info["n_prims"] == n_prims
    assert info["max_leaf_size"] <= 3
    if n_prims:
        assert info["n_wide_nodes"] >= 1
        assert info["wide_depth"] <= MAX_WIDE_DEPTH
        # a wide node replaces about three binary node pairs
        assert info["n_wide_nodes"] <= info["n_nodes"]
        assert info["device_bytes"] >= info["n_prims"] * 48 + info["n_nodes"] * 64 + info["n_wide_nodes"] * 80
    else:
        assert info["n_wide_nodes"] == 0
    return info


def spheres(centres, radii, material=None):
    m = material or LambertianMaterial((0.5, 0.5, 0.5))
    return Scene(objects=[SimpleObject(SphereMesh(tuple(map(float, c)), float(r)), m) for c, r in zip(centres, radii)])


def test_preset_scenes():
    check(presets.random_spheres(seed=0)[0], 488)
    check(presets.cornell_mesh(level=5)[0], 20 * 4 ** 5 + 12)
    scene = presets.sdf_volumes(n_spheres=30)[0]
    info = inspect_scene(scene)
    assert info["n_wide_nodes"] >= 1 and info["n_unbounded"] == 2
    check(presets.adjoint_scene()[0], inspect_scene(presets.adjoint_scene()[0])["n_prims"])


def test_wide_tree_is_shallower():
    info = check(presets.cornell_mesh(level=6)[0], 20 * 4 ** 6 + 12)
    assert info["wide_depth"] * 2 <= info["max_depth"] + 2
    assert info["n_wide_nodes"] * 2 < info["n_nodes"]


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 24, 25, 100])
def test_tiny_scenes(n):
    rng = np.random.default_rng(n)
    check(spheres(rng.uniform(-5, 5, (n, 3)), rng.uniform(0.1, 1, n)), n)


def test_coincident_centroids():
    # 500 identical spheres: the split falls back to the median of equal keys
    check(spheres(np.zeros((500, 3)), np.ones(500)), 500)


def test_flat_and_point_extents():
    # all spheres on a plane, and triangles that are all in the plane z = 0
    rng = np.random.default_rng(1)
    c = rng.uniform(-10, 10, (300, 3))
    c[:, 1] = 2.0
    check(spheres(c, np.full(300, 1e-3)), 300)
    tris = []
    for k in range(200):
        x, y = rng.uniform(-1, 1, 2)
        v = [(x, y, 0.0), (x + 0.01, y, 0.0), (x, y + 0.01, 0.0)]
        tris.append(Triangle(v, [(0, 0, 1)] * 3))
    check(Scene(objects=[SimpleObject(BvhMesh(tris), LambertianMaterial())]), 200)


def test_extreme_ranges():
    # a 1000-radius ground sphere, tiny spheres far apart, and large offsets
    rng = np.random.default_rng(2)
    c = np.concatenate([[[0, -1000, 0]], rng.uniform(-1e4, 1e4, (50, 3)), 1e6 + rng.uniform(0, 1e-2, (50, 3))])
    r = np.concatenate([[1000.0], np.full(50, 1e-4), np.full(50, 1e-4)])
    check(spheres(c, r), 101)


def test_every_primitive_kind():
    objs = [
        SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial()),
        SimpleObject(AxisBoxMesh((2, 0, 0), (3, 1, 1)), MetalMaterial((0.5, 0.5, 0.5), 0.1)),
        VolumetricObject(SphereMesh((0, 3, 0), 1.0), IsotropicMaterial((0.5, 0.5, 0.5)), 0.5),
        VolumetricObject(AxisBoxMesh((-3, -1, -1), (-2, 1, 1)), IsotropicMaterial((0.5, 0.5, 0.5)), 0.2),
        SimpleObject(Triangle([(0, 0, 5), (1, 0, 5), (0, 1, 5)], [(0, 0, -1)] * 3), LambertianMaterial()),
        SimpleObject(RaymarchedIsosurfaceMesh(SdfTorus((0, 0, -4), 1.0, 0.3)), LambertianMaterial()),
    ]
    info = check(Scene(objects=objs), 5)
    assert info["n_unbounded"] == 1


def test_bad_scene_still_rejected():
    with pytest.raises(RaynaError):
        inspect_scene(spheres([(float("nan"), 0, 0)], [1.0]))
