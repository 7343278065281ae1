"""Seeded ray-query suites and small scenes for the parity tests."""
import numpy as np

from rayna_gb300 import presets
from rayna_gb300.scene import (
    AxisBoxMesh, BvhMesh, DielectricMaterial, IsotropicMaterial, LambertianMaterial, MetalMaterial,
    RaymarchedIsosurfaceMesh, Scene, SdfMandelbulb, SdfSphere, SdfTorus, SimpleObject, SimpleSkybox, SphereMesh,
    VolumetricObject,
)


def rays_at(rng, n, lo, hi, targets=None, inside_frac=0.1, miss_frac=0.2):
    """Origins on a shell around the box [lo, hi] (some inside it), directions
    aimed at random targets (primitive points when given) or random."""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    c, ext = (lo + hi) / 2, np.linalg.norm(hi - lo) / 2 + 1e-3
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = c + d * ext * (1.2 + 1.5 * rng.random((n, 1)))
    k_in = int(n * inside_frac)
    o[:k_in] = lo + (hi - lo) * rng.random((k_in, 3))
    if targets is not None and len(targets):
        tgt = targets[rng.integers(0, len(targets), n)]
    else:
        tgt = lo + (hi - lo) * rng.random((n, 3))
    dirs = tgt - o
    k_miss = int(n * miss_frac)
    rnd = rng.normal(size=(k_miss, 3))
    dirs[-k_miss:] = rnd
    # a stratum of near-grazing directions: perturb aimed directions slightly
    k_g = n // 10
    dirs[k_in:k_in + k_g] += rng.normal(scale=0.02, size=(k_g, 3)) * np.linalg.norm(dirs[k_in:k_in + k_g], axis=1, keepdims=True)
    return o.astype(np.float32), dirs.astype(np.float32)


def sphere_scene(seed=0):
    scene, _, _ = presets.random_spheres(seed=seed)
    return scene


def triangle_scene(level=4, seed=0):
    verts, norms = presets.displaced_icosphere(level, (0.5, 0.3, 0.5), 0.25, seed)
    objs = presets.cornell_box_triangles()
    objs.append(SimpleObject(BvhMesh.from_arrays(verts, norms), LambertianMaterial((0.7, 0.7, 0.7))))
    return Scene(objects=objs), verts


def box_scene(seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    objs = []
    for _ in range(40):
        c = rng.uniform(-3, 3, 3)
        s = rng.uniform(0.1, 1.0, 3)
        objs.append(SimpleObject(AxisBoxMesh(tuple(c - s / 2), tuple(c + s / 2)), LambertianMaterial(tuple(rng.random(3)))))
    return Scene(objects=objs)


def volume_scene(transformed=False):
    """Two media (a sphere and a box) and two spheres; with `transformed` the
    box medium is turned 30 degrees about a tilted axis and the sphere medium
    moved, both as object transforms."""
    from rayna_gb300.scene import Angle, Transform3
    turn = Transform3.from_axis_angle(np.array([0.3, 1.0, 0.2]) / np.linalg.norm([0.3, 1.0, 0.2]),
                                      Angle.from_degrees(30.0)) if transformed else None
    move = Transform3.from_translation((0.1, 0.15, -0.1)) if transformed else None
    objs = [
        VolumetricObject(SphereMesh((0.0, 0.0, 0.0), 1.0), IsotropicMaterial((0.8, 0.8, 0.8), 0.0), 0.7, move),
        VolumetricObject(AxisBoxMesh((1.5, -0.5, -0.5), (2.5, 0.5, 0.5)), IsotropicMaterial((0.5, 0.6, 0.7), 0.0), 1.5,
                         turn),
        SimpleObject(SphereMesh((0.3, 0.0, 0.0), 0.3), LambertianMaterial((0.5, 0.5, 0.5))),
        SimpleObject(SphereMesh((-3.0, 0.0, 0.0), 0.5), LambertianMaterial((0.5, 0.5, 0.5))),
    ]
    return Scene(objects=objs)


def sdf_scene():
    objs = [
        SimpleObject(RaymarchedIsosurfaceMesh(SdfTorus((0.0, 0.0, 0.0), 1.0, 0.3), 256, 1e-4), DielectricMaterial((1, 1, 1), 1.5, 0)),
        SimpleObject(RaymarchedIsosurfaceMesh(SdfSphere((2.5, 0.0, 0.0), 0.5), 256, 1e-4), LambertianMaterial((0.5, 0.5, 0.5))),
        SimpleObject(RaymarchedIsosurfaceMesh(SdfMandelbulb((-2.5, 0.0, 0.0), 8.0, 8, 1.0), 256, 1e-4), MetalMaterial((0.8, 0.8, 0.8), 0.1)),
        SimpleObject(SphereMesh((0.0, 1.5, 0.0), 0.4), LambertianMaterial((0.5, 0.5, 0.5))),
    ]
    return Scene(objects=objs, skybox=SimpleSkybox())


def planar_scene(seed=0):
    """Parallelograms of random orientation and shape (some thin, some large),
    cylinders of random axis, two infinite planes, and a few spheres."""
    from rayna_gb300.scene import CylinderMesh, InfinitePlaneMesh, ParallelogramMesh, Planar
    rng = np.random.Generator(np.random.PCG64(seed))
    objs = []
    for _ in range(150):
        p = rng.uniform(-3, 3, 3)
        u = rng.normal(size=3) * rng.uniform(0.05, 1.5)
        v = rng.normal(size=3) * rng.uniform(0.05, 1.5)
        objs.append(SimpleObject(ParallelogramMesh(Planar.new(p, u, v)), LambertianMaterial(tuple(rng.random(3)))))
    for _ in range(60):
        p1 = rng.uniform(-3, 3, 3)
        p2 = p1 + rng.normal(size=3) * rng.uniform(0.1, 1.5)
        objs.append(SimpleObject(CylinderMesh(tuple(p1), tuple(p2), float(rng.uniform(0.05, 0.5))),
                                 MetalMaterial(tuple(rng.uniform(0.5, 1, 3)), 0.1)))
    objs.append(SimpleObject(InfinitePlaneMesh(Planar.new((0, -3.5, 0), (1, 0, 0), (0, 0, 1))), LambertianMaterial((0.5, 0.5, 0.5))))
    objs.append(SimpleObject(InfinitePlaneMesh(Planar.new((0, 0, -4), (0.3, 1, 0), (1, 0, 0.2))), LambertianMaterial((0.3, 0.6, 0.3))))
    for _ in range(10):
        objs.append(SimpleObject(SphereMesh(tuple(rng.uniform(-3, 3, 3)), float(rng.uniform(0.1, 0.6))),
                                 LambertianMaterial((0.5, 0.5, 0.5))))
    return Scene(objects=objs)


def transform_scene(seed=0, rigid=True):
    """Transformed boxes, spheres, parallelograms, cylinders and one triangle
    mesh (rotations about random axes and translations; with rigid=False also
    per-axis scales and shears), among a few untransformed primitives."""
    from rayna_gb300.scene import CylinderMesh, ParallelogramMesh, Planar, Transform3
    rng = np.random.Generator(np.random.PCG64(seed))

    def xf():
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        t = Transform3.from_axis_angle(ax, float(rng.uniform(-np.pi, np.pi)))
        if not rigid:
            m = np.eye(4)
            m[:3, :3] = np.diag(rng.uniform(0.4, 2.5, 3))
            m[0, 1] = rng.uniform(-0.5, 0.5)
            t = Transform3(m).then(t)
        return t.then_translate(rng.uniform(-0.5, 0.5, 3))

    objs = []
    for _ in range(30):
        c = rng.uniform(-3, 3, 3)
        s = rng.uniform(0.1, 1.0, 3)
        objs.append(SimpleObject(AxisBoxMesh(tuple(c - s / 2), tuple(c + s / 2)), LambertianMaterial(tuple(rng.random(3))), xf()))
    for _ in range(20):
        objs.append(SimpleObject(SphereMesh(tuple(rng.uniform(-3, 3, 3)), float(rng.uniform(0.1, 0.6))),
                                 MetalMaterial((0.8, 0.8, 0.8), 0.1), xf()))
    for _ in range(30):
        p = rng.uniform(-3, 3, 3)
        objs.append(SimpleObject(ParallelogramMesh(Planar.new(p, rng.normal(size=3) * 0.7, rng.normal(size=3) * 0.7)),
                                 LambertianMaterial(tuple(rng.random(3))), xf()))
    for _ in range(20):
        p1 = rng.uniform(-3, 3, 3)
        p2 = p1 + rng.normal(size=3) * rng.uniform(0.1, 1.5)
        objs.append(SimpleObject(CylinderMesh(tuple(p1), tuple(p2), float(rng.uniform(0.05, 0.5))),
                                 LambertianMaterial((0.5, 0.5, 0.5)), xf()))
    verts, norms = presets.displaced_icosphere(3, (1.0, 0.5, -1.0), 0.8, seed)
    objs.append(SimpleObject(BvhMesh.from_arrays(verts, norms), LambertianMaterial((0.7, 0.7, 0.7)), xf()))
    for _ in range(10):
        c = rng.uniform(-3, 3, 3)
        objs.append(SimpleObject(AxisBoxMesh(tuple(c - 0.3), tuple(c + 0.3)), LambertianMaterial((0.5, 0.5, 0.5))))
        objs.append(SimpleObject(SphereMesh(tuple(rng.uniform(-3, 3, 3)), 0.3), LambertianMaterial((0.5, 0.5, 0.5))))
    return Scene(objects=objs)
