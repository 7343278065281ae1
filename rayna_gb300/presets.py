"""Seeded synthetic workloads of the path-tracing hot path.

* ``random_spheres`` — "Ray Tracing in One Weekend" random spheres, the scene
  the reference's RTIAW_DEMO preset renders (scene/preset.rs:157-254), with
  the sizes and material draws of the random-spheres workload: ground sphere
  r=1000, 22x22 grid of r=0.2 spheres, three r=1 spheres. 400x225, 32 spp,
  depth 50.
* ``cornell_mesh`` — a displaced icosphere (8 subdivisions: 1,310,720
  triangles) inside a Cornell box of 12 triangles lit by a 0.25x0.25 quad of
  radiance 15, after the reference's CORNELL preset (preset.rs:608-683).
  1024x1024, 64 spp, depth 8.
* ``sdf_volumes`` — power-8 Mandelbulb (metal, fuzz 0.1) and torus
  (dielectric 1.5) sphere-traced SDFs, a sphere medium of density 0.2 and a
  box medium of random density/albedo, 100 random Lambertian spheres.
  1280x720, 128 spp, depth 16.

All draws come from numpy's PCG64 seeded with `seed`.

Triangle winding: the reference's Triangle::intersect reports the front face
when det < 0 and orients ray_normal by -sign(det) (triangle.rs:95-105), so a
face is seen from the front when e1 x e2 points away from the viewer. Meshes
here are wound that way: e1 x e2 opposite to the vertex normals.
"""
from __future__ import annotations

import math

import numpy as np

from .scene import (
    Angle, AxisBoxMesh, BvhMesh, Camera, DielectricMaterial, IsotropicMaterial, LambertianMaterial,
    LightMaterial, MetalMaterial, NoSkybox, RaymarchedIsosurfaceMesh, RenderOpts, Scene, SdfMandelbulb,
    SdfTorus, SimpleObject, SimpleSkybox, SphereMesh, Triangle, VolumetricObject,
)


def look_at_camera(pos, target, v_fov_deg, focus_dist=None, defocus_angle_rad=0.0) -> Camera:
    pos = np.asarray(pos, float)
    d = np.asarray(target, float) - pos
    fwd = d / np.linalg.norm(d)
    return Camera(pos=tuple(pos), v_fov=Angle.from_degrees(v_fov_deg), fwd=tuple(fwd),
                  focus_dist=float(np.linalg.norm(d) if focus_dist is None else focus_dist),
                  defocus_angle=Angle(defocus_angle_rad))


# ---------------------------------------------------------------------------
# Random spheres
# ---------------------------------------------------------------------------
def random_spheres(seed: int = 0, grid: int = 11, extra_spheres: int = 0):
    """Returns (scene, camera, opts) of the random-spheres workload.

    `extra_spheres` adds further r=0.2 Lambertian spheres on a wider grid.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    objs = [SimpleObject(SphereMesh((0.0, -1000.0, 0.0), 1000.0), LambertianMaterial((0.5, 0.5, 0.5)))]
    for a in range(-grid, grid):
        for b in range(-grid, grid):
            centre = (a + 0.9 * rng.random(), 0.2, b + 0.9 * rng.random())
            choose = rng.random()
            if choose < 0.8:
                alb = tuple(rng.random(3) * rng.random(3))
                mat = LambertianMaterial(alb)
            elif choose < 0.95:
                mat = MetalMaterial(tuple(0.5 + 0.5 * rng.random(3)), 0.5 * rng.random())
            else:
                mat = DielectricMaterial((1.0, 1.0, 1.0), 1.5, 0.0)
            objs.append(SimpleObject(SphereMesh(centre, 0.2), mat))
    side = int(math.ceil(math.sqrt(max(extra_spheres, 0))))
    for k in range(extra_spheres):
        i, j = divmod(k, side)
        centre = (-side / 2 + i + 0.9 * rng.random(), 0.2, -side / 2 - 12 + j + 0.9 * rng.random())
        objs.append(SimpleObject(SphereMesh(centre, 0.2), LambertianMaterial(tuple(rng.random(3)))))
    objs.append(SimpleObject(SphereMesh((0.0, 1.0, 0.0), 1.0), DielectricMaterial((1.0, 1.0, 1.0), 1.5, 0.0)))
    objs.append(SimpleObject(SphereMesh((-4.0, 1.0, 0.0), 1.0), LambertianMaterial((0.4, 0.2, 0.1))))
    objs.append(SimpleObject(SphereMesh((4.0, 1.0, 0.0), 1.0), MetalMaterial((0.7, 0.6, 0.5), 0.0)))
    scene = Scene(objects=objs, skybox=SimpleSkybox())
    # aperture 0.1 at focus distance 10: lens radius 0.05 = 10 * tan(angle / 2)
    cam = look_at_camera((13.0, 2.0, 3.0), (0.0, 0.0, 0.0), 20.0, focus_dist=10.0,
                         defocus_angle_rad=2.0 * math.atan(0.05 / 10.0))
    opts = RenderOpts(width=400, height=225, samples=32, ray_depth=50)
    return scene, cam, opts


# ---------------------------------------------------------------------------
# Displaced icosphere in a Cornell box
# ---------------------------------------------------------------------------
def icosphere(level: int):
    """Unit icosphere: (vertices (V,3) float64, faces (F,3) int64), outward CCW faces."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        edges = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)])
        key = np.sort(edges, axis=1)
        uniq, inv = np.unique(key[:, 0] * (v.shape[0] + 1) + key[:, 1], return_inverse=True)
        e0 = uniq // (v.shape[0] + 1)
        e1 = uniq % (v.shape[0] + 1)
        mid = v[e0] + v[e1]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = v.shape[0]
        v = np.concatenate([v, mid])
        nf = f.shape[0]
        ab, bc, ca = inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                            np.stack([ab, bc, ca], 1)])
    return v, f


def _hash3(ix, iy, iz, seed: int):
    """Lattice hash to [0,1): a 32-bit integer mix (PCG output permutation)."""
    h = (ix.astype(np.uint64) * np.uint64(73856093)) ^ (iy.astype(np.uint64) * np.uint64(19349663)) ^ \
        (iz.astype(np.uint64) * np.uint64(83492791)) ^ np.uint64(seed * 2654435761 & 0xFFFFFFFF)
    h = h & np.uint64(0xFFFFFFFF)
    h = (h * np.uint64(747796405) + np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
    w = (((h >> ((h >> np.uint64(28)) + np.uint64(4))) ^ h) * np.uint64(277803737)) & np.uint64(0xFFFFFFFF)
    w = (w >> np.uint64(22)) ^ w
    return (w & np.uint64(0xFFFFFF)).astype(np.float64) / float(1 << 24)


def value_noise(p: np.ndarray, seed: int, octaves: int = 3, freq: float = 4.0) -> np.ndarray:
    """Seeded fractal value noise in [-1, 1]: trilinear lattice noise with a
    smoothstep fade, octaves at doubling frequency and halving amplitude."""
    total = np.zeros(p.shape[0])
    amp, norm = 1.0, 0.0
    for o in range(octaves):
        q = p * freq * (2.0 ** o)
        i = np.floor(q)
        fr = q - i
        s = fr * fr * (3.0 - 2.0 * fr)
        i = i.astype(np.int64)
        acc = np.zeros(p.shape[0])
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    w = (s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) * (s[:, 2] if dz else 1 - s[:, 2])
                    acc += w * _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed + 7919 * o)
        total += amp * (2.0 * acc - 1.0)
        norm += amp
        amp *= 0.5
    return total / norm


def displaced_icosphere(level: int, centre, radius: float, seed: int = 0, amplitude: float = 0.05):
    """Triangles (F,3,3) and vertex normals (F,3,3) of a noise-displaced
    icosphere, wound with e1 x e2 opposite to the (outward) vertex normals."""
    v, f = icosphere(level)
    disp = v * (1.0 + amplitude * value_noise(v, seed))[:, None]
    pos = disp * radius + np.asarray(centre, float)
    tri = pos[f]
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])  # outward, area-weighted
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    fr = f[:, [0, 2, 1]]  # reversed winding
    return pos[fr].astype(np.float32), vn[fr].astype(np.float32)


def _quad(p, u, v, normal):
    """Two triangles of the parallelogram p, p+u, p+v, p+u+v with flat normal
    `normal`, wound so that (e1 x e2) . normal < 0."""
    p, u, v, n = (np.asarray(x, float) for x in (p, u, v, normal))
    a, b, c, d = p, p + u, p + u + v, p + v
    tris = [np.array([a, b, c]), np.array([a, c, d])]
    out = []
    for t in tris:
        if np.dot(np.cross(t[1] - t[0], t[2] - t[0]), n) > 0:
            t = t[[0, 2, 1]]
        out.append(Triangle(t, [n, n, n]))
    return out


def cornell_box_triangles():
    red, green, white = (0.65, 0.05, 0.05), (0.12, 0.45, 0.15), (0.65, 0.65, 0.65)
    walls = [
        ((0, 0, 0), (0, 1, 0), (0, 0, 1), (1, 0, 0), red),      # left, x = 0
        ((1, 0, 0), (0, 0, 1), (0, 1, 0), (-1, 0, 0), green),   # right, x = 1
        ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), white),    # back, z = 0
        ((0, 0, 0), (0, 0, 1), (1, 0, 0), (0, 1, 0), white),    # floor, y = 0
        ((0, 1, 0), (1, 0, 0), (0, 0, 1), (0, -1, 0), white),   # ceiling, y = 1
    ]
    objs = []
    for p, u, v, n, col in walls:
        mat = LambertianMaterial(col)
        for t in _quad(p, u, v, n):
            objs.append(SimpleObject(t, mat))
    light = LightMaterial((15.0, 15.0, 15.0))
    for t in _quad((0.375, 0.9999, 0.375), (0.25, 0, 0), (0, 0, 0.25), (0, -1, 0)):
        objs.append(SimpleObject(t, light))
    return objs


def cornell(width: int = 512, height: int = 512, spp: int = 64, ray_depth: int = 8):
    """The reference's CORNELL preset (scene/preset.rs:608-687): five
    ParallelogramMesh walls, a parallelogram light, and two boxes rotated
    about Y by 15 and -18 degrees about their centres. Returns (scene,
    camera, opts)."""
    from .scene import AxisBoxMesh, ParallelogramMesh, Planar, Transform3
    red, green, warm_grey = (0.65, 0.05, 0.05), (0.12, 0.45, 0.15), (0.85, 0.74, 0.55)
    X, Y, Z = (1, 0, 0), (0, 1, 0), (0, 0, 1)

    def quad(p, u, v, col):
        return SimpleObject(ParallelogramMesh(Planar.new(p, u, v)), LambertianMaterial(col))

    objs = [quad((0, 0, 0), Y, Z, red), quad((0, 0, 0), X, Y, warm_grey), quad((0, 0, 0), Z, X, warm_grey),
            quad((1, 0, 0), Z, Y, green), quad((0, 1, 0), X, Z, warm_grey),
            SimpleObject(ParallelogramMesh(Planar.new((0.4, 0.9999, 0.4), (0.2, 0, 0), (0, 0, 0.2))),
                         LightMaterial((15.0, 15.0, 15.0))),
            SimpleObject(AxisBoxMesh((0.231, 0.0, 0.117), (0.531, 0.595, 0.414)), LambertianMaterial(warm_grey),
                         Transform3.from_axis_angle(Y, Angle.from_degrees(15.0))),
            SimpleObject(AxisBoxMesh((0.477, 0.0, 0.531), (0.774, 0.297, 0.829)), LambertianMaterial(warm_grey),
                         Transform3.from_axis_angle(Y, Angle.from_degrees(-18.0)))]
    scene = Scene(objects=objs, skybox=NoSkybox())
    cam = Camera(pos=(0.5, 0.5, 2.3), v_fov=Angle.from_degrees(40.0), fwd=(0.0, 0.0, -1.0), focus_dist=1.0,
                 defocus_angle=Angle(0.0))
    return scene, cam, RenderOpts(width=width, height=height, samples=spp, ray_depth=ray_depth)


def cornell_quads(width: int = 512, height: int = 512, spp: int = 64, ray_depth: int = 8):
    """The reference's CORNELL preset (scene/preset.rs:608-687) with its two
    boxes left axis-aligned (`cornell` rotates them as the preset does) and a
    capped cylinder added."""
    from .scene import AxisBoxMesh, CylinderMesh, ParallelogramMesh, Planar
    red, green, warm_grey = (0.65, 0.05, 0.05), (0.12, 0.45, 0.15), (0.85, 0.74, 0.55)
    X, Y, Z = (1, 0, 0), (0, 1, 0), (0, 0, 1)

    def quad(p, u, v, col):
        return SimpleObject(ParallelogramMesh(Planar.new(p, u, v)), LambertianMaterial(col))

    objs = [quad((0, 0, 0), Y, Z, red), quad((0, 0, 0), X, Y, warm_grey), quad((0, 0, 0), Z, X, warm_grey),
            quad((1, 0, 0), Z, Y, green), quad((0, 1, 0), X, Z, warm_grey),
            SimpleObject(ParallelogramMesh(Planar.new((0.4, 0.9999, 0.4), (0.2, 0, 0), (0, 0, 0.2))),
                         LightMaterial((15.0, 15.0, 15.0))),
            SimpleObject(AxisBoxMesh((0.231, 0.0, 0.117), (0.531, 0.595, 0.414)), LambertianMaterial(warm_grey)),
            SimpleObject(AxisBoxMesh((0.477, 0.0, 0.531), (0.774, 0.297, 0.829)), LambertianMaterial(warm_grey)),
            SimpleObject(CylinderMesh((0.8, 0.297, 0.62), (0.8, 0.55, 0.68), 0.09), MetalMaterial((0.8, 0.7, 0.6), 0.05))]
    scene = Scene(objects=objs, skybox=NoSkybox())
    cam = Camera(pos=(0.5, 0.5, 2.3), v_fov=Angle.from_degrees(40.0), fwd=(0.0, 0.0, -1.0), focus_dist=1.0,
                 defocus_angle=Angle(0.0))
    return scene, cam, RenderOpts(width=width, height=height, samples=spp, ray_depth=ray_depth)


def cornell_mesh(level: int = 8, seed: int = 0, width: int = 1024, height: int = 1024, spp: int = 64,
                 centre=(0.5, 0.3, 0.5), radius: float = 0.25):
    """Returns (scene, camera, opts) of the triangle-mesh workload."""
    verts, norms = displaced_icosphere(level, centre, radius, seed)
    objs = cornell_box_triangles()
    objs.append(SimpleObject(BvhMesh.from_arrays(verts, norms), LambertianMaterial((0.7, 0.7, 0.7))))
    scene = Scene(objects=objs, skybox=NoSkybox())
    cam = Camera(pos=(0.5, 0.5, 2.3), v_fov=Angle.from_degrees(40.0), fwd=(0.0, 0.0, -1.0), focus_dist=1.0,
                 defocus_angle=Angle(0.0))
    opts = RenderOpts(width=width, height=height, samples=spp, ray_depth=8)
    return scene, cam, opts


# ---------------------------------------------------------------------------
# SDFs and media
# ---------------------------------------------------------------------------
def sdf_volumes(seed: int = 0, width: int = 1280, height: int = 720, spp: int = 128, n_spheres: int = 100):
    """Returns (scene, camera, opts) of the SDF + media workload.

    Placement (not fixed by the workload definition, fixed here): Mandelbulb
    at (0, 1.2, 0), torus at (2.8, 0.3, 0.8), sphere medium at (-2.6, 1, 0.6)
    radius 0.9, box medium [-1, 1.5] x [-0.5, 0.6] x [2, 3.2], Lambertian
    spheres of radius U[0.15, 0.45] scattered over [-6, 6] x [-1.5, 0] x [-6, 6].
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    objs = []
    for _ in range(n_spheres):
        r = 0.15 + 0.3 * rng.random()
        c = (-6 + 12 * rng.random(), -1.5 + 1.5 * rng.random(), -6 + 12 * rng.random())
        objs.append(SimpleObject(SphereMesh(c, r), LambertianMaterial(tuple(rng.random(3)))))
    box_density = 0.01 + 0.49 * rng.random()
    box_albedo = tuple(0.3 + 0.6 * rng.random(3))
    objs.append(VolumetricObject(SphereMesh((-2.6, 1.0, 0.6), 0.9), IsotropicMaterial((0.8, 0.8, 0.8), 0.0), 0.2))
    objs.append(VolumetricObject(AxisBoxMesh((-1.0, -0.5, 2.0), (1.5, 0.6, 3.2)), IsotropicMaterial(box_albedo, 0.0),
                                 box_density))
    objs.append(SimpleObject(RaymarchedIsosurfaceMesh(SdfMandelbulb((0.0, 1.2, 0.0), 8.0, 8, 1.0), 256, 1e-4),
                             MetalMaterial((0.8, 0.85, 0.88), 0.1)))
    objs.append(SimpleObject(RaymarchedIsosurfaceMesh(SdfTorus((2.8, 0.3, 0.8), 1.0, 0.3), 256, 1e-4),
                             DielectricMaterial((1.0, 1.0, 1.0), 1.5, 0.0)))
    scene = Scene(objects=objs, skybox=SimpleSkybox())
    cam = look_at_camera((0.0, 2.2, 8.5), (0.0, 0.9, 0.0), 35.0)
    opts = RenderOpts(width=width, height=height, samples=spp, ray_depth=16)
    return scene, cam, opts


def adjoint_scene(n_spheres: int = 1000, seed: int = 0, ground_truth: bool = True, width: int = 512,
                  height: int = 512, spp: int = 16, ray_depth: int = 8, medium_density: float | None = None):
    """Returns (scene, camera, opts) of the differentiable-rendering workload.

    The random-spheres layout with `n_spheres` Lambertian spheres, each with
    its own material (one RGB albedo parameter per sphere: ground, three r=1
    spheres, and r=0.2 spheres on a grid), plus one constant-density medium
    (a sphere of radius 1 at (0, 1, 0) with an isotropic material). With
    `ground_truth` the albedos are U[0.05, 0.95] and the medium has density
    0.8 and albedo (0.8, 0.6, 0.4); otherwise the albedos start at U[0.2, 0.8]
    and the medium at density 0.4, albedo 0.5. Parameters: 3 x n_spheres
    albedos + 3 medium albedos + 1 medium density.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    init = np.random.Generator(np.random.PCG64(seed + 7))

    def albedo():
        gt = tuple(0.05 + 0.9 * rng.random(3))
        return gt if ground_truth else tuple(0.2 + 0.6 * init.random(3))

    objs = [SimpleObject(SphereMesh((0.0, -1000.0, 0.0), 1000.0), LambertianMaterial(albedo()))]
    for c in [(-4.0, 1.0, 0.0), (4.0, 1.0, 0.0), (0.0, 1.0, -3.0)]:
        objs.append(SimpleObject(SphereMesh(c, 1.0), LambertianMaterial(albedo())))
    n_small = max(0, n_spheres - 4)
    side = int(math.ceil(math.sqrt(max(n_small, 1))))
    for k in range(n_small):
        a, b = divmod(k, side)
        centre = (a - side / 2 + 0.9 * rng.random(), 0.2, b - side / 2 + 0.9 * rng.random())
        objs.append(SimpleObject(SphereMesh(centre, 0.2), LambertianMaterial(albedo())))
    if medium_density is None:
        medium_density = 0.8 if ground_truth else 0.4
    mat = IsotropicMaterial((0.8, 0.6, 0.4) if ground_truth else (0.5, 0.5, 0.5), 0.0)
    objs.append(VolumetricObject(SphereMesh((0.0, 1.0, 0.0), 1.0), mat, medium_density))
    scene = Scene(objects=objs, skybox=SimpleSkybox())
    cam = look_at_camera((13.0, 2.0, 3.0), (0.0, 0.0, 0.0), 20.0, focus_dist=10.0)
    opts = RenderOpts(width=width, height=height, samples=spp, ray_depth=ray_depth)
    return scene, cam, opts


def decimated_icosphere(n_tris: int, centre, radius: float, seed: int = 0):
    """A displaced icosphere with about `n_tris` triangles: the nearest
    subdivision level at or above the count, then a seeded random subset."""
    level = 0
    while 20 * 4 ** level < n_tris:
        level += 1
    verts, norms = displaced_icosphere(level, centre, radius, seed)
    if verts.shape[0] > n_tris:
        keep = np.sort(np.random.Generator(np.random.PCG64(seed + 3)).choice(verts.shape[0], n_tris, replace=False))
        verts, norms = verts[keep], norms[keep]
    return verts, norms


RESOLUTIONS = [(256, 256), (640, 480), (1280, 720), (1920, 1080)]


def batch_scenes(n: int = 64, seed: int = 0, scale: float = 1.0, max_tris: int = 500_000):
    """The batched workload: `n` seeded scenes of uneven size. Sphere counts
    log-uniform in [10, 5000]; with probability 1/2 a displaced mesh of
    log-uniform [1k, max_tris] triangles; 0 to 2 media; resolution from
    {256^2, 640x480, 1280x720, 1920x1080}; 16 to 64 spp; depth 8. `scale`
    shrinks resolutions (for tests). Returns a list of (scene, camera, opts)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        n_sph = int(round(math.exp(rng.uniform(math.log(10), math.log(5000)))))
        extent = 2.0 + 0.08 * math.sqrt(n_sph)
        objs = [SimpleObject(SphereMesh((0.0, -1000.0, 0.0), 1000.0), LambertianMaterial((0.5, 0.5, 0.5)))]
        for _ in range(n_sph - 1):
            r = 0.1 + 0.25 * rng.random()
            c = (extent * (2 * rng.random() - 1), r, extent * (2 * rng.random() - 1))
            u = rng.random()
            if u < 0.75:
                mat = LambertianMaterial(tuple(rng.random(3)))
            elif u < 0.92:
                mat = MetalMaterial(tuple(0.5 + 0.5 * rng.random(3)), 0.3 * rng.random())
            else:
                mat = DielectricMaterial((1.0, 1.0, 1.0), 1.5, 0.0)
            objs.append(SimpleObject(SphereMesh(c, r), mat))
        if rng.random() < 0.5:
            n_tris = int(round(math.exp(rng.uniform(math.log(1000), math.log(max_tris)))))
            v, nn = decimated_icosphere(n_tris, (0.0, 1.2, 0.0), 1.0, seed=seed * 1000 + k)
            objs.append(SimpleObject(BvhMesh.from_arrays(v, nn), LambertianMaterial(tuple(0.3 + 0.6 * rng.random(3)))))
        for _ in range(int(rng.integers(0, 3))):
            c = (extent * (rng.random() - 0.5), 0.8, extent * (rng.random() - 0.5))
            objs.append(VolumetricObject(SphereMesh(c, 0.8), IsotropicMaterial(tuple(0.3 + 0.6 * rng.random(3)), 0.0),
                                         0.05 + 0.5 * rng.random()))
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        w, h = max(8, int(w * scale)), max(8, int(h * scale))
        spp = int(rng.integers(16, 65))
        cam = look_at_camera((extent * 1.6, 2.0 + 0.3 * extent, extent * 1.2), (0.0, 0.6, 0.0), 40.0)
        out.append((Scene(objects=objs, skybox=SimpleSkybox()), cam, RenderOpts(width=w, height=h, samples=spp, ray_depth=8)))
    return out


def single_sphere(albedo, skybox=None):
    """The scene of rayna_engine/tests/simple_renders.rs:36-48: a Lambertian
    unit sphere at the origin under WhiteSkybox."""
    from .scene import WhiteSkybox
    return Scene(objects=[SimpleObject(SphereMesh((0.0, 0.0, 0.0), 1.0), LambertianMaterial(tuple(albedo)))],
                 skybox=skybox if skybox is not None else WhiteSkybox())


def synthetic_sky(width: int = 128, height: int = 64, seed: int = 0):
    """An HDR environment image ([x][y][rgb]) standing in for an HDRI file: a
    horizon gradient, a bright sun disc and seeded low-frequency clouds."""
    from .scene import Image
    rng = np.random.Generator(np.random.PCG64(seed))
    x = (np.arange(width) + 0.5) / width
    y = (np.arange(height) + 0.5) / height
    u, v = np.meshgrid(x, y, indexing="ij")        # v = 0 at the image top (the zenith, sphere_uv v = 1)
    up = 1.0 - v
    sky = np.stack([0.5 + 0.4 * up, 0.6 + 0.3 * up, 0.9 + 0.1 * up], axis=-1)
    ground = np.stack([0.25 + 0 * up, 0.2 + 0 * up, 0.15 + 0 * up], axis=-1)
    img = np.where((up > 0.5)[..., None], sky, ground)
    cloud = np.zeros_like(u)
    for k in range(1, 5):
        ph = rng.uniform(0, 2 * math.pi, 2)
        cloud += np.sin(2 * math.pi * k * u + ph[0]) * np.sin(math.pi * k * up + ph[1]) / k
    img = img + 0.15 * np.clip(cloud, 0, None)[..., None] * (up > 0.5)[..., None]
    su, sv = 0.3, 0.25                              # the sun
    d2 = ((u - su) * 2) ** 2 + (v - sv) ** 2
    img = img + (20.0 * np.exp(-d2 / 0.0008))[..., None]
    return Image(img.astype(np.float32))


def textures_demo(width: int = 320, height: int = 180, spp: int = 32, ray_depth: int = 16, seed: int = 0):
    """Returns (scene, camera, opts) exercising every texture kind and the
    image sky: a world-checker ground, an image-textured sphere, a world-noise
    sphere (the reference's RTTNW noise sphere: Perlin(69) scaled by 4), a
    rotated box with local RGB noise, a metal sphere with a uv checker, a
    uv-noise parallelogram light, under an HdrImageSkybox."""
    from .scene import (
        ColourSource, HdrImageSkybox, Image, ImageTexture, LocalNoiseTexture, ParallelogramMesh, Perlin, Planar,
        ScalePoint, Transform3, UvCheckerTexture, UvNoiseTexture, WorldCheckerTexture, WorldNoiseTexture,
    )
    rng = np.random.Generator(np.random.PCG64(seed))
    # a 64 x 32 "planet" image: latitude bands and seeded blotches
    u, v = np.meshgrid((np.arange(64) + 0.5) / 64, (np.arange(32) + 0.5) / 32, indexing="ij")
    planet = np.stack([0.2 + 0.6 * v, 0.3 + 0.4 * np.abs(np.sin(6 * math.pi * v)), 0.8 - 0.5 * v], axis=-1)
    for _ in range(12):
        cu, cv, r = rng.uniform(0, 1), rng.uniform(0.1, 0.9), rng.uniform(0.03, 0.1)
        planet[((u - cu) ** 2 + (v - cv) ** 2) < r * r] = rng.uniform(0.2, 0.9, 3)
    planet_img = Image(planet.astype(np.float32))
    Y = (0.0, 1.0, 0.0)
    objs = [
        SimpleObject(ParallelogramMesh(Planar.new((-50, 0, -50), (100, 0, 0), (0, 0, 100))),
                     # offset half a cell in y: the ground plane then lies inside a cell, not on the cell
                     # boundary y = 0, where the parity would follow the sign of the hit point's rounding
                     LambertianMaterial(WorldCheckerTexture(even=(0.2, 0.3, 0.1), odd=(0.9, 0.9, 0.9), scale=1.0,
                                                            offset=(0.0, 0.5, 0.0)))),
        SimpleObject(SphereMesh((0.0, 1.0, 0.0), 1.0), LambertianMaterial(ImageTexture(planet_img))),
        SimpleObject(SphereMesh((-2.4, 1.0, 0.6), 1.0),
                     LambertianMaterial(WorldNoiseTexture(ColourSource.Greyscale(ScalePoint(Perlin(69)).set_scale(4.0))))),
        SimpleObject(AxisBoxMesh((1.8, 0.0, -0.6), (3.0, 1.2, 0.6)),
                     LambertianMaterial(LocalNoiseTexture(ColourSource.Rgb(
                         [ScalePoint(Perlin(5 + i)).set_scale(3.0) for i in range(3)]))),
                     Transform3.from_axis_angle(Y, Angle.from_degrees(30.0))),
        SimpleObject(SphereMesh((1.2, 0.5, 2.0), 0.5),
                     MetalMaterial(UvCheckerTexture(even=(0.9, 0.8, 0.3), odd=(0.5, 0.5, 0.6), scale=0.125), 0.05)),
        SimpleObject(ParallelogramMesh(Planar.new((-1.0, 3.5, -1.0), (2.0, 0, 0), (0, 0, 2.0))),
                     LightMaterial(UvNoiseTexture(ColourSource.Greyscale(ScalePoint(Perlin(11)).set_scale(6.0))))),
    ]
    scene = Scene(objects=objs, skybox=HdrImageSkybox(synthetic_sky(seed=seed)))
    cam = look_at_camera((0.0, 2.2, 8.0), (0.0, 0.8, 0.0), 40.0)
    return scene, cam, RenderOpts(width=width, height=height, samples=spp, ray_depth=ray_depth)


def rtiaw_demo(seed: int = 0, width: int = 400, height: int = 225, spp: int = 32, ray_depth: int = 50):
    """The reference's RTIAW_DEMO preset (scene/preset.rs:157-254), its random
    draws from PCG64(seed) instead of thread_rng: a 31 x 31 grid of r = 0.2
    spheres (70 %) and boxes (30 %; AxisBoxMesh::new_centred with a size in
    [0, 0.8]^3) with Lambertian (70 %), metal (20 %) or dielectric (ior in
    [1, 10], density 69) materials, three r = 1 spheres, and the ground sphere
    with LocalNoiseTexture(Perlin(69) scaled by 10000). Returns (scene,
    camera, opts)."""
    from .scene import ColourSource, LocalNoiseTexture, Perlin, ScalePoint
    rng = np.random.Generator(np.random.PCG64(seed))
    objs = []
    big = np.array([4.0, 0.2, 0.0])
    for a in range(-15, 16):
        for b in range(-15, 16):
            centre = np.array([a, 0.2, b], float) + np.array([rng.random(), 0.0, rng.random()]) * 0.9
            if np.linalg.norm(centre - big) <= 0.9:
                continue
            choice = rng.random()
            if choice < 0.7:
                mat = LambertianMaterial(tuple(rng.random(3) * rng.random(3)))
            elif choice <= 0.9:
                mat = MetalMaterial(tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(0.0, 0.5)))
            else:
                mat = DielectricMaterial(tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(1.0, 10.0)), 69.0)
            if rng.random() < 0.7:
                mesh = SphereMesh(tuple(centre), 0.2)
            else:
                mesh = AxisBoxMesh.new_centred(centre, rng.random(3) * 0.8)
            objs.append(SimpleObject(mesh, mat))
    objs.append(SimpleObject(SphereMesh((0.0, 1.0, 0.0), 1.0), DielectricMaterial((1.0, 1.0, 1.0), 1.5, 69.0)))
    objs.append(SimpleObject(SphereMesh((-4.0, 1.0, 0.0), 1.0), LambertianMaterial((0.4, 0.2, 0.1))))
    objs.append(SimpleObject(SphereMesh((4.0, 1.0, 0.0), 1.0), MetalMaterial((0.7, 0.6, 0.5), 0.0)))
    ground = LocalNoiseTexture(ColourSource.Greyscale(ScalePoint(Perlin(69)).set_scale(10000.0)))
    objs.append(SimpleObject(SphereMesh((0.0, -1000.0, 0.0), 1000.0), LambertianMaterial(ground)))
    fwd = np.array([-13.0, -2.0, -3.0])
    cam = Camera(pos=(13.0, 2.0, 3.0), fwd=tuple(fwd / np.linalg.norm(fwd)), v_fov=Angle.from_degrees(20.0),
                 focus_dist=10.0, defocus_angle=Angle.from_degrees(0.6))
    return Scene(objects=objs, skybox=SimpleSkybox()), cam, RenderOpts(width=width, height=height, samples=spp,
                                                                          ray_depth=ray_depth)


def rttnw_demo(seed: int = 0, width: int = 400, height: int = 400, spp: int = 64, ray_depth: int = 16):
    """The reference's RTTNW_DEMO preset (scene/preset.rs:394-604), its random
    draws from PCG64(seed) instead of thread_rng: a BvhMesh floor of 20 x 20
    boxes of random height, a parallelogram light, brown, glass, fuzzed-metal
    spheres, a dielectric sphere holding a blue medium, the WorldNoiseTexture
    sphere (Perlin(69) scaled by 4) and a BvhMesh "cube" of 1000 r = 0.1 balls
    rotated 15 degrees about Y and translated. No sky. Returns (scene, camera,
    opts)."""
    from .scene import (
        ColourSource, ParallelogramMesh, Perlin, Planar, ScalePoint, Transform3, WorldNoiseTexture,
    )
    rng = np.random.Generator(np.random.PCG64(seed))
    floor = []
    for i in range(20):
        for j in range(20):
            low = np.array([-10.0 + i, 0.0, -10.0 + j])
            high = low + np.array([1.0, rng.uniform(0.0, 1.0), 1.0])
            floor.append(AxisBoxMesh(tuple(low), tuple(high)))
    objs = [
        SimpleObject(BvhMesh(floor), LambertianMaterial((0.48, 0.83, 0.53))),
        SimpleObject(ParallelogramMesh(Planar.new((1.23, 5.54, 1.47), (3.0, 0.0, 0.0), (0.0, 0.0, 2.65))),
                     LightMaterial((7.0, 7.0, 7.0))),
        SimpleObject(SphereMesh((4.0, 4.0, 2.0), 0.5), LambertianMaterial((0.7, 0.3, 0.1))),
        SimpleObject(SphereMesh((2.6, 1.5, 0.45), 0.5), DielectricMaterial((1.0, 1.0, 1.0), 1.5, 1.0)),
        SimpleObject(SphereMesh((0.0, 1.5, 1.45), 0.5), MetalMaterial((0.8, 0.8, 0.9), 1.0)),
        SimpleObject(SphereMesh((3.6, 1.5, 1.45), 0.7), DielectricMaterial((1.0, 1.0, 1.0), 1.5, 0.0)),
        VolumetricObject(SphereMesh((3.6, 1.5, 1.45), 0.6999), IsotropicMaterial((0.2, 0.4, 0.9), 0.3), 2.0),
        SimpleObject(SphereMesh((2.2, 2.8, 3.0), 0.8),
                     LambertianMaterial(WorldNoiseTexture(ColourSource.Greyscale(ScalePoint(Perlin(69)).set_scale(4.0))))),
    ]
    spread = 0.825
    balls = [SphereMesh(tuple(rng.uniform(-1.0, 1.0, 3) * spread), 0.1) for _ in range(1000)]
    turn = Transform3.from_scale_rotation_translation((1.0, 1.0, 1.0), (0.0, 1.0, 0.0), Angle.from_degrees(15.0),
                                                      np.array([-1.0, 2.7, 3.95]) + spread)
    objs.append(SimpleObject(BvhMesh(balls), LambertianMaterial((0.85, 0.85, 0.85)), turn))
    fwd = np.array([-1.0, 0.0, 3.0])
    cam = Camera(pos=(4.78, 2.78, -6.0), fwd=tuple(fwd / np.linalg.norm(fwd)), v_fov=Angle.from_degrees(40.0),
                 focus_dist=1.0, defocus_angle=Angle(0.0))
    return Scene(objects=objs, skybox=NoSkybox()), cam, RenderOpts(width=width, height=height, samples=spp,
                                                                     ray_depth=ray_depth)


def rtiaw_demo_dark(seed: int = 0, width: int = 400, height: int = 225, spp: int = 32, ray_depth: int = 50):
    """The reference's RTIAW_DEMO_DARK preset (scene/preset.rs:257-392), its
    random draws from PCG64(seed) instead of thread_rng: the RTIAW grid with
    5 % emissive objects, a sparse second grid of bright lights at y = 3.2, the
    three r = 1 spheres, and an infinite ground plane with
    LocalNoiseTexture(Perlin(69) scaled by 10000), under no sky. Returns
    (scene, camera, opts)."""
    from .scene import ColourSource, InfinitePlaneMesh, LocalNoiseTexture, NoSkybox, Perlin, Planar, ScalePoint
    rng = np.random.Generator(np.random.PCG64(seed))
    objs = []
    big = np.array([4.0, 0.2, 0.0])
    for a in range(-15, 16):
        for b in range(-15, 16):
            centre = np.array([a, 0.2, b], float) + np.array([rng.random(), 0.0, rng.random()]) * 0.9
            if np.linalg.norm(centre - big) <= 1.0:
                continue
            choice = rng.random()
            if choice < 0.6:
                mat = LambertianMaterial(tuple(rng.random(3) * rng.random(3)))
            elif choice <= 0.8:
                mat = MetalMaterial(tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(0.0, 0.5)))
            elif choice <= 0.95:
                mat = DielectricMaterial(tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(1.0, 10.0)), 69.0)
            else:
                mat = LightMaterial(tuple(rng.uniform(0.0, 0.8, 3)))
            mesh = SphereMesh(tuple(centre), 0.2) if rng.random() < 0.7 else AxisBoxMesh.new_centred(
                centre, rng.random(3) * 0.8)
            objs.append(SimpleObject(mesh, mat))
    for a in range(-15, 16):
        for b in range(-15, 16):
            centre = np.array([a, 3.2, b], float) + np.array([rng.random(), 0.0, rng.random()]) * 0.9
            if np.linalg.norm(centre - big) <= 1.8:
                continue
            mat = LightMaterial(tuple(rng.uniform(10.0, 50.0, 3)))
            choice = rng.random()
            if choice <= 0.99:
                continue
            mesh = SphereMesh(tuple(centre), 0.2) if choice <= 0.995 else AxisBoxMesh.new_centred(
                centre, rng.random(3) * 0.8)
            objs.append(SimpleObject(mesh, mat))
    objs.append(SimpleObject(SphereMesh((0.0, 1.0, 0.0), 1.0), DielectricMaterial((1.0, 1.0, 1.0), 1.5, 69.0)))
    objs.append(SimpleObject(SphereMesh((-4.0, 1.0, 0.0), 1.0), LambertianMaterial((0.4, 0.2, 0.1))))
    objs.append(SimpleObject(SphereMesh((4.0, 1.0, 0.0), 1.0), MetalMaterial((0.7, 0.6, 0.5), 0.0)))
    ground = LocalNoiseTexture(ColourSource.Greyscale(ScalePoint(Perlin(69)).set_scale(10000.0)))
    objs.append(SimpleObject(InfinitePlaneMesh(Planar.new((0, 0, 0), (1, 0, 0), (0, 0, 1)), uv_wrap="wrap"),
                             LambertianMaterial(ground)))
    fwd = np.array([-13.0, -2.0, -3.0])
    cam = Camera(pos=(13.0, 2.0, 3.0), fwd=tuple(fwd / np.linalg.norm(fwd)), v_fov=Angle.from_degrees(20.0),
                 focus_dist=10.0, defocus_angle=Angle.from_degrees(0.6))
    return Scene(objects=objs, skybox=NoSkybox()), cam, RenderOpts(width=width, height=height, samples=spp,
                                                                     ray_depth=ray_depth)


def ALL(seed: int = 0) -> list:  # noqa: N802 (preset::ALL, scene/preset.rs:65)
    """The reference's presets that run on this library, as (name, scene,
    camera, opts): its RTIAW_DEMO, RTIAW_DEMO_DARK, RTTNW_DEMO and CORNELL
    (TESTING needs a polygonised isosurface)."""
    out = []
    for name, fn in (("RTIAW Demo", rtiaw_demo), ("RTIAW Demo (Night)", rtiaw_demo_dark), ("RTTNW Demo", rttnw_demo)):
        out.append((name, *fn(seed=seed)))
    out.append(("Cornell Box", *cornell()))
    return out
