"""Scene, camera and render-option types mirroring rayna_engine's public API.

Names, fields and defaults follow the reference so that code written against
`rayna_engine` reads the same here:

* meshes        — SphereMesh (mesh/primitive/sphere.rs), Triangle
                  (mesh/primitive/triangle.rs), BvhMesh (mesh/advanced/bvh.rs),
                  AxisBoxMesh (mesh/primitive/axis_box.rs), CylinderMesh
                  (mesh/primitive/cylinder.rs), ParallelogramMesh and
                  InfinitePlaneMesh over a Planar (mesh/planar/*.rs),
                  RaymarchedIsosurfaceMesh (mesh/isosurface/raymarched.rs)
* objects       — SimpleObject (object/simple.rs), VolumetricObject
                  (object/volumetric.rs), ObjectList (object/list.rs)
* materials     — Lambertian/Metal/Dielectric/Isotropic/LightMaterial
                  (material/*.rs) with SolidTexture albedos (texture/solid.rs)
* sky           — SimpleSkybox, WhiteSkybox, NoSkybox (skybox/*.rs)
* Camera, Angle (scene/camera.rs), RenderOpts, RenderMode
  (render/render_opts.rs), Scene / StandardScene (scene/mod.rs)
* transforms    — Transform3 (glamour 0.11 `Transform3<f64, f64>`, the
                  core/types.rs alias) and ObjectTransform
                  (object/transform.rs)

`flatten()` turns a scene into the flat arrays of ``rg_scene_desc``. The
reference takes SDFs as closures; closures cannot cross a C ABI, so an SDF is
given as one of the descriptor types below. Variants this library does not
run (transformed volumes, SDFs and infinite planes, dynamic meshes) raise
UnsupportedVariant.
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field
from typing import Any, Iterable, Sequence

import numpy as np

from . import _abi as A


class UnsupportedVariant(ValueError):
    """A reference scene variant the GPU path does not run (RG_UNSUPPORTED_VARIANT)."""


def _vec3(v) -> tuple:
    t = tuple(float(x) for x in v)
    if len(t) != 3:
        raise ValueError(f"expected 3 components, got {v!r}")
    return t


# ---------------------------------------------------------------------------
# Transforms
# ---------------------------------------------------------------------------
class Transform3:
    """An affine map from mesh space to world space, held as a 4 x 4 f64
    matrix acting on column vectors (glamour's Transform3 over glam's DMat4).

    ``a.then(b)`` applies ``a`` first, then ``b`` (matrix ``b @ a``).
    """

    __slots__ = ("matrix",)

    def __init__(self, matrix=None):
        m = np.eye(4) if matrix is None else np.array(matrix, dtype=np.float64)
        if m.shape == (3, 4):
            m = np.vstack([m, [0.0, 0.0, 0.0, 1.0]])
        if m.shape != (4, 4):
            raise ValueError(f"expected a 4 x 4 or 3 x 4 matrix, got shape {m.shape}")
        if not np.array_equal(m[3], [0.0, 0.0, 0.0, 1.0]):
            raise ValueError("a Transform3 is affine: its bottom row must be (0, 0, 0, 1)")
        self.matrix = m

    @staticmethod
    def from_translation(v) -> "Transform3":
        m = np.eye(4)
        m[:3, 3] = _vec3(v)
        return Transform3(m)

    @staticmethod
    def from_scale(v) -> "Transform3":
        return Transform3(np.diag([*_vec3(v), 1.0]))

    @staticmethod
    def from_axis_angle(axis, angle: "Angle") -> "Transform3":
        """Rotation by `angle` (right-handed) about the unit vector `axis`
        (Rodrigues' rotation formula)."""
        x, y, z = _vec3(axis)
        a = angle.radians if isinstance(angle, Angle) else float(angle)
        c, s_ = math.cos(a), math.sin(a)
        k = 1.0 - c
        m = np.eye(4)
        m[:3, :3] = [[x * x * k + c, x * y * k - z * s_, x * z * k + y * s_],
                     [x * y * k + z * s_, y * y * k + c, y * z * k - x * s_],
                     [x * z * k - y * s_, y * z * k + x * s_, z * z * k + c]]
        return Transform3(m)

    @staticmethod
    def from_scale_rotation_translation(scale, axis, angle: "Angle", translation) -> "Transform3":
        """Scale, then rotate about `axis` by `angle`, then translate."""
        return Transform3.from_scale(scale).then(Transform3.from_axis_angle(axis, angle)).then_translate(translation)

    def then(self, other: "Transform3") -> "Transform3":
        return Transform3(other.matrix @ self.matrix)

    def then_translate(self, v) -> "Transform3":
        return self.then(Transform3.from_translation(v))

    def inverse(self) -> "Transform3":
        return Transform3(np.linalg.inv(self.matrix))

    def map_point(self, p) -> np.ndarray:
        return self.matrix[:3, :3] @ np.asarray(_vec3(p)) + self.matrix[:3, 3]

    def map_vector(self, v) -> np.ndarray:
        return self.matrix[:3, :3] @ np.asarray(_vec3(v))

    def is_identity(self) -> bool:
        return bool(np.array_equal(self.matrix, np.eye(4)))

    def __eq__(self, other):
        return isinstance(other, Transform3) and np.array_equal(self.matrix, other.matrix)

    def __repr__(self):
        return f"Transform3({self.matrix[:3].tolist()})"


Transform3.IDENTITY = Transform3()


class ObjectTransform:
    """object/transform.rs: a mesh-to-world Transform3 and its inverse.

    ``ObjectTransform.new(t)`` is uncorrected; ``new_corrected(t, centre)``
    rotates and scales about `centre` instead of the origin:
    translate(-centre), then `t`, then translate(centre)."""

    __slots__ = ("transform",)

    def __init__(self, transform: Transform3 = None):
        self.transform = Transform3.IDENTITY if transform is None else _transform3(transform)

    @staticmethod
    def new(transform) -> "ObjectTransform":
        return ObjectTransform(_transform3(transform))

    @staticmethod
    def new_corrected(transform, obj_centre) -> "ObjectTransform":
        c = np.asarray(_vec3(obj_centre))
        t = Transform3.from_translation(-c).then(_transform3(transform)).then_translate(c)
        return ObjectTransform(t)

    def with_correction(self, obj_centre) -> "ObjectTransform":
        return ObjectTransform.new_corrected(self.transform, obj_centre)

    @property
    def inv_transform(self) -> Transform3:
        return self.transform.inverse()

    @property
    def is_identity(self) -> bool:
        return self.transform.is_identity()


ObjectTransform.IDENTITY = ObjectTransform()


def _transform3(t) -> Transform3:
    if t is None:
        return Transform3.IDENTITY
    if isinstance(t, ObjectTransform):
        return t.transform
    if isinstance(t, Transform3):
        return t
    return Transform3(t)


# ---------------------------------------------------------------------------
# Camera and options
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Angle:
    """glamour::Angle<f64>: an angle stored in radians."""
    radians: float

    @staticmethod
    def from_degrees(deg: float) -> "Angle":
        return Angle(math.radians(deg))

    @staticmethod
    def from_radians(rad: float) -> "Angle":
        return Angle(float(rad))

    @property
    def degrees(self) -> float:
        return math.degrees(self.radians)


@dataclass
class Camera:
    """scene/camera.rs:10-25. Defaults follow Camera::default (:27-37)."""
    pos: tuple = (0.0, 0.0, 0.0)
    v_fov: Angle = Angle.from_degrees(45.0)
    fwd: tuple = (0.0, 0.0, 1.0)
    focus_dist: float = 1.0
    defocus_angle: Angle = Angle(0.0)

    def to_c(self) -> A.rg_camera:
        c = A.rg_camera()
        c.pos[:] = _vec3(self.pos)
        c.fwd[:] = _vec3(self.fwd)
        c.v_fov = self.v_fov.radians
        c.focus_dist = float(self.focus_dist)
        c.defocus_angle = self.defocus_angle.radians
        return c


class RenderMode(enum.IntEnum):
    """render/render_opts.rs:34-52."""
    PBR = 0
    RayNormal = 1
    OutwardNormal = 2
    Scatter = 3
    FrontFace = 4
    Distance = 5
    Uv = 6
    Side = 7


@dataclass
class RenderOpts:
    """render/render_opts.rs:8-29; defaults from :61-72."""
    width: int = 740
    height: int = 480
    samples: int = 1
    mode: RenderMode = RenderMode.PBR
    ray_depth: int = 5
    ray_branching: int = 1

    def dims(self) -> tuple:
        return (self.width, self.height)

    def aspect_ratio(self) -> float:
        return self.width / self.height

    def to_c(self) -> A.rg_render_opts:
        for name in ("width", "height", "samples", "ray_branching"):
            if int(getattr(self, name)) <= 0:
                raise ValueError(f"RenderOpts.{name} is a NonZeroUsize; got {getattr(self, name)}")
        o = A.rg_render_opts()
        o.width, o.height, o.samples = int(self.width), int(self.height), int(self.samples)
        o.mode, o.ray_depth, o.ray_branching = int(self.mode), int(self.ray_depth), int(self.ray_branching)
        return o


# ---------------------------------------------------------------------------
# Textures and materials
# ---------------------------------------------------------------------------
@dataclass
class SolidTexture:
    """texture/solid.rs: a constant colour."""
    albedo: tuple = (0.0, 0.0, 0.0)


class Image:
    """core/image.rs: an RGB f32 image indexed [x][y] (an ndarray of shape
    (width, height)); ``data`` has shape (width, height, 3)."""

    def __init__(self, data):
        a = np.ascontiguousarray(data, dtype=np.float32)
        if a.ndim != 3 or a.shape[2] != 3 or a.shape[0] == 0 or a.shape[1] == 0:
            raise ValueError(f"an Image is (width, height, 3), got shape {a.shape}")
        self.data = a

    @property
    def width(self) -> int:
        return self.data.shape[0]

    @property
    def height(self) -> int:
        return self.data.shape[1]

    @staticmethod
    def new_filled(width: int, height: int, fill) -> "Image":
        return Image(np.broadcast_to(np.asarray(_vec3(fill), np.float32), (width, height, 3)))

    @staticmethod
    def from_fn(width: int, height: int, func) -> "Image":
        return Image(np.array([[_vec3(func(x, y)) for y in range(height)] for x in range(width)], np.float32))

    def get_bilinear(self, px: float, py: float) -> np.ndarray:
        """Image::get_bilinear (core/image.rs:87-109), in f64."""
        def coords(val, n):
            fl = min(max(math.floor(val), 0), n - 1) if not math.isnan(val) else 0
            ce = min(max(math.ceil(val), 0), n - 1) if not math.isnan(val) else 0
            return int(fl), int(ce), val - fl
        x1, x2, xl = coords(px, self.width)
        y1, y2, yl = coords(py, self.height)
        d = self.data.astype(np.float64)
        lerp = lambda a, b, t: a + (b - a) * t
        return lerp(lerp(d[x1, y1], d[x2, y1], xl), lerp(d[x1, y2], d[x2, y2], xl), yl)


@dataclass(eq=False)
class WorldCheckerTexture:
    """texture/checker.rs:20-27: cells of `scale` in world space, shifted by `offset`."""
    even: Any
    odd: Any
    scale: float = 1.0
    offset: tuple = (0.0, 0.0, 0.0)


@dataclass(eq=False)
class UvCheckerTexture:
    """texture/checker.rs:37-44: cells of `scale` in uv, shifted by `offset`."""
    even: Any
    odd: Any
    scale: float = 1.0
    offset: tuple = (0.0, 0.0)


@dataclass(eq=False)
class ImageTexture:
    """texture/image.rs:29-39: the image at offset + uv * scale, v flipped, bilinear."""
    image: Image
    scale: tuple = (1.0, 1.0)
    offset: tuple = (0.0, 0.0)


@dataclass(eq=False)
class DynamicTexture:
    """texture/dynamic.rs: a shared texture; flattened to its inner texture."""
    inner: Any


@dataclass(frozen=True)
class Perlin:
    """noise::Perlin::new(seed): gradient noise. The GPU path evaluates Perlin's
    improved noise over its own seeded permutation, not the noise crate's."""
    seed: int = 0


class ScalePoint:
    """noise::ScalePoint: the source evaluated at the point times `scale`."""

    def __init__(self, source, scale=(1.0, 1.0, 1.0)):
        self.source = source
        self.scale = _vec3(scale)

    def set_scale(self, s: float) -> "ScalePoint":
        self.scale = (float(s),) * 3
        return self


class ColourSource:
    """texture/noise.rs ColourSource: Greyscale(noise) or Rgb([r, g, b])."""

    def __init__(self, kind: str, sources):
        self.kind, self.sources = kind, list(sources)

    @staticmethod
    def Greyscale(noise) -> "ColourSource":  # noqa: N802 (the reference's variant name)
        return ColourSource("greyscale", [noise])

    @staticmethod
    def Rgb(noises) -> "ColourSource":  # noqa: N802
        return ColourSource("rgb", noises)

    def to_dyn_box(self) -> "ColourSource":
        return self


@dataclass(eq=False)
class WorldNoiseTexture:
    source: ColourSource


@dataclass(eq=False)
class LocalNoiseTexture:
    source: ColourSource


@dataclass(eq=False)
class UvNoiseTexture:
    source: ColourSource


def _noise_params(src: ColourSource) -> tuple:
    """(seed, channels, scale) of a Perlin ColourSource: each source is
    Perlin(seed) or ScalePoint(Perlin(seed)) with one scale on all axes; the
    channels of an Rgb source must be seeded seed, seed + 1, seed + 2 and share
    the scale."""
    if not isinstance(src, ColourSource) or src.kind not in ("greyscale", "rgb"):
        raise UnsupportedVariant("noise textures take ColourSource.Greyscale or ColourSource.Rgb")
    parsed = []
    for n in src.sources:
        scale = 1.0
        if isinstance(n, ScalePoint):
            if len(set(n.scale)) != 1:
                raise UnsupportedVariant("ScalePoint needs one scale on every axis")
            scale, n = n.scale[0], n.source
        if not isinstance(n, Perlin):
            raise UnsupportedVariant(f"noise source {type(n).__name__} is not supported (Perlin only)")
        parsed.append((int(n.seed), scale))
    if src.kind == "rgb":
        if len(parsed) != 3 or any(p[0] != parsed[0][0] + i or p[1] != parsed[0][1] for i, p in enumerate(parsed)):
            raise UnsupportedVariant("Rgb noise must be three Perlin sources seeded s, s + 1, s + 2 with one scale")
    return parsed[0][0], len(parsed), parsed[0][1]


def _is_solid(tex) -> bool:
    while isinstance(tex, DynamicTexture):
        tex = tex.inner
    return isinstance(tex, (SolidTexture, tuple, list, np.ndarray))


def _colour(tex) -> tuple:
    while isinstance(tex, DynamicTexture):
        tex = tex.inner
    if isinstance(tex, SolidTexture):
        return _vec3(tex.albedo)
    if isinstance(tex, (tuple, list, np.ndarray)):
        return _vec3(tex)
    raise UnsupportedVariant(f"texture {type(tex).__name__} cannot cross the C ABI")


@dataclass(eq=False)
class LambertianMaterial:
    albedo: Any = (0.5, 0.5, 0.5)


@dataclass(eq=False)
class MetalMaterial:
    albedo: Any
    fuzz: float


@dataclass(eq=False)
class DielectricMaterial:
    albedo: Any
    refractive_index: float
    density: float


@dataclass(eq=False)
class IsotropicMaterial:
    albedo: Any = (0.5, 0.5, 0.5)
    density: float = 1.0


@dataclass(eq=False)
class LightMaterial:
    emissive: Any


def material_record(m, texture_index=None) -> A.rg_material:
    """The rg_material of `m`. A non-solid texture is registered through
    `texture_index(tex) -> int` (its position in the scene's texture table)."""
    r = A.rg_material()

    def colour(tex):
        if _is_solid(tex):
            r.albedo[:] = _colour(tex)
        elif texture_index is None:
            raise UnsupportedVariant(f"texture {type(tex).__name__} needs a scene texture table")
        else:
            r.texture = texture_index(tex) + 1

    if isinstance(m, LambertianMaterial):
        r.kind = A.RG_MAT_LAMBERTIAN
        colour(m.albedo)
    elif isinstance(m, MetalMaterial):
        r.kind = A.RG_MAT_METAL
        colour(m.albedo)
        r.fuzz = float(m.fuzz)
    elif isinstance(m, DielectricMaterial):
        r.kind = A.RG_MAT_DIELECTRIC
        colour(m.albedo)
        r.refractive_index = float(m.refractive_index)
        r.density = float(m.density)
    elif isinstance(m, IsotropicMaterial):
        r.kind = A.RG_MAT_ISOTROPIC
        colour(m.albedo)
        r.density = float(m.density)
    elif isinstance(m, LightMaterial):
        r.kind = A.RG_MAT_LIGHT
        colour(m.emissive)
    else:
        raise UnsupportedVariant(f"material {type(m).__name__} cannot cross the C ABI")
    return r


# ---------------------------------------------------------------------------
# Skyboxes
# ---------------------------------------------------------------------------
class SimpleSkybox:
    kind = A.RG_SKY_SIMPLE


class WhiteSkybox:
    kind = A.RG_SKY_WHITE


class NoSkybox:
    kind = A.RG_SKY_NONE


class HdrImageSkybox:
    """skybox/hdri.rs:17-26: the image sampled at sphere_uv(dir), v flipped."""
    kind = A.RG_SKY_IMAGE

    def __init__(self, image: Image):
        self.image = image if isinstance(image, Image) else Image(image)


# ---------------------------------------------------------------------------
# Meshes
# ---------------------------------------------------------------------------
@dataclass
class SphereMesh:
    pos: tuple
    radius: float

    def centre(self) -> np.ndarray:  # sphere.rs:106
        return np.asarray(_vec3(self.pos))


@dataclass
class Triangle:
    """mesh/primitive/triangle.rs:22-36; the constructor's asserts are kept."""
    vertices: Sequence
    normals: Sequence

    def __post_init__(self):
        v = np.asarray(self.vertices, dtype=np.float64).reshape(3, 3)
        n = np.asarray(self.normals, dtype=np.float64).reshape(3, 3)
        if (v[0] == v[1]).all() or (v[1] == v[2]).all() or (v[2] == v[0]).all():
            raise ValueError("triangles cannot have duplicate vertices")
        if not np.all(np.abs(np.linalg.norm(n, axis=1) - 1.0) < 2e-4):
            raise ValueError("normals must be normalised")
        self.vertices, self.normals = v, n

    def centre(self) -> np.ndarray:  # triangle.rs:42-45
        return (self.vertices[0] + self.vertices[1] + self.vertices[2]) / 3.0


class BvhMesh:
    """mesh/advanced/bvh.rs: a BVH over bounded meshes (triangles, spheres,
    boxes, parallelograms, cylinders, nested BvhMeshes) sharing one material
    and one transform.

    ``BvhMesh(list_of_meshes)`` mirrors the reference constructor;
    ``BvhMesh.from_arrays(vertices, normals)`` takes (n, 3, 3) triangle arrays.
    """

    def __init__(self, meshes: Iterable = ()):
        items = list(meshes)
        for t in items:
            if not isinstance(t, (Triangle, SphereMesh, AxisBoxMesh, ParallelogramMesh, CylinderMesh, BvhMesh)):
                raise UnsupportedVariant(f"BvhMesh over {type(t).__name__} cannot cross the C ABI "
                                         "(a BvhMesh holds bounded meshes)")
        tris = [t for t in items if isinstance(t, Triangle)]
        self.items = [m for m in items if not isinstance(m, Triangle)]
        if tris:
            self.vertices = np.stack([t.vertices for t in tris]).astype(np.float32)
            self.normals = np.stack([t.normals for t in tris]).astype(np.float32)
        else:
            self.vertices = np.zeros((0, 3, 3), np.float32)
            self.normals = np.zeros((0, 3, 3), np.float32)
        # bvh.rs:36-44: the mean of the sub-meshes' centres, in f64
        acc = np.zeros(3)
        for m in items:
            acc = acc + m.centre()
        self._centre = acc / len(items) if items else np.full(3, np.nan)

    @staticmethod
    def from_arrays(vertices, normals) -> "BvhMesh":
        m = BvhMesh()
        m.items = []
        m.vertices = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3, 3)
        m.normals = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3, 3)
        if m.vertices.shape != m.normals.shape:
            raise ValueError("vertices and normals must have the same shape")
        if len(m.vertices):
            m._centre = m.vertices.astype(np.float64).sum(axis=1).mean(axis=0) / 3.0
        return m

    def centre(self) -> np.ndarray:
        return self._centre

    def __len__(self):
        return self.vertices.shape[0] + len(self.items)


@dataclass
class AxisBoxMesh:
    a: tuple
    b: tuple

    @staticmethod
    def new_centred(centre, size) -> "AxisBoxMesh":
        c, s = np.asarray(centre, float), np.asarray(size, float)
        return AxisBoxMesh(tuple(c + s / 2), tuple(c - s / 2))

    def centre(self) -> np.ndarray:  # axis_box.rs:26-33: (min + max) / 2
        a, b = np.asarray(_vec3(self.a)), np.asarray(_vec3(self.b))
        return (np.minimum(a, b) + np.maximum(a, b)) / 2.0


@dataclass
class Planar:
    """mesh/planar/mod.rs:33-121: a corner `p` and two sides `u`, `v`."""
    p: tuple
    u: tuple
    v: tuple

    @staticmethod
    def new(p, u, v) -> "Planar":
        return Planar(_vec3(p), _vec3(u), _vec3(v))

    @staticmethod
    def new_centred(centre, u, v) -> "Planar":
        """Planar::new_centred (mod.rs:82-86): sides 2u and 2v around `centre`."""
        c, u, v = np.asarray(_vec3(centre)), np.asarray(_vec3(u)), np.asarray(_vec3(v))
        return Planar.new(c - u - v, u * 2.0, v * 2.0)

    @staticmethod
    def new_points(a, b, c) -> "Planar":
        """Planar::new_points (mod.rs:116-119): corner b, sides a - b and c - b."""
        a, b, c = np.asarray(_vec3(a)), np.asarray(_vec3(b)), np.asarray(_vec3(c))
        return Planar.new(b, a - b, c - b)

    def flat(self) -> tuple:
        return (*self.p, *self.u, *self.v)


def _planar(x) -> Planar:
    if isinstance(x, Planar):
        return x
    if isinstance(x, (tuple, list)) and len(x) == 3:  # From<[P; 3]>: three points (mod.rs:124-131)
        return Planar.new_points(*x)
    raise TypeError(f"cannot make a Planar from {type(x).__name__}")


@dataclass
class ParallelogramMesh:
    """mesh/planar/parallelogram.rs: the points p + a u + b v with a, b in [0, 1]."""
    plane: Any

    def __post_init__(self):
        self.plane = _planar(self.plane)

    def centre(self) -> np.ndarray:  # parallelogram.rs:64: the corner p
        return np.asarray(self.plane.p, np.float64)


@dataclass
class InfinitePlaneMesh:
    """mesh/planar/infinite_plane.rs: the whole plane (unbounded). uv_wrap
    ("wrap", "mirror" or "clamp_zero", UvWrappingMode) maps its texture
    coordinates; solid textures do not read them, the Uv render mode does."""
    plane: Any
    uv_wrap: str = "wrap"

    def __post_init__(self):
        self.plane = _planar(self.plane)

    def centre(self) -> np.ndarray:  # infinite_plane.rs:100: the corner p
        return np.asarray(self.plane.p, np.float64)


@dataclass
class CylinderMesh:
    """mesh/primitive/cylinder.rs: capped cylinder from p1 to p2."""
    p1: tuple
    p2: tuple
    radius: float

    def centre(self) -> np.ndarray:  # cylinder.rs:40
        return (np.asarray(_vec3(self.p1)) + np.asarray(_vec3(self.p2))) / 2.0


@dataclass
class SdfSphere:
    centre: tuple
    radius: float


@dataclass
class SdfTorus:
    """Torus around the +y axis: length((length(p.xz) - major, p.y)) - minor."""
    centre: tuple
    major: float
    minor: float


@dataclass
class SdfMandelbulb:
    """Power-n Mandelbulb distance estimator, scaled by `scale` world units."""
    centre: tuple
    power: float = 8.0
    iterations: int = 8
    scale: float = 1.0


@dataclass
class RaymarchedIsosurfaceMesh:
    """mesh/isosurface/raymarched.rs; defaults from :36-37."""
    sdf: Any
    max_iterations: int = 150
    epsilon: float = 1e-7

    DEFAULT_EPSILON = 1e-7
    DEFAULT_ITERATIONS = 150

    def centre(self) -> np.ndarray:  # raymarched.rs:69: the origin
        return np.zeros(3)


# ---------------------------------------------------------------------------
# Objects and scene
# ---------------------------------------------------------------------------
@dataclass(eq=False)
class SimpleObject:
    """object/simple.rs. `transform` (None, a Transform3, an ObjectTransform
    or a 4 x 4 / 3 x 4 matrix) maps mesh space to world space; like
    SimpleObject::new it is corrected to act about the mesh's centre, unless
    the object was made by `new_uncorrected`."""
    mesh: Any
    material: Any
    transform: Any = None
    corrected: bool = True

    @staticmethod
    def new(mesh, material, transform=None) -> "SimpleObject":
        return SimpleObject(mesh, material, transform)

    @staticmethod
    def new_uncorrected(mesh, material, transform=None) -> "SimpleObject":
        return SimpleObject(mesh, material, transform, corrected=False)

    def object_transform(self) -> ObjectTransform:
        t = ObjectTransform(_transform3(self.transform))
        if self.corrected and not t.is_identity:
            centre = self.mesh.centre() if hasattr(self.mesh, "centre") else np.zeros(3)
            t = t.with_correction(centre)
        return t


@dataclass(eq=False)
class VolumetricObject:
    """object/volumetric.rs: a constant-density medium bounded by a sphere or
    a box. `transform` is corrected about the mesh's centre, as
    VolumetricObject::new does (volumetric.rs:21-30), unless `corrected` is
    False (new_uncorrected)."""
    mesh: Any
    material: Any
    density: float
    transform: Any = None
    corrected: bool = True

    def object_transform(self) -> ObjectTransform:
        t = ObjectTransform(_transform3(self.transform))
        if self.corrected and not t.is_identity:
            t = t.with_correction(self.mesh.centre())
        return t


class ObjectList(list):
    """object/list.rs: a list of objects (BVH over bounded ones + unbounded list)."""


@dataclass
class Scene:
    """scene/mod.rs:11-24 (StandardScene)."""
    objects: Any = field(default_factory=ObjectList)
    skybox: Any = field(default_factory=SimpleSkybox)


StandardScene = Scene


# ---------------------------------------------------------------------------
# Flattening
# ---------------------------------------------------------------------------
def _identity(t) -> bool:
    return _transform3(t).is_identity()


class FlatScene:
    """Flat host arrays of one scene plus the rg_scene_desc pointing at them."""

    def __init__(self):
        self.materials: list = []
        self._mat_index: dict = {}
        self.textures: list = []
        self._tex_index: dict = {}
        self.images: list = []
        self._img_index: dict = {}
        self.sky_image = 0
        self.spheres, self.sphere_mat = [], []
        self.tri_v, self.tri_n, self.tri_mat, self.tri_mesh = [], [], [], []
        self.boxes, self.box_mat = [], []
        self.volumes: list = []
        self.sdfs: list = []
        self.quads, self.quad_mat = [], []
        self.cylinders, self.cyl_mat = [], []
        self.planes, self.plane_mat, self.plane_wrap = [], [], []
        # per transformed object: its corrected 3 x 4 matrix; per primitive: its index
        self.transforms: list = []
        self.sphere_xf, self.tri_xf, self.box_xf, self.quad_xf, self.cyl_xf = [], [], [], [], []
        self.vol_xf = []
        self.skybox = A.RG_SKY_SIMPLE
        self.n_meshes = 0

    def material(self, m) -> int:
        k = id(m)
        if k not in self._mat_index:
            self._mat_index[k] = (len(self.materials), m)
            self.materials.append(material_record(m, self.texture))
        return self._mat_index[k][0]

    def image(self, img: Image) -> int:
        k = id(img)
        if k not in self._img_index:
            self._img_index[k] = (len(self.images), img)
            self.images.append(img)
        return self._img_index[k][0]

    def texture(self, tex) -> int:
        """Index of `tex` in the texture table (registered on first use, its
        checker cells first)."""
        while isinstance(tex, DynamicTexture):
            tex = tex.inner
        k = id(tex)
        if k in self._tex_index:
            idx = self._tex_index[k][0]
            if idx < 0:
                raise ValueError("a checker texture contains itself")
            return idx
        self._tex_index[k] = (-1, tex)
        t = A.rg_texture()
        if _is_solid(tex):
            t.kind = A.RG_TEX_SOLID
            t.colour[:] = _colour(tex)
        elif isinstance(tex, (WorldCheckerTexture, UvCheckerTexture)):
            world = isinstance(tex, WorldCheckerTexture)
            t.kind = A.RG_TEX_WORLD_CHECKER if world else A.RG_TEX_UV_CHECKER
            t.odd, t.even = self.texture(tex.odd), self.texture(tex.even)
            t.scale[0] = float(tex.scale)
            off = _vec3(tex.offset) if world else tuple(float(x) for x in tex.offset) + (0.0,)
            if len(off) != 3:
                raise ValueError(f"a checker offset has {2 if not world else 3} components")
            t.offset[:] = off
        elif isinstance(tex, ImageTexture):
            t.kind = A.RG_TEX_IMAGE
            t.image = self.image(tex.image)
            t.scale[:] = tuple(float(x) for x in tex.scale)
            t.offset[:] = (float(tex.offset[0]), float(tex.offset[1]), 0.0)
        elif isinstance(tex, (WorldNoiseTexture, LocalNoiseTexture, UvNoiseTexture)):
            t.kind = A.RG_TEX_NOISE
            t.noise_seed, t.noise_channels, scale = _noise_params(tex.source)
            t.scale[0] = float(scale)
            t.noise_place = {WorldNoiseTexture: A.RG_NOISE_WORLD, LocalNoiseTexture: A.RG_NOISE_LOCAL,
                             UvNoiseTexture: A.RG_NOISE_UV}[type(tex)]
        else:
            raise UnsupportedVariant(f"texture {type(tex).__name__} cannot cross the C ABI")
        idx = len(self.textures)
        self.textures.append(t)
        self._tex_index[k] = (idx, tex)
        return idx

    def add(self, obj):
        if isinstance(obj, (list, tuple, ObjectList)):
            for o in obj:
                self.add(o)
            return
        if isinstance(obj, SimpleObject):
            mesh, mat = obj.mesh, self.material(obj.material)
            ot = obj.object_transform()
            if not ot.is_identity and isinstance(mesh, (RaymarchedIsosurfaceMesh, InfinitePlaneMesh)):
                raise UnsupportedVariant(f"a transformed {type(mesh).__name__} is not supported by the GPU path")
            self._add_mesh(mesh, mat, self._transform_index(ot))
        elif isinstance(obj, VolumetricObject):
            self.vol_xf.append(self._transform_index(obj.object_transform()))
            v = A.rg_volume()
            if isinstance(obj.mesh, SphereMesh):
                v.boundary = A.RG_BOUNDARY_SPHERE
                v.a[:] = _vec3(obj.mesh.pos)
                v.b[:] = (float(obj.mesh.radius), 0.0, 0.0)
            elif isinstance(obj.mesh, AxisBoxMesh):
                v.boundary = A.RG_BOUNDARY_BOX
                v.a[:] = _vec3(obj.mesh.a)
                v.b[:] = _vec3(obj.mesh.b)
            else:
                raise UnsupportedVariant(f"volume boundary {type(obj.mesh).__name__} is not supported")
            v.density = float(obj.density)
            v.material = self.material(obj.material)
            self.volumes.append(v)
        else:
            raise UnsupportedVariant(f"object {type(obj).__name__} cannot cross the C ABI")

    def _transform_index(self, ot: ObjectTransform) -> int:
        """The index of an object's (corrected) transform in the transform
        table, or RG_NO_TRANSFORM for the identity."""
        if ot.is_identity:
            return A.RG_NO_TRANSFORM
        m = ot.transform.matrix
        if not np.all(np.isfinite(m)) or abs(np.linalg.det(m[:3, :3])) == 0:
            raise ValueError("an object transform must be finite and invertible")
        self.transforms.append(m[:3].copy())
        return len(self.transforms) - 1

    def _add_mesh(self, mesh, mat: int, xf: int):
        """One mesh of a SimpleObject (or of a BvhMesh) with its material and
        transform index."""
        if isinstance(mesh, SphereMesh):
            self.spheres.append((*_vec3(mesh.pos), float(mesh.radius)))
            self.sphere_mat.append(mat)
            self.sphere_xf.append(xf)
        elif isinstance(mesh, Triangle):
            self.tri_v.append(np.asarray(mesh.vertices, np.float32).reshape(1, 3, 3))
            self.tri_n.append(np.asarray(mesh.normals, np.float32).reshape(1, 3, 3))
            self.tri_mat.append(np.full(1, mat, np.uint32))
            self.tri_mesh.append(np.full(1, -1, np.int32))
            self.tri_xf.append(np.full(1, xf, np.uint32))
        elif isinstance(mesh, BvhMesh):
            n = mesh.vertices.shape[0]
            if n:
                self.tri_v.append(mesh.vertices)
                self.tri_n.append(mesh.normals)
                self.tri_mat.append(np.full(n, mat, np.uint32))
                self.tri_mesh.append(np.full(n, self.n_meshes, np.int32))
                self.tri_xf.append(np.full(n, xf, np.uint32))
                self.n_meshes += 1
            for m in mesh.items:  # its other meshes: one object each, with the mesh's material and transform
                self._add_mesh(m, mat, xf)
        elif isinstance(mesh, AxisBoxMesh):
            self.boxes.append((*_vec3(mesh.a), *_vec3(mesh.b)))
            self.box_mat.append(mat)
            self.box_xf.append(xf)
        elif isinstance(mesh, RaymarchedIsosurfaceMesh):
            self.sdfs.append(self._sdf(mesh, mat))
        elif isinstance(mesh, ParallelogramMesh):
            self.quads.append(mesh.plane.flat())
            self.quad_mat.append(mat)
            self.quad_xf.append(xf)
        elif isinstance(mesh, CylinderMesh):
            self.cylinders.append((*_vec3(mesh.p1), *_vec3(mesh.p2), float(mesh.radius)))
            self.cyl_mat.append(mat)
            self.cyl_xf.append(xf)
        elif isinstance(mesh, InfinitePlaneMesh):
            self.planes.append(mesh.plane.flat())
            self.plane_mat.append(mat)
            self.plane_wrap.append({"wrap": A.RG_UV_WRAP, "mirror": A.RG_UV_MIRROR,
                                    "clamp_zero": A.RG_UV_CLAMP_ZERO}[mesh.uv_wrap])
        else:
            raise UnsupportedVariant(f"mesh {type(mesh).__name__} cannot cross the C ABI")

    @staticmethod
    def _sdf(mesh: RaymarchedIsosurfaceMesh, mat: int) -> A.rg_sdf:
        s = A.rg_sdf()
        f = mesh.sdf
        if isinstance(f, SdfSphere):
            s.kind, s.centre[:], s.params[:] = A.RG_SDF_SPHERE, _vec3(f.centre), (float(f.radius), 0, 0, 0)
        elif isinstance(f, SdfTorus):
            s.kind, s.centre[:], s.params[:] = A.RG_SDF_TORUS, _vec3(f.centre), (float(f.major), float(f.minor), 0, 0)
        elif isinstance(f, SdfMandelbulb):
            s.kind, s.centre[:] = A.RG_SDF_MANDELBULB, _vec3(f.centre)
            s.params[:] = (float(f.power), float(f.iterations), float(f.scale), 0.0)
        else:
            raise UnsupportedVariant("SDF closures cannot cross the C ABI; use SdfSphere/SdfTorus/SdfMandelbulb")
        s.max_iterations = int(mesh.max_iterations)
        s.epsilon = float(mesh.epsilon)
        s.material = mat
        return s

    def finish(self) -> "FlatScene":
        f32, u32 = np.float32, np.uint32
        self.a_spheres = np.ascontiguousarray(np.asarray(self.spheres, f32).reshape(-1, 4))
        self.a_sphere_mat = np.ascontiguousarray(np.asarray(self.sphere_mat, u32))
        if self.tri_v:
            self.a_tri_v = np.ascontiguousarray(np.concatenate(self.tri_v).astype(f32))
            self.a_tri_n = np.ascontiguousarray(np.concatenate(self.tri_n).astype(f32))
            self.a_tri_mat = np.ascontiguousarray(np.concatenate(self.tri_mat))
            self.a_tri_mesh = np.ascontiguousarray(np.concatenate(self.tri_mesh))
            self.a_tri_xf = np.ascontiguousarray(np.concatenate(self.tri_xf).astype(u32))
        else:
            self.a_tri_v = np.zeros((0, 3, 3), f32)
            self.a_tri_n = np.zeros((0, 3, 3), f32)
            self.a_tri_mat = np.zeros(0, u32)
            self.a_tri_mesh = np.zeros(0, np.int32)
            self.a_tri_xf = np.zeros(0, u32)
        self.a_boxes = np.ascontiguousarray(np.asarray(self.boxes, f32).reshape(-1, 6))
        self.a_box_mat = np.ascontiguousarray(np.asarray(self.box_mat, u32))
        self.a_quads = np.ascontiguousarray(np.asarray(self.quads, f32).reshape(-1, 9))
        self.a_quad_mat = np.ascontiguousarray(np.asarray(self.quad_mat, u32))
        self.a_cyls = np.ascontiguousarray(np.asarray(self.cylinders, f32).reshape(-1, 7))
        self.a_cyl_mat = np.ascontiguousarray(np.asarray(self.cyl_mat, u32))
        self.a_planes = np.ascontiguousarray(np.asarray(self.planes, f32).reshape(-1, 9))
        self.a_plane_mat = np.ascontiguousarray(np.asarray(self.plane_mat, u32))
        self.a_plane_wrap = np.ascontiguousarray(np.asarray(self.plane_wrap, u32))
        self.a_transforms = np.ascontiguousarray(np.asarray(self.transforms, np.float64).reshape(-1, 12))
        self.a_sphere_xf = np.ascontiguousarray(np.asarray(self.sphere_xf, u32))
        self.a_box_xf = np.ascontiguousarray(np.asarray(self.box_xf, u32))
        self.a_quad_xf = np.ascontiguousarray(np.asarray(self.quad_xf, u32))
        self.a_cyl_xf = np.ascontiguousarray(np.asarray(self.cyl_xf, u32))
        self.a_vol_xf = np.ascontiguousarray(np.asarray(self.vol_xf, u32))
        self.c_volumes = (A.rg_volume * max(1, len(self.volumes)))(*self.volumes)
        self.c_sdfs = (A.rg_sdf * max(1, len(self.sdfs)))(*self.sdfs)
        self.c_materials = (A.rg_material * max(1, len(self.materials)))(*self.materials)
        self.c_textures = (A.rg_texture * max(1, len(self.textures)))(*self.textures)
        self.c_images = (A.rg_image * max(1, len(self.images)))()
        for i, img in enumerate(self.images):
            self.c_images[i].width, self.c_images[i].height = img.width, img.height
            self.c_images[i].rgb = img.data.ctypes.data_as(C.POINTER(C.c_float))
        d = A.rg_scene_desc()
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        up = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint32))
        d.n_spheres, d.spheres, d.sphere_material = len(self.a_spheres), fp(self.a_spheres), up(self.a_sphere_mat)
        d.n_triangles = self.a_tri_v.shape[0]
        d.tri_vertices, d.tri_normals = fp(self.a_tri_v), fp(self.a_tri_n)
        d.tri_material = up(self.a_tri_mat)
        d.tri_mesh = self.a_tri_mesh.ctypes.data_as(C.POINTER(C.c_int32))
        d.n_boxes, d.boxes, d.box_material = len(self.a_boxes), fp(self.a_boxes), up(self.a_box_mat)
        d.n_volumes, d.volumes = len(self.volumes), self.c_volumes
        d.n_sdfs, d.sdfs = len(self.sdfs), self.c_sdfs
        d.n_materials, d.materials = len(self.materials), self.c_materials
        d.skybox = self.skybox
        d.n_quads, d.quads, d.quad_material = len(self.a_quads), fp(self.a_quads), up(self.a_quad_mat)
        d.n_cylinders, d.cylinders, d.cylinder_material = len(self.a_cyls), fp(self.a_cyls), up(self.a_cyl_mat)
        d.n_planes, d.planes, d.plane_material = len(self.a_planes), fp(self.a_planes), up(self.a_plane_mat)
        d.plane_uv_wrap = up(self.a_plane_wrap)
        d.n_textures, d.textures = len(self.textures), self.c_textures
        d.n_images, d.images = len(self.images), self.c_images
        d.sky_image = self.sky_image
        if len(self.a_transforms):
            d.n_transforms = len(self.a_transforms)
            d.transforms = self.a_transforms.ctypes.data_as(C.POINTER(C.c_double))
            d.sphere_transform, d.tri_transform = up(self.a_sphere_xf), up(self.a_tri_xf)
            d.box_transform, d.quad_transform = up(self.a_box_xf), up(self.a_quad_xf)
            d.cylinder_transform = up(self.a_cyl_xf)
            d.volume_transform = up(self.a_vol_xf)
        self.desc = d
        return self

    @property
    def n_prims(self) -> int:
        d = self.desc
        return (d.n_spheres + d.n_triangles + d.n_boxes + d.n_volumes + d.n_sdfs + d.n_quads + d.n_cylinders +
                d.n_planes)


def flatten(scene: Scene) -> FlatScene:
    """Flattens a Scene into rg_scene_desc arrays (object order: spheres,
    standalone triangles, meshes, boxes, volumes, parallelograms, cylinders;
    unbounded: SDFs, infinite planes)."""
    fs = FlatScene()
    sky = scene.skybox
    if sky is None:
        sky = NoSkybox()  # `None.into()` is NoSkybox (skybox/mod.rs:39-43)
    if not hasattr(sky, "kind"):
        raise UnsupportedVariant(f"skybox {type(sky).__name__} cannot cross the C ABI")
    fs.skybox = sky.kind
    if isinstance(sky, HdrImageSkybox):
        fs.sky_image = fs.image(sky.image)
    fs.add(scene.objects)
    return fs.finish()
