"""Oracle pins for the non-solid textures and the image sky (CPU).

Known answers from the reference's definitions: do_checker
(texture/checker.rs:46-63: the floors of the scaled, offset coordinates
summed, even cells where rem_euclid(sum, 2) < 1), ImageTexture::value
(texture/image.rs:29-39: offset + uv * scale, v flipped, times the image size),
Image::get_bilinear (core/image.rs:87-109: floor and ceil clamped to the
image, the fraction against the clamped floor) and HdrImageSkybox
(skybox/hdri.rs:17-26: sphere_uv of the direction). The colour a ray sees is
read through a light (its emission is the texture value) or the sky. Noise
textures use Perlin's improved noise over this library's own seeded
permutation (the noise crate's permutation generator is not reproduced):
their values are pinned only by properties (zero at lattice points, range,
determinism).
"""
import math

import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300.scene import (
    AxisBoxMesh, ColourSource, HdrImageSkybox, Image, ImageTexture, LambertianMaterial, LightMaterial,
    LocalNoiseTexture, NoSkybox, ParallelogramMesh, Perlin, Planar, ScalePoint, Scene, SimpleObject, SphereMesh,
    Transform3, UvCheckerTexture, UvNoiseTexture, WorldCheckerTexture, WorldNoiseTexture, flatten,
)

POLICIES = [ob.POLICY_REF_F64, ob.POLICY_GPU_F32]
WHITE, BLACK, RED = (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (1.0, 0.0, 0.0)


def floor_scene(tex, sky=None):
    """A 20 x 20 light on y = 0 (corner (-10, 0, -10), sides along x and z)."""
    q = ParallelogramMesh(Planar.new((-10, 0, -10), (20, 0, 0), (0, 0, 20)))
    return flatten(Scene(objects=[SimpleObject(q, LightMaterial(tex))], skybox=sky or NoSkybox()))


def down_at(xz):
    xz = np.asarray(xz, np.float64)
    o = np.stack([xz[:, 0], np.ones(len(xz)), xz[:, 1]], axis=1)
    d = np.tile([0.0, -1.0, 0.0], (len(xz), 1))
    return o, d


@pytest.mark.parametrize("policy", POLICIES)
def test_world_checker_cells(policy):
    flat = floor_scene(WorldCheckerTexture(even=WHITE, odd=BLACK, scale=1.0))
    pts = [(0.5, 0.5), (1.5, 0.5), (1.5, 1.5), (-0.5, 0.5), (-0.5, -0.5), (-1.5, 2.5), (3.25, -7.75)]
    o, d = down_at(pts)
    c = ob.query_colour(flat, o, d, policy)
    for (x, z), col in zip(pts, c):
        s = math.floor(x) + 0 + math.floor(z)  # y = 0 on the floor
        want = WHITE if (s % 2) < 1 else BLACK  # Python's % is rem_euclid for a positive modulus
        np.testing.assert_array_equal(col, want, err_msg=f"{x}, {z}")
    # scale and offset: cells of 2, shifted by one cell along x
    flat = floor_scene(WorldCheckerTexture(even=WHITE, odd=BLACK, scale=2.0, offset=(1.0, 0.0, 0.0)))
    c = ob.query_colour(flat, *down_at([(0.5, 0.5), (2.5, 0.5), (-1.5, 0.5)]), policy)
    np.testing.assert_array_equal(c, [BLACK, WHITE, WHITE])


@pytest.mark.parametrize("policy", POLICIES)
def test_uv_checker_nested(policy):
    # uv on the floor: u = (x + 10) / 20, v = (z + 10) / 20; cells of 0.25 in uv
    inner = UvCheckerTexture(even=RED, odd=BLACK, scale=0.125)
    flat = floor_scene(UvCheckerTexture(even=WHITE, odd=inner, scale=0.25))
    pts = [(-9.0, -9.0), (-4.0, -9.0), (-6.0, -9.0), (-1.0, -9.0)]
    c = ob.query_colour(flat, *down_at(pts), policy)
    for (x, z), col in zip(pts, c):
        u, v = (x + 10) / 20, (z + 10) / 20
        if (math.floor(u / 0.25) + math.floor(v / 0.25)) % 2 < 1:
            want = WHITE
        else:
            want = RED if (math.floor(u / 0.125) + math.floor(v / 0.125)) % 2 < 1 else BLACK
        np.testing.assert_array_equal(col, want, err_msg=f"{x}, {z}")


def test_image_bilinear_reference_rules():
    img = Image(np.arange(2 * 3 * 3, dtype=np.float32).reshape(2, 3, 3))
    np.testing.assert_allclose(img.get_bilinear(0.0, 0.0), img.data[0, 0])
    np.testing.assert_allclose(img.get_bilinear(0.5, 0.0), (img.data[0, 0] + img.data[1, 0]) / 2)
    # beyond the last texel both corners clamp to it: no wrap, no extrapolation
    np.testing.assert_allclose(img.get_bilinear(1.7, 2.4), img.data[1, 2])
    np.testing.assert_allclose(img.get_bilinear(-3.0, 0.0), img.data[0, 0])


@pytest.mark.parametrize("policy", POLICIES)
def test_image_texture_known_answers(policy):
    rng = np.random.Generator(np.random.PCG64(5))
    img = Image(rng.random((5, 4, 3)).astype(np.float32))
    tex = ImageTexture(img, scale=(1.0, 1.0), offset=(0.0, 0.0))
    flat = floor_scene(tex)
    pts = rng.uniform(-9.9, 9.9, (64, 2))
    c = ob.query_colour(flat, *down_at(pts), policy)
    for (x, z), col in zip(pts, c):
        u, v = (x + 10) / 20, (z + 10) / 20
        want = img.get_bilinear(u * img.width, (1 - v) * img.height)
        np.testing.assert_allclose(col, want, rtol=2e-5, atol=2e-6)
    # scale and offset: uv * 2 + 0.25, read in the same image
    tex2 = ImageTexture(img, scale=(2.0, 0.5), offset=(0.25, 0.1))
    c = ob.query_colour(floor_scene(tex2), *down_at(pts[:16]), policy)
    for (x, z), col in zip(pts[:16], c):
        u, v = 0.25 + 2.0 * (x + 10) / 20, 0.1 + 0.5 * (z + 10) / 20
        np.testing.assert_allclose(col, img.get_bilinear(u * img.width, (1 - v) * img.height), rtol=2e-5, atol=2e-6)


@pytest.mark.parametrize("policy", POLICIES)
def test_hdri_sky(policy):
    rng = np.random.Generator(np.random.PCG64(6))
    img = Image(rng.random((16, 8, 3)).astype(np.float32) * 4)  # HDR: values above 1
    flat = flatten(Scene(objects=[], skybox=HdrImageSkybox(img)))
    d = rng.normal(size=(200, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    c = ob.query_colour(flat, np.zeros((200, 3)), d, policy)
    for di, col in zip(d.astype(np.float32).astype(np.float64), c):
        di = di / np.linalg.norm(di)
        theta = math.acos(-di[1])
        phi = math.atan2(-di[2], di[0]) + math.pi
        u, v = phi / (2 * math.pi), theta / math.pi
        want = img.get_bilinear(u * img.width, (1 - v) * img.height)
        np.testing.assert_allclose(col, want, rtol=1e-4, atol=1e-5)
    # +x: theta = pi / 2, phi = pi: the image centre
    c = ob.query_colour(flat, [(0, 0, 0)], [(1, 0, 0)], policy)
    np.testing.assert_allclose(c[0], img.get_bilinear(8.0, 4.0), rtol=1e-5)


def noise(place, seed=69, scale=4.0, rgb=False):
    if rgb:
        src = ColourSource.Rgb([ScalePoint(Perlin(seed + i)).set_scale(scale) for i in range(3)])
    else:
        src = ColourSource.Greyscale(ScalePoint(Perlin(seed)).set_scale(scale))
    return {"world": WorldNoiseTexture, "local": LocalNoiseTexture, "uv": UvNoiseTexture}[place](src)


@pytest.mark.parametrize("policy", POLICIES)
def test_noise_properties(policy):
    rng = np.random.Generator(np.random.PCG64(7))
    # at lattice points gradient noise is 0, so the colour is 0.5
    flat = floor_scene(noise("world", scale=1.0))
    lattice = [(float(x), float(z)) for x in range(-3, 4) for z in (-2, 1, 5)]
    c = ob.query_colour(flat, *down_at(lattice), policy)
    np.testing.assert_allclose(c, 0.5, atol=1e-6)
    pts = rng.uniform(-9, 9, (500, 2))
    c = ob.query_colour(flat, *down_at(pts), policy)
    assert np.all((c >= 0) & (c <= 1))
    assert np.all(c[:, 0] == c[:, 1]) and c.std() > 0.03  # greyscale, and not constant
    c2 = ob.query_colour(floor_scene(noise("world", scale=1.0)), *down_at(pts), policy)
    np.testing.assert_array_equal(c, c2)  # deterministic
    c3 = ob.query_colour(floor_scene(noise("world", seed=70, scale=1.0)), *down_at(pts), policy)
    assert np.mean(np.abs(c - c3)) > 0.02  # another seed, another field
    crgb = ob.query_colour(floor_scene(noise("world", scale=1.0, rgb=True)), *down_at(pts), policy)
    np.testing.assert_array_equal(crgb[:, 0], c[:, 0])  # red is the seed's own source
    assert np.mean(np.abs(crgb[:, 1] - crgb[:, 0])) > 0.02


def test_noise_f32_agrees_with_f64():
    rng = np.random.Generator(np.random.PCG64(8))
    pts = rng.uniform(-9, 9, (2000, 2))
    for place in ("world", "local", "uv"):
        flat = floor_scene(noise(place, scale=3.0, rgb=True))
        a = ob.query_colour(flat, *down_at(pts), ob.POLICY_REF_F64)
        b = ob.query_colour(flat, *down_at(pts), ob.POLICY_GPU_F32)
        assert np.max(np.abs(a - b)) < 1e-4, place


@pytest.mark.parametrize("policy", POLICIES)
def test_local_point_per_primitive(policy):
    """pos_l (the point a LocalNoiseTexture reads): a sphere's unit local point
    (sphere.rs:77-91), a box's point less its centre (axis_box.rs:122); under a
    transform the reference maps pos_l as a point too (transform.rs:123)."""
    def colour_of(mesh, transform, o, d):
        src = LocalNoiseTexture(ColourSource.Greyscale(Perlin(3)))
        flat = flatten(Scene(objects=[SimpleObject(mesh, LightMaterial(src), transform)], skybox=NoSkybox()))
        return ob.query_colour(flat, [o], [d], policy)[0]

    def world_at(p):
        src = WorldNoiseTexture(ColourSource.Greyscale(Perlin(3)))
        q = ParallelogramMesh(Planar.new((p[0] - 1, p[1], p[2] - 1), (2, 0, 0), (0, 0, 2)))
        flat = flatten(Scene(objects=[SimpleObject(q, LightMaterial(src))], skybox=NoSkybox()))
        return ob.query_colour(flat, [(p[0], p[1] + 1, p[2])], [(0, -1, 0)], policy)[0]

    # sphere of radius 2 at (5, 0, 0), hit at its top: local point (0, 1, 0)
    c = colour_of(SphereMesh((5, 0, 0), 2.0), None, (5, 5, 0), (0, -1, 0))
    np.testing.assert_allclose(c, world_at((0.0, 1.0, 0.0)), atol=1e-6)
    # box centred at (1, 1, 1), half size 0.5, hit at (1.2, 1.5, 0.9): local (0.2, 0.5, -0.1)
    c = colour_of(AxisBoxMesh((0.5, 0.5, 0.5), (1.5, 1.5, 1.5)), None, (1.2, 3.0, 0.9), (0, -1, 0))
    np.testing.assert_allclose(c, world_at((0.2, 0.5, -0.1)), atol=2e-5)
    # the same box translated by (0, 0, 3): pos_l is (0.2, 0.5, -0.1) mapped, (0.2, 0.5, 2.9)
    c = colour_of(AxisBoxMesh((0.5, 0.5, 0.5), (1.5, 1.5, 1.5)), Transform3.from_translation((0, 0, 3)),
                  (1.2, 3.0, 3.9), (0, -1, 0))
    np.testing.assert_allclose(c, world_at((0.2, 0.5, 2.9)), atol=2e-5)


def test_texture_table_validation():
    import ctypes as C
    from rayna_gb300 import _abi as A
    lib = A.load_library()
    info = A.rg_scene_info()
    flat = floor_scene(UvCheckerTexture(even=WHITE, odd=BLACK))
    assert lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info)) == A.RG_OK
    flat.c_textures[2].odd = 2  # the checker refers to itself
    assert lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info)) == A.RG_INVALID_ARG
    assert "cycle" in A.last_error(lib, None)
    flat = floor_scene(ImageTexture(Image(np.zeros((2, 2, 3)))))
    flat.c_textures[0].image = 5
    assert lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info)) == A.RG_INVALID_ARG
    flat = floor_scene(WHITE)
    flat.c_materials[0].texture = 3
    assert lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info)) == A.RG_INVALID_ARG


@pytest.mark.parametrize("policy", POLICIES)
def test_world_checker_on_a_transformed_object_reads_world_space(policy):
    """WorldCheckerTexture reads pos_w, the mapped point (transform.rs:123): a
    floor light moved 3 along x by its transform shows the cells of its world
    position, not of its mesh-space one."""
    q = ParallelogramMesh(Planar.new((-10, 0, -10), (20, 0, 0), (0, 0, 20)))
    tex = WorldCheckerTexture(even=WHITE, odd=BLACK, scale=1.0, offset=(0.0, 0.5, 0.0))
    flat = flatten(Scene(objects=[SimpleObject(q, LightMaterial(tex), Transform3.from_translation((3.0, 0.0, 0.0)))],
                         skybox=NoSkybox()))
    pts = [(0.5, 0.5), (1.5, 0.5), (-0.5, 0.5), (4.25, -2.5)]
    c = ob.query_colour(flat, *down_at(pts), policy)
    for (x, z), col in zip(pts, c):
        want = WHITE if (math.floor(x) + math.floor(0.5) + math.floor(z)) % 2 < 1 else BLACK
        np.testing.assert_array_equal(col, want, err_msg=f"{x}, {z}")
