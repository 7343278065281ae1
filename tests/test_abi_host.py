"""C-ABI and host-logic tests that need no GPU.

The library must load, export every entry point include/rayna_gpu.h declares,
report RG_NO_DEVICE cleanly when no GPU is visible, and validate/build scenes
on the host (rg_inspect_scene) exactly as rg_set_scene would.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from rayna_gb300 import _abi as A
from rayna_gb300 import presets
from rayna_gb300.scene import (
    AxisBoxMesh, BvhMesh, DielectricMaterial, LambertianMaterial, RaymarchedIsosurfaceMesh, Scene, SdfTorus,
    SimpleObject, SphereMesh, Transform3, Triangle, UnsupportedVariant, VolumetricObject, IsotropicMaterial, flatten,
)

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "rayna_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rg_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = A.load_library()
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(A.SIGNATURES), "ctypes signatures must cover the header exactly"
    assert lib.rg_abi_version() == A.RG_ABI_VERSION == 8


@pytest.mark.parametrize("exact", [False, True])
def test_both_arithmetic_builds_load_and_export_the_same_symbols(exact):
    lib = A.load_library(exact=exact)
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert lib.rg_abi_version() == 8
    assert A.load_library(exact=exact) is lib


def test_header_constants_match_the_ctypes_mirror():
    text = open(HEADER).read()
    assert re.search(r"#define RG_SHARED_STACK_NONE 0xFFFFFFFFu", text)
    for name in ("RG_DEVICE_STACK_OVERFLOW", "RG_DEVICE_BAD_INDEX", "RG_DEVICE_QUEUE_OVERFLOW"):
        m = re.search(name + r" = (\d+)u", text)
        assert m and int(m.group(1)) == getattr(A, name), name


def _run_child(code, env_extra):
    import subprocess
    import sys
    env = dict(os.environ, **env_extra)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip().splitlines()[-1]


@pytest.mark.parametrize("exact", ["0", "1"])
def test_forced_host_allocation_failure_reports_oom(exact):
    """RAYNA_GPU_FAIL_ALLOC=1 fails the first allocation the library counts
    (here the host arrays of the scene build): rg_inspect_scene returns
    RG_OOM with a message instead of unwinding through the C ABI, and the
    next call, with the injection spent, builds the scene."""
    code = (
        "import ctypes as C\n"
        "from rayna_gb300 import _abi as A, presets\n"
        "from rayna_gb300.scene import flatten\n"
        "lib = A.load_library()\n"
        "flat = flatten(presets.random_spheres(seed=0)[0])\n"
        "info = A.rg_scene_info()\n"
        "a = lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info))\n"
        "msg = A.last_error(lib, None)\n"
        "b = lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info))\n"
        "print(a, b, info.n_prims, 'memory' in msg)\n")
    out = _run_child(code, {"RAYNA_GPU_FAIL_ALLOC": "1", "RAYNA_GB300_EXACT": exact})
    assert out == f"{A.RG_OOM} {A.RG_OK} 488 True", out


def test_struct_sizes_match_header_layout():
    assert C.sizeof(A.rg_material) == 32
    assert C.sizeof(A.rg_hit) == 48
    assert C.sizeof(A.rg_camera) == 9 * 8
    assert C.sizeof(A.rg_render_opts) == 24


def test_create_without_device_reports_no_device(gpu_available):
    if gpu_available:
        pytest.skip("a GPU is visible")
    lib = A.load_library()
    h = C.c_void_p()
    st = lib.rg_create(None, C.byref(h))
    assert st == A.RG_NO_DEVICE
    assert "no CUDA device" in A.last_error(lib, None)


def inspect(scene):
    lib = A.load_library()
    flat = flatten(scene)
    info = A.rg_scene_info()
    st = lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info))
    return st, info, A.last_error(lib, None)


def test_inspect_random_spheres_bvh():
    scene, _, _ = presets.random_spheres(seed=0)
    st, info, _ = inspect(scene)
    assert st == A.RG_OK
    assert info.n_prims == 488
    assert info.max_leaf_size <= 4
    assert info.n_leaves >= 488 // 4
    assert info.max_depth < 60
    assert info.n_nodes == info.n_leaves - 1 or info.n_nodes >= info.n_leaves // 2


def test_inspect_mesh_bvh_depth_and_size():
    scene, _, _ = presets.cornell_mesh(level=5)
    st, info, _ = inspect(scene)
    assert st == A.RG_OK
    assert info.n_prims == 20 * 4 ** 5 + 12
    assert info.max_leaf_size <= 4
    assert info.max_depth < 60
    assert info.sah_cost > 0
    assert info.device_bytes >= info.n_prims * 48 + info.n_nodes * 64


@pytest.mark.parametrize("bad,status", [
    (Scene(objects=[SimpleObject(SphereMesh((float("nan"), 0, 0), 1.0), LambertianMaterial())]), A.RG_INVALID_ARG),
    (Scene(objects=[VolumetricObject(SphereMesh((0, 0, 0), 1.0), IsotropicMaterial(), -1.0)]), A.RG_INVALID_ARG),
    (Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), DielectricMaterial((1, 1, 1), float("inf"), 0.0))]),
     A.RG_INVALID_ARG),
])
def test_inspect_rejects_invalid_descriptors(bad, status):
    st, _, msg = inspect(bad)
    assert st == status
    assert msg


def test_inspect_rejects_bad_material_index_and_null_arrays():
    lib = A.load_library()
    flat = flatten(Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial())]))
    flat.a_sphere_mat[0] = 7
    info = A.rg_scene_info()
    assert lib.rg_inspect_scene(C.byref(flat.desc), C.byref(info)) == A.RG_INVALID_ARG
    d = A.rg_scene_desc()
    d.n_spheres = 3
    assert lib.rg_inspect_scene(C.byref(d), C.byref(info)) == A.RG_INVALID_ARG
    assert "NULL" in A.last_error(lib, None)


def test_triangle_constructor_asserts():
    with pytest.raises(ValueError):
        Triangle([[0, 0, 0], [0, 0, 0], [1, 0, 0]], [[0, 0, 1]] * 3)
    with pytest.raises(ValueError):
        Triangle([[0, 0, 0], [0, 1, 0], [1, 0, 0]], [[0, 0, 2]] * 3)


def test_flatten_order_and_unsupported_variants():
    objs = [
        SimpleObject(RaymarchedIsosurfaceMesh(SdfTorus((0, 0, 0), 1.0, 0.3)), LambertianMaterial()),
        SimpleObject(AxisBoxMesh((0, 0, 0), (1, 1, 1)), LambertianMaterial()),
        SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial()),
    ]
    flat = flatten(Scene(objects=objs))
    assert (flat.desc.n_spheres, flat.desc.n_boxes, flat.desc.n_sdfs) == (1, 1, 1)
    assert flat.desc.n_materials == 3
    with pytest.raises(ValueError):  # not affine: the bottom row is not (0, 0, 0, 1)
        flatten(Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial(), transform=np.eye(4) * 2)]))
    scaled = Transform3.from_scale((2, 2, 2))
    flat = flatten(Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial(), transform=scaled)]))
    assert flat.desc.n_transforms == 1 and flat.desc.sphere_transform[0] == 0
    with pytest.raises(UnsupportedVariant):
        flatten(Scene(objects=[SimpleObject(RaymarchedIsosurfaceMesh(SdfTorus((0, 0, 0), 1.0, 0.3)),
                                            LambertianMaterial(), transform=scaled)]))
    flat = flatten(Scene(objects=[VolumetricObject(SphereMesh((0, 0, 0), 1.0), IsotropicMaterial((1, 1, 1)), 0.5,
                                                   transform=scaled)]))
    assert flat.desc.n_transforms == 1 and flat.desc.volume_transform[0] == 0
    with pytest.raises(ValueError):
        flatten(Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial(),
                                            transform=Transform3.from_scale((1, 0, 1)))]))
    with pytest.raises(UnsupportedVariant):
        flatten(Scene(objects=[SimpleObject(RaymarchedIsosurfaceMesh(lambda p: 0.0), LambertianMaterial())]))


def test_presets_shapes_and_winding():
    scene, cam, opts = presets.random_spheres(seed=0)
    flat = flatten(scene)
    assert flat.desc.n_spheres == 488
    assert (opts.width, opts.height, opts.samples, opts.ray_depth) == (400, 225, 32, 50)
    v, f = presets.icosphere(3)
    assert f.shape[0] == 20 * 4 ** 3 and v.shape[0] == 10 * 4 ** 3 + 2
    verts, norms = presets.displaced_icosphere(3, (0.5, 0.3, 0.5), 0.25, seed=0)
    e1 = verts[:, 1] - verts[:, 0]
    e2 = verts[:, 2] - verts[:, 0]
    g = np.cross(e1, e2)
    # reference convention: e1 x e2 points away from the side the normals face
    assert np.all(np.einsum("ij,ij->i", g, norms.mean(axis=1)) < 0)
    np.testing.assert_allclose(np.linalg.norm(norms, axis=2), 1.0, atol=1e-5)
    v2, n2 = presets.displaced_icosphere(3, (0.5, 0.3, 0.5), 0.25, seed=0)
    assert np.array_equal(verts, v2)
    for t in presets.cornell_box_triangles():
        tv = t.mesh.vertices
        assert np.dot(np.cross(tv[1] - tv[0], tv[2] - tv[0]), t.mesh.normals[0]) < 0


def test_flatten_textures_and_images():
    """Non-solid textures go to the texture table once each (checker cells
    first, DynamicTexture unwrapped); images once each; unsupported noise
    sources and unbounded meshes in a BvhMesh are refused."""
    from rayna_gb300.scene import (
        ColourSource, DynamicTexture, HdrImageSkybox, Image, ImageTexture, InfinitePlaneMesh, LightMaterial, Perlin,
        Planar, ScalePoint, UvCheckerTexture, WorldCheckerTexture, WorldNoiseTexture,
    )
    img = Image(np.zeros((4, 2, 3), np.float32))
    inner = ImageTexture(img, scale=(2.0, 1.0))
    chk = WorldCheckerTexture(even=(1, 1, 1), odd=DynamicTexture(inner), scale=0.5, offset=(0, 0.5, 0))
    objs = [SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial(chk)),
            SimpleObject(SphereMesh((3, 0, 0), 1.0), LambertianMaterial(DynamicTexture(chk))),
            SimpleObject(SphereMesh((6, 0, 0), 1.0), LightMaterial(inner))]
    flat = flatten(Scene(objects=objs, skybox=HdrImageSkybox(img)))
    d = flat.desc
    assert (d.n_textures, d.n_images, d.skybox, d.sky_image) == (3, 1, A.RG_SKY_IMAGE, 0)
    kinds = [flat.c_textures[i].kind for i in range(3)]
    assert kinds == [A.RG_TEX_IMAGE, A.RG_TEX_SOLID, A.RG_TEX_WORLD_CHECKER]
    assert (flat.c_textures[2].odd, flat.c_textures[2].even) == (0, 1)
    assert [m.texture for m in flat.materials] == [3, 3, 1]
    assert flat.c_textures[0].scale[0] == 2.0 and flat.c_textures[2].offset[1] == 0.5
    with pytest.raises(UnsupportedVariant):  # a non-uniform ScalePoint
        flatten(Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial(
            WorldNoiseTexture(ColourSource.Greyscale(ScalePoint(Perlin(1), scale=(1, 2, 1))))))]))
    with pytest.raises(UnsupportedVariant):  # Rgb channels must be seeded s, s + 1, s + 2
        flatten(Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), LambertianMaterial(
            WorldNoiseTexture(ColourSource.Rgb([Perlin(1), Perlin(5), Perlin(3)]))))]))
    with pytest.raises(UnsupportedVariant):  # a BvhMesh holds bounded meshes
        BvhMesh([InfinitePlaneMesh(Planar.new((0, 0, 0), (1, 0, 0), (0, 0, 1)))])
    flat = flatten(Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0),
                                               LambertianMaterial(UvCheckerTexture(even=(1, 1, 1), odd=(0, 0, 0))))]))
    assert flat.desc.n_textures == 3 and flat.materials[0].texture == 3


def test_ctypes_layout_equals_the_c_header(tmp_path):
    """Every ctypes structure has the C header's size and, field by field,
    its offsets (a small C program built with the host compiler prints them)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = [getattr(A, n) for n in dir(A) if n.startswith("rg_") and isinstance(getattr(A, n), type)
               and issubclass(getattr(A, n), C.Structure)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rayna_gpu.h"', 'int main(void) {']
    for s in structs:
        lines.append(f'  printf("{s.__name__} size %zu\\n", sizeof({s.__name__}));')
        for name, _ in s._fields_:
            lines.append(f'  printf("{s.__name__} {name} %zu\\n", offsetof({s.__name__}, {name}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout.split("\n")
    want = []
    for s in structs:
        want.append(f"{s.__name__} size {C.sizeof(s)}")
        for name, _ in s._fields_:
            want.append(f"{s.__name__} {name} {getattr(s, name).offset}")
    assert [g for g in got if g] == want


@pytest.mark.parametrize("preset", ["cornell", "cornell_quads", "rtiaw_demo", "rtiaw_demo_dark", "rttnw_demo",
                                    "textures_demo", "sdf_volumes"])
def test_inspect_every_preset(preset):
    """The host side of rg_set_scene (validation, transforms, textures, both
    trees) accepts every preset; the tree holds every bounded primitive (SDFs
    and infinite planes stay in the unbounded list)."""
    scene, _, _ = getattr(presets, preset)()
    flat = flatten(scene)
    st, info, _ = inspect(scene)
    assert st == A.RG_OK, A.last_error(A.load_library(), None)
    d = flat.desc
    assert info.n_prims == d.n_spheres + d.n_triangles + d.n_boxes + d.n_volumes + d.n_quads + d.n_cylinders
    assert info.max_depth < 60


def test_all_reference_presets_render_on_the_oracle():
    """presets.ALL() (preset::ALL): each scene flattens, builds on the host,
    and renders a few pixels on the f64 oracle with finite, non-negative
    colours."""
    from oracle import binding as ob
    from rayna_gb300.scene import RenderOpts
    names = []
    for name, scene, cam, _ in presets.ALL():
        names.append(name)
        assert inspect(scene)[0] == A.RG_OK
        st, mean, _, _ = ob.render(flatten(scene), cam, RenderOpts(width=8, height=6, samples=2, ray_depth=4), seed=3)
        assert st == 0 and np.all(np.isfinite(mean)) and np.all(mean >= 0)
    assert names == ["RTIAW Demo", "RTIAW Demo (Night)", "RTTNW Demo", "Cornell Box"]
