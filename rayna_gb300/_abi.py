"""ctypes mirror of include/rayna_gpu.h and the loader of the native library.

The library is built in-tree by ``__graft_entry__.build()`` in two arithmetic
builds of one source: ``rayna_gb300/_lib/librayna_gpu.so`` (the performance
build, loaded by default) and ``librayna_gpu_exact.so`` (fused multiply-adds
only where the source writes them, loaded with ``exact=True`` or
RAYNA_GB300_EXACT=1). Loading fails loudly when a library is missing: there is
no CPU fallback behind this package.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librayna_gpu.so")
LIB_EXACT_PATH = os.path.join(_HERE, "_lib", "librayna_gpu_exact.so")

RG_OK = 0
RG_INVALID_ARG = 1
RG_UNSUPPORTED_VARIANT = 2
RG_INVALID_CAMERA = 3
RG_OOM = 4
RG_CUDA_ERROR = 5
RG_QUEUE_OVERFLOW = 6
RG_STEP_LIMIT = 7
RG_TIMEOUT = 8
RG_NO_DEVICE = 9
RG_NOT_READY = 10

STATUS_NAMES = {
    0: "RG_OK", 1: "RG_INVALID_ARG", 2: "RG_UNSUPPORTED_VARIANT", 3: "RG_INVALID_CAMERA",
    4: "RG_OOM", 5: "RG_CUDA_ERROR", 6: "RG_QUEUE_OVERFLOW", 7: "RG_STEP_LIMIT",
    8: "RG_TIMEOUT", 9: "RG_NO_DEVICE", 10: "RG_NOT_READY",
}

RG_MAT_LAMBERTIAN, RG_MAT_METAL, RG_MAT_DIELECTRIC, RG_MAT_ISOTROPIC, RG_MAT_LIGHT = range(5)
RG_SKY_SIMPLE, RG_SKY_WHITE, RG_SKY_NONE, RG_SKY_IMAGE = range(4)
RG_TEX_SOLID, RG_TEX_WORLD_CHECKER, RG_TEX_UV_CHECKER, RG_TEX_IMAGE, RG_TEX_NOISE = range(5)
RG_NOISE_WORLD, RG_NOISE_LOCAL, RG_NOISE_UV = range(3)
RG_MAX_TEXTURE_DEPTH = 16
RG_BOUNDARY_SPHERE, RG_BOUNDARY_BOX = range(2)
RG_SDF_SPHERE, RG_SDF_TORUS, RG_SDF_MANDELBULB = range(3)
RG_FORM_MEGAKERNEL, RG_FORM_WAVEFRONT = range(2)
RG_FLAG_COUNTERS = 1
RG_FLAG_STAGE_TIMES = 2
RG_FLAG_VALIDATE = 4
(RG_INVALID_NONFINITE, RG_INVALID_NOT_NORMALISED, RG_INVALID_INTERVAL, RG_INVALID_POSITION, RG_INVALID_UV,
 RG_INVALID_COLOUR) = (1, 2, 4, 8, 16, 32)
RG_BATCH_WAVEFRONT = 0
RG_UV_WRAP, RG_UV_MIRROR, RG_UV_CLAMP_ZERO = 0, 1, 2
RG_NO_TRANSFORM = 0xFFFFFFFF
RG_BATCH_TILES = 1
RG_SHARED_STACK_NONE = 0xFFFFFFFF
RG_DEVICE_STACK_OVERFLOW, RG_DEVICE_BAD_INDEX, RG_DEVICE_QUEUE_OVERFLOW = 1, 2, 4
RG_ABI_VERSION = 8


class rg_material(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("albedo", C.c_float * 3), ("fuzz", C.c_float),
                ("refractive_index", C.c_float), ("density", C.c_float), ("texture", C.c_uint32)]


class rg_texture(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("odd", C.c_uint32), ("even", C.c_uint32), ("image", C.c_uint32),
                ("scale", C.c_float * 2), ("offset", C.c_float * 3), ("colour", C.c_float * 3),
                ("noise_seed", C.c_uint32), ("noise_place", C.c_uint32), ("noise_channels", C.c_uint32),
                ("reserved", C.c_uint32)]


class rg_image(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgb", C.POINTER(C.c_float))]


class rg_volume(C.Structure):
    _fields_ = [("boundary", C.c_uint32), ("a", C.c_float * 3), ("b", C.c_float * 3),
                ("density", C.c_float), ("material", C.c_uint32)]


class rg_sdf(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("centre", C.c_float * 3), ("params", C.c_float * 4),
                ("max_iterations", C.c_uint32), ("epsilon", C.c_float), ("material", C.c_uint32)]


class rg_scene_desc(C.Structure):
    _fields_ = [
        ("n_spheres", C.c_uint32), ("spheres", C.POINTER(C.c_float)), ("sphere_material", C.POINTER(C.c_uint32)),
        ("n_triangles", C.c_uint32), ("tri_vertices", C.POINTER(C.c_float)), ("tri_normals", C.POINTER(C.c_float)),
        ("tri_material", C.POINTER(C.c_uint32)), ("tri_mesh", C.POINTER(C.c_int32)),
        ("n_boxes", C.c_uint32), ("boxes", C.POINTER(C.c_float)), ("box_material", C.POINTER(C.c_uint32)),
        ("n_volumes", C.c_uint32), ("volumes", C.POINTER(rg_volume)),
        ("n_sdfs", C.c_uint32), ("sdfs", C.POINTER(rg_sdf)),
        ("n_materials", C.c_uint32), ("materials", C.POINTER(rg_material)),
        ("skybox", C.c_uint32),
        ("n_quads", C.c_uint32), ("quads", C.POINTER(C.c_float)), ("quad_material", C.POINTER(C.c_uint32)),
        ("n_cylinders", C.c_uint32), ("cylinders", C.POINTER(C.c_float)),
        ("cylinder_material", C.POINTER(C.c_uint32)),
        ("n_planes", C.c_uint32), ("planes", C.POINTER(C.c_float)), ("plane_material", C.POINTER(C.c_uint32)),
        ("plane_uv_wrap", C.POINTER(C.c_uint32)),
        ("n_transforms", C.c_uint32), ("transforms", C.POINTER(C.c_double)),
        ("sphere_transform", C.POINTER(C.c_uint32)), ("tri_transform", C.POINTER(C.c_uint32)),
        ("box_transform", C.POINTER(C.c_uint32)), ("quad_transform", C.POINTER(C.c_uint32)),
        ("cylinder_transform", C.POINTER(C.c_uint32)),
        ("n_textures", C.c_uint32), ("textures", C.POINTER(rg_texture)),
        ("n_images", C.c_uint32), ("images", C.POINTER(rg_image)), ("sky_image", C.c_uint32),
        ("volume_transform", C.POINTER(C.c_uint32)),
    ]


class rg_camera(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("fwd", C.c_double * 3), ("v_fov", C.c_double),
                ("focus_dist", C.c_double), ("defocus_angle", C.c_double)]


class rg_render_opts(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("samples", C.c_uint32),
                ("mode", C.c_uint32), ("ray_depth", C.c_uint32), ("ray_branching", C.c_uint32)]


class rg_device_opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("stream", C.c_void_p), ("form", C.c_uint32), ("flags", C.c_uint32)]


class rg_render_stats(C.Structure):
    _fields_ = [("duration_ms", C.c_double), ("kernel_ms", C.c_double), ("samples", C.c_uint64),
                ("rays", C.c_uint64), ("node_visits", C.c_uint64), ("prim_tests", C.c_uint64),
                ("sdf_steps", C.c_uint64), ("accum_frames", C.c_uint32), ("img_width", C.c_uint32),
                ("img_height", C.c_uint32), ("num_threads", C.c_uint32), ("error_flags", C.c_uint32),
                ("kernel_launches", C.c_uint32), ("traverse_ms", C.c_double), ("invalid_hits", C.c_uint64),
                ("invalid_mask", C.c_uint32), ("reserved0", C.c_uint32), ("hits", C.c_uint64),
                ("sdf_iterations", C.c_uint64)]


class rg_scene_info(C.Structure):
    _fields_ = [("n_prims", C.c_uint32), ("n_unbounded", C.c_uint32), ("n_nodes", C.c_uint32),
                ("max_depth", C.c_uint32), ("n_leaves", C.c_uint32), ("max_leaf_size", C.c_uint32),
                ("sah_cost", C.c_double), ("device_bytes", C.c_uint64), ("n_wide_nodes", C.c_uint32),
                ("wide_depth", C.c_uint32)]


class rg_tuning(C.Structure):
    _fields_ = [("wave_paths", C.c_uint32), ("sort_materials", C.c_uint32), ("bvh_width", C.c_uint32),
                ("fetch_budget", C.c_uint32), ("shared_stack", C.c_uint32), ("block", C.c_uint32),
                ("stack_limit", C.c_uint32), ("march_budget", C.c_uint32), ("shade_lanes", C.c_uint32),
                ("tail_paths", C.c_uint32), ("reserved", C.c_uint32)]


class rg_gradients(C.Structure):
    _fields_ = [("albedo", C.POINTER(C.c_float)), ("emission", C.POINTER(C.c_float)),
                ("density", C.POINTER(C.c_float)), ("loss", C.c_double)]


class rg_batch_tuning(C.Structure):
    _fields_ = [("block", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("rounds_per_item", C.c_uint32),
                ("bvh_width", C.c_uint32), ("form", C.c_uint32), ("wave_paths", C.c_uint32),
                ("shade_lanes", C.c_uint32), ("reserved", C.c_uint32)]


class rg_hit(C.Structure):
    _fields_ = [("hit", C.c_uint32), ("prim", C.c_uint32), ("t", C.c_float), ("normal", C.c_float * 3),
                ("ray_normal", C.c_float * 3), ("front_face", C.c_uint32), ("material", C.c_uint32),
                ("side", C.c_uint32)]


assert C.sizeof(rg_material) == 32
assert C.sizeof(rg_hit) == 48

# Every entry point declared in include/rayna_gpu.h, with its ctypes signature.
_P = C.c_void_p
_F = C.POINTER(C.c_float)
SIGNATURES = {
    "rg_abi_version": (C.c_uint32, []),
    "rg_create": (C.c_int, [C.POINTER(rg_device_opts), C.POINTER(_P)]),
    "rg_destroy": (C.c_int, [_P]),
    "rg_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "rg_inspect_scene": (C.c_int, [C.POINTER(rg_scene_desc), C.POINTER(rg_scene_info)]),
    "rg_set_scene": (C.c_int, [_P, C.POINTER(rg_scene_desc)]),
    "rg_set_tuning": (C.c_int, [_P, C.POINTER(rg_tuning)]),
    "rg_get_tuning": (C.c_int, [_P, C.POINTER(rg_tuning)]),
    "rg_set_camera": (C.c_int, [_P, C.POINTER(rg_camera)]),
    "rg_set_options": (C.c_int, [_P, C.POINTER(rg_render_opts)]),
    "rg_clear_accumulation": (C.c_int, [_P]),
    "rg_render": (C.c_int, [_P, C.c_uint64, _F, C.POINTER(rg_render_stats)]),
    "rg_render_async": (C.c_int, [_P, C.c_uint64, _P, C.POINTER(rg_render_stats)]),
    "rg_sync_stats": (C.c_int, [_P, C.POINTER(rg_render_stats)]),
    "rg_get_accumulation": (C.c_int, [_P, _F, C.POINTER(C.c_uint32)]),
    "rg_set_accumulation": (C.c_int, [_P, _F, C.c_uint32]),
    "rg_frame_moments": (C.c_int, [_P, _F, _F]),
    "rg_query_rays": (C.c_int, [_P, C.c_uint32, _F, _F, _F, _F, _F, C.POINTER(rg_hit)]),
    "rg_render_static_scratch": (C.c_int, [_P, C.c_uint64, _P, C.c_uint32, _P]),
    "rg_set_parameters": (C.c_int, [_P, _F, _F]),
    "rg_batch_create": (C.c_int, [C.POINTER(rg_device_opts), C.c_uint32, C.POINTER(C.POINTER(rg_scene_desc)),
                                  C.POINTER(rg_camera), C.POINTER(rg_render_opts), C.POINTER(_P)]),
    "rg_batch_destroy": (C.c_int, [_P]),
    "rg_batch_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "rg_batch_set_tuning": (C.c_int, [_P, C.c_void_p]),
    "rg_batch_render": (C.c_int, [_P, C.c_uint64, C.POINTER(rg_render_stats)]),
    "rg_batch_render_sequential": (C.c_int, [_P, C.c_uint64, C.POINTER(rg_render_stats)]),
    "rg_batch_image": (C.c_int, [_P, C.c_uint32, _F]),
    "rg_batch_item_seed": (C.c_uint64, [C.c_uint64, C.c_uint32]),
    "rg_backward": (C.c_int, [_P, C.c_uint64, _F, _F, C.POINTER(rg_gradients)]),
    "rg_backward_frame": (C.c_int, [_P, C.c_uint64, _F, C.POINTER(rg_gradients)]),
    "rg_set_sample_range": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
}

_libs = {}


def default_exact() -> bool:
    """Whether the arithmetic-contract build is the default (RAYNA_GB300_EXACT=1)."""
    return os.environ.get("RAYNA_GB300_EXACT", "0") not in ("", "0")


class RaynaError(RuntimeError):
    """A non-zero rg_status from the native library."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load_library(path: str | None = None, exact: bool | None = None) -> C.CDLL:
    """Loads the native library and binds every declared signature: the
    performance build, or the arithmetic-contract build with `exact` (default:
    RAYNA_GB300_EXACT), or the library at `path`."""
    if path is None:
        if exact is None:
            exact = default_exact()
        path = LIB_EXACT_PATH if exact else LIB_PATH
    lib = _libs.get(path)
    if lib is not None:
        return lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"native library {path} is missing; build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _libs[path] = lib
    return lib


def last_error(lib, handle) -> str:
    buf = C.create_string_buffer(1024)
    lib.rg_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(lib, handle, status: int) -> None:
    if status != RG_OK:
        raise RaynaError(status, last_error(lib, handle))
