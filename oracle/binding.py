"""ctypes binding of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
the checker. The rayna_gb300 package never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from rayna_gb300 import _abi as A
from rayna_gb300.renderer import HIT_DTYPE

from . import build as _build

POLICY_REF_F64 = 0
POLICY_GPU_F32 = 1

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        fp, dp, up = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_uint32)
        L.orc_philox.argtypes = [up, up, up]
        L.orc_viewport.argtypes = [C.POINTER(A.rg_camera), dp]
        L.orc_viewport.restype = C.c_int
        L.orc_query.argtypes = [C.POINTER(A.rg_scene_desc), C.c_int, C.c_int, C.c_uint32, fp, fp, fp, fp, fp,
                                C.POINTER(A.rg_hit), dp, dp]
        L.orc_query.restype = C.c_int
        L.orc_render.argtypes = [C.POINTER(A.rg_scene_desc), C.POINTER(A.rg_camera), C.POINTER(A.rg_render_opts),
                                 C.c_uint64, C.c_uint32, C.c_int, C.c_int, C.c_int, dp, dp, dp]
        L.orc_render.restype = C.c_int
        L.orc_render_window.argtypes = [C.POINTER(A.rg_scene_desc), C.POINTER(A.rg_camera),
                                        C.POINTER(A.rg_render_opts), C.c_uint64, C.c_uint32, C.c_int, C.c_int, C.c_int,
                                        C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                        dp, dp, dp]
        L.orc_render_window.restype = C.c_int
        L.orc_hardware_threads.restype = C.c_int
        L.orc_query_colour.argtypes = [C.POINTER(A.rg_scene_desc), C.c_int, C.c_uint32, fp, fp, fp]
        L.orc_query_colour.restype = C.c_int
        _lib = L
    return _lib


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def viewport(camera):
    out = (C.c_double * 18)()
    st = lib().orc_viewport(C.byref(camera.to_c()), out)
    return st, np.array(out).reshape(6, 3)


STRUCT_NO_PRETEST = 0
STRUCT_REFERENCE = 1
STRUCT_BRUTE_FORCE = 2


def query(flat, origins, dirs, tmin=1e-3, tmax=3.4028235e38, volume_u=None, policy=POLICY_GPU_F32, pretest=True):
    """Closest hits from the oracle. Returns (hits structured array, t64, n64).

    `pretest`: True = the reference's BVH with its per-object box test,
    False = the same BVH without it, "brute" = no bounding volumes."""
    o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    n = o.shape[0]
    t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(tmin, np.float32), (n,)))
    t1 = np.ascontiguousarray(np.broadcast_to(np.asarray(tmax, np.float32), (n,)))
    out = (A.rg_hit * max(n, 1))()
    t64 = np.zeros(n)
    n64 = np.zeros((n, 3))
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    vu = None
    if volume_u is not None:
        vu_arr = np.ascontiguousarray(volume_u, np.float32)
        vu = fp(vu_arr)
    structure = STRUCT_BRUTE_FORCE if pretest == "brute" else (STRUCT_REFERENCE if pretest else STRUCT_NO_PRETEST)
    st = lib().orc_query(C.byref(flat.desc), policy, structure, n, fp(o), fp(d), fp(t0), fp(t1), vu, out,
                         t64.ctypes.data_as(C.POINTER(C.c_double)), n64.ctypes.data_as(C.POINTER(C.c_double)))
    assert st == 0
    hits = np.frombuffer(out, dtype=HIT_DTYPE, count=n).copy()
    return hits, t64, n64


def query_colour(flat, origins, dirs, policy=POLICY_REF_F64):
    """The colour each ray sees at its closest hit (the material's texture
    value or albedo, a light's emission) or the sky on a miss; (n, 3)."""
    o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros((o.shape[0], 3), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    assert lib().orc_query_colour(C.byref(flat.desc), policy, o.shape[0], fp(o), fp(d), fp(out)) == 0
    return out


def render(flat, camera, opts, seed=0, frames=1, policy=POLICY_REF_F64, gpu_sampling=False, threads=0):
    """Renders with the oracle. Returns (status, mean (w,h,3), var (w,h,3), seconds)."""
    w, h = opts.width, opts.height
    mean = np.zeros((w, h, 3))
    var = np.zeros((w, h, 3))
    secs = C.c_double(0.0)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    st = lib().orc_render(C.byref(flat.desc), C.byref(camera.to_c()), C.byref(opts.to_c()), int(seed), int(frames),
                          int(policy), 1 if gpu_sampling else 0, int(threads), dp(mean), dp(var), C.byref(secs))
    return st, mean, var, secs.value


def render_window(flat, camera, opts, window, seed=0, frames=1, policy=POLICY_REF_F64, gpu_sampling=False,
                  threads=0, samples=None):
    """Renders the pixels window = (x0, y0, w, h) of the full frame (the
    frame's own pixel coordinates and random streams) and, with `samples` =
    (first, count), only those samples of each pixel. Returns (status, mean
    (w,h,3), var (w,h,3), seconds) over the traced samples."""
    x0, y0, ww, wh = (int(v) for v in window)
    s0, ns = (0, 0) if samples is None else (int(samples[0]), int(samples[1]))
    mean = np.zeros((ww, wh, 3))
    var = np.zeros((ww, wh, 3))
    secs = C.c_double(0.0)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    st = lib().orc_render_window(C.byref(flat.desc), C.byref(camera.to_c()), C.byref(opts.to_c()), int(seed),
                                 int(frames), int(policy), 1 if gpu_sampling else 0, int(threads), x0, y0, ww, wh, s0,
                                 ns, dp(mean), dp(var), C.byref(secs))
    return st, mean, var, secs.value


def ln_f32(x) -> np.ndarray:
    """The f32 natural logarithm the f32 policy and the device share."""
    L = lib()
    if not hasattr(L, "_ln_bound"):
        L.orc_ln_f32.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32]
        L.orc_ln_f32.restype = None
        L._ln_bound = True
    a = np.ascontiguousarray(x, np.float32).ravel()
    out = np.empty_like(a)
    fp = lambda v: v.ctypes.data_as(C.POINTER(C.c_float))
    L.orc_ln_f32(fp(a), fp(out), a.size)
    return out


def hardware_threads() -> int:
    return int(lib().orc_hardware_threads())


def backward(flat, camera, opts, seed, target=None, adjoint=None, policy=POLICY_REF_F64, threads=0):
    """Path-replay adjoint on the CPU. Returns dict(loss, albedo, emission, density)."""
    L = lib()
    if not hasattr(L, "_bw_bound"):
        fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
        L.orc_backward.argtypes = [C.POINTER(A.rg_scene_desc), C.POINTER(A.rg_camera), C.POINTER(A.rg_render_opts),
                                   C.c_uint64, C.c_int, C.c_int, fp, fp, dp, dp, dp, dp]
        L.orc_backward.restype = C.c_int
        L._bw_bound = True
    nm, nv = flat.desc.n_materials, flat.desc.n_volumes
    ga, ge, gd = np.zeros(nm * 3), np.zeros(nm * 3), np.zeros(max(nv, 1))
    loss = C.c_double(0.0)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    t = np.ascontiguousarray(target, np.float32) if target is not None else None
    a = np.ascontiguousarray(adjoint, np.float32) if adjoint is not None else None
    st = L.orc_backward(C.byref(flat.desc), C.byref(camera.to_c()), C.byref(opts.to_c()), int(seed), int(policy),
                        int(threads), fp(t), fp(a), dp(ga), dp(ge), dp(gd), C.byref(loss))
    assert st == 0, st
    return {"loss": loss.value, "albedo": ga.reshape(nm, 3), "emission": ge.reshape(nm, 3), "density": gd[:nv]}


def set_albedo(flat, m, c, value):
    """Sets one albedo channel of material m in a flattened scene (in place)."""
    flat.c_materials[m].albedo[c] = value


def set_density(flat, v, value):
    flat.c_volumes[v].density = value
