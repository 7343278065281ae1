"""Closed-form answers of the reference's render and intersection rules, for
pinning the oracle (test_oracle_known_answers.py) and the device
(test_gpu_known_answers.py) to something other than each other.

Each case is derived from the reference's formulas on a scene whose answer
can be written down:

* glass_furnace: a clear dielectric sphere (albedo 1, density 0) under
  WhiteSkybox. Refraction and Schlick reflection only redirect paths and the
  exit factor albedo * exp(-density * chord) is 1 (material/dielectric.rs:
  19-79), so every escaping path carries exactly 1.
* beer_chord: a dielectric sphere of radius 1 with albedo a and density rho,
  seen along its diameter under WhiteSkybox. A path reflects at entry with
  Schlick's R0 = ((1 - ior) / (1 + ior))^2, else it crosses the diameter and,
  at each inner hit (front_face false), is multiplied by T = a exp(-rho * 2)
  and leaves with 1 - R0 or reflects back with R0:
  V = R0 + (1 - R0) T (1 - R0) / (1 - R0 T).
* medium_transmission: a constant-density sphere medium (object/volumetric.rs:
  86-160) of radius 1 and density rho with a black isotropic material, seen
  along its diameter under WhiteSkybox: only paths that cross without a
  free-flight event reach the sky, V = exp(-2 rho).
* mirror_sky: a fuzz-0 metal sphere under SimpleSkybox hit at a chosen
  point: the colour is albedo x sky(reflect(d, n)) (material/metal.rs:17-45,
  skybox/simple.rs:12-30).
* sdf_sphere: sphere tracing an exact sphere SDF (mesh/isosurface/
  raymarched.rs:73-122) stops within epsilon of the analytic distance; the
  normal is the gradient (the outward radius), and the ray normal is the
  normal itself, not flipped, also for rays from inside.
* triangle: Moller-Trumbore's barycentrics of a chosen point, the normal
  interpolated from distinct vertex normals and normalised, front_face =
  det < 0 and ray_normal = normal * -sign(det) (mesh/primitive/triangle.rs:
  53-119).
"""
import math

import numpy as np

from rayna_gb300.scene import (
    Angle, Camera, DielectricMaterial, IsotropicMaterial, LambertianMaterial, MetalMaterial, RaymarchedIsosurfaceMesh,
    RenderOpts, Scene, SdfSphere, SimpleObject, SimpleSkybox, SphereMesh, Triangle, VolumetricObject, WhiteSkybox,
)

IOR = 1.5
R0 = ((1.0 - IOR) / (1.0 + IOR)) ** 2


def narrow_camera(target=(0.0, 0.0, 0.0), pos=(0.0, 0.0, -20.0)):
    """A pinhole 20 units away with a 0.002 degree field: every pixel's rays
    lie within 4e-5 radians of the line to `target` (within 7e-4 units of it
    at the unit sphere, so a mirror's reflected direction stays within 1.4e-3
    radians of the analytic one)."""
    fwd = tuple(np.asarray(target, float) - np.asarray(pos, float))
    return Camera(pos=pos, fwd=fwd, v_fov=Angle.from_degrees(0.002), focus_dist=20.0,
                  defocus_angle=Angle.from_degrees(0.0))


def glass_furnace():
    scene = Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), DielectricMaterial((1, 1, 1), IOR, 0.0))],
                  skybox=WhiteSkybox())
    cam = Camera(pos=(0.0, 0.0, -2.7), v_fov=Angle.from_degrees(45.0), fwd=(0.0, 0.0, 1.0), focus_dist=1.0,
                 defocus_angle=Angle.from_degrees(0.0))
    return scene, cam, np.ones(3)


def beer_chord(albedo=(0.9, 0.7, 0.5), rho=0.3):
    scene = Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), DielectricMaterial(albedo, IOR, rho))],
                  skybox=WhiteSkybox())
    t = np.asarray(albedo) * math.exp(-rho * 2.0)
    v = R0 + (1 - R0) * t * (1 - R0) / (1 - R0 * t)
    return scene, narrow_camera(), v


def medium_transmission(rho=0.5):
    scene = Scene(objects=[VolumetricObject(SphereMesh((0, 0, 0), 1.0), IsotropicMaterial((0, 0, 0), 0.0), rho)],
                  skybox=WhiteSkybox())
    return scene, narrow_camera(), np.full(3, math.exp(-2.0 * rho))


def mirror_sky(albedo=(0.9, 0.8, 0.6), polar_deg=35.0, azim_deg=20.0):
    """The sphere point seen at (polar, azimuth) from the -z pole."""
    th, ph = math.radians(polar_deg), math.radians(azim_deg)
    n = np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), -math.cos(th)])
    pos = np.array([0.0, 0.0, -20.0])
    scene = Scene(objects=[SimpleObject(SphereMesh((0, 0, 0), 1.0), MetalMaterial(albedo, 0.0))], skybox=SimpleSkybox())
    d = n - pos
    d /= np.linalg.norm(d)
    refl = d - 2 * np.dot(d, n) * n
    a = 0.5 * refl[1] + 0.5
    sky = (1 - a) * np.ones(3) + a * np.array([0.5, 0.7, 1.0])
    return scene, narrow_camera(target=tuple(n), pos=tuple(pos)), np.asarray(albedo) * sky


RENDER_CASES = {
    "glass_furnace": glass_furnace,
    "beer_chord": beer_chord,
    "medium_transmission": medium_transmission,
    "mirror_sky": mirror_sky,
}
RENDER_OPTS = RenderOpts(width=4, height=4, samples=1024, ray_depth=50)


def check_render(name, mean, var, n):
    """Asserts the rendered mean against the case's answer: within 4 standard
    errors of the whole window's mean (plus the narrow camera's 1e-4 spread),
    and per pixel for the deterministic cases."""
    _, _, expect = RENDER_CASES[name]()
    expect = np.asarray(expect, float)
    m = mean.reshape(-1, 3).mean(axis=0)
    se = np.sqrt(var.reshape(-1, 3).mean(axis=0) / (n * mean.shape[0] * mean.shape[1]))
    assert np.all(np.abs(m - expect) <= 4 * se + 1e-4 + 1e-4 * expect), (name, m, expect, se)
    if name in ("glass_furnace", "mirror_sky"):
        np.testing.assert_allclose(mean.reshape(-1, 3), np.broadcast_to(expect, (mean.size // 3, 3)),
                                   rtol=1e-3 if name == "mirror_sky" else 1e-6, atol=1e-6)
    return m, expect, se


def sdf_sphere_scene(eps=1e-4):
    return Scene(objects=[SimpleObject(RaymarchedIsosurfaceMesh(SdfSphere((0.5, -0.25, 0.3), 1.0), 256, eps),
                                       LambertianMaterial((0.5, 0.5, 0.5)))])


def sdf_sphere_rays(n=2000, seed=3):
    """Rays from outside aimed at points of the sphere's front half, and rays
    from inside in random directions; returns (origins, dirs, t_true, n_true)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = np.array([0.5, -0.25, 0.3])
    k = n // 2
    u = rng.normal(size=(k, 3)); u /= np.linalg.norm(u, axis=1, keepdims=True)
    o_out = c + u * rng.uniform(2.0, 6.0, (k, 1))
    tgt = rng.normal(size=(k, 3)); tgt /= np.linalg.norm(tgt, axis=1, keepdims=True)
    tgt = np.where(np.einsum("ij,ij->i", tgt, u)[:, None] < 0.2, -tgt, tgt)  # the half facing the origin
    p_out = c + tgt
    d_out = p_out - o_out
    o_in = c + rng.uniform(-0.4, 0.4, (n - k, 3))
    d_in = rng.normal(size=(n - k, 3))
    o = np.vstack([o_out, o_in]).astype(np.float32).astype(np.float64)  # the rays as given, in f32
    d = np.vstack([d_out, d_in]).astype(np.float32).astype(np.float64)
    dn = d / np.linalg.norm(d, axis=1, keepdims=True)
    oc = o - c
    b = np.einsum("ij,ij->i", oc, dn)
    cc = np.einsum("ij,ij->i", oc, oc) - 1.0
    sq = np.sqrt(np.maximum(b * b - cc, 0.0))
    t = np.where(cc > 0, -b - sq, -b + sq)
    p = o + dn * t[:, None]
    return o.astype(np.float32), d.astype(np.float32), t, p - c


def check_sdf_sphere(hits, t_true, n_true, dirs, eps, normal_tol):
    """The march stops once an evaluation is below epsilon, which leaves the
    point within about epsilon of the surface: within epsilon / cos(incidence)
    along the ray, so the distance is held to that, and the normal (the
    outward radius at the point) to the point's offset plus `normal_tol`."""
    assert np.all(hits["hit"] == 1)
    dn = dirs.astype(np.float64) / np.linalg.norm(dirs, axis=1, keepdims=True)
    cos = np.maximum(np.abs(np.einsum("ij,ij->i", dn, n_true)), 1e-3)
    dt = np.abs(hits["t"].astype(np.float64) - t_true)
    tol_t = 2 * eps / cos + 1e-6 * np.abs(t_true)
    assert np.all(dt <= tol_t), (dt / tol_t).max()
    nerr = np.abs(hits["normal"].astype(np.float64) - n_true).max(axis=1)
    assert np.all(nerr <= normal_tol + dt), (nerr - dt).max()
    # the ray normal is the normal itself (raymarched.rs:113-114), even from inside
    np.testing.assert_array_equal(hits["ray_normal"], hits["normal"])
    return dt.max(), nerr.max()


def triangle_case():
    v = np.array([[0.0, 0.0, 0.0], [2.0, 0.2, 0.1], [0.3, 1.7, -0.2]])
    nrm = np.array([[0.0, 0.0, 1.0], [0.6, 0.0, 0.8], [0.0, 0.28, 0.96]])
    scene = Scene(objects=[SimpleObject(Triangle(v, nrm), LambertianMaterial((0.5, 0.5, 0.5)))])
    rng = np.random.Generator(np.random.PCG64(11))
    m = 4000
    uv = rng.uniform(0.02, 0.98, (m, 2))
    uv = np.where(uv.sum(axis=1, keepdims=True) < 0.96, uv, 0.5 * uv)
    p = v[0] + uv[:, :1] * (v[1] - v[0]) + uv[:, 1:] * (v[2] - v[0])
    side = np.where(rng.random(m) < 0.5, 1.0, -1.0)[:, None]
    o = p + side * rng.uniform(0.5, 3.0, (m, 1)) * np.array([0.1, -0.2, 1.0]) + rng.normal(scale=0.2, size=(m, 3))
    d = p - o
    # the exact intersection of the f32 ray as given: o + t d = v0 + u e1 + v e2, solved in f64
    o = o.astype(np.float32).astype(np.float64)
    d = d.astype(np.float32).astype(np.float64)
    dn = d / np.linalg.norm(d, axis=1, keepdims=True)
    e1, e2 = v[1] - v[0], v[2] - v[0]
    a_mat = np.stack([np.broadcast_to(e1, dn.shape), np.broadcast_to(e2, dn.shape), -dn], axis=2)
    sol = np.linalg.solve(a_mat, (o - v[0])[:, :, None])[:, :, 0]
    uv, t = sol[:, :2], sol[:, 2]
    n_int = (1 - uv.sum(axis=1, keepdims=True)) * nrm[0] + uv[:, :1] * nrm[1] + uv[:, 1:] * nrm[2]
    n_int /= np.linalg.norm(n_int, axis=1, keepdims=True)
    det = np.einsum("j,ij->i", e1, np.cross(dn, e2))
    front = det < 0
    ray_n = n_int * (-np.sign(det))[:, None]
    return scene, o.astype(np.float32), d.astype(np.float32), t, n_int, front, ray_n


def check_triangle(hits, t, n_int, front, ray_n, rtol, t_hits=None, n_hits=None):
    """`t_hits`, `n_hits`: the distance and normal at full precision where the
    caller has them (the f64 oracle), else the f32 hit record's."""
    assert np.all(hits["hit"] == 1)
    np.testing.assert_allclose(hits["t"] if t_hits is None else t_hits, t, rtol=rtol)
    np.testing.assert_allclose(hits["normal"] if n_hits is None else n_hits, n_int, atol=rtol * 10)
    np.testing.assert_allclose(hits["ray_normal"], ray_n, atol=max(rtol * 10, 1e-6))
    np.testing.assert_array_equal(hits["front_face"] == 1, front)
