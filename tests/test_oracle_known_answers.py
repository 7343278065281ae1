"""The CPU oracle against closed-form answers of the reference's rules
(tests/known_answers.py): dielectric energy conservation, Beer attenuation
on a known chord, free-flight transmission of a medium, mirror reflection of
the sky, sphere tracing of an exact SDF, Moller-Trumbore's barycentric normal
and face conventions. Both oracle policies: the faithful f64 one with the
reference's samplers, and the f32 one with the device's."""
import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300.scene import flatten

import known_answers as K


@pytest.mark.parametrize("policy", [ob.POLICY_REF_F64, ob.POLICY_GPU_F32])
@pytest.mark.parametrize("name", list(K.RENDER_CASES))
def test_render_known_answers(name, policy):
    scene, cam, _ = K.RENDER_CASES[name]()
    opts = K.RENDER_OPTS
    st, mean, var, _ = ob.render(flatten(scene), cam, opts, seed=5, frames=2, policy=policy)
    assert st == 0
    m, expect, se = K.check_render(name, mean, var, 2 * opts.samples)
    print(f"{name} (policy {policy}): {m} vs {expect} (SE {se})")


@pytest.mark.parametrize("policy,normal_tol", [(ob.POLICY_REF_F64, 1e-6), (ob.POLICY_GPU_F32, 5e-3)])
def test_sdf_sphere_known_answers(policy, normal_tol):
    eps = 1e-4
    scene = K.sdf_sphere_scene(eps)
    o, d, t, n = K.sdf_sphere_rays()
    hits, _, _ = ob.query(flatten(scene), o, d, policy=policy, pretest=False)
    dt, ne = K.check_sdf_sphere(hits, t, n, d, eps, normal_tol)
    print(f"sdf sphere (policy {policy}): max |t - t*| {dt:.2e}, max normal error {ne:.2e}")


@pytest.mark.parametrize("policy,rtol", [(ob.POLICY_REF_F64, 1e-7), (ob.POLICY_GPU_F32, 2e-4)])
def test_triangle_known_answers(policy, rtol):
    scene, o, d, t, n_int, front, ray_n = K.triangle_case()
    hits, t64, n64 = ob.query(flatten(scene), o, d, policy=policy, pretest=False)
    if policy == ob.POLICY_REF_F64:
        K.check_triangle(hits, t, n_int, front, ray_n, rtol, t_hits=t64, n_hits=n64)
    else:
        K.check_triangle(hits, t, n_int, front, ray_n, rtol)


def test_ln_f32_within_three_ulp():
    """The logarithm the f32 policy and the device share (the atanh series of
    Abramowitz & Stegun 4.1.27): within 3 ulp of the exact value over normal
    and subnormal arguments, and the IEEE special cases."""
    rng = np.random.Generator(np.random.PCG64(1))
    x = np.concatenate([
        rng.uniform(0, 1, 200000).astype(np.float32),
        np.exp(rng.uniform(-87, 88, 200000)).astype(np.float32),
        np.float32(2.0) ** np.arange(-149, 128, dtype=np.float64).astype(np.float32),
        np.nextafter(np.float32(1.0), np.float32(2.0)) + np.zeros(1, np.float32),
        np.array([1.0, 0.5, 2.0, 1.4142135, 1.4142137, 0.70710677], np.float32),
    ])
    x = x[x > 0]
    got = ob.ln_f32(x).astype(np.float64)
    exact = np.log(x.astype(np.float64))
    ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
    err = np.abs(got - exact) / np.maximum(ulp, np.finfo(np.float32).tiny)
    assert err.max() <= 3.0, (err.max(), x[np.argmax(err)])
    assert ob.ln_f32([1.0])[0] == 0.0
    sp = ob.ln_f32([0.0, -1.0, np.inf, np.nan])
    assert sp[0] == -np.inf and np.isnan(sp[1]) and sp[2] == np.inf and np.isnan(sp[3])
