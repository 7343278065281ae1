"""The device against closed-form answers of the reference's rules
(tests/known_answers.py), in both arithmetic builds, through the C ABI:
dielectric energy conservation, Beer attenuation on a known chord,
free-flight transmission of a medium, mirror reflection of the sky, sphere
tracing of an exact SDF, Moller-Trumbore's barycentric normal and face
conventions."""
import numpy as np
import pytest

from rayna_gb300 import Renderer
from rayna_gb300.scene import Camera, RenderOpts

import known_answers as K

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("name", list(K.RENDER_CASES))
def test_render_known_answers(name, exact):
    scene, cam, _ = K.RENDER_CASES[name]()
    opts = RenderOpts(width=8, height=8, samples=4096, ray_depth=50)
    with Renderer.new_from(scene, cam, opts, 0, exact=exact, seed=9) as r:
        out = r.render()
        mean, var = r.frame_moments()
    assert out.stats.error_flags == 0
    m, expect, se = K.check_render(name, mean.astype(np.float64), var.astype(np.float64), opts.samples)
    print(f"{name} ({'exact' if exact else 'performance'} build): {m} vs {expect} (SE {se})")


@pytest.mark.parametrize("exact", [True, False])
def test_sdf_sphere_known_answers(exact):
    eps = 1e-4
    scene = K.sdf_sphere_scene(eps)
    o, d, t, n = K.sdf_sphere_rays()
    with Renderer.new_from(scene, Camera(), RenderOpts(width=8, height=8), exact=exact) as r:
        hits = r.query_rays(o, d)
    dt, ne = K.check_sdf_sphere(hits, t, n, d, eps, 5e-3)
    print(f"sdf sphere: max |t - t*| {dt:.2e}, max normal error {ne:.2e}")


@pytest.mark.parametrize("exact", [True, False])
def test_triangle_known_answers(exact):
    scene, o, d, t, n_int, front, ray_n = K.triangle_case()
    with Renderer.new_from(scene, Camera(), RenderOpts(width=8, height=8), exact=exact) as r:
        hits = r.query_rays(o, d)
    K.check_triangle(hits, t, n_int, front, ray_n, 2e-4)
