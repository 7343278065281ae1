"""Parity on the benchmarked workloads at their full sizes, on the GPU.

The reduced scenes of test_gpu_render.py check every code path; these run
the three single-render workloads exactly as bench.py times them:

* random spheres: 488 spheres, 400x225, 32 spp, depth 50 (the whole frame);
* triangle mesh: the displaced icosphere of 1,310,720 triangles in the
  12-triangle Cornell box, 1024x1024, 64 spp, depth 8;
* SDF + media: the Mandelbulb and torus SDFs (256 steps, eps 1e-4), the
  sphere and box media and 100 spheres, 1280x720, 128 spp, depth 16.

The device renders whole frames; the CPU oracle renders windows of the same
frames (the same pixel coordinates and random streams) where the CPU cost of
the whole frame is too high: around the mesh's silhouette, into each SDF and
medium.

* Path by path: the arithmetic-contract build against the f32 oracle with
  the same frame key.
* Statistically: the performance build's per-pixel means against the
  faithful f64 oracle (the reference's samplers) within 3 standard errors
  (at most 1% of pixel channels beyond), relRMSE printed.
* relRMSE at the timed spp, against a 4096-spp device mean of the same
  camera, for every kernel form: the forms render bit-identical frames, so
  they reach equal image error at equal samples, and the Msamples/s ratio of
  the forms is their ratio at equal error. The test prints the relRMSE (with
  the 4096-spp mean's own noise subtracted) and the samples per pixel at
  which it would reach 1%.
"""
import functools

import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300 import Renderer, presets
from rayna_gb300.scene import flatten

pytestmark = pytest.mark.gpu


@functools.lru_cache(maxsize=None)
def workload(name):
    if name == "spheres":
        return presets.random_spheres(seed=0)
    if name == "mesh":
        return presets.cornell_mesh(level=8, seed=0)
    if name == "sdf":
        return presets.sdf_volumes(seed=0)
    raise ValueError(name)


@functools.lru_cache(maxsize=None)
def flat_of(name):
    return flatten(workload(name)[0])


def project(cam, opts, point):
    """Image coordinates (x, y) of a world point (Camera::calc_ray inverted)."""
    st, vp = ob.viewport(cam)
    assert st == 0
    pos, pc, vu, vv = vp[0], vp[1], vp[2], vp[3]
    a = np.stack([np.asarray(point, float) - pos, -vu, -vv], axis=1)
    s, u, v = np.linalg.solve(a, pc - pos)
    return u * opts.height + opts.width / 2, v * opts.height + opts.height / 2


def window_at(cam, opts, point, size):
    x, y = project(cam, opts, point)
    x0 = int(np.clip(round(x) - size // 2, 0, opts.width - size))
    y0 = int(np.clip(round(y) - size // 2, 0, opts.height - size))
    return (x0, y0, size, size)


# Windows of the mesh and SDF frames: (world point, size).
WINDOWS = {
    "mesh": [((0.5, 0.3, 0.5), 48), ((0.75, 0.3, 0.5), 48), ((0.5, 0.99, 0.5), 32)],
    "sdf": [((0.55, 1.25, 0.0), 40), ((3.8, 0.3, 0.8), 32), ((-2.6, 1.0, 0.6), 32), ((0.25, 0.05, 2.6), 32)],
}


def device_frames(name, frames, seed, exact=False, form="wavefront", window=None, windows=None):
    """Renders `frames` whole frames; returns (mean, per-sample variance, n)
    over the window (or a list of them over `windows`), from the per-frame
    moments."""
    scene, cam, opts = workload(name)
    wins = windows if windows is not None else [window or (0, 0, opts.width, opts.height)]
    spp = opts.samples
    s1 = [0.0] * len(wins)
    s2 = [0.0] * len(wins)
    with Renderer.new_from(scene, cam, opts, 0, seed=seed, exact=exact, form=form) as r:
        for _ in range(frames):
            out = r.render()
            assert out.stats.error_flags == 0
            fm_all, fv_all = r.frame_moments()
            for k, (x0, y0, ww, wh) in enumerate(wins):
                fm = fm_all[x0:x0 + ww, y0:y0 + wh].astype(np.float64)
                fv = fv_all[x0:x0 + ww, y0:y0 + wh].astype(np.float64)
                s1[k] = s1[k] + spp * fm
                s2[k] = s2[k] + (spp - 1) * fv + spp * fm ** 2
    n = frames * spp
    res = []
    for a, b in zip(s1, s2):
        mean = a / n
        res.append((mean, np.maximum(b / n - mean ** 2, 0.0) * n / (n - 1), n))
    return res if windows is not None else res[0]


def statistical(label, gm, gv, gn, om, ov, on):
    se = np.sqrt(gv / gn + ov / on)
    z = (gm - om) / np.maximum(se, 1e-6)
    beyond = float(np.mean(np.abs(z) > 3))
    rel_rmse = float(np.sqrt(np.mean((gm - om) ** 2)) / max(np.sqrt(np.mean(om ** 2)), 1e-12))
    print(f"{label}: {beyond:.4f} of pixel channels beyond 3 SE, relRMSE {rel_rmse:.4f}, mean z {np.mean(z):+.4f}")
    assert beyond <= 0.01, (label, beyond)
    se_img = np.sqrt(np.mean(gv / gn + ov / on) / gm.size) * 3  # neighbouring pixels are correlated: allow 3x
    assert abs(gm.mean() - om.mean()) <= 4 * se_img + 1e-6, (label, gm.mean(), om.mean(), se_img)


def test_spheres_full_frame_path_by_path():
    scene, cam, opts = workload("spheres")
    seed = 0xC0FFEE
    with Renderer.new_from(scene, cam, opts, 0, exact=True) as r:
        r.render(seed=seed)
        gm, _ = r.frame_moments()
    st, om, _, _ = ob.render(flat_of("spheres"), cam, opts, seed=seed, frames=1, policy=ob.POLICY_GPU_F32)
    assert st == 0
    frac = np.all(np.abs(gm - om) <= 1e-4 * (1 + np.abs(om)), axis=2).mean()
    print(f"random spheres 400x225x32: {frac:.4f} of pixels match the f32 oracle path for path")
    assert frac >= 0.97


def test_spheres_full_frame_statistical():
    scene, cam, opts = workload("spheres")
    gm, gv, gn = device_frames("spheres", 32, seed=21)
    st, om, ov, _ = ob.render(flat_of("spheres"), cam, opts, seed=23, frames=8, policy=ob.POLICY_REF_F64)
    assert st == 0
    statistical("random spheres 400x225 (whole frame)", gm, gv, gn, om, ov, 8 * opts.samples)


@pytest.mark.parametrize("name", ["mesh", "sdf"])
def test_full_workload_windows_path_by_path(name):
    scene, cam, opts = workload(name)
    seed = 0xBEEF + len(name)
    with Renderer.new_from(scene, cam, opts, 0, exact=True) as r:
        out = r.render(seed=seed)
        assert out.stats.error_flags == 0
        gm, _ = r.frame_moments()
    for k, (point, size) in enumerate(WINDOWS[name]):
        # The Mandelbulb window's paths bounce between the fuzzy metal fractal's
        # folds: a last-ulp difference of the host's and the device's sine and
        # cosine in the fuzz direction changes later marches (the distance
        # estimator itself is bit-exact on both sides)
        bar = 0.80 if (name, k) == ("sdf", 0) else {"mesh": 0.97, "sdf": 0.90}[name]
        win = window_at(cam, opts, point, size)
        st, om, _, _ = ob.render_window(flat_of(name), cam, opts, win, seed=seed, policy=ob.POLICY_GPU_F32)
        assert st == 0
        x0, y0, ww, wh = win
        g = gm[x0:x0 + ww, y0:y0 + wh]
        frac = np.all(np.abs(g - om) <= 1e-4 * (1 + np.abs(om)), axis=2).mean()
        print(f"{name} {opts.width}x{opts.height}x{opts.samples}, window {win}: {frac:.4f} of pixels match the f32 "
              f"oracle path for path")
        assert frac >= bar, (win, frac)


@pytest.mark.parametrize("name", ["mesh", "sdf"])
def test_full_workload_windows_statistical(name):
    """The mesh scene's paths reach its small light rarely (heavy-tailed
    samples): a mean of few samples tends to miss the rare bright ones and to
    underestimate its own variance, which biases z towards the side with more
    samples. Both sides therefore take the same 4096 spp per pixel there."""
    scene, cam, opts = workload(name)
    dev_frames, ora_frames = {"mesh": (64, 64), "sdf": (8, 4)}[name]
    wins = [window_at(cam, opts, point, size) for point, size in WINDOWS[name]]
    dev = device_frames(name, dev_frames, seed=40, windows=wins)
    for k, (win, (gm, gv, gn)) in enumerate(zip(wins, dev)):
        st, om, ov, _ = ob.render_window(flat_of(name), cam, opts, win, seed=60 + k, frames=ora_frames,
                                         policy=ob.POLICY_REF_F64)
        assert st == 0
        statistical(f"{name} window {win}", gm, gv, gn, om, ov, ora_frames * opts.samples)


FORMS = [("megakernel", None), ("wavefront", False), ("wavefront", True)]


@pytest.mark.parametrize("name", ["spheres", "mesh", "sdf"])
def test_relrmse_at_timed_spp_equal_across_forms(name):
    scene, cam, opts = workload(name)
    ref_frames = 4096 // opts.samples
    rm, rv, rn = device_frames(name, ref_frames, seed=777)
    rms = np.sqrt(np.mean(rm ** 2))
    ref_noise = np.mean(rv / rn)  # the 4096-spp mean's own variance, per channel on average
    print(f"{name}: 4096-spp reference mean, its own relRMSE {np.sqrt(ref_noise) / rms:.4f}")
    imgs = {}
    for form, sort in FORMS:
        with Renderer.new_from(scene, cam, opts, 0, form=form) as r:
            if sort is not None:
                r.set_tuning(sort_materials=sort)
            out = r.render(seed=991)
            assert out.stats.error_flags == 0
            imgs[(form, sort)] = out.img.astype(np.float64)
    base = imgs[FORMS[0]]
    for key, img in imgs.items():
        np.testing.assert_array_equal(img, base, err_msg=f"{name}: form {key} differs from the megakernel")
    mse = np.mean((base - rm) ** 2)
    rel = np.sqrt(mse) / rms
    rel_corr = np.sqrt(max(mse - ref_noise, 0.0)) / rms
    spp_1pc = opts.samples * (rel_corr / 0.01) ** 2
    print(f"{name} {opts.width}x{opts.height}x{opts.samples}: every form's frame is the same image; relRMSE against "
          f"the 4096-spp mean {rel:.4f} ({rel_corr:.4f} with the mean's own noise removed); 1% relRMSE at about "
          f"{spp_1pc:.0f} spp")
    assert rel_corr < 1.0
