"""Autotuner keys and cache (CPU), and a measured tuning pass (GPU)."""
import json

import pytest

from rayna_gb300 import autotune, presets
from rayna_gb300.scene import RenderOpts


def test_keys_bucket_by_size():
    assert autotune.render_key(1_310_732, 1024, 1024, 64) == "render:p20:r20:s6"
    assert autotune.render_key(488, 400, 225, 32) == "render:p8:r16:s5"
    assert autotune.batch_key(64, 2_700_000, 52_000_000, 2_000_000_000).startswith("batch:n6:")


def test_wavefront_axes_cover_the_launch_knobs():
    axes = dict(autotune.WAVE_AXES)
    assert axes["shade_lanes"] == autotune.SHADE_LANES and 16 in autotune.SHADE_LANES
    assert axes["tail_paths"] == autotune.TAIL_PATHS and 1 in autotune.TAIL_PATHS  # 1: no continuation
    assert axes["wave_paths"][-1] == 1 << 27
    assert dict(autotune.WAVE_SDF_AXES)["march_budget"] == autotune.MARCH_BUDGETS


def test_default_cache_is_outside_the_package():
    import os
    pkg = os.path.dirname(os.path.abspath(autotune.__file__))
    assert not os.path.abspath(autotune.DEFAULT_CACHE).startswith(pkg)


def test_cache_round_trip(tmp_path):
    path = tmp_path / "tune.json"
    t = autotune.Tuner(str(path))
    assert t.lookup("render:p1:r2:s3") is None
    t.store("render:p1:r2:s3", {"form": "wavefront", "wave_paths": 1 << 22}, [{"ms": 1.0}])
    t2 = autotune.Tuner(str(path))
    assert t2.lookup("render:p1:r2:s3") == {"form": "wavefront", "wave_paths": 1 << 22}
    assert json.loads(path.read_text())["render:p1:r2:s3"]["timings"] == [{"ms": 1.0}]


@pytest.mark.gpu
def test_tuning_pass_picks_a_measured_candidate(tmp_path):
    from rayna_gb300 import Renderer
    from rayna_gb300.batch import BatchRenderer
    t = autotune.Tuner(str(tmp_path / "tune.json"))
    scene, cam, _ = presets.random_spheres(seed=0)
    opts = RenderOpts(width=64, height=36, samples=8, ray_depth=8)
    cfg = t.tune_render(scene, cam, opts, frames=1)
    assert cfg["form"] in ("megakernel", "wavefront")
    entry = t.table[autotune.render_key(488, 64, 36, 8)]
    assert len(entry["timings"]) >= 2 and all(x["ms"] > 0 for x in entry["timings"])
    # the stack placement and the megakernel's block size were searched
    mega = [x for x in entry["timings"] if x["form"] == "megakernel"]
    assert {x["block"] for x in mega} == set(autotune.MEGA_BLOCKS)
    assert {x["shared_stack"] for x in mega} == set(autotune.SHARED_STACKS)
    wave = [x for x in entry["timings"] if x["form"] == "wavefront"]
    assert {x["shade_lanes"] for x in wave} == set(autotune.SHADE_LANES)
    with Renderer.tuned(scene, cam, opts, tuner=t) as r:
        assert r.form == cfg["form"]
        r.render()
    with BatchRenderer(presets.batch_scenes(n=4, seed=2, scale=0.05, max_tris=5000)) as b:
        bcfg = t.tune_batch(b)
        assert bcfg["form"] in ("wavefront", "tiles")
        b.render(seed=3)
