"""The batched forms through the C ABI: the batched wavefront and the
persistent tile launch (each replayed as a CUDA graph) render the same images
as one megakernel launch per scene, and as standalone renderers given the
same frame keys."""
import numpy as np
import pytest

from rayna_gb300 import Renderer, presets
from rayna_gb300.batch import BatchRenderer

pytestmark = pytest.mark.gpu


def small_batch():
    return presets.batch_scenes(n=7, seed=3, scale=0.08, max_tris=20_000)


@pytest.mark.parametrize("exact", [True, False])
def test_batch_equals_sequential_and_standalone(exact):
    items = small_batch()
    seeds = [11, 12]
    with BatchRenderer(items, exact=exact) as b:
        for s in seeds:
            st = b.render(seed=s)
            assert st.error_flags == 0
            assert st.samples == b.n_samples
        graph_imgs = [b.image(i) for i in range(len(items))]
        keys = [[b.item_seed(s, i) for s in seeds] for i in range(len(items))]
    with BatchRenderer(items, exact=exact) as b:
        for s in seeds:
            b.render_sequential(seed=s)
        seq_imgs = [b.image(i) for i in range(len(items))]
    for i, (scene, cam, opts) in enumerate(items):
        np.testing.assert_array_equal(graph_imgs[i], seq_imgs[i])
        with Renderer.new_from(scene, cam, opts, 0, exact=exact) as r:
            for k in keys[i]:
                img = r.render(seed=k).img
        np.testing.assert_array_equal(graph_imgs[i], img)


def test_batch_tuning_does_not_change_images():
    items = small_batch()[:4]
    imgs = []
    # tiles in three shapes; the wavefront with waves small enough that renders
    # are cut into runs spanning several waves, on either tree
    for tune in [dict(), dict(form="tiles"), dict(form="tiles", block=128, rounds_per_item=1),
                 dict(form="tiles", block=64, blocks_per_sm=1, rounds_per_item=16),
                 dict(wave_paths=50_000), dict(wave_paths=50_000, bvh_width=8),
                 dict(shade_lanes=1), dict(wave_paths=50_000, shade_lanes=32)]:
        with BatchRenderer(items) as b:
            b.set_tuning(**tune)
            b.render(seed=5)
            b.render(seed=6)
            imgs.append([b.image(i) for i in range(len(items))])
    for other in imgs[1:]:
        for a, c in zip(imgs[0], other):
            np.testing.assert_array_equal(a, c)


def test_batch_rejects_launch_shapes_it_cannot_run():
    from rayna_gb300._abi import RaynaError
    with BatchRenderer(small_batch()[:2]) as b:
        with pytest.raises(RaynaError) as e:
            b.set_tuning(block=1024)
        assert e.value.status == 1
        with pytest.raises(RaynaError) as e:
            b.set_tuning(shade_lanes=33)
        assert e.value.status == 1
        try:  # 512 threads fit only if the kernel uses <= 128 registers
            b.set_tuning(block=512)
        except RaynaError as err:
            assert err.status == 1 and "threads per block" in str(err)
        else:
            b.render(seed=1)


def test_batch_with_transformed_objects():
    """The reference's Cornell preset (rotated boxes) in both batched forms
    renders what a standalone renderer renders with the same frame keys."""
    from rayna_gb300.scene import RenderOpts
    scene, cam, _ = presets.cornell()
    items = [(scene, cam, RenderOpts(width=40, height=32, samples=8, ray_depth=6))] + small_batch()[:2]
    for form in ("wavefront", "tiles"):
        with BatchRenderer(items) as b:
            b.set_tuning(form=form)
            st = b.render(seed=21)
            assert st.error_flags == 0
            img = b.image(0)
            key = b.item_seed(21, 0)
        with Renderer.new_from(scene, cam, items[0][2], 0) as r:
            ref = r.render(seed=key).img
        np.testing.assert_array_equal(img, ref)


def test_batch_with_textures_and_image_sky():
    """A textured scene under an image sky in both batched forms renders what
    a standalone renderer renders with the same frame keys."""
    from rayna_gb300.scene import RenderOpts
    scene, cam, _ = presets.textures_demo()
    items = [(scene, cam, RenderOpts(width=48, height=27, samples=8, ray_depth=6))] + small_batch()[:2]
    for form in ("wavefront", "tiles"):
        with BatchRenderer(items) as b:
            b.set_tuning(form=form)
            st = b.render(seed=23)
            assert st.error_flags == 0
            img = b.image(0)
            key = b.item_seed(23, 0)
        with Renderer.new_from(scene, cam, items[0][2], 0) as r:
            ref = r.render(seed=key).img
        np.testing.assert_array_equal(img, ref)
