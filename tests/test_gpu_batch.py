"""Multi-scene batches (lg_batch_upload / lg_batch_render) on the GPU.

Bar: every scene's RGBA16F image from the batch is bit-identical to lg_render of that scene
alone (fixed-point accumulation makes the result independent of which other rays share the
wavefront), and the batch's statistics are the sums of the scenes' own.
"""
import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W

pytestmark = pytest.mark.gpu


def _alone(packed):
    from light_garden_gb300.runtime import Context
    with Context() as c:
        c.upload(packed)
        img, st = c.render()
    return img, st


def _mixed_scenes():
    out = [W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed(),
           W.mid_scene(rays_per_light=1 << 11).packed(),
           W.csg_scene(total_rays=1 << 13, width=384, height=256, string_mod=False).packed()]
    rng = np.random.default_rng(11)
    for _ in range(5):
        w = W.batch_scene(rng)
        out.append(W.scale_rays(w, 1 / 64).packed())
    return out


@pytest.mark.parametrize("precision", [abi.LG_PRECISION_EXACT, abi.LG_PRECISION_FAST])
def test_batch_images_equal_scenes_rendered_alone(ctx, precision):
    scenes = _mixed_scenes()
    for pk in scenes:
        pk.params.precision = precision
    ctx.batch_upload(scenes)
    imgs, st = ctx.batch_render()
    segs = pix = 0
    for k, (pk, img) in enumerate(zip(scenes, imgs)):
        ref, rst = _alone(pk)
        assert img.shape == ref.shape
        assert np.array_equal(img, ref), f"scene {k}: {np.count_nonzero(img != ref)} values differ"
        segs += rst["segments"]
        pix += rst["pixels"]
    assert st["segments"] == segs
    assert st["pixels"] == pix
    assert st["primary_rays"] == sum(sum(pk.lights[i].num_rays for i in range(pk.n_lights)) for pk in scenes)


def test_batch_is_deterministic_and_repeatable(ctx):
    scenes = _mixed_scenes()[:4]
    ctx.batch_upload(scenes)
    a, _ = ctx.batch_render()
    b, _ = ctx.batch_render()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_batch_of_one_and_back_to_single_scene(ctx):
    pk = W.mid_scene(rays_per_light=1 << 10).packed()
    ctx.batch_upload([pk])
    (img,), _ = ctx.batch_render()
    ref, _ = _alone(pk)
    assert np.array_equal(img, ref)
    # the single-scene entry points need a scene again, then work as before
    with pytest.raises(abi.LgError) as e:
        ctx.trace()
    assert e.value.status == abi.LG_ERR_NO_SCENE
    ctx.upload(pk)
    img2, _ = ctx.render()
    assert np.array_equal(img2, ref)


def test_batch_many_small_scenes(ctx):
    """64 mixed-size scenes (objects 4..1024, canvases 256..2048) with reduced ray counts:
    the many-bin path (multi-block tile scan) and the scene tables at scale."""
    ws = W.batch_scenes(seed=5, count=64)
    scenes = [W.scale_rays(w, 1 / 256).packed() for w in ws]
    ctx.batch_upload(scenes)
    imgs, st = ctx.batch_render()
    assert len(imgs) == 64
    for k in (0, 17, 42, 63):
        ref, _ = _alone(scenes[k])
        assert np.array_equal(imgs[k], ref), f"scene {k}"


def test_batch_rejects_mixed_blend_and_string_mod(ctx):
    a = W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed()
    b = W.plain_small(accum=abi.LG_ACCUM_F32).packed()
    with pytest.raises(abi.LgError) as e:
        ctx.batch_upload([a, b])
    assert e.value.status == abi.LG_ERR_UNSUPPORTED
    c = W.csg_scene(total_rays=1 << 10, width=256, height=256).packed()
    with pytest.raises(abi.LgError) as e:
        ctx.batch_upload([a, c])
    assert e.value.status == abi.LG_ERR_UNSUPPORTED
    with pytest.raises(abi.LgError) as e:
        ctx.batch_upload([])
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
    with pytest.raises(abi.LgError) as e:
        ctx.batch_render_into(0, 0, False)
    assert e.value.status == abi.LG_ERR_NO_SCENE
