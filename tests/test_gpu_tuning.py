"""The per-context autotuners: every choice they can make renders the same frame.

lg_device_opts.scan_pairs picks the FP32 scan's pair slots per lane (8 or 16); 0 lets the first
lg_render (lg_batch_render) of each scene (batch) time both and keep the faster.  The candidate
set the scan hands to the exact solve is fixed by its final bound, not by how the pairs were
batched, so every size gives the same bits.
"""
import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scene", ["csg", "mid"])
def test_scan_pair_sizes_render_identical_frames(gpu, scene):
    from light_garden_gb300.runtime import Context
    pk = (W.csg_scene(total_rays=1 << 14, width=512, height=512) if scene == "csg"
          else W.mid_scene(rays_per_light=1 << 10)).packed()
    imgs = []
    for sp in (8, 16, 0):
        with Context(scan_pairs=sp) as ctx:
            ctx.upload(pk)
            img, st = ctx.render()
            img2, st2 = ctx.render()  # the auto context now runs the size it kept
            assert np.array_equal(img, img2) and st["segments"] == st2["segments"]
            imgs.append(img)
    assert np.array_equal(imgs[0], imgs[1]) and np.array_equal(imgs[0], imgs[2])


def test_scan_pair_sizes_batch_identical(gpu):
    from light_garden_gb300.runtime import Context
    scenes = [W.scale_rays(w, 1.0 / 64).packed() for w in W.batch_scenes(seed=11, count=8)]
    out = []
    for sp in (8, 0):
        with Context(scan_pairs=sp) as ctx:
            ctx.batch_upload(scenes)
            imgs, _ = ctx.batch_render()
            out.append(imgs)
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_scan_pairs_option_is_checked(gpu):
    from light_garden_gb300.runtime import Context
    with pytest.raises(abi.LgError) as e:
        Context(scan_pairs=12)
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
