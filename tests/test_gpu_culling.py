"""Culled nearest-hit search (uniform grid per scene) against the full scan and the oracle.

The culled scan visits a ray's objects cell by cell, nearest cell first, and stops at the
first cell beyond its bound; it must hand the precise solve the same candidates as the
full scan, so a culled trace equals an unculled one path for path (hit ids, endpoints,
colours), whatever the cell size, and meets the oracle parity bar on its own.
"""
import copy

import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W
from light_garden_gb300.scene import Circle, Material, Object, PointLight, Rect, SpotLight, pack
from parity import compare

pytestmark = pytest.mark.gpu


def _trace(pk, culling, density=0.0):
    from light_garden_gb300.runtime import Context
    ctx = Context(culling=culling, grid_density=density)
    try:
        pk = copy.deepcopy(pk)
        pk.params.record_paths = 1
        ctx.upload(pk)
        st = ctx.trace()
        segs, paths = ctx.segments(paths=True)
        return st, segs, paths
    finally:
        ctx.close()


def _by_key(segs, paths):
    order = np.lexsort((paths["path"], paths["gen"], paths["primary"], paths["light"], paths["source"]))
    return segs[order], paths[order]


def _assert_same_trace(a, b):
    sa, pa = _by_key(*a)
    sb, pb = _by_key(*b)
    assert len(sa) == len(sb)
    for f in ("source", "light", "primary", "gen", "path", "hit"):
        assert np.array_equal(pa[f], pb[f]), f
    # everything but the full-scan fallback bit (a route, not a result); the double-float mode's
    # two reasons for a flag compare as one: with more or fewer candidates a route can see a
    # path's ill-conditioning as a tie in the band, or the other way round
    def flags(p):
        f = p["flags"] & np.uint8(0xff & ~abi.LG_PATH_FALLBACK)
        ill = (f & np.uint8(abi.LG_PATH_ILL_CONDITIONED)) != 0
        return (f & np.uint8(0xff & ~abi.LG_PATH_ILL_CONDITIONED)) | np.where(ill, np.uint8(1), np.uint8(0))
    assert np.array_equal(flags(pa), flags(pb))
    for f in ("x0", "y0", "x1", "y1"):
        assert np.allclose(sa[f], sb[f], rtol=1e-6, atol=1e-6), f
    assert np.array_equal(sa["color"], sb["color"])


def _far_light_scene():
    """Objects clustered near the origin, lights far outside the objects' box: their
    primaries start beyond the grid's reach and take the full scan."""
    rng = np.random.default_rng(11)
    objs = []
    for _ in range(40):
        c = tuple(rng.uniform(-0.3, 0.3, 2))
        if rng.uniform() < 0.5:
            objs.append(Object(abi.LG_OBJ_CIRCLE, Circle(c, rng.uniform(0.01, 0.05)), Material(1.5)))
        else:
            objs.append(Object(abi.LG_OBJ_RECT, Rect(c, 0.06, 0.03, (0.8, 0.6)), Material(1.4)))
    lights = [SpotLight((40.0, 0.5), 0.05, (-1.0, -0.012), 4096, (1.0, 0.8, 0.6, 1.0)),
              PointLight((0.9, 0.9), 4096, (0.5, 0.7, 1.0, 1.0))]
    p = abi.params_default()
    p.max_bounce = 10
    p.width, p.height = 800, 600
    return pack(objs, lights, p)


CASES = {
    "plain_small": lambda: W.plain_small().packed(),
    "mid_scene": lambda: W.mid_scene(rays_per_light=1 << 12).packed(),
    "csg_scene": lambda: W.csg_scene(total_rays=1 << 14, width=512, height=512, string_mod=False).packed(),
    "shapes_scene": lambda: W.shapes_scene(rays_per_light=1 << 12).packed(),
    "far_lights": _far_light_scene,
}


@pytest.mark.parametrize("precision", [abi.LG_PRECISION_EXACT, abi.LG_PRECISION_FAST])
@pytest.mark.parametrize("name", sorted(CASES))
def test_culled_trace_equals_full_scan(gpu, name, precision):
    pk = CASES[name]()
    pk.params.precision = precision
    st0, *full = _trace(pk, abi.LG_CULL_OFF)
    st1, *grid = _trace(pk, abi.LG_CULL_ON)
    _assert_same_trace(full, grid)
    assert st0["ray_visits"] == st1["ray_visits"]
    assert st1["bound_tests"] <= st0["bound_tests"]


@pytest.mark.parametrize("density", [0.05, 0.5, 8.0, 64.0])
def test_cell_size_does_not_change_the_trace(gpu, density):
    pk = W.csg_scene(total_rays=1 << 13, width=512, height=512, string_mod=False).packed()
    _, *full = _trace(pk, abi.LG_CULL_OFF)
    _, *grid = _trace(pk, abi.LG_CULL_ON, density)
    _assert_same_trace(full, grid)


def test_culled_mid_scene_meets_oracle_parity(gpu, oracle):
    pk = W.mid_scene(rays_per_light=1 << 14).packed()
    _, segs, paths = _trace(pk, abi.LG_CULL_ON)
    pk.params.record_paths = 1
    o_segs, o_paths, o64, _ = oracle.trace(pk, ray_stride=7)
    rep = compare(segs, paths, o_segs, o_paths, o64, lambda p: p % 7 == 0)
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(o_segs)


def test_culled_far_lights_meet_oracle_parity(gpu, oracle):
    pk = _far_light_scene()
    _, segs, paths = _trace(pk, abi.LG_CULL_ON)
    pk.params.record_paths = 1
    o_segs, o_paths, o64, _ = oracle.trace(pk)
    rep = compare(segs, paths, o_segs, o_paths, o64)
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(o_segs)


def test_culling_cuts_the_bounding_tests(gpu):
    """256 CSG objects: the culled search tests a small fraction of the objects per ray."""
    pk = W.csg_scene(total_rays=1 << 14, width=512, height=512, string_mod=False).packed()
    st0, *_ = _trace(pk, abi.LG_CULL_OFF)
    st1, *_ = _trace(pk, abi.LG_CULL_AUTO)
    assert st0["bound_tests"] >= 256 * st0["ray_visits"] * 0.9
    assert st1["bound_tests"] < 0.25 * st0["bound_tests"]
    # the classifications stay about the same: the objects that pass the bounding test
    assert st1["object_tests"] <= 1.1 * st0["object_tests"]


def test_culled_batch_images_equal_full_scan(gpu):
    from light_garden_gb300.runtime import Context
    rng = np.random.default_rng(5)
    scenes = [W.scale_rays(W.batch_scene(rng), 1 / 64).packed() for _ in range(12)]
    imgs = {}
    for cull in (abi.LG_CULL_OFF, abi.LG_CULL_ON):
        ctx = Context(culling=cull)
        ctx.batch_upload(scenes)
        imgs[cull], _ = ctx.batch_render()
        ctx.close()
    for a, b in zip(imgs[abi.LG_CULL_OFF], imgs[abi.LG_CULL_ON]):
        assert np.array_equal(a, b)


def test_tracer_tile_map_toggle_keeps_the_image(gpu):
    """Tracer::enable_tile_map (tracer.rs:137-160) switches the culling option; with the
    exact grid the rendered image is the same on and off."""
    from light_garden_gb300.tracer import Tracer
    w = W.csg_scene(total_rays=1 << 12, width=256, height=256, string_mod=False)
    t = Tracer(256, 256)
    for o in w.objects:
        t.push_object(o)
    for l in w.lights:
        t.push_light(l)
    t.max_bounce = 8
    on = t.render_to_texture()
    t.enable_tile_map(False)
    assert not t.tile_map_enabled()
    off = t.render_to_texture()
    assert np.array_equal(on, off)
    t.close()
