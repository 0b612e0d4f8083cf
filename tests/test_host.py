"""Host-side logic without a GPU: scene packing into the C ABI tables, the seeded workload
generators, the ``Tracer`` mirror of the reference's list API, and the oracle's CPU
reference-arm sampling used by ``bench.py``."""
import ctypes as C

import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W
from light_garden_gb300 import scene as S
from light_garden_gb300.tracer import Tracer


def test_pack_flattens_csg_trees_preorder():
    lens = S.Object.new_lens((0.1, -0.2), 2.0, 3.8)
    nested = S.Object.new_geo(S.Logic(abi.LG_OP_OR, S.Circle((0, 0), 0.1),
                                      S.Circle((0.2, 0), 0.1).and_not(S.Rect((0.2, 0), 0.05, 0.05))))
    m = S.Object.new_mirror((0, 0), (1, 0))
    pk = S.pack([lens, nested, m], [])
    assert pk.n_objects == 3 and pk.n_geo == 3 + 5 + 1
    g = pk.geos
    # lens: Logic(And) with two circles at (±d/2, 0) in its own frame (object.rs:393-411)
    assert (g[0].kind, g[0].op, g[0].a, g[0].b) == (abi.LG_GEO_LOGIC, abi.LG_OP_AND, 1, 2)
    assert list(g[0].origin) == [0.1, -0.2]
    assert (g[1].origin[0], g[2].origin[0], g[1].v[0]) == (1.9, -1.9, 2.0)
    # nested: Or(circle, AndNot(circle, rect)), children indexed after their parent
    r = pk.objects[1].geo
    assert r == 3 and g[r].kind == abi.LG_GEO_LOGIC and g[r].op == abi.LG_OP_OR
    assert g[g[r].b].op == abi.LG_OP_AND_NOT and g[g[g[r].b].b].kind == abi.LG_GEO_RECT
    assert pk.objects[2].kind == abi.LG_OBJ_STRAIGHT_MIRROR and pk.objects[2].has_material == 0


def test_materials_and_defaults():
    # Material::default n = 1.2 (object.rs:441-447); mirrors have none
    assert S.Object.new_circle((0, 0), 1).material_opt.refractive_index == 1.2
    assert S.Object.new_curved_mirror(S.CubicBezier(((0, 0), (1, 1), (2, 1), (3, 0)))).material_opt is None
    pk = S.pack([S.Object.new_rect((0, 0), 1, 1)], [])
    assert pk.objects[0].has_material == 1 and pk.objects[0].refractive_index == 1.2


def test_pack_lights():
    pl = S.pack_light(S.PointLight((0.5, 0.25), 100, (1, 0.5, 0.25, 1)))
    assert (pl.kind, pl.num_rays, list(pl.origin)) == (abi.LG_LIGHT_POINT, 100, [0.5, 0.25])
    sp = S.pack_light(S.SpotLight((0, 0), 0.3, (0.0, 1.0), 7, (1, 1, 1, 1)))
    assert (sp.kind, sp.spot_angle, list(sp.v)) == (abi.LG_LIGHT_SPOT, 0.3, [0.0, 1.0])
    dl = S.pack_light(S.DirectionalLight((1, 1, 1, 1), 3, S.LineSegment((0, 0), (1, 0))))
    assert (dl.kind, list(dl.origin), list(dl.v)) == (abi.LG_LIGHT_DIRECTIONAL, [0.0, 0.0], [1.0, 0.0])
    with pytest.raises(TypeError):
        S.pack_light(object())


def test_canvas_bounds_uses_f32_aspect():
    # sub_render_pass.rs:146-156: Rect::from_tlbr(1, -aspect, -1, aspect), aspect an f32
    r = S.canvas_bounds(1920, 1080)
    aspect = float(np.float32(1920) / np.float32(1080))
    assert r.origin == (0.0, 0.0) and r.width == 2 * aspect and r.height == 2.0


def test_plain_small_is_the_small_configuration():
    w = W.plain_small()
    p = w.params
    assert (p.width, p.height, p.max_bounce, p.accum) == (512, 512, 8, abi.LG_ACCUM_F32)
    assert len(w.lights) == 1 and w.lights[0].position == (-0.8, 0.0) and w.primary_rays == 4096
    kinds = [o.kind for o in w.objects]
    assert kinds == [abi.LG_OBJ_CIRCLE, abi.LG_OBJ_STRAIGHT_MIRROR]
    assert w.objects[0].geo.radius == 0.2 and w.objects[0].material_opt.refractive_index == 1.5
    assert (w.objects[1].geo.a, w.objects[1].geo.b) == ((0.6, -0.5), (0.6, 0.5))


def test_mid_scene_distributions_and_determinism():
    w = W.mid_scene()
    p = w.params
    assert (p.width, p.height, p.max_bounce, p.accum) == (1920, 1080, 16, abi.LG_ACCUM_FIXED64)
    assert len(w.objects) == 64 and len(w.lights) == 8 and w.primary_rays == 8 << 18
    kinds = {o.kind for o in w.objects}
    assert kinds == {abi.LG_OBJ_RECT, abi.LG_OBJ_CIRCLE, abi.LG_OBJ_STRAIGHT_MIRROR, abi.LG_OBJ_CURVED_MIRROR}
    for o in w.objects:
        if o.material_opt is not None:
            assert 1.3 <= o.material_opt.refractive_index <= 1.8
        if o.kind == abi.LG_OBJ_CIRCLE:
            assert 0.02 <= o.geo.radius <= 0.15 and all(-1 <= c <= 1 for c in o.geo.origin)
    a, b = W.mid_scene().packed(), W.mid_scene().packed()
    assert bytes(a.geos) == bytes(b.geos) and bytes(a.lights) == bytes(b.lights)
    assert bytes(W.mid_scene(seed=5).packed().geos) != bytes(a.geos)


def test_csg_scene_configuration():
    w = W.csg_scene()
    p = w.params
    assert (p.width, p.height, p.max_bounce) == (4096, 4096, 32)
    assert len(w.objects) == 256 and w.primary_rays == 1 << 22
    ops = {o.geo.op for o in w.objects}
    assert ops == {abi.LG_OP_AND, abi.LG_OP_OR, abi.LG_OP_AND_NOT}
    assert all(isinstance(o.geo.a, S.Circle) and isinstance(o.geo.b, S.Rect) for o in w.objects)
    assert (p.string_mod.modulo, p.string_mod.num, p.string_mod.mode) == (4096, 7, abi.LG_SM_MUL)


def test_batch_scene_ranges():
    ws = W.batch_scenes(count=64)
    for w in ws:
        assert 4 <= len(w.objects) <= 1024
        assert 4 <= w.params.max_bounce <= 32
        assert w.params.width in (256, 512, 1024, 2048) and w.params.width == w.params.height
        assert 1 <= len(w.lights) <= 8
    assert [len(w.objects) for w in W.batch_scenes(count=64)] == [len(w.objects) for w in ws]


def test_scale_rays():
    w = W.mid_scene()
    w2 = W.scale_rays(w, 1 / 64)
    assert w2.primary_rays == 8 << 12 and w.primary_rays == 8 << 18


def test_string_mod_types_mirror_the_reference():
    """StringMod / Curve / ModRemColor / StringModMode with the reference's names and defaults
    (StringMod::new, string_mod.rs:18-31) fill lg_params.string_mod, nested mod included, exactly
    as the nested workload sets it field by field."""
    d = S.StringMod()
    assert (d.modulo, d.num, d.pow, d.color, d.turns, d.init_curve, d.mode, d.modulo_colors, d.modulo_color_index,
            d.nested) == (5, 1, 0, (1.0, 1.0, 1.0, 1.0), 1, S.Curve.circle(), S.StringModMode.Mul, [], 0, None)
    sm = S.StringMod(modulo=400, num=13, color=(0.3, 0.3, 0.3, 1.0), turns=3, init_curve=S.Curve.hypotrochoid(3, 5, 2),
                     modulo_colors=[S.ModRemColor(4, 3, (0.0, 1.0, 1.0, 1.0))],
                     nested=S.StringMod(modulo=6000, num=17, color=(0.9, 0.9, 0.2, 1.0), mode=S.StringModMode.Add,
                                        modulo_colors=[S.ModRemColor(5, 1, (0.1, 0.8, 1.0, 1.0)),
                                                       S.ModRemColor(7, 3, (1.0, 0.5, 0.0, 0.7))]))
    mine = sm.apply(abi.params_default()).string_mod
    ref = W.nested_string_mod_art(abi.LG_CURVE_HYPOTROCHOID).params.string_mod

    def fields(x, skip=()):
        return {f: (list(getattr(x, f)) if hasattr(getattr(x, f), "__len__") else getattr(x, f))
                for f, *_ in x._fields_ if f not in ("colors", "nested") + skip}

    def table(x):
        return [(e.modulo, e.rem, list(e.color)) for e in (abi.lg_mod_color * x.n_colors).from_address(x.colors)] \
            if x.n_colors else []

    assert fields(mine) == fields(ref) and table(mine) == table(ref)
    nm = abi.lg_string_mod.from_address(mine.nested)
    nr = abi.lg_string_mod.from_address(ref.nested)
    unused = ("turns", "curve", "curve_f", "curve_u")  # a nested mod's points are the crossings
    assert fields(nm, unused) == fields(nr, unused) and table(nm) == table(nr)
    c = S.Curve.complex_exp(complex(0.6, 0.8))
    assert (c.kind, c.f) == (abi.LG_CURVE_COMPLEX_EXP, (0.6, 0.8))
    c = S.Curve.lissajous(3, 4, 0.5)
    assert (c.kind, c.f, c.u) == (abi.LG_CURVE_LISSAJOUS, (0.5, 0.0), (3, 4, 0))


def test_tracer_list_api_matches_the_reference_surface():
    """tracer.rs:48-129: push / index / replace / remove / clear, without touching the GPU."""
    t = Tracer(1920, 1080)
    c = S.Object.new_circle((0, 0), 0.2)
    m = S.Object.new_mirror((0.6, -0.5), (0.6, 0.5))
    t.push_object(c)
    t.push_object(m)
    t.push_light(S.PointLight((-0.8, 0), 16, (1, 1, 1, 1)))
    assert t.index_object(1) is m and list(t.object_iterator()) == [c, m]
    t.replace_object(0, S.Object.new_rect((0, 0), 0.1, 0.1))
    assert t.index_object(0).kind == abi.LG_OBJ_RECT
    t.remove_object(0)
    assert list(t.object_iterator()) == [m]
    assert len(list(t.light_iterator())) == 1
    t.max_bounce = 12
    t.cutoff_color = [0.01, 0.02, 0.03, 0.04]
    p = t.params()
    assert (p.max_bounce, p.width, p.height) == (12, 1920, 1080)
    assert list(p.cutoff_color) == pytest.approx([0.01, 0.02, 0.03, 0.04])
    pk = t.packed()
    assert pk.n_objects == 1 and pk.n_lights == 1
    t.resize(800, 600)
    assert t.params().width == 800 and t.canvas_bounds.height == 2.0
    t.remove_light(0)
    t.clear()
    assert t.packed().n_objects == 0 and t.packed().n_lights == 0
    # tracer.rs:137-164: the tile map toggle maps to the culling option (on by default)
    assert t.tile_map_enabled()
    t.enable_tile_map(False)
    assert not t.tile_map_enabled() and t._culling == abi.LG_CULL_OFF
    t.enable_tile_map(True)
    assert t.tile_map_enabled() and t._culling == abi.LG_CULL_AUTO
    assert t._ctx is None  # nothing above needed the GPU
    t.close()


def test_reference_arm_sample_is_bounded(monkeypatch):
    """bench.py's CPU samples: every stride-th primary of each light of the mid and CSG frames."""
    import bench
    pk, segs, paths, acc, px, tt, tr, prim = bench.cpu_sample("mid", 4096)
    assert prim == 8 * (1 << 18) // 4096
    assert len(segs) > prim and px > len(segs) and acc.shape == (1080, 1920, 4)
    pk, segs, paths, acc, px, tt, tr, prim = bench.cpu_sample("csg", 1 << 16)
    assert prim == 8 * ((1 << 22) // 8) // (1 << 16)
    assert len(segs) > prim and len(paths) == len(segs)
