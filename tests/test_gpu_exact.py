"""The exact FP64 precision mode (LG_PRECISION_EXACT, the default) against the CPU oracle.

In this mode the GPU evaluates the same FP64 formulas as the oracle, operation by operation,
so a trace must equal the oracle's bit for bit: the same set of segments (keyed by source,
light, primary, generation and path bits) with identical endpoints, colours, hit objects and
TIR flags, and the fixed-point image of the frame identical to the oracle's CPU raster of its
own segments.  Nothing is excused.  Full-size configurations are compared on sampled frames
(every k-th primary of each light, lg_params.ray_stride) traced by both sides.
"""
import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W
from light_garden_gb300.scene import (Circle, ConvexPolygon, CubicBezier, DirectionalLight, Ellipse, LineSegment,
                                      Logic, Material, Object, PointLight, Rect, SpotLight, pack)
from parity import exact

pytestmark = pytest.mark.gpu


def _trace_exact(ctx, oracle, pk, stride=1, offset=0, image=False):
    pk.params.record_paths = 1
    pk.params.precision = abi.LG_PRECISION_EXACT
    pk.params.ray_stride, pk.params.ray_offset = stride, offset
    ctx.upload(pk)
    st = ctx.trace()
    gs, gp = ctx.segments(paths=True)
    os_, op, _, _ = oracle.trace(pk, ray_stride=stride, ray_offset=offset)
    rep = exact(gs, gp, os_, op)
    assert rep.ok(), rep
    assert rep.segments == len(os_) == len(gs) == st["segments"]
    # the string-mod lines (drawn when the sample starts at primary 0), bit for bit
    o_ch = oracle.string_mod_chords(pk.params) if offset == 0 else np.zeros(0, abi.chord_dtype())
    assert ctx.chords().tobytes() == o_ch.tobytes()
    if image:  # the frame's fixed-point image equals the oracle's raster of its own segments and lines
        ctx.accumulate()
        acc = ctx.accum()
        o_acc, _ = oracle.raster(os_, pk.params, chords=o_ch)
        assert np.array_equal(acc, o_acc)
        assert np.array_equal(ctx.resolve_f16(), oracle.resolve_f16(o_acc))
    return st, rep


def test_plain_small_exact_and_image(ctx, oracle):
    st, rep = _trace_exact(ctx, oracle, W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed(), image=True)
    assert st["primary_rays"] == 4096 and rep.segments > 8000


def test_mid_scene_full_size_sampled_exact(ctx, oracle):
    """64 objects, 8 lights x 2^18 rays, 16 bounces, 1920x1080: every 97th primary."""
    st, rep = _trace_exact(ctx, oracle, W.mid_scene().packed(), stride=97, offset=13, image=True)
    assert st["primary_rays"] == sum((n - 13 + 96) // 97 for n in [1 << 18] * 8)
    assert rep.segments > 1_000_000


def test_csg_scene_full_size_sampled_exact(ctx, oracle):
    """256 CSG objects, 2^22 rays, 32 bounces, 4096^2, string-mod overlay: every 257th
    primary (the overlay is drawn with offset 0)."""
    st, rep = _trace_exact(ctx, oracle, W.csg_scene().packed(), stride=257, offset=0, image=True)
    assert rep.segments > 4_000_000


def test_fixtures_reproduced_exactly(ctx, oracle):
    """The committed oracle fixtures (written on another machine) are reproduced bit for bit
    by the GPU: the trace does not depend on the host's math library."""
    import json
    from pathlib import Path
    gold = Path(__file__).resolve().parent / "golden"
    index = json.loads((gold / "golden.json").read_text())
    for name, make in (("mid_scene_subset", W.mid_scene), ("csg_scene_subset", W.csg_scene)):
        z = np.load(gold / f"{name}.npz")
        pk = make().packed()
        pk.params.record_paths = 1
        pk.params.ray_stride = index[name]["stride"]
        ctx.upload(pk)
        ctx.trace()
        gs, gp = ctx.segments(paths=True)
        rep = exact(gs, gp, z["segs"], z["paths"])
        assert rep.ok(), (name, rep)
        assert rep.segments == len(z["segs"])
        assert ctx.chords().tobytes() == z["chords"].tobytes()


def test_culling_grid_exact(gpu, oracle):
    """A 300-object scene traced through the culling grid equals the oracle's brute-force
    nearest-hit scan exactly."""
    from light_garden_gb300.runtime import Context
    w = max(W.batch_scenes(seed=21, count=64), key=lambda x: len(x.objects))
    assert len(w.objects) >= 96
    rays = sum(l.num_rays for l in w.lights)
    for cull in (abi.LG_CULL_ON, abi.LG_CULL_OFF):
        with Context(culling=cull) as ctx:
            _trace_exact(ctx, oracle, w.packed(), stride=max(1, rays // 20000))


def test_shapes_and_nested_csg_exact(ctx, oracle):
    """Polygons, ellipses, lenses, straight and curved mirrors and a three-level Logic tree."""
    nested = Logic(abi.LG_OP_OR,
                   Logic(abi.LG_OP_AND_NOT, Circle((0.0, 0.0), 0.2), Rect((0.05, 0.0), 0.1, 0.1, (0.6, 0.8)),
                         (0.0, 0.0), (1.0, 0.0)),
                   Logic(abi.LG_OP_AND, Ellipse((0.15, 0.1), 0.12, 0.05, (0.8, -0.6)), Circle((0.2, 0.05), 0.1),
                         (0.02, -0.01), (0.96, 0.28)),
                   (0.3, -0.4), (0.6, 0.8))
    objs = [
        Object(abi.LG_OBJ_GEO, nested, Material(1.45)),
        Object(abi.LG_OBJ_CONVEX_POLYGON, ConvexPolygon(((-0.1, -0.1), (0.12, -0.08), (0.15, 0.1), (-0.05, 0.14)),
                                                        (-0.5, 0.3), (0.8, 0.6)), Material(1.6)),
        Object(abi.LG_OBJ_ELLIPSE, Ellipse((0.5, 0.4), 0.15, 0.08, (0.6, 0.8)), Material(1.33)),
        Object.new_lens((-0.3, -0.4), 0.25, 0.12),
        Object.new_mirror((-0.9, 0.7), (-0.6, 0.95)),
        Object.new_curved_mirror(CubicBezier(((0.6, -0.8), (0.8, -0.5), (0.9, -0.9), (0.95, -0.4)))),
    ]
    lights = [PointLight((-0.05, 0.02), 3000, (1.0, 0.8, 0.6, 1.0)),
              SpotLight((0.9, 0.9), 1.2, (-1.0, -0.7), 2000, (0.3, 0.9, 0.4, 1.0)),
              DirectionalLight((0.5, 0.5, 1.0, 1.0), 1500, LineSegment((-1.0, -0.95), (0.2, -0.95)))]
    p = abi.params_default()
    p.width, p.height, p.max_bounce = 800, 600, 24
    _trace_exact(ctx, oracle, pack(objs, lights, p), image=True)


def test_cubic_mirrors_exact(ctx, oracle):
    """24 seeded cubic-Bezier mirrors (every third an S-curve that a line can cross three
    times) around a glass disc, 32,000 rays, 16 bounces: the cubic hits whose root the FP32
    scan proved are solved in their own bracket alone, and must still equal the oracle's
    full three-bracket solve bit for bit."""
    rng = np.random.default_rng(1234)
    objs = []
    for k in range(24):
        c = rng.uniform(-0.8, 0.8, 2)
        r = rng.uniform(0.08, 0.25)
        a = rng.uniform(0, 2 * np.pi)
        u = np.array([np.cos(a), np.sin(a)])
        n = np.array([-u[1], u[0]])
        if k % 3 == 0:
            h = r * 1.5
            pts = [c - r * u - h * n, c - r / 3 * u + 3 * h * n, c + r / 3 * u - 3 * h * n, c + r * u + h * n]
        else:
            pts = [c + r * rng.uniform(-1, 1, 2) for _ in range(4)]
        objs.append(Object.new_curved_mirror(CubicBezier(tuple(tuple(map(float, q)) for q in pts))))
    objs.append(Object(abi.LG_OBJ_GEO, Circle((0.05, -0.1), 0.12), Material(1.5)))
    lights = [PointLight((0.0, 0.0), 20000, (1.0, 0.9, 0.7, 1.0)),
              SpotLight((-0.95, 0.9), 0.9, (1.0, -0.8), 12000, (0.4, 0.8, 1.0, 1.0))]
    p = abi.params_default()
    p.width, p.height, p.max_bounce = 1024, 1024, 16
    st, rep = _trace_exact(ctx, oracle, pack(objs, lights, p), image=True)
    assert rep.segments > 900_000


def test_default_scene_from_ron_exact(ctx, oracle):
    from pathlib import Path
    from light_garden_gb300 import ron
    objs, lights = ron.load(Path(__file__).resolve().parent / "golden" / "default_scene.ron")
    p = abi.params_default()
    p.width, p.height, p.max_bounce = 1024, 768, 12
    _trace_exact(ctx, oracle, pack(objs, lights, p), image=True)


def test_exact_rejects_trees_deeper_than_eight(ctx):
    g = Circle((0.0, 0.0), 0.1)
    for i in range(9):
        g = Logic(abi.LG_OP_OR, g, Circle((0.01 * i, 0.0), 0.1))
    pk = pack([Object(abi.LG_OBJ_GEO, g, Material(1.5))], [PointLight((-0.8, 0.0), 16, (1, 1, 1, 1))])
    with pytest.raises(abi.LgError) as e:
        ctx.upload(pk)
    assert e.value.status == abi.LG_ERR_UNSUPPORTED
    pk.params.precision = abi.LG_PRECISION_FAST
    ctx.upload(pk)  # the double-float mode flattens any tree


def test_batch_exact_images_equal_oracle(gpu, oracle):
    """Exact mode in a multi-scene batch: every image equals the oracle's raster of the
    oracle's trace of that scene."""
    from light_garden_gb300.runtime import Context
    scenes = [W.scale_rays(w, 1.0 / 64).packed() for w in W.batch_scenes(seed=9, count=6)]
    with Context() as ctx:
        ctx.batch_upload(scenes)
        imgs, _ = ctx.batch_render()
    for pk, img in zip(scenes, imgs):
        os_, _, _, _ = oracle.trace(pk)
        o_acc, _ = oracle.raster(os_, pk.params)
        assert np.array_equal(img, oracle.resolve_f16(o_acc))


@pytest.mark.parametrize("curve", [abi.LG_CURVE_CIRCLE, abi.LG_CURVE_COMPLEX_EXP, abi.LG_CURVE_HYPOTROCHOID,
                                   abi.LG_CURVE_LISSAJOUS])
def test_string_mod_lines_and_blends_exact(ctx, oracle, curve):
    """String-mod art on every curve with modulo colours: the lines bit for bit, and the image
    (interpolated vertex colours) bit for bit in additive and max blending; in FP32
    accumulation within the summation bound of the FP64 raster."""
    w = W.string_mod_art(curve, 768, 512)
    pk = w.packed()
    _trace_exact(ctx, oracle, pk, image=True)
    pk.params.color_blend = abi.lg_blend_component(abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_MAX)
    pk.params.alpha_blend = abi.lg_blend_component(abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_MIN)
    _trace_exact(ctx, oracle, pk, image=True)
    pk = w.packed()
    pk.params.accum = abi.LG_ACCUM_F32
    pk.params.record_paths = 1
    ctx.upload(pk)
    ctx.trace()
    ctx.accumulate()
    os_, _, _, _ = oracle.trace(pk)
    o_ch = oracle.string_mod_chords(pk.params)
    f64, _ = oracle.raster_f64(os_, pk.params, chords=o_ch)
    acc = ctx.accum().astype(np.float64)
    # the number of terms n of every pixel: the same lines in white, One/One added in fixed point
    ones, ch1 = os_.copy(), o_ch.copy()
    ones["color"], ch1["color0"], ch1["color1"] = 1.0, 1.0, 1.0
    cp = abi.params_default()
    cp.width, cp.height = pk.params.width, pk.params.height
    cp.clear_color[:] = (0.0, 0.0, 0.0, 0.0)
    cp.alpha_blend = abi.lg_blend_component(abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_ADD)
    cnt, _ = oracle.raster(ones, cp, chords=ch1)
    n = (cnt[..., :1] >> 32).astype(np.float64) + 1.0
    # FP32 atomics add the same non-negative f32 terms in no fixed order: within 2 n u |sum|
    tol = 2.0 * n * 2.0 ** -24 * np.abs(f64) + 1e-30
    assert (np.abs(acc - f64) <= tol).all(), (np.abs(acc - f64) / tol).max()


@pytest.mark.parametrize("curve", [abi.LG_CURVE_CIRCLE, abi.LG_CURVE_COMPLEX_EXP, abi.LG_CURVE_HYPOTROCHOID,
                                   abi.LG_CURVE_LISSAJOUS])
def test_nested_string_mod_exact(ctx, oracle, curve):
    """A nested mod over the crossings of 400 lines of each curve: the crossings (computed on
    the GPU at upload), the nested lines and the image equal the oracle's bit for bit."""
    w = W.nested_string_mod_art(curve, 768, 512)
    _trace_exact(ctx, oracle, w.packed(), image=True)
    assert len(ctx.chords()) == 6000


def test_nested_string_mod_at_the_limit_and_edge_cases(ctx, oracle):
    # 4096 outer lines: 16.8 M line pairs in 4096 blocks, about 6 M crossings
    pk = W.nested_string_mod_art(abi.LG_CURVE_CIRCLE, 1024, 1024, outer_modulo=4096).packed()
    _trace_exact(ctx, oracle, pk, image=True)
    # the same scene with another nested mod: the new lines, not the old ones
    ns = abi.lg_string_mod()
    ns.modulo, ns.num, ns.mode = 2500, 3, abi.LG_SM_POW
    ns.color[:] = (0.2, 1.0, 0.4, 1.0)
    abi.set_nested(pk.params, ns)
    _trace_exact(ctx, oracle, pk, image=True)
    assert len(ctx.chords()) == 2500
    # lines that never cross (each from a point to itself): no nested lines, and the image is
    # the trace's alone
    pk = W.nested_string_mod_art(abi.LG_CURVE_CIRCLE, 256, 256, outer_modulo=64).packed()
    pk.params.string_mod.mode, pk.params.string_mod.num = abi.LG_SM_ADD, 0
    _trace_exact(ctx, oracle, pk, image=True)
    assert len(ctx.chords()) == 0
    # one outer line: no pairs at all
    pk = W.nested_string_mod_art(abi.LG_CURVE_CIRCLE, 256, 256, outer_modulo=1).packed()
    _trace_exact(ctx, oracle, pk, image=True)
    assert len(ctx.chords()) == 0


def test_nested_string_mod_rejects_bad_parameters(ctx):
    pk = W.nested_string_mod_art(abi.LG_CURVE_CIRCLE, 256, 256,
                                 outer_modulo=abi.LG_STRING_MOD_NESTED_MAX + 1).packed()
    with pytest.raises(abi.LgError) as e:
        ctx.upload(pk)
    assert e.value.status == abi.LG_ERR_UNSUPPORTED
    for field, value in (("mode", 4), ("modulo", (1 << 26) + 1)):
        pk = W.nested_string_mod_art(abi.LG_CURVE_CIRCLE, 256, 256).packed()
        ns = abi.lg_string_mod()
        ns.modulo, ns.num, ns.mode = 100, 3, abi.LG_SM_ADD
        setattr(ns, field, value)
        abi.set_nested(pk.params, ns)
        with pytest.raises(abi.LgError) as e:
            ctx.upload(pk)
        assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT


def test_string_mod_lines_dropped_by_accumulate_segments(ctx, oracle):
    pk = W.string_mod_art(abi.LG_CURVE_CIRCLE, 256, 256).packed()
    ctx.upload(pk)
    ctx.render()
    assert len(ctx.chords()) == pk.params.string_mod.modulo
    segs, _, _, _ = oracle.trace(pk)
    ctx.accumulate_segments(segs)  # the caller's segments replace the trace: no lines drawn
    assert len(ctx.chords()) == 0
    o_acc, _ = oracle.raster(segs, pk.params)
    assert np.array_equal(ctx.accum(), o_acc)


def test_string_mod_rejects_bad_parameters(ctx):
    pk = W.string_mod_art(abi.LG_CURVE_CIRCLE, 256, 256).packed()
    for field, value in (("curve", 4), ("mode", 4)):
        bad = W.string_mod_art(abi.LG_CURVE_CIRCLE, 256, 256).packed()
        setattr(bad.params.string_mod, field, value)
        with pytest.raises(abi.LgError) as e:
            ctx.upload(bad)
        assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
    abi.set_mod_colors(pk.params, [(0, 0, (1.0, 1.0, 1.0, 1.0))])  # ix % 0
    with pytest.raises(abi.LgError) as e:
        ctx.upload(pk)
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
