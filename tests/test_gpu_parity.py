"""GPU trace / raster / resolve against the CPU oracle (through the C ABI).

Bars: per-segment hit ids and the segment set match exactly outside the near-degenerate set;
endpoints within 1e-5 relative; colours bit-exact; the fixed-point image of identical
segments bit-exact; resolve bit-exact; image of the full pipeline within relative L2 1e-3
of the oracle's FP64 trace rasterised on the CPU.
"""
import copy

import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W
from light_garden_gb300.scene import (Circle, ConvexPolygon, CubicBezier, DirectionalLight, LineSegment, Logic, Material,
                                      Object, PointLight, Rect, SpotLight, pack)
from parity import compare, rel_l2

pytestmark = pytest.mark.gpu


def _trace_both(ctx, oracle, packed, stride=1, precision=abi.LG_PRECISION_FAST):
    """The tolerance bar of the double-float mode (the exact mode has its own bit-for-bit
    tests in test_gpu_exact.py and meets this bar trivially)."""
    packed.params.record_paths = 1
    packed.params.precision = precision
    ctx.upload(packed)
    st = ctx.trace()
    g_segs, g_paths = ctx.segments(paths=True)
    o_segs, o_paths, o64, ost = oracle.trace(packed, ray_stride=stride)
    flt = (lambda p: p % stride == 0) if stride > 1 else None
    rep = compare(g_segs, g_paths, o_segs, o_paths, o64, flt)
    return st, rep, (g_segs, g_paths), (o_segs, o_paths, o64)


PRECISIONS = pytest.mark.parametrize("precision", [abi.LG_PRECISION_FAST, abi.LG_PRECISION_EXACT])


@PRECISIONS
def test_plain_small_trace_parity(ctx, oracle, precision):
    pk = W.plain_small().packed()
    st, rep, (gs, gp), (os_, op, o64) = _trace_both(ctx, oracle, pk, precision=precision)
    assert rep.ok(), rep
    assert rep.matched == len(os_) - rep.oracle_only
    assert st["segments"] == len(gs)
    assert rep.matched > 0.99 * len(os_)
    assert st["primary_rays"] == 4096


@PRECISIONS
def test_mid_scene_trace_parity_subsampled(ctx, oracle, precision):
    pk = W.mid_scene(rays_per_light=1 << 14).packed()
    st, rep, _, (os_, _, _) = _trace_both(ctx, oracle, pk, stride=7, precision=precision)
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(os_)


@PRECISIONS
def test_csg_scene_trace_parity_subsampled(ctx, oracle, precision):
    pk = W.csg_scene(total_rays=1 << 16, width=1024, height=1024).packed()
    st, rep, _, (os_, _, _) = _trace_both(ctx, oracle, pk, stride=5, precision=precision)
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(os_)


@pytest.mark.parametrize("variant", [1, 2])
def test_raster_bit_exact_on_same_segments(gpu, oracle, variant):
    from light_garden_gb300.runtime import Context
    ctx = Context(raster_variant=variant)
    w = W.mid_scene(rays_per_light=1 << 12)
    pk = w.packed()
    ctx.upload(pk)
    ctx.trace()
    segs = ctx.segments()
    st = ctx.accumulate()
    g_acc = ctx.accum()
    o_acc, o_px = oracle.raster(segs, pk.params)
    assert st["pixels"] == o_px
    assert np.array_equal(g_acc, o_acc)
    # resolve is bit-exact too
    assert np.array_equal(ctx.resolve_f16(), oracle.resolve_f16(o_acc))
    ctx.close()


def test_raster_variants_agree_on_a_large_frame(gpu):
    """The two tile rasters (shared-memory split planes, 16384-segment units; warp-private
    tiles, 8192-segment units) give the same fixed-point image on a frame with far more
    (segment, tile) references than bins, where the unit table must hold the smaller units."""
    from light_garden_gb300.runtime import Context
    pk = W.mid_scene(rays_per_light=1 << 15).packed()
    accs = []
    for variant in (1, 2):
        ctx = Context(raster_variant=variant)
        ctx.upload(pk)
        ctx.trace()
        st = ctx.accumulate()
        assert st["tile_refs"] > 8192 * 2 * 4080
        accs.append(ctx.accum())
        ctx.close()
    assert np.array_equal(accs[0], accs[1])


def test_accumulate_segments_matches_oracle(ctx, oracle):
    pk = W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed()
    o_segs, _, _, _ = oracle.trace(pk)
    ctx.upload(pk)
    st = ctx.accumulate_segments(o_segs)
    o_acc, o_px = oracle.raster(o_segs, pk.params)
    assert st["pixels"] == o_px
    assert np.array_equal(ctx.accum(), o_acc)


def test_full_pipeline_image_vs_oracle(ctx, oracle):
    pk = W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed()
    ctx.upload(pk)
    img, st = ctx.render()
    o_segs, _, _, _ = oracle.trace(pk)
    o_acc, _ = oracle.raster(o_segs, pk.params)
    o_img = oracle.resolve_f16(o_acc)
    f = lambda u: u.view(np.float16).astype(np.float64)
    assert rel_l2(f(img), f(o_img)) <= 1e-3
    assert rel_l2(ctx.accum() * 2.0 ** -32, o_acc * 2.0 ** -32) <= 1e-3


def test_render_deterministic_and_equal_to_stepwise(ctx):
    pk = W.mid_scene(rays_per_light=1 << 13).packed()
    ctx.upload(pk)
    a, _ = ctx.render()
    acc_a = ctx.accum()
    b, _ = ctx.render()
    acc_b = ctx.accum()
    assert np.array_equal(a, b) and np.array_equal(acc_a, acc_b)
    ctx.trace()
    ctx.accumulate()
    assert np.array_equal(ctx.accum(), acc_a)
    assert np.array_equal(ctx.resolve_f16(), a)


def test_f32_accumulation_within_tolerance(ctx, oracle):
    pk = W.plain_small(accum=abi.LG_ACCUM_F32).packed()
    ctx.upload(pk)
    ctx.trace()
    segs = ctx.segments()
    st = ctx.accumulate()
    g = ctx.accum().astype(np.float64)
    o, px = oracle.raster_f64(segs, pk.params)
    assert st["pixels"] == px
    assert np.abs(g - o).max() <= 1e-5 * max(1.0, np.abs(o).max())


def test_ring_overflow_grows_and_retraces(gpu, oracle):
    from light_garden_gb300.runtime import Context
    pk = W.plain_small().packed()
    pk.params.record_paths = 1
    with Context(segment_capacity=1000, queue_capacity=600) as c:
        c.upload(pk)
        st = c.trace()
        assert st["retries"] >= 1
        gs, gp = c.segments(paths=True)
    os_, op, o64, _ = oracle.trace(pk)
    assert compare(gs, gp, os_, op, o64).ok()


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("cb,ab", [
    ((abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_REVERSE_SUBTRACT), (abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_ADD)),
    ((abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_MAX), (abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_MIN)),
    ((abi.LG_BF_SRC_ALPHA, abi.LG_BF_ONE, abi.LG_BO_ADD), (abi.LG_BF_ONE_MINUS_SRC, abi.LG_BF_ONE, abi.LG_BO_ADD)),
    ((abi.LG_BF_CONSTANT, abi.LG_BF_ONE, abi.LG_BO_ADD), (abi.LG_BF_ONE_MINUS_CONSTANT, abi.LG_BF_ONE, abi.LG_BO_ADD)),
])
def test_blend_modes_bit_exact(gpu, oracle, cb, ab, variant):
    from light_garden_gb300.runtime import Context
    ctx = Context(raster_variant=variant)
    pk = W.plain_small(accum=abi.LG_ACCUM_FIXED64, num_rays=1024).packed()
    pk.params.color_blend = abi.lg_blend_component(*cb)
    pk.params.alpha_blend = abi.lg_blend_component(*ab)
    pk.params.blend_constant[:] = (0.25, 0.5, 0.75, 0.125)
    ctx.upload(pk)
    ctx.trace()
    segs = ctx.segments()
    ctx.accumulate()
    o_acc, _ = oracle.raster(segs, pk.params)
    assert np.array_equal(ctx.accum(), o_acc)
    ctx.close()


def test_overlays_match_oracle(ctx, oracle):
    w = W.csg_scene(total_rays=64, n_objects=4, width=256, height=256)
    w.objects.append(Object.new_curved_mirror(CubicBezier(((-0.5, 0.5), (-0.2, 0.9), (0.2, 0.9), (0.5, 0.5)))))
    pk = w.packed()
    pk.params.record_paths = 1
    ctx.upload(pk)
    ctx.trace()
    gs, gp = ctx.segments(paths=True)
    os_, op, o64, _ = oracle.trace(pk)
    assert ctx.chords().tobytes() == oracle.string_mod_chords(pk.params).tobytes()
    for src, n in ((abi.LG_SRC_CONTROL_LINE, 3),):
        g = gs[gp["source"] == src]
        o = os_[op["source"] == src]
        gk = gp[gp["source"] == src]
        ok = op[op["source"] == src]
        assert len(g) == len(o) == n
        g = g[np.lexsort((gk["gen"], gk["primary"]))]
        o = o[np.lexsort((ok["gen"], ok["primary"]))]
        for f in ("x0", "y0", "x1", "y1"):
            assert np.abs(g[f] - o[f]).max() <= 2e-7
        assert np.array_equal(g["color"], o["color"])
    rep = compare(gs, gp, os_, op, o64)
    assert rep.ok(), rep


def test_scene_edge_cases(ctx, oracle):
    # no objects: every primary leaves through the canvas
    pk = pack([], [PointLight((0.1, 0.2), 360, (1, 1, 1, 1))])
    pk.params.record_paths = 1
    ctx.upload(pk)
    st = ctx.trace()
    assert st["segments"] == 360
    gs, gp = ctx.segments(paths=True)
    os_, op, o64, _ = oracle.trace(pk)
    assert compare(gs, gp, os_, op, o64).ok()
    # no lights: nothing traced, image = clear colour
    pk = pack([Object.new_circle((0, 0), 0.3)], [])
    ctx.upload(pk)
    img, st = ctx.render()
    assert st["segments"] == 0
    assert np.all(img.view(np.float16)[..., 3] == 1.0) and np.all(img.view(np.float16)[..., :3] == 0.0)
    # max_bounce 0: the tracer loop does not run (tracer.rs:373)
    pk = W.plain_small().packed()
    pk.params.max_bounce = 0
    ctx.upload(pk)
    assert ctx.trace()["segments"] == 0
    # lights inside objects, spot with -0.0 direction, directional light, lens
    objs = [Object.new_lens((0.0, 0.0), 2.0, 3.8), Object.new_rect((0.5, 0.5), 0.4, 0.3),
            Object.new_mirror((-0.9, -0.9), (0.9, -0.8))]
    lights = [PointLight((0.5, 0.5), 500, (0.3, 0.2, 0.1, 1.0)),
              SpotLight((-0.5, 0.3), 0.7, (-0.0, 1.0), 300, (1, 1, 1, 1)),
              DirectionalLight((0.5, 0.5, 1.0, 1.0), 400, LineSegment((-0.9, 0.9), (-0.2, 0.95)))]
    pk = pack(objs, lights)
    pk.params.max_bounce = 12
    _, rep, _, _ = _trace_both(ctx, oracle, pk)
    assert rep.ok(), rep


def test_error_statuses(ctx):
    pk = W.plain_small().packed()
    bad = copy.deepcopy(pk.params)
    bad.color_blend = abi.lg_blend_component(abi.LG_BF_DST, abi.LG_BF_ONE, abi.LG_BO_ADD)
    with pytest.raises(abi.LgError) as e:
        ctx.upload(pack(W.plain_small().objects, W.plain_small().lights, bad))
    assert e.value.status == abi.LG_ERR_UNSUPPORTED
    pk2 = W.plain_small().packed()
    pk2.objects[0].kind = abi.LG_OBJ_CONVEX_POLYGON  # a polygon object over a circle geometry
    with pytest.raises(abi.LgError) as e:
        ctx.upload(pk2)
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
    pk4 = pack([Object(abi.LG_OBJ_CONVEX_POLYGON, ConvexPolygon(((0, 0), (1, 0), (2, 0))), Material())], [])
    with pytest.raises(abi.LgError) as e:  # collinear vertices: no interior
        ctx.upload(pk4)
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
    pk3 = W.plain_small().packed()
    pk3.objects[1].geo = 99
    with pytest.raises(abi.LgError) as e:
        ctx.upload(pk3)
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
    pk4 = W.plain_small().packed()
    pk4.params.max_bounce = 65
    with pytest.raises(abi.LgError) as e:
        ctx.upload(pk4)
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT


def test_no_scene_and_truncation(gpu):
    import ctypes as C
    from light_garden_gb300.runtime import Context
    with Context() as c:
        s = abi.lg_trace_stats()
        assert c.lib.lg_trace(c.h, C.byref(s)) == abi.LG_ERR_NO_SCENE
        c.upload(W.plain_small().packed())
        c.trace()
        n = C.c_uint64()
        buf = (abi.lg_segment * 4)()
        assert c.lib.lg_segments_download(c.h, buf, None, 4, C.byref(n)) == abi.LG_ERR_TRUNCATED
        assert n.value > 4


def test_streaming_frame_matches_single_pass(gpu):
    """A frame rendered with the accumulation interleaved between generations (the mode
    lg_render switches to when a frame has more segments than its ring threshold) equals the
    single-pass frame bit for bit, string-mod overlay included."""
    from light_garden_gb300.runtime import Context
    pk = W.csg_scene(total_rays=1 << 14, width=640, height=480).packed()
    with Context() as a:
        a.upload(pk)
        ref, st_ref = a.render()
    with Context(stream_segments=20000) as b:
        b.upload(pk)
        img, st = b.render()
        img2, st2 = b.render()
    assert st_ref["segments"] > 3 * 20000  # several accumulation passes
    assert np.array_equal(img, ref) and np.array_equal(img2, ref)
    assert st["segments"] == st_ref["segments"] and st["pixels"] == st_ref["pixels"]


@pytest.mark.parametrize("variant", [1, 2])
def test_raster_large_terms_bit_exact(gpu, oracle, variant):
    """Colour terms of 2^10 and more (the tile raster's split planes take |q| < 2^42) mixed
    with ordinary ones, added and reverse-subtracted: bit-exact against the CPU raster."""
    from light_garden_gb300.runtime import Context
    rng = np.random.default_rng(5)
    n = 20000
    segs = np.zeros(n, abi.segment_dtype())
    segs["x0"], segs["y0"] = rng.uniform(-1.2, 1.2, n), rng.uniform(-1.2, 1.2, n)
    segs["x1"], segs["y1"] = rng.uniform(-1.2, 1.2, n), rng.uniform(-1.2, 1.2, n)
    col = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    big = rng.random(n) < 0.05
    col[big] *= np.float32(5000.0)
    col[rng.random(n) < 0.01] = np.float32(3.0e6)  # beyond the clamp of 2^20
    segs["color"] = col
    for op in (abi.LG_BO_ADD, abi.LG_BO_REVERSE_SUBTRACT):
        p = abi.params_default()
        p.width, p.height = 640, 480
        p.color_blend = abi.lg_blend_component(abi.LG_BF_ONE, abi.LG_BF_ONE, op)
        pk = pack([], [], p)
        with Context(raster_variant=variant) as c:
            c.upload(pk)
            c.accumulate_segments(segs)
            acc = c.accum()
        ref, _ = oracle.raster(segs, p)
        assert np.array_equal(acc, ref), f"op {op}: {np.count_nonzero(acc != ref)} values differ"


def test_polygons_and_ellipses_parity(ctx, oracle):
    """ConvexPolygon (the And of its edges' half-planes on the GPU, edge segments in the
    oracle) and Ellipse objects among the other shapes: trace parity and image parity."""
    pk = W.shapes_scene().packed()
    st, rep, (gs, gp), (os_, op, o64) = _trace_both(ctx, oracle, pk, stride=11)
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(os_)
    pk2 = W.shapes_scene().packed()
    ctx.upload(pk2)
    img, _ = ctx.render()
    full, _, _, _ = oracle.trace(pk2)
    ref_acc, _ = oracle.raster(full, pk2.params)
    ref = oracle.resolve_f16(ref_acc)
    assert rel_l2(img.view(np.float16).astype(np.float32), ref.view(np.float16).astype(np.float32)) < 1e-3
