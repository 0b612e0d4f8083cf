"""Known-answer tests of the CPU oracle, derived by hand from the geometry and optics.

The reference ships no tests and its geometry crate is not on disk, so these analytic cases
(plus the committed golden fixtures of ``test_golden.py``) are what pins the oracle before
it is used to check the CUDA path.  Each case states the mathematics it checks.
"""
import math

import numpy as np
import pytest

from light_garden_gb300 import abi
from light_garden_gb300 import scene as S

pytestmark = pytest.mark.filterwarnings("ignore::DeprecationWarning")


def hits(O, geo, o, d):
    pk = S.pack([S.Object.new_geo(geo)], [])
    h, flags = O.geo_hits(pk.geos, pk.n_geo, 0, o, d)
    return sorted(h), flags


def contains(O, geo, p):
    pk = S.pack([S.Object.new_geo(geo)], [])
    return O.geo_contains(pk.geos, pk.n_geo, 0, p)


def assert_hit(h, t, p, n):
    """t and point exactly as derived; normal up to sign (the bounce orients it against the ray)."""
    assert h[0] == pytest.approx(t, abs=1e-12)
    assert h[1] == pytest.approx(p, abs=1e-12)
    dot = h[2][0] * n[0] + h[2][1] * n[1]
    assert abs(dot) == pytest.approx(1.0, abs=1e-12)


# ---- lights (light.rs) ----------------------------------------------------------------------
def test_point_light_directions(oracle):
    # light.rs:163-174: direction i = (cos 2πi/n, sin 2πi/n) from the position
    rays = oracle.light_rays(S.pack_light(S.PointLight((0.25, -0.5), 8, (1, 1, 1, 1))))
    for i, r in enumerate(rays):
        th = 2 * math.pi * i / 8
        assert r[:2].tolist() == [0.25, -0.5]
        assert r[2:] == pytest.approx([math.cos(th), math.sin(th)], abs=1e-15)


def test_spot_light_fan(oracle):
    # light.rs:225-249: angle_s = atan(dy/dx) - spot/2 + (s/n) spot for s = 1..n, times sign(dx)
    spot = math.pi / 2
    rays = oracle.light_rays(S.pack_light(S.SpotLight((0, 0), spot, (1.0, 0.0), 4, (1, 1, 1, 1))))
    want = [-spot / 2 + s / 4 * spot for s in range(1, 5)]
    for r, a in zip(rays, want):
        assert r[2:] == pytest.approx([math.cos(a), math.sin(a)], abs=1e-15)
    # dx < 0: base angle atan(dy/dx) and the whole fan negated
    rays = oracle.light_rays(S.pack_light(S.SpotLight((0, 0), spot, (-1.0, 0.0), 4, (1, 1, 1, 1))))
    for r, a in zip(rays, want):
        assert r[2:] == pytest.approx([-math.cos(a), -math.sin(a)], abs=1e-15)
    # |dx| below EPSILON: base angle ±π/2 by the sign of dy
    rays = oracle.light_rays(S.pack_light(S.SpotLight((0, 0), spot, (0.0, -1.0), 4, (1, 1, 1, 1))))
    for r, a in zip(rays, want):
        b = -math.pi / 2 + a
        assert r[2:] == pytest.approx([math.cos(b), math.sin(b)], abs=1e-15)


def _ulps(a: float, b: float) -> float:
    """distance in units of the last place of b"""
    return abs(a - b) / math.ulp(max(abs(b), 1e-300))


def test_generator_sincos_and_atan_within_a_few_ulp_of_libm(oracle):
    # the ray generators' own sin / cos / atan (plain IEEE double operations, so the oracle,
    # the GPU and any machine produce the same bits) stay within a few ulp of the C library
    rng = np.random.default_rng(11)
    xs = np.concatenate([rng.uniform(-8.0, 8.0, 20000), 2 * math.pi * np.arange(4096) / 4096,
                         [0.0, -0.0, math.pi / 4, math.pi / 2, math.pi, 1e-300, 5e-9]])
    worst_s = worst_c = 0.0
    for x in xs.tolist():
        s, c = oracle.sincos(x)
        # sin/cos near zero: measure against the ulp of 1 (absolute error of a unit vector)
        worst_s = max(worst_s, abs(s - math.sin(x)) / math.ulp(max(abs(math.sin(x)), 0.5)))
        worst_c = max(worst_c, abs(c - math.cos(x)) / math.ulp(max(abs(math.cos(x)), 0.5)))
    assert worst_s <= 2.0 and worst_c <= 2.0, (worst_s, worst_c)
    worst_a = max(_ulps(oracle.atan(x), math.atan(x))
                  for x in np.concatenate([rng.uniform(-4, 4, 20000), 10.0 ** rng.uniform(-12, 12, 2000),
                                           [0.2679491924311227, 1.0, -1.0, 1e300, -1e300, 0.0]]).tolist())
    assert worst_a <= 4.0, worst_a
    assert oracle.atan(float("inf")) == pytest.approx(math.pi / 2, abs=0) or abs(oracle.atan(float("inf")) - math.pi / 2) < 1e-15
    s, c = oracle.sincos(0.0)
    assert (s, c) == (0.0, 1.0)


def test_directional_light_origins_and_normal(oracle):
    # origins evenly spaced along the segment from a, direction the unit left normal of b - a
    lt = S.DirectionalLight((1, 1, 1, 1), 4, S.LineSegment((-1.0, 0.0), (1.0, 0.0)))
    rays = oracle.light_rays(S.pack_light(lt))
    assert rays[:, 0].tolist() == [-1.0, -0.5, 0.0, 0.5]
    assert rays[:, 1].tolist() == [0.0] * 4
    assert rays[:, 2:] == pytest.approx(np.tile([0.0, 1.0], (4, 1)), abs=1e-15)


def test_light_start_medium(oracle):
    # tracer.rs:280-287: the last object with a material containing the light's origin
    c = S.Object.new_circle((0, 0), 0.5)
    c.material_opt.refractive_index = 1.5
    big = S.Object.new_rect((0, 0), 3.0, 3.0)
    big.material_opt.refractive_index = 1.3
    m = S.Object.new_mirror((-1, 0), (1, 0))
    import ctypes as C
    for objs, pos, want in (([c], (0.1, 0.1), 1.5), ([c], (0.9, 0.0), 1.0), ([c, big], (0.0, 0.2), 1.3),
                            ([big, c], (0.0, 0.2), 1.5), ([m], (0.0, 0.0), 1.0)):
        pk = S.pack(objs, [S.PointLight(pos, 4, (1, 1, 1, 1))])
        got = oracle.lib().lgo_light_medium(pk.geos, pk.n_geo, pk.objects, pk.n_objects, C.byref(pk.lights[0]))
        assert got == want


# ---- shapes (the ray-shape intersections the reference takes from its geometry crate) ----------
def test_circle(oracle):
    # |o + t d - c|² = r²: from (-2, 0) along +x, r = 1: t = 1 and 3, outward normals
    h, fl = hits(oracle, S.Circle((0, 0), 1.0), (-2, 0), (1, 0))
    assert len(h) == 2 and fl == 0
    assert_hit(h[0], 1.0, (-1.0, 0.0), (-1, 0))
    assert_hit(h[1], 3.0, (1.0, 0.0), (1, 0))
    # from the centre only the exit remains (t > t_min)
    h, _ = hits(oracle, S.Circle((0, 0), 1.0), (0, 0), (1, 0))
    assert len(h) == 1
    assert_hit(h[0], 1.0, (1.0, 0.0), (1, 0))
    # a miss
    assert hits(oracle, S.Circle((0, 0), 1.0), (-2, 1.5), (1, 0))[0] == []


def test_circle_far_origin_and_grazing(oracle):
    # roots q/a and c/q with q = -(b + sgn(b) sqrt(disc))/2: exact for these representable cases
    h, _ = hits(oracle, S.Circle((100, 0), 0.5), (0, 0), (1, 0))
    assert [x[0] for x in h] == [99.5, 100.5]
    # grazing chord at height 1 - 1e-8: half-length sqrt(1 - y²)
    y = 1 - 1e-8
    h, _ = hits(oracle, S.Circle((0, 0), 1.0), (-2, y), (1, 0))
    half = math.sqrt((1 - y) * (1 + y))
    assert [x[0] for x in h] == pytest.approx([2 - half, 2 + half], abs=1e-12)


def test_rect_axis_aligned_and_rotated(oracle):
    h, _ = hits(oracle, S.Rect((0, 0), 2.0, 1.0), (-3, 0), (1, 0))
    assert_hit(h[0], 2.0, (-1.0, 0.0), (-1, 0))
    assert_hit(h[1], 4.0, (1.0, 0.0), (1, 0))
    # rotated by 90°: width now along y
    h, _ = hits(oracle, S.Rect((0, 0), 2.0, 1.0, (0.0, 1.0)), (0, -3), (0, 1))
    assert_hit(h[0], 2.0, (0.0, -1.0), (0, -1))
    assert_hit(h[1], 4.0, (0.0, 1.0), (0, 1))
    # through the corner region diagonally: enters on the left face, leaves through the top
    h, _ = hits(oracle, S.Rect((0, 0), 2.0, 2.0), (-2, -0.5), (1 / math.sqrt(2), 1 / math.sqrt(2)))
    assert h[0][1] == pytest.approx((-1.0, 0.5), abs=1e-12)
    assert h[1][1] == pytest.approx((-0.5, 1.0), abs=1e-12)


def test_rect_contains(oracle):
    r = S.Rect((1.0, 1.0), 2.0, 1.0)
    assert contains(oracle, r, (1.9, 1.4))
    assert not contains(oracle, r, (2.1, 1.0))
    assert not contains(oracle, r, (1.0, 1.6))


def test_segment(oracle):
    # 2x2 solve o + t d = a + s (b - a), s in [0, 1]
    h, _ = hits(oracle, S.LineSegment((0, -1), (0, 1)), (-1, 0.5), (1, 0))
    assert len(h) == 1
    assert_hit(h[0], 1.0, (0.0, 0.5), (1, 0))
    assert hits(oracle, S.LineSegment((0, -1), (0, 1)), (-1, 1.5), (1, 0))[0] == []
    # parallel ray: no hit
    assert hits(oracle, S.LineSegment((0, -1), (0, 1)), (-1, 0.0), (0, 1))[0] == []


def test_cubic_bezier(oracle):
    # evenly spaced x control points make x(s) = -1 + 2s; y(s) = 3 s (1 - s).  The vertical
    # ray x = 0 meets s = 1/2 at y = 3/4; the tangent there is (2, 0), so the normal is ±y.
    cb = S.CubicBezier(((-1, 0), (-1 / 3, 1), (1 / 3, 1), (1, 0)))
    h, _ = hits(oracle, cb, (0, -1), (0, 1))
    assert len(h) == 1
    assert_hit(h[0], 1.75, (0.0, 0.75), (0, 1))
    # a horizontal ray at y = 0.5 crosses twice: 3 s (1 - s) = 1/2
    h, _ = hits(oracle, cb, (-2, 0.5), (1, 0))
    s = [(1 - math.sqrt(1 / 3)) / 2, (1 + math.sqrt(1 / 3)) / 2]
    assert [x[1][0] for x in h] == pytest.approx([-1 + 2 * v for v in s], abs=1e-12)
    for x, v in zip(h, s):  # normal ⟂ tangent (2, 3 - 6 s)
        tx, ty = 2.0, 3 - 6 * v
        assert abs(x[2][0] * tx + x[2][1] * ty) < 1e-12


def test_cubic_three_crossings(oracle):
    # y(s) = 4 (s - 1/2)^3-like S curve: control points (−1,−1), (−1/3, 3), (1/3, −3), (1, 1)
    # give y(s) = -1 + 12 s - 30 s² + 20 s³, which crosses y = 0 three times in (0, 1)
    cb = S.CubicBezier(((-1, -1), (-1 / 3, 3), (1 / 3, -3), (1, 1)))
    h, _ = hits(oracle, cb, (-2, 0.0), (1, 0))
    roots = sorted(r.real for r in np.roots([20, -30, 12, -1]) if abs(r.imag) < 1e-12 and 0 <= r.real <= 1)
    assert len(roots) == 3
    assert [x[1][0] for x in h] == pytest.approx([-1 + 2 * v for v in roots], abs=1e-11)


def test_csg_and_or_and_not(oracle):
    A, B = S.Circle((-0.5, 0), 1.0), S.Circle((0.5, 0), 1.0)
    # And: [-0.5, 0.5]
    h, _ = hits(oracle, A & B, (-3, 0), (1, 0))
    assert [x[0] for x in h] == pytest.approx([2.5, 3.5])
    # Or: [-1.5, 1.5]
    h, _ = hits(oracle, A | B, (-3, 0), (1, 0))
    assert [x[0] for x in h] == pytest.approx([1.5, 4.5])
    # AndNot: [-1.5, -0.5)
    h, _ = hits(oracle, A.and_not(B), (-3, 0), (1, 0))
    assert [x[0] for x in h] == pytest.approx([1.5, 2.5])
    for g, p, want in ((A & B, (0, 0), True), (A & B, (-1, 0), False), (A | B, (-1, 0), True),
                       (A | B, (1.6, 0), False), (A.and_not(B), (-1, 0), True), (A.and_not(B), (0, 0), False)):
        assert contains(oracle, g, p) == want


def test_csg_local_frame(oracle):
    # Lens::new (object.rs:393-411): And of circles at (±d/2, 0) in the node's frame; rotate
    # by 90° and move to (0.5, 0.5): the lens spans y in [0.4, 0.6] along x = 0.5
    lens = S.Logic(abi.LG_OP_AND, S.Circle((1.9, 0), 2.0), S.Circle((-1.9, 0), 2.0), (0.5, 0.5), (0.0, 1.0))
    h, _ = hits(oracle, lens, (0.5, -3), (0, 1))
    assert [x[0] for x in h] == pytest.approx([3.4, 3.6], abs=1e-12)
    assert contains(oracle, lens, (0.5, 0.5))
    # at y = 0.5 the lens spans |x - 0.5| <= sqrt(2² - 1.9²)
    assert contains(oracle, lens, (0.5 + 0.62, 0.5))
    assert not contains(oracle, lens, (0.5 + 0.63, 0.5))
    assert not contains(oracle, lens, (0.5, 0.61))


def test_mirror_never_contains(oracle):
    # object.rs:243-244: mirrors contain nothing, even points on the mirror
    assert not contains(oracle, S.LineSegment((0, -1), (0, 1)), (0, 0))


# ---- optics ---------------------------------------------------------------------------------
def test_fresnel_normal_incidence(oracle):
    # R = ((n1 - n2)/(n1 + n2))² = 0.04 for 1 → 1.5; refracted straight through
    rl, rr, R = oracle.refract((1, 0), (-1, 0), 1.0, 1.5)
    assert R == pytest.approx(0.04, abs=1e-15)
    assert rl == pytest.approx((-1, 0)) and rr == pytest.approx((1, 0))
    # the normal's orientation does not matter
    assert oracle.refract((1, 0), (1, 0), 1.0, 1.5) == (rl, rr, R)


def test_snell_and_fresnel_oblique(oracle):
    n1, n2, th = 1.0, 1.5, math.radians(30)
    d = (math.sin(th), -math.cos(th))
    rl, rr, R = oracle.refract(d, (0, 1), n1, n2)
    tt = math.asin(n1 / n2 * math.sin(th))
    assert rr == pytest.approx((math.sin(tt), -math.cos(tt)), abs=1e-14)
    assert rl == pytest.approx((math.sin(th), math.cos(th)), abs=1e-14)
    rs = ((n1 * math.cos(th) - n2 * math.cos(tt)) / (n1 * math.cos(th) + n2 * math.cos(tt))) ** 2
    rp = ((n1 * math.cos(tt) - n2 * math.cos(th)) / (n1 * math.cos(tt) + n2 * math.cos(th))) ** 2
    assert R == pytest.approx((rs + rp) / 2, abs=1e-14)


def test_brewster_angle(oracle):
    # at tan θ = n2/n1 the p-polarised reflectance vanishes: R = Rs / 2
    n1, n2 = 1.0, 1.5
    th = math.atan(n2 / n1)
    tt = math.pi / 2 - th
    _, _, R = oracle.refract((math.sin(th), -math.cos(th)), (0, 1), n1, n2)
    assert R == pytest.approx(0.5 * (math.sin(th - tt) / math.sin(th + tt)) ** 2, abs=1e-14)


def test_total_internal_reflection(oracle):
    th = math.radians(60)  # above the critical angle asin(1/1.5) = 41.8°
    rl, rr, R = oracle.refract((math.sin(th), -math.cos(th)), (0, 1), 1.5, 1.0)
    assert rr is None and R == 1.0
    assert rl == pytest.approx((math.sin(th), math.cos(th)), abs=1e-15)


# ---- the trace (tracer.rs:360-493) ------------------------------------------------------------
def one_ray_scene(max_bounce=8):
    p = abi.params_default()
    p.max_bounce = max_bounce
    p.emit_control_lines = 0
    c = S.Object.new_circle((0, 0), 0.2)
    c.material_opt.refractive_index = 1.5
    m = S.Object.new_mirror((0.6, -0.5), (0.6, 0.5))
    return S.pack([c, m], [S.PointLight((-0.8, 0), 1, (1, 1, 1, 1))], p)


def test_trace_one_ray_on_axis(oracle):
    """One ray along the axis of a glass disc (n = 1.5) in front of a mirror: every interface
    is at normal incidence, so every colour is a product of R = 0.04 and T = 0.96."""
    segs, paths, s64, st = oracle.trace(one_ray_scene(), threads=1)
    by = {(int(q["gen"]), int(q["path"])): (tuple(e), tuple(float(c) for c in s["color"]))
          for q, e, s in zip(paths, s64, segs)}
    R, T = 0.04, 0.96
    want = {
        (0, 0): ((-0.8, 0, -0.2, 0), 1.0),           # to the disc
        (1, 0): ((-0.2, 0, -1.0, 0), R),             # reflected back out of the canvas
        (1, 1): ((-0.2, 0, 0.2, 0), T),              # through the disc
        (2, 1): ((0.2, 0, -0.2, 0), T * R),          # internal reflection
        (2, 3): ((0.2, 0, 0.6, 0), T * T),           # out to the mirror
        (3, 3): ((0.6, 0, 0.2, 0), T * T),           # mirror: full reflection
        (3, 1): ((-0.2, 0, 0.2, 0), T * R * R),
        (3, 5): ((-0.2, 0, -1.0, 0), T * R * T),
    }
    for k, (e, c) in want.items():
        assert k in by, k
        assert by[k][0] == pytest.approx(e, abs=1e-15)
        assert by[k][1][:3] == pytest.approx((c, c, c), rel=1e-6)
        assert by[k][1][3] == 1.0  # alpha is never split (tracer.rs:454-471)
    assert int(st.primary_rays) == 1
    assert len(segs) == int(st.segments)
    assert max(int(q["gen"]) for q in paths) == 7  # max_bounce generations


def test_trace_cutoff(oracle):
    # tracer.rs:378-384: an entry with r, g, b all below the cutoff (or alpha below it) is skipped
    pk = one_ray_scene()
    pk.params.cutoff_color[:] = (0.05, 0.05, 0.05, 0.0)
    segs, paths, _, _ = oracle.trace(pk, threads=1)
    assert all(min(float(s["color"][0]), 1.0) >= 0.05 for s in segs)
    assert len(segs) < len(oracle.trace(one_ray_scene(), threads=1)[0])


def test_trace_max_bounce(oracle):
    for mb in (1, 2, 3):
        _, paths, _, _ = oracle.trace(one_ray_scene(mb), threads=1)
        assert max(int(q["gen"]) for q in paths) == mb - 1


def test_trace_miss_goes_to_canvas_exit(oracle):
    p = abi.params_default()
    p.width, p.height = 1024, 512  # canvas [-2, 2] x [-1, 1]
    pk = S.pack([], [S.PointLight((0.5, 0.25), 4, (1, 1, 1, 1))], p)
    segs, _, s64, _ = oracle.trace(pk, threads=1)
    ends = sorted(tuple(np.round(e[2:], 12)) for e in s64)
    assert ends == sorted([(2.0, 0.25), (0.5, 1.0), (-2.0, 0.25), (0.5, -1.0)])


def test_trace_light_outside_canvas_emits_nothing_when_pointing_away(oracle):
    p = abi.params_default()
    pk = S.pack([], [S.SpotLight((3.0, 0.0), 0.1, (1.0, 0.0), 8, (1, 1, 1, 1))], p)
    segs, _, _, _ = oracle.trace(pk, threads=1)
    assert len(segs) == 0


def test_trace_is_thread_count_independent(oracle):
    from light_garden_gb300 import workloads as W
    pk = W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed()
    a = oracle.trace(pk, threads=1)
    b = oracle.trace(pk, threads=4)

    def canon(r):
        segs, paths, s64, _ = r
        order = np.lexsort((paths["path"], paths["gen"], paths["primary"], paths["light"], paths["source"]))
        return segs[order].tobytes(), s64[order].tobytes()
    assert canon(a) == canon(b)


# ---- raster, fixed point, resolve -----------------------------------------------------------
def raster_params(w=8, h=8):
    p = abi.params_default()
    p.width, p.height = w, h
    return p


def seg(x0, y0, x1, y1, c=(0.5, 0.25, 1.0, 1.0)):
    s = np.zeros(1, abi.segment_dtype())
    s[0]["x0"], s[0]["y0"], s[0]["x1"], s[0]["y1"] = x0, y0, x1, y1
    s[0]["color"] = c
    return s


def test_fixed_point(oracle):
    L = oracle.lib()
    assert L.lgo_fixed(1.0) == 1 << 32
    assert L.lgo_fixed(-1.5) == -(3 << 31)
    assert L.lgo_fixed(float("nan")) == 0
    assert L.lgo_fixed(float("inf")) == 1 << 52  # clamped to ±2^20
    assert L.lgo_fixed(-float("inf")) == -(1 << 52)
    assert L.lgo_fixed(2.0 ** -32) == 1


def test_raster_horizontal_row(oracle):
    # px = x H/2 + W/2, py = H/2 - y H/2; x in [-1, 1] covers pixel centres 0.5 .. 7.5 and
    # y = 0.125 puts the line on py = 3.5, row 3
    p = raster_params()
    acc, px = oracle.raster(seg(-1, 0.125, 1, 0.125), p)
    assert px == 8
    one = 1 << 32
    ref = np.zeros((8, 8, 4), np.int64)
    ref[:, :, 3] = one  # clear colour (0, 0, 0, 1)
    ref[3, :, :3] = [one // 2, one // 4, one]  # One/One Add
    ref[3, :, 3] += one  # SrcAlpha/One Add: a·a = 1
    assert (acc == ref).all()
    assert (oracle.clear(p) == np.where(np.arange(4) == 3, one, 0)).all()


def test_raster_half_open_and_empty(oracle):
    p = raster_params()
    # a degenerate segment covers no pixel centre
    assert oracle.raster(seg(0.1, 0.1, 0.1, 0.1), p)[1] == 0
    # one pixel long, starting on a centre: exactly one sample ([3.5, 4.5) holds centre 3.5)
    x0 = (3.5 - 4) / 4
    acc, px = oracle.raster(seg(x0, 0.125, x0 + 0.25, 0.125), p)
    assert px == 1 and acc[3, 3, 0] == 1 << 31
    # a segment ending exactly on a centre does not touch it
    acc, px = oracle.raster(seg(x0 - 0.25, 0.125, x0, 0.125), p)
    assert px == 1 and acc[3, 2, 0] == 1 << 31 and acc[3, 3, 0] == 0


def test_raster_vertical_and_diagonal(oracle):
    p = raster_params()
    acc, px = oracle.raster(seg(0.125, -1, 0.125, 1), p)  # column 4
    assert px == 8 and (acc[:, 4, 2] == 1 << 32).all()
    acc, px = oracle.raster(seg(-1, 1, 1, -1), p)  # the main diagonal
    assert px == 8
    assert [int(acc[i, i, 2] > 0) for i in range(8)] == [1] * 8


def test_raster_clips_to_the_canvas(oracle):
    p = raster_params()
    acc, px = oracle.raster(seg(-10, 0.125, 10, 0.125), p)
    assert px == 8
    assert oracle.raster(seg(-10, 5, 10, 5), p)[1] == 0


def test_raster_min_max_blend(oracle):
    p = raster_params()
    p.color_blend = abi.lg_blend_component(abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_MAX)
    s = np.concatenate([seg(-1, 0.125, 1, 0.125, (0.5, 0.1, 0.2, 1.0)),
                        seg(-1, 0.125, 1, 0.125, (0.25, 0.3, 0.1, 1.0))])
    acc, _ = oracle.raster(s, p)
    assert acc[3, 0, :3].tolist() == [1 << 31, oracle.lib().lgo_fixed(np.float32(0.3)),
                                      oracle.lib().lgo_fixed(np.float32(0.2))]


def test_resolve_f16_rounding(oracle):
    L = oracle.lib()
    assert L.lgo_f32_to_f16(1.0) == 0x3C00
    assert L.lgo_f32_to_f16(0.5) == 0x3800
    assert L.lgo_f32_to_f16(65504.0) == 0x7BFF
    assert L.lgo_f32_to_f16(65520.0) == 0x7C00  # rounds to infinity
    assert L.lgo_f32_to_f16(2.0 ** -24) == 0x0001  # smallest subnormal
    assert L.lgo_f32_to_f16(2.0 ** -25) == 0x0000  # tie to even
    assert L.lgo_f32_to_f16(3 * 2.0 ** -25) == 0x0002  # tie to even
    assert L.lgo_f32_to_f16(-2.0) == 0xC000
    vals = np.float32([0.1, 1 / 3, 1000.1, 1e-5, -7.25])
    assert [L.lgo_f32_to_f16(float(v)) for v in vals] == vals.astype(np.float16).view(np.uint16).tolist()


def test_resolve_images(oracle):
    acc = np.zeros((1, 6, 4), np.int64)
    for i, v in enumerate([0, 1.0, 0.5, 2.0, -1.0, 0.25]):
        acc[0, i, :] = int(v * 2 ** 32)
    f16 = oracle.resolve_f16(acc)
    assert f16[0, :, 0].tolist() == np.float16([0, 1, 0.5, 2, -1, 0.25]).view(np.uint16).tolist()
    # renderer.rs:325-328: u8 = sat(f^(1/2.2) · 255), truncated
    rgba = oracle.resolve_rgba8(acc)
    assert rgba[0, :, 0].tolist() == [0, 255, int(0.5 ** (1 / 2.2) * 255), 255, 0, int(0.25 ** (1 / 2.2) * 255)]


def test_ellipse(oracle):
    # x^2/4 + y^2 = 1: the x axis meets it at +-2, the y axis at +-1
    e = S.Ellipse((0.0, 0.0), 2.0, 1.0)
    h, _ = hits(oracle, e, (-3, 0), (1, 0))
    assert_hit(h[0], 1.0, (-2.0, 0.0), (-1, 0))
    assert_hit(h[1], 5.0, (2.0, 0.0), (1, 0))
    # at (sqrt(2), 1/sqrt(2)) the gradient (x/4, y) points along (1, 2)/sqrt(5)
    s2 = math.sqrt(2.0)
    h, _ = hits(oracle, e, (s2, -3), (0, 1))
    assert h[1][1] == pytest.approx((s2, 1 / s2), abs=1e-12)
    assert h[1][2] == pytest.approx((1 / math.sqrt(5), 2 / math.sqrt(5)), abs=1e-12)
    # rotated by 90 degrees: the long axis along y
    h, _ = hits(oracle, S.Ellipse((0.0, 0.0), 2.0, 1.0, (0.0, 1.0)), (0, -3), (0, 1))
    assert [x[0] for x in h] == pytest.approx([1.0, 5.0], abs=1e-12)
    assert contains(oracle, e, (1.9, 0.0)) and not contains(oracle, e, (1.5, 0.7))


def test_convex_polygon(oracle):
    # a unit square written as a polygon hits like the rect of the same size
    sq = S.ConvexPolygon(((-0.5, -0.5), (0.5, -0.5), (0.5, 0.5), (-0.5, 0.5)))
    rect = S.Rect((0.0, 0.0), 1.0, 1.0)
    for o, d in (((-2, 0.1), (1, 0)), ((0.3, -2), (0.2, 1)), ((-1, -0.9), (1, 1))):
        hp, _ = hits(oracle, sq, o, d)
        hr, _ = hits(oracle, rect, o, d)
        assert [x[0] for x in hp] == pytest.approx([x[0] for x in hr], abs=1e-12)
        for a, b in zip(hp, hr):
            assert a[2] == pytest.approx(b[2], abs=1e-12)
    # clockwise vertices give the same solid
    cw = S.ConvexPolygon(tuple(reversed(sq.points)))
    assert [x[0] for x in hits(oracle, cw, (-2, 0.1), (1, 0))[0]] == pytest.approx([1.5, 2.5])
    # a regular heptagon (more vertices than one record holds), in a rotated frame
    hept = S.ConvexPolygon(tuple((math.cos(2 * math.pi * k / 7), math.sin(2 * math.pi * k / 7)) for k in range(7)),
                           (0.5, 0.25), (0.0, 1.0))
    assert contains(oracle, hept, (0.5, 0.25)) and not contains(oracle, hept, (1.6, 0.25))
    # vertex 0 maps to (0.5, 1.25): a vertical ray just beside it crosses two edges, the exit
    # on the two edges meeting there
    h, fl = hits(oracle, hept, (0.51, -3), (0, 1))
    assert len(h) == 2 and fl == 0
    top = h[1][1][1]
    assert 1.2 < top < 1.25
    # straight through the vertex both edges report it, and the decision is flagged
    h, _ = hits(oracle, hept, (0.5, -3), (0, 1))
    assert len(h) == 3 and h[1][0] == pytest.approx(h[2][0], abs=1e-12)
    assert S.convex_hull([(0, 0), (1, 0), (0.5, 0.2), (1, 1), (0, 1), (0.5, 0.5)]) == ((0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0))


# ---- string mod (string_mod.rs:33-150) ------------------------------------------------------
def sm_params(m, num, mode, curve=abi.LG_CURVE_CIRCLE, turns=1, colors=(), cf=(0.0, 0.0), cu=(0, 0, 0)):
    p = abi.params_default()
    sm = p.string_mod
    sm.modulo, sm.num, sm.mode, sm.curve, sm.turns = m, num, mode, curve, turns
    sm.color[:] = (0.3, 0.3, 0.3, 1.0)
    sm.curve_f[:] = cf
    sm.curve_u[:] = cu
    abi.set_mod_colors(p, colors)
    return p


def test_string_mod_modes_on_the_circle(oracle):
    m = 12
    ang = lambda n: 2 * math.pi * n / m
    for mode, target in ((abi.LG_SM_ADD, lambda i: (i + 5) % m), (abi.LG_SM_MUL, lambda i: (i * 5) % m),
                         (abi.LG_SM_POW, lambda i: pow(i, 5, m)), (abi.LG_SM_BASE, lambda i: pow(5, i, m))):
        ch = oracle.string_mod_chords(sm_params(m, 5, mode))
        assert len(ch) == m
        for i in range(m):
            j = target(i)
            assert ch[i]["x0"] == pytest.approx(math.cos(ang(i)), abs=1e-7)
            assert ch[i]["y0"] == pytest.approx(math.sin(ang(i)), abs=1e-7)
            assert ch[i]["x1"] == pytest.approx(math.cos(ang(j)), abs=1e-7)
            assert ch[i]["y1"] == pytest.approx(math.sin(ang(j)), abs=1e-7)


def test_string_mod_modulo_colours_are_averaged(oracle):
    red, blue = (1.0, 0.0, 0.0, 1.0), (0.0, 0.0, 1.0, 0.5)
    ch = oracle.string_mod_chords(sm_params(12, 1, abi.LG_SM_ADD, colors=[(2, 0, red), (3, 0, blue)]))
    assert ch[1]["color0"].tolist() == pytest.approx([0.3, 0.3, 0.3, 1.0])  # no entry matches 1
    assert ch[2]["color0"].tolist() == list(red)
    assert ch[3]["color0"].tolist() == list(blue)
    assert ch[6]["color0"].tolist() == [0.5, 0.0, 0.5, 0.75]  # both match: the mean
    # the second vertex takes the colour of its own point (i + 1)
    assert ch[5]["color1"].tolist() == [0.5, 0.0, 0.5, 0.75] and ch[1]["color1"].tolist() == list(red)
    with pytest.raises(oracle.OracleError):  # ix % 0 is undefined in the reference
        oracle.string_mod_chords(sm_params(12, 1, abi.LG_SM_ADD, colors=[(0, 0, red)]))


def test_string_mod_curves(oracle):
    m = 64
    th = 2 * math.pi / 40
    ch = oracle.string_mod_chords(sm_params(m, 3, abi.LG_SM_MUL, abi.LG_CURVE_COMPLEX_EXP,
                                            cf=(math.cos(th), math.sin(th))))
    for i in (0, 1, 7, 63):  # c^n on the unit circle = (cos n th, sin n th)
        assert ch[i]["x0"] == pytest.approx(math.cos(i * th), abs=1e-6)
        assert ch[i]["y0"] == pytest.approx(math.sin(i * th), abs=1e-6)
    r, s, d = 3, 5, 2
    ch = oracle.string_mod_chords(sm_params(m, 3, abi.LG_SM_MUL, abi.LG_CURVE_HYPOTROCHOID, turns=2, cu=(r, s, d)))
    for i in (0, 5, 33):
        a = 2 * i * 2 * math.pi / m
        k = s - r
        assert ch[i]["x0"] == pytest.approx((k * math.cos(a) + d * math.cos(a * k / r)) / (k + d), abs=1e-6)
        assert ch[i]["y0"] == pytest.approx((k * math.sin(a) - d * math.sin(a * k / r)) / (k + d), abs=1e-6)
    ch = oracle.string_mod_chords(sm_params(m, 3, abi.LG_SM_MUL, abi.LG_CURVE_LISSAJOUS, cf=(0.5, 0.0), cu=(3, 4, 0)))
    for i in (0, 9, 40):
        a = i * 2 * math.pi / m
        assert ch[i]["x0"] == pytest.approx(math.sin(3 * a + 0.5), abs=1e-6)
        assert ch[i]["y0"] == pytest.approx(math.sin(4 * a), abs=1e-6)


# ---- nested string mods (StringMod::line_crossings_as_points, string_mod.rs:87-102, 152-158) ---
def nested_mod(m, num, mode, colors=(), color=(0.6, 0.2, 0.1, 1.0)):
    ns = abi.lg_string_mod()
    ns.modulo, ns.num, ns.mode = m, num, mode
    ns.color[:] = color
    holder = abi.params_default()
    abi.set_mod_colors(holder, colors)
    ns.n_colors, ns.colors = holder.string_mod.n_colors, holder.string_mod.colors
    return ns


def _target(m, num, mode, i):
    if mode == abi.LG_SM_ADD:
        return (i + num) % m
    if mode == abi.LG_SM_MUL:
        return (i * num) % (1 << 64) % m
    if mode == abi.LG_SM_POW:
        return pow(i, num & 0xffffffff, 1 << 64) % m
    return pow(num, i & 0xffffffff, 1 << 64) % m


def _cpow(re, im, e):
    # binary powering with each product rounded on its own (Python floats are IEEE doubles)
    if e == 0:
        return 1.0, 0.0
    br, bi = re, im
    while e & 1 == 0:
        br, bi = br * br - bi * bi, br * bi + bi * br
        e >>= 1
    if e == 1:
        return br, bi
    ar, ai = br, bi
    while e > 1:
        e >>= 1
        br, bi = br * br - bi * bi, br * bi + bi * br
        if e & 1:
            ar, ai = ar * br - ai * bi, ar * bi + ai * br
    return ar, ai


def _cross(a, b, c, d):
    rx, ry, sx, sy = b[0] - a[0], b[1] - a[1], d[0] - c[0], d[1] - c[1]
    den = rx * sy - ry * sx
    if den == 0.0:
        return None
    wx, wy = c[0] - a[0], c[1] - a[1]
    t = (wx * sy - wy * sx) / den
    u = (wx * ry - wy * rx) / den
    if not (0.0 <= t <= 1.0 and 0.0 <= u <= 1.0):
        return None
    return a[0] + rx * t, a[1] + ry * t


def test_segment_crossing_known_answers(oracle):
    """The crossing definition of nested string mods: a + t (b - a) = c + u (d - c) with a
    non-zero determinant and t, u in [0, 1] (both ends included)."""
    # an X: the diagonals of the unit square cross at its centre, t = u = 1/2 exactly
    assert oracle.seg_cross((0, 0), (1, 1), (0, 1), (1, 0)) == (0.5, 0.5)
    # a T: c d passes through b, t = 1 exactly, u = 1/2
    assert oracle.seg_cross((0, 0), (1, 0), (1, -1), (1, 1)) == (1.0, 0.0)
    # sharing an end point: w = c - a = 0, so t = u = 0
    assert oracle.seg_cross((0.25, 0.5), (1, 2), (0.25, 0.5), (-3, 1)) == (0.25, 0.5)
    # stopping short of the other line (t > 1), and missing its extent (u > 1)
    assert oracle.seg_cross((0, 0), (0.9, 0), (1, -1), (1, 1)) is None
    assert oracle.seg_cross((0, 0), (2, 0), (1, 0.5), (1, 2)) is None
    # parallel, collinear and overlapping, and a zero-length line: the determinant is 0
    assert oracle.seg_cross((0, 0), (1, 0), (0, 1), (1, 1)) is None
    assert oracle.seg_cross((0, 0), (2, 0), (1, 0), (3, 0)) is None
    assert oracle.seg_cross((0.5, 0.5), (0.5, 0.5), (0, 0), (1, 1)) is None
    # the point is taken on the first line: a + t (b - a)
    p = oracle.seg_cross((0, 0), (3, 1), (0, 1), (3, 0))
    assert p == (0 + 3 * 0.5, 0 + 1 * 0.5)


def test_nested_string_mod_restated_bit_for_bit(oracle):
    """The crossings and the nested lines restated in Python on the complex-power curve (whose
    points are products only, so the restatement is exact): the oracle's FP64 crossing points,
    their order (diff outer, line inner, every crossing twice) and the nested lines' f32
    endpoints and averaged colours equal it bit for bit."""
    m, num, mode = 48, 5, abi.LG_SM_MUL
    th = 2 * math.pi / 48
    c = (0.999 * math.cos(th), 0.999 * math.sin(th))
    p = sm_params(m, num, mode, abi.LG_CURVE_COMPLEX_EXP, turns=1, cf=c)
    pts = [_cpow(c[0], c[1], (1 * n) & 0xffffffff) for n in range(m)]
    lines = [(pts[i % m], pts[_target(m, num, mode, i) % m]) for i in range(m)]
    want = []
    for diff in range(1, m):
        for a in range(m):
            q = _cross(*lines[a], *lines[(a + diff) % m])
            if q is not None:
                want.append(q)
    got = oracle.string_mod_crossings(p.string_mod)
    assert len(want) > 500
    assert got.tolist() == [list(q) for q in want]
    red, blue = (1.0, 0.0, 0.0, 1.0), (0.0, 0.2, 1.0, 0.5)
    table = [(3, 1, red), (4, 0, blue)]
    ns = nested_mod(700, 11, abi.LG_SM_ADD, table)
    abi.set_nested(p, ns)
    ch = oracle.string_mod_chords(p)
    assert len(ch) == 700

    def colour(ix):
        hit = [col for (mo, r, col) in table if ix % mo == r]
        if not hit:
            return [np.float32(v) for v in (0.6, 0.2, 0.1, 1.0)]
        acc = [np.float32(0.0)] * 4
        for col in hit:
            acc = [np.float32(a + np.float32(v)) for a, v in zip(acc, col)]
        return [np.float32(a / np.float32(len(hit))) for a in acc]

    n = len(want)
    for i in range(700):
        j = (i + 11) % 700
        a, b = want[i % n], want[j % n]
        assert (ch[i]["x0"], ch[i]["y0"], ch[i]["x1"], ch[i]["y1"]) == \
            tuple(np.float32(v) for v in (a[0], a[1], b[0], b[1]))
        assert ch[i]["color0"].tolist() == [float(v) for v in colour(i)]
        assert ch[i]["color1"].tolist() == [float(v) for v in colour(j)]


def test_nested_string_mod_known_answers(oracle):
    # two diameters, each drawn both ways (ADD 2 on 4 circle points): a horizontal and a vertical
    # line cross at the centre, a line and its reverse are parallel (determinant exactly 0):
    # 8 crossings, all at the origin up to the rounding of cos(pi / 2)
    p = sm_params(4, 2, abi.LG_SM_ADD)
    got = oracle.string_mod_crossings(p.string_mod)
    assert got.shape == (8, 2) and np.abs(got).max() < 1e-15
    abi.set_nested(p, nested_mod(5, 1, abi.LG_SM_ADD))
    assert len(oracle.string_mod_chords(p)) == 5
    # every line from a point to itself (ADD 0): no crossings, so no nested lines
    p = sm_params(16, 0, abi.LG_SM_ADD)
    assert len(oracle.string_mod_crossings(p.string_mod)) == 0
    abi.set_nested(p, nested_mod(9, 1, abi.LG_SM_ADD))
    assert len(oracle.string_mod_chords(p)) == 0
    # a nested mod of modulo 0 draws nothing; an outer mod of modulo 0 disables the overlay
    p = sm_params(12, 5, abi.LG_SM_MUL)
    abi.set_nested(p, nested_mod(0, 1, abi.LG_SM_ADD))
    assert len(oracle.string_mod_chords(p)) == 0
    p = sm_params(0, 5, abi.LG_SM_MUL)
    abi.set_nested(p, nested_mod(9, 1, abi.LG_SM_ADD))
    assert len(oracle.string_mod_chords(p)) == 0
    # limits: the outer modulo of a nested mod, the nested mode and colour table
    p = sm_params(abi.LG_STRING_MOD_NESTED_MAX + 1, 5, abi.LG_SM_MUL)
    abi.set_nested(p, nested_mod(9, 1, abi.LG_SM_ADD))
    with pytest.raises(oracle.OracleError):
        oracle.string_mod_chords(p)
    p = sm_params(12, 5, abi.LG_SM_MUL)
    abi.set_nested(p, nested_mod(9, 1, 7))
    with pytest.raises(oracle.OracleError):
        oracle.string_mod_chords(p)
    abi.set_nested(p, nested_mod(9, 1, abi.LG_SM_ADD, [(0, 0, (1, 1, 1, 1))]))
    with pytest.raises(oracle.OracleError):
        oracle.string_mod_chords(p)


def test_chord_colour_is_interpolated_along_the_major_axis(oracle):
    p = raster_params()
    ch = np.zeros(2, abi.chord_dtype())
    ch[0]["x0"], ch[0]["y0"], ch[0]["x1"], ch[0]["y1"] = -1, 0.125, 1, 0.125  # row 3, left to right
    ch[0]["color0"], ch[0]["color1"] = (0, 0, 0, 1), (1, 1, 1, 1)
    ch[1]["x0"], ch[1]["y0"], ch[1]["x1"], ch[1]["y1"] = 0.125, -1, 0.125, 1  # column 4, bottom to top
    ch[1]["color0"], ch[1]["color1"] = (1, 0, 0, 1), (0, 0, 1, 1)
    acc, px = oracle.raster(np.zeros(0, abi.segment_dtype()), p, chords=ch[:1])
    assert px == 8
    # sample i sits at i + 1/2 of the 8-pixel span: f = (i + 1/2) / 8
    assert [int(acc[3, i, 0]) for i in range(8)] == [int((i + 0.5) / 8 * 2 ** 32) for i in range(8)]
    acc, px = oracle.raster(np.zeros(0, abi.segment_dtype()), p, chords=ch[1:])
    # y grows downwards in pixel space: row 7 is the first vertex (y = -1), row 0 the second
    assert [int(acc[j, 4, 2]) for j in range(8)] == [int((7 - j + 0.5) / 8 * 2 ** 32) for j in range(8)]
    assert [int(acc[j, 4, 0]) for j in range(8)] == [int((j + 0.5) / 8 * 2 ** 32) for j in range(8)]
