"""Seeded synthetic scenes with the shapes, sizes and value distributions of the five
benchmark configurations of the trace-and-accumulate path.

The reference publishes no benchmark scenes; its only scene file is ``default.ron``.  These
generators stand in for the configurations:

* :func:`plain_small`   1 point light (4096 rays) + circle (r 0.2, n 1.5) + flat mirror,
                        8 bounces, 512x512, FP32 accumulation;
* :func:`mid_scene`     64 objects (rect / circle / mirror / curved mirror), 8 lights x 2^18
                        rays, 16 bounces, 1920x1080, 64-bit fixed point;
* :func:`csg_scene`     256 CSG objects (circle op rect), 2^22 rays, 32 bounces, 4096x4096,
                        string-mod overlay (m = 4096, chords i -> 7 i mod m);
* :func:`batch_scenes`  mixed sizes: objects log-uniform [4, 1024], rays log-uniform
                        [2^12, 2^20], bounces U{4..32}, canvases {256, 512, 1024, 2048}^2;
* :func:`string_mod_art` string-mod line art on each of the four curves, with modulo colours.
* :func:`nested_string_mod_art` a nested string mod over the crossings of one of those.

Choices the configurations leave open (spot angle U[10, 90] degrees, directional segment
length U[0.1, 0.5], the curved-mirror template, the CSG child placement) are made here
and fixed by the seed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import abi
from .scene import (Circle, ConvexPolygon, CubicBezier, DirectionalLight, Ellipse, LineSegment, Logic, Material,
                    Object, PackedScene, PointLight, Rect, SpotLight, convex_hull, pack)

# control polygon of a curved mirror in its local frame (an arch), scaled by the object size
_CUBIC_TEMPLATE = np.array([[-1.0, -0.5], [-0.35, 0.6], [0.35, 0.6], [1.0, -0.5]])


@dataclass
class Workload:
    name: str
    objects: List[Object]
    lights: list
    params: abi.lg_params

    def packed(self) -> PackedScene:
        return pack(self.objects, self.lights, self.params)

    @property
    def primary_rays(self) -> int:
        return int(sum(l.num_rays for l in self.lights))


def _params(max_bounce: int, width: int, height: int, accum: int) -> abi.lg_params:
    p = abi.params_default()
    p.max_bounce = max_bounce
    p.width, p.height = width, height
    p.accum = accum
    return p


def plain_small(accum: int = abi.LG_ACCUM_F32, num_rays: int = 4096) -> Workload:
    objects = [
        Object(abi.LG_OBJ_CIRCLE, Circle((0.0, 0.0), 0.2), Material(1.5)),
        Object.new_mirror((0.6, -0.5), (0.6, 0.5)),
    ]
    lights = [PointLight((-0.8, 0.0), num_rays, (1.0, 1.0, 1.0, 1.0))]
    return Workload("plain_small", objects, lights, _params(8, 512, 512, accum))


def _rand_rot(rng) -> tuple:
    a = rng.uniform(0.0, 2.0 * math.pi)
    return (math.cos(a), math.sin(a))


def _rand_object(rng, kind: str) -> Object:
    c = tuple(rng.uniform(-1.0, 1.0, 2))
    size = rng.uniform(0.02, 0.15)
    cs = _rand_rot(rng)
    n = rng.uniform(1.3, 1.8)
    if kind == "circle":
        return Object(abi.LG_OBJ_CIRCLE, Circle(c, size), Material(n))
    if kind == "rect":
        hh = rng.uniform(0.02, 0.15)
        return Object(abi.LG_OBJ_RECT, Rect(c, 2.0 * size, 2.0 * hh, cs), Material(n))
    if kind == "mirror":
        d = np.array(cs) * size
        return Object.new_mirror((c[0] - d[0], c[1] - d[1]), (c[0] + d[0], c[1] + d[1]))
    # curved mirror
    R = np.array([[cs[0], -cs[1]], [cs[1], cs[0]]])
    pts = (_CUBIC_TEMPLATE * size) @ R.T + np.array(c)
    return Object.new_curved_mirror(CubicBezier(tuple(tuple(p) for p in pts)))


def _rand_light(rng, kind: str, num_rays: int):
    pos = tuple(rng.uniform(-1.0, 1.0, 2))
    color = (float(rng.uniform()), float(rng.uniform()), float(rng.uniform()), 1.0)
    if kind == "point":
        return PointLight(pos, num_rays, color)
    if kind == "spot":
        a = rng.uniform(0.0, 2.0 * math.pi)
        ang = math.radians(rng.uniform(10.0, 90.0))
        return SpotLight(pos, ang, (math.cos(a), math.sin(a)), num_rays, color)
    half = 0.5 * rng.uniform(0.1, 0.5)
    cs = _rand_rot(rng)
    a = (pos[0] - half * cs[0], pos[1] - half * cs[1])
    b = (pos[0] + half * cs[0], pos[1] + half * cs[1])
    return DirectionalLight(color, num_rays, LineSegment(a, b))


def mid_scene(seed: int = 2, accum: int = abi.LG_ACCUM_FIXED64, rays_per_light: int = 1 << 18,
              n_objects: int = 64, n_lights: int = 8) -> Workload:
    rng = np.random.default_rng(seed)
    kinds = ["rect", "circle", "mirror", "curved"]
    objects = [_rand_object(rng, kinds[rng.integers(0, 4)]) for _ in range(n_objects)]
    lkinds = ["point", "directional", "spot"]
    lights = [_rand_light(rng, lkinds[rng.integers(0, 3)], rays_per_light) for _ in range(n_lights)]
    return Workload("mid_scene", objects, lights, _params(16, 1920, 1080, accum))


def _csg_object(rng) -> Object:
    op = int(rng.integers(0, 3))
    c = tuple(rng.uniform(-1.0, 1.0, 2))
    circle = Circle(tuple(rng.uniform(-0.05, 0.05, 2)), rng.uniform(0.02, 0.15))
    rect = Rect((0.0, 0.0), 2.0 * rng.uniform(0.02, 0.15), 2.0 * rng.uniform(0.02, 0.15), _rand_rot(rng))
    return Object(abi.LG_OBJ_GEO, Logic(op, circle, rect, c, _rand_rot(rng)), Material(rng.uniform(1.3, 1.8)))


def csg_scene(seed: int = 3, total_rays: int = 1 << 22, n_objects: int = 256, n_lights: int = 8,
              width: int = 4096, height: int = 4096, string_mod: bool = True) -> Workload:
    rng = np.random.default_rng(seed)
    objects = [_csg_object(rng) for _ in range(n_objects)]
    lkinds = ["point", "directional", "spot"]
    per = total_rays // n_lights
    lights = [_rand_light(rng, lkinds[rng.integers(0, 3)], per) for _ in range(n_lights)]
    p = _params(32, width, height, abi.LG_ACCUM_FIXED64)
    if string_mod:
        p.string_mod.modulo = 4096
        p.string_mod.num = 7
        p.string_mod.turns = 1
        p.string_mod.mode = abi.LG_SM_MUL
        p.string_mod.curve = 0
        p.string_mod.color[:] = (0.25, 0.25, 0.25, 1.0)
    return Workload("csg_scene", objects, lights, p)


# string-mod line art of each curve (string_mod.rs:182-188): (curve, modulo, num, mode, turns,
# curve_f, curve_u, modulo colours)
_STRING_MOD_ART = {
    abi.LG_CURVE_CIRCLE: (1500, 7, abi.LG_SM_MUL, 1, (0.0, 0.0), (0, 0, 0),
                          [(3, 0, (1.0, 0.1, 0.1, 1.0)), (5, 2, (0.1, 1.0, 0.2, 1.0)), (7, 1, (0.2, 0.4, 1.0, 0.5))]),
    abi.LG_CURVE_COMPLEX_EXP: (2000, 2, abi.LG_SM_POW, 1,
                               (0.9998 * math.cos(2 * math.pi / 400), 0.9998 * math.sin(2 * math.pi / 400)), (0, 0, 0),
                               [(2, 1, (0.9, 0.6, 0.1, 1.0)), (9, 4, (0.2, 0.2, 1.0, 0.8))]),
    abi.LG_CURVE_HYPOTROCHOID: (1800, 13, abi.LG_SM_MUL, 3, (0.0, 0.0), (3, 5, 2),
                                [(4, 3, (0.0, 1.0, 1.0, 1.0))]),
    abi.LG_CURVE_LISSAJOUS: (2048, 5, abi.LG_SM_BASE, 1, (0.5, 0.0), (3, 4, 0),
                             [(2, 0, (1.0, 1.0, 0.0, 1.0)), (3, 0, (1.0, 0.0, 1.0, 1.0)), (6, 0, (0.0, 0.0, 0.0, 1.0))]),
}


def string_mod_art(curve: int = abi.LG_CURVE_CIRCLE, width: int = 1024, height: int = 1024,
                   colors: bool = True) -> Workload:
    """String-mod line art (StringMod::draw, string_mod.rs:152-158) on one curve, with
    modulo colours, over a small traced scene (one point light, 64 rays, no objects)."""
    m, num, mode, turns, cf, cu, table = _STRING_MOD_ART[curve]
    p = _params(4, width, height, abi.LG_ACCUM_FIXED64)
    sm = p.string_mod
    sm.modulo, sm.num, sm.mode, sm.turns, sm.curve = m, num, mode, turns, curve
    sm.color[:] = (0.3, 0.3, 0.3, 1.0)
    sm.curve_f[:] = cf
    sm.curve_u[:] = cu
    abi.set_mod_colors(p, table if colors else [])
    return Workload(f"string_mod_art_{curve}", [], [PointLight((0.1, -0.2), 64, (1.0, 1.0, 1.0, 1.0))], p)


# nested string-mod art (StringMod::nested, string_mod.rs:152-158): the nested mod's lines join
# crossings of the outer mod's lines; (nested modulo, num, mode, modulo colours)
_NESTED_ART = (6000, 17, abi.LG_SM_ADD, [(5, 1, (0.1, 0.8, 1.0, 1.0)), (7, 3, (1.0, 0.5, 0.0, 0.7))])


def nested_string_mod_art(curve: int = abi.LG_CURVE_CIRCLE, width: int = 1024, height: int = 1024,
                          outer_modulo: int = 400) -> Workload:
    """Nested string-mod art: the outer mod of :func:`string_mod_art` on one curve with
    ``outer_modulo`` lines (at most 4096), whose crossings are the points of a nested mod."""
    w = string_mod_art(curve, width, height)
    w.params.string_mod.modulo = outer_modulo
    m, num, mode, table = _NESTED_ART
    ns = abi.lg_string_mod()
    ns.modulo, ns.num, ns.mode = m, num, mode
    ns.color[:] = (0.9, 0.9, 0.2, 1.0)
    holder = abi.params_default()
    abi.set_mod_colors(holder, table)
    ns.n_colors, ns.colors = holder.string_mod.n_colors, holder.string_mod.colors
    abi.set_nested(w.params, ns)
    return Workload(f"nested_string_mod_art_{curve}", w.objects, w.lights, w.params)


def _shape_object(rng, kind: str) -> Object:
    c = tuple(rng.uniform(-1.0, 1.0, 2))
    size = rng.uniform(0.04, 0.15)
    if kind == "ellipse":
        return Object(abi.LG_OBJ_ELLIPSE, Ellipse(c, size, size * rng.uniform(0.3, 1.0), _rand_rot(rng)),
                      Material(rng.uniform(1.3, 1.8)))
    if kind == "polygon":
        k = int(rng.integers(3, 10))
        ang = rng.uniform(0, 2 * math.pi, k)
        rad = size * rng.uniform(0.6, 1.0, k)
        pts = [(c[0] + r * math.cos(a), c[1] + r * math.sin(a)) for a, r in zip(ang, rad)]
        hull = convex_hull(pts)
        if len(hull) < 3:
            hull = convex_hull(pts + [(c[0] + size, c[1]), (c[0], c[1] + size), (c[0] - size, c[1] - size)])
        return Object(abi.LG_OBJ_CONVEX_POLYGON, ConvexPolygon(hull), Material(rng.uniform(1.3, 1.8)))
    return _rand_object(rng, kind)


def shapes_scene(seed: int = 8, rays_per_light: int = 1 << 14, n_objects: int = 48) -> Workload:
    """Every shape of the scene model: ellipses and convex polygons (object.rs:13-14) beside
    rects, circles, mirrors and curved mirrors; 4 lights, 12 bounces, 1024x768."""
    rng = np.random.default_rng(seed)
    kinds = ["ellipse", "polygon", "rect", "circle", "mirror", "curved"]
    objects = [_shape_object(rng, kinds[rng.integers(0, len(kinds))]) for _ in range(n_objects)]
    lkinds = ["point", "directional", "spot"]
    lights = [_rand_light(rng, lkinds[rng.integers(0, 3)], rays_per_light) for _ in range(4)]
    return Workload("shapes_scene", objects, lights, _params(12, 1024, 768, abi.LG_ACCUM_FIXED64))


def _log_uniform_int(rng, lo: float, hi: float) -> int:
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def batch_scene(rng) -> Workload:
    n_obj = _log_uniform_int(rng, 4, 1024)
    rays = _log_uniform_int(rng, 1 << 12, 1 << 20)
    bounces = int(rng.integers(4, 33))
    side = int(rng.choice([256, 512, 1024, 2048]))
    kinds = ["rect", "circle", "mirror", "curved", "csg"]
    objects = []
    for _ in range(n_obj):
        k = kinds[rng.integers(0, 5)]
        objects.append(_csg_object(rng) if k == "csg" else _rand_object(rng, k))
    n_lights = int(rng.integers(1, 9))
    per = max(1, rays // n_lights)
    lkinds = ["point", "directional", "spot"]
    lights = [_rand_light(rng, lkinds[rng.integers(0, 3)], per) for _ in range(n_lights)]
    return Workload("batch_scene", objects, lights, _params(bounces, side, side, abi.LG_ACCUM_FIXED64))


def batch_scenes(seed: int = 4, count: int = 512) -> List[Workload]:
    rng = np.random.default_rng(seed)
    return [batch_scene(rng) for _ in range(count)]


def scale_rays(w: Workload, factor: float) -> Workload:
    """The same scene with every light's ray count scaled (for bounded CPU samples)."""
    import copy
    w2 = copy.deepcopy(w)
    for l in w2.lights:
        l.num_rays = max(1, int(round(l.num_rays * factor)))
    return w2
