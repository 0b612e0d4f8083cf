"""Scene model with the reference's names, packed into the C ABI tables of ``lg.h``.

Mirrors light_garden's scene types:

* geometry  (collision2d ``Geo``): :class:`Circle`, :class:`Rect`, :class:`LineSegment`,
  :class:`CubicBezier`, :class:`Logic` (with ``&``, ``|`` and :meth:`Geo.and_not`, as
  used by ``LightGarden::mouse_clicked``, src/light_garden/mod.rs:366-372);
* objects   (``Object``/``ObjectE``, src/light_garden/object.rs:7-16,51-113):
  :class:`Object` with the constructors ``new_mirror``, ``new_curved_mirror``,
  ``new_circle``, ``new_rect``, ``new_lens``, ``new_geo`` and ``material_opt``;
* lights    (``Light``, src/light_garden/light.rs:10-14): :class:`PointLight`,
  :class:`SpotLight`, :class:`DirectionalLight`;
* string mods (src/light_garden/string_mod.rs): :class:`StringMod`, :class:`Curve`,
  :class:`ModRemColor`, :class:`StringModMode`, filling ``lg_params.string_mod``.

:func:`pack` flattens a list of objects and lights into ``lg_geo``/``lg_object``/
``lg_light`` arrays: one node array holding every geometry tree, objects naming their
root node.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

from . import abi

P2 = Tuple[float, float]
Color = Tuple[float, float, float, float]


def _rot(angle: float) -> Tuple[float, float]:
    return (math.cos(angle), math.sin(angle))


class Geo:
    """Base class of geometry nodes (collision2d ``Geo``)."""

    def __and__(self, other: "Geo") -> "Logic":
        return Logic(abi.LG_OP_AND, self, other)

    def __or__(self, other: "Geo") -> "Logic":
        return Logic(abi.LG_OP_OR, self, other)

    def and_not(self, other: "Geo") -> "Logic":
        return Logic(abi.LG_OP_AND_NOT, self, other)


@dataclass
class Circle(Geo):
    origin: P2
    radius: float


@dataclass
class Rect(Geo):
    """Rect { origin (centre), rotation, width, height }; ``rotation`` is (cos, sin)."""
    origin: P2
    width: float
    height: float
    rotation: Tuple[float, float] = (1.0, 0.0)

    @staticmethod
    def from_tlbr(top: float, left: float, bottom: float, right: float) -> "Rect":
        return Rect(((left + right) * 0.5, (top + bottom) * 0.5), right - left, top - bottom)


@dataclass
class LineSegment(Geo):
    a: P2
    b: P2

    @staticmethod
    def from_ab(a: P2, b: P2) -> "LineSegment":
        return LineSegment(a, b)


@dataclass
class CubicBezier(Geo):
    points: Tuple[P2, P2, P2, P2]

    def get_control_lines(self) -> List[Tuple[P2, Color]]:
        """CurvedMirror::get_control_lines (object.rs:355-365): red control polygon."""
        red = (1.0, 0.0, 0.0, 1.0)
        p = self.points
        return [(p[0], red), (p[1], red), (p[1], red), (p[2], red), (p[2], red), (p[3], red)]


def convex_hull(points: Sequence[P2]) -> Tuple[P2, ...]:
    """Counter-clockwise convex hull (Andrew's monotone chain), as ConvexPolygon::new_convex_hull
    builds it (object.rs:34-36); collinear points are dropped."""
    pts = sorted(set((float(x), float(y)) for x, y in points))
    if len(pts) < 3:
        return tuple(pts)

    def turn(o, a, b):
        return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])
    lower: list = []
    for p in pts:
        while len(lower) >= 2 and turn(lower[-2], lower[-1], p) <= 0:
            lower.pop()
        lower.append(p)
    upper: list = []
    for p in reversed(pts):
        while len(upper) >= 2 and turn(upper[-2], upper[-1], p) <= 0:
            upper.pop()
        upper.append(p)
    return tuple(lower[:-1] + upper[:-1])


@dataclass
class ConvexPolygon(Geo):
    """Convex polygon: vertices in order around it (either orientation), in the frame
    (origin, rotation)."""
    points: Tuple[P2, ...]
    origin: P2 = (0.0, 0.0)
    rotation: Tuple[float, float] = (1.0, 0.0)


@dataclass
class Ellipse(Geo):
    """Ellipse { origin, a, b, rot } (object.rs:37-44): semi-axis a along the rotated x."""
    origin: P2
    a: float
    b: float
    rotation: Tuple[float, float] = (1.0, 0.0)


@dataclass
class Logic(Geo):
    """Logic { op, a, b, origin, rotation }: children live in the node's local frame."""
    op: int
    a: Geo
    b: Geo
    origin: P2 = (0.0, 0.0)
    rotation: Tuple[float, float] = (1.0, 0.0)


@dataclass
class Material:
    refractive_index: float = 1.2  # Material::default, object.rs:441-447


@dataclass
class Object:
    kind: int
    geo: Geo
    material_opt: Optional[Material]

    @staticmethod
    def new_mirror(a: P2, b: P2) -> "Object":
        return Object(abi.LG_OBJ_STRAIGHT_MIRROR, LineSegment(a, b), None)

    @staticmethod
    def new_curved_mirror(cubic: CubicBezier) -> "Object":
        return Object(abi.LG_OBJ_CURVED_MIRROR, cubic, None)

    @staticmethod
    def new_circle(origin: P2, radius: float) -> "Object":
        return Object(abi.LG_OBJ_CIRCLE, Circle(origin, radius), Material())

    @staticmethod
    def new_rect(origin: P2, width: float, height: float) -> "Object":
        return Object(abi.LG_OBJ_RECT, Rect(origin, width, height), Material())

    @staticmethod
    def new_lens(origin: P2, radius: float, distance: float) -> "Object":
        # Lens::new, object.rs:393-411: And of two circles at (+-distance/2, 0)
        lg = Logic(abi.LG_OP_AND, Circle((distance * 0.5, 0.0), radius),
                   Circle((-distance * 0.5, 0.0), radius), origin)
        return Object(abi.LG_OBJ_LENS, lg, Material())

    @staticmethod
    def new_convex_polygon(points: Sequence[P2]) -> "Object":
        # Object::new_convex_polygon (object.rs:92-98): the convex hull, default material
        return Object(abi.LG_OBJ_CONVEX_POLYGON, ConvexPolygon(convex_hull(points)), Material())

    @staticmethod
    def new_ellipse(origin: P2, a: float, b: float) -> "Object":
        # Object::new_ellipse (object.rs:99-105): unrotated, default material
        return Object(abi.LG_OBJ_ELLIPSE, Ellipse(origin, a, b), Material())

    @staticmethod
    def new_geo(geo: Geo) -> "Object":
        return Object(abi.LG_OBJ_GEO, geo, Material())

    def get_material(self) -> Optional[Material]:
        return self.material_opt


@dataclass
class PointLight:
    position: P2
    num_rays: int
    color: Color

    def set_num_rays(self, n: Optional[int]) -> None:
        if n is not None:
            self.num_rays = n


@dataclass
class SpotLight:
    position: P2
    spot_angle: float
    spot_direction: P2
    num_rays: int
    color: Color

    def set_num_rays(self, n: Optional[int]) -> None:
        if n is not None:
            self.num_rays = n


@dataclass
class DirectionalLight:
    color: Color
    num_rays: int
    start: LineSegment

    def set_num_rays(self, n: Optional[int]) -> None:
        if n is not None:
            self.num_rays = n


Light = object  # PointLight | SpotLight | DirectionalLight


# ---- packing --------------------------------------------------------------------------------
def _emit_geo(g: Geo, nodes: list) -> int:
    idx = len(nodes)
    rec = abi.lg_geo()
    rec.rot[0], rec.rot[1] = 1.0, 0.0
    nodes.append(rec)
    if isinstance(g, Circle):
        rec.kind = abi.LG_GEO_CIRCLE
        rec.origin[:] = g.origin
        rec.v[0] = g.radius
    elif isinstance(g, Rect):
        rec.kind = abi.LG_GEO_RECT
        rec.origin[:] = g.origin
        rec.rot[:] = g.rotation
        rec.v[0], rec.v[1] = g.width, g.height
    elif isinstance(g, LineSegment):
        rec.kind = abi.LG_GEO_SEGMENT
        rec.v[0], rec.v[1] = g.a
        rec.v[2], rec.v[3] = g.b
    elif isinstance(g, CubicBezier):
        rec.kind = abi.LG_GEO_CUBIC
        for k, p in enumerate(g.points):
            rec.v[2 * k], rec.v[2 * k + 1] = p
    elif isinstance(g, Ellipse):
        rec.kind = abi.LG_GEO_ELLIPSE
        rec.origin[:] = g.origin
        rec.rot[:] = g.rotation
        rec.v[0], rec.v[1] = g.a, g.b
    elif isinstance(g, ConvexPolygon):
        pts = list(g.points)
        if not 3 <= len(pts) <= 63:
            raise ValueError("a convex polygon has 3..63 vertices")
        rec.kind = abi.LG_GEO_POLYGON
        rec.origin[:] = g.origin
        rec.rot[:] = g.rotation
        rec.a, rec.b = len(pts), -1
        for i, (x, y) in enumerate(pts[:4]):
            rec.v[2 * i], rec.v[2 * i + 1] = x, y
        prev = idx
        for c0 in range(4, len(pts), 4):  # continuation records, 4 vertices each
            cont = abi.lg_geo()
            cont.kind = abi.LG_GEO_VERTICES
            cont.b = -1
            cont.rot[0] = 1.0
            for i, (x, y) in enumerate(pts[c0:c0 + 4]):
                cont.v[2 * i], cont.v[2 * i + 1] = x, y
            nodes[prev].b = len(nodes)
            prev = len(nodes)
            nodes.append(cont)
    elif isinstance(g, Logic):
        rec.kind = abi.LG_GEO_LOGIC
        rec.op = g.op
        rec.origin[:] = g.origin
        rec.rot[:] = g.rotation
        a = _emit_geo(g.a, nodes)
        b = _emit_geo(g.b, nodes)
        nodes[idx].a, nodes[idx].b = a, b
    else:
        raise TypeError(f"unsupported geometry {type(g).__name__}")
    return idx


def pack_light(light) -> abi.lg_light:
    if not isinstance(light, (PointLight, SpotLight, DirectionalLight)):
        raise TypeError(f"unsupported light {type(light).__name__}")
    rec = abi.lg_light()
    rec.num_rays = int(light.num_rays)
    rec.color[:] = tuple(float(c) for c in light.color)
    if isinstance(light, PointLight):
        rec.kind = abi.LG_LIGHT_POINT
        rec.origin[:] = light.position
    elif isinstance(light, SpotLight):
        rec.kind = abi.LG_LIGHT_SPOT
        rec.origin[:] = light.position
        rec.v[:] = light.spot_direction
        rec.spot_angle = light.spot_angle
    elif isinstance(light, DirectionalLight):
        rec.kind = abi.LG_LIGHT_DIRECTIONAL
        rec.origin[:] = light.start.a
        rec.v[:] = light.start.b
    return rec


@dataclass
class PackedScene:
    geos: object
    n_geo: int
    objects: object
    n_objects: int
    lights: object
    n_lights: int
    params: abi.lg_params = field(default_factory=abi.params_default)

    def args(self):
        """Positional arguments of lg_scene_upload / lgo_trace after the context."""
        return (self.geos, self.n_geo, self.objects, self.n_objects, self.lights, self.n_lights)


def pack(objects: Sequence[Object], lights: Sequence, params: Optional[abi.lg_params] = None) -> PackedScene:
    nodes: list = []
    objs = (abi.lg_object * max(1, len(objects)))()
    for k, ob in enumerate(objects):
        root = _emit_geo(ob.geo, nodes)
        objs[k].kind = ob.kind
        objs[k].geo = root
        objs[k].has_material = 1 if ob.material_opt is not None else 0
        objs[k].refractive_index = ob.material_opt.refractive_index if ob.material_opt else 1.0
    geos = (abi.lg_geo * max(1, len(nodes)))(*nodes)
    lts = (abi.lg_light * max(1, len(lights)))(*[pack_light(l) for l in lights])
    return PackedScene(geos, len(nodes), objs, len(objects), lts, len(lights),
                       params if params is not None else abi.params_default())


def canvas_bounds(width: int, height: int) -> Rect:
    """Rect::from_tlbr(1, -aspect, -1, aspect) with the f32 aspect of sub_render_pass.rs:146-156."""
    import numpy as np
    aspect = float(np.float32(width) / np.float32(height))
    return Rect.from_tlbr(1.0, -aspect, -1.0, aspect)


def rotation(angle: float) -> Tuple[float, float]:
    """A Rot2 as (cos, sin)."""
    return _rot(angle)


# ---- string mods (src/light_garden/string_mod.rs) ------------------------------------------------
class StringModMode:
    """StringModMode (string_mod.rs:174-180)."""
    Add, Mul, Pow, Base = abi.LG_SM_ADD, abi.LG_SM_MUL, abi.LG_SM_POW, abi.LG_SM_BASE


@dataclass
class Curve:
    """Curve (string_mod.rs:182-188): ``Curve.circle()``, ``Curve.complex_exp(c)``,
    ``Curve.hypotrochoid(r, s, d)``, ``Curve.lissajous(a, b, delta)``."""
    kind: int = abi.LG_CURVE_CIRCLE
    f: Tuple[float, float] = (0.0, 0.0)
    u: Tuple[int, int, int] = (0, 0, 0)

    @staticmethod
    def circle() -> "Curve":
        return Curve()

    @staticmethod
    def complex_exp(c: complex) -> "Curve":
        return Curve(abi.LG_CURVE_COMPLEX_EXP, (float(c.real), float(c.imag)))

    @staticmethod
    def hypotrochoid(r: int, s: int, d: int) -> "Curve":
        return Curve(abi.LG_CURVE_HYPOTROCHOID, u=(int(r), int(s), int(d)))

    @staticmethod
    def lissajous(a: int, b: int, delta: float) -> "Curve":
        return Curve(abi.LG_CURVE_LISSAJOUS, (float(delta), 0.0), (int(a), int(b), 0))


@dataclass
class ModRemColor:
    """ModRemColor (string_mod.rs:167-172): point n takes ``color`` when n % modulo == rem."""
    modulo: int
    rem: int
    color: Color


@dataclass
class StringMod:
    """StringMod (string_mod.rs:3-31) with the reference's defaults (``StringMod::new``).
    ``pow`` and ``modulo_color_index`` are GUI state of the reference and do not change what
    is drawn."""
    modulo: int = 5
    num: int = 1
    pow: int = 0
    color: Color = (1.0, 1.0, 1.0, 1.0)
    turns: int = 1
    init_curve: Curve = field(default_factory=Curve)
    mode: int = StringModMode.Mul
    modulo_colors: List[ModRemColor] = field(default_factory=list)
    modulo_color_index: int = 0
    nested: Optional["StringMod"] = None

    def to_abi(self) -> abi.lg_string_mod:
        """The lg_string_mod of this mod (its colour table and nested mod kept alive by abi)."""
        holder = abi.params_default()
        sm = holder.string_mod
        sm.modulo, sm.num, sm.turns, sm.mode, sm.curve = self.modulo, self.num, self.turns, self.mode, \
            self.init_curve.kind
        sm.color[:] = tuple(float(x) for x in self.color)
        sm.curve_f[:] = self.init_curve.f
        sm.curve_u[:] = self.init_curve.u
        abi.set_mod_colors(holder, [(c.modulo, c.rem, c.color) for c in self.modulo_colors])
        if self.nested is not None:
            abi.set_nested(holder, self.nested.to_abi())
        return holder.string_mod

    def apply(self, params: abi.lg_params) -> abi.lg_params:
        """Draw this mod over the frame of ``params`` (StringMod::draw, string_mod.rs:152-158)."""
        params.string_mod = self.to_abi()
        return params
