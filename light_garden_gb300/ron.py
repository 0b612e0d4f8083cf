"""Scene files in the reference's RON format: ``(Vec<Object>, Vec<Light>)``.

``Tracer::load`` / ``Tracer::serialize`` (src/light_garden/tracer.rs:183-204) and
``LightGarden::load_from_file`` (src/light_garden/mod.rs:708-725) read and write the object
and light lists with serde + ron; ``default.ron`` is the shipped example.  This module parses
that text into :mod:`light_garden_gb300.scene` objects and writes it back.

Field names follow the reference's serde types: ``Object { object_enum, material_opt,
moved }`` (object.rs:51-55), the ``ObjectE`` variants (object.rs:7-16), ``Material {
refractive_index }``, ``Lens { l: Logic }``, ``CurvedMirror { cubic }``, ``StraightMirror {
line_segment }`` and the ``Light`` variants (light.rs:10-14, 79-85, 139-145, 190-198).  The
geometry types come from collision2d, which is not on disk; their layout here is the one
default.ron shows (``GeoCircle { origin, radius }``, ``Rect { origin, rotation, width,
height }``, ``Logic { op, a, b, origin, rotation }``, ``CubicBezier { points }``), the
reference's own ``Ellipse { origin, a, b, rot }`` (object.rs:37-44) and a convex polygon as
its list of points (``ConvexPolygon { points }``), with a
rotation written as the four entries of nalgebra's column-major 2x2 matrix
(cos, sin, -sin, cos), and a line segment as two points (fields ``a`` and ``b``, or any two
point-valued fields in order).
"""
from __future__ import annotations

import math
import re
from typing import Any, List, Tuple

from . import abi
from .scene import (Circle, ConvexPolygon, CubicBezier, DirectionalLight, Ellipse, Geo, LineSegment, Logic, Material,
                    Object, PointLight, Rect, SpotLight)


class RonError(ValueError):
    pass


# ---- generic RON values ---------------------------------------------------------------------
class Struct(dict):
    """``(name: value, ...)``"""


class Tup(tuple):
    """``(value, ...)``"""


class Variant:
    """``Name`` or ``Name(payload)``"""

    def __init__(self, name: str, payload: Any = None):
        self.name, self.payload = name, payload

    def __repr__(self):
        return f"{self.name}({self.payload!r})"


_TOKEN = re.compile(r"""\s*(?:
    (?P<num>[-+]?(?:\d+\.?\d*(?:[eE][-+]?\d+)?|\.\d+(?:[eE][-+]?\d+)?|inf|NaN))|
    (?P<str>"(?:[^"\\]|\\.)*")|
    (?P<ident>[A-Za-z_][A-Za-z0-9_]*)|
    (?P<punct>[()\[\]{}:,])
)""", re.X)


def _tokens(text: str) -> List[Tuple[str, str]]:
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out, pos = [], 0
    while pos < len(text):
        if text[pos:].strip() == "":
            break
        m = _TOKEN.match(text, pos)
        if not m or m.end() == pos:
            raise RonError(f"unexpected character at offset {pos}: {text[pos:pos + 20]!r}")
        kind = m.lastgroup
        out.append((kind, m.group(kind)))
        pos = m.end()
    return out


class _Parser:
    def __init__(self, text: str):
        self.t = _tokens(text)
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else ("eof", "")

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise RonError(f"expected {val!r}, found {tok[1]!r}")
        self.i += 1
        return tok

    def value(self):
        kind, v = self.peek()
        if kind == "num":
            self.take()
            return float(v) if any(c in v for c in ".eEn") or v in ("inf", "NaN") else int(v)
        if kind == "str":
            self.take()
            return bytes(v[1:-1], "utf-8").decode("unicode_escape")
        if kind == "ident":
            self.take()
            if v == "true":
                return True
            if v == "false":
                return False
            if v == "None":
                return None
            if self.peek()[1] == "(":
                payload = self.paren()
                if v == "Some":
                    return payload[0] if isinstance(payload, Tup) and len(payload) == 1 else payload
                return Variant(v, payload)
            return Variant(v)
        if v == "(":
            return self.paren()
        if v == "[":
            self.take("[")
            items = []
            while self.peek()[1] != "]":
                items.append(self.value())
                if self.peek()[1] == ",":
                    self.take(",")
            self.take("]")
            return items
        raise RonError(f"unexpected token {v!r}")

    def paren(self):
        self.take("(")
        if self.peek()[0] == "ident" and self.peek(1)[1] == ":":
            st = Struct()
            while self.peek()[1] != ")":
                key = self.take()[1]
                self.take(":")
                st[key] = self.value()
                if self.peek()[1] == ",":
                    self.take(",")
            self.take(")")
            return st
        items = []
        while self.peek()[1] != ")":
            items.append(self.value())
            if self.peek()[1] == ",":
                self.take(",")
        self.take(")")
        return Tup(items)


def parse(text: str) -> Any:
    p = _Parser(text)
    v = p.value()
    if p.peek()[0] != "eof":
        raise RonError(f"trailing input at token {p.peek()[1]!r}")
    return v


# ---- mapping to the scene model ---------------------------------------------------------------
def _unwrap(payload):
    """A newtype variant ``X((fields))`` carries a one-element tuple around the struct."""
    while isinstance(payload, Tup) and len(payload) == 1:
        payload = payload[0]
    return payload


def _p2(v) -> Tuple[float, float]:
    if isinstance(v, (list, Tup)) and len(v) == 2:
        return float(v[0]), float(v[1])
    if isinstance(v, Struct) and "x" in v and "y" in v:
        return float(v["x"]), float(v["y"])
    raise RonError(f"not a point: {v!r}")


def _rot(v) -> Tuple[float, float]:
    """Rotation2 as (cos, sin): a 2x2 matrix in column-major order, or an angle."""
    if isinstance(v, (int, float)):
        return math.cos(v), math.sin(v)
    v = _unwrap(v)
    if isinstance(v, (list, Tup)) and len(v) == 4:
        return float(v[0]), float(v[1])
    if isinstance(v, (list, Tup)) and len(v) == 2 and all(isinstance(x, (list, Tup)) for x in v):
        return float(v[0][0]), float(v[0][1])
    raise RonError(f"not a rotation: {v!r}")


def _segment(v) -> LineSegment:
    v = _unwrap(v)
    if isinstance(v, Struct):
        if "a" in v and "b" in v:
            return LineSegment(_p2(v["a"]), _p2(v["b"]))
        pts = [x for x in v.values() if _is_point(x)]
        if len(pts) >= 2:
            return LineSegment(_p2(pts[0]), _p2(pts[1]))
    if isinstance(v, (list, Tup)) and len(v) == 2:
        return LineSegment(_p2(v[0]), _p2(v[1]))
    raise RonError(f"not a line segment: {v!r}")


def _is_point(x) -> bool:
    try:
        _p2(x)
        return True
    except RonError:
        return False


def _geo(v) -> Geo:
    """collision2d Geo variants on the path."""
    if not isinstance(v, Variant):
        raise RonError(f"not a geometry: {v!r}")
    f = _unwrap(v.payload)
    n = v.name
    if n in ("GeoCircle", "Circle"):
        return Circle(_p2(f["origin"]), float(f["radius"]))
    if n in ("GeoRect", "Rect"):
        return Rect(_p2(f["origin"]), float(f["width"]), float(f["height"]), _rot(f.get("rotation", [1, 0, 0, 1])))
    if n in ("GeoLineSegment", "LineSegment"):
        return _segment(f)
    if n in ("GeoCubicBezier", "CubicBezier"):
        return _cubic(f)
    if n in ("GeoLogic", "Logic"):
        return _logic(f)
    if n in ("GeoConvexPolygon", "ConvexPolygon"):
        return _polygon(f)
    if n in ("GeoEllipse", "Ellipse"):
        return _ellipse(f)
    raise RonError(f"geometry {n} is not on this path")


def _polygon(f) -> ConvexPolygon:
    pts = f["points"] if isinstance(f, Struct) else f
    pts = [_p2(p) for p in _unwrap(pts)] if not (isinstance(pts, list) and pts and _is_point(pts[0])) else [_p2(p) for p in pts]
    if len(pts) < 3:
        raise RonError("a convex polygon has at least 3 points")
    return ConvexPolygon(tuple(pts))


def _ellipse(f) -> Ellipse:
    return Ellipse(_p2(f["origin"]), float(f["a"]), float(f["b"]), _rot(f.get("rot", f.get("rotation", [1, 0, 0, 1]))))


def _cubic(f) -> CubicBezier:
    pts = f["points"] if isinstance(f, Struct) else f
    pts = _unwrap(pts) if not (isinstance(pts, (list, Tup)) and len(pts) == 4) else pts
    if len(pts) != 4:
        raise RonError("a cubic Bezier has 4 points")
    return CubicBezier(tuple(_p2(p) for p in pts))


_OPS = {"And": abi.LG_OP_AND, "Or": abi.LG_OP_OR, "AndNot": abi.LG_OP_AND_NOT}


def _logic(f) -> Logic:
    op = f["op"]
    name = op.name if isinstance(op, Variant) else str(op)
    if name not in _OPS:
        raise RonError(f"unknown logic op {name}")
    return Logic(_OPS[name], _geo(f["a"]), _geo(f["b"]), _p2(f.get("origin", [0, 0])),
                 _rot(f.get("rotation", [1, 0, 0, 1])))


def _material(m):
    if m is None:
        return None
    m = _unwrap(m)
    return Material(float(m["refractive_index"]))


def _object(v) -> Object:
    v = _unwrap(v)
    e = v["object_enum"]
    if not isinstance(e, Variant):
        raise RonError("object_enum must be a variant")
    f = _unwrap(e.payload)
    mat = _material(v.get("material_opt"))
    if e.name == "StraightMirror":
        return Object(abi.LG_OBJ_STRAIGHT_MIRROR, _segment(f["line_segment"] if isinstance(f, Struct) and "line_segment" in f else f), mat)
    if e.name == "CurvedMirror":
        return Object(abi.LG_OBJ_CURVED_MIRROR, _cubic(_unwrap(f["cubic"]) if isinstance(f, Struct) and "cubic" in f else f), mat)
    if e.name == "Circle":
        return Object(abi.LG_OBJ_CIRCLE, Circle(_p2(f["origin"]), float(f["radius"])), mat)
    if e.name == "Rect":
        return Object(abi.LG_OBJ_RECT, Rect(_p2(f["origin"]), float(f["width"]), float(f["height"]),
                                            _rot(f.get("rotation", [1, 0, 0, 1]))), mat)
    if e.name == "Lens":
        return Object(abi.LG_OBJ_LENS, _logic(_unwrap(f["l"])), mat)
    if e.name == "ConvexPolygon":
        return Object(abi.LG_OBJ_CONVEX_POLYGON, _polygon(f), mat)
    if e.name == "Ellipse":
        return Object(abi.LG_OBJ_ELLIPSE, _ellipse(f), mat)
    if e.name == "Geo":
        return Object(abi.LG_OBJ_GEO, _geo(f if isinstance(f, Variant) else _unwrap(e.payload)), mat)
    raise RonError(f"object {e.name} is not on this path")


def _color(c) -> Tuple[float, float, float, float]:
    c = list(_unwrap(c)) if not isinstance(c, list) else c
    if len(c) != 4:
        raise RonError("a colour has 4 components")
    return tuple(float(x) for x in c)


def _light(v):
    if not isinstance(v, Variant):
        raise RonError("a light is a variant")
    f = _unwrap(v.payload)
    if v.name == "PointLight":
        return PointLight(_p2(f["position"]), int(f["num_rays"]), _color(f["color"]))
    if v.name == "SpotLight":
        return SpotLight(_p2(f["position"]), float(f["spot_angle"]), _p2(f["spot_direction"]), int(f["num_rays"]),
                         _color(f["color"]))
    if v.name == "DirectionalLight":
        return DirectionalLight(_color(f["color"]), int(f["num_rays"]), _segment(f["start"]))
    raise RonError(f"unknown light {v.name}")


def loads(text: str):
    """(objects, lights) from the text of a scene file (Tracer::load, tracer.rs:190-204)."""
    v = parse(text)
    if not isinstance(v, (Tup, list)) or len(v) != 2:
        raise RonError("a scene file holds the tuple (objects, lights)")
    return [_object(o) for o in v[0]], [_light(l) for l in v[1]]


def load(path) -> tuple:
    with open(path, "r", encoding="utf-8") as fh:
        return loads(fh.read())


# ---- writing ------------------------------------------------------------------------------
def _f(x: float) -> str:
    r = repr(float(x))
    return r[:-2] if r.endswith(".0") else r


def _w_p2(p) -> str:
    return f"[{_f(p[0])}, {_f(p[1])}]"


def _w_rot(r) -> str:
    c, s = r
    return f"[{_f(c)}, {_f(s)}, {_f(-s)}, {_f(c)}]"


def _w_geo(g) -> str:
    if isinstance(g, Circle):
        return f"GeoCircle((origin: {_w_p2(g.origin)}, radius: {_f(g.radius)}))"
    if isinstance(g, Rect):
        return (f"GeoRect((origin: {_w_p2(g.origin)}, rotation: {_w_rot(g.rotation)}, width: {_f(g.width)}, "
                f"height: {_f(g.height)}))")
    if isinstance(g, LineSegment):
        return f"GeoLineSegment((a: {_w_p2(g.a)}, b: {_w_p2(g.b)}))"
    if isinstance(g, CubicBezier):
        return f"GeoCubicBezier((points: ({', '.join(_w_p2(p) for p in g.points)})))"
    if isinstance(g, Logic):
        return f"GeoLogic({_w_logic(g)})"
    if isinstance(g, ConvexPolygon):
        return f"GeoConvexPolygon({_w_polygon(g)})"
    if isinstance(g, Ellipse):
        return f"GeoEllipse({_w_ellipse(g)})"
    raise TypeError(type(g).__name__)


def _w_polygon(g: ConvexPolygon) -> str:
    if g.origin != (0.0, 0.0) or g.rotation != (1.0, 0.0):  # the file format holds world points
        c, s = g.rotation
        pts = [(g.origin[0] + c * x - s * y, g.origin[1] + s * x + c * y) for x, y in g.points]
    else:
        pts = list(g.points)
    return f"(points: [{', '.join(_w_p2(p) for p in pts)}])"


def _w_ellipse(g: Ellipse) -> str:
    return f"(origin: {_w_p2(g.origin)}, a: {_f(g.a)}, b: {_f(g.b)}, rot: {_w_rot(g.rotation)})"


def _w_logic(g: Logic) -> str:
    op = {v: k for k, v in _OPS.items()}[g.op]
    return (f"(op: {op}, a: {_w_geo(g.a)}, b: {_w_geo(g.b)}, origin: {_w_p2(g.origin)}, "
            f"rotation: {_w_rot(g.rotation)})")


def _w_object(o: Object) -> str:
    g = o.geo
    if o.kind == abi.LG_OBJ_STRAIGHT_MIRROR:
        e = f"StraightMirror((line_segment: (a: {_w_p2(g.a)}, b: {_w_p2(g.b)})))"
    elif o.kind == abi.LG_OBJ_CURVED_MIRROR:
        e = f"CurvedMirror((cubic: (points: ({', '.join(_w_p2(p) for p in g.points)}))))"
    elif o.kind == abi.LG_OBJ_CIRCLE:
        e = f"Circle((origin: {_w_p2(g.origin)}, radius: {_f(g.radius)}))"
    elif o.kind == abi.LG_OBJ_RECT:
        e = (f"Rect((origin: {_w_p2(g.origin)}, rotation: {_w_rot(g.rotation)}, width: {_f(g.width)}, "
             f"height: {_f(g.height)}))")
    elif o.kind == abi.LG_OBJ_LENS:
        e = f"Lens((l: {_w_logic(g)}))"
    elif o.kind == abi.LG_OBJ_CONVEX_POLYGON:
        e = f"ConvexPolygon({_w_polygon(g)})"
    elif o.kind == abi.LG_OBJ_ELLIPSE:
        e = f"Ellipse({_w_ellipse(g)})"
    else:
        e = f"Geo({_w_geo(g)})"
    m = "None" if o.material_opt is None else f"Some((refractive_index: {_f(o.material_opt.refractive_index)}))"
    return f"(object_enum: {e}, material_opt: {m}, moved: false)"


def _w_color(c) -> str:
    return "(" + ", ".join(_f(x) for x in c) + ")"


def _w_light(l) -> str:
    if isinstance(l, PointLight):
        return f"PointLight((position: {_w_p2(l.position)}, color: {_w_color(l.color)}, num_rays: {int(l.num_rays)}))"
    if isinstance(l, SpotLight):
        return (f"SpotLight((position: {_w_p2(l.position)}, color: {_w_color(l.color)}, num_rays: {int(l.num_rays)}, "
                f"spot_angle: {_f(l.spot_angle)}, spot_direction: {_w_p2(l.spot_direction)}))")
    if isinstance(l, DirectionalLight):
        return (f"DirectionalLight((color: {_w_color(l.color)}, num_rays: {int(l.num_rays)}, "
                f"start: (a: {_w_p2(l.start.a)}, b: {_w_p2(l.start.b)})))")
    raise TypeError(type(l).__name__)


def dumps(objects, lights) -> str:
    """Text of a scene file (Tracer::serialize, tracer.rs:183-188; one item per line)."""
    def block(items):
        return "[\n" + "".join(f"    {x},\n" for x in items) + "]" if items else "[]"
    return f"({block([_w_object(o) for o in objects])}, {block([_w_light(l) for l in lights])})\n"
