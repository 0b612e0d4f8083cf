"""Scene files in the reference's RON format (light_garden_gb300.ron): the parser, the
mapping onto the scene model, the writer, and the shipped default scene."""
import math
import os
from pathlib import Path

import numpy as np
import pytest

from light_garden_gb300 import abi, ron
from light_garden_gb300 import scene as S
from light_garden_gb300.tracer import Tracer

GOLD = Path(__file__).resolve().parent / "golden"
# the reference checkout's own default.ron, when LG_REFERENCE_SCENE names it (optional)
REFERENCE_SCENE = Path(os.environ["LG_REFERENCE_SCENE"]) if os.environ.get("LG_REFERENCE_SCENE") else None


def test_parser_values():
    v = ron.parse('''// a comment
    (a: 1, b: -2.5e-3, c: [1, 2,], d: Some((x: 3)), e: None, f: true, g: "s", h: Var, i: Var2((1, 2)),
     /* block */ j: (1, 2),)''')
    assert v["a"] == 1 and v["b"] == -2.5e-3 and v["c"] == [1, 2]
    assert v["d"] == {"x": 3} and v["e"] is None and v["f"] is True and v["g"] == "s"
    assert isinstance(v["h"], ron.Variant) and v["h"].name == "Var"
    assert v["i"].name == "Var2" and tuple(ron._unwrap(v["i"].payload)) == (1, 2)
    assert tuple(v["j"]) == (1, 2)
    with pytest.raises(ron.RonError):
        ron.parse("(a: 1")
    with pytest.raises(ron.RonError):
        ron.parse("(a: 1) extra")
    with pytest.raises(ron.RonError):
        ron.parse("(a: #)")


SCENE = '''([
    (object_enum: StraightMirror((line_segment: (a: [0.6, -0.5], b: [0.6, 0.5]))), material_opt: None, moved: false),
    (object_enum: Circle((origin: [0, 0], radius: 0.2)), material_opt: Some((refractive_index: 1.5)), moved: false),
    (object_enum: Rect((origin: [0.1, 0.2], rotation: [0, 1, -1, 0], width: 0.3, height: 0.1)),
     material_opt: Some((refractive_index: 1.2)), moved: true),
    (object_enum: Geo(GeoLogic((op: AndNot, a: GeoCircle((origin: [0, 0], radius: 0.1)),
        b: GeoRect((origin: [0, 0], rotation: [1, 0, -0, 1], width: 0.05, height: 0.05)),
        origin: [-0.5, 0.5], rotation: [1, 0, -0, 1]))), material_opt: Some((refractive_index: 1.3)), moved: false),
], [
    PointLight((position: [-0.8, 0], color: (1, 1, 1, 1), num_rays: 4096)),
    DirectionalLight((color: (0.5, 0.25, 1, 1), num_rays: 16, start: (a: [-1, -1], b: [1, -1]))),
])'''


def test_scene_mapping():
    objs, lights = ron.loads(SCENE)
    assert [o.kind for o in objs] == [abi.LG_OBJ_STRAIGHT_MIRROR, abi.LG_OBJ_CIRCLE, abi.LG_OBJ_RECT, abi.LG_OBJ_GEO]
    assert objs[0].geo == S.LineSegment((0.6, -0.5), (0.6, 0.5)) and objs[0].material_opt is None
    assert objs[1].geo == S.Circle((0.0, 0.0), 0.2) and objs[1].material_opt.refractive_index == 1.5
    # nalgebra's column-major matrix [cos, sin, -sin, cos]: a quarter turn
    assert objs[2].geo.rotation == (0.0, 1.0)
    lg = objs[3].geo
    assert isinstance(lg, S.Logic) and lg.op == abi.LG_OP_AND_NOT and lg.origin == (-0.5, 0.5)
    assert isinstance(lights[0], S.PointLight) and lights[0].num_rays == 4096
    assert isinstance(lights[1], S.DirectionalLight) and lights[1].start == S.LineSegment((-1.0, -1.0), (1.0, -1.0))
    pk = S.pack(objs, lights)
    assert pk.n_objects == 4 and pk.n_lights == 2


def test_round_trip():
    objs, lights = ron.loads(SCENE)
    o2, l2 = ron.loads(ron.dumps(objs, lights))
    assert o2 == objs and l2 == lights
    assert ron.loads(ron.dumps([], [])) == ([], [])


def test_polygon_and_ellipse_objects():
    objs, _ = ron.loads("""([
        (object_enum: Ellipse((origin: [0.1, 0.2], a: 0.3, b: 0.2, rot: [0, 1, -1, 0])),
         material_opt: Some((refractive_index: 1.4)), moved: false),
        (object_enum: ConvexPolygon((points: [[0, 0], [1, 0], [1, 1], [0, 1]])), material_opt: None, moved: false),
    ], [])""")
    assert objs[0].kind == abi.LG_OBJ_ELLIPSE and objs[0].geo == S.Ellipse((0.1, 0.2), 0.3, 0.2, (0.0, 1.0))
    assert objs[1].kind == abi.LG_OBJ_CONVEX_POLYGON and len(objs[1].geo.points) == 4
    o2, _ = ron.loads(ron.dumps(objs, []))
    assert o2 == objs


def test_unsupported_objects_are_rejected():
    with pytest.raises(ron.RonError, match="not on this path"):
        ron.loads("([(object_enum: Spline((points: [])), material_opt: None, moved: false)], [])")
    with pytest.raises(ron.RonError):
        ron.loads("([], [UnknownLight((position: [0, 0]))])")


def test_tracer_load_and_serialize():
    t = Tracer(512, 512)
    t.load(SCENE)
    assert len(list(t.object_iterator())) == 4 and len(list(t.light_iterator())) == 2
    t2 = Tracer(512, 512)
    t2.load(t.serialize())
    assert t2.objects == t.objects and t2.lights == t.lights
    assert t._ctx is None


def test_default_scene_fixture():
    objs, lights = ron.load(GOLD / "default_scene.ron")
    kinds = [o.kind for o in objs]
    assert kinds == [abi.LG_OBJ_LENS, abi.LG_OBJ_CURVED_MIRROR, abi.LG_OBJ_RECT]
    assert [type(l).__name__ for l in lights] == ["PointLight", "SpotLight"]
    assert objs[0].material_opt.refractive_index == 1.05 and objs[2].material_opt.refractive_index == 1.73
    assert lights[0].num_rays == 10000 and lights[1].num_rays == 2000
    if REFERENCE_SCENE is not None and REFERENCE_SCENE.exists():  # the fixture is the reference's file, parsed and written back
        o_ref, l_ref = ron.load(REFERENCE_SCENE)
        assert o_ref == objs and l_ref == lights


def test_default_scene_oracle_fixture(oracle):
    import hashlib
    import json
    meta = json.loads((GOLD / "default_scene.json").read_text())
    objs, lights = ron.load(GOLD / "default_scene.ron")
    p = abi.params_default()
    p.width, p.height = meta["width"], meta["height"]
    pk = S.pack(objs, lights, p)
    segs, paths, s64, st = oracle.trace(pk, ray_stride=meta["stride"])
    order = np.lexsort((paths["path"], paths["gen"], paths["primary"], paths["light"], paths["source"]))
    z = np.load(GOLD / "default_scene.npz")
    assert segs[order].tobytes() == z["segs"].tobytes()
    assert s64[order].tobytes() == z["s64"].tobytes()
    fsegs, _, _, _ = oracle.trace(pk)
    acc, px = oracle.raster(fsegs, pk.params)
    assert px == meta["pixels"] and len(fsegs) == meta["segments"]
    assert hashlib.sha256(oracle.resolve_f16(acc).tobytes()).hexdigest() == meta["f16_sha256"]
