"""``Tracer`` with the reference's call surface, backed by the CUDA library.

Mirrors ``light_garden::Tracer`` (src/light_garden/tracer.rs:4-208): the object and light
lists with ``push_object`` / ``push_light`` / ``replace_object`` / ``remove_*`` /
``clear`` / ``index_*`` / iterators, the public fields ``max_bounce``, ``cutoff_color``
and ``chunk_size``, ``resize`` and ``trace_all``.  ``trace_all`` returns the same
``Vec<(P2, Color)>`` line list (two entries per segment) — traced on the GPU;
``render_to_texture`` is the Renderer's accumulate + resolve (renderer.rs:164-188,
330-418) and returns the RGBA16F texture as uint16 bit patterns.

The scene is re-uploaded when it changed since the last call, like the reference which
re-traces everything every frame.
"""
from __future__ import annotations

from typing import Iterator, List, Optional, Tuple

import numpy as np

from . import abi
from .runtime import Context
from .scene import Object, P2, Color, canvas_bounds, pack


class Tracer:
    def __init__(self, width: int = 512, height: int = 512, device: int = 0):
        self.objects: List[Object] = []
        self.lights: list = []
        self.max_bounce = 5                 # tracer.rs:37
        self.cutoff_color = [0.001] * 4     # tracer.rs:38
        self.chunk_size = 100               # tracer.rs:39 (CPU chunking; no effect on the GPU)
        self.width, self.height = width, height
        self.canvas_bounds = canvas_bounds(width, height)
        self.emit_control_lines = True
        self.accum = abi.LG_ACCUM_FIXED64
        self.color_blend = (abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_ADD)
        self.alpha_blend = (abi.LG_BF_SRC_ALPHA, abi.LG_BF_ONE, abi.LG_BO_ADD)
        self.trace_time_vd: List[float] = []
        self.device = device
        self._culling = abi.LG_CULL_AUTO  # the tile map is on by default (tile_map.rs:61)
        self._ctx: Optional[Context] = None  # created by the first GPU call

    # -- object / light list (tracer.rs:48-129) ---------------------------------------------
    def clear_objects(self) -> None:
        self.objects.clear()

    def clear(self) -> None:
        self.objects.clear()
        self.lights.clear()

    def push_object(self, obj: Object) -> None:
        self.objects.append(obj)

    def push_light(self, light) -> None:
        self.lights.append(light)

    def index_object(self, ix: int) -> Object:
        return self.objects[ix]

    def index_light(self, ix: int):
        return self.lights[ix]

    def replace_object(self, ix: int, obj: Object) -> None:
        self.objects[ix] = obj

    def remove_object(self, ix: int) -> None:
        del self.objects[ix]

    def remove_light(self, ix: int) -> None:
        del self.lights[ix]

    def object_iterator(self) -> Iterator[Object]:
        return iter(self.objects)

    def light_iterator(self) -> Iterator:
        return iter(self.lights)

    def resize(self, width: int, height: int) -> None:
        self.width, self.height = width, height
        self.canvas_bounds = canvas_bounds(width, height)

    # -- scene files (tracer.rs:183-204) -------------------------------------------------------
    def serialize(self) -> str:
        """The object and light lists as RON text (Tracer::serialize)."""
        from . import ron
        return ron.dumps(self.objects, self.lights)

    def load(self, data: str) -> None:
        """Replace the object and light lists with those of a RON scene (Tracer::load)."""
        from . import ron
        objects, lights = ron.loads(data)
        self.clear()
        self.objects.extend(objects)
        self.lights.extend(lights)

    def get_trace_time(self) -> float:
        """Mean of the last 20 trace times in ms (tracer.rs:206-208)."""
        v = self.trace_time_vd
        return sum(v) / len(v) if v else float("nan")

    # -- GPU path ------------------------------------------------------------------------------
    def params(self) -> abi.lg_params:
        p = abi.params_default()
        p.max_bounce = int(self.max_bounce)
        p.width, p.height = self.width, self.height
        p.cutoff_color[:] = tuple(float(c) for c in self.cutoff_color)
        p.color_blend = abi.lg_blend_component(*self.color_blend)
        p.alpha_blend = abi.lg_blend_component(*self.alpha_blend)
        p.accum = self.accum
        p.emit_control_lines = 1 if self.emit_control_lines else 0
        return p

    def packed(self):
        """The scene as the C ABI's tables (what ``lg_scene_upload`` receives)."""
        return pack(self.objects, self.lights, self.params())

    # -- culling (tracer.rs:137-164: enable_tile_map / tile_map_enabled) -----------------------
    def enable_tile_map(self, enable: bool) -> None:
        """The reference's approximate tile map becomes the exact culling grid (``LG_CULL_AUTO``)
        or the full scan (``LG_CULL_OFF``); the traced segments are the same either way."""
        culling = abi.LG_CULL_AUTO if enable else abi.LG_CULL_OFF
        if culling != self._culling:
            self._culling = culling
            if self._ctx is not None:  # culling is a context option: the next call makes a new one
                self._ctx.close()
                self._ctx = None

    def tile_map_enabled(self) -> bool:
        return self._culling != abi.LG_CULL_OFF

    def _sync(self) -> None:
        if self._ctx is None:
            self._ctx = Context(self.device, culling=self._culling)
        self._ctx.upload(self.packed())

    def trace_all_array(self) -> np.ndarray:
        """All segments of one frame as a structured array (x0, y0, x1, y1, color[4])."""
        self._sync()
        st = self._ctx.trace()
        self.trace_time_vd.append(st["trace_ms"])
        del self.trace_time_vd[:-20]
        return self._ctx.segments()

    def trace_all(self) -> List[Tuple[P2, Color]]:
        """Tracer::trace_all: the line list, two (P2, Color) entries per segment."""
        segs = self.trace_all_array()
        out: List[Tuple[P2, Color]] = []
        for s in segs:
            c = tuple(float(x) for x in s["color"])
            out.append(((float(s["x0"]), float(s["y0"])), c))
            out.append(((float(s["x1"]), float(s["y1"])), c))
        return out

    def render_to_texture(self) -> np.ndarray:
        """Trace, accumulate and resolve one frame: (height, width, 4) binary16 bit patterns."""
        self._sync()
        img, st = self._ctx.render()
        self.trace_time_vd.append(st["total_ms"])
        del self.trace_time_vd[:-20]
        return img

    def close(self) -> None:
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None
