"""ctypes mirror of ``include/lg.h`` and the loader of ``liblightgarden_cuda.so``.

The structs here are byte-for-byte the C ABI; ``tests/test_abi.py`` checks every size and
field offset against the C compiler.  The library is loaded from the package directory
(``light_garden_gb300/_lib``) where ``__graft_entry__.build()`` / ``python -m
light_garden_gb300.build`` put it; there is no CPU fallback: if the shared library is
missing, :func:`load` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "_lib"
LIB_PATH = LIB_DIR / "liblightgarden_cuda.so"

# ---- enums (lg.h) -----------------------------------------------------------------------
LG_OK = 0
LG_ERR_INVALID_ARGUMENT = 1
LG_ERR_UNSUPPORTED = 2
LG_ERR_OUT_OF_MEMORY = 3
LG_ERR_CUDA = 4
LG_ERR_NO_SCENE = 5
LG_ERR_TRUNCATED = 6
LG_ERR_TIMEOUT = 7
LG_ERR_BUDGET = 8
LG_ERR_NOT_READY = 9
LG_ERR_NOT_FOUND = 10
STATUS_NAMES = {
    0: "LG_OK", 1: "LG_ERR_INVALID_ARGUMENT", 2: "LG_ERR_UNSUPPORTED", 3: "LG_ERR_OUT_OF_MEMORY",
    4: "LG_ERR_CUDA", 5: "LG_ERR_NO_SCENE", 6: "LG_ERR_TRUNCATED", 7: "LG_ERR_TIMEOUT",
    8: "LG_ERR_BUDGET", 9: "LG_ERR_NOT_READY", 10: "LG_ERR_NOT_FOUND",
}

(LG_GEO_CIRCLE, LG_GEO_RECT, LG_GEO_SEGMENT, LG_GEO_CUBIC, LG_GEO_LOGIC, LG_GEO_POLYGON, LG_GEO_ELLIPSE,
 LG_GEO_VERTICES) = range(8)
LG_OP_AND, LG_OP_OR, LG_OP_AND_NOT = range(3)
(LG_OBJ_STRAIGHT_MIRROR, LG_OBJ_CURVED_MIRROR, LG_OBJ_CIRCLE, LG_OBJ_RECT, LG_OBJ_LENS,
 LG_OBJ_CONVEX_POLYGON, LG_OBJ_ELLIPSE, LG_OBJ_GEO) = range(8)
LG_LIGHT_POINT, LG_LIGHT_DIRECTIONAL, LG_LIGHT_SPOT = range(3)
(LG_BF_ZERO, LG_BF_ONE, LG_BF_SRC, LG_BF_ONE_MINUS_SRC, LG_BF_SRC_ALPHA, LG_BF_ONE_MINUS_SRC_ALPHA,
 LG_BF_DST, LG_BF_ONE_MINUS_DST, LG_BF_DST_ALPHA, LG_BF_ONE_MINUS_DST_ALPHA,
 LG_BF_SRC_ALPHA_SATURATED, LG_BF_CONSTANT, LG_BF_ONE_MINUS_CONSTANT) = range(13)
LG_BO_ADD, LG_BO_SUBTRACT, LG_BO_REVERSE_SUBTRACT, LG_BO_MIN, LG_BO_MAX = range(5)
LG_ACCUM_FIXED64, LG_ACCUM_F32 = 0, 1
LG_SM_ADD, LG_SM_MUL, LG_SM_POW, LG_SM_BASE = range(4)
LG_CURVE_CIRCLE, LG_CURVE_COMPLEX_EXP, LG_CURVE_HYPOTROCHOID, LG_CURVE_LISSAJOUS = range(4)
LG_PATH_NEAR_DEGENERATE, LG_PATH_TIR, LG_PATH_FALLBACK, LG_PATH_ILL_CONDITIONED = 1, 2, 4, 8
LG_SRC_TRACE, LG_SRC_CONTROL_LINE, LG_SRC_STRING_MOD = 0, 1, 2


class lg_geo(C.Structure):
    _fields_ = [("kind", C.c_int32), ("op", C.c_int32), ("a", C.c_int32), ("b", C.c_int32),
                ("origin", C.c_double * 2), ("rot", C.c_double * 2), ("v", C.c_double * 8)]


class lg_object(C.Structure):
    _fields_ = [("kind", C.c_int32), ("geo", C.c_int32), ("has_material", C.c_int32),
                ("_pad", C.c_int32), ("refractive_index", C.c_double)]


class lg_light(C.Structure):
    _fields_ = [("kind", C.c_int32), ("num_rays", C.c_uint32), ("color", C.c_float * 4),
                ("origin", C.c_double * 2), ("v", C.c_double * 2), ("spot_angle", C.c_double)]


class lg_blend_component(C.Structure):
    _fields_ = [("src_factor", C.c_int32), ("dst_factor", C.c_int32), ("op", C.c_int32)]


class lg_mod_color(C.Structure):
    _fields_ = [("modulo", C.c_uint64), ("rem", C.c_uint64), ("color", C.c_float * 4)]


class lg_string_mod(C.Structure):
    # ``colors`` (const lg_mod_color*) and ``nested`` (const lg_string_mod*) are C pointers;
    # they are declared as integer addresses so that parameter blocks stay copyable, and set
    # through set_mod_colors() and set_nested().
    _fields_ = [("modulo", C.c_uint64), ("num", C.c_uint64), ("turns", C.c_uint64),
                ("mode", C.c_uint32), ("curve", C.c_uint32), ("color", C.c_float * 4),
                ("curve_f", C.c_double * 2), ("curve_u", C.c_uint64 * 3),
                ("n_colors", C.c_uint32), ("_pad", C.c_uint32), ("colors", C.c_uint64),
                ("nested", C.c_uint64)]


class lg_params(C.Structure):
    _fields_ = [("max_bounce", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("cutoff_color", C.c_float * 4), ("clear_color", C.c_float * 4),
                ("blend_constant", C.c_float * 4),
                ("color_blend", lg_blend_component), ("alpha_blend", lg_blend_component),
                ("accum", C.c_int32), ("emit_control_lines", C.c_int32),
                ("record_paths", C.c_int32), ("precision", C.c_int32),
                ("string_mod", lg_string_mod), ("ray_stride", C.c_uint32), ("ray_offset", C.c_uint32)]


class lg_segment(C.Structure):
    _fields_ = [("x0", C.c_float), ("y0", C.c_float), ("x1", C.c_float), ("y1", C.c_float),
                ("color", C.c_float * 4)]


class lg_chord(C.Structure):
    _fields_ = [("x0", C.c_float), ("y0", C.c_float), ("x1", C.c_float), ("y1", C.c_float),
                ("color0", C.c_float * 4), ("color1", C.c_float * 4)]


class lg_path_record(C.Structure):
    _fields_ = [("path", C.c_uint64), ("primary", C.c_uint32), ("light", C.c_uint16),
                ("gen", C.c_uint8), ("flags", C.c_uint8), ("hit", C.c_int32), ("source", C.c_uint32)]


class lg_trace_stats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("ray_visits", C.c_uint64), ("segments", C.c_uint64),
                ("fp64_solves", C.c_uint64), ("fp64_fallbacks", C.c_uint64),
                ("near_degenerate", C.c_uint64), ("pixels", C.c_uint64), ("tile_refs", C.c_uint64),
                ("bound_tests", C.c_uint64), ("object_tests", C.c_uint64),
                ("retries", C.c_uint32), ("_pad", C.c_uint32),
                ("trace_ms", C.c_float), ("accumulate_ms", C.c_float), ("resolve_ms", C.c_float),
                ("total_ms", C.c_float), ("bin_ms", C.c_float), ("raster_ms", C.c_float),
                ("scan_ms", C.c_float), ("solve_ms", C.c_float), ("bounce_ms", C.c_float), ("_pad2", C.c_float),
                ("ill_conditioned", C.c_uint64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if not name.startswith("_")}


class lg_device_opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("raster_variant", C.c_int32), ("segment_capacity", C.c_uint64),
                ("queue_capacity", C.c_uint64), ("stream_segments", C.c_uint64), ("culling", C.c_int32),
                ("grid_density", C.c_float), ("wait_polls", C.c_int32), ("scan_pairs", C.c_int32)]


LG_ABI_VERSION = 5  # include/lg.h
LG_STRING_MOD_NESTED_MAX = 4096  # include/lg.h
LG_CULL_AUTO, LG_CULL_OFF, LG_CULL_ON = 0, 1, 2
LG_PRECISION_EXACT, LG_PRECISION_FAST = 0, 1
LG_CULL_AUTO_MIN = 16
LG_CULL_WALK_MIN = 96


# numpy dtypes with the same layout, for bulk conversion of downloads
def segment_dtype():
    import numpy as np
    return np.dtype([("x0", "<f4"), ("y0", "<f4"), ("x1", "<f4"), ("y1", "<f4"), ("color", "<f4", (4,))])


def chord_dtype():
    import numpy as np
    return np.dtype([("x0", "<f4"), ("y0", "<f4"), ("x1", "<f4"), ("y1", "<f4"), ("color0", "<f4", (4,)),
                     ("color1", "<f4", (4,))])


# colour tables handed to the library by address; kept alive for the life of the process
_mod_color_tables: list = []


def set_mod_colors(params: "lg_params", entries) -> None:
    """StringMod::modulo_colors: ``entries`` is a sequence of (modulo, rem, (r, g, b, a))."""
    entries = list(entries)
    sm = params.string_mod
    if not entries:
        sm.n_colors, sm.colors = 0, 0
        return
    arr = (lg_mod_color * len(entries))()
    for e, (m, r, col) in zip(arr, entries):
        e.modulo, e.rem = int(m), int(r)
        e.color[:] = tuple(float(x) for x in col)
    _mod_color_tables.append(arr)
    sm.n_colors, sm.colors = len(entries), C.addressof(arr)


def set_nested(params: "lg_params", nested: "lg_string_mod | None") -> None:
    """StringMod::nested: the mod drawn between the crossings of params.string_mod's lines
    (a copy of ``nested`` is kept alive and handed to the library by address; None clears)."""
    if nested is None:
        params.string_mod.nested = 0
        return
    keep = lg_string_mod()
    C.memmove(C.addressof(keep), C.addressof(nested), C.sizeof(lg_string_mod))
    keep.nested = 0
    _mod_color_tables.append(keep)
    params.string_mod.nested = C.addressof(keep)


def path_dtype():
    import numpy as np
    return np.dtype([("path", "<u8"), ("primary", "<u4"), ("light", "<u2"), ("gen", "u1"),
                     ("flags", "u1"), ("hit", "<i4"), ("source", "<u4")])


def params_default() -> lg_params:
    """The reference defaults (tracer.rs:37-39, mod.rs:57-73), without needing the library."""
    p = lg_params()
    p.max_bounce = 5
    p.width, p.height = 512, 512
    for i in range(4):
        p.cutoff_color[i] = 0.001
    p.clear_color[:] = (0.0, 0.0, 0.0, 1.0)
    p.blend_constant[:] = (0.0, 0.0, 0.0, 0.0)
    p.color_blend = lg_blend_component(LG_BF_ONE, LG_BF_ONE, LG_BO_ADD)
    p.alpha_blend = lg_blend_component(LG_BF_SRC_ALPHA, LG_BF_ONE, LG_BO_ADD)
    p.accum = LG_ACCUM_FIXED64
    p.emit_control_lines = 1
    p.record_paths = 0
    p.precision = LG_PRECISION_EXACT
    p.string_mod = lg_string_mod()
    p.ray_stride, p.ray_offset = 1, 0
    return p


class lg_scene_desc(C.Structure):
    _fields_ = [("geos", C.POINTER(lg_geo)), ("objects", C.POINTER(lg_object)), ("lights", C.POINTER(lg_light)),
                ("params", C.POINTER(lg_params)), ("n_geo", C.c_uint32), ("n_objects", C.c_uint32),
                ("n_lights", C.c_uint32), ("_pad", C.c_uint32)]


class lg_serve_opts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_slots", C.c_uint32), ("_pad", C.c_uint32)]


class lg_serve_step_stats(C.Structure):
    _fields_ = [("admitted", C.c_uint32), ("finished", C.c_uint32), ("in_flight", C.c_uint32),
                ("pending", C.c_uint32), ("rasterised", C.c_uint32), ("restarted", C.c_uint32),
                ("live_rays", C.c_uint64), ("segments", C.c_uint64), ("step_ms", C.c_float), ("_pad", C.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("_")}


# ---- library loading --------------------------------------------------------------------
_lib = None

EXPORTS = [
    # name, restype, argtypes
    ("lg_abi_version", C.c_uint32, []),
    ("lg_params_default", None, [C.POINTER(lg_params)]),
    ("lg_create", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(lg_device_opts)]),
    ("lg_destroy", C.c_int, [C.c_void_p]),
    ("lg_last_error", C.c_char_p, [C.c_void_p]),
    ("lg_scene_upload", C.c_int, [C.c_void_p, C.POINTER(lg_geo), C.c_uint32, C.POINTER(lg_object),
                                  C.c_uint32, C.POINTER(lg_light), C.c_uint32, C.POINTER(lg_params)]),
    ("lg_trace", C.c_int, [C.c_void_p, C.POINTER(lg_trace_stats)]),
    ("lg_accumulate", C.c_int, [C.c_void_p, C.POINTER(lg_trace_stats)]),
    ("lg_accumulate_segments", C.c_int, [C.c_void_p, C.POINTER(lg_segment), C.c_uint64,
                                         C.POINTER(lg_trace_stats)]),
    ("lg_resolve_f16", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int32]),
    ("lg_resolve_rgba8", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int32]),
    ("lg_render", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int32, C.POINTER(lg_trace_stats)]),
    ("lg_segments_download", C.c_int, [C.c_void_p, C.POINTER(lg_segment), C.POINTER(lg_path_record),
                                       C.c_uint64, C.POINTER(C.c_uint64)]),
    ("lg_accum_download", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    ("lg_chords_download", C.c_int, [C.c_void_p, C.POINTER(lg_chord), C.c_uint64, C.POINTER(C.c_uint64)]),
    ("lg_batch_upload", C.c_int, [C.c_void_p, C.POINTER(lg_scene_desc), C.c_uint32]),
    ("lg_batch_render", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int32, C.POINTER(lg_trace_stats)]),
    ("lg_batch_image_offset", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64)]),
    ("lg_serve_begin", C.c_int, [C.c_void_p, C.POINTER(lg_serve_opts)]),
    ("lg_serve_submit", C.c_int, [C.c_void_p, C.POINTER(lg_scene_desc), C.POINTER(C.c_uint64)]),
    ("lg_serve_step", C.c_int, [C.c_void_p, C.POINTER(lg_serve_step_stats)]),
    ("lg_serve_poll", C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_int32]),
    ("lg_serve_end", C.c_int, [C.c_void_p]),
    ("lg_accumulate_segments_noalloc", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(lg_params), C.c_void_p,
                                                 C.c_void_p, C.POINTER(C.c_uint64)]),
]


class LgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load the CUDA library.  Raises if it has not been built: there is no fallback."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python -m light_garden_gb300.build)")
    lib = C.CDLL(str(p))
    for name, res, args in EXPORTS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    version = lib.lg_abi_version()
    if version != LG_ABI_VERSION:  # the structs below would not match the library's
        raise RuntimeError(f"{p} has C ABI version {version}, this package expects {LG_ABI_VERSION}: rebuild it")
    if path is None:
        _lib = lib
    return lib
