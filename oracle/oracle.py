"""ctypes wrapper of the CPU oracle (``oracle/lg_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py``.  PARITY UNPINNED (see lg_oracle.h): the reference's geometry
crate is absent and the reference ships no tests or golden outputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from light_garden_gb300 import abi

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblg_oracle.so"


LGO_ERR_TRUNCATED = -6  # lg_oracle.h


class lgo_stats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("ray_visits", C.c_uint64), ("segments", C.c_uint64),
                ("near_degenerate", C.c_uint64), ("pixels", C.c_uint64), ("seconds", C.c_double)]


class lgo_hit(C.Structure):
    _fields_ = [("t", C.c_double), ("px", C.c_double), ("py", C.c_double), ("nx", C.c_double),
                ("ny", C.c_double)]


def build(force: bool = False) -> Path:
    srcs = [HERE / "lg_oracle.c", HERE / "lg_oracle.h", HERE.parent / "include" / "lg.h"]
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.POINTER
        L.lgo_trace.argtypes = [P(abi.lg_geo), C.c_uint32, P(abi.lg_object), C.c_uint32, P(abi.lg_light),
                                C.c_uint32, P(abi.lg_params), C.c_uint32, C.c_uint32, C.c_int,
                                P(abi.lg_segment), P(abi.lg_path_record), P(C.c_double), C.c_uint64,
                                P(C.c_uint64), P(lgo_stats)]
        L.lgo_light_rays.argtypes = [P(abi.lg_light), P(C.c_double), C.c_uint64]
        L.lgo_sincos.argtypes = [C.c_double, P(C.c_double), P(C.c_double)]
        L.lgo_atan.restype = C.c_double
        L.lgo_atan.argtypes = [C.c_double]
        L.lgo_geo_hits.argtypes = [P(abi.lg_geo), C.c_uint32, C.c_int32, C.c_double, C.c_double,
                                   C.c_double, C.c_double, P(lgo_hit), C.c_int, P(C.c_uint32)]
        L.lgo_geo_contains.argtypes = [P(abi.lg_geo), C.c_uint32, C.c_int32, C.c_double, C.c_double]
        L.lgo_refract.argtypes = [C.c_double] * 6 + [P(C.c_double), P(C.c_double), P(C.c_double)]
        L.lgo_light_medium.restype = C.c_double
        L.lgo_light_medium.argtypes = [P(abi.lg_geo), C.c_uint32, P(abi.lg_object), C.c_uint32, P(abi.lg_light)]
        L.lgo_clear.argtypes = [P(C.c_int64), C.c_uint32, C.c_uint32, P(abi.lg_params)]
        L.lgo_raster.argtypes = [P(abi.lg_segment), C.c_uint64, P(abi.lg_params), P(C.c_int64), C.c_int,
                                 P(C.c_uint64)]
        L.lgo_raster_f64.argtypes = [P(abi.lg_segment), C.c_uint64, P(abi.lg_params), P(C.c_double),
                                     P(C.c_uint64)]
        L.lgo_string_mod_chords.argtypes = [P(abi.lg_params), P(abi.lg_chord), C.c_uint64, P(C.c_uint64)]
        L.lgo_string_mod_crossings.argtypes = [P(abi.lg_string_mod), P(C.c_double), C.c_uint64, P(C.c_uint64)]
        L.lgo_seg_cross.argtypes = [C.c_double] * 8 + [P(C.c_double), P(C.c_double)]
        L.lgo_raster_chords.argtypes = [P(abi.lg_chord), C.c_uint64, P(abi.lg_params), P(C.c_int64), P(C.c_uint64)]
        L.lgo_raster_chords_f64.argtypes = [P(abi.lg_chord), C.c_uint64, P(abi.lg_params), P(C.c_double),
                                            P(C.c_uint64)]
        L.lgo_resolve_f16.argtypes = [P(C.c_int64), C.c_uint32, C.c_uint32, P(C.c_uint16)]
        L.lgo_resolve_rgba8.argtypes = [P(C.c_int64), C.c_uint32, C.c_uint32, P(C.c_uint8)]
        L.lgo_f32_to_f16.restype = C.c_uint16
        L.lgo_f32_to_f16.argtypes = [C.c_float]
        L.lgo_f16_to_f32.restype = C.c_float
        L.lgo_f16_to_f32.argtypes = [C.c_uint16]
        L.lgo_fixed.restype = C.c_int64
        L.lgo_fixed.argtypes = [C.c_float]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def trace(packed, ray_stride: int = 1, ray_offset: int = 0, threads: int = 0, cap: int | None = None):
    """Trace a packed scene.  Returns (segments, path records, fp64 endpoints, stats)."""
    L = lib()
    seg_dt, path_dt = abi.segment_dtype(), abi.path_dtype()
    if cap is None:
        prim = sum(packed.lights[i].num_rays for i in range(packed.n_lights))
        cap = max(1024, 4 * prim // max(1, ray_stride))
    for _ in range(2):
        segs = np.zeros(cap, seg_dt)
        paths = np.zeros(cap, path_dt)
        s64 = np.zeros((cap, 4), np.float64)
        n = C.c_uint64(0)
        st = lgo_stats()
        rc = L.lgo_trace(*packed.args(), C.byref(packed.params), ray_stride, ray_offset, threads,
                         segs.ctypes.data_as(C.POINTER(abi.lg_segment)),
                         paths.ctypes.data_as(C.POINTER(abi.lg_path_record)),
                         s64.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(n), C.byref(st))
        if rc == -6:
            cap = int(n.value) + 16
            continue
        if rc != 0:
            raise OracleError(f"lgo_trace failed: {rc}")
        k = int(n.value)
        return segs[:k], paths[:k], s64[:k], st
    raise OracleError("lgo_trace: truncated twice")


def light_rays(light: abi.lg_light) -> np.ndarray:
    out = np.zeros((light.num_rays, 4), np.float64)
    rc = lib().lgo_light_rays(C.byref(light), out.ctypes.data_as(C.POINTER(C.c_double)), light.num_rays)
    if rc:
        raise OracleError(f"lgo_light_rays: {rc}")
    return out


def geo_hits(packed_geos, n_geo: int, root: int, o, d, cap: int = 64):
    out = (lgo_hit * cap)()
    fl = C.c_uint32(0)
    n = lib().lgo_geo_hits(packed_geos, n_geo, root, o[0], o[1], d[0], d[1], out, cap, C.byref(fl))
    if n < 0:
        raise OracleError(f"lgo_geo_hits: {n}")
    return [(h.t, (h.px, h.py), (h.nx, h.ny)) for h in out[:n]], fl.value


def geo_contains(packed_geos, n_geo: int, root: int, p) -> bool:
    r = lib().lgo_geo_contains(packed_geos, n_geo, root, p[0], p[1])
    if r < 0:
        raise OracleError(f"lgo_geo_contains: {r}")
    return bool(r)


def refract(d, n, n1, n2):
    rl = (C.c_double * 2)()
    rr = (C.c_double * 2)()
    R = C.c_double()
    ok = lib().lgo_refract(d[0], d[1], n[0], n[1], n1, n2, rl, rr, C.byref(R))
    return (rl[0], rl[1]), ((rr[0], rr[1]) if ok else None), R.value


def clear(params) -> np.ndarray:
    acc = np.zeros((params.height, params.width, 4), np.int64)
    lib().lgo_clear(acc.ctypes.data_as(C.POINTER(C.c_int64)), params.width, params.height, C.byref(params))
    return acc


def string_mod_chords(params) -> np.ndarray:
    """The string-mod lines of params.string_mod (lgo_string_mod_chords)."""
    n = C.c_uint64(0)
    rc = lib().lgo_string_mod_chords(C.byref(params), None, 0, C.byref(n))
    if rc not in (0, LGO_ERR_TRUNCATED):
        raise OracleError(f"lgo_string_mod_chords: {rc}")
    out = np.zeros(int(n.value), abi.chord_dtype())
    rc = lib().lgo_string_mod_chords(C.byref(params), out.ctypes.data_as(C.POINTER(abi.lg_chord)), len(out),
                                     C.byref(n))
    if rc:
        raise OracleError(f"lgo_string_mod_chords: {rc}")
    return out


def seg_cross(a, b, c, d):
    """The crossing point of segments ab and cd, or None (lgo_seg_cross)."""
    x, y = C.c_double(0.0), C.c_double(0.0)
    if lib().lgo_seg_cross(a[0], a[1], b[0], b[1], c[0], c[1], d[0], d[1], C.byref(x), C.byref(y)):
        return x.value, y.value
    return None


def string_mod_crossings(sm) -> np.ndarray:
    """Crossing points of the lines of an lg_string_mod, (n, 2) FP64 (lgo_string_mod_crossings)."""
    n = C.c_uint64(0)
    rc = lib().lgo_string_mod_crossings(C.byref(sm), None, 0, C.byref(n))
    if rc:
        raise OracleError(f"lgo_string_mod_crossings: {rc}")
    out = np.zeros((int(n.value), 2), np.float64)
    rc = lib().lgo_string_mod_crossings(C.byref(sm), out.ctypes.data_as(C.POINTER(C.c_double)), len(out),
                                        C.byref(n))
    if rc:
        raise OracleError(f"lgo_string_mod_crossings: {rc}")
    return out


def raster(segs: np.ndarray, params, threads: int = 0, acc: np.ndarray | None = None, chords=None):
    """Fixed-point raster of segments (and string-mod lines) into a cleared image.
    Returns (image int64, pixels)."""
    if acc is None:
        acc = clear(params)
    segs = np.ascontiguousarray(segs)
    px = C.c_uint64(0)
    rc = lib().lgo_raster(segs.ctypes.data_as(C.POINTER(abi.lg_segment)), len(segs), C.byref(params),
                          acc.ctypes.data_as(C.POINTER(C.c_int64)), threads, C.byref(px))
    if rc:
        raise OracleError(f"lgo_raster: {rc}")
    total = int(px.value)
    if chords is not None and len(chords):
        ch = np.ascontiguousarray(chords, dtype=abi.chord_dtype())
        rc = lib().lgo_raster_chords(ch.ctypes.data_as(C.POINTER(abi.lg_chord)), len(ch), C.byref(params),
                                     acc.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(px))
        if rc:
            raise OracleError(f"lgo_raster_chords: {rc}")
        total += int(px.value)
    return acc, total


def raster_f64(segs: np.ndarray, params, chords=None):
    acc = np.zeros((params.height, params.width, 4), np.float64)
    acc[...] = np.array(params.clear_color[:], np.float64)
    segs = np.ascontiguousarray(segs)
    px = C.c_uint64(0)
    rc = lib().lgo_raster_f64(segs.ctypes.data_as(C.POINTER(abi.lg_segment)), len(segs), C.byref(params),
                              acc.ctypes.data_as(C.POINTER(C.c_double)), C.byref(px))
    if rc:
        raise OracleError(f"lgo_raster_f64: {rc}")
    total = int(px.value)
    if chords is not None and len(chords):
        ch = np.ascontiguousarray(chords, dtype=abi.chord_dtype())
        rc = lib().lgo_raster_chords_f64(ch.ctypes.data_as(C.POINTER(abi.lg_chord)), len(ch), C.byref(params),
                                         acc.ctypes.data_as(C.POINTER(C.c_double)), C.byref(px))
        if rc:
            raise OracleError(f"lgo_raster_chords_f64: {rc}")
        total += int(px.value)
    return acc, total


def resolve_f16(acc: np.ndarray) -> np.ndarray:
    h, w = acc.shape[:2]
    out = np.zeros((h, w, 4), np.uint16)
    a = np.ascontiguousarray(acc)
    lib().lgo_resolve_f16(a.ctypes.data_as(C.POINTER(C.c_int64)), w, h, out.ctypes.data_as(C.POINTER(C.c_uint16)))
    return out


def resolve_rgba8(acc: np.ndarray) -> np.ndarray:
    h, w = acc.shape[:2]
    out = np.zeros((h, w, 4), np.uint8)
    a = np.ascontiguousarray(acc)
    lib().lgo_resolve_rgba8(a.ctypes.data_as(C.POINTER(C.c_int64)), w, h, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def sincos(x: float):
    """(sin x, cos x) of the ray generators (lg_oracle.c lgo_sincos)."""
    s, c = C.c_double(), C.c_double()
    lib().lgo_sincos(float(x), C.byref(s), C.byref(c))
    return s.value, c.value


def atan(x: float) -> float:
    """atan of the spot-light generator (lg_oracle.c lgo_atan)."""
    return lib().lgo_atan(float(x))
