"""Thin Python handle over one ``lg_ctx`` of liblightgarden_cuda.so.

Every method calls exactly one C entry point and raises :class:`abi.LgError` with the
library's status and message on failure.  No computation happens here: there is no CPU
fallback, and constructing a :class:`Context` without the CUDA library raises.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np

from . import abi
from .scene import PackedScene


class Context:
    def __init__(self, device: int = 0, segment_capacity: int = 0, queue_capacity: int = 0, raster_variant: int = 0):
        self.lib = abi.load()
        opts = abi.lg_device_opts(device, raster_variant, segment_capacity, queue_capacity)
        h = C.c_void_p()
        st = self.lib.lg_create(C.byref(h), C.byref(opts))
        if st != abi.LG_OK:
            raise abi.LgError(st, "lg_create failed")
        self.h = h
        self.params: Optional[abi.lg_params] = None

    # -- helpers -------------------------------------------------------------------------
    def _check(self, st: int, what: str) -> None:
        if st != abi.LG_OK:
            msg = self.lib.lg_last_error(self.h)
            raise abi.LgError(st, f"{what}: {msg.decode() if msg else ''}")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.lg_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- one scene -----------------------------------------------------------------------
    def upload(self, scene: PackedScene) -> None:
        st = self.lib.lg_scene_upload(self.h, *scene.args(), C.byref(scene.params))
        self._check(st, "lg_scene_upload")
        self.params = scene.params

    def trace(self) -> dict:
        s = abi.lg_trace_stats()
        self._check(self.lib.lg_trace(self.h, C.byref(s)), "lg_trace")
        return s.as_dict()

    def accumulate(self) -> dict:
        s = abi.lg_trace_stats()
        self._check(self.lib.lg_accumulate(self.h, C.byref(s)), "lg_accumulate")
        return s.as_dict()

    def accumulate_segments(self, segs: np.ndarray) -> dict:
        segs = np.ascontiguousarray(segs, dtype=abi.segment_dtype())
        s = abi.lg_trace_stats()
        st = self.lib.lg_accumulate_segments(self.h, segs.ctypes.data_as(C.POINTER(abi.lg_segment)), len(segs),
                                             C.byref(s))
        self._check(st, "lg_accumulate_segments")
        return s.as_dict()

    def _shape(self) -> Tuple[int, int]:
        return self.params.height, self.params.width

    def resolve_f16(self) -> np.ndarray:
        h, w = self._shape()
        out = np.zeros((h, w, 4), np.uint16)
        self._check(self.lib.lg_resolve_f16(self.h, out.ctypes.data_as(C.c_void_p), w * 8, 0), "lg_resolve_f16")
        return out

    def resolve_rgba8(self) -> np.ndarray:
        h, w = self._shape()
        out = np.zeros((h, w, 4), np.uint8)
        self._check(self.lib.lg_resolve_rgba8(self.h, out.ctypes.data_as(C.c_void_p), w * 4, 0), "lg_resolve_rgba8")
        return out

    def render(self, out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, dict]:
        h, w = self._shape()
        if out is None:
            out = np.zeros((h, w, 4), np.uint16)
        s = abi.lg_trace_stats()
        st = self.lib.lg_render(self.h, out.ctypes.data_as(C.c_void_p), out.strides[0], 0, C.byref(s))
        self._check(st, "lg_render")
        return out, s.as_dict()

    def render_into(self, ptr: int, pitch: int, on_device: bool) -> dict:
        s = abi.lg_trace_stats()
        st = self.lib.lg_render(self.h, C.c_void_p(ptr), pitch, 1 if on_device else 0, C.byref(s))
        self._check(st, "lg_render")
        return s.as_dict()

    def segments(self, paths: bool = False):
        n = C.c_uint64(0)
        st = self.lib.lg_segments_download(self.h, None, None, 0, C.byref(n))
        if st not in (abi.LG_OK, abi.LG_ERR_TRUNCATED):
            self._check(st, "lg_segments_download")
        k = int(n.value)
        segs = np.zeros(k, abi.segment_dtype())
        recs = np.zeros(k, abi.path_dtype()) if paths else None
        st = self.lib.lg_segments_download(
            self.h, segs.ctypes.data_as(C.POINTER(abi.lg_segment)),
            recs.ctypes.data_as(C.POINTER(abi.lg_path_record)) if paths else None, k, C.byref(n))
        self._check(st, "lg_segments_download")
        return (segs, recs) if paths else segs

    def accum(self) -> np.ndarray:
        h, w = self._shape()
        dt = np.float32 if self.params.accum == abi.LG_ACCUM_F32 else np.int64
        out = np.zeros((h, w, 4), dt)
        self._check(self.lib.lg_accum_download(self.h, out.ctypes.data_as(C.c_void_p), out.nbytes),
                    "lg_accum_download")
        return out
