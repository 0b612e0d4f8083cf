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
    def __init__(self, device: int = 0, segment_capacity: int = 0, queue_capacity: int = 0, raster_variant: int = 0,
                 stream_segments: int = 0, culling: int = abi.LG_CULL_AUTO, grid_density: float = 0.0,
                 wait_polls: int = 0, scan_pairs: int = 0):
        self.lib = abi.load()
        opts = abi.lg_device_opts(device, raster_variant, segment_capacity, queue_capacity, stream_segments, culling,
                                  grid_density, wait_polls, scan_pairs)
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

    def chords(self):
        """The frame's string-mod lines (lg_chord records), two colours each."""
        n = C.c_uint64(0)
        st = self.lib.lg_chords_download(self.h, None, 0, C.byref(n))
        if st not in (abi.LG_OK, abi.LG_ERR_TRUNCATED):
            self._check(st, "lg_chords_download")
        out = np.zeros(int(n.value), abi.chord_dtype())
        self._check(self.lib.lg_chords_download(self.h, out.ctypes.data_as(C.POINTER(abi.lg_chord)), len(out),
                                                C.byref(n)), "lg_chords_download")
        return out

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

    # -- many scenes -------------------------------------------------------------------------
    @staticmethod
    def _desc(d, sc) -> None:
        d.geos = C.cast(sc.geos, C.POINTER(abi.lg_geo))
        d.objects = C.cast(sc.objects, C.POINTER(abi.lg_object))
        d.lights = C.cast(sc.lights, C.POINTER(abi.lg_light))
        d.params = C.pointer(sc.params)
        d.n_geo, d.n_objects, d.n_lights = sc.n_geo, sc.n_objects, sc.n_lights

    def batch_upload(self, scenes) -> None:
        """Upload a batch of PackedScene (lg_batch_upload)."""
        descs = (abi.lg_scene_desc * len(scenes))()
        for d, sc in zip(descs, scenes):
            self._desc(d, sc)
        self._check(self.lib.lg_batch_upload(self.h, descs, len(scenes)), "lg_batch_upload")
        self.batch_shapes = [(sc.params.height, sc.params.width) for sc in scenes]
        self.batch_offsets = []
        for i in range(len(scenes)):
            off = C.c_uint64(0)
            self._check(self.lib.lg_batch_image_offset(self.h, i, C.byref(off)), "lg_batch_image_offset")
            self.batch_offsets.append(int(off.value))
        self.params = None

    def batch_pixels(self) -> int:
        return sum(h * w for h, w in self.batch_shapes)

    def batch_render_into(self, ptr: int, nbytes: int, on_device: bool) -> dict:
        s = abi.lg_trace_stats()
        st = self.lib.lg_batch_render(self.h, C.c_void_p(ptr), nbytes, 1 if on_device else 0, C.byref(s))
        self._check(st, "lg_batch_render")
        return s.as_dict()

    def batch_render(self):
        """All images of the batch as a list of (height, width, 4) binary16 bit patterns."""
        flat = np.zeros(self.batch_pixels() * 4, np.uint16)
        stats = self.batch_render_into(flat.ctypes.data, flat.nbytes, False)
        imgs = [flat[4 * o:4 * (o + h * w)].reshape(h, w, 4) for o, (h, w) in zip(self.batch_offsets, self.batch_shapes)]
        return imgs, stats

    # -- serving ------------------------------------------------------------------------------
    def serve_begin(self, hbm_budget_bytes: int = 0, max_slots: int = 1024) -> None:
        opts = abi.lg_serve_opts(hbm_budget_bytes, max_slots, 0)
        self._check(self.lib.lg_serve_begin(self.h, C.byref(opts)), "lg_serve_begin")
        self.serve_shapes = {}

    def serve_submit(self, scene: PackedScene) -> int:
        d = abi.lg_scene_desc()
        self._desc(d, scene)
        rid = C.c_uint64(0)
        self._check(self.lib.lg_serve_submit(self.h, C.byref(d), C.byref(rid)), "lg_serve_submit")
        self.serve_shapes[int(rid.value)] = (scene.params.height, scene.params.width)
        return int(rid.value)

    def serve_step(self) -> dict:
        s = abi.lg_serve_step_stats()
        self._check(self.lib.lg_serve_step(self.h, C.byref(s)), "lg_serve_step")
        return s.as_dict()

    def serve_poll(self, rid: int) -> Optional[np.ndarray]:
        """The finished image of request rid, or None while it is queued or in flight."""
        h, w = self.serve_shapes[rid]
        out = np.zeros((h, w, 4), np.uint16)
        st = self.lib.lg_serve_poll(self.h, rid, out.ctypes.data_as(C.c_void_p), out.nbytes, 0)
        if st == abi.LG_ERR_NOT_READY:
            return None
        self._check(st, "lg_serve_poll")
        del self.serve_shapes[rid]
        return out

    def serve_end(self) -> None:
        self._check(self.lib.lg_serve_end(self.h), "lg_serve_end")

    def accum(self) -> np.ndarray:
        h, w = self._shape()
        dt = np.float32 if self.params.accum == abi.LG_ACCUM_F32 else np.int64
        out = np.zeros((h, w, 4), dt)
        self._check(self.lib.lg_accum_download(self.h, out.ctypes.data_as(C.c_void_p), out.nbytes),
                    "lg_accum_download")
        return out
