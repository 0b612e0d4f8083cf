"""light_garden_gb300 — GB300-native (sm_103a) trace-and-accumulate path of light_garden.

The compute lives in ``_lib/liblightgarden_cuda.so`` (hand-written CUDA, C ABI in
``include/lg.h``).  This package holds the host-side mirror of the reference's scene model
and ``Tracer`` API, seeded benchmark scenes, and a ctypes handle over the library.
"""
from . import abi
from .scene import (Circle, CubicBezier, DirectionalLight, Geo, LineSegment, Logic, Material, Object,
                    PointLight, Rect, SpotLight, pack)

__all__ = ["abi", "Circle", "CubicBezier", "DirectionalLight", "Geo", "LineSegment", "Logic", "Material",
           "Object", "PointLight", "Rect", "SpotLight", "pack", "Context", "Tracer"]


def __getattr__(name):
    # the CUDA-backed classes load the shared library on first use
    if name == "Context":
        from .runtime import Context
        return Context
    if name == "Tracer":
        from .tracer import Tracer
        return Tracer
    raise AttributeError(name)
