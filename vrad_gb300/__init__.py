"""GB300 (sm_103a) radiosity hot path behind the VRAD ("VRADiant") entry points.

The product is libvradgpu.so (C ABI: include/vradgpu.h).  This package builds
it (``build``), binds it (``_lib``) and mirrors the reference's Go API on top
(``environment``); ``scenes`` holds the seeded synthetic scene generators.
"""
from . import build  # noqa: F401
from .environment import Context, Environment, Light, make_light  # noqa: F401

__all__ = ["Context", "Environment", "Light", "make_light", "build"]
