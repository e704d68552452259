"""draw_gb300: a GB300-native (sm_103a) drop-in for the CPU draw call of the
draw software renderer (mororo18/draw): vertex transform, near/far clipping,
triangle setup, edge-function rasterization, depth test, Phong-style shading
with texture mapping.

The compute path is the CUDA library ``_lib/libdrawgpu.so`` (C ABI in
include/draw_gpu.h); ``renderer`` mirrors the reference's Scene / Camera /
Object / Texture / TextureMap / Canvas API on top of it. The library is loaded
when the first Context is created.
"""
from . import renderer, scenes  # noqa: F401

__all__ = ["scenes", "renderer"]
