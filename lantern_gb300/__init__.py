"""lantern_gb300 -- GB300-native rebuild of Lantern's per-pixel path-tracing loop.

The compute path is liblantern_gpu.so (hand-written sm_103a CUDA behind the C
ABI in include/lantern_gpu.h); this package builds it in-tree, binds it with
ctypes and mirrors the reference's Scene / FrameBuffer / Integrator interface.
"""
from .native import LanternError, Context, load  # noqa: F401

__all__ = ["LanternError", "Context", "load"]
