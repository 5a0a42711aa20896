"""GB300-native sculpt-brush dab path (PBVH search, brushes, normals, bounds).

The compute lives in libsculptgpu.so (hand-written CUDA for sm_103a behind the
C ABI of include/sculpt_gpu.h); ``sculpt`` binds it, ``synth`` makes the seeded
workloads.
"""
from . import synth  # noqa: F401
from .sculpt import PBVH, SculptGPUError, load  # noqa: F401

__all__ = ["PBVH", "SculptGPUError", "load", "synth"]
