"""GB300-native LIC volume ray-caster (a drop-in for the voLIC LIC hot path).

The compute lives in libvvlic.so (CUDA kernels for sm_103a behind the C ABI of
include/vvlic.h); this package holds its ctypes binding (`capi`), the in-tree build step
(`build`) and the seeded synthetic workloads (`workloads`).
"""
from . import capi  # noqa: F401

__all__ = ["capi"]
