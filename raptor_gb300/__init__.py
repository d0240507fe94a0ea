"""GB300-native ray-tracing core for RAPTor's raytracer hot path.

The product is the shared library built from csrc/ (C ABI in
include/rtcore.h).  `core` binds it through ctypes, `scenes` generates the
seeded synthetic workloads, `build` compiles the library in-tree.
"""
__all__ = ["build", "core", "scenes"]
