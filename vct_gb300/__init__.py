"""GB300-native voxel cone tracing hot path (voxelize, inject, mip, trace).

The product is the CUDA library `libvct.so` with the C ABI of
include/vct.h; this package holds its sources (csrc/), its build recipe
(build.py), a ctypes binding (_lib.py), a thin Python mirror of the C ABI
(api.py) and the seeded synthetic scenes of the benchmarks (scenes.py).
"""

__all__ = ["api", "scenes", "build"]
