"""pbrt-v2 ray-batch intersection path, GB300-native (sm_103a).

Modules:
  accel   NaiveAccel / RayHieararchy / RayBVH over the C ABI
  scenes  seeded synthetic scenes and ray batches
  _lib    ctypes binding of include/pbrt_gb300.h
"""
from . import _lib  # noqa: F401
