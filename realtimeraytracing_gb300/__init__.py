"""GB300-native ray-tracing core: Morton codes, Onesweep radix sort, PLOC BVH
build and BVH2 closest-hit / any-hit traversal as hand-written CUDA kernels
for sm_103a behind the C ABI in include/crt.h (libcrt.so).

It replaces the BVH build (srcCommon/scene/geometry/bvh.cpp) and the traversal
compute shader (srcCommon/shaders/raytracer.glsl) of MrBigoudi/RealTimeRaytracing.
"""
from . import crt, scenes  # noqa: F401
from .bvh import BVH, Raytracer, default_context  # noqa: F401
from .crt import Context, CrtError  # noqa: F401
