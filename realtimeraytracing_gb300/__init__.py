"""GB300-native ray-tracing core: Morton codes, Onesweep radix sort, PLOC BVH
build and refit, BVH2 closest-hit / any-hit traversal, the shading pass and
mesh input as hand-written CUDA kernels for sm_103a behind the C ABI in
include/crt.h (libcrt.so).

It replaces the BVH build (srcCommon/scene/geometry/bvh.cpp), the compute
shader's traversal and shading (srcCommon/shaders/raytracer.glsl) and the
TriangleGPU assembly of the mesh loader (srcCommon/scene/geometry/mesh.cpp)
of MrBigoudi/RealTimeRaytracing.
"""
from . import crt, image, scenes  # noqa: F401
from .bvh import BVH, Mesh, Raytracer, default_context  # noqa: F401
from .crt import Context, CrtError, parse_obj  # noqa: F401
