"""Host-side mirror of the reference's BVH interface, backed by libcrt.

The reference builds its BVH with
    cr::BVH::BVH(uint32_t nbTriangles,
                 const std::vector<TriangleGPU>& unsortedTriangles,
                 const std::vector<MeshModelGPU>& meshesInTheScene)
        srcCommon/scene/geometry/bvh.hpp:89-91, bvh.cpp:11-24
and Scene::getBVH_NodesToGPUData (srcOpenGL/scene/scene.cpp:203-208)
flattens it into the node array the shader reads; getClosestHitBVH
(srcCommon/shaders/raytracer.glsl:246-295) traces it per pixel and getColor
(:159-179) shades it.  BVH and Raytracer below keep those names and argument
meanings; all work runs in the CUDA library.
"""
from __future__ import annotations

import numpy as np

from . import crt

MAX_NB_TRIANGLES = 2 << 15   # Triangle::MAX_NB_TRIANGLES (triangle.hpp:21); the GPU path has no such cap
MAX_NB_MESHES = 2 << 5       # Mesh::MAX_NB_MESHES (mesh.hpp:26)

_default_ctx = None


def default_context() -> crt.Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = crt.Context()
    return _default_ctx


class Mesh:
    """cr::Mesh::load (srcCommon/scene/geometry/mesh.cpp:186-263): an OBJ
    file's faces as TriangleGPU records of model `meshId`, read on the host
    and assembled on the GPU.  Scenes concatenate meshes' records, as
    Scene::getTriangleToGPUData does (srcOpenGL/scene/scene.cpp:26-40)."""

    @staticmethod
    def load(path: str, meshId: int = 0, ctx: crt.Context | None = None, out=None):
        ctx = ctx or default_context()
        vertices, indices = crt.parse_obj(path)
        return ctx.triangles_from_indexed(vertices, indices, meshId, out)


class BVH:
    """cr::BVH.  `unsortedTriangles` is the (n_buffer, 16) float32 TriangleGPU
    buffer — the reference scans every entry of it for the scene box
    (bvh.cpp:237) and builds over the first `nbTriangles`; `meshesInTheScene`
    is the (m <= 64, 17) MeshModelGPU buffer."""

    def __init__(self, nbTriangles: int, unsortedTriangles, meshesInTheScene=None, ctx: crt.Context | None = None):
        if nbTriangles < 1:
            raise ValueError("nbTriangles must be >= 1")
        self._ctx = ctx or default_context()
        self._NbTriangles = int(nbTriangles)
        self._bvh = self._ctx.build(unsortedTriangles, n_tris=self._NbTriangles, models=meshesInTheScene)
        self.build_stats = self._ctx.last_build_stats()

    @property
    def _TriangleIndices(self) -> np.ndarray:
        """Sorted position -> triangle index (BVH_Params::_TriangleIndices)."""
        return self._bvh.perm()

    @property
    def _MortonCodes(self) -> np.ndarray:
        """Sorted Morton codes (PlocParams::_MortonCodes after the sort)."""
        return self._bvh.codes()

    def getBVH_NodesToGPUData(self) -> np.ndarray:
        """The (2N-1, 12) node array Scene::getBVH_NodesToGPUData returns:
        DFS pre-order, left subtree first, BVH_NodeGPU records."""
        return self._bvh.nodes()

    @property
    def handle(self) -> crt.Bvh:
        return self._bvh


class Raytracer:
    """The compute pass of Application::drawOneFrame (application.cpp:220-262):
    getRay for every texel, getClosestHitBVH, getColor and imageStore.  The
    shader's uniforms (application.cpp:229-232) are the attributes below."""

    def __init__(self, ctx: crt.Context | None = None):
        self._ctx = ctx or default_context()
        self.uIsWireframeModeOn = False
        self.uIsBVHDisplayed = False
        self.uDepthDisplayBVH = 0

    def _shade_flags(self) -> int:
        return (crt.SHADE_WIREFRAME if self.uIsWireframeModeOn else 0) | (crt.SHADE_BVH if self.uIsBVHDisplayed else 0)

    def getColor(self, bvh: BVH, rays, hits, models=None, materials=None, out=None):
        """getColor (raytracer.glsl:159-179) for each hit: (n, 4) RGBA32F texels."""
        return self._ctx.shade(bvh.handle, rays, hits, models, materials, self._shade_flags(),
                               self.uDepthDisplayBVH, out)

    def drawOneFrame(self, bvh: BVH, camera_gpu, width: int, height: int, models=None, materials=None,
                     watertight: bool = False, out=None):
        """One dispatch of raytracer.glsl main: the (width*height, 4) RGBA32F
        oImage texels, texel (x, y) at row y * width + x."""
        flags = crt.TRI_WATERTIGHT if watertight else crt.TRI_REFERENCE
        return self._ctx.render_frame(bvh.handle, camera_gpu, width, height, models, materials,
                                      self._shade_flags(), self.uDepthDisplayBVH, flags, out)

    def getRays(self, camera_gpu, width: int, height: int, out=None):
        return self._ctx.raygen(camera_gpu, width, height, out)

    def getClosestHitBVH(self, bvh: BVH, rays, watertight: bool = False, out=None):
        flags = crt.TRACE_CLOSEST | (crt.TRI_WATERTIGHT if watertight else crt.TRI_REFERENCE)
        return self._ctx.trace(bvh.handle, rays, flags, out)

    def getAnyHitBVH(self, bvh: BVH, rays, watertight: bool = True, out=None):
        flags = crt.TRACE_ANY | (crt.TRI_WATERTIGHT if watertight else crt.TRI_REFERENCE)
        return self._ctx.trace(bvh.handle, rays, flags, out)
