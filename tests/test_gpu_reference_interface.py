"""The host mirror of the reference's interface (realtimeraytracing_gb300.bvh),
used the way the reference uses its own classes, against the CPU oracle bit
for bit.

Reference: cr::BVH::BVH(nbTriangles, unsortedTriangles, meshesInTheScene)
(srcCommon/scene/geometry/bvh.hpp:89-91, bvh.cpp:11-24) over the padded
65,536-entry triangle buffer Scene allocates (srcOpenGL/scene/scene.cpp:27);
Scene::getBVH_NodesToGPUData (scene.cpp:189-208); and the compute pass of
Application::drawOneFrame (application.cpp:220-262): getRay, getClosestHitBVH
and getColor (srcCommon/shaders/raytracer.glsl:92-100, 246-295, 159-179).
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import bvh as B
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 3, 1000, 20000])
def test_bvh_over_the_padded_buffer_matches_oracle(ctx, n):
    """nbTriangles real records at the front of a zero-padded buffer of
    MAX_NB_TRIANGLES entries: the scene box covers the padding too (bvh.cpp:237)."""
    buf = np.zeros((B.MAX_NB_TRIANGLES, 16), np.float32)
    buf[:n] = S.uniform_soup(n, seed=40 + n)
    models = S.identity_models(1)
    bvh = B.BVH(n, buf, models, ctx=ctx)
    ref = O.build_bvh(buf, n, models)
    assert np.array_equal(bvh._MortonCodes, ref["codes"])
    assert np.array_equal(bvh._TriangleIndices, ref["perm"])
    nodes = bvh.getBVH_NodesToGPUData()
    assert nodes.shape == (2 * n - 1, 12)
    assert np.array_equal(nodes.view(np.uint32), ref["nodes"].view(np.uint32))


def test_raytracer_compute_pass_matches_oracle(ctx):
    n = 20000
    tris = S.uniform_soup(n, seed=17, edge_lo=0.005, edge_hi=0.04)
    models = S.identity_models(1)
    mats = S.materials([[0.75, 0.5, 0.25, 1.0]])
    bvh = B.BVH(n, tris, models, ctx=ctx)
    nodes = bvh.getBVH_NodesToGPUData()
    rt = B.Raytracer(ctx)
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    w, h = 128, 96
    rays = rt.getRays(cam, w, h)
    assert np.array_equal(rays.view(np.uint32), O.raygen(cam, w, h).view(np.uint32))
    for watertight, tri_flags in ((False, crt.TRI_REFERENCE), (True, crt.TRI_WATERTIGHT)):
        hits = rt.getClosestHitBVH(bvh, rays, watertight=watertight)
        want, _ = O.trace(nodes, tris, models, rays, tri_flags)
        assert np.array_equal(hits.view(np.uint32), want.view(np.uint32))
        assert (hits.view(np.int32)[:, 0] >= 0).sum() > 100
        occluded = rt.getAnyHitBVH(bvh, rays, watertight=watertight)
        assert np.array_equal(occluded.view(np.int32)[:, 0] >= 0, want.view(np.int32)[:, 0] >= 0)
    # getColor / drawOneFrame with the shader's uniforms set
    rt.uIsWireframeModeOn = True
    rt.uIsBVHDisplayed = True
    rt.uDepthDisplayBVH = 2
    flags = crt.SHADE_WIREFRAME | crt.SHADE_BVH
    ref_hits, _ = O.trace(nodes, tris, models, rays, crt.TRI_REFERENCE)
    want = O.shade(nodes, tris, models, mats, rays, ref_hits, flags, 2)
    img = rt.drawOneFrame(bvh, cam, w, h, models=models, materials=mats)
    assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
    texels = rt.getColor(bvh, rays, ref_hits, models=models, materials=mats)
    assert np.array_equal(texels.view(np.uint32), want.view(np.uint32))
