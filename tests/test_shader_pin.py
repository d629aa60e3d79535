"""The traversal oracle pinned to the reference's own compute shader.

srcCommon/shaders/raytracer.glsl cannot run here (no graphics stack), but its
code compiles as C++: oracle/glsl_to_cpp.py rewrites only its declarations
(layout, uniform, buffer blocks, inout, main) and the project's GLSL shim
supplies the built-in types and functions (oracle/Makefile, target `ref`,
builds oracle/_ref/libref_shader.so where the reference checkout exists).
These tests run the shader's getClosestHitBVH (:246-295), getAllHits
(:149-157) and main (:299-331, with getRay, intersectBVH, getColor and
imageStore) on seeded scenes and require the oracle's restatement — the one
every GPU test compares the CUDA path with — to give the same bits.  The
golden index (tests/golden/index.json) carries the shader's outputs on the
65,536-triangle soup to machines without the reference checkout.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))
needs_shader = pytest.mark.skipif(not os.path.isdir(os.path.join(O.REFERENCE_DIR, "srcCommon")),
                                  reason="reference checkout not present (golden fixtures cover this machine)")


@pytest.fixture(scope="module", autouse=True)
def _shader_lib():
    if os.path.isdir(os.path.join(O.REFERENCE_DIR, "srcCommon")) and not O.shader_available():
        O.build(ref=True)


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _u32(a):
    return np.ascontiguousarray(a).view(np.uint32)


@needs_shader
def test_closest_hits_config0_soup():
    """All 262,144 primary rays of the 65,536-triangle soup: the shader's
    right-child-first DFS and triangle test against the restatement."""
    tris, models, cam, (w, h) = S.config0_scene(seed=0)
    nodes = O.build_bvh(tris, tris.shape[0], models)["nodes"]
    rays = O.raygen(cam, w, h)
    got = O.shader_closest_hits(nodes, tris, models, rays)
    want, _ = O.trace(nodes, tris, models, rays, 0)
    np.testing.assert_array_equal(_u32(got), _u32(want))
    assert (_u32(got)[:, 0] != 0xFFFFFFFF).sum() > 60000


@needs_shader
def test_closest_hits_models_and_ties():
    """Three model matrices, and 64 copies of one triangle (every leaf ties:
    the first leaf the shader's walk reaches must win)."""
    t = S.uniform_soup(2000, seed=78)
    t.view(np.uint32)[:, 12] = np.arange(2000) % 3
    m = S.identity_models(3)
    m[1, 12:15] = [0.5, -0.25, 2.0]
    m[2, 0:16] = np.array([0, 2, 0, 0, -1, 0, 0, 0, 0, 0, 0.5, 0, 0.125, 1, -1, 1], np.float32)
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = O.raygen(cam, 96, 96)
    nodes = O.build_bvh(t, t.shape[0], m)["nodes"]
    np.testing.assert_array_equal(_u32(O.shader_closest_hits(nodes, t, m, rays)),
                                  _u32(O.trace(nodes, t, m, rays, 0)[0]))
    # one triangle facing the camera (the shader culls back faces), 64 times
    v = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (64, 1))
    dup = S.pack_triangles(v, v + np.float32([0.0, 1.0, 0.0]), v + np.float32([1.0, 0.0, 0.0]))
    one = S.identity_models(1)
    dn = O.build_bvh(dup, 64, one)["nodes"]
    r2 = O.raygen(S.camera_gpu_data((0.5, 0.5, -1.5)), 64, 64)
    got = O.shader_closest_hits(dn, dup, one, r2)
    assert (_u32(got)[:, 0] != 0xFFFFFFFF).sum() > 400
    np.testing.assert_array_equal(_u32(got), _u32(O.trace(dn, dup, one, r2, 0)[0]))


@needs_shader
def test_all_hits_brute_force():
    tris = S.uniform_soup(4096, seed=80)
    models = S.identity_models(1)
    rays = O.raygen(S.camera_gpu_data((0.5, 0.5, -1.5)), 64, 64)
    np.testing.assert_array_equal(_u32(O.shader_all_hits(tris, models, rays)),
                                  _u32(O.trace_brute(tris, models, rays, 0)))


@needs_shader
@pytest.mark.parametrize("flags,depth", [(0, 0), (1, 0), (2, 0), (2, 3), (3, 2), (2, 7)])
def test_whole_compute_pass(flags, depth):
    """main: getRay per texel, closest hit, bvhColor of the box at uDepthDisplayBVH
    (flags 2), getColor with the wireframe (flags 1) and imageStore."""
    tris, models, cam, _ = S.config0_scene(seed=0)
    models = S.models_with_materials([1])
    mats = S.materials([[0.1, 0.2, 0.3, 1.0], [0.75, 0.5, 0.25, 1.0]])
    nodes = O.build_bvh(tris, tris.shape[0], models)["nodes"]
    w = h = 128
    img = O.shader_frame(cam, w, h, nodes, tris, models, mats, flags, depth)
    rays = O.raygen(cam, w, h)
    hits, _ = O.trace(nodes, tris, models, rays, 0)
    want = O.shade(nodes, tris, models, mats, rays, hits, flags, depth)
    np.testing.assert_array_equal(_u32(img), _u32(want))


@needs_shader
def test_golden_index_holds_the_shaders_outputs():
    with open(os.path.join(HERE, "golden", "index.json")) as f:
        index = json.load(f)
    tm = index["config0_trace"]
    assert "raytracer.glsl compiled as C++" in tm["source"]
    tris, models, cam, (w, h) = S.config0_scene(seed=0)
    nodes = O.build_bvh(tris, tris.shape[0], models)["nodes"]
    rays = O.raygen(cam, w, h)
    assert sha(O.shader_closest_hits(nodes, tris, models, rays)) == tm["hits_reference_sha256"]
    fr = index["config0_frame"]
    img = O.shader_frame(cam, fr["width"], fr["height"], nodes, tris, S.models_with_materials([1]),
                         S.materials(fr["materials"]), fr["flags"], fr["depth"])
    assert sha(img) == fr["texels_sha256"]
