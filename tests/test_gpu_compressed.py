"""Compressed 4-wide traversal nodes (CRT_TRACE_COMPRESSED): 64-byte nodes
whose child boxes are 8-bit step counts from the node's origin, rounded
outward.  The walk must return the oracle's hits bit for bit in both
predicates — with the shader's predicate by re-checking each leaf's exact box
(from its triangle) with the shader's slab test before the triangle test —
while the reference-layout node array stays the export."""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

from test_gpu_trace import _cmp_hits
from test_refit_oracle import moved

pytestmark = pytest.mark.gpu

FLAGS = [crt.TRI_REFERENCE, crt.TRI_WATERTIGHT, crt.TRI_WATERTIGHT | crt.TRACE_ANY, crt.TRI_REFERENCE | crt.TRACE_ANY]


@pytest.fixture(scope="module")
def scenes(ctx):
    out = {}
    tris, models, cam, (w, h) = S.config0_scene(seed=0)
    out["soup"] = (tris, models, O.raygen(cam, w, h))
    v, f = S.displaced_icosphere(level=6, seed=1)
    ico = S.indexed_to_triangles(v, f)
    out["icosphere"] = (ico, S.identity_models(1),
                        np.concatenate([O.raygen(S.camera_gpu_data((0.0, 0.0, -3.0)), 96, 96), S.sphere_rays(8192, 2, 3.0, (0, 0, 0))]))
    dup = np.concatenate([S.uniform_soup(3000, seed=9)] * 3)  # exact duplicates: equal-t ties
    two = S.uniform_soup(4000, seed=10)
    two.view(np.uint32)[:, 12] = np.arange(4000, dtype=np.uint32) % 2
    m2 = S.identity_models(2)
    m2[1, 12:15] = (0.5, -0.25, 1.0)
    out["duplicates"] = (dup, S.identity_models(1), O.raygen(S.camera_gpu_data((0.5, 0.5, -1.5)), 128, 128))
    out["two_models"] = (two, m2, S.sphere_rays(20000, seed=3))
    return out


@pytest.mark.parametrize("name", ["soup", "icosphere", "duplicates", "two_models"])
@pytest.mark.parametrize("flags", FLAGS)
def test_compressed_walk_matches_oracle(ctx, scenes, name, flags):
    tris, models, rays = scenes[name]
    bvh = ctx.build(tris, models=models)
    ref, _ = O.trace(bvh.nodes(), tris, models, rays, flags & (crt.TRI_WATERTIGHT | crt.TRACE_ANY))
    any_hit = bool(flags & crt.TRACE_ANY)
    _cmp_hits(ctx.trace(bvh, rays, flags | crt.TRACE_COMPRESSED), ref, any_hit)
    bvh.free()


def test_compressed_fetches_and_refit(ctx, scenes):
    """Half the binary walk's node fetches (about the 4-wide walk's), and the
    compressed nodes follow a refit."""
    tris, models, rays = scenes["soup"]
    bvh = ctx.build(tris, models=models)
    counts = {}
    for name, f in (("binary", 0), ("wide", crt.TRACE_WIDE), ("compressed", crt.TRACE_COMPRESSED)):
        ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.TRACE_STATS | f)
        counts[name] = ctx.last_trace_stats()[0]
    assert counts["compressed"] < 0.75 * counts["binary"]
    assert counts["wide"] <= counts["compressed"] < 1.5 * counts["wide"]
    new = moved(tris, 0.9, amp=0.03)
    bvh.refit(new, models=models)
    nodes = bvh.nodes()
    for f in (crt.TRI_REFERENCE, crt.TRI_WATERTIGHT):
        ref, _ = O.trace(nodes, new, models, rays, f)
        _cmp_hits(ctx.trace(bvh, rays, f | crt.TRACE_COMPRESSED), ref)
    bvh.free()


def test_compressed_frame(ctx):
    tris, models, cam, (w, h), light = S.config1_scene(seed=0, level=5)
    bvh = ctx.build(tris, models=models)
    hp, hs = ctx.trace_frame(bvh, cam, 128, 96, light, crt.TRI_WATERTIGHT)
    cp, cs = ctx.trace_frame(bvh, cam, 128, 96, light, crt.TRI_WATERTIGHT | crt.TRACE_COMPRESSED)
    np.testing.assert_array_equal(cp.view(np.uint32), hp.view(np.uint32))
    np.testing.assert_array_equal(cs.view(np.uint32)[:, 0] == crt.MISS, hs.view(np.uint32)[:, 0] == crt.MISS)
    bvh.free()


@pytest.mark.parametrize("n", [1, 2, 3, 5, 33, 1025])
def test_compressed_small_trees(ctx, n):
    tris = S.uniform_soup(n, seed=40 + n, edge_lo=0.05, edge_hi=0.3)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    rays = S.sphere_rays(4096, seed=n)
    for flags in (crt.TRI_REFERENCE, crt.TRI_WATERTIGHT):
        ref, _ = O.trace(bvh.nodes(), tris, models, rays, flags)
        _cmp_hits(ctx.trace(bvh, rays, flags | crt.TRACE_COMPRESSED), ref)
    bvh.free()
