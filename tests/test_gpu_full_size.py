"""Parity at the bench's own sizes, bit for bit against the CPU oracle.

The headline workload: the 1,310,720-triangle displaced icosphere and the
1920x1080 frame.  The build (codes, permutation, node array) must equal the
oracle's; the one-launch frame (crt_trace_frame: camera ray, closest hit,
shadow ray, any hit per pixel) must give the oracle's closest hits for every
pixel (both triangle predicates) and the oracle's occlusion for every shadow
ray; the shaded frame must equal the oracle's texels; and the treelet-
restructured tree (crt_optimize) must equal the oracle's at this size.  The
incoherent-bounce workload (4,194,304 clustered triangles, 8,388,608 bounce
rays) is checked the same way on a sample of its rays.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

from test_gpu_trace import _cmp_hits

pytestmark = pytest.mark.gpu


def _u(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def config1(ctx):
    tris, models, cam, (w, h), light = S.config1_scene(seed=0)
    ref = O.build_bvh(tris, tris.shape[0], models)
    bvh = ctx.build(tris, models=models)
    yield tris, models, cam, w, h, light, ref, bvh
    bvh.free()


def test_config1_build_bit_exact(ctx, config1):
    tris, models, cam, w, h, light, ref, bvh = config1
    np.testing.assert_array_equal(bvh.codes(), ref["codes"])
    np.testing.assert_array_equal(bvh.perm(), ref["perm"])
    bad = np.nonzero((_u(bvh.nodes()) != _u(ref["nodes"])).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} node records differ, first at {bad[:5]}"
    assert ctx.last_build_stats()["ploc_iterations"] == ref["iterations"]


def test_config1_frame_every_pixel(ctx, config1):
    tris, models, cam, w, h, light, ref, bvh = config1
    rays = O.raygen(cam, w, h)
    hp, hs = ctx.trace_frame(bvh, cam, w, h, light, crt.TRI_WATERTIGHT)
    want_p, _ = O.trace(ref["nodes"], tris, models, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(hp, want_p)
    assert 0.2 < float((_u(hp)[:, 0] != crt.MISS).mean()) < 0.6
    sh = O.shadow_rays(rays, want_p, light)
    want_s, _ = O.trace(ref["nodes"], tris, models, sh, crt.TRACE_ANY | crt.TRI_WATERTIGHT)
    _cmp_hits(hs, want_s, any_hit=True)
    hr, _ = ctx.trace_frame(bvh, cam, w, h, None, crt.TRI_REFERENCE)
    _cmp_hits(hr, O.trace(ref["nodes"], tris, models, rays, crt.TRI_REFERENCE)[0])


def test_config1_shaded_frame(ctx, config1):
    tris, models, cam, w, h, light, ref, bvh = config1
    mats = S.materials([[0.8, 0.6, 0.4, 1.0]])
    flags = crt.SHADE_WIREFRAME | crt.SHADE_BVH
    img = ctx.render_frame(bvh, cam, w, h, models=models, materials=mats, shade_flags=flags, bvh_depth=6)
    rays = O.raygen(cam, w, h)
    hits, _ = O.trace(ref["nodes"], tris, models, rays, crt.TRI_REFERENCE)
    want = O.shade(ref["nodes"], tris, models, mats, rays, hits, flags, 6)
    bad = np.nonzero((_u(img) != _u(want)).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} texels differ, first at {bad[:5]}"


def test_config1_optimized_tree(ctx, config1):
    tris, models, cam, w, h, light, ref, bvh = config1
    b = ctx.build(tris, models=models)
    b.optimize(1)
    want, _ = O.optimize(ref["nodes"], 1)
    bad = np.nonzero((_u(b.nodes()) != _u(want)).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} node records differ, first at {bad[:5]}"
    rays = O.raygen(cam, 480, 270)
    _cmp_hits(ctx.trace(b, rays, crt.TRI_WATERTIGHT), O.trace(want, tris, models, rays, crt.TRI_WATERTIGHT)[0])
    b.free()


def test_config3_build_and_bounce_rays(ctx):
    """The incoherent-bounce workload: the 4,194,304-triangle clustered soup
    built bit for bit, 2048x2048 primary hits, 8,388,608 cosine bounce rays;
    the plain trace matches the oracle's closest hits (every 8th ray), and the
    rays traced in sorted order and over the restructured tree give the plain
    trace's hits for every ray."""
    tris, models = S.config3_scene(seed=0)
    ref = O.build_bvh(tris, tris.shape[0], models)
    bvh = ctx.build(tris, models=models)
    bad = np.nonzero((_u(bvh.nodes()) != _u(ref["nodes"])).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} node records differ, first at {bad[:5]}"
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    prim = ctx.raygen(cam, 2048, 2048)
    ph = ctx.trace(bvh, prim, crt.TRI_WATERTIGHT)
    rays = ctx.bounce_rays(bvh, prim, ph, 8 * 1024 * 1024, seed=11)
    sample = rays[::8].copy()
    want, _ = O.trace(ref["nodes"], tris, models, sample, crt.TRI_WATERTIGHT)
    plain = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(plain[::8], want)
    assert float((_u(plain)[:, 0] != crt.MISS).mean()) > 0.3
    np.testing.assert_array_equal(_u(ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.SORT_RAYS)), _u(plain))
    bvh.optimize(1)
    np.testing.assert_array_equal(_u(ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)), _u(plain))
    bvh.free()
