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


def test_config2_batch_full_scale_matches_single_scenes(ctx):
    """The batched workload at its full size: 64 scenes with log-uniform 1k-2M
    triangles (17.1 M in total; even scenes uniform soups, odd scenes 32-blob
    clustered soups) and their own log-uniform 64k-4M rays (55 M in total),
    built and traced as one graph-replayed launch per stage.  Every hit equals
    the single-scene crt_build + crt_trace of its scene, bit for bit (both
    predicates; the shader's rejects every triangle this small, so its hits
    are all misses), and so do the node arrays of every 8th scene and of the
    largest one; the sorted trace of the batch returns the same hits."""
    torch = pytest.importorskip("torch")
    tri_n, ray_n = S.config2_sizes(64, seed=0)
    assert int(tri_n.sum()) > 16_000_000 and int(ray_n.sum()) > 50_000_000
    gen = torch.Generator(device="cuda")
    gen.manual_seed(2)
    tris = torch.cat([S.device_soup(int(n), gen, clustered=(k % 2 == 1)) for k, n in enumerate(tri_n)])
    rays = torch.cat([S.device_sphere_rays(int(m), gen) for m in ray_n])
    models = S.identity_models(1)
    b = crt.Batch(ctx, tri_n, ray_n, models=models)
    tri_off = np.concatenate([[0], np.cumsum(tri_n)]).astype(np.int64)
    ray_off = np.concatenate([[0], np.cumsum(ray_n)]).astype(np.int64)
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    seq = torch.empty_like(hits)
    check_nodes = set(range(0, 64, 8)) | {int(np.argmax(tri_n))}
    for flags in (crt.TRI_WATERTIGHT, crt.TRI_REFERENCE):
        assert b.run(tris, rays, hits, flags, graph=True)
        b.run(tris, rays, hits, flags, graph=True)  # replayed
        for k in range(64):
            tk = tris[int(tri_off[k]):int(tri_off[k + 1])]
            bv = ctx.build(tk, models=models)
            ctx.trace(bv, rays[int(ray_off[k]):int(ray_off[k + 1])], flags, out=seq[int(ray_off[k]):int(ray_off[k + 1])])
            if flags == crt.TRI_WATERTIGHT and k in check_nodes:
                np.testing.assert_array_equal(_u(b.nodes(k)), _u(bv.nodes()), err_msg=f"scene {k}")
            bv.free()
        torch.cuda.synchronize()
        assert torch.equal(seq.view(torch.int32), hits.view(torch.int32)), flags
        if flags == crt.TRI_WATERTIGHT:  # the shader's predicate rejects these small triangles
            assert int((hits[:, 0].view(torch.int32) != -1).sum().item()) > 1_000_000
            srt = torch.empty_like(hits)
            b.trace(rays, srt, flags | crt.SORT_RAYS)
            assert torch.equal(srt.view(torch.int32), hits.view(torch.int32))
            del srt
    b.free()
