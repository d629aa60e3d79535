"""GPU parity of ray generation and traversal against the CPU oracle.

Reference: srcCommon/shaders/raytracer.glsl — getRay :92-100, the triangle
test :102-147, the slab test :182-221 and getClosestHitBVH :246-295.
Closest-hit triangle ids must match exactly; t, u, v are compared bit for
bit (the CUDA path evaluates the same IEEE operations in the same order, so
the stated 1e-6 relative bound on t is met with zero error).
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu

T_RTOL = 1e-6


def _cmp_hits(got, ref, any_hit=False):
    gt, rt = got[:, 0].view(np.uint32), ref[:, 0].view(np.uint32)
    if any_hit:
        np.testing.assert_array_equal(gt == crt.MISS, rt == crt.MISS)
        return
    bad = np.nonzero(gt != rt)[0]
    assert bad.size == 0, f"{bad.size} rays differ in triangle id, first {bad[:5]}: {gt[bad[:5]]} vs {rt[bad[:5]]}"
    hit = gt != crt.MISS
    np.testing.assert_allclose(got[hit, 1], ref[hit, 1], rtol=T_RTOL, atol=0)
    np.testing.assert_array_equal(got[hit, 1:].view(np.uint32), ref[hit, 1:].view(np.uint32))


@pytest.fixture(scope="module")
def config0(ctx):
    tris, models, cam, (w, h) = S.config0_scene(seed=0)
    bvh = ctx.build(tris, models=models)
    return tris, models, cam, w, h, bvh


def test_raygen_bit_exact(ctx, config0):
    tris, models, cam, w, h, bvh = config0
    rays = ctx.raygen(cam, w, h)
    np.testing.assert_array_equal(rays.view(np.uint32), O.raygen(cam, w, h).view(np.uint32))


def test_closest_hit_reference_predicate_config0(ctx, config0):
    tris, models, cam, w, h, bvh = config0
    rays = O.raygen(cam, w, h)
    got = ctx.trace(bvh, rays, crt.TRI_REFERENCE)
    ref, _ = O.trace(bvh.nodes(), tris, models, rays, crt.TRI_REFERENCE)
    _cmp_hits(got, ref)
    assert (got[:, 0].view(np.uint32) != crt.MISS).sum() > 10000


def test_config0_hits_and_frame_equal_the_shaders(ctx, config0):
    """Against the reference's own compute shader: tests/golden/index.json
    holds the digests of what raytracer.glsl (compiled as C++, see
    tests/test_shader_pin.py) computes on this scene — getClosestHitBVH for
    all 262,144 primary rays, and main's texels for a 128x128 frame with the
    wireframe and the depth-2 BVH boxes shown."""
    import hashlib
    import json
    import os
    tris, models, cam, w, h, bvh = config0
    with open(os.path.join(os.path.dirname(__file__), "golden", "index.json")) as f:
        index = json.load(f)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    hits, _ = ctx.trace_frame(bvh, cam, w, h, None, crt.TRI_REFERENCE)
    assert sha(hits) == index["config0_trace"]["hits_reference_sha256"]
    fr = index["config0_frame"]
    img = ctx.render_frame(bvh, cam, fr["width"], fr["height"], models=S.models_with_materials(fr["material_ids"]),
                           materials=S.materials(fr["materials"]), shade_flags=fr["flags"], bvh_depth=fr["depth"])
    assert sha(img) == fr["texels_sha256"]


def test_closest_hit_watertight_config0(ctx, config0):
    tris, models, cam, w, h, bvh = config0
    rays = O.raygen(cam, w, h)
    got = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    ref, _ = O.trace(bvh.nodes(), tris, models, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(got, ref)


def test_watertight_against_brute_force(ctx):
    tris = S.uniform_soup(3000, seed=12)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = O.raygen(cam, 96, 96)
    got = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(got, O.trace_brute(tris, models, rays, crt.TRI_WATERTIGHT))


def test_any_hit_and_shadow_rays(ctx, config0):
    tris, models, cam, w, h, bvh = config0
    rays = O.raygen(cam, w, h)
    prim = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    light = np.array([2.0, 2.0, -2.0], np.float32)
    sh = ctx.shadow_rays(rays, prim, light)
    np.testing.assert_array_equal(sh.view(np.uint32), O.shadow_rays(rays, prim, light).view(np.uint32))
    for pred in (crt.TRI_WATERTIGHT, crt.TRI_REFERENCE):
        got = ctx.trace(bvh, sh, crt.TRACE_ANY | pred)
        ref, _ = O.trace(bvh.nodes(), tris, models, sh, crt.TRACE_ANY | pred)
        _cmp_hits(got, ref, any_hit=True)


def test_icosphere_primary_and_shadow(ctx):
    v, f = S.displaced_icosphere(level=6, seed=4)
    tris = S.indexed_to_triangles(v, f)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    cam = S.camera_gpu_data((0.0, 0.0, -3.0), aspect=16 / 9)
    rays = ctx.raygen(cam, 320, 180)
    got = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    nodes = bvh.nodes()
    ref, _ = O.trace(nodes, tris, models, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(got, ref)
    assert (got[:, 0].view(np.uint32) != crt.MISS).mean() > 0.2
    sh = ctx.shadow_rays(rays, got, np.array([2.0, 2.0, -2.0], np.float32))
    gs = ctx.trace(bvh, sh, crt.TRACE_ANY | crt.TRI_WATERTIGHT)
    rs, _ = O.trace(nodes, tris, models, sh, crt.TRACE_ANY | crt.TRI_WATERTIGHT)
    _cmp_hits(gs, rs, any_hit=True)


def test_device_resident_rays(ctx, config0):
    torch = pytest.importorskip("torch")
    tris, models, cam, w, h, bvh = config0
    rays = torch.empty((w * h, 8), dtype=torch.float32, device="cuda")
    ctx.raygen(cam, w, h, out=rays)
    hits = torch.empty((w * h, 4), dtype=torch.float32, device="cuda")
    ctx.trace(bvh, rays, crt.TRI_REFERENCE, out=hits)
    ref, _ = O.trace(bvh.nodes(), tris, models, rays.cpu().numpy(), crt.TRI_REFERENCE)
    _cmp_hits(hits.cpu().numpy(), ref)


def test_trace_frame_matches_separate_calls(ctx):
    """crt_trace_frame = raygen + closest hit + shadow rays + any hit."""
    v, f = S.displaced_icosphere(level=5, seed=8)
    tris = S.indexed_to_triangles(v, f)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    cam = S.camera_gpu_data((0.0, 0.0, -3.0), aspect=16 / 9)
    light = np.array([2.0, 2.0, -2.0], np.float32)
    hp, hs = ctx.trace_frame(bvh, cam, 160, 90, light, crt.TRI_WATERTIGHT)
    rays = O.raygen(cam, 160, 90)
    ref_p, _ = O.trace(bvh.nodes(), tris, models, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(hp, ref_p)
    sh = O.shadow_rays(rays, ref_p, light)
    ref_s, _ = O.trace(bvh.nodes(), tris, models, sh, crt.TRACE_ANY | crt.TRI_WATERTIGHT)
    _cmp_hits(hs, ref_s, any_hit=True)
    hp2, hs2 = ctx.trace_frame(bvh, cam, 160, 90, None, crt.TRI_REFERENCE)
    assert hs2 is None
    _cmp_hits(hp2, O.trace(bvh.nodes(), tris, models, rays, crt.TRI_REFERENCE)[0])


def test_trace_stats_counts(ctx, config0):
    tris, models, cam, w, h, bvh = config0
    rays = O.raygen(cam, 64, 64)
    got = ctx.trace(bvh, rays, crt.TRI_REFERENCE | crt.TRACE_STATS)
    visited, tested = ctx.last_trace_stats()
    assert visited > rays.shape[0] and tested > 0
    _cmp_hits(got, O.trace(bvh.nodes(), tris, models, rays, crt.TRI_REFERENCE)[0])


@pytest.mark.parametrize("flags", [crt.TRI_REFERENCE, crt.TRI_WATERTIGHT, crt.TRI_WATERTIGHT | crt.TRACE_ANY])
def test_binary_and_wide_walks_agree(ctx, config0, flags):
    """The binary walk (default) and the 4-wide walk (CRT_TRACE_WIDE) return
    the oracle's hits."""
    tris, models, cam, w, h, bvh = config0
    rays = O.raygen(cam, w, h)
    ref, _ = O.trace(bvh.nodes(), tris, models, rays, flags)
    any_hit = bool(flags & crt.TRACE_ANY)
    _cmp_hits(ctx.trace(bvh, rays, flags), ref, any_hit)
    _cmp_hits(ctx.trace(bvh, rays, flags | crt.TRACE_WIDE), ref, any_hit)


def test_trace_frame_tiles_bands_and_host_outputs(ctx):
    """crt_trace_frame on an image of 8x4 pixel tiles: one launch per row band
    (camera ray, closest hit, shadow ray, any hit), hits copied to host memory
    band by band, the same hits as the oracle and as device-memory outputs."""
    torch = pytest.importorskip("torch")
    v, f = S.displaced_icosphere(level=5, seed=21)
    tris = S.indexed_to_triangles(v, f)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    cam = S.camera_gpu_data((0.3, -0.2, -2.5), aspect=256 / 120)
    light = np.array([2.0, 2.0, -2.0], np.float32)
    w, h = 256, 120
    hp, hs = ctx.trace_frame(bvh, cam, w, h, light, crt.TRI_WATERTIGHT | crt.TRACE_STATS)
    visited, _ = ctx.last_trace_stats()
    assert visited > w * h
    rays = O.raygen(cam, w, h)
    ref_p, _ = O.trace(bvh.nodes(), tris, models, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(hp, ref_p)
    ref_s, _ = O.trace(bvh.nodes(), tris, models, O.shadow_rays(rays, ref_p, light), crt.TRACE_ANY | crt.TRI_WATERTIGHT)
    _cmp_hits(hs, ref_s, any_hit=True)
    assert (hp[:, 0].view(np.uint32) != crt.MISS).mean() > 0.2
    dp = torch.empty((w * h, 4), dtype=torch.float32, device="cuda")
    ds = torch.empty((w * h, 4), dtype=torch.float32, device="cuda")
    ctx.trace_frame(bvh, cam, w, h, light, crt.TRI_WATERTIGHT, hits_primary=dp, hits_shadow=ds)
    np.testing.assert_array_equal(dp.cpu().numpy().view(np.uint32), hp.view(np.uint32))
    np.testing.assert_array_equal(ds.cpu().numpy().view(np.uint32), hs.view(np.uint32))
    # page-locked host outputs: written by the frame kernel itself
    pp = torch.empty((w * h, 4), dtype=torch.float32, pin_memory=True)
    ps = torch.empty((w * h, 4), dtype=torch.float32, pin_memory=True)
    ctx.trace_frame(bvh, cam, w, h, light, crt.TRI_WATERTIGHT, hits_primary=pp, hits_shadow=ps)
    np.testing.assert_array_equal(pp.numpy().view(np.uint32), hp.view(np.uint32))
    np.testing.assert_array_equal(ps.numpy().view(np.uint32), hs.view(np.uint32))
    hr, _ = ctx.trace_frame(bvh, cam, w, h, None, crt.TRI_REFERENCE)
    _cmp_hits(hr, O.trace(bvh.nodes(), tris, models, rays, crt.TRI_REFERENCE)[0])


@pytest.mark.parametrize("flags", [crt.TRI_REFERENCE, crt.TRI_WATERTIGHT, crt.TRI_WATERTIGHT | crt.TRACE_ANY])
def test_sorted_rays_same_hits(ctx, flags):
    """CRT_TRACE_SORT_RAYS: incoherent rays traced in coherence order (origin
    cell, direction bin) get the oracle's hits, for any ray count."""
    v, f = S.displaced_icosphere(level=5, seed=31)
    tris = S.indexed_to_triangles(v, f)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    rays = S.sphere_rays(12345, seed=3, radius=1.5, center=(0.0, 0.0, 0.0))
    ref, _ = O.trace(bvh.nodes(), tris, models, rays, flags)
    any_hit = bool(flags & crt.TRACE_ANY)
    _cmp_hits(ctx.trace(bvh, rays, flags | crt.SORT_RAYS), ref, any_hit)
    _cmp_hits(ctx.trace(bvh, rays[:1], flags | crt.SORT_RAYS), ref[:1], any_hit)


def test_trace_into_page_locked_host_memory(ctx, config0):
    """crt_trace with page-locked host hits (written by the kernel directly)
    and pageable host hits give the oracle's hits."""
    torch = pytest.importorskip("torch")
    tris, models, cam, w, h, bvh = config0
    rays = O.raygen(cam, w, h)
    ref, _ = O.trace(bvh.nodes(), tris, models, rays, crt.TRI_WATERTIGHT)
    pinned = torch.empty((rays.shape[0], 4), dtype=torch.float32, pin_memory=True)
    ctx.trace(bvh, rays, crt.TRI_WATERTIGHT, out=pinned)
    _cmp_hits(pinned.numpy(), ref)
    _cmp_hits(ctx.trace(bvh, rays, crt.TRI_WATERTIGHT), ref)


@pytest.mark.parametrize("flags", [crt.TRI_REFERENCE, crt.TRI_WATERTIGHT | crt.TRACE_ANY,
                                   crt.TRI_WATERTIGHT | crt.SORT_RAYS])
def test_trace_from_page_locked_host_rays(ctx, config0, flags):
    """Page-locked host rays are read in place by the trace kernel (in-order
    traces) or copied in first (reordered traces): the oracle's hits either way."""
    torch = pytest.importorskip("torch")
    tris, models, cam, w, h, bvh = config0
    rays = O.raygen(cam, w, h)
    ref, _ = O.trace(bvh.nodes(), tris, models, rays, flags & (crt.TRI_WATERTIGHT | crt.TRACE_ANY))
    pinned_rays = torch.from_numpy(rays).pin_memory()
    pinned_hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, pin_memory=True)
    ctx.trace(bvh, pinned_rays, flags, out=pinned_hits)
    _cmp_hits(pinned_hits.numpy(), ref, any_hit=bool(flags & crt.TRACE_ANY))


@pytest.mark.parametrize("flags", [crt.TRI_WATERTIGHT, crt.TRI_REFERENCE])
def test_persistent_warps_equal_one_thread_per_ray(ctx, flags):
    """Large closest-hit batches run on persistent warps that refill finished
    lanes and postpone leaf tests until many lanes hold one;
    CRT_TRACE_PER_RAY_THREADS keeps one thread per ray testing leaves at once.
    Same hits bit for bit, on incoherent rays: rays between sphere points and
    cube points, and bounce rays from their hits, in caller order and in
    sorted order.  A postponed leaf tightens the pruning bound later, so the
    persistent walk may fetch a few more nodes and test a few more triangles."""
    tris = S.clustered_soup(200_000, 64, 0.03, 0.004, 0.5, seed=95)
    if flags == crt.TRI_REFERENCE:   # large triangles, so that the shader's predicate finds hits
        tris[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]] = (tris[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]] - 0.5) * 8.0 + 0.5
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    rays = S.sphere_rays(150_000, seed=96)
    prim = ctx.trace(bvh, rays, flags)
    bounce = S.bounce_rays(rays, prim, tris, 120_000, seed=3)
    for rs in (rays, bounce):
        for order in (0, crt.SORT_RAYS):
            a = ctx.trace(bvh, rs, flags | order | crt.TRACE_STATS)
            sa = ctx.last_trace_stats()
            b = ctx.trace(bvh, rs, flags | order | crt.PER_RAY_THREADS | crt.TRACE_STATS)
            sb = ctx.last_trace_stats()
            np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
            assert 0.9 * sb[0] <= sa[0] <= 1.25 * sb[0] and 0.9 * sb[1] <= sa[1] <= 1.5 * sb[1], (sa, sb)
            assert (a[:, 0].view(np.uint32) != crt.MISS).sum() > 1000
    bvh.free()
