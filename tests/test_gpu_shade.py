"""GPU parity of the shading pass against the CPU oracle, bit for bit.

Reference: srcCommon/shaders/raytracer.glsl — getColor :159-179, the
bvhColor of getClosestHitBVH :246-277 with intersectBVH's border test
:182-236, and main's initial value and imageStore :299-331.  crt_shade
shades given hits; crt_render_frame runs the whole compute pass (camera ray,
closest hit, texel) and must equal oracle raygen -> trace -> shade.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu

MATERIALS = S.materials([[0.25, 0.5, 0.75, 1.0], [1.0, 0.0, 0.0, 0.5], [0.0, 0.125, 1.0, 0.25],
                         [0.1, 0.2, 0.3, 0.4]])
FLAGS = [0, crt.SHADE_WIREFRAME, crt.SHADE_BVH, crt.SHADE_BVH | crt.SHADE_WIREFRAME]


def _eq(got, want, what=""):
    g, w = np.asarray(got).view(np.uint32), np.asarray(want).view(np.uint32)
    bad = np.nonzero(np.any(g != w, axis=1))[0]
    assert bad.size == 0, f"{what}: {bad.size} texels differ, first {bad[:4]}: {got[bad[:4]]} vs {want[bad[:4]]}"


@pytest.fixture(scope="module")
def scene(ctx):
    """20k-triangle soup over four models (model 3 >= n_models uses material
    0; model 2 names material 9 >= n_materials), model 1 translated."""
    n = 20000
    tris = S.uniform_soup(n, seed=11, edge_lo=0.005, edge_hi=0.04)
    tris.view(np.uint32)[:, 12] = np.arange(n, dtype=np.uint32) % 4
    models = S.models_with_materials([1, 3, 9])
    models[1, 12] = 0.0625  # translation x of model 1 (column-major m[12])
    bvh = ctx.build(tris, models=models)
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    return tris, models, cam, bvh


@pytest.mark.parametrize("flags", FLAGS)
@pytest.mark.parametrize("tri_flags", [crt.TRI_REFERENCE, crt.TRI_WATERTIGHT])
def test_render_frame_matches_oracle_pipeline(ctx, scene, flags, tri_flags):
    tris, models, cam, bvh = scene
    w, h = 256, 192
    nodes = bvh.nodes()
    rays = O.raygen(cam, w, h)
    hits, _ = O.trace(nodes, tris, models, rays, tri_flags)
    for depth in ((0, 4, 10) if flags & crt.SHADE_BVH else (0,)):
        want = O.shade(nodes, tris, models, MATERIALS, rays, hits, flags, depth)
        got = ctx.render_frame(bvh, cam, w, h, models=models, materials=MATERIALS, shade_flags=flags,
                               bvh_depth=depth, flags=tri_flags)
        _eq(got, want, f"flags {flags} depth {depth}")
    assert len({tuple(r) for r in want.tolist()}) >= 4  # misses, several materials


@pytest.mark.parametrize("flags", FLAGS)
def test_shade_incoherent_rays_and_deep_levels(ctx, scene, flags):
    tris, models, cam, bvh = scene
    nodes = bvh.nodes()
    rays = S.sphere_rays(30000, seed=4)
    hits = ctx.trace(bvh, rays)
    for depth in ((1, 7, 20, crt.SHADE_MAX_BVH_DEPTH) if flags & crt.SHADE_BVH else (0,)):
        want = O.shade(nodes, tris, models, MATERIALS, rays, hits, flags, depth)
        got = ctx.shade(bvh, rays, hits, models=models, materials=MATERIALS, shade_flags=flags, bvh_depth=depth)
        _eq(got, want, f"flags {flags} depth {depth}")


def test_render_paths_and_outputs_agree(ctx, scene):
    """One-launch frame, the separate raygen/trace/shade path (4-wide walk) and
    device, page-locked and pageable outputs give the same texels."""
    torch = pytest.importorskip("torch")
    tris, models, cam, bvh = scene
    w, h = 200, 150  # not a multiple of the 8x4 pixel tile
    flags = crt.SHADE_BVH | crt.SHADE_WIREFRAME
    ref = ctx.render_frame(bvh, cam, w, h, models=models, materials=MATERIALS, shade_flags=flags, bvh_depth=3)
    wide = ctx.render_frame(bvh, cam, w, h, models=models, materials=MATERIALS, shade_flags=flags, bvh_depth=3,
                            flags=crt.TRACE_WIDE)
    _eq(wide, ref, "4-wide path")
    dev = torch.empty((w * h, 4), dtype=torch.float32, device="cuda")
    ctx.render_frame(bvh, cam, w, h, models=torch.from_numpy(models).cuda(), materials=torch.from_numpy(MATERIALS).cuda(),
                     shade_flags=flags, bvh_depth=3, out=dev)
    _eq(dev.cpu().numpy(), ref, "device output")
    pin = torch.empty((w * h, 4), dtype=torch.float32, pin_memory=True)
    ctx.render_frame(bvh, cam, w, h, models=models, materials=MATERIALS, shade_flags=flags, bvh_depth=3, out=pin)
    _eq(pin.numpy(), ref, "page-locked output")
    rays = ctx.raygen(cam, w, h)
    hits = ctx.trace(bvh, rays)
    _eq(ctx.shade(bvh, rays, hits, models=models, materials=MATERIALS, shade_flags=flags, bvh_depth=3), ref,
        "crt_shade")
    # page-locked host rays and hits, read in place
    _eq(ctx.shade(bvh, torch.from_numpy(rays).pin_memory(), torch.from_numpy(hits).pin_memory(), models=models,
                  materials=MATERIALS, shade_flags=flags, bvh_depth=3), ref, "crt_shade, page-locked inputs")


def test_no_models_or_materials(ctx, scene):
    """Without buffers every hit reads material 0 -> colour (0,0,0,0): texels stay (0,0,0,1)."""
    tris, models, cam, bvh = scene
    got = ctx.render_frame(bvh, cam, 64, 64)
    assert np.all(got == np.array([0, 0, 0, 1], np.float32))


def test_shading_arguments_are_checked(ctx, scene):
    tris, models, cam, bvh = scene
    rays = S.sphere_rays(100, seed=1)
    hits = ctx.trace(bvh, rays)
    with pytest.raises(crt.CrtError) as e:
        ctx.shade(bvh, rays, hits, shade_flags=crt.SHADE_BVH, bvh_depth=crt.SHADE_MAX_BVH_DEPTH + 1)
    assert e.value.status == 1
    with pytest.raises(crt.CrtError):
        ctx.shade(bvh, None, hits, shade_flags=crt.SHADE_BVH)
    with pytest.raises(crt.CrtError):
        ctx.shade(bvh, rays, hits, shade_flags=0x4)
    with pytest.raises(crt.CrtError):
        ctx.render_frame(bvh, cam, 16, 16, models=S.models_with_materials(np.zeros(65, np.uint32)))
    ok = ctx.shade(bvh, None, hits, models=models, materials=MATERIALS)  # rays unused without SHADE_BVH
    _eq(ok, O.shade(bvh.nodes(), tris, models, MATERIALS, rays, hits, 0, 0), "no rays")
