"""GPU treelet restructuring (crt_optimize) against the oracle, bit for bit.

The restructured node array must equal the oracle's for every pass count
(including after a refit, and on small and tie-heavy trees); traces over the
new tree must equal the oracle's traces over that node array (both triangle
predicates, closest and any hit, binary, 4-wide and compressed walks);
watertight closest hits must equal those over the built tree; and a refit or
shaded frame afterwards must work on the new tree.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

from test_gpu_trace import _cmp_hits
from test_refit_oracle import moved

pytestmark = pytest.mark.gpu


def _u(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def scene():
    n = 30000
    tris = S.clustered_soup(n, 24, 0.04, 0.004, 0.5, seed=31)
    tris.view(np.uint32)[:, 12] = np.arange(n, dtype=np.uint32) % 2
    models = S.identity_models(2)
    models[1, 14] = 0.0625  # model 1 shifted along z
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = np.concatenate([O.raygen(cam, 96, 96), S.sphere_rays(6000, seed=32)])
    return tris, models, cam, rays


@pytest.mark.parametrize("passes", [0, 1, 3])
def test_optimize_matches_oracle(ctx, scene, passes):
    tris, models, cam, rays = scene
    bvh = ctx.build(tris, models=models)
    built = bvh.nodes()
    want, _ = O.optimize(built, passes)
    bvh.optimize(passes)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(want))
    if passes == 0:
        np.testing.assert_array_equal(_u(want), _u(built))
    for f in (crt.TRI_REFERENCE, crt.TRI_WATERTIGHT, crt.TRI_WATERTIGHT | crt.TRACE_WIDE,
              crt.TRI_WATERTIGHT | crt.TRACE_COMPRESSED, crt.TRI_REFERENCE | crt.TRACE_COMPRESSED,
              crt.TRI_WATERTIGHT | crt.TRACE_ANY, crt.TRI_REFERENCE | crt.TRACE_ANY):
        got = ctx.trace(bvh, rays, f)
        ref, _ = O.trace(want, tris, models, rays, f & (crt.TRI_WATERTIGHT | crt.TRACE_ANY))
        _cmp_hits(got, ref, bool(f & crt.TRACE_ANY))
    # watertight closest hits do not depend on the tree
    fresh = ctx.build(tris, models=models)
    np.testing.assert_array_equal(_u(ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)),
                                  _u(ctx.trace(fresh, rays, crt.TRI_WATERTIGHT)))
    fresh.free()
    bvh.free()


@pytest.mark.parametrize("n", [2, 3, 6, 7, 8, 9, 15, 64, 1025])
def test_optimize_small_trees(ctx, n):
    tris = S.uniform_soup(n, seed=40 + n)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    built = bvh.nodes()
    for passes in (0, 2):
        bvh.optimize(passes)
        want, _ = O.optimize(built, passes)
        np.testing.assert_array_equal(_u(bvh.nodes()), _u(want), err_msg=f"n {n} passes {passes}")
        built = want
    rays = S.sphere_rays(2000, seed=n)
    ref, _ = O.trace(built, tris, models, rays, 0)
    np.testing.assert_array_equal(_u(ctx.trace(bvh, rays)), _u(ref))
    bvh.free()


def test_optimize_single_triangle(ctx):
    tris = S.uniform_soup(1, seed=1)
    bvh = ctx.build(tris)
    before = bvh.nodes()
    bvh.optimize(3)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(before))
    bvh.free()


def test_optimize_ties(ctx):
    """Identical and flat triangles: equal areas and costs everywhere."""
    base = S.uniform_soup(2500, seed=9)
    tris = np.concatenate([base, base, base, base])
    tris[::3, 1] = tris[::3, 5] = tris[::3, 9] = 0.25
    bvh = ctx.build(tris)
    built = bvh.nodes()
    bvh.optimize(2)
    want, _ = O.optimize(built, 2)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(want))
    bvh.free()


def test_refit_then_optimize_then_refit(ctx, scene):
    """An optimized refit tree equals the oracle's; a refit afterwards derives
    the new topology; a shaded frame over it is the oracle's."""
    tris, models, cam, rays = scene
    bvh = ctx.build(tris, models=models)
    built = bvh.nodes()
    new = moved(tris, 1.7, amp=0.1)
    bvh.refit(new, models=models)
    refit = O.refit(built, new, models)
    bvh.optimize(2)
    opt, _ = O.optimize(refit, 2)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(opt))
    third = moved(new, 0.3, amp=0.02)
    bvh.refit(third, models=models)
    want = O.refit(opt, third, models)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(want))
    for f in (crt.TRI_REFERENCE, crt.TRI_WATERTIGHT):
        ref, _ = O.trace(want, third, models, rays, f)
        np.testing.assert_array_equal(_u(ctx.trace(bvh, rays, f)), _u(ref))
    mats = S.materials([[0.5, 0.25, 1.0, 1.0], [1.0, 1.0, 0.0, 1.0]])
    mm = S.models_with_materials([0, 1])
    mm[:, :16] = models[:, :16]
    img = ctx.render_frame(bvh, cam, 96, 96, models=mm, materials=mats, shade_flags=crt.SHADE_BVH, bvh_depth=6)
    prim = O.raygen(cam, 96, 96)
    h, _ = O.trace(want, third, mm, prim, 0)
    np.testing.assert_array_equal(_u(img), _u(O.shade(want, third, mm, mats, prim, h, crt.SHADE_BVH, 6)))
    bvh.free()


def test_optimize_arguments(ctx, scene):
    tris, models, cam, rays = scene
    bvh = ctx.build(tris[:100].copy(), models=models)
    with pytest.raises(crt.CrtError) as e:
        bvh.optimize(crt.OPTIMIZE_MAX_PASSES + 1)
    assert e.value.status == 1
    with pytest.raises(crt.CrtError):
        crt._check(crt.lib().crt_optimize(ctx.handle, None, 1))
    bvh.optimize(1)  # usable after the errors
    bvh.free()
