"""GPU refit (crt_refit) against the oracle's refit, bit for bit.

A refit of unmoved triangles must give back the built node array; after a
move the node array must equal the oracle's refit of the built tree, traces
over it must equal the oracle's traces over that node array (both triangle
predicates, binary and 4-wide walks), and watertight hits must equal those of
a full rebuild on the moved triangles.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

from test_refit_oracle import moved

pytestmark = pytest.mark.gpu


def _u(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def soup():
    n = 40000
    tris = S.uniform_soup(n, seed=21, edge_lo=0.003, edge_hi=0.03)
    tris.view(np.uint32)[:, 12] = np.arange(n, dtype=np.uint32) % 3
    models = S.identity_models(3)
    models[2, 13] = 0.03125  # model 2 shifted up
    return tris, models


@pytest.mark.parametrize("n", [1, 2, 3, 1025, 40000])
def test_refit_unmoved_gives_the_built_tree(ctx, soup, n):
    tris, models = soup[0][:n].copy(), soup[1]
    bvh = ctx.build(tris, models=models)
    built = bvh.nodes()
    rays = S.sphere_rays(4096, seed=2)
    before = {f: ctx.trace(bvh, rays, f) for f in (crt.TRI_REFERENCE, crt.TRI_WATERTIGHT)}
    bvh.refit(tris, models=models)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(built))
    for f, h in before.items():
        np.testing.assert_array_equal(_u(ctx.trace(bvh, rays, f)), _u(h))
    bvh.free()


def test_refit_after_motion_matches_oracle(ctx, soup):
    tris, models = soup
    bvh = ctx.build(tris, models=models)
    built = bvh.nodes()
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = np.concatenate([O.raygen(cam, 128, 128), S.sphere_rays(8192, seed=3)])
    for step, phase in enumerate((0.4, 2.1, 5.0)):
        new = moved(tris, phase, amp=0.02)
        new_models = models.copy()
        new_models[1, 12] = 0.01 * (step + 1)  # model 1 slides along x
        bvh.refit(new, models=new_models)
        want = O.refit(built, new, new_models)
        np.testing.assert_array_equal(_u(bvh.nodes()), _u(want))
        for f in (crt.TRI_REFERENCE, crt.TRI_WATERTIGHT, crt.TRI_WATERTIGHT | crt.TRACE_WIDE):
            got = ctx.trace(bvh, rays, f)
            ref, _ = O.trace(want, new, new_models, rays, f & crt.TRI_WATERTIGHT)
            np.testing.assert_array_equal(_u(got), _u(ref), err_msg=f"step {step} flags {f}")
        # watertight hits do not depend on the tree: a rebuild finds the same
        fresh = ctx.build(new, models=new_models)
        np.testing.assert_array_equal(_u(ctx.trace(fresh, rays, crt.TRI_WATERTIGHT)),
                                      _u(ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)))
        fresh.free()
    # a shaded frame over the refit tree is the oracle's
    mats = S.materials([[0.5, 0.25, 1.0, 1.0], [1.0, 1.0, 0.0, 1.0], [0.0, 1.0, 0.5, 1.0]])
    mm = S.models_with_materials([0, 1, 2])
    mm[:, :16] = new_models[:, :16]
    img = ctx.render_frame(bvh, cam, 128, 128, models=mm, materials=mats, shade_flags=crt.SHADE_BVH, bvh_depth=5)
    prim = O.raygen(cam, 128, 128)
    h, _ = O.trace(want, new, mm, prim, 0)
    np.testing.assert_array_equal(_u(img), _u(O.shade(want, new, mm, mats, prim, h, crt.SHADE_BVH, 5)))
    bvh.free()


def test_refit_then_rebuild_then_refit(ctx, soup):
    """The refit topology is derived again after a rebuild changes the tree."""
    tris, models = soup
    bvh = ctx.build(tris, models=models)
    bvh.refit(moved(tris, 1.0), models=models)
    other = moved(tris, 3.0, amp=0.2)
    bvh.rebuild(other, models=models)
    built = bvh.nodes()
    third = moved(other, 0.5, amp=0.01)
    bvh.refit(third, models=models)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(O.refit(built, third, models)))
    bvh.free()


def test_refit_device_inputs_and_errors(ctx, soup):
    torch = pytest.importorskip("torch")
    tris, models = soup
    bvh = ctx.build(tris, models=models)
    built = bvh.nodes()
    new = moved(tris, 0.7)
    bvh.refit(torch.from_numpy(new).cuda(), models=torch.from_numpy(models).cuda())
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(O.refit(built, new, models)))
    with pytest.raises(crt.CrtError) as e:  # the triangle count must be the build's
        crt._check(crt.lib().crt_refit(ctx.handle, bvh.handle, crt._ptr(new), new.shape[0] - 1, None, 0))
    assert e.value.status == 1
    bad = new.copy()
    bad.view(np.uint32)[5, 12] = 64
    with pytest.raises(crt.CrtError) as e:
        bvh.refit(bad, models=models)
    assert e.value.status == 7
    bvh.refit(new, models=models)  # usable after the error
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(O.refit(built, new, models)))
    bvh.free()
