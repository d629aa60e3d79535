"""crt_bvh_from_nodes: a caller's DFS node array made traceable, checked
against the oracle bit for bit.

The array is what Scene::getBVH_NodesToGPUData hands the shader
(srcOpenGL/scene/scene.cpp:189-208, binding 5 of raytracer.glsl).  Imported
from this library's own build, the tree must trace exactly like the built
handle; imported from the oracle (the reference's bvh.cpp restated, and a
restructured tree of different topology), traces must equal the oracle's
over that array in both predicates and every walk; refit, restructuring and
shading must work on it; malformed arrays must be rejected on the host.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

from test_gpu_trace import _cmp_hits
from test_refit_oracle import moved

pytestmark = pytest.mark.gpu

FLAGS = [crt.TRI_REFERENCE, crt.TRI_WATERTIGHT, crt.TRI_WATERTIGHT | crt.TRACE_WIDE,
         crt.TRI_WATERTIGHT | crt.TRACE_COMPRESSED, crt.TRI_WATERTIGHT | crt.TRACE_ANY]


def _u(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def scene():
    n = 25000
    tris = S.clustered_soup(n, 20, 0.04, 0.004, 0.5, seed=51)
    tris.view(np.uint32)[:, 12] = np.arange(n, dtype=np.uint32) % 2
    models = S.identity_models(2)
    models[1, 13] = 0.03125
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = np.concatenate([O.raygen(cam, 96, 96), S.sphere_rays(5000, seed=52)])
    return tris, models, cam, rays


def test_import_of_own_build_traces_like_it(ctx, scene):
    tris, models, cam, rays = scene
    built = ctx.build(tris, models=models)
    imp = ctx.bvh_from_nodes(built.nodes(), tris, models=models)
    np.testing.assert_array_equal(_u(imp.nodes()), _u(built.nodes()))
    for f in FLAGS:
        np.testing.assert_array_equal(_u(ctx.trace(imp, rays, f)), _u(ctx.trace(built, rays, f)), err_msg=f"{f:#x}")
    hp, hs = ctx.trace_frame(imp, cam, 96, 96, np.array([2.0, 2.0, -2.0], np.float32), crt.TRI_WATERTIGHT)
    bp, bs = ctx.trace_frame(built, cam, 96, 96, np.array([2.0, 2.0, -2.0], np.float32), crt.TRI_WATERTIGHT)
    np.testing.assert_array_equal(_u(hp), _u(bp))
    np.testing.assert_array_equal(_u(hs), _u(bs))
    with pytest.raises(crt.CrtError):
        imp.codes()
    imp.free()
    built.free()


@pytest.mark.parametrize("kind", ["oracle_build", "restructured"])
def test_import_of_oracle_trees(ctx, scene, kind):
    tris, models, cam, rays = scene
    nodes = O.build_bvh(tris, tris.shape[0], models)["nodes"]
    if kind == "restructured":
        nodes, _ = O.optimize(nodes, 2)
    imp = ctx.bvh_from_nodes(nodes, tris, models=models)
    for f in FLAGS:
        ref, _ = O.trace(nodes, tris, models, rays, f & (crt.TRI_WATERTIGHT | crt.TRACE_ANY))
        _cmp_hits(ctx.trace(imp, rays, f), ref, bool(f & crt.TRACE_ANY))
    mats = S.materials([[0.5, 0.25, 1.0, 1.0], [1.0, 1.0, 0.0, 1.0]])
    mm = S.models_with_materials([0, 1])
    mm[:, :16] = models[:, :16]
    img = ctx.render_frame(imp, cam, 96, 96, models=mm, materials=mats, shade_flags=crt.SHADE_BVH, bvh_depth=5)
    prim = O.raygen(cam, 96, 96)
    h, _ = O.trace(nodes, tris, mm, prim, 0)
    np.testing.assert_array_equal(_u(img), _u(O.shade(nodes, tris, mm, mats, prim, h, crt.SHADE_BVH, 5)))
    # refit and restructuring work on the imported tree
    new = moved(tris, 0.8, amp=0.03)
    imp.refit(new, models=models)
    want = O.refit(nodes, new, models)
    np.testing.assert_array_equal(_u(imp.nodes()), _u(want))
    imp.optimize(1)
    np.testing.assert_array_equal(_u(imp.nodes()), _u(O.optimize(want, 1)[0]))
    imp.free()


def test_import_from_device_memory_and_small_trees(ctx, scene):
    torch = pytest.importorskip("torch")
    tris, models, cam, rays = scene
    nodes = O.build_bvh(tris, tris.shape[0], models)["nodes"]
    imp = ctx.bvh_from_nodes(torch.from_numpy(nodes).cuda(), torch.from_numpy(tris).cuda(),
                             models=torch.from_numpy(models).cuda())
    ref, _ = O.trace(nodes, tris, models, rays, crt.TRI_WATERTIGHT)
    _cmp_hits(ctx.trace(imp, rays, crt.TRI_WATERTIGHT), ref)
    imp.free()
    for n in (1, 2, 3, 7):
        t = S.uniform_soup(n, seed=n)
        m = S.identity_models(1)
        nd = O.build_bvh(t, n, m)["nodes"]
        b = ctx.bvh_from_nodes(nd, t, models=m)
        r = S.sphere_rays(500, seed=n)
        _cmp_hits(ctx.trace(b, r, crt.TRI_REFERENCE), O.trace(nd, t, m, r, 0)[0])
        b.free()


def test_malformed_arrays_are_rejected(ctx, scene):
    tris, models, cam, rays = scene
    t = tris[:100].copy()
    nodes = O.build_bvh(t, 100, models)["nodes"]
    u = nodes.view(np.uint32)
    leaf = np.nonzero((u[:, 9] == 0) & (u[:, 10] == 0))[0]
    inner = np.nonzero(~((u[:, 9] == 0) & (u[:, 10] == 0)))[0]
    cases = []
    bad = nodes.copy(); bad.view(np.uint32)[leaf[3], 8] = bad.view(np.uint32)[leaf[4], 8]; cases.append(bad)  # duplicate
    bad = nodes.copy(); bad.view(np.uint32)[leaf[3], 8] = 100; cases.append(bad)                            # id range
    bad = nodes.copy(); bad.view(np.uint32)[inner[2], 9] += 1; cases.append(bad)                            # not pre-order
    bad = nodes.copy(); bad.view(np.uint32)[inner[1], 10] = 2 * 100 - 1; cases.append(bad)                  # out of range
    bad = nodes.copy(); bad.view(np.uint32)[0, 10] = bad.view(np.uint32)[0, 9]; cases.append(bad)          # right == left
    for k, bad in enumerate(cases):
        with pytest.raises(crt.CrtError) as e:
            ctx.bvh_from_nodes(bad, t, models=models)
        assert e.value.status == 1, k
    with pytest.raises(crt.CrtError):
        ctx.bvh_from_nodes(nodes[:-1], t, models=models)  # 2n-2 records
    ok = ctx.bvh_from_nodes(nodes, t, models=models)  # the context stays usable
    ok.free()


def test_misaligned_device_buffers_are_rejected(ctx, scene):
    """Kernels read and write records as 16-byte vectors: a device pointer
    off that boundary is refused on the host, before any launch."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    tris, models, cam, rays = scene
    bvh = ctx.build(tris, models=models)
    r = torch.from_numpy(rays).cuda()
    h = torch.empty((rays.shape[0] + 1, 4), dtype=torch.float32, device="cuda")
    lib = crt.lib()
    st = lib.crt_trace(ctx.handle, bvh.handle, C.c_void_p(r.data_ptr() + 4), 100, 0, C.c_void_p(h.data_ptr()))
    assert st == 1
    st = lib.crt_trace(ctx.handle, bvh.handle, C.c_void_p(r.data_ptr()), 100, 0, C.c_void_p(h.data_ptr() + 8))
    assert st == 1
    t = torch.from_numpy(tris).cuda()
    out = C.c_void_p()
    st = lib.crt_build(ctx.handle, C.c_void_p(t.data_ptr() + 4), 100, 100, None, 0, C.byref(out))
    assert st == 1
    # aligned pointers into the same buffers still work
    got = ctx.trace(bvh, r, crt.TRI_WATERTIGHT, out=h[1:])
    np.testing.assert_array_equal(_u(got.cpu().numpy()), _u(ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)))
    bvh.free()
