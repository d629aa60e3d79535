"""GPU assembly of TriangleGPU records from indexed meshes
(crt_triangles_from_indexed) against the oracle, bit for bit, and a scene of
two parsed OBJ meshes with their own model ids built and traced through the
pipeline (Scene::getTriangleToGPUData concatenation, srcOpenGL/scene/
scene.cpp:26-40)."""
import numpy as np
import pytest

from oracle import obj_oracle as OO
from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _u(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_indexed_to_triangles_bit_exact(ctx):
    v, f = S.displaced_icosphere(level=6, seed=2)
    v, f = np.asarray(v, np.float32), np.asarray(f, np.uint32)
    got = ctx.triangles_from_indexed(v, f, model_id=5)
    np.testing.assert_array_equal(_u(got), _u(OO.triangles_from_indexed(v, f, 5)))
    same = S.indexed_to_triangles(v, f)  # the bench scenes' host packing agrees (model 0)
    same.view(np.uint32)[:, 12] = 5
    np.testing.assert_array_equal(_u(got), _u(same))


def test_device_arrays_and_bad_indices(ctx):
    torch = pytest.importorskip("torch")
    v, f = S.icosphere(4)
    v, f = np.asarray(v, np.float32), np.asarray(f, np.uint32)
    out = torch.empty((f.shape[0], 16), dtype=torch.float32, device="cuda")
    ctx.triangles_from_indexed(torch.from_numpy(v).cuda(), torch.from_numpy(f.astype(np.int32)).cuda(), 3, out=out)
    np.testing.assert_array_equal(_u(out.cpu().numpy()), _u(OO.triangles_from_indexed(v, f, 3)))
    bad = f.copy()
    bad[7, 1] = v.shape[0]
    with pytest.raises(crt.CrtError) as e:
        ctx.triangles_from_indexed(v, bad)
    assert e.value.status == 7
    ctx.triangles_from_indexed(v, f)  # the context stays usable


def test_two_obj_meshes_build_and_trace(ctx):
    """Two meshes from OBJ text (the second a different corner syntax and
    model 1, translated by its model matrix) concatenated into one buffer."""
    v0, f0 = S.displaced_icosphere(level=5, seed=3)
    v1, f1 = S.icosphere(4)
    m0 = crt.parse_obj(OO.to_obj_text(v0, f0, style=0))
    m1 = crt.parse_obj(OO.to_obj_text(np.asarray(v1, np.float32) * np.float32(0.5), f1, style=3))
    t0 = ctx.triangles_from_indexed(*m0, model_id=0)
    t1 = ctx.triangles_from_indexed(*m1, model_id=1)
    tris = np.concatenate([t0, t1])
    models = S.identity_models(2)
    models[1, 12:15] = (1.25, 0.0, 0.5)
    bvh = ctx.build(tris, models=models)
    ref = O.build_bvh(tris, tris.shape[0], models)
    np.testing.assert_array_equal(_u(bvh.nodes()), _u(ref["nodes"]))
    cam = S.camera_gpu_data((0.5, 0.0, -4.0))
    rays = O.raygen(cam, 160, 120)
    for flags in (crt.TRI_REFERENCE, crt.TRI_WATERTIGHT):
        h = ctx.trace(bvh, rays, flags)
        rh, _ = O.trace(ref["nodes"], tris, models, rays, flags)
        np.testing.assert_array_equal(_u(h), _u(rh))
    hit_ids = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)[:, 0].view(np.uint32)
    assert ((hit_ids != crt.MISS) & (hit_ids >= t0.shape[0])).sum() > 100  # the second mesh is seen
    bvh.free()
