"""The oracle's refit restatement on the CPU.

A refit keeps the tree and recomputes every box with the build's own rules
(AABB::buildFromTriangle for leaves, AABB::merge(left, right) for internal
nodes, srcCommon/scene/geometry/bvh.cpp:383-413), so:
1. a refit of unmoved triangles gives back the built node array bit for bit;
2. after a move, every box holds its triangles and is the merge of its
   children, and watertight traversal over the refit tree finds the brute
   force's closest hits.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import scenes as S


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build(ref=False)


def moved(tris, phase, amp=0.01):
    """Config-4 motion: every vertex moves by amp * sin(phase + 7 x) along y."""
    out = tris.copy()
    for c in (0, 4, 8):
        out[:, c + 1] = (tris[:, c + 1].astype(np.float64)
                         + amp * np.sin(phase + 7.0 * tris[:, c].astype(np.float64))).astype(np.float32)
    return out


@pytest.mark.parametrize("n", [1, 2, 3, 1000])
def test_refit_of_unmoved_triangles_is_the_build(n):
    tris = S.uniform_soup(n, seed=7)
    models = S.identity_models(2)
    tris.view(np.uint32)[:, 12] = np.arange(n, dtype=np.uint32) % 2
    models[1, 12:15] = (0.25, -0.5, 0.125)
    b = O.build_bvh(tris, n, models)
    np.testing.assert_array_equal(O.refit(b["nodes"], tris, models).view(np.uint32), b["nodes"].view(np.uint32))


def test_refit_after_motion_is_consistent_and_exact():
    n = 3000
    tris = S.uniform_soup(n, seed=8)
    models = S.identity_models(1)
    b = O.build_bvh(tris, n, models)
    new = moved(tris, 1.3, amp=0.05)
    r = O.refit(b["nodes"], new, models)
    u = r.view(np.uint32)
    np.testing.assert_array_equal(u[:, 8:12], b["nodes"].view(np.uint32)[:, 8:12])  # topology kept
    leaf = (u[:, 9] == 0) & (u[:, 10] == 0)
    t = new[u[leaf, 8]]
    lo = np.minimum(np.minimum(t[:, 0:3], t[:, 4:7]), t[:, 8:11])
    hi = np.maximum(np.maximum(t[:, 0:3], t[:, 4:7]), t[:, 8:11])
    np.testing.assert_array_equal(r[leaf, 0:3], lo)
    np.testing.assert_array_equal(r[leaf, 4:7], hi)
    inner = np.nonzero(~leaf)[0]
    L, R = u[inner, 9], u[inner, 10]
    np.testing.assert_array_equal(r[inner, 0:3], np.minimum(r[L, 0:3], r[R, 0:3]))
    np.testing.assert_array_equal(r[inner, 4:7], np.maximum(r[L, 4:7], r[R, 4:7]))
    assert not np.array_equal(r, b["nodes"])
    rays = O.raygen(S.camera_gpu_data((0.5, 0.5, -1.5)), 40, 40)
    h_fit, _ = O.trace(r, new, models, rays, 2)
    h_bf = O.trace_brute(new, models, rays, 2)
    assert (h_bf[:, 0].view(np.uint32) != 0xFFFFFFFF).sum() > 20
    np.testing.assert_array_equal(h_fit.view(np.uint32), h_bf.view(np.uint32))
