"""The oracle's treelet restructuring (crt_optimize) on the CPU.

Restructuring keeps the leaves, recomputes every box with AABB::merge
(srcCommon/scene/geometry/bvh.cpp:401-413) and lowers the surface-area cost,
so:
1. zero passes give back the built node array bit for bit (boxes recomputed
   with the build's own rule, tree laid out in the build's DFS order);
2. after passes the result is a valid DFS node array over the same
   triangles, each internal box the merge of its children, its SAH cost no
   higher than before, and watertight traversal finds the same hits.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build(ref=False)


def sah(nodes, ci=1.2):
    """Surface-area cost as crt_optimize counts it (leaf 1 x area, internal 1.2 x area)."""
    d = nodes[:, 4:7].astype(np.float64) - nodes[:, 0:3]
    a = 2 * (d[:, 0] * d[:, 1] + d[:, 1] * d[:, 2] + d[:, 2] * d[:, 0])
    u = nodes.view(np.uint32)
    leaf = (u[:, 9] == 0) & (u[:, 10] == 0)
    return float((np.where(leaf, 1.0, ci) * a).sum())


def check_tree(nodes, n):
    """DFS pre-order node array over triangles 0..n-1, boxes merged exactly."""
    u = nodes.view(np.uint32)
    leaf = (u[:, 9] == 0) & (u[:, 10] == 0)
    np.testing.assert_array_equal(np.sort(u[leaf, 8]), np.arange(n, dtype=np.uint32))
    inner = np.nonzero(~leaf)[0]
    L, R = u[inner, 9], u[inner, 10]
    np.testing.assert_array_equal(L, inner + 1)
    assert np.all(R > L) and np.all(R < nodes.shape[0])
    np.testing.assert_array_equal(u[inner, 8], 0)
    np.testing.assert_array_equal(nodes[inner, 0:3], np.minimum(nodes[L, 0:3], nodes[R, 0:3]))
    np.testing.assert_array_equal(nodes[inner, 4:7], np.maximum(nodes[L, 4:7], nodes[R, 4:7]))
    # the right child starts after the left subtree: 2 * leaves(left) - 1 nodes
    leaves_below = np.zeros(nodes.shape[0], np.int64)
    for d in range(nodes.shape[0] - 1, -1, -1):
        leaves_below[d] = 1 if leaf[d] else leaves_below[u[d, 9]] + leaves_below[u[d, 10]]
    np.testing.assert_array_equal(R, L + 2 * leaves_below[L] - 1)


@pytest.mark.parametrize("n", [1, 2, 3, 6, 7, 8, 100, 2000])
def test_zero_passes_reproduce_the_build(n):
    tris = S.uniform_soup(n, seed=3)
    models = S.identity_models(1)
    nodes = O.build_bvh(tris, n, models)["nodes"]
    out, _ = O.optimize(nodes, 0)
    np.testing.assert_array_equal(out.view(np.uint32), nodes.view(np.uint32))


@pytest.mark.parametrize("kind", ["uniform", "clustered", "duplicates"])
def test_passes_lower_the_cost_and_keep_the_hits(kind):
    n = 6000
    if kind == "uniform":
        tris = S.uniform_soup(n, seed=5)
    elif kind == "clustered":
        tris = S.clustered_soup(n, 12, 0.04, 0.004, 0.5, seed=6)
    else:  # many identical and axis-flat triangles: ties everywhere
        base = S.uniform_soup(n // 4, seed=7)
        tris = np.concatenate([base, base, base, base])
        tris[::5, 1] = tris[::5, 5] = tris[::5, 9] = 0.5
    models = S.identity_models(1)
    nodes = O.build_bvh(tris, n, models)["nodes"]
    costs = [sah(nodes)]
    prev = nodes
    for p in (1, 2, 3):
        out, h = O.optimize(nodes, p)
        check_tree(out, n)
        costs.append(sah(out))
        assert h >= int(np.ceil(np.log2(n)))
        prev = out
    assert costs[1] < costs[0] and costs[3] <= costs[1] * 1.0001, costs
    # a pass more over the restructured tree is a pass more from the start
    again, _ = O.optimize(O.optimize(nodes, 2)[0], 1)
    np.testing.assert_array_equal(again.view(np.uint32), prev.view(np.uint32))
    rays = np.concatenate([S.sphere_rays(3000, seed=8), O.raygen(S.camera_gpu_data((0.5, 0.5, -1.5)), 48, 48)])
    for flags in (crt.TRI_WATERTIGHT, crt.TRI_WATERTIGHT | crt.TRACE_ANY):
        a, _ = O.trace(nodes, tris, models, rays, flags)
        b, _ = O.trace(prev, tris, models, rays, flags)
        if flags & crt.TRACE_ANY:  # any hit: which occluder is found depends on the order
            np.testing.assert_array_equal(a.view(np.uint32)[:, 0] == crt.MISS, b.view(np.uint32)[:, 0] == crt.MISS)
        else:
            np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    # reference predicate: same hits up to equal-t ties, which follow the new DFS order
    a, _ = O.trace(nodes, tris, models, rays, crt.TRI_REFERENCE)
    b, _ = O.trace(prev, tris, models, rays, crt.TRI_REFERENCE)
    np.testing.assert_array_equal(a[:, 1], b[:, 1])


def _height(nodes):
    u = nodes.view(np.uint32)
    depth = np.zeros(nodes.shape[0], np.int64)
    for d in range(nodes.shape[0]):
        if u[d, 9] or u[d, 10]:
            depth[u[d, 9]] = depth[d] + 1
            depth[u[d, 10]] = depth[d] + 1
    return int(depth.max())


def test_reported_height_and_refit_trees():
    """The returned height is the tree's; a refit tree restructured keeps the
    moved triangles' watertight hits (those of the brute force)."""
    from test_refit_oracle import moved
    n = 4000
    tris = S.uniform_soup(n, seed=12)
    models = S.identity_models(1)
    nodes = O.build_bvh(tris, n, models)["nodes"]
    for p in (0, 1, 2):
        out, h = O.optimize(nodes, p)
        assert h == _height(out)
    new = moved(tris, 2.2, amp=0.2)
    refit = O.refit(nodes, new, models)
    out, _ = O.optimize(refit, 2)
    check_tree(out, n)
    assert sah(out) < sah(refit)
    rays = S.sphere_rays(3000, seed=13)
    got, _ = O.trace(out, new, models, rays, crt.TRI_WATERTIGHT)
    want = O.trace_brute(new, models, rays, crt.TRI_WATERTIGHT)
    np.testing.assert_array_equal(got.view(np.uint32)[:, 0], want.view(np.uint32)[:, 0])


@pytest.mark.parametrize("seed", range(12))
def test_random_small_scenes(seed):
    """Random sizes 1..300 and pass counts 0..3: always a valid tree over the
    same triangles, never a higher cost, zero passes the identity."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 301))
    kind = seed % 3
    if kind == 0:
        tris = S.uniform_soup(n, seed=100 + seed)
    elif kind == 1:
        tris = S.clustered_soup(n, 3, 0.05, 0.01, 0.5, seed=100 + seed)
    else:  # a few distinct triangles repeated: equal boxes and costs
        base = S.uniform_soup(max(1, n // 5), seed=100 + seed)
        tris = np.concatenate([base] * 6)[:n].copy()
    models = S.identity_models(1)
    nodes = O.build_bvh(tris, n, models)["nodes"]
    out0, _ = O.optimize(nodes, 0)
    np.testing.assert_array_equal(out0.view(np.uint32), nodes.view(np.uint32))
    passes = int(rng.integers(1, 4))
    out, h = O.optimize(nodes, passes)
    if n > 1:
        check_tree(out, n)
    assert h == _height(out)
    assert sah(out) <= sah(nodes) * (1 + 1e-6)
