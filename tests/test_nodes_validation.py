"""The host-side structure check of a caller's DFS node array
(crt_validate_nodes, the check crt_bvh_from_nodes runs before any upload),
on the CPU: no context and no GPU are needed.

A well-formed array is the DFS pre-order of Scene::getBVH_NodesToGPUData
(srcOpenGL/scene/scene.cpp:189-208): left child right after its parent, the
right child after the left subtree, leaves with both children 0 (the shader's
leaf test, raytracer.glsl:239-244), each triangle in exactly one leaf.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build(ref=False)


def _height(nodes):
    u = nodes.view(np.uint32)
    depth = np.zeros(nodes.shape[0], np.int64)
    for d in range(nodes.shape[0]):
        if u[d, 9] or u[d, 10]:
            depth[u[d, 9]] = depth[u[d, 10]] = depth[d] + 1
    return int(depth.max())


@pytest.mark.parametrize("n", [1, 2, 3, 7, 100, 5000])
def test_well_formed_arrays_pass(n):
    tris = S.uniform_soup(n, seed=n)
    nodes = O.build_bvh(tris, n, S.identity_models(1))["nodes"]
    info = crt.validate_nodes(nodes)
    assert info == {"leaves": n, "internal": n - 1, "height": _height(nodes)}
    opt, h = O.optimize(nodes, 2)  # a restructured tree is a well-formed array too
    assert crt.validate_nodes(opt)["height"] == h


def _corrupt(nodes, what):
    bad = nodes.copy()
    u = bad.view(np.uint32)
    leaf = np.nonzero((u[:, 9] == 0) & (u[:, 10] == 0))[0]
    inner = np.nonzero(~((u[:, 9] == 0) & (u[:, 10] == 0)))[0]
    n = (bad.shape[0] + 1) // 2
    if what == "duplicate triangle":
        u[leaf[3], 8] = u[leaf[4], 8]
    elif what == "triangle id out of range":
        u[leaf[3], 8] = n
    elif what == "left child not next":
        u[inner[2], 9] += 1
    elif what == "right child out of range":
        u[inner[1], 10] = bad.shape[0]
    elif what == "right child not after left subtree":
        u[0, 10] -= 1  # the root's right child moved into its left subtree
    elif what == "right equals left":
        u[0, 10] = u[0, 9]
    elif what == "leaf made internal":
        u[leaf[5], 9] = leaf[5] + 1
        u[leaf[5], 10] = leaf[5] + 2
    return bad


@pytest.mark.parametrize("what", ["duplicate triangle", "triangle id out of range", "left child not next",
                                  "right child out of range", "right child not after left subtree",
                                  "right equals left", "leaf made internal"])
def test_malformed_arrays_are_named(what):
    n = 200
    nodes = O.build_bvh(S.uniform_soup(n, seed=9), n, S.identity_models(1))["nodes"]
    with pytest.raises(crt.CrtError) as e:
        crt.validate_nodes(_corrupt(nodes, what))
    assert e.value.status == 1


def test_wrong_counts_are_refused():
    n = 50
    nodes = O.build_bvh(S.uniform_soup(n, seed=2), n, S.identity_models(1))["nodes"]
    with pytest.raises(crt.CrtError):
        crt.validate_nodes(nodes[:-1])
    with pytest.raises(crt.CrtError):
        crt.validate_nodes(nodes, n_tris=n + 1)
    assert crt.validate_nodes(nodes)["leaves"] == n
