"""Checks of the reference-interface mirror (realtimeraytracing_gb300.bvh)
that need no GPU: its limits are the reference's, and a BVH of no triangles
raises ValueError before any device work."""
import numpy as np
import pytest

from realtimeraytracing_gb300 import bvh as B


def test_limits_are_the_references():
    assert B.MAX_NB_TRIANGLES == 65536  # Triangle::MAX_NB_TRIANGLES = 2<<15 (triangle.hpp:21)
    assert B.MAX_NB_MESHES == 64        # Mesh::MAX_NB_MESHES = 2<<5 (mesh.hpp:26)


@pytest.mark.parametrize("n", [0, -1])
def test_bvh_refuses_no_triangles(n):
    with pytest.raises(ValueError):
        B.BVH(n, np.zeros((1, 16), np.float32))
