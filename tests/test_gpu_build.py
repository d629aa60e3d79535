"""GPU parity of the BVH build: Morton codes, (code, index) sort and the DFS
node array of the CUDA path against the CPU oracle, bit for bit.

Reference: srcCommon/scene/geometry/bvh.cpp (BVH::BVH and PLOC) and
srcOpenGL/scene/scene.cpp:189-208 (DFS flattening).  The oracle itself is
pinned to the reference's own bvh.cpp by tests/test_oracle.py.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _check_build(ctx, tris, n, models, radius=16):
    ref = O.build_bvh(tris, n, models, radius=radius)
    bvh = ctx.build(tris, n_tris=n, models=models)
    codes, perm, nodes = bvh.codes(), bvh.perm(), bvh.nodes()
    np.testing.assert_array_equal(codes, ref["codes"], err_msg="sorted Morton codes")
    np.testing.assert_array_equal(perm, ref["perm"], err_msg="permutation")
    bad = np.nonzero((nodes.view(np.uint32) != ref["nodes"].view(np.uint32)).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} node records differ, first at {bad[:5]}"
    st = ctx.last_build_stats()
    assert st["ploc_iterations"] == ref["iterations"]
    return st


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 100, 1000, 1023, 1024, 1025, 4097, 65536])
def test_uniform_soup_bit_exact(ctx, n):
    tris = S.uniform_soup(n, seed=1000 + n)
    _check_build(ctx, tris, n, S.identity_models(1))


def test_padded_buffer_scene_box(ctx):
    """Scene::getTriangleToGPUData pads to 65,536 zero records and the
    reference scans all of them for the scene box (bvh.cpp:237)."""
    n = 1000
    tris = np.concatenate([S.uniform_soup(n, seed=7) + np.float32(0.5), np.zeros((65536 - n, 16), np.float32)])
    tris.view(np.uint32)[:, 12] = 0
    _check_build(ctx, tris, n, S.identity_models(1))


def test_large_soup(ctx):
    n = 300_000
    _check_build(ctx, S.uniform_soup(n, seed=3), n, S.identity_models(1))


def test_clustered_soup(ctx):
    n = 200_000
    _check_build(ctx, S.clustered_soup(n, 32, 0.03, 0.005, 0.5, seed=5), n, S.identity_models(1))


def test_icosphere(ctx):
    v, f = S.displaced_icosphere(level=6, seed=2)
    tris = S.indexed_to_triangles(v, f)
    _check_build(ctx, tris, tris.shape[0], S.identity_models(1))


def test_duplicate_triangles_degenerate(ctx):
    """All-identical boxes: every iteration merges only the first pair, as
    in the reference (N-1 iterations)."""
    n = 300
    tris = np.repeat(S.uniform_soup(1, seed=9), n, axis=0)
    st = _check_build(ctx, tris, n, S.identity_models(1))
    assert st["ploc_iterations"] == n - 1


def test_model_matrices(ctx):
    """Several meshes with non-identity model matrices (mat4 * vec4 in glm order)."""
    n = 5000
    tris = S.uniform_soup(n, seed=11)
    tris.view(np.uint32)[:, 12] = np.arange(n) % 3
    models = S.identity_models(3)
    models[1, 12:15] = [0.25, -1.0, 3.0]                     # translation
    models[2, 0:16] = np.array([0.0, 1.0, 0.0, 0.0, -2.0, 0.0, 0.0, 0.0,
                                0.0, 0.0, 0.5, 0.0, 1.0, 1.0, 1.0, 1.0], np.float32)  # rotate+scale+translate
    _check_build(ctx, tris, n, models)


@pytest.mark.parametrize("radius", [8, 32, 1, 5, 12, 31])
def test_other_radius(ctx, radius):
    """Radii with a compiled search (8, 16, 32) and the generic one (any
    other radius in [1, 32]), through the tile iterations and the
    shared-memory tail: the oracle's tree bit for bit."""
    from realtimeraytracing_gb300 import crt
    c = crt.Context(ploc_radius=radius)
    n = 20000
    tris = S.uniform_soup(n, seed=21)
    _check_build(c, tris, n, S.identity_models(1), radius=radius)
    c.close()


def test_digit_bits_4(ctx):
    from realtimeraytracing_gb300 import crt
    c = crt.Context(sort_digit_bits=4)
    n = 50000
    _check_build(c, S.uniform_soup(n, seed=22), n, S.identity_models(1))
    c.close()


def test_rebuild_reuses_handle(ctx):
    tris = S.uniform_soup(3000, seed=31)
    bvh = ctx.build(tris, models=S.identity_models(1))
    tris2 = S.uniform_soup(2000, seed=32)
    bvh.rebuild(tris2, models=S.identity_models(1))
    ref = O.build_bvh(tris2, 2000, S.identity_models(1))
    np.testing.assert_array_equal(bvh.nodes().view(np.uint32), ref["nodes"].view(np.uint32))


def test_device_resident_inputs(ctx):
    torch = pytest.importorskip("torch")
    n = 10000
    tris = S.uniform_soup(n, seed=41)
    models = S.identity_models(1)
    bvh = ctx.build(torch.from_numpy(tris).cuda(), n_tris=n, models=torch.from_numpy(models).cuda())
    out = torch.empty((2 * n - 1, 12), dtype=torch.float32, device="cuda")
    bvh.nodes(out)
    ref = O.build_bvh(tris, n, models)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), ref["nodes"].view(np.uint32))


def test_bad_model_id_is_an_error(ctx):
    from realtimeraytracing_gb300 import crt
    tris = S.uniform_soup(100, seed=1)
    tris.view(np.uint32)[5, 12] = 64
    with pytest.raises(crt.CrtError) as e:
        ctx.build(tris, models=S.identity_models(1))
    assert e.value.status == 7


@pytest.mark.parametrize("n", [2, 1000, 70000])
def test_multi_launch_build_matches(ctx, n):
    """The one-launch persistent PLOC+layout and the per-iteration launches
    produce the same node array."""
    from realtimeraytracing_gb300 import crt
    c = crt.Context(multi_launch_build=True)
    tris = S.uniform_soup(n, seed=60 + n)
    _check_build(c, tris, n, S.identity_models(1))
    c.close()


def test_bounded_wait_times_out_and_the_context_stays_usable(ctx):
    """A device wait on a flag that nothing sets gives up after its bound and
    reports CRT_ERR_DEVICE_TIMEOUT (no trap, no hang); the same wait on a set
    flag passes; builds and traces on the context still match the oracle."""
    ctx.selftest_wait(True, spin_limit=1 << 12)
    with pytest.raises(crt.CrtError) as e:
        ctx.selftest_wait(False, spin_limit=1 << 12)
    assert e.value.status == 4  # CRT_ERR_DEVICE_TIMEOUT
    tris = S.uniform_soup(3000, seed=17)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    ref = O.build_bvh(tris, 3000, models)
    assert np.array_equal(bvh.nodes().view(np.uint32), ref["nodes"].view(np.uint32))
    rays = S.sphere_rays(2000, seed=8)
    h = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    rh, _ = O.trace(ref["nodes"], tris, models, rays, crt.TRI_WATERTIGHT)
    assert np.array_equal(h.view(np.uint32), rh.view(np.uint32))
    bvh.free()
