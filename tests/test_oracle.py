"""The CPU oracle against the reference (CPU only).

1. Where the reference checkout exists, oracle/_ref/libref_bvh.so is the
   reference's own srcCommon/scene/geometry/bvh.cpp + triangle.cpp compiled
   unmodified; the oracle's restatement must reproduce its Morton codes,
   permutation and DFS node array bit for bit.
2. Everywhere, the restatement must reproduce the committed golden fixtures
   that tests/golden/make_golden.py generated from that reference library.
3. Sub-step pins from the reference's own tests: the 4-digit segmented
   exclusive scan of tests/testsSortGPU/testHistogramPrefixSum.cpp:53-85.
4. Internal consistency of the traversal restatement (BVH DFS vs brute force).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(O.REFERENCE_DIR, "srcCommon")),
                               reason="reference checkout not present (golden fixtures cover this machine)")


@needs_ref
@pytest.mark.parametrize("n,pad", [(1, 0), (2, 0), (3, 0), (5, 0), (17, 0), (100, 0), (1023, 0), (1024, 0),
                                   (4097, 0), (65536, 0), (1000, 65536 - 1000), (1, 7)])
def test_restatement_matches_reference_bvh_cpp(n, pad):
    tris = S.uniform_soup(n, seed=900 + n)
    if pad:
        tris[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]] += np.float32(0.5)
        tris = np.concatenate([tris, np.zeros((pad, 16), np.float32)])
    models = S.identity_models(1)
    ref = O.ref_build_bvh(tris, n, models)
    mine = O.build_bvh(tris, n, models)
    codes_u, _, _ = O.morton(tris, n, models)
    np.testing.assert_array_equal(codes_u, ref["codes_unsorted"])
    np.testing.assert_array_equal(mine["codes"], ref["codes"])
    np.testing.assert_array_equal(mine["perm"], ref["perm"])
    np.testing.assert_array_equal(mine["nodes"].view(np.uint32), ref["nodes"].view(np.uint32))


@needs_ref
def test_restatement_matches_reference_models_and_duplicates():
    tris = S.uniform_soup(3000, seed=31)
    tris.view(np.uint32)[:, 12] = (np.arange(3000) * 7) % 5
    models = S.identity_models(5)
    models[3, 12:15] = [1.5, 0.0, -2.0]
    models[4, 0:16] = np.array([0, 1, 0, 0, 0, 0, 3, 0, 0.5, 0, 0, 0, 0.1, 0.2, 0.3, 1], np.float32)
    for t, n, m in ((tris, 3000, models), (np.repeat(S.uniform_soup(1, seed=3), 150, axis=0), 150, S.identity_models(1))):
        ref = O.ref_build_bvh(t, n, m)
        mine = O.build_bvh(t, n, m, faithful=True)
        np.testing.assert_array_equal(mine["nodes"].view(np.uint32), ref["nodes"].view(np.uint32))
        np.testing.assert_array_equal(mine["perm"], ref["perm"])


def _golden_cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.build_cases()


def test_golden_fixtures():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        index = json.load(f)
    cases = _golden_cases()
    assert len(cases) >= 8
    for name, tris, n, models in cases:
        meta = index[name]
        assert sha(tris) == meta["input_sha256"], f"{name}: scene generator drifted"
        g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        mine = O.build_bvh(tris, n, models)
        np.testing.assert_array_equal(mine["codes"], g["codes"], err_msg=name)
        np.testing.assert_array_equal(mine["perm"], g["perm"], err_msg=name)
        np.testing.assert_array_equal(mine["nodes"].view(np.uint32), g["nodes"].view(np.uint32), err_msg=name)
        codes_u, _, _ = O.morton(tris, n, models)
        np.testing.assert_array_equal(codes_u, g["codes_unsorted"], err_msg=name)


def test_golden_config0_hashes():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        index = json.load(f)
    tris, models, cam, (w, h) = S.config0_scene(seed=0)
    meta = index["config0"]
    assert sha(tris) == meta["input_sha256"]
    mine = O.build_bvh(tris, tris.shape[0], models)
    assert sha(mine["codes"]) == meta["codes_sha256"]
    assert sha(mine["perm"]) == meta["perm_sha256"]
    assert sha(mine["nodes"]) == meta["nodes_sha256"]
    tm = index["config0_trace"]
    rays = O.raygen(cam, w, h)
    assert sha(rays) == tm["rays_sha256"]
    hr, _ = O.trace(mine["nodes"], tris, models, rays, 0)
    assert sha(hr) == tm["hits_reference_sha256"]


def test_digit_group_exclusive_scan_known_answer():
    """testHistogramPrefixSum.cpp:53-85: exclusive scan inside each 4-digit
    group of a digit-count histogram (the digit-offset step of the sort)."""
    counts = np.array([[37, 41, 49, 53], [37, 48, 44, 51], [35, 51, 53, 41]], np.uint32)
    expected = np.array([[0, 37, 78, 127], [0, 37, 85, 129], [0, 35, 86, 139]], np.uint32)
    got = np.concatenate([np.zeros((3, 1), np.uint32), np.cumsum(counts, axis=1)[:, :-1]], axis=1).astype(np.uint32)
    np.testing.assert_array_equal(got, expected)


@pytest.mark.parametrize("flags", [0, 2])
def test_traversal_restatement_vs_brute_force(flags):
    tris = S.uniform_soup(2000, seed=44)
    models = S.identity_models(1)
    b = O.build_bvh(tris, 2000, models)
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = O.raygen(cam, 48, 48)
    h_bvh, _ = O.trace(b["nodes"], tris, models, rays, flags)
    h_bf = O.trace_brute(tris, models, rays, flags)
    np.testing.assert_array_equal(h_bvh[:, 0].view(np.uint32), h_bf[:, 0].view(np.uint32))
    hit = h_bf[:, 0].view(np.uint32) != 0xFFFFFFFF
    assert hit.sum() > 5
    np.testing.assert_array_equal(h_bvh[hit].view(np.uint32), h_bf[hit].view(np.uint32))


def test_reference_predicate_rejects_small_triangles():
    """raytracer.glsl:117-119 rejects |a| < 1e-4: triangles much smaller than
    0.01 never hit with the shader predicate (why the large scenes use the
    watertight predicate)."""
    v, f = S.displaced_icosphere(level=6, seed=1)
    tris = S.indexed_to_triangles(v * np.float32(0.5), f)
    models = S.identity_models(1)
    b = O.build_bvh(tris, tris.shape[0], models)
    rays = O.raygen(S.camera_gpu_data((0.0, 0.0, -3.0)), 32, 32)
    hr, _ = O.trace(b["nodes"], tris, models, rays, 0)
    hw, _ = O.trace(b["nodes"], tris, models, rays, 2)
    assert (hr[:, 0].view(np.uint32) != 0xFFFFFFFF).sum() == 0
    assert (hw[:, 0].view(np.uint32) != 0xFFFFFFFF).sum() > 100


def test_scene_generators_are_deterministic():
    a = S.uniform_soup(5000, seed=3)
    b = S.uniform_soup(5000, seed=3)
    assert sha(a) == sha(b)
    c = S.uniform_soup(5000, seed=4)
    assert sha(a) != sha(c)
    ctr = (a[:, 0:3] + a[:, 4:7] + a[:, 8:11]) / 3
    assert ctr.min() > -0.05 and ctr.max() < 1.05
    e = np.linalg.norm(a[:, 0:3] - a[:, 4:7], axis=1)
    assert e.max() < 0.041
