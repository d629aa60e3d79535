"""The allocation-free Morton + sort entry point (crt_morton_sort_noalloc)
against the allocating build (crt_build + crt_bvh_copy_codes/perm).

crt_morton_sort_noalloc exists for callers that must not let this library
allocate device memory — engines that own all device memory through their
own pool and forbid embedded libraries from calling cudaMalloc.  Its scratch
is a fixed array inside the library that every call reuses, so this test
makes two different calls in a row (the second one smaller, on a padded
buffer) and checks both against the allocating path bit for bit — codes and
permutations are integers, so the tolerance is exact equality, as in the
other build tests.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _noalloc(d_tris, n_buffer, n_tris, models, d_codes, d_perm, n_models=None):
    """models: a host array, a device tensor (must be refused) or None."""
    L = crt.lib()
    if models is None:
        mp, nm = None, 0
    elif hasattr(models, "data_ptr"):
        mp, nm = C.c_void_p(models.data_ptr()), models.shape[0]
    else:
        mp, nm = models.ctypes.data_as(C.c_void_p), models.shape[0]
    if n_models is not None:
        nm = n_models
    return L.crt_morton_sort_noalloc(C.c_void_p(d_tris.data_ptr()), n_buffer, n_tris, mp, nm,
                                     C.c_void_p(d_codes.data_ptr()), C.c_void_p(d_perm.data_ptr()), None)


def _three_models():
    models = S.identity_models(3)
    models[1, 12:15] = [0.25, -1.0, 3.0]                     # translation
    models[2, 0:16] = np.array([0.0, 1.0, 0.0, 0.0, -2.0, 0.0, 0.0, 0.0,
                                0.0, 0.0, 0.5, 0.0, 1.0, 1.0, 1.0, 1.0], np.float32)  # rotate+scale+translate
    return models


def _check_against_build(torch, ctx, tris, n, models):
    ref = ctx.build(tris, n_tris=n, models=models)
    ref_codes, ref_perm = ref.codes(), ref.perm()
    ref.free()
    d_tris = torch.from_numpy(tris).cuda()
    d_codes = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    d_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = _noalloc(d_tris, tris.shape[0], n, models, d_codes, d_perm)
    assert st == 0, crt.lib().crt_last_error_string().decode()
    np.testing.assert_array_equal(d_codes.cpu().numpy().view(np.uint32), ref_codes)
    np.testing.assert_array_equal(d_perm.cpu().numpy().view(np.uint32), ref_perm)


def test_noalloc_sort_matches_crt_build_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    ctx = crt.Context()
    models = S.identity_models(1)
    big = S.uniform_soup(crt_max(), seed=71)
    small = S.clustered_soup(40000, 32, 0.03, 0.005, 0.5, seed=72)
    small_padded = np.concatenate([small, np.zeros((5000, 16), np.float32)])
    cases = [(big, big.shape[0]), (small_padded, small.shape[0])]
    for tris, n in cases:
        ref = ctx.build(tris, n_tris=n, models=models)
        ref_codes, ref_perm = ref.codes(), ref.perm()
        d_tris = torch.from_numpy(tris).cuda()
        d_codes = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        d_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        st = _noalloc(d_tris, tris.shape[0], n, models, d_codes, d_perm)
        assert st == 0, crt.lib().crt_last_error_string().decode()
        np.testing.assert_array_equal(d_codes.cpu().numpy().view(np.uint32), ref_codes)
        np.testing.assert_array_equal(d_perm.cpu().numpy().view(np.uint32), ref_perm)
        ref.free()
    ctx.close()


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    n = crt_max() + 1
    d_tris = torch.zeros((n, 16), dtype=torch.float32, device="cuda")
    d_out = torch.empty((n,), dtype=torch.int32, device="cuda")
    st = _noalloc(d_tris, n, n, S.identity_models(1), d_out, d_out)
    assert st == 1
    assert "CRT_NOALLOC_MAX_TRIANGLES" in crt.lib().crt_last_error_string().decode()


def crt_max():
    with open(__file__.replace("tests/test_zz_no_alloc.py", "include/crt.h")) as f:
        for line in f:
            if line.startswith("#define CRT_NOALLOC_MAX_TRIANGLES"):
                return int(line.split()[2].rstrip("u"))
    raise AssertionError("CRT_NOALLOC_MAX_TRIANGLES not found")


def test_noalloc_model_table():
    """Three non-identity model matrices with model ids spread over the
    triangles, then no models at all (NULL, n_models = 0: every id uses the
    identity, as crt_build pads the table), each against crt_build."""
    torch = pytest.importorskip("torch")
    ctx = crt.Context()
    n = 30000
    tris = S.uniform_soup(n, seed=73)
    tris.view(np.uint32)[:, 12] = (np.arange(n) * 7) % 3
    _check_against_build(torch, ctx, tris, n, _three_models())
    plain = S.uniform_soup(20000, seed=74)
    ref = ctx.build(plain, models=S.identity_models(1))
    want_codes, want_perm = ref.codes(), ref.perm()
    ref.free()
    d_tris = torch.from_numpy(plain).cuda()
    d_codes = torch.empty((20000,), dtype=torch.int32, device="cuda")
    d_perm = torch.empty((20000,), dtype=torch.int32, device="cuda")
    st = _noalloc(d_tris, 20000, 20000, None, d_codes, d_perm)
    assert st == 0, crt.lib().crt_last_error_string().decode()
    np.testing.assert_array_equal(d_codes.cpu().numpy().view(np.uint32), want_codes)
    np.testing.assert_array_equal(d_perm.cpu().numpy().view(np.uint32), want_perm)
    ctx.close()


def test_noalloc_refuses_device_models_and_reports_bad_model_ids():
    torch = pytest.importorskip("torch")
    n = 1000
    tris = S.uniform_soup(n, seed=75)
    d_tris = torch.from_numpy(tris).cuda()
    d_out = torch.empty((2, n), dtype=torch.int32, device="cuda")
    d_models = torch.from_numpy(S.identity_models(1)).cuda()
    st = _noalloc(d_tris, n, n, d_models, d_out[0], d_out[1])
    assert st == 1 and "host memory" in crt.lib().crt_last_error_string().decode()
    bad = tris.copy()
    bad.view(np.uint32)[17, 12] = 64
    st = _noalloc(torch.from_numpy(bad).cuda(), n, n, S.identity_models(1), d_out[0], d_out[1])
    assert st == 7, crt.lib().crt_last_error_string().decode()
    # a bad call leaves the shared scratch usable: the next call is exact again
    ctx = crt.Context()
    _check_against_build(torch, ctx, tris, n, S.identity_models(1))
    ctx.close()
