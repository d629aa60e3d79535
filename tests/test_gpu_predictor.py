"""The learned hit predictor on the GPU.

* Its tcgen05 forward/backward gradients against the CPU oracle's numpy
  restatement (oracle/predictor_oracle.py), per parameter block.
* Seeded traversal (network, true or random treelet classes) returns exactly
  the plain traversal's hits, for both triangle predicates.
* Online training on the tracer's own hits lowers the loss and lifts the
  treelet hit rate well above chance; the test reports what seeding gains
  (or costs) in node fetches against the plain traversal.
"""
import numpy as np
import pytest

from oracle import predictor_oracle as PO
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def scene(ctx):
    tris = S.clustered_soup(200_000, 64, 0.03, 0.004, 0.5, seed=13)
    models = S.identity_models(1)
    bvh = ctx.build(torch.from_numpy(tris).cuda(), models=torch.from_numpy(models).cuda())
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    w = 512
    rays = torch.empty((w * w, 8), dtype=torch.float32, device="cuda")
    ctx.raygen(cam, w, w, out=rays)
    hits = torch.empty((w * w, 4), dtype=torch.float32, device="cuda")
    ctx.trace(bvh, rays, crt.TRI_WATERTIGHT, out=hits)
    nb = 400_000
    bounce = torch.empty((nb, 8), dtype=torch.float32, device="cuda")
    ctx.bounce_rays(bvh, rays, hits, nb, seed=5, out=bounce)
    return bvh, bounce


def _primary(ctx, bvh):
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = torch.empty((512 * 512, 8), dtype=torch.float32, device="cuda")
    ctx.raygen(cam, 512, 512, out=rays)
    hits = torch.empty((512 * 512, 4), dtype=torch.float32, device="cuda")
    ctx.trace(bvh, rays, crt.TRI_WATERTIGHT, out=hits)
    return rays, hits


def _i32(t):
    return t.view(torch.int32)


def test_gradients_match_cpu_oracle(ctx, scene):
    bvh, bounce = scene
    pred = crt.Predictor(ctx, bvh, seed=3)
    rays = bounce[:640].cpu().numpy()
    targets = np.random.default_rng(1).integers(0, 128, rays.shape[0]).astype(np.uint16)
    g, loss = pred.gradients(rays, targets)
    root = bvh.nodes()[0]
    g_ref, loss_ref, _ = PO.forward_backward(pred.params(), rays, targets, root[0:3], root[4:7])
    assert abs(loss - loss_ref) <= 1e-3 * abs(loss_ref)
    for name, a, b in PO.BLOCKS:
        da, db = g[a:b].astype(np.float64), g_ref[a:b].astype(np.float64)
        rel = np.linalg.norm(da - db) / max(np.linalg.norm(db), 1e-30)
        assert rel < 2e-3, f"gradient block {name}: relative error {rel:.3e}"
    pred.free()


def test_params_round_trip(ctx, scene):
    bvh, _ = scene
    pred = crt.Predictor(ctx, bvh, seed=4)
    p = pred.params()
    p2 = p.copy()
    p2[:100] += 1.0
    pred.set_params(p2)
    np.testing.assert_array_equal(pred.params(), p2)
    assert pred.info()["treelets"] >= 2
    pred.free()


@pytest.mark.parametrize("flags", [crt.TRI_WATERTIGHT, crt.TRI_REFERENCE])
def test_seeded_traversal_is_exact(ctx, scene, flags):
    bvh, bounce = scene
    pred = crt.Predictor(ctx, bvh, seed=5)
    n = bounce.shape[0]
    plain = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    ctx.trace(bvh, bounce, flags, out=plain)
    pred.train(bounce, plain)
    seeded = torch.empty_like(plain)
    ctx.trace(bvh, bounce, flags | crt.USE_PREDICTOR, out=seeded)
    assert torch.equal(_i32(seeded), _i32(plain))
    truth = torch.from_numpy(pred.classes_of_hits(plain).astype(np.int16)).cuda()
    ctx.trace_seeded(bvh, bounce, truth, flags, out=seeded)
    assert torch.equal(_i32(seeded), _i32(plain))
    rnd = torch.randint(0, 127, (n,), device="cuda", dtype=torch.int16)
    ctx.trace_seeded(bvh, bounce, rnd, flags, out=seeded)
    assert torch.equal(_i32(seeded), _i32(plain))
    # any-hit with seeding agrees on occlusion
    a0 = torch.empty_like(plain)
    a1 = torch.empty_like(plain)
    ctx.trace(bvh, bounce, flags | crt.TRACE_ANY, out=a0)
    ctx.trace(bvh, bounce, flags | crt.TRACE_ANY | crt.USE_PREDICTOR, out=a1)
    assert torch.equal(_i32(a0)[:, 0] == -1, _i32(a1)[:, 0] == -1)
    pred.free()


def test_training_learns_and_reports_gain(ctx, scene):
    bvh, bounce = scene
    pred = crt.Predictor(ctx, bvh, seed=6, miss_threshold=0.9)
    n = bounce.shape[0]
    plain = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    ctx.trace(bvh, bounce, crt.TRI_WATERTIGHT | crt.TRACE_STATS, out=plain)
    plain_fetch, _ = ctx.last_trace_stats()
    truth = pred.classes_of_hits(plain)
    hit = truth != 127
    before = (pred.infer(bounce)[hit] == truth[hit]).mean()
    losses = [pred.train(bounce, plain, offset=e % 20) for e in range(40)]
    after = (pred.infer(bounce)[hit] == truth[hit]).mean()
    assert losses[-1] < losses[0]
    n_classes = pred.info()["treelets"]
    assert after > max(2.0 / n_classes, 2 * before), (before, after)
    seeded = torch.empty_like(plain)
    ctx.trace(bvh, bounce, crt.TRI_WATERTIGHT | crt.USE_PREDICTOR | crt.TRACE_STATS, out=seeded)
    seeded_fetch, _ = ctx.last_trace_stats()
    assert torch.equal(_i32(seeded), _i32(plain))
    print(f"\nlearned seeding: treelet hit rate {before:.3f} -> {after:.3f} over {n_classes} treelets; "
          f"node fetches per ray plain {plain_fetch / n:.2f}, seeded {seeded_fetch / n:.2f} "
          f"(gain {(plain_fetch - seeded_fetch) / plain_fetch:+.1%})")
    pred.free()


def test_bounce_rays_deterministic_and_traced_like_the_oracle(ctx, scene):
    from oracle import oracle as O
    bvh, bounce = scene
    tris = S.clustered_soup(200_000, 64, 0.03, 0.004, 0.5, seed=13)  # the scene fixture's triangles
    sub = bounce[:20000].cpu().numpy()
    d = np.linalg.norm(sub[:, 4:7], axis=1)
    assert np.all(np.abs(d - 1) < 1e-3)
    again = ctx.bounce_rays(bvh, *_primary(ctx, bvh), 20000, seed=5)
    np.testing.assert_array_equal(again.view(np.uint32), sub.view(np.uint32))
    got = ctx.trace(bvh, sub, crt.TRI_WATERTIGHT)
    ref, _ = O.trace(bvh.nodes(), tris, S.identity_models(1), sub, crt.TRI_WATERTIGHT)
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("flags", [crt.TRI_WATERTIGHT, crt.TRI_REFERENCE, crt.TRI_WATERTIGHT | crt.TRACE_ANY])
def test_predictor_ordered_traversal_is_exact(ctx, scene, flags):
    """CRT_TRACE_PREDICTOR_ORDER traces the rays grouped by predicted treelet
    (alone and with seeding): every ray gets the plain traversal's hit."""
    bvh, bounce = scene
    pred = crt.Predictor(ctx, bvh, seed=8)
    n = bounce.shape[0]
    plain = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    ctx.trace(bvh, bounce, flags, out=plain)
    pred.train(bounce, plain)
    got = torch.empty_like(plain)
    ctx.trace(bvh, bounce, flags | crt.PREDICTOR_ORDER, out=got)
    ok = torch.equal(_i32(got), _i32(plain)) if not flags & crt.TRACE_ANY else \
        torch.equal(_i32(got)[:, 0] == -1, _i32(plain)[:, 0] == -1)
    assert ok
    ctx.trace(bvh, bounce, flags | crt.PREDICTOR_ORDER | crt.USE_PREDICTOR, out=got)
    ok = torch.equal(_i32(got), _i32(plain)) if not flags & crt.TRACE_ANY else \
        torch.equal(_i32(got)[:, 0] == -1, _i32(plain)[:, 0] == -1)
    assert ok
    pred.free()


def test_mma_wait_times_out_frees_tensor_memory_and_the_context_stays_usable(ctx):
    """The predictor kernels' MMA wait: a commit that completes passes and
    reads the right product; a phase nothing completes gives up after a short
    bound with CRT_ERR_DEVICE_TIMEOUT, without reading tensor memory, and the
    CTA still frees it — so the next tcgen05 kernels (the predictor's own
    inference and training) allocate and run as before."""
    ctx.selftest_tc_wait(True)
    with pytest.raises(crt.CrtError) as e:
        ctx.selftest_tc_wait(False, spin_limit=1 << 10)
    assert e.value.status == 4  # CRT_ERR_DEVICE_TIMEOUT
    ctx.selftest_tc_wait(True)
    tris = S.uniform_soup(20000, seed=91)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    rays = S.sphere_rays(4096, seed=92)
    hits = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    pred = crt.Predictor(ctx, bvh, seed=5)
    loss = pred.train(rays, hits, offset=0)
    assert np.isfinite(loss)
    seeded = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.USE_PREDICTOR)
    assert np.array_equal(seeded.view(np.uint32), hits.view(np.uint32))
    pred.free()
    bvh.free()


def test_adam_step_matches_numpy(ctx):
    """One training step over a single batch equals Adam (b1 0.9, b2 0.999,
    eps 1e-8, bias-corrected) applied in numpy to the mean of the kernels'
    own gradients (crt_predictor_gradients), for every parameter."""
    tris = S.clustered_soup(50_000, 16, 0.03, 0.004, 0.5, seed=93)
    models = S.identity_models(1)
    bvh = ctx.build(tris, models=models)
    rays = S.sphere_rays(4096, seed=94)
    hits = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    pred = crt.Predictor(ctx, bvh, seed=7, lr=1e-3, train_stride=1, batch=4096)
    p0 = pred.params()
    targets = pred.classes_of_hits(hits)
    grad, _ = pred.gradients(rays, targets)
    pred.train(rays, hits, offset=0)
    p1 = pred.params()
    g = grad.astype(np.float64) / 4096.0
    m = 0.1 * g
    v = 0.001 * g * g
    want = p0 - 1e-3 * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    np.testing.assert_allclose(p1, want, rtol=2e-5, atol=2e-7)
    assert np.abs(p1 - p0).max() > 1e-4  # the step moved the weights
    pred.free()
    bvh.free()


def test_learned_order_from_host_rays_in_pieces(ctx, scene):
    """crt_trace of host rays with CRT_TRACE_PREDICTOR_ORDER: from pageable
    memory (1 M rays or more) the rays are copied in pieces on a second stream
    and each piece's inference runs as soon as it has landed; from page-locked
    memory the inference kernel reads them in place and stores the device copy
    the trace reads.  The hits equal the plain trace's bit for bit, both ways,
    above and below the piece threshold."""
    bvh, _ = scene
    pred = crt.Predictor(ctx, bvh, seed=9)
    rays = S.sphere_rays(1_200_000, seed=97)
    plain = ctx.trace(bvh, rays, crt.TRI_WATERTIGHT)
    pred.train(rays[:200_000], plain[:200_000], offset=0)
    flags = crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER
    got = ctx.trace(bvh, rays, flags)
    np.testing.assert_array_equal(got.view(np.uint32), plain.view(np.uint32))
    pinned_rays = torch.from_numpy(rays).pin_memory()
    pinned_hits = torch.empty((rays.shape[0], 4), dtype=torch.float32).pin_memory()
    ctx.trace(bvh, pinned_rays, flags, out=pinned_hits)
    np.testing.assert_array_equal(pinned_hits.numpy().view(np.uint32), plain.view(np.uint32))
    small = ctx.trace(bvh, rays[:300_001], flags)
    np.testing.assert_array_equal(small.view(np.uint32), plain[:300_001].view(np.uint32))
    small_pinned = torch.from_numpy(rays[:300_001]).pin_memory()
    small_hits = ctx.trace(bvh, small_pinned, flags)
    np.testing.assert_array_equal(small_hits.view(np.uint32), plain[:300_001].view(np.uint32))
    pred.free()
