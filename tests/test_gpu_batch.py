"""Batched scenes (config 2 launch structure): every scene's BVH from the
one-launch-per-stage batch equals crt_build on that scene alone, bit for
bit; batched traces equal per-scene traces; the CUDA-graph replay and the
autotuned configuration give the same hits."""
import numpy as np
import pytest

from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SIZES = [1, 2, 1000, 4097, 20000, 70000, 3]
RAYS = [100, 64, 5000, 3000, 10000, 7000, 50]


@pytest.fixture(scope="module")
def batch_data(ctx):
    scenes = [S.config2_scene(k, n, seed=7) for k, n in enumerate(SIZES)]
    rays = [S.sphere_rays(m, seed=10 + k) for k, m in enumerate(RAYS)]
    tris = torch.from_numpy(np.concatenate(scenes)).cuda()
    r = torch.from_numpy(np.concatenate(rays)).cuda()
    b = crt.Batch(ctx, SIZES, RAYS, models=S.identity_models(1))
    return scenes, rays, tris, r, b


def _i32(t):
    return t.view(torch.int32)


def test_batch_build_matches_single_scene_builds(ctx, batch_data):
    scenes, rays, tris, r, b = batch_data
    b.build(tris)
    for k, sc in enumerate(scenes):
        single = ctx.build(sc, models=S.identity_models(1))
        ref = single.nodes()
        got = b.nodes(k)
        bad = np.nonzero((got.view(np.uint32) != ref.view(np.uint32)).any(axis=1))[0]
        assert bad.size == 0, f"scene {k}: {bad.size} node records differ"
        assert b.scene_info(k)["iterations"] == ctx.last_build_stats()["ploc_iterations"]


@pytest.mark.parametrize("flags", [crt.TRI_WATERTIGHT, crt.TRI_REFERENCE, crt.TRI_WATERTIGHT | crt.TRACE_ANY])
def test_batch_trace_matches_single_scene_traces(ctx, batch_data, flags):
    scenes, rays, tris, r, b = batch_data
    b.build(tris)
    hits = torch.empty((r.shape[0], 4), dtype=torch.float32, device="cuda")
    b.trace(r, hits, flags)
    got = hits.cpu().numpy()
    off = 0
    for k, sc in enumerate(scenes):
        single = ctx.build(sc, models=S.identity_models(1))
        ref = ctx.trace(single, rays[k], flags)
        g = got[off:off + len(rays[k])]
        if flags & crt.TRACE_ANY:
            np.testing.assert_array_equal(g[:, 0].view(np.uint32) == crt.MISS, ref[:, 0].view(np.uint32) == crt.MISS)
        else:
            np.testing.assert_array_equal(g.view(np.uint32), ref.view(np.uint32), err_msg=f"scene {k}")
        off += len(rays[k])


def test_graph_replay_and_autotune(ctx, batch_data):
    scenes, rays, tris, r, b = batch_data
    h0 = torch.empty((r.shape[0], 4), dtype=torch.float32, device="cuda")
    b.run(tris, r, h0, crt.TRI_WATERTIGHT, graph=False)
    h1 = torch.empty_like(h0)
    used = b.run(tris, r, h1, crt.TRI_WATERTIGHT, graph=True)
    assert torch.equal(_i32(h0), _i32(h1))
    h1.zero_()
    used2 = b.run(tris, r, h1, crt.TRI_WATERTIGHT, graph=True)
    assert used == used2
    assert torch.equal(_i32(h0), _i32(h1))
    print(f"\ngraph path used: {used}")
    cfg, ms = b.autotune(tris, r, h1, crt.TRI_WATERTIGHT)
    assert cfg["ploc_radius"] in (8, 16, 32) and cfg["sort_digit_bits"] in (4, 8)
    assert cfg["trace_block"] in (128, 256, 512) and ms > 0
    h2 = torch.empty_like(h0)
    b.run(tris, r, h2, crt.TRI_WATERTIGHT, graph=True)
    # watertight closest hits do not depend on the BVH (ties keep the lower triangle id)
    assert torch.equal(_i32(h0), _i32(h2))


@pytest.mark.parametrize("flags", [crt.TRI_WATERTIGHT, crt.TRI_REFERENCE, crt.TRI_WATERTIGHT | crt.TRACE_ANY])
def test_batch_sorted_rays_same_hits(ctx, batch_data, flags):
    """CRT_TRACE_SORT_RAYS traces every scene's rays in coherence order
    (scene, origin cell, direction); each ray keeps its own hit, through
    crt_batch_trace and through the graph-replayed crt_batch_run."""
    scenes, rays, tris, r, b = batch_data
    b.build(tris)
    h0 = torch.empty((r.shape[0], 4), dtype=torch.float32, device="cuda")
    h1 = torch.empty_like(h0)
    b.trace(r, h0, flags)
    b.trace(r, h1, flags | crt.SORT_RAYS)
    if flags & crt.TRACE_ANY:
        assert torch.equal(_i32(h0)[:, 0] == -1, _i32(h1)[:, 0] == -1)
    else:
        assert torch.equal(_i32(h0), _i32(h1))
    h2 = torch.empty_like(h0)
    b.run(tris, r, h2, flags | crt.SORT_RAYS, graph=True)
    b.run(tris, r, h2, flags | crt.SORT_RAYS, graph=True)
    if flags & crt.TRACE_ANY:
        assert torch.equal(_i32(h0)[:, 0] == -1, _i32(h2)[:, 0] == -1)
    else:
        assert torch.equal(_i32(h0), _i32(h2))


def test_batch_learned_modes_give_the_plain_hits(ctx):
    """A predictor over every scene of a batch (crt_batch_predictor_create):
    trained online on the batch's own exact hits, it lowers its loss; traces
    ordered by its prediction (CRT_TRACE_PREDICTOR_ORDER), seeded by it
    (CRT_TRACE_USE_PREDICTOR) or both, direct or replayed from the batch's
    CUDA graph, return the plain batch trace's hits bit for bit, for both
    triangle predicates and closest or any hit."""
    sizes = [30000, 1, 5000, 60000, 2]
    n_rays = [20000, 30, 6000, 40000, 10]
    scenes = [S.clustered_soup(n, 16, 0.03, 0.004, 0.5, seed=40 + k) if n > 2 else S.uniform_soup(n, seed=40 + k)
              for k, n in enumerate(sizes)]
    rays = [S.sphere_rays(m, seed=50 + k) for k, m in enumerate(n_rays)]
    tris = torch.from_numpy(np.concatenate(scenes)).cuda()
    r = torch.from_numpy(np.concatenate(rays)).cuda()
    b = crt.Batch(ctx, sizes, n_rays, models=S.identity_models(1))
    b.build(tris)
    total = int(sum(n_rays))
    plain = torch.empty((total, 4), dtype=torch.float32, device="cuda")
    b.trace(r, plain, crt.TRI_WATERTIGHT)
    pred = crt.Predictor(ctx, b, seed=4, train_stride=1, batch=8192)
    assert pred.info()["treelets"] > 100
    truth = pred.classes_of_hits(plain)
    pc = plain[:, 0].view(torch.int32).cpu().numpy()
    assert ((truth == 127) == (pc == -1)).all()
    losses = [pred.train(r, plain, offset=0) for _ in range(8)]
    assert losses[-1] < losses[0]
    got = torch.empty_like(plain)
    for pf in (crt.TRI_WATERTIGHT, crt.TRI_REFERENCE):
        ref = torch.empty_like(plain)
        b.trace(r, ref, pf)
        for lf in (crt.PREDICTOR_ORDER, crt.USE_PREDICTOR, crt.PREDICTOR_ORDER | crt.USE_PREDICTOR):
            b.trace(r, got, pf | lf)
            assert torch.equal(_i32(got), _i32(ref)), (pf, lf)
    anyref = torch.empty_like(plain)
    b.trace(r, anyref, crt.TRI_WATERTIGHT | crt.TRACE_ANY)
    b.trace(r, got, crt.TRI_WATERTIGHT | crt.TRACE_ANY | crt.PREDICTOR_ORDER | crt.USE_PREDICTOR)
    assert torch.equal(_i32(got)[:, 0] == -1, _i32(anyref)[:, 0] == -1)
    # build + learned trace replayed from the graph; a rebuild needs a retarget
    for _ in range(2):
        used = b.run(tris, r, got, crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER, graph=True)
        pred.retarget()
        assert torch.equal(_i32(got), _i32(plain))
    assert used
    pred.free()
    b.free()


def test_batch_ray_counts_graph_key_and_bounce_rays(ctx):
    """crt_batch_set_ray_counts: traces of fewer rays per scene (within the
    batch's capacity) equal the single-scene traces of the same rays; the
    graph captured with one set of counts replays when those counts return and
    is recaptured for others; crt_batch_bounce_rays equals crt_bounce_rays on
    the scene built alone, bit for bit; a learned trace after a count change
    keeps the plain hits; counts above the capacity are refused."""
    sizes = [20000, 3, 9000]
    cap = [12000, 40, 8000]
    scenes = [S.clustered_soup(n, 8, 0.05, 0.004, 0.5, seed=60 + k) if n > 3 else S.uniform_soup(n, seed=60 + k)
              for k, n in enumerate(sizes)]
    rays = [S.sphere_rays(m, seed=70 + k) for k, m in enumerate(cap)]
    tris = torch.from_numpy(np.concatenate(scenes)).cuda()
    r_full = torch.from_numpy(np.concatenate(rays)).cuda()
    b = crt.Batch(ctx, sizes, cap, models=S.identity_models(1))
    h_full = torch.empty((r_full.shape[0], 4), dtype=torch.float32, device="cuda")
    assert b.run(tris, r_full, h_full, crt.TRI_WATERTIGHT, graph=True)
    singles = [ctx.build(sc, models=S.identity_models(1)) for sc in scenes]
    # fewer rays per scene, one of them none at all
    small = [5000, 0, 7999]
    r_small = torch.from_numpy(np.concatenate([rays[k][:m] for k, m in enumerate(small)])).cuda()
    h_small = torch.empty((r_small.shape[0], 4), dtype=torch.float32, device="cuda")
    b.set_ray_counts(small)
    assert b.scene_info(2)["rays"] == 7999
    for flags in (crt.TRI_WATERTIGHT, crt.TRI_REFERENCE, crt.TRI_WATERTIGHT | crt.SORT_RAYS):
        b.trace(r_small, h_small, flags)
        got = h_small.cpu().numpy()
        off = 0
        for k, m in enumerate(small):
            if m:
                ref = ctx.trace(singles[k], rays[k][:m], flags & ~crt.SORT_RAYS)
                np.testing.assert_array_equal(got[off:off + m].view(np.uint32), ref.view(np.uint32), err_msg=f"{k} {flags}")
            off += m
    # the graph of the full counts replays once they are back
    b.set_ray_counts(cap)
    h2 = torch.empty_like(h_full)
    assert b.run(tris, r_full, h2, crt.TRI_WATERTIGHT, graph=True)
    assert torch.equal(_i32(h2), _i32(h_full))
    with pytest.raises(crt.CrtError):
        b.set_ray_counts([cap[0] + cap[1] + cap[2] + 1, 0, 0])
    # bounce rays from scene 2's primary hits, as the single-scene call makes them
    off2 = cap[0] + cap[1]
    prim2, hit2 = r_full[off2:], h_full[off2:]
    n_out = 2 * int((hit2[:, 0].view(torch.int32) != -1).sum().item())
    assert n_out > 400
    got = b.bounce_rays(2, prim2, hit2, n_out, seed=5)
    want = torch.empty_like(got)
    ctx.bounce_rays(singles[2], prim2, hit2, n_out, seed=5, out=want)
    assert torch.equal(_i32(got), _i32(want))
    # a learned trace of those bounce rays as the batch's only rays
    b.set_ray_counts([0, 0, n_out])
    pred = crt.Predictor(ctx, b, seed=2, train_stride=1, batch=4096)
    plain = torch.empty((n_out, 4), dtype=torch.float32, device="cuda")
    b.trace(got, plain, crt.TRI_WATERTIGHT)
    pred.train(got, plain, offset=0)
    learned = torch.empty_like(plain)
    b.trace(got, learned, crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER | crt.USE_PREDICTOR)
    assert torch.equal(_i32(learned), _i32(plain))
    ref = ctx.trace(singles[2], got.cpu().numpy(), crt.TRI_WATERTIGHT)
    np.testing.assert_array_equal(plain.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    pred.free()
    for s_ in singles:
        s_.free()
    b.free()
