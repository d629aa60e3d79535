#!/usr/bin/env python
"""Throughput benchmark of the GB300 ray-tracing core.

Workload (one "step" = one frame of the reference's compute pass,
Application::drawOneFrame in srcOpenGL/application.cpp:220-262, minus shading):
  scene   1,310,720-triangle displaced icosphere (subdivision 8, radius 1,
          3-octave value noise of amplitude 0.05), seeded synthetic data;
          the BVH is built by the CUDA PLOC path (build time reported apart
          as build_ms, as the reference builds once at scene load)
  frame   1920x1080 primary rays (getRay) -> closest hit (watertight
          predicate) -> one any-hit shadow ray per hit toward (2, 2, -2);
          crt_trace_frame runs it as one kernel launch (frame_kernel)
  value   rays traced per second (primary + shadow rays of hits), Mrays/s,
          inputs resident in HBM, CUDA events on the library's stream
  e2e     the same frame through the public C ABI call crt_trace_frame with
          the camera in from pinned host memory and both hit buffers out to
          pinned host memory (the frame kernel writes them there directly),
          timed on the host clock around the call

--impl reference times the reference's CPU path on the host cores instead:
its PLOC build (bvh.cpp restated for N > 65,536, the reference's own cap)
and its shader traversal restated in C++ (right-child-first DFS without
t pruning, the shader's triangle predicate), on a bounded sample of rays.

Multi-GPU: replicas (each rank traces its own full frame); value is the
total over ranks divided by the slowest rank's time (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s closest-hit: hit-predictor vs plain, 1 GB300, exact hits; BVH build ms"
WORKLOAD = "displaced icosphere 1,310,720 tris; 1920x1080 primary closest-hit + shadow any-hit to (2,2,-2)"
W, H = 1920, 1080


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_profile_traffic():
    """Per-launch DRAM bytes of the frame kernel from the committed ncu
    summary, if one exists."""
    path = os.path.join(ROOT, "profiles", "frame_kernel_config1.md")
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        # the raw samples go to CRT_CLOCKS_DIR (kept beside the run's other
        # outputs when set), else to the temporary directory
        out_dir = os.environ.get("CRT_CLOCKS_DIR") or tempfile.gettempdir()
        os.makedirs(out_dir, exist_ok=True)
        self.path = os.path.join(out_dir, f"clocks_bench_{os.getpid()}.csv")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def slowest_ms(t_ms: float, world: int, dev=None) -> float:
    """Max of a per-rank time over all ranks (every rank gets it): replicas
    finish together only when the slowest one does."""
    if world <= 1:
        return t_ms
    import torch
    tt = torch.tensor([t_ms], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def whole_job_mrays(world: int, rays_per_replica: int, t_ms: float) -> float:
    """Weak scaling: every replica traces its own frame of rays_per_replica
    rays; the job's throughput is all of them over the slowest time."""
    return world * rays_per_replica / (t_ms * 1e-3) / 1e6


def make_scene():
    from realtimeraytracing_gb300 import scenes as S
    tris, models, cam, (w, h), light = S.config1_scene(seed=0)
    assert (w, h) == (W, H)
    return tris, models, cam, light


# --------------------------------------------------------------- our arm
def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from realtimeraytracing_gb300 import crt

    tris, models, cam, light = make_scene()
    n_tris = tris.shape[0]
    ctx = crt.Context(device=local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    d_tris = torch.from_numpy(tris).to(dev)
    d_models = torch.from_numpy(models).to(dev)
    d_cam = torch.from_numpy(cam).to(dev)
    torch.cuda.synchronize()

    # ---- BVH build (scene load), device-timed inside the library
    bvh = ctx.build(d_tris, models=d_models)
    build_ms = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        bvh.rebuild(d_tris, models=d_models)
        wall = (time.perf_counter() - t0) * 1e3
        st = ctx.last_build_stats()
        if i >= args.warmup:
            build_ms.append((st["ms_total"], wall, st))
    build_dev = statistics.median(b[0] for b in build_ms)
    build_wall = statistics.median(b[1] for b in build_ms)
    stages = {k: round(statistics.median(b[2][k] for b in build_ms), 4)
              for k in ("ms_morton", "ms_sort", "ms_ploc", "ms_layout")}
    iters = build_ms[-1][2]["ploc_iterations"]

    n_rays = W * H
    hp = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
    hs = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
    flags = crt.TRI_WATERTIGHT
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def frame():
        ctx.trace_frame(bvh, d_cam, W, H, light, flags, hits_primary=hp, hits_shadow=hs)

    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    n_hits = int((hp[:, 0].view(torch.int32) != -1).sum().item())
    rays_per_frame = n_rays + n_hits

    # ---- timed frames (device resident), L2 flushed before each frame
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            l2_flush.zero_()
            ev[k][0].record(stream)
            frame()
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    frame_ms = [a.elapsed_time(b) for a, b in ev]
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_frame = slowest_ms(sum(frame_ms) / len(frame_ms), world, dev)
    value = whole_job_mrays(world, rays_per_frame, t_frame)

    # ---- the dominant kernel: the frame is one frame_kernel launch; its node
    # fetches and triangle tests (primary + shadow) from a CRT_TRACE_STATS frame
    ctx.trace_frame(bvh, d_cam, W, H, light, flags | crt.TRACE_STATS, hits_primary=hp, hits_shadow=hs)
    visited, tested = ctx.last_trace_stats()
    k_ms = statistics.mean(frame_ms)  # this rank's frame_kernel launch, L2 flushed before it
    alg_bytes = 64.0 * visited + 48.0 * tested + 2 * 16.0 * n_rays  # nodes, triangles, both hit buffers
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (k_ms * 1e-3) / 1e9
    traffic = read_profile_traffic()
    # the primary closest-hit trace alone (crt_trace over stored rays), for reference
    rays = torch.empty((n_rays, 8), dtype=torch.float32, device=dev)
    ctx.raygen(d_cam, W, H, out=rays)
    ctx.trace(bvh, rays, flags | crt.TRACE_STATS, out=hp)
    p_visited, p_tested = ctx.last_trace_stats()
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            l2_flush.zero_()
            kev[k][0].record(stream)
            ctx.trace(bvh, rays, flags, out=hp)
            kev[k][1].record(stream)
    torch.cuda.synchronize()
    p_ms = statistics.mean(a.elapsed_time(b) for a, b in kev)
    # the same primary trace over the other node formats (same hits)
    node_formats = {"binary_64B": {"ms": round(p_ms, 4), "node_fetches_per_ray": round(p_visited / n_rays, 2)}}
    hp_alt = torch.empty_like(hp)
    for fname, fflag in (("wide4_128B", crt.TRACE_WIDE), ("compressed4_64B", crt.TRACE_COMPRESSED)):
        ctx.trace(bvh, rays, flags | fflag | crt.TRACE_STATS, out=hp_alt)
        f_visited, _ = ctx.last_trace_stats()
        fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                l2_flush.zero_()
                fev[k][0].record(stream)
                ctx.trace(bvh, rays, flags | fflag, out=hp_alt)
                fev[k][1].record(stream)
        torch.cuda.synchronize()
        node_formats[fname] = {"ms": round(statistics.mean(a.elapsed_time(b) for a, b in fev), 4),
                               "node_fetches_per_ray": round(f_visited / n_rays, 2),
                               "identical_hits": bool(torch.equal(hp_alt.view(torch.int32), hp.view(torch.int32)))}
    del hp_alt

    # ---- mesh input: the scene's indexed mesh to TriangleGPU records on the GPU
    from realtimeraytracing_gb300 import scenes as S
    mv, mf = S.displaced_icosphere(8, 0.05, 0)
    d_mv = torch.from_numpy(np.ascontiguousarray(mv, np.float32)).to(dev)
    d_mf = torch.from_numpy(np.ascontiguousarray(mf, np.uint32).view(np.int32)).to(dev)
    d_mt = torch.empty((mf.shape[0], 16), dtype=torch.float32, device=dev)
    for _ in range(2):
        ctx.triangles_from_indexed(d_mv, d_mf, 0, out=d_mt)
    mev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            l2_flush.zero_()
            mev[k][0].record(stream)
            ctx.triangles_from_indexed(d_mv, d_mf, 0, out=d_mt)
            mev[k][1].record(stream)
    torch.cuda.synchronize()
    m_ms = statistics.mean(a.elapsed_time(b) for a, b in mev)
    mesh_upload = {"triangles": int(mf.shape[0]), "ms": round(m_ms, 4),
                   "gbs": round((12 + 36 + 64) * mf.shape[0] / (m_ms * 1e-3) / 1e9, 1),
                   "identical_to_scene_records": bool(torch.equal(d_mt.cpu(), torch.from_numpy(tris))),
                   "note": "crt_triangles_from_indexed on device arrays: 12 B indices + 36 B gathered vertices + "
                           "64 B record per triangle, L2 flushed before each call"}
    del d_mv, d_mf, d_mt

    # ---- the trace side alone over a node array built elsewhere: the reference's
    # CPU build hands its shader this same DFS array (host memory), which
    # crt_bvh_from_nodes makes traceable; the frame over it must equal the frame
    # over the built handle
    nodes_h = bvh.nodes()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    imp = ctx.bvh_from_nodes(nodes_h, tris, models=models)
    import_ms = (time.perf_counter() - t0) * 1e3
    hp_i, hs_i = torch.empty_like(hp), torch.empty_like(hs)
    ctx.trace_frame(bvh, d_cam, W, H, light, flags, hits_primary=hp, hits_shadow=hs)
    iev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    ctx.trace_frame(imp, d_cam, W, H, light, flags, hits_primary=hp_i, hits_shadow=hs_i)
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            l2_flush.zero_()
            iev[k][0].record(stream)
            ctx.trace_frame(imp, d_cam, W, H, light, flags, hits_primary=hp_i, hits_shadow=hs_i)
            iev[k][1].record(stream)
    torch.cuda.synchronize()
    imported_tree = {
        "import_ms": round(import_ms, 3),
        "frame_ms": round(statistics.mean(a.elapsed_time(b) for a, b in iev), 4),
        "identical_hits": bool(torch.equal(hp_i.view(torch.int32), hp.view(torch.int32)) and
                               torch.equal(hs_i[:, 0].view(torch.int32) == -1, hs[:, 0].view(torch.int32) == -1)),
        "note": "crt_bvh_from_nodes from the 2,621,439-record node array in host memory (structure check, "
                "upload, traversal records; host-timed), then the one-launch frame over the imported tree"}
    imp.free()
    del hp_i, hs_i

    # ---- the reference's whole compute pass (getRay, closest hit, getColor,
    # imageStore) into a device RGBA32F image: crt_render_frame, one launch
    img = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
    d_mats = torch.tensor([[0.8, 0.7, 0.6, 1.0]], dtype=torch.float32, device=dev)
    shaded = {}
    for name, sflags, depth in (("plain", 0, 0), ("wireframe_bvh_depth3", crt.SHADE_WIREFRAME | crt.SHADE_BVH, 3)):
        def render():
            ctx.render_frame(bvh, d_cam, W, H, models=d_models, materials=d_mats, shade_flags=sflags,
                             bvh_depth=depth, flags=flags, out=img)
        for _ in range(2):
            render()
        sev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                l2_flush.zero_()
                sev[k][0].record(stream)
                render()
                sev[k][1].record(stream)
        torch.cuda.synchronize()
        s_ms = statistics.mean(a.elapsed_time(b) for a, b in sev)
        shaded[name] = {"ms": round(s_ms, 4), "mrays_s": round(n_rays / (s_ms * 1e-3) / 1e6, 1)}

    # ---- end to end through the public API: camera in, hits out (pinned host)
    hp_h = torch.empty((n_rays, 4), dtype=torch.float32, pin_memory=True)
    hs_h = torch.empty((n_rays, 4), dtype=torch.float32, pin_memory=True)
    cam_h = torch.from_numpy(cam.copy()).pin_memory()
    for _ in range(2):
        ctx.trace_frame(bvh, cam_h, W, H, light, flags, hits_primary=hp_h, hits_shadow=hs_h)
    e2e_ms = []
    for _ in range(args.steps):
        l2_flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.trace_frame(bvh, cam_h, W, H, light, flags, hits_primary=hp_h, hits_shadow=hs_h)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_t = slowest_ms(statistics.mean(e2e_ms), world, dev)
    e2e_value = whole_job_mrays(world, rays_per_frame, e2e_t)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(tris, models, cam)
    batch = None
    if rank == 0 and not args.no_batch:
        batch = run_batch_experiment(ctx, torch, crt, dev, args)
    dynamic = None
    if rank == 0 and not args.no_dynamic:
        dynamic = run_dynamic_experiment(ctx, torch, crt, dev, args)
    predictor = None
    if rank == 0 and not args.no_predictor:
        del d_tris, bvh
        torch.cuda.empty_cache()
        predictor = run_predictor_experiment(ctx, torch, crt, dev, stream, args)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": round(value, 2),
            "unit": "Mrays/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(t_frame, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded displaced icosphere)",
            "config": {"workload": WORKLOAD, "triangles": n_tris, "image": [W, H],
                       "rays_per_step": rays_per_frame, "primary_hits": n_hits,
                       "predicate": "watertight", "ploc_radius": 16, "sort_digit_bits": 8,
                       "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "build_ms": round(build_dev, 4),
            "build_ms_wall": round(build_wall, 4),
            "build_stages_ms": stages,
            "ploc_iterations": iters,
            "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s", "h2d_bytes_per_step": int(cam.nbytes),
                    "d2h_bytes_per_step": int(2 * n_rays * 16), "ms_per_step": round(e2e_t, 4),
                    "transfer": "camera in by cudaMemcpyAsync; both hit buffers (page-locked host memory) written by "
                                "the frame kernel over the CPU-GPU link, host-timed around crt_trace_frame"},
            "gpu_launches": args.steps,
            "roofline": {"kernel": "frame_kernel (camera ray, closest hit, shadow ray, any hit)", "bound": "hbm",
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": peak_kind, "ms_per_launch": round(k_ms, 4),
                         "alg_bytes_per_launch": int(alg_bytes),
                         "node_fetches_per_pixel": round(visited / n_rays, 2),
                         "tris_per_pixel": round(tested / n_rays, 2)},
            "primary_trace_node_formats": node_formats,
            "primary_trace_kernel": {"ms": round(p_ms, 4), "mrays_s": round(n_rays / (p_ms * 1e-3) / 1e6, 1),
                                     "node_fetches_per_ray": round(p_visited / n_rays, 2),
                                     "tris_per_ray": round(p_tested / n_rays, 2)},
            "mesh_upload": mesh_upload,
            "imported_tree": imported_tree,
            "shaded_frame": dict(shaded, note="crt_render_frame: camera ray, closest hit, getColor and "
                                              "imageStore per texel into a device RGBA32F image, no shadow rays"),
            "cpu_baseline": cpu,
            "clocks": clk,
            "batch": batch,
            "dynamic": dynamic,
            "predictor": predictor,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batch_experiment(ctx, torch, crt, dev, args):
    """Config 2: 64 scenes, triangle counts log-uniform over 1k-2M (even scenes
    uniform soups, odd scenes 32-blob clustered soups), each with its own
    log-uniform 64k-4M rays from a radius-2 sphere toward the unit cube.  The
    whole build + trace runs as one launch per stage, autotuned, replayed
    from a CUDA graph; the same work as 64 separate crt_build + crt_trace
    calls is timed beside it."""
    from realtimeraytracing_gb300 import scenes as S
    tri_n, ray_n = S.config2_sizes(64, seed=0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(2)
    tris = torch.cat([S.device_soup(int(n), gen, clustered=(k % 2 == 1)) for k, n in enumerate(tri_n)])
    rays = torch.cat([S.device_sphere_rays(int(m), gen) for m in ray_n])
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device=dev)
    models = S.identity_models(1)
    b = crt.Batch(ctx, tri_n, ray_n, models=models)
    flags = crt.TRI_WATERTIGHT

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3 / reps

    reps = max(3, min(args.steps, 5))
    b.run(tris, rays, hits, flags, graph=False)
    t_default = timed(lambda: b.run(tris, rays, hits, flags, graph=True), reps)
    default_cfg = b.config()
    cfg, tuned_ms = b.autotune(tris, rays, hits, flags)
    used = b.run(tris, rays, hits, flags, graph=True)
    t_graph = timed(lambda: b.run(tris, rays, hits, flags, graph=True), reps)
    t_nograph = timed(lambda: b.run(tris, rays, hits, flags, graph=False), reps)
    t_build = timed(lambda: b.build(tris), reps)
    ref_hits = hits.clone()
    # the same pipeline with every scene's rays traced in coherence order
    sorted_hits = torch.empty_like(hits)
    b.run(tris, rays, sorted_hits, flags | crt.SORT_RAYS, graph=True)
    t_sorted = timed(lambda: b.run(tris, rays, sorted_hits, flags | crt.SORT_RAYS, graph=True), reps)
    sorted_identical = bool(torch.equal(sorted_hits.view(torch.int32), ref_hits.view(torch.int32)))
    # the same work scene by scene through the single-scene API
    c1 = crt.Context(device=dev.index or 0)
    tri_off = np.concatenate([[0], np.cumsum(tri_n)])
    ray_off = np.concatenate([[0], np.cumsum(ray_n)])
    seq_hits = torch.empty_like(hits)
    bvhs = [None] * 64

    def sequential():
        for k in range(64):
            tk = tris[int(tri_off[k]):int(tri_off[k + 1])]
            if bvhs[k] is None:
                bvhs[k] = c1.build(tk, models=models)
            else:
                bvhs[k].rebuild(tk, models=models)
            c1.trace(bvhs[k], rays[int(ray_off[k]):int(ray_off[k + 1])], flags,
                     out=seq_hits[int(ray_off[k]):int(ray_off[k + 1])])

    t_seq = timed(sequential, max(2, reps // 2))
    identical = bool(torch.equal(seq_hits.view(torch.int32), ref_hits.view(torch.int32)))
    for bv in bvhs:
        bv.free()
    c1.close()
    b.free()
    n_rays = int(ray_n.sum())
    return {
        "workload": "64 scenes, tris log-uniform 1k-2M (half uniform, half 32-blob clustered), rays log-uniform 64k-4M",
        "triangles": int(tri_n.sum()), "rays": n_rays,
        "pipeline_ms": round(t_graph, 3), "mrays_s": round(n_rays / t_graph / 1e3, 1),
        "pipeline_ms_no_graph": round(t_nograph, 3), "build_ms": round(t_build, 3),
        "graph_used": used, "default_config_ms": round(t_default, 3),
        "autotuned": {k: cfg[k] for k in ("ploc_radius", "sort_digit_bits", "trace_block", "stack_depth")},
        "default_config": {k: default_cfg[k] for k in ("ploc_radius", "sort_digit_bits", "trace_block", "stack_depth")},
        "sequential_single_scene_ms": round(t_seq, 3), "speedup_vs_sequential": round(t_seq / t_graph, 3),
        "hits_identical_to_sequential": identical,
        "sorted_rays": {"pipeline_ms": round(t_sorted, 3), "mrays_s": round(n_rays / t_sorted / 1e3, 1),
                        "speedup": round(t_graph / t_sorted, 3), "hits_identical": sorted_identical,
                        "note": "CRT_TRACE_SORT_RAYS: rays traced by (scene, Morton code of the cell where the ray enters the scene box, direction bin)"},
    }


def run_dynamic_experiment(ctx, torch, crt, dev, args, frames=60):
    """Config 4: a 16,777,216-triangle clustered soup (1024 clusters, sigma
    0.02, edges lognormal(ln 0.003, 0.6)) animated over 60 frames: every
    vertex moves by 0.01 sin(2 pi f / 60 + 7 x) along y and the whole PLOC BVH
    is rebuilt each frame; per frame 1920x1080 primary rays and 2 cosine
    bounce rays per hit are traced, and the hit predictor is retrained on the
    frame's exact hits (5%) and used for the bounce rays, which are traced in
    the order of their predicted treelets (CRT_TRACE_PREDICTOR_ORDER).  Frame =
    rebuild + primary + bounce generation + ordered bounce trace + training.
    Every 15 frames the same bounce rays are also traced plain, seeded and
    sorted without the network, off the frame clock.  The same 60 frames then
    run again with crt_refit of the frame-0 tree in place of the rebuild; the
    primary hits of every frame must equal the rebuild run's (watertight hits
    do not depend on the tree)."""
    from realtimeraytracing_gb300 import scenes as S
    n = 16 * 1024 * 1024
    gen = torch.Generator(device=dev)
    gen.manual_seed(4)
    base = S.device_soup(n, gen, clustered=True, clusters=1024, sigma=0.02, edge_mu=0.003, edge_sigma=0.6)
    x0 = base[:, [0, 4, 8]].clone()
    y0 = base[:, [1, 5, 9]].clone()
    tris = base.clone()
    models = torch.from_numpy(S.identity_models(1)).to(dev)
    cam = torch.from_numpy(S.camera_gpu_data((0.5, 0.5, -1.5), aspect=1920 / 1080)).to(dev)
    W, H = 1920, 1080
    hp = torch.empty((W * H, 4), dtype=torch.float32, device=dev)
    prim = torch.empty((W * H, 8), dtype=torch.float32, device=dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    primary_sums = {}

    def animate(refit):
        bvh = ctx.build(base, models=models)
        pred = crt.Predictor(ctx, bvh, seed=3)
        frame_ms, update_ms, sort_ms, prim_ms, compare, ordered_ms, rays_traced = [], [], [], [], [], [], []
        identical = True
        bounce = hb_plain = hb_seed = None
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        for f in range(frames):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            tris[:, [1, 5, 9]] = y0 + 0.01 * torch.sin(2 * np.pi * f / 60 + 7 * x0)
            if refit:
                stream.wait_stream(torch.cuda.current_stream(dev))  # the clock starts after the vertex update
                e[0].record(stream)
                bvh.refit(tris, models=models)
                e[1].record(stream)
            else:
                bvh.rebuild(tris, models=models)
                st = ctx.last_build_stats()
                sort_ms.append(st["ms_sort"])
                update_ms.append(st["ms_total"])
            pred.retarget()
            ctx.raygen(cam, W, H, out=prim)
            ts = time.perf_counter()
            ctx.trace(bvh, prim, crt.TRI_WATERTIGHT, out=hp)
            prim_ms.append((time.perf_counter() - ts) * 1e3)
            # order-independent digest of the frame's primary hits (ids and t bits)
            hv = hp.view(torch.int32).to(torch.int64)
            digest = int(((hv[:, 0] * 1000003 + hv[:, 1]) * (torch.arange(W * H, device=dev) + 1)).sum().item())
            if refit:
                identical = identical and primary_sums.get(f) == digest
            else:
                primary_sums[f] = digest
            n_hits = int((hp[:, 0].view(torch.int32) != -1).sum().item())
            nb = max(2 * n_hits, 1)
            if bounce is None or bounce.shape[0] < nb:
                bounce = torch.empty((nb, 8), dtype=torch.float32, device=dev)
                hb_plain = torch.empty((nb, 4), dtype=torch.float32, device=dev)
                hb_seed = torch.empty((nb, 4), dtype=torch.float32, device=dev)
            br, hs = bounce[:nb], hb_seed[:nb]
            ctx.bounce_rays(bvh, prim, hp, nb, seed=100 + f, out=br)
            ts = time.perf_counter()
            ctx.trace(bvh, br, crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER, out=hs)
            torch.cuda.synchronize()
            ordered_ms.append((time.perf_counter() - ts) * 1e3)
            pred.train(br, hs, offset=f % 20)   # retrain on this frame's exact hits
            torch.cuda.synchronize()
            frame_ms.append((time.perf_counter() - t0) * 1e3)
            if refit:
                update_ms.append(e[0].elapsed_time(e[1]))
            rays_traced.append(W * H + nb)
            if not refit and (f % 15 == 0 or f == frames - 1):
                # the same bounce rays plain, seeded and sorted without the network, off the frame clock
                row = {"rays": int(nb), "predictor_ordered_ms": round(ordered_ms[-1], 3)}
                for name, fl in (("plain_ms", 0), ("seeded_ms", crt.USE_PREDICTOR),
                                 ("sorted_no_network_ms", crt.SORT_RAYS)):
                    tp = time.perf_counter()
                    ctx.trace(bvh, br, crt.TRI_WATERTIGHT | fl, out=hb_plain[:nb])
                    torch.cuda.synchronize()
                    row[name] = round((time.perf_counter() - tp) * 1e3, 3)
                    identical = identical and bool(torch.equal(hb_plain[:nb].view(torch.int32), hs.view(torch.int32)))
                compare.append(row)
        pred.free()
        bvh.free()
        fm = np.array(frame_ms[1:])
        out = {
            "frame_ms_p50": round(float(np.percentile(fm, 50)), 3), "frame_ms_p99": round(float(np.percentile(fm, 99)), 3),
            ("refit_ms_p50" if refit else "build_ms_p50"): round(float(np.median(update_ms[1:])), 3),
            "primary_trace_ms_p50": round(float(np.median(prim_ms[1:])), 3),
            "primary_trace_ms_last": round(prim_ms[-1], 3),
            "mrays_s": round(float(sum(rays_traced[1:]) / fm.sum() / 1e3), 1),
            "identical_hits": identical,
        }
        if not refit:
            sort_bytes = 16.0 * n * 4 - 4.0 * n  # 4 passes x (8 B in + 8 B out); pass 0 synthesises values
            out["sort_ms_p50"] = round(float(np.median(sort_ms[1:])), 4)
            out["sort_gbs"] = round(sort_bytes / (float(np.median(sort_ms[1:])) * 1e-3) / 1e9, 1)
            out["bounce_trace_ms"] = compare
        return out

    rebuild = animate(refit=False)
    refit = animate(refit=True)
    return dict(rebuild, **{
        "workload": "16,777,216-tri clustered soup (1024 clusters), 60 animated frames, full rebuild per frame, "
                    "1920x1080 primary + 2 bounce rays per hit traced in predicted-treelet order, predictor retrained "
                    "per frame",
        "frames": frames,
        "refit": dict(refit, note="the same 60 frames with crt_refit of the frame-0 tree instead of a rebuild; "
                                  "identical_hits compares every frame's primary hits with the rebuild run's"),
    })


def run_predictor_experiment(ctx, torch, crt, dev, stream, args):
    """Learned hit predictor vs plain traversal on the incoherent-bounce
    workload: 4,194,304-triangle clustered soup (256 Gaussian clusters,
    sigma 0.02, edges lognormal(ln 0.003, 0.6)), 2048x2048 primary rays from
    (0.5, 0.5, -1.5) toward +z, 8,388,608 cosine-weighted bounce rays from
    their first hits.  The network trains online on every 20th traced ray
    (5%) for `passes` passes, then plain and seeded traversal are timed on
    the same rays; the hits must be identical."""
    from realtimeraytracing_gb300 import scenes as S
    tris, models = S.config3_scene(seed=0)
    d_tris = torch.from_numpy(tris).to(dev)
    bvh = ctx.build(d_tris, models=torch.from_numpy(models).to(dev))
    bst = ctx.last_build_stats()
    build_ms, scene_box = bst["ms_total"], bst["scene_box"]  # scene box = root box (no padding)
    del d_tris
    cam = torch.from_numpy(S.camera_gpu_data((0.5, 0.5, -1.5))).to(dev)
    w = 2048
    prim = torch.empty((w * w, 8), dtype=torch.float32, device=dev)
    ctx.raygen(cam, w, w, out=prim)
    ph = torch.empty((w * w, 4), dtype=torch.float32, device=dev)
    ctx.trace(bvh, prim, crt.TRI_WATERTIGHT, out=ph)
    n = 8 * 1024 * 1024
    rays = torch.empty((n, 8), dtype=torch.float32, device=dev)
    ctx.bounce_rays(bvh, prim, ph, n, seed=11, out=rays)
    del prim, ph
    plain = torch.empty((n, 4), dtype=torch.float32, device=dev)
    seeded = torch.empty_like(plain)
    cls = torch.empty((n,), dtype=torch.int16, device=dev)

    def timed(fn, reps):
        # every call, the warm-up included, on the library's stream: torch work
        # inside fn is then ordered with the library's kernels
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        with torch.cuda.stream(stream):
            fn()
            torch.cuda.synchronize()
            for a, b in evs:
                a.record(stream)
                fn()
                b.record(stream)
        torch.cuda.synchronize()
        return statistics.mean(a.elapsed_time(b) for a, b in evs)

    reps = max(3, min(args.steps, 10))
    t_plain = timed(lambda: ctx.trace(bvh, rays, crt.TRI_WATERTIGHT, out=plain), reps)
    ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.TRACE_STATS, out=plain)
    f_plain, _ = ctx.last_trace_stats()
    # the other node formats on the same incoherent rays (same hits)
    incoherent_formats = {}
    for fname, fflag in (("wide4_128B", crt.TRACE_WIDE), ("compressed4_64B", crt.TRACE_COMPRESSED)):
        t_f = timed(lambda: ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | fflag, out=seeded), reps)
        incoherent_formats[fname] = {"mrays_s": round(n / (t_f * 1e-3) / 1e6, 1), "vs_binary": round(t_plain / t_f, 3),
                                     "identical_hits": bool(torch.equal(seeded.view(torch.int32), plain.view(torch.int32)))}
    pred = crt.Predictor(ctx, bvh, seed=1, miss_threshold=0.9)
    truth = pred.classes_of_hits(plain)
    hit = truth != 127
    passes = 20
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = [pred.train(rays, plain, offset=k % 20) for k in range(passes)]
    train_ms = (time.perf_counter() - t0) * 1e3 / passes
    t_infer = timed(lambda: pred.infer(rays, out=cls), reps)
    t_seeded = timed(lambda: ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.USE_PREDICTOR, out=seeded), reps)
    ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.USE_PREDICTOR | crt.TRACE_STATS, out=seeded)
    f_seeded, _ = ctx.last_trace_stats()
    identical = bool(torch.equal(seeded.view(torch.int32), plain.view(torch.int32)))
    pc = cls.cpu().numpy().view(np.uint16)
    hit_rate = float((pc[hit] == truth[hit]).mean()) if hit.any() else 0.0
    tcls = torch.from_numpy(truth.astype(np.int16)).to(dev)
    t_perfect = timed(lambda: ctx.trace_seeded(bvh, rays, tcls, crt.TRI_WATERTIGHT, out=seeded), reps)
    ctx.trace_seeded(bvh, rays, tcls, crt.TRI_WATERTIGHT | crt.TRACE_STATS, out=seeded)
    f_perfect, _ = ctx.last_trace_stats()
    identical = identical and bool(torch.equal(seeded.view(torch.int32), plain.view(torch.int32)))
    # rays grouped by predicted treelet (inference + one radix pass + trace), alone and with seeding
    t_ordered = timed(lambda: ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER, out=seeded), reps)
    identical = identical and bool(torch.equal(seeded.view(torch.int32), plain.view(torch.int32)))
    ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER | crt.TRACE_STATS, out=seeded)
    f_ordered, _ = ctx.last_trace_stats()
    t_ord_seed = timed(lambda: ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER | crt.USE_PREDICTOR,
                                         out=seeded), reps)
    identical = identical and bool(torch.equal(seeded.view(torch.int32), plain.view(torch.int32)))
    # no network: rays sorted by the network's own input key (origin cell on the 64^3 grid of the scene
    # box, octahedral direction bin 32x32), gathered, traced; the sort + gather is timed apart
    key = ray_input_keys(torch, rays, scene_box)
    def key_sort():
        order = torch.argsort(key)
        return rays.index_select(0, order), order
    t_keysort = timed(key_sort, reps)
    with torch.cuda.stream(stream):
        srays, sorder = key_sort()
        sh = torch.empty_like(plain)
    torch.cuda.synchronize()
    t_keytrace = timed(lambda: ctx.trace(bvh, srays, crt.TRI_WATERTIGHT, out=sh), reps)
    t_native_sort = timed(lambda: ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.SORT_RAYS, out=seeded), reps)
    identical = identical and bool(torch.equal(seeded.view(torch.int32), plain.view(torch.int32)))
    keysort_identical = bool(torch.equal(sh.view(torch.int32), plain.index_select(0, sorder).view(torch.int32)))
    info = pred.info()
    pred.free()
    # the same rays over the treelet-restructured tree (crt_optimize, 2 passes; one call timed)
    nodes_before = bvh.nodes()
    oa, ob = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    oa.record(stream)
    bvh.optimize(2)
    ob.record(stream)
    torch.cuda.synchronize()
    t_optimize = oa.elapsed_time(ob)
    t_opt_trace = timed(lambda: ctx.trace(bvh, rays, crt.TRI_WATERTIGHT, out=seeded), reps)
    opt_identical = bool(torch.equal(seeded.view(torch.int32), plain.view(torch.int32)))
    ctx.trace(bvh, rays, crt.TRI_WATERTIGHT | crt.TRACE_STATS, out=seeded)
    f_opt, _ = ctx.last_trace_stats()
    sah_before, sah_after = sah_cost(nodes_before), sah_cost(bvh.nodes())
    bvh.free()
    return {
        "workload": "clustered soup 4,194,304 tris (256 clusters); 8,388,608 cosine bounce rays from 2048x2048 primary hits",
        "build_ms": round(build_ms, 3),
        "plain_mrays_s": round(n / t_plain / 1e3, 1),
        "node_formats": incoherent_formats,
        "seeded_mrays_s": round(n / t_seeded / 1e3, 1),
        "speedup": round(t_plain / t_seeded, 3),
        "infer_ms": round(t_infer, 3),
        "overhead_frac": round(t_infer / t_seeded, 3),
        "identical_hits": identical,
        "treelet_hit_rate": round(hit_rate, 4),
        "rays_hitting": round(float(hit.mean()), 4),
        "treelets": info["treelets"],
        "node_fetches_per_ray": {"plain": round(f_plain / n, 2), "seeded": round(f_seeded / n, 2),
                                 "perfect_prediction": round(f_perfect / n, 2)},
        "perfect_prediction_speedup": round(t_plain / t_perfect, 3),
        "predictor_ordered": {"mrays_s": round(n / t_ordered / 1e3, 1), "speedup": round(t_plain / t_ordered, 3),
                              "node_fetches_per_ray": round(f_ordered / n, 2),
                              "note": "CRT_TRACE_PREDICTOR_ORDER: inference + order by (predicted treelet, origin-cell Morton code, direction bin) + trace"},
        "predictor_ordered_seeded": {"mrays_s": round(n / t_ord_seed / 1e3, 1),
                                     "speedup": round(t_plain / t_ord_seed, 3)},
        "sorted_rays_no_network": {"mrays_s": round(n / t_native_sort / 1e3, 1),
                                   "speedup": round(t_plain / t_native_sort, 3),
                                   "note": "CRT_TRACE_SORT_RAYS: order by (origin-cell Morton code, direction bin) + trace"},
        "key_sorted_no_network": {"sort_gather_ms": round(t_keysort, 3), "trace_ms": round(t_keytrace, 3),
                                  "speedup_trace_only": round(t_plain / t_keytrace, 3),
                                  "speedup_with_sort": round(t_plain / (t_keysort + t_keytrace), 3),
                                  "identical_hits": keysort_identical},
        "treelet_optimized_tree": {"optimize_ms": round(t_optimize, 3), "passes": 2,
                                   "sah_cost": [round(sah_before, 2), round(sah_after, 2)],
                                   "mrays_s": round(n / t_opt_trace / 1e3, 1), "vs_built_tree": round(t_plain / t_opt_trace, 3),
                                   "node_fetches_per_ray": round(f_opt / n, 2), "identical_hits": opt_identical,
                                   "note": "crt_optimize: treelet restructuring of the built tree (SAH cost = sum of "
                                           "1.2 x internal + leaf box areas over the root area), then the plain trace"},
        "training": {"passes": passes, "adam_steps": info["steps"], "loss_first": round(losses[0], 4),
                     "loss_last": round(losses[-1], 4), "ms_per_pass": round(train_ms, 2),
                     "samples_per_pass": n // 20},
    }


def sah_cost(nodes, ci=1.2):
    """Surface-area cost of a node array as crt_optimize counts it (internal
    nodes ci x area, leaves 1 x area), relative to the root's area."""
    d = nodes[:, 4:7].astype(np.float64) - nodes[:, 0:3]
    a = 2.0 * (d[:, 0] * d[:, 1] + d[:, 1] * d[:, 2] + d[:, 2] * d[:, 0])
    u = np.ascontiguousarray(nodes).view(np.uint32)
    leaf = (u[:, 9] == 0) & (u[:, 10] == 0)
    return float((np.where(leaf, 1.0, ci) * a).sum() / a[0])


def ray_input_keys(torch, rays, box):
    """The predictor's input key of each ray without the network: origin cell
    on the 64^3 grid of the scene box (min xyz, max xyz; x-major) * 1024 +
    octahedral direction bin on 32x32, as int64 (the quantisation the
    network's embeddings use)."""
    mn = torch.tensor(list(box[0:3]), dtype=torch.float32, device=rays.device)
    mx = torch.tensor(list(box[3:6]), dtype=torch.float32, device=rays.device)
    ext = torch.clamp(mx - mn, min=1e-20)
    c = torch.clamp(((rays[:, 0:3] - mn) * (64.0 / ext)).floor().long(), 0, 63)
    cell = (c[:, 0] * 64 + c[:, 1]) * 64 + c[:, 2]
    d = rays[:, 4:7]
    a = d.abs().sum(dim=1).clamp(min=1e-30)
    px, py = d[:, 0] / a, d[:, 1] / a
    neg = d[:, 2] < 0
    qx = (1 - py.abs()) * torch.where(px >= 0, 1.0, -1.0)
    qy = (1 - px.abs()) * torch.where(py >= 0, 1.0, -1.0)
    px, py = torch.where(neg, qx, px), torch.where(neg, qy, py)
    bu = torch.clamp(((px + 1) * 16).long(), 0, 31)
    bv = torch.clamp(((py + 1) * 16).long(), 0, 31)
    return cell * 1024 + bu * 32 + bv


def cpu_baseline(tris, models, cam, sample_stride=8):
    """The reference's CPU path on the host cores: the shader traversal
    restated in C++ (oracle), every `sample_stride`-th ray of the frame."""
    from oracle import oracle as O
    n = tris.shape[0]
    nb = O.build_bvh(tris, n, models, faithful=True)
    rays = O.raygen(cam, W, H)[::sample_stride].copy()
    O.trace(nb["nodes"], tris, models, rays[:4096], 0)
    t0 = time.perf_counter()
    reps = 0
    while True:
        hits, _ = O.trace(nb["nodes"], tris, models, rays, 0)
        reps += 1
        if time.perf_counter() - t0 > 2.0:
            break
    dt = (time.perf_counter() - t0) / reps
    cores = os.cpu_count()
    return {"value": round(rays.shape[0] / dt / 1e6, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
            "sample": f"every {sample_stride}th primary ray of the 1920x1080 frame ({rays.shape[0]} rays), "
                      f"shader predicate, no t pruning; shadow rays: none (the shader predicate hits nothing "
                      f"on this mesh)",
            "build_ms": round(float(sum(nb["ms"])), 2)}


# --------------------------------------------------------- reference arm
def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    tris, models, cam, light = make_scene()
    n = tris.shape[0]
    t0 = time.perf_counter()
    nb = O.build_bvh(tris, n, models, faithful=True)
    build_ms = (time.perf_counter() - t0) * 1e3
    rays_all = O.raygen(cam, W, H)
    stride = 8
    times, counted = [], []
    for k in range(args.warmup + args.steps):
        sub = rays_all[(k % stride)::stride].copy()
        t0 = time.perf_counter()
        hits, _ = O.trace(nb["nodes"], tris, models, sub, 0)
        nh = int((hits[:, 0].view(np.uint32) != 0xFFFFFFFF).sum())
        if nh:
            sh = O.shadow_rays(sub, hits, light)
            O.trace(nb["nodes"], tris, models, sh, 1)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
            counted.append(sub.shape[0] + nh)
    value = sum(counted) / sum(times) / 1e6
    cores = os.cpu_count()
    line = {
        "metric": METRIC, "impl": "reference", "value": round(value, 4), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * statistics.mean(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded displaced icosphere)",
        "config": {"workload": WORKLOAD, "triangles": n, "image": [W, H], "sample": f"1/{stride} of the frame per step"},
        "build_ms": round(build_ms, 2),
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": f"every {stride}th primary ray per step (rotating offset), shader predicate, "
                                   f"right-child-first DFS without t pruning; shadow rays for its hits"},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-predictor", action="store_true", help="skip the learned-predictor (4M-triangle) experiment")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched experiment")
    ap.add_argument("--no-dynamic", action="store_true", help="skip the 16M-triangle 60-frame dynamic experiment")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
