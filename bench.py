#!/usr/bin/env python
"""Throughput benchmark of the GB300 ray-tracing core.

Headline workload (the hit-predictor metric's own scene): one "step" traces
a batch of incoherent rays with the learned hit predictor.
  scene   4,194,304-triangle clustered soup (256 Gaussian clusters, sigma
          0.02, edges lognormal(ln 0.003, 0.6)), seeded synthetic data, BVH
          built by the CUDA PLOC path (build ms reported apart)
  rays    8,388,608 cosine-weighted diffuse bounce rays from the closest hits
          of 2048x2048 primary rays from (0.5, 0.5, -1.5) toward +z, made on
          the host from the seed (scenes.bounce_rays: IEEE-exact float64
          arithmetic, so every run and both arms get the same bytes)
  step    crt_trace with CRT_TRACE_PREDICTOR_ORDER: predictor inference (FP16
          MLP on tcgen05, trained online on the tracer's own hits), rays
          ordered by (predicted treelet, origin cell, direction bin), closest
          hit with the watertight predicate; the hits must equal the plain
          traversal's bit for bit
  value   rays per second of that step, Mrays/s, rays resident in HBM, L2
          flushed before each step, CUDA events on the library's stream
  e2e     the same step through the public C ABI call crt_trace with the
          rays in page-locked host memory and the hits written back to it,
          host-timed around the call
The plain traversal (rays in caller order), the no-network ordering
(CRT_TRACE_SORT_RAYS) and the other learned modes are timed beside it on
the same rays.  The 1,310,720-triangle icosphere frame (primary + shadow
rays, one launch), the 65,536-triangle soup under the shader's own triangle
predicate, the 64-scene batch and the 16M-triangle animation are reported as
extra keys.

--impl reference times the reference's CPU path on the host cores instead,
on the same rays: the shader's traversal (raytracer.glsl:246-295: DFS, right
child popped first, every box the ray crosses entered, no t pruning) restated
in C++ with the watertight triangle predicate the GPU arm uses, over the same
BVH (its PLOC build restated from bvh.cpp), on a bounded rotating 1/64
sample of the rays per step.  Both arms print a digest of the rays and of the
hits on that sample, which must agree.

Multi-GPU: replicas (each rank traces its own copy of the batch); value is
the total over ranks divided by the slowest rank's time (weak scaling).
"""
from __future__ import annotations

import argparse
import hashlib
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
WORKLOAD = ("clustered soup 4,194,304 tris (256 clusters); 8,388,608 cosine bounce rays from the closest hits of "
            "2048x2048 primary rays; closest hit (watertight)")
N_BOUNCE = 8 * 1024 * 1024   # --rays: smaller copies of the batch for profilers
BOUNCE_SEED = 11
REF_STRIDE = 64        # the reference arm traces rays k % 64, k % 64 + 64, ... in step k
TRI_WATERTIGHT = 0x2   # crt.h flags, also understood by the oracle
PROFILE = "trace_pool_kernel_bounce_config3.md"  # ncu summary of the headline's dominant kernel
TRI_REFERENCE = 0x0
W1, H1 = 1920, 1080    # the icosphere frame


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_profile_value(name, key):
    """A number from a committed ncu summary (a line 'key: value ...')."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith(key + ":"):
                    return float(line.split(":", 1)[1].split()[0])
    except (OSError, ValueError):
        pass
    return None


def digest(a) -> str:
    """Short SHA-256 of an array's bytes."""
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def ref_sample(k: int, n: int) -> np.ndarray:
    """Indices of the rays the reference arm traces in step k."""
    return np.arange(k % REF_STRIDE, n, REF_STRIDE)


def edge_hits(hits) -> int:
    """Closest hits within about one float ulp of a triangle edge: a
    barycentric coordinate (u, v or 1 - u - v) below 2^-22.  Such rays may
    take either neighbour of a shared edge; both predicates report them."""
    u32 = np.ascontiguousarray(hits).view(np.uint32)
    hit = u32[:, 0] != 0xFFFFFFFF
    u, v = hits[hit, 2].astype(np.float64), hits[hit, 3].astype(np.float64)
    w = 1.0 - u - v
    return int((np.minimum(np.minimum(u, v), w) < 2.0 ** -22).sum())


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


def headline_config():
    """The workload description both arms put in `config`."""
    wl = WORKLOAD if N_BOUNCE == 8 * 1024 * 1024 else WORKLOAD.replace("8,388,608", f"{N_BOUNCE:,}")
    return {"workload": wl, "triangles": 4194304, "rays_per_step": N_BOUNCE, "predicate": "watertight",
            "rays": "host-generated from seed 11 (scenes.bounce_rays), identical bytes in both arms",
            "l2": "rays, nodes and triangles (1.2 GB) exceed L2; a 256 MB buffer is also written before every timed step",
            "parallelism": "single GPU"}


def config3_inputs(primary_hits_fn):
    """(triangles, models, bounce rays) of the headline workload; the primary
    hits come from primary_hits_fn(rays) (the GPU in the product arm, the
    CPU oracle in the reference arm: the same hits bit for bit)."""
    from realtimeraytracing_gb300 import scenes as S
    tris, models = S.config3_scene(seed=0)
    _, _, rays = S.config3_rays(tris, models, primary_hits_fn, seed=BOUNCE_SEED, n_out=N_BOUNCE)
    return tris, models, rays


# --------------------------------------------------------------- our arm
def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from realtimeraytracing_gb300 import crt

    dev = torch.device("cuda", local)
    ctx = crt.Context(device=local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    WT = crt.TRI_WATERTIGHT

    # ---- scene, BVH build (scene load; device-timed inside the library)
    from realtimeraytracing_gb300 import scenes as S
    tris, models = S.config3_scene(seed=0)
    n_tris = tris.shape[0]
    d_tris = torch.from_numpy(tris).to(dev)
    d_models = torch.from_numpy(models).to(dev)
    bvh = ctx.build(d_tris, models=d_models)
    builds = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        bvh.rebuild(d_tris, models=d_models)
        wall = (time.perf_counter() - t0) * 1e3
        if i >= args.warmup:
            builds.append((ctx.last_build_stats(), wall))
    build_ms = statistics.median(b[0]["ms_total"] for b in builds)
    stages = {k: round(statistics.median(b[0][k] for b in builds), 4)
              for k in ("ms_morton", "ms_sort", "ms_ploc", "ms_layout")}

    # ---- the rays: primary hits on the GPU, bounce rays on the host
    def primary_hits(prim):
        dp = torch.from_numpy(prim).to(dev)
        h = torch.empty((prim.shape[0], 4), dtype=torch.float32, device=dev)
        ctx.trace(bvh, dp, WT, out=h)
        torch.cuda.synchronize()
        return h.cpu().numpy()

    _, _, rays_h = S.config3_rays(tris, models, primary_hits, seed=BOUNCE_SEED, n_out=N_BOUNCE)
    n = N_BOUNCE
    d_rays = torch.from_numpy(rays_h).to(dev)
    plain = torch.empty((n, 4), dtype=torch.float32, device=dev)
    out = torch.empty_like(plain)
    ctx.trace(bvh, d_rays, WT, out=plain)
    torch.cuda.synchronize()

    # ---- the learned part: trained online on the tracer's own exact hits
    # (every 20th ray = 5% per pass, rotating offset), then deployed
    pred = crt.Predictor(ctx, bvh, seed=1, miss_threshold=0.9)
    passes = 20
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = [pred.train(d_rays, plain, offset=k % 20) for k in range(passes)]
    torch.cuda.synchronize()
    train_ms = (time.perf_counter() - t0) * 1e3 / passes
    LEARNED = WT | crt.PREDICTOR_ORDER

    def run_steps(flags, steps, warmup, hits_out):
        for _ in range(warmup):
            ctx.trace(bvh, d_rays, flags, out=hits_out)
        torch.cuda.synchronize()
        evs, kern = [], []
        with torch.cuda.stream(stream):
            for _ in range(steps):
                l2_flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ctx.trace(bvh, d_rays, flags, out=hits_out)
                b.record(stream)
                kern.append(ctx.last_trace_timing())
                evs.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs], kern

    def same(h):
        return bool(torch.equal(h.view(torch.int32), plain.view(torch.int32)))

    # ---- timed steps of the headline (learned) mode
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms, kern = run_steps(LEARNED, args.steps, args.warmup, out)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_step = slowest_ms(statistics.mean(step_ms), world, dev)
    value = whole_job_mrays(world, n, t_step)
    identical = same(out)

    # ---- the same rays plain, sorted without the network, seeded
    reps = max(3, min(args.steps, 10))
    t_plain = statistics.mean(run_steps(WT, reps, 2, out)[0])
    identical = identical and same(out)
    t_per_ray = statistics.mean(run_steps(WT | crt.PER_RAY_THREADS, reps, 2, out)[0])
    identical = identical and same(out)
    t_sorted = statistics.mean(run_steps(WT | crt.SORT_RAYS, reps, 2, out)[0])
    identical = identical and same(out)
    t_seeded = statistics.mean(run_steps(WT | crt.USE_PREDICTOR, reps, 2, out)[0])
    identical = identical and same(out)
    # online training inside the step: trace + one 5% training pass
    ev_t = []
    with torch.cuda.stream(stream):
        for k in range(reps):
            l2_flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.trace(bvh, d_rays, LEARNED, out=out)
            pred.train(d_rays, out, offset=k % 20)
            b.record(stream)
            ev_t.append((a, b))
    torch.cuda.synchronize()
    t_online = statistics.mean(a.elapsed_time(b) for a, b in ev_t)
    identical = identical and same(out)

    # node fetches and triangle tests per ray
    ctx.trace(bvh, d_rays, WT | crt.TRACE_STATS, out=out)
    f_plain, tt_plain = ctx.last_trace_stats()
    ctx.trace(bvh, d_rays, LEARNED | crt.TRACE_STATS, out=out)
    f_learned, tt_learned = ctx.last_trace_stats()
    # prediction quality: treelet hit rate on hitting rays
    cls = torch.empty((n,), dtype=torch.int16, device=dev)
    pred.infer(d_rays, out=cls)
    truth = pred.classes_of_hits(plain)
    pc = cls.cpu().numpy().view(np.uint16)
    hit = truth != 127
    hit_rate = float((pc[hit] == truth[hit]).mean()) if hit.any() else 0.0

    # ---- the dominant kernel (trace_pool_kernel in the learned step), timed
    # by the library's CUDA events on its stream around that launch
    k_ms = statistics.mean(k[1] for k in kern)
    order_ms = statistics.mean(k[0] for k in kern)
    alg_bytes = 64.0 * f_learned + 48.0 * tt_learned + (32.0 + 16.0 + 4.0) * n  # nodes, triangles, ray, hit, order
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (k_ms * 1e-3) / 1e9
    traffic = read_profile_value(PROFILE, "traffic_bytes_per_launch")

    # ---- end to end through the public API: host rays in, host hits out
    rays_pin = torch.from_numpy(rays_h).pin_memory()
    hits_pin = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
    for _ in range(2):
        ctx.trace(bvh, rays_pin, LEARNED, out=hits_pin)
    e2e_ms = []
    for _ in range(args.steps):
        l2_flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.trace(bvh, rays_pin, LEARNED, out=hits_pin)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_t = slowest_ms(statistics.mean(e2e_ms), world, dev)
    e2e_value = whole_job_mrays(world, n, e2e_t)
    plain_h = plain.cpu().numpy()
    identical = identical and bool(np.array_equal(hits_pin.numpy().view(np.uint32), plain_h.view(np.uint32)))

    # the hits on the reference arm's timed samples, for comparison with its digest
    ref_hits = np.concatenate([plain_h[ref_sample(k, n)] for k in range(args.warmup, args.warmup + args.steps)])
    nodes_h = bvh.nodes()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(nodes_h, tris, models, rays_h, plain_h)
    del rays_pin, hits_pin
    extras = {}
    if rank == 0 and not args.no_extras:
        extras["treelet_optimized_tree"] = optimized_tree_experiment(ctx, torch, crt, bvh, d_rays, plain, out,
                                                                     run_steps, t_plain)
    pred.free()
    bvh.free()
    del d_tris, d_rays, plain, out, cls
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_extras:
        extras["config0_shader_predicate"] = run_config0(ctx, torch, crt, dev, stream, args)
        extras["frame"] = run_frame_experiment(ctx, torch, crt, dev, stream, l2_flush, args)
    if rank == 0 and not args.no_batch:
        extras["batch"] = run_batch_experiment(ctx, torch, crt, dev, args)
    if rank == 0 and not args.no_dynamic:
        extras["dynamic"] = run_dynamic_experiment(ctx, torch, crt, dev, args)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": round(value, 2),
            "unit": "Mrays/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(t_step, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded clustered soup and host-generated bounce rays)",
            "config": headline_config(),
            "learned_vs_plain": {
                "learned_mrays_s": round(value / world, 2), "plain_mrays_s": round(n / t_plain / 1e3, 2),
                "speedup": round(t_plain / t_step, 3), "identical_hits": identical,
                "plain_one_thread_per_ray_mrays_s": round(n / t_per_ray / 1e3, 2),
                "no_network_sorted_mrays_s": round(n / t_sorted / 1e3, 2),
                "no_network_speedup": round(t_plain / t_sorted, 3),
                "learned_vs_no_network": round(t_sorted / t_step, 3),
                "seeded_tmax_mrays_s": round(n / t_seeded / 1e3, 2), "seeded_speedup": round(t_plain / t_seeded, 3),
                "with_online_training_mrays_s": round(n / t_online / 1e3, 2),
                "with_online_training_speedup": round(t_plain / t_online, 3),
                "ordering_ms": round(order_ms, 4), "trace_kernel_ms": round(k_ms, 4),
                "node_fetches_per_ray": {"plain": round(f_plain / n, 2), "learned": round(f_learned / n, 2)},
                "tris_per_ray": {"plain": round(tt_plain / n, 2), "learned": round(tt_learned / n, 2)},
                "treelet_hit_rate": round(hit_rate, 4), "rays_hitting": round(float(hit.mean()), 4),
                "training": {"passes": passes, "loss_first": round(losses[0], 4), "loss_last": round(losses[-1], 4),
                             "ms_per_pass": round(train_ms, 3), "samples_per_pass": n // 20},
                "modes": "learned = CRT_TRACE_PREDICTOR_ORDER (inference + order by the likeliest class, origin "
                         "cell, direction bin + trace); no network = CRT_TRACE_SORT_RAYS (order by origin cell and "
                         "direction bin + trace); seeded = CRT_TRACE_USE_PREDICTOR (t_max from an exact search of "
                         "the predicted treelet); plain and ordered modes trace on persistent warps that refill "
                         "finished lanes, one_thread_per_ray = CRT_TRACE_PER_RAY_THREADS (the launch-per-ray kernel)"},
            "build_ms": round(build_ms, 4),
            "build_ms_wall": round(statistics.median(b[1] for b in builds), 4),
            "build_stages_ms": stages,
            "ploc_iterations": builds[-1][0]["ploc_iterations"],
            "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s", "h2d_bytes_per_step": int(n * 32),
                    "d2h_bytes_per_step": int(n * 16), "ms_per_step": round(e2e_t, 4),
                    "transfer": "crt_trace on page-locked host rays (read across the CPU-GPU link by the inference "
                                "kernel, which stores the device copy the trace reads) and host hits (written by the "
                                "trace kernel over the link), host-timed around the call"},
            "gpu_launches": 6 * args.steps,
            "gpu_launches_note": "per step: infer_kernel (which also writes the order keys and their digit histograms), "
                                 "4 onesweep_kernel passes, trace_pool_kernel",
            "roofline": {"kernel": "trace_pool_kernel (learned step: persistent warps over the rays in predicted "
                                   "order, closest hit, watertight)",
                         "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                         "ms_per_launch": round(k_ms, 4), "alg_bytes_per_launch": int(alg_bytes),
                         "alg_bytes_model": "64 B per node fetched + 48 B per triangle tested + 32 B ray + 16 B hit "
                                            "+ 4 B order index per ray (fetched bytes; most are L1/L2 hits)",
                         "l2_and_issue": {
                             "lts_throughput_pct": read_profile_value(PROFILE, "lts_throughput_pct"),
                             "issue_active_pct": read_profile_value(PROFILE, "issue_active_pct"),
                             "threads_per_instruction": read_profile_value(PROFILE, "threads_per_instruction"),
                             "source": "ncu full set of this kernel on a 1,048,576-ray copy of the workload "
                                       "(profiles/" + PROFILE + "); the walk is latency-bound, DRAM traffic is "
                                       "the 'traffic' bytes"}},
            "rays_sha256": digest(rays_h),
            "reference_sample_hits_sha256": digest(ref_hits),
            "reference_sample_hits": int((ref_hits[:, 0].view(np.uint32) != 0xFFFFFFFF).sum()),
            "edge_hits": edge_hits(plain_h),
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        line.update(extras)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def optimized_tree_experiment(ctx, torch, crt, bvh, d_rays, plain, out, run_steps, t_plain):
    """The same rays over the treelet-restructured tree (crt_optimize, 2
    passes; the build's tree is replaced)."""
    n = d_rays.shape[0]
    nodes_before = bvh.nodes()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bvh.optimize(2)
    torch.cuda.synchronize()
    t_opt = (time.perf_counter() - t0) * 1e3
    t_tr = statistics.mean(run_steps(crt.TRI_WATERTIGHT, 5, 1, out)[0])
    ident = bool(torch.equal(out.view(torch.int32), plain.view(torch.int32)))
    return {"optimize_ms_wall": round(t_opt, 2), "passes": 2,
            "sah_cost": [round(sah_cost(nodes_before), 2), round(sah_cost(bvh.nodes()), 2)],
            "plain_mrays_s": round(n / t_tr / 1e3, 1), "vs_built_tree": round(t_plain / t_tr, 3),
            "identical_hits": ident}


def run_config0(ctx, torch, crt, dev, stream, args):
    """The 65,536-triangle soup (512x512 primary rays) under the shader's own
    triangle predicate (raytracer.glsl:102-147), the one scene of the set
    where that predicate finds hits: GPU and CPU oracle on the same rays,
    and how the watertight predicate differs on them."""
    from oracle import oracle as O
    from realtimeraytracing_gb300 import scenes as S
    tris, models, cam, (w, h) = S.config0_scene(seed=0)
    bvh = ctx.build(tris, models=models)
    rays = S.pinhole_rays(cam, w, h)
    d_rays = torch.from_numpy(rays).to(dev)
    out = torch.empty((rays.shape[0], 4), dtype=torch.float32, device=dev)
    res = {}
    for name, fl in (("reference", crt.TRI_REFERENCE), ("watertight", crt.TRI_WATERTIGHT)):
        for _ in range(3):
            ctx.trace(bvh, d_rays, fl, out=out)
        torch.cuda.synchronize()
        evs = []
        with torch.cuda.stream(stream):
            for _ in range(10):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ctx.trace(bvh, d_rays, fl, out=out)
                b.record(stream)
                evs.append((a, b))
        torch.cuda.synchronize()
        ms = statistics.mean(a.elapsed_time(b) for a, b in evs)
        res[name] = (out.cpu().numpy(), ms)
    gh, g_ms = res["reference"]
    wh, w_ms = res["watertight"]
    nodes = bvh.nodes()
    bvh.free()
    t0 = time.perf_counter()
    oh, _ = O.trace(nodes, tris, models, rays, TRI_REFERENCE)
    o_ms = (time.perf_counter() - t0) * 1e3
    gt, wt = gh[:, 0].view(np.uint32), wh[:, 0].view(np.uint32)
    both = (gt != 0xFFFFFFFF) & (wt != 0xFFFFFFFF)
    return {
        "workload": "uniform soup 65,536 tris, 512x512 primary rays from (0.5, 0.5, -1.5), closest hit",
        "gpu_reference_predicate_mrays_s": round(rays.shape[0] / g_ms / 1e3, 1),
        "gpu_watertight_mrays_s": round(rays.shape[0] / w_ms / 1e3, 1),
        "cpu_reference_predicate_mrays_s": round(rays.shape[0] / o_ms / 1e3, 3),
        "cpu_cores": os.cpu_count(),
        "hits": int((gt != 0xFFFFFFFF).sum()),
        "gpu_equals_cpu": bool(np.array_equal(gh.view(np.uint32), oh.view(np.uint32))),
        "hits_sha256": digest(gh),
        "predicates_disagree": {"rays": int((gt != wt).sum()), "hit_by_reference_only": int(((gt != 0xFFFFFFFF) & (wt == 0xFFFFFFFF)).sum()),
                                "hit_by_watertight_only": int(((gt == 0xFFFFFFFF) & (wt != 0xFFFFFFFF)).sum()),
                                "different_triangle": int((both & (gt != wt)).sum())},
        "edge_hits": {"reference": edge_hits(gh), "watertight": edge_hits(wh)},
        "note": "reference = CRT_TRI_REFERENCE (|a| < 1e-4 rejected, back faces culled); the shader's predicate "
                "rejects every triangle of the larger scenes (their |a| is below 1e-4)",
    }


def run_frame_experiment(ctx, torch, crt, dev, stream, l2_flush, args):
    """The 1,310,720-triangle displaced icosphere: 1920x1080 primary rays,
    closest hit, one any-hit shadow ray per hit toward (2, 2, -2), one
    frame_kernel launch (crt_trace_frame); plus the shaded frame, mesh upload
    and a tree imported from its node array."""
    from realtimeraytracing_gb300 import scenes as S
    tris, models, cam, (w, h), light = S.config1_scene(seed=0)
    d_tris = torch.from_numpy(tris).to(dev)
    d_models = torch.from_numpy(models).to(dev)
    d_cam = torch.from_numpy(cam).to(dev)
    bvh = ctx.build(d_tris, models=d_models)
    builds = []
    for i in range(args.warmup + args.steps):
        bvh.rebuild(d_tris, models=d_models)
        if i >= args.warmup:
            builds.append(ctx.last_build_stats())
    n_rays = w * h
    hp = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
    hs = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
    flags = crt.TRI_WATERTIGHT

    def frame():
        ctx.trace_frame(bvh, d_cam, w, h, light, flags, hits_primary=hp, hits_shadow=hs)

    def timed(fn, steps):
        evs = []
        with torch.cuda.stream(stream):
            for _ in range(steps):
                l2_flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                evs.append((a, b))
        torch.cuda.synchronize()
        return statistics.mean(a.elapsed_time(b) for a, b in evs)

    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    n_hits = int((hp[:, 0].view(torch.int32) != -1).sum().item())
    rays_per_frame = n_rays + n_hits
    f_ms = timed(frame, args.steps)
    ctx.trace_frame(bvh, d_cam, w, h, light, flags | crt.TRACE_STATS, hits_primary=hp, hits_shadow=hs)
    visited, tested = ctx.last_trace_stats()
    alg_bytes = 64.0 * visited + 48.0 * tested + 2 * 16.0 * n_rays
    # the primary trace alone over the three node formats (same hits)
    rays = torch.empty((n_rays, 8), dtype=torch.float32, device=dev)
    ctx.raygen(d_cam, w, h, out=rays)
    ctx.trace(bvh, rays, flags, out=hp)
    formats = {}
    hp_alt = torch.empty_like(hp)
    for fname, fflag in (("binary_64B", 0), ("wide4_128B", crt.TRACE_WIDE), ("compressed4_64B", crt.TRACE_COMPRESSED)):
        ctx.trace(bvh, rays, flags | fflag | crt.TRACE_STATS, out=hp_alt)
        fv, _ = ctx.last_trace_stats()
        ms = timed(lambda: ctx.trace(bvh, rays, flags | fflag, out=hp_alt), args.steps)
        formats[fname] = {"ms": round(ms, 4), "node_fetches_per_ray": round(fv / n_rays, 2),
                          "identical_hits": bool(torch.equal(hp_alt.view(torch.int32), hp.view(torch.int32)))}
    # mesh upload: the indexed icosphere to TriangleGPU records on the GPU
    mv, mf = S.displaced_icosphere(8, 0.05, 0)
    d_mv = torch.from_numpy(np.ascontiguousarray(mv, np.float32)).to(dev)
    d_mf = torch.from_numpy(np.ascontiguousarray(mf, np.uint32).view(np.int32)).to(dev)
    d_mt = torch.empty((mf.shape[0], 16), dtype=torch.float32, device=dev)
    ctx.triangles_from_indexed(d_mv, d_mf, 0, out=d_mt)
    m_ms = timed(lambda: ctx.triangles_from_indexed(d_mv, d_mf, 0, out=d_mt), args.steps)
    mesh = {"triangles": int(mf.shape[0]), "ms": round(m_ms, 4),
            "gbs": round((12 + 36 + 64) * mf.shape[0] / (m_ms * 1e-3) / 1e9, 1),
            "identical_to_scene_records": bool(torch.equal(d_mt.cpu(), torch.from_numpy(tris)))}
    del d_mv, d_mf, d_mt
    # the trace side alone over a node array built elsewhere (host memory)
    frame()
    nodes_h = bvh.nodes()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    imp = ctx.bvh_from_nodes(nodes_h, tris, models=models)
    import_ms = (time.perf_counter() - t0) * 1e3
    hp_i, hs_i = torch.empty_like(hp), torch.empty_like(hs)
    i_ms = timed(lambda: ctx.trace_frame(imp, d_cam, w, h, light, flags, hits_primary=hp_i, hits_shadow=hs_i),
                 args.steps)
    imported = {"import_ms": round(import_ms, 3), "frame_ms": round(i_ms, 4),
                "identical_hits": bool(torch.equal(hp_i.view(torch.int32), hp.view(torch.int32)) and
                                       torch.equal(hs_i[:, 0].view(torch.int32) == -1, hs[:, 0].view(torch.int32) == -1))}
    imp.free()
    # the reference's whole compute pass into a device RGBA32F image
    img = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
    d_mats = torch.tensor([[0.8, 0.7, 0.6, 1.0]], dtype=torch.float32, device=dev)
    shaded = {}
    for name, sflags, depth in (("plain", 0, 0), ("wireframe_bvh_depth3", crt.SHADE_WIREFRAME | crt.SHADE_BVH, 3)):
        def render():
            ctx.render_frame(bvh, d_cam, w, h, models=d_models, materials=d_mats, shade_flags=sflags,
                             bvh_depth=depth, flags=flags, out=img)
        render()
        s_ms = timed(render, args.steps)
        shaded[name] = {"ms": round(s_ms, 4), "mrays_s": round(n_rays / (s_ms * 1e-3) / 1e6, 1)}
    # end to end: camera in, both hit buffers out to page-locked host memory
    hp_h = torch.empty((n_rays, 4), dtype=torch.float32, pin_memory=True)
    hs_h = torch.empty((n_rays, 4), dtype=torch.float32, pin_memory=True)
    cam_h = torch.from_numpy(cam.copy()).pin_memory()
    for _ in range(2):
        ctx.trace_frame(bvh, cam_h, w, h, light, flags, hits_primary=hp_h, hits_shadow=hs_h)
    e2e = []
    for _ in range(args.steps):
        l2_flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.trace_frame(bvh, cam_h, w, h, light, flags, hits_primary=hp_h, hits_shadow=hs_h)
        e2e.append((time.perf_counter() - t0) * 1e3)
    bvh.free()
    return {
        "workload": "displaced icosphere 1,310,720 tris; 1920x1080 primary closest-hit + shadow any-hit to (2,2,-2)",
        "rays_per_frame": rays_per_frame, "primary_hits": n_hits,
        "frame_ms": round(f_ms, 4), "mrays_s": round(rays_per_frame / (f_ms * 1e-3) / 1e6, 2),
        "e2e_mrays_s": round(rays_per_frame / (statistics.mean(e2e) * 1e-3) / 1e6, 2),
        "build_ms": round(statistics.median(b["ms_total"] for b in builds), 4),
        "build_stages_ms": {k: round(statistics.median(b[k] for b in builds), 4)
                            for k in ("ms_morton", "ms_sort", "ms_ploc", "ms_layout")},
        "ploc_iterations": builds[-1]["ploc_iterations"],
        "frame_kernel": {"fetched_bytes_gbs": round(alg_bytes / (f_ms * 1e-3) / 1e9, 1),
                         "node_fetches_per_pixel": round(visited / n_rays, 2),
                         "tris_per_pixel": round(tested / n_rays, 2),
                         "dram_bytes_per_launch": read_profile_value("frame_kernel_config1.md",
                                                                     "traffic_bytes_per_launch")},
        "primary_trace_node_formats": formats,
        "mesh_upload": mesh,
        "imported_tree": imported,
        "shaded_frame": shaded,
    }


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

    def animate_batch(learned):
        """The same frames on the batched persistent graph: a one-scene
        crt_batch with room for 2 bounce rays per pixel.  Per frame the
        batch's CUDA graph replays the rebuild (batched Morton, sort, PLOC and
        layout launches) and the primary trace; crt_batch_bounce_rays makes
        the bounce rays, crt_batch_set_ray_counts switches the batch to them,
        and crt_batch_trace traces them, in predicted-treelet order with the
        predictor retrained on the frame's hits (learned) or plain."""
        b = crt.Batch(ctx, [n], [2 * W * H], models=S.identity_models(1))
        bounce = torch.empty((2 * W * H, 8), dtype=torch.float32, device=dev)
        hb = torch.empty((2 * W * H, 4), dtype=torch.float32, device=dev)
        hb_cmp = torch.empty((2 * W * H, 4), dtype=torch.float32, device=dev)
        ctx.raygen(cam, W, H, out=prim)
        tris.copy_(base)
        b.set_ray_counts([W * H])
        b.run(tris, prim, hp, crt.TRI_WATERTIGHT, graph=True)
        pred = crt.Predictor(ctx, b, seed=3) if learned else None
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        frame_ms, run_ms, bounce_ms, rays_traced, compare = [], [], [], [], []
        identical, graph_frames = True, 0
        for f in range(frames):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            tris[:, [1, 5, 9]] = y0 + 0.01 * torch.sin(2 * np.pi * f / 60 + 7 * x0)
            b.set_ray_counts([W * H])
            stream.wait_stream(torch.cuda.current_stream(dev))
            e[0].record(stream)
            graph_frames += int(b.run(tris, prim, hp, crt.TRI_WATERTIGHT, graph=True))
            e[1].record(stream)
            hv = hp.view(torch.int32).to(torch.int64)
            digest = int(((hv[:, 0] * 1000003 + hv[:, 1]) * (torch.arange(W * H, device=dev) + 1)).sum().item())
            identical = identical and primary_sums.get(f) == digest
            n_hits = int((hp[:, 0].view(torch.int32) != -1).sum().item())
            nb = max(2 * n_hits, 1)
            br, hs = bounce[:nb], hb[:nb]
            b.bounce_rays(0, prim, hp, nb, seed=100 + f, out=br)
            b.set_ray_counts([nb])
            ts = time.perf_counter()
            if learned:
                pred.retarget()
                b.trace(br, hs, crt.TRI_WATERTIGHT | crt.PREDICTOR_ORDER)
                torch.cuda.synchronize()
                bounce_ms.append((time.perf_counter() - ts) * 1e3)
                pred.train(br, hs, offset=f % 20)
            else:
                b.trace(br, hs, crt.TRI_WATERTIGHT)
                torch.cuda.synchronize()
                bounce_ms.append((time.perf_counter() - ts) * 1e3)
            torch.cuda.synchronize()
            frame_ms.append((time.perf_counter() - t0) * 1e3)
            run_ms.append(e[0].elapsed_time(e[1]))
            rays_traced.append(W * H + nb)
            if learned and (f % 15 == 0 or f == frames - 1):
                # the same bounce rays through the batch plain, seeded and sorted without the network
                row = {"rays": int(nb), "predictor_ordered_ms": round(bounce_ms[-1], 3)}
                for name, fl in (("plain_ms", 0), ("seeded_ms", crt.USE_PREDICTOR),
                                 ("sorted_no_network_ms", crt.SORT_RAYS)):
                    tp = time.perf_counter()
                    b.trace(br, hb_cmp[:nb], crt.TRI_WATERTIGHT | fl)
                    torch.cuda.synchronize()
                    row[name] = round((time.perf_counter() - tp) * 1e3, 3)
                    identical = identical and bool(torch.equal(hb_cmp[:nb].view(torch.int32), hs.view(torch.int32)))
                compare.append(row)
        if pred is not None:
            pred.free()
        b.set_ray_counts([W * H])
        bms = []
        for _ in range(3):   # the batched rebuild alone, host-timed around the call
            torch.cuda.synchronize()
            ts = time.perf_counter()
            b.build(tris)
            bms.append((time.perf_counter() - ts) * 1e3)
        b.free()
        fm = np.array(frame_ms[1:])
        out = {"frame_ms_p50": round(float(np.percentile(fm, 50)), 3),
               "frame_ms_p99": round(float(np.percentile(fm, 99)), 3),
               "rebuild_and_primary_ms_p50": round(float(np.median(run_ms[1:])), 3),
               "bounce_trace_ms_p50": round(float(np.median(bounce_ms[1:])), 3),
               "batch_build_ms": round(float(np.median(bms)), 3),
               "mrays_s": round(float(sum(rays_traced[1:]) / fm.sum() / 1e3), 1),
               "graph_replayed_frames": graph_frames,
               "identical_hits": identical}
        if learned:
            out["bounce_trace_ms"] = compare
        return out

    rebuild = animate(refit=False)
    refit = animate(refit=True)
    batch_learned = animate_batch(learned=True)
    batch_plain = animate_batch(learned=False)
    return {
        "workload": "16,777,216-tri clustered soup (1024 clusters), 60 animated frames, full rebuild per frame, "
                    "1920x1080 primary + 2 bounce rays per hit; on the batched graph (rebuild + primary replayed, "
                    "bounce rays traced in predicted-treelet order, predictor retrained per frame) against the same "
                    "frames with plain bounce traces, and through the single-scene calls",
        "frames": frames,
        "batched_graph": dict(batch_learned, note="crt_batch of one scene: crt_batch_run replays the captured "
                              "rebuild + primary trace every frame; bounce rays by crt_batch_bounce_rays, traced by "
                              "crt_batch_trace with CRT_TRACE_PREDICTOR_ORDER after crt_predictor_retarget, then "
                              "crt_predictor_train on the frame's hits; identical_hits: every frame's primary hits "
                              "equal the single-scene run's and every sampled learned bounce trace equals plain"),
        "batched_graph_plain": dict(batch_plain, note="the same frames, bounce rays traced plain, no predictor"),
        "learned_vs_plain_frame": round(batch_plain["frame_ms_p50"] / batch_learned["frame_ms_p50"], 3),
        "single_scene": rebuild,
        "refit": dict(refit, note="the same 60 frames with crt_refit of the frame-0 tree instead of a rebuild; "
                                  "identical_hits compares every frame's primary hits with the rebuild run's"),
    }


def sah_cost(nodes, ci=1.2):
    """Surface-area cost of a node array as crt_optimize counts it (internal
    nodes ci x area, leaves 1 x area), relative to the root's area."""
    d = nodes[:, 4:7].astype(np.float64) - nodes[:, 0:3]
    a = 2.0 * (d[:, 0] * d[:, 1] + d[:, 1] * d[:, 2] + d[:, 2] * d[:, 0])
    u = np.ascontiguousarray(nodes).view(np.uint32)
    leaf = (u[:, 9] == 0) & (u[:, 10] == 0)
    return float((np.where(leaf, 1.0, ci) * a).sum() / a[0])


def cpu_baseline(nodes, tris, models, rays, gpu_hits):
    """The reference's traversal on the host cores: the shader's walk
    (raytracer.glsl:246-295, right child popped first, no t pruning)
    restated in C++ (oracle) with the watertight predicate, on the reference
    arm's step-0 sample of the same rays; its hits are compared with the GPU's."""
    from oracle import oracle as O
    idx = ref_sample(0, rays.shape[0])
    sub = np.ascontiguousarray(rays[idx])
    O.trace(nodes, tris, models, sub[:2048], TRI_WATERTIGHT)
    t0 = time.perf_counter()
    hits, _ = O.trace(nodes, tris, models, sub, TRI_WATERTIGHT)
    dt = time.perf_counter() - t0
    return {"value": round(sub.shape[0] / dt / 1e6, 4), "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"every {REF_STRIDE}th ray of the same 8,388,608 bounce rays ({sub.shape[0]} rays), watertight "
                      f"predicate, the shader's DFS without t pruning, OpenMP over rays",
            "hits_equal_gpu": bool(np.array_equal(hits.view(np.uint32), gpu_hits[idx].view(np.uint32))),
            "hits": int((hits[:, 0].view(np.uint32) != 0xFFFFFFFF).sum())}


# --------------------------------------------------------- reference arm
def run_reference(args):
    """The reference's path on the host cores, on the headline workload:
    its PLOC build (bvh.cpp restated for N > 65,536, the reference's own cap)
    and its shader traversal restated in C++, a rotating 1/64 sample of the
    same bounce rays per step."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    from oracle import oracle as O
    from realtimeraytracing_gb300 import scenes as S
    O.build()
    tris, models = S.config3_scene(seed=0)
    n_tris = tris.shape[0]
    t0 = time.perf_counter()
    nb = O.build_bvh(tris, n_tris, models, faithful=True)
    build_ms = (time.perf_counter() - t0) * 1e3
    nodes = nb["nodes"]

    def primary_hits(prim):  # input generation only: the pruned walk, same hits
        h, _ = O.trace(nodes, tris, models, prim, TRI_WATERTIGHT | O.PRUNED)
        return h

    _, _, rays = S.config3_rays(tris, models, primary_hits, seed=BOUNCE_SEED, n_out=N_BOUNCE)
    times, counted, parts = [], [], []
    for k in range(args.warmup + args.steps):
        sub = np.ascontiguousarray(rays[ref_sample(k, N_BOUNCE)])
        t0 = time.perf_counter()
        hits, _ = O.trace(nodes, tris, models, sub, TRI_WATERTIGHT)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
            counted.append(sub.shape[0])
            parts.append(hits)
    value = sum(counted) / sum(times) / 1e6
    allh = np.concatenate(parts)
    cores = os.cpu_count()
    # the 65,536-triangle soup under the shader's own triangle predicate
    t0s, m0, cam0, (w0, h0) = S.config0_scene(seed=0)
    nb0 = O.build_bvh(t0s, t0s.shape[0], m0, faithful=True)
    r0 = S.pinhole_rays(cam0, w0, h0)
    t0 = time.perf_counter()
    h0, _ = O.trace(nb0["nodes"], t0s, m0, r0, TRI_REFERENCE)
    c0_ms = (time.perf_counter() - t0) * 1e3
    sample = (f"every {REF_STRIDE}th bounce ray per step, offset rotating with the step ({N_BOUNCE // REF_STRIDE} rays); "
              f"watertight predicate, the shader's DFS (raytracer.glsl:246-295) without t pruning, OpenMP over rays")
    line = {
        "metric": METRIC, "impl": "reference", "value": round(value, 4), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * statistics.mean(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded clustered soup and host-generated bounce rays)",
        "config": headline_config(),
        "build_ms": round(build_ms, 2),
        "rays_sha256": digest(rays),
        "sample_hits_sha256": digest(allh),
        "sample_hits": int((allh[:, 0].view(np.uint32) != 0xFFFFFFFF).sum()),
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "config0_shader_predicate": {"cpu_reference_predicate_mrays_s": round(r0.shape[0] / c0_ms / 1e3, 3),
                                     "hits": int((h0[:, 0].view(np.uint32) != 0xFFFFFFFF).sum()),
                                     "hits_sha256": digest(h0)},
    }
    print(json.dumps(line))


def main():
    global N_BOUNCE
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the restructured tree, the shader-predicate soup and the icosphere frame")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched experiment")
    ap.add_argument("--no-dynamic", action="store_true", help="skip the 16M-triangle 60-frame dynamic experiment")
    ap.add_argument("--rays", type=int, default=N_BOUNCE,
                    help="bounce rays per step (default 8,388,608; smaller batches for profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    N_BOUNCE = args.rays
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
