"""Build timing from the command line: crt_build on a seeded scene, repeated.

    python -m realtimeraytracing_gb300.buildbench [--scene icosphere|soup|clustered]
        [--tris N] [--reps K] [--multi-launch] [--radius R] [--digit-bits B]

Prints one JSON line with the median device-timed stages of the last K
builds (crt_last_build_stats) and the host wall time of a build call.
--multi-launch builds with CRT_BUILD_MULTI_LAUNCH: one launch per PLOC
iteration and one per layout level (then layout_emit), so that a profiler
sees every stage as its own kernel.
"""
from __future__ import annotations

import argparse
import json
import statistics
import time

import numpy as np


def scene(kind: str, n: int):
    from . import scenes as S
    if kind == "icosphere":
        level = 8
        while 20 * 4 ** level > n and level > 1:
            level -= 1
        v, f = S.displaced_icosphere(level, 0.05, 0)
        return S.indexed_to_triangles(v, f)
    if kind == "clustered":
        return S.clustered_soup(n, 256, 0.02, 0.003, 0.6, seed=0)
    return S.uniform_soup(n, seed=0)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", choices=["icosphere", "soup", "clustered"], default="icosphere")
    ap.add_argument("--tris", type=int, default=1310720)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--multi-launch", action="store_true")
    ap.add_argument("--radius", type=int, default=16)
    ap.add_argument("--digit-bits", type=int, default=8)
    a = ap.parse_args()
    from . import crt
    from . import scenes as S
    tris = scene(a.scene, a.tris)
    models = S.identity_models(1)
    ctx = crt.Context(ploc_radius=a.radius, sort_digit_bits=a.digit_bits, multi_launch_build=a.multi_launch)
    try:
        import torch
        d_tris = torch.from_numpy(tris).cuda()
        d_models = torch.from_numpy(models).cuda()
        torch.cuda.synchronize()
    except ImportError:
        d_tris, d_models = tris, models
    bvh = ctx.build(d_tris, models=d_models)
    stats, walls = [], []
    for _ in range(a.reps):
        t0 = time.perf_counter()
        bvh.rebuild(d_tris, models=d_models)
        walls.append((time.perf_counter() - t0) * 1e3)
        stats.append(ctx.last_build_stats())
    bvh.free()
    ctx.close()
    keys = ("ms_morton", "ms_sort", "ms_ploc", "ms_layout", "ms_total")
    print(json.dumps({"scene": a.scene, "triangles": int(tris.shape[0]), "reps": a.reps,
                      "multi_launch": a.multi_launch, "ploc_iterations": stats[-1]["ploc_iterations"],
                      **{k: round(statistics.median(s[k] for s in stats), 4) for k in keys},
                      "wall_ms": round(float(np.median(walls)), 4)}))


if __name__ == "__main__":
    main()
