"""Regenerates the golden fixtures in this directory.

Build fixtures come from the reference's OWN BVH builder: its unmodified
srcCommon/scene/geometry/bvh.cpp and triangle.cpp, compiled by
oracle/Makefile (target `ref`) into oracle/_ref/libref_bvh.so.  This script
therefore needs the reference checkout; the fixtures it writes let the oracle
be pinned on machines without it.

Trace and frame fixtures come from the reference's own compute shader,
srcCommon/shaders/raytracer.glsl compiled as C++ (oracle/glsl_to_cpp.py
rewrites its declarations, the project's GLSL shim supplies the built-ins;
oracle/Makefile target `ref` builds oracle/_ref/libref_shader.so), after
checking that the oracle's restatement gives the same bits.

Inputs are regenerated from seeds by realtimeraytracing_gb300.scenes, whose
generators use exact arithmetic only; each fixture stores the sha256 of its
input buffer so generator drift is caught.

Run:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from realtimeraytracing_gb300 import scenes as S  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def build_cases():
    """(name, triangles, n_tris, models) — inputs derivable from seeds."""
    cases = []
    for n in (1, 2, 3, 17, 1000):
        cases.append((f"soup_n{n}", S.uniform_soup(n, seed=500 + n), n, S.identity_models(1)))
    t = S.uniform_soup(1000, seed=77)
    t[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]] += np.float32(0.25)   # keep the origin outside the soup
    cases.append(("soup_n1000_padded4096", np.concatenate([t, np.zeros((3096, 16), np.float32)]), 1000,
                  S.identity_models(1)))
    t = S.uniform_soup(2000, seed=78)
    t.view(np.uint32)[:, 12] = np.arange(2000) % 3
    m = S.identity_models(3)
    m[1, 12:15] = [0.5, -0.25, 2.0]
    m[2, 0:16] = np.array([0, 2, 0, 0, -1, 0, 0, 0, 0, 0, 0.5, 0, 0.125, 1, -1, 1], np.float32)
    cases.append(("soup_n2000_models3", t, 2000, m))
    cases.append(("dup_n64", np.repeat(S.uniform_soup(1, seed=79), 64, axis=0), 64, S.identity_models(1)))
    # the renderer's own buffer: N triangles padded with zero records to 65,536 (scene.cpp:26-40)
    for n in (1, 3, 1000):
        t = S.uniform_soup(n, seed=600 + n)
        cases.append((f"soup_n{n}_padded65536", np.concatenate([t, np.zeros((65536 - n, 16), np.float32)]), n,
                      S.identity_models(1)))
    return cases


def main():
    O.build(ref=True)
    index = {}
    for name, tris, n, models in build_cases():
        r = O.ref_build_bvh(tris, n, models)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), codes=r["codes"], perm=r["perm"], nodes=r["nodes"],
                            codes_unsorted=r["codes_unsorted"])
        index[name] = {"input_sha256": sha(tris), "models_sha256": sha(models), "n_tris": n,
                       "n_buffer": int(tris.shape[0])}
    # config 0 (65,536-triangle soup): hashes only
    tris, models, cam, (w, h) = S.config0_scene(seed=0)
    r = O.ref_build_bvh(tris, tris.shape[0], models)
    index["config0"] = {"input_sha256": sha(tris), "n_tris": int(tris.shape[0]),
                        "codes_sha256": sha(r["codes"]), "perm_sha256": sha(r["perm"]),
                        "nodes_sha256": sha(r["nodes"]), "codes_unsorted_sha256": sha(r["codes_unsorted"])}
    rays = O.raygen(cam, w, h)
    hr = O.shader_closest_hits(r["nodes"], tris, models, rays)
    ho, _ = O.trace(r["nodes"], tris, models, rays, 0)
    assert sha(hr) == sha(ho), "the oracle's traversal differs from the shader's"
    hw, _ = O.trace(r["nodes"], tris, models, rays, 2)
    index["config0_trace"] = {"camera": [float(x) for x in cam], "rays_sha256": sha(rays),
                              "hits_reference_sha256": sha(hr), "hits_watertight_sha256": sha(hw),
                              "source": "reference predicate: the reference's raytracer.glsl compiled as C++ "
                                        "(getClosestHitBVH); watertight: the oracle's restatement"}
    # the whole compute pass (main: getRay, closest hit, bvhColor, getColor, imageStore)
    fw = fh = 128
    mats = [[0.1, 0.2, 0.3, 1.0], [0.75, 0.5, 0.25, 1.0]]
    fm = S.models_with_materials([1])
    img = O.shader_frame(cam, fw, fh, r["nodes"], tris, fm, S.materials(mats), 3, 2)
    r2 = O.raygen(cam, fw, fh)
    h2, _ = O.trace(r["nodes"], tris, fm, r2, 0)
    assert sha(img) == sha(O.shade(r["nodes"], tris, fm, S.materials(mats), r2, h2, 3, 2))
    index["config0_frame"] = {"width": fw, "height": fh, "flags": 3, "depth": 2, "materials": mats,
                              "material_ids": [1], "texels_sha256": sha(img),
                              "source": "the reference's raytracer.glsl main compiled as C++, "
                                        "wireframe on, BVH boxes of depth 2 displayed"}
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)
    print("wrote", len(index), "fixtures")


if __name__ == "__main__":
    main()
