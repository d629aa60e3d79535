"""ORACLE — test infrastructure, never part of the product path.

ctypes front end of the CPU oracle:
  * _build/liboracle.so — the project's CPU restatement of the reference's
    BVH build (srcCommon/scene/geometry/bvh.cpp) and of its GLSL traversal
    (srcCommon/shaders/raytracer.glsl); see crt_oracle.cpp for line citations.
  * _ref/libref_bvh.so — the reference's own bvh.cpp/triangle.cpp compiled in
    place with the project's glm shim (only where the reference checkout is
    present; N <= 65,536).
  * _ref/libref_shader.so — the reference's own raytracer.glsl compiled as
    C++ (declarations rewritten by glsl_to_cpp.py, bodies unchanged, the
    project's GLSL shim), where the reference checkout is present.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_bvh.so")
SHADER_LIB = os.path.join(HERE, "_ref", "libref_shader.so")
# The reference checkout: CRT_REFERENCE_DIR, else a directory named
# "reference" beside the repository.
REFERENCE_DIR = os.environ.get("CRT_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

_lib = None
_ref = None
_shader = None

# oracle_trace flag (with CRT_TRI_WATERTIGHT, closest hit): the pruned
# near-first walk, same hits as the full walk; for making large test inputs.
PRUNED = 0x100


def build(ref: bool | None = None) -> None:
    """Compile the restatement (always) and the reference library (when the
    reference checkout exists and ref is not False)."""
    targets = ["all"]
    if ref is None:
        ref = os.path.isdir(os.path.join(REFERENCE_DIR, "srcCommon"))
    if ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE, f"REFERENCE_DIR={REFERENCE_DIR}", *targets], check=True)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(ref=False)
        L = C.CDLL(LIB)
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        L.oracle_morton.argtypes = [vp, u32, u32, vp, u32, vp, vp, vp]
        L.oracle_build.argtypes = [vp, u32, u32, vp, u32, u32, i32, vp, vp, vp, vp, vp]
        L.oracle_build.restype = i32
        L.oracle_raygen.argtypes = [vp, u32, u32, vp]
        L.oracle_shadow_rays.argtypes = [vp, vp, u32, vp, vp]
        L.oracle_trace.argtypes = [vp, u32, vp, u32, vp, u32, vp, u32, u32, vp, vp]
        L.oracle_trace_brute.argtypes = [vp, u32, vp, u32, vp, u32, u32, vp]
        L.oracle_shade.argtypes = [vp, u32, vp, u32, vp, u32, vp, u32, vp, vp, u32, u32, u32, vp]
        L.oracle_refit.argtypes = [vp, u32, vp, u32, vp, u32]
        L.oracle_optimize.argtypes = [vp, u32, u32, vp]
        L.oracle_optimize.restype = u32
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_LIB)
        vp, u32 = C.c_void_p, C.c_uint32
        L.ref_bvh_build.argtypes = [vp, u32, u32, vp, u32, vp, vp, vp, vp, vp]
        L.ref_bvh_build.restype = C.c_int
        L.ref_max_triangles.restype = u32
        _ref = L
    return _ref


def shader_available() -> bool:
    return os.path.exists(SHADER_LIB)


def shader_lib():
    """The reference's raytracer.glsl compiled as C++ (shader_driver.cpp)."""
    global _shader
    if _shader is None:
        L = C.CDLL(SHADER_LIB)
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        L.glsl_closest_hits.argtypes = [vp, vp, u32, vp, u32, vp, u32, vp]
        L.glsl_all_hits.argtypes = [vp, u32, vp, u32, vp, u32, vp]
        L.glsl_frame.argtypes = [vp, u32, u32, vp, vp, u32, vp, u32, vp, u32, u32, i32, vp]
        _shader = L
    return _shader


def shader_closest_hits(nodes, tris, models, rays):
    """getClosestHitBVH (raytracer.glsl:246-295) of the shader itself, per ray."""
    nodes = _f32(nodes, 12)
    tris, models, rays = _f32(tris, 16), _f32(models, 17), _f32(rays, 8)
    hits = np.zeros((rays.shape[0], 4), np.float32)
    shader_lib().glsl_closest_hits(_p(nodes), _p(tris), tris.shape[0], _p(models), models.shape[0], _p(rays),
                                   rays.shape[0], _p(hits))
    return hits


def shader_all_hits(tris, models, rays):
    """getAllHits (raytracer.glsl:149-157) of the shader itself, per ray."""
    tris, models, rays = _f32(tris, 16), _f32(models, 17), _f32(rays, 8)
    hits = np.zeros((rays.shape[0], 4), np.float32)
    shader_lib().glsl_all_hits(_p(tris), tris.shape[0], _p(models), models.shape[0], _p(rays), rays.shape[0],
                               _p(hits))
    return hits


def shader_frame(cam, width, height, nodes, tris, models, materials, flags=0, depth=0):
    """The shader's main (raytracer.glsl:299-331) over (width/16) x
    (height/16) work groups: RGBA32F texels, row y at y * width."""
    cam = np.ascontiguousarray(cam, np.float32)
    nodes = _f32(nodes, 12)
    tris, models, materials = _f32(tris, 16), _f32(models, 17), _f32(materials, 4)
    out = np.zeros((width * height, 4), np.float32)
    shader_lib().glsl_frame(_p(cam), width, height, _p(nodes), _p(tris), tris.shape[0], _p(models), models.shape[0],
                            _p(materials), materials.shape[0], flags, depth, _p(out))
    return out


def _f32(a, cols):
    a = np.ascontiguousarray(a, dtype=np.float32)
    assert a.ndim == 2 and a.shape[1] == cols
    return a


def morton(tris, n_tris, models):
    tris, models = _f32(tris, 16), _f32(models, 17)
    codes = np.zeros(n_tris, np.uint32)
    scene = np.zeros(6, np.float32)
    cube = np.zeros(6, np.float32)
    lib().oracle_morton(_p(tris), tris.shape[0], n_tris, _p(models), models.shape[0], _p(codes), _p(scene), _p(cube))
    return codes, scene, cube


def build_bvh(tris, n_tris, models, radius=16, faithful=False):
    """Returns dict(codes, perm, nodes (2n-1,12) float32, iterations, ms[4])."""
    tris, models = _f32(tris, 16), _f32(models, 17)
    codes = np.zeros(n_tris, np.uint32)
    perm = np.zeros(n_tris, np.uint32)
    nodes = np.zeros((2 * n_tris - 1, 12), np.float32)
    it = np.zeros(1, np.uint32)
    ms = np.zeros(4, np.float64)
    rc = lib().oracle_build(_p(tris), tris.shape[0], n_tris, _p(models), models.shape[0], radius,
                            1 if faithful else 0, _p(codes), _p(perm), _p(nodes), _p(it), _p(ms))
    if rc != 0:
        raise ValueError(f"oracle_build failed ({rc})")
    return dict(codes=codes, perm=perm, nodes=nodes, iterations=int(it[0]), ms=ms)


def ref_build_bvh(tris, n_tris, models):
    """The reference's own cr::BVH on the same input (N <= 65,536)."""
    tris, models = _f32(tris, 16), _f32(models, 17)
    codes_u = np.zeros(n_tris, np.uint32)
    codes = np.zeros(n_tris, np.uint32)
    perm = np.zeros(n_tris, np.uint32)
    nodes = np.zeros((2 * n_tris - 1, 12), np.float32)
    ms = np.zeros(1, np.float64)
    rc = ref_lib().ref_bvh_build(_p(tris), tris.shape[0], n_tris, _p(models), models.shape[0],
                                 _p(codes_u), _p(codes), _p(perm), _p(nodes), _p(ms))
    if rc != 0:
        raise ValueError(f"ref_bvh_build failed ({rc})")
    return dict(codes_unsorted=codes_u, codes=codes, perm=perm, nodes=nodes, ms=float(ms[0]))


def raygen(cam, width, height):
    cam = np.ascontiguousarray(cam, np.float32)
    rays = np.zeros((width * height, 8), np.float32)
    lib().oracle_raygen(_p(cam), width, height, _p(rays))
    return rays


def shadow_rays(prim, hits, light):
    prim = _f32(prim, 8)
    hits = np.ascontiguousarray(hits, np.float32)
    light = np.ascontiguousarray(light, np.float32)
    out = np.zeros_like(prim)
    lib().oracle_shadow_rays(_p(prim), _p(hits), prim.shape[0], _p(light), _p(out))
    return out


def trace(nodes, tris, models, rays, flags=0):
    nodes = _f32(nodes, 12)
    tris, models, rays = _f32(tris, 16), _f32(models, 17), _f32(rays, 8)
    hits = np.zeros((rays.shape[0], 4), np.float32)
    stats = np.zeros(2, np.uint64)
    lib().oracle_trace(_p(nodes), nodes.shape[0], _p(tris), tris.shape[0], _p(models), models.shape[0],
                       _p(rays), rays.shape[0], flags, _p(hits), _p(stats))
    return hits, stats


def trace_brute(tris, models, rays, flags=0):
    tris, models, rays = _f32(tris, 16), _f32(models, 17), _f32(rays, 8)
    hits = np.zeros((rays.shape[0], 4), np.float32)
    lib().oracle_trace_brute(_p(tris), tris.shape[0], _p(models), models.shape[0], _p(rays), rays.shape[0], flags, _p(hits))
    return hits


def shade(nodes, tris, models, materials, rays, hits, flags=0, depth=0):
    """getColor + imageStore per hit: (n, 4) float32 RGBA (rays read with the BVH flag)."""
    nodes = _f32(nodes, 12)
    tris, models, rays = _f32(tris, 16), _f32(models, 17), _f32(rays, 8)
    materials = _f32(materials, 4)
    hits = np.ascontiguousarray(hits, np.float32)
    out = np.zeros((hits.shape[0], 4), np.float32)
    lib().oracle_shade(_p(nodes), nodes.shape[0], _p(tris), tris.shape[0], _p(models), models.shape[0],
                       _p(materials), materials.shape[0], _p(rays), _p(hits), hits.shape[0], flags, depth, _p(out))
    return out


def refit(nodes, tris, models):
    """The node array with every box recomputed from the moved triangles (same topology)."""
    out = np.array(_f32(nodes, 12), copy=True)
    tris, models = _f32(tris, 16), _f32(models, 17)
    lib().oracle_refit(_p(out), out.shape[0], _p(tris), tris.shape[0], _p(models), models.shape[0])
    return out


def optimize(nodes, passes=1):
    """Treelet-restructured node array (the product's crt_optimize) and the
    new root height."""
    nodes = _f32(nodes, 12)
    out = np.zeros_like(nodes)
    h = lib().oracle_optimize(_p(nodes), nodes.shape[0], passes, _p(out))
    return out, int(h)
