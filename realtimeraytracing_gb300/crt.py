"""ctypes binding of libcrt.so (include/crt.h).

Arrays may be numpy arrays (host memory: the library copies in and out) or
torch CUDA tensors (device memory: used in place).  Record layouts are the
ones documented in realtimeraytracing_gb300.scenes.  Every entry point runs
the CUDA kernels; there is no host fallback — without the built library or a
GPU the calls raise CrtError.
"""
from __future__ import annotations

import ctypes as C
import sys
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcrt.so")

CRT_OK = 0
STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "DEVICE_TIMEOUT", 5: "STACK_OVERFLOW",
          6: "UNSUPPORTED", 7: "BAD_INPUT"}

TRACE_CLOSEST = 0x0
TRACE_ANY = 0x1
TRI_REFERENCE = 0x0
TRI_WATERTIGHT = 0x2
TRACE_USE_PREDICTOR = 0x4
TRACE_STATS = 0x8
TRACE_WIDE = 0x10
PREDICTOR_ORDER = 0x20  # CRT_TRACE_PREDICTOR_ORDER: trace rays grouped by predicted treelet
SORT_RAYS = 0x40  # CRT_TRACE_SORT_RAYS: trace rays ordered by origin cell and direction
TRACE_COMPRESSED = 0x80  # CRT_TRACE_COMPRESSED: walk 64-byte compressed 4-wide nodes
PER_RAY_THREADS = 0x100  # CRT_TRACE_PER_RAY_THREADS: one thread per ray instead of persistent refilling warps
USE_PREDICTOR = TRACE_USE_PREDICTOR
MISS = 0xFFFFFFFF

SHADE_WIREFRAME = 0x1  # CRT_SHADE_WIREFRAME: uIsWireframeModeOn
SHADE_BVH = 0x2  # CRT_SHADE_BVH: uIsBVHDisplayed
SHADE_MAX_BVH_DEPTH = 63
OPTIMIZE_MAX_PASSES = 16  # CRT_OPTIMIZE_MAX_PASSES

# Every symbol include/crt.h declares.
EXPORTS = [
    "crt_abi_version", "crt_default_config", "crt_create", "crt_destroy", "crt_sync", "crt_last_error_string",
    "crt_stream", "crt_build", "crt_rebuild", "crt_bvh_free", "crt_bvh_node_count", "crt_bvh_triangle_count",
    "crt_bvh_nodes_device", "crt_bvh_copy_nodes", "crt_bvh_copy_codes", "crt_bvh_copy_perm", "crt_last_build_stats",
    "crt_raygen_pinhole", "crt_shadow_rays", "crt_trace", "crt_last_trace_stats", "crt_trace_frame",
    "crt_morton_sort_noalloc", "crt_predictor_default_config", "crt_predictor_create", "crt_batch_predictor_create", "crt_predictor_destroy",
    "crt_predictor_retarget", "crt_predictor_train", "crt_predictor_infer", "crt_predictor_classes_of_hits",
    "crt_predictor_gradients", "crt_predictor_params", "crt_predictor_info", "crt_bounce_rays", "crt_trace_seeded",
    "crt_batch_create", "crt_batch_free", "crt_batch_set_models", "crt_batch_set_config", "crt_batch_get_config",
    "crt_batch_build", "crt_batch_trace", "crt_batch_run", "crt_batch_copy_nodes", "crt_batch_scene_info",
    "crt_batch_set_ray_counts", "crt_batch_bounce_rays",
    "crt_batch_autotune", "crt_shade", "crt_render_frame", "crt_refit", "crt_optimize", "crt_bvh_from_nodes",
    "crt_validate_nodes", "crt_obj_parse",
    "crt_triangles_from_indexed", "crt_selftest_wait", "crt_selftest_tc_wait", "crt_last_trace_timing",
    "crt_radix_digit_counts", "crt_radix_digit_offsets",
]

PREDICTOR_CLASSES = 128
PREDICTOR_PARAMS = 4225280


class CrtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("ploc_radius", C.c_uint32), ("sort_digit_bits", C.c_uint32),
                ("trace_block", C.c_uint32), ("stack_depth", C.c_uint32), ("spin_limit", C.c_uint32),
                ("build_flags", C.c_uint32)]


class BuildStats(C.Structure):
    _fields_ = [("n_tris", C.c_uint32), ("ploc_iterations", C.c_uint32), ("ms_morton", C.c_float),
                ("ms_sort", C.c_float), ("ms_ploc", C.c_float), ("ms_layout", C.c_float), ("ms_total", C.c_float),
                ("scene_box", C.c_float * 6)]

    def as_dict(self):
        return {f: (list(getattr(self, f)) if f == "scene_box" else getattr(self, f)) for f, _ in self._fields_}


_lib = None


def lib():
    """Load libcrt.so (fails loudly if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with realtimeraytracing_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        sig = {
            "crt_abi_version": ([], u32),
            "crt_default_config": ([vp], None),
            "crt_create": ([C.POINTER(vp), vp], i32),
            "crt_destroy": ([vp], i32),
            "crt_sync": ([vp], i32),
            "crt_last_error_string": ([], C.c_char_p),
            "crt_stream": ([vp], vp),
            "crt_build": ([vp, vp, u32, u32, vp, u32, C.POINTER(vp)], i32),
            "crt_rebuild": ([vp, vp, vp, u32, u32, vp, u32], i32),
            "crt_bvh_free": ([vp], i32),
            "crt_bvh_node_count": ([vp], u32),
            "crt_bvh_triangle_count": ([vp], u32),
            "crt_bvh_nodes_device": ([vp], vp),
            "crt_bvh_copy_nodes": ([vp, vp, vp], i32),
            "crt_bvh_copy_codes": ([vp, vp, vp], i32),
            "crt_bvh_copy_perm": ([vp, vp, vp], i32),
            "crt_last_build_stats": ([vp, vp], i32),
            "crt_raygen_pinhole": ([vp, vp, u32, u32, vp], i32),
            "crt_shadow_rays": ([vp, vp, vp, u32, vp, vp], i32),
            "crt_trace": ([vp, vp, vp, u32, u32, vp], i32),
            "crt_last_trace_stats": ([vp, vp], i32),
            "crt_trace_frame": ([vp, vp, vp, u32, u32, vp, u32, vp, vp], i32),
            "crt_morton_sort_noalloc": ([vp, u32, u32, vp, u32, vp, vp, vp], i32),
            "crt_predictor_default_config": ([vp], None),
            "crt_predictor_create": ([vp, vp, vp, C.POINTER(vp)], i32),
            "crt_batch_predictor_create": ([vp, vp, vp, C.POINTER(vp)], i32),
            "crt_predictor_destroy": ([vp], i32),
            "crt_predictor_retarget": ([vp, vp], i32),
            "crt_predictor_train": ([vp, vp, vp, vp, u32, u32, vp], i32),
            "crt_predictor_infer": ([vp, vp, vp, u32, vp], i32),
            "crt_predictor_classes_of_hits": ([vp, vp, vp, u32, vp], i32),
            "crt_predictor_gradients": ([vp, vp, vp, vp, u32, vp, vp], i32),
            "crt_predictor_params": ([vp, vp, vp, i32], i32),
            "crt_predictor_info": ([vp, vp], i32),
            "crt_bounce_rays": ([vp, vp, vp, vp, u32, u32, u32, vp], i32),
            "crt_trace_seeded": ([vp, vp, vp, u32, u32, vp, vp], i32),
            "crt_batch_create": ([vp, vp, vp, u32, C.POINTER(vp)], i32),
            "crt_batch_free": ([vp], i32),
            "crt_batch_set_models": ([vp, vp, vp, u32], i32),
            "crt_batch_set_config": ([vp, vp], i32),
            "crt_batch_get_config": ([vp, vp], i32),
            "crt_batch_build": ([vp, vp, vp], i32),
            "crt_batch_trace": ([vp, vp, vp, u32, vp], i32),
            "crt_batch_run": ([vp, vp, vp, vp, u32, vp, i32, vp], i32),
            "crt_batch_copy_nodes": ([vp, vp, u32, vp], i32),
            "crt_batch_scene_info": ([vp, u32, vp], i32),
            "crt_batch_set_ray_counts": ([vp, vp, vp], i32),
            "crt_batch_bounce_rays": ([vp, vp, u32, vp, vp, u32, u32, u32, vp], i32),
            "crt_batch_autotune": ([vp, vp, vp, vp, u32, vp, vp, vp], i32),
            "crt_shade": ([vp, vp, vp, vp, u32, vp, vp], i32),
            "crt_render_frame": ([vp, vp, vp, u32, u32, u32, vp, vp], i32),
            "crt_refit": ([vp, vp, vp, u32, vp, u32], i32),
            "crt_optimize": ([vp, vp, u32], i32),
            "crt_bvh_from_nodes": ([vp, vp, u32, vp, u32, vp, u32, C.POINTER(vp)], i32),
            "crt_validate_nodes": ([vp, u32, u32, vp], i32),
            "crt_obj_parse": ([C.c_char_p, C.c_size_t, vp, u32, vp, u32, vp], i32),
            "crt_triangles_from_indexed": ([vp, vp, u32, vp, u32, u32, vp], i32),
            "crt_selftest_wait": ([vp, i32, u32], i32),
            "crt_selftest_tc_wait": ([vp, i32, u32], i32),
            "crt_last_trace_timing": ([vp, vp], i32),
            "crt_radix_digit_counts": ([vp, vp, u32, u32, vp], i32),
            "crt_radix_digit_offsets": ([vp, vp, u32, u32, vp], i32),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _check(status: int):
    if status != CRT_OK:
        raise CrtError(status, lib().crt_last_error_string().decode(errors="replace"))


def _ptr(a):
    """Address of a numpy array or torch tensor (contiguous)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return C.c_void_p(a.data_ptr())
    raise TypeError(f"unsupported array type {type(a)}")


def _rows(a):
    return a.shape[0]


class Shading(C.Structure):
    """crt_shading: getColor's uniforms and its model / material buffers."""
    _fields_ = [("models", C.c_void_p), ("n_models", C.c_uint32), ("materials", C.c_void_p),
                ("n_materials", C.c_uint32), ("flags", C.c_uint32), ("bvh_depth", C.c_uint32)]


def _shading(models, materials, flags, bvh_depth):
    """(crt_shading, arrays it points to — keep them alive for the call)."""
    models = _models(models)
    if materials is not None and isinstance(materials, np.ndarray):
        materials = np.ascontiguousarray(materials, np.float32)
    sh = Shading()
    sh.models = _ptr(models) if models is not None else None
    sh.n_models = 0 if models is None else _rows(models)
    sh.materials = _ptr(materials) if materials is not None else None
    sh.n_materials = 0 if materials is None else _rows(materials)
    sh.flags, sh.bvh_depth = flags, bvh_depth
    return sh, (models, materials)


def validate_nodes(nodes, n_tris=None) -> dict:
    """crt_validate_nodes: the structure check of a DFS node array ((2n-1, 12)
    float32 records) on the host; raises CrtError naming the first problem."""
    nodes = np.ascontiguousarray(nodes, np.float32)
    n_tris = (nodes.shape[0] + 1) // 2 if n_tris is None else n_tris
    info = np.zeros(4, np.uint32)
    _check(lib().crt_validate_nodes(_ptr(nodes), nodes.shape[0], n_tris, _ptr(info)))
    return {"leaves": int(info[0]), "internal": int(info[1]), "height": int(info[2])}


def parse_obj(source):
    """crt_obj_parse on OBJ text (str / bytes) or a file path: (vertices (n, 3)
    float32, indices (m, 3) uint32).  Host-side parsing, as Mesh::load's."""
    if isinstance(source, str) and "\n" not in source and os.path.exists(source):
        with open(source, "rb") as f:
            data = f.read()
    else:
        data = source.encode() if isinstance(source, str) else bytes(source)
    counts = np.zeros(2, np.uint32)
    _check(lib().crt_obj_parse(data, len(data), None, 0, None, 0, _ptr(counts)))
    verts = np.empty((int(counts[0]), 3), np.float32)
    idx = np.empty((int(counts[1]), 3), np.uint32)
    _check(lib().crt_obj_parse(data, len(data), _ptr(verts), verts.shape[0], _ptr(idx), idx.shape[0], _ptr(counts)))
    return verts, idx


class PredictorConfig(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("lr", C.c_float), ("train_stride", C.c_uint32), ("batch", C.c_uint32),
                ("miss_threshold", C.c_float)]


class Predictor:
    """The learned hit predictor bound to one BVH (crt_predictor)."""

    def __init__(self, ctx: "Context", bvh, seed: int = 1, lr: float = 1e-3, train_stride: int = 20,
                 batch: int = 16384, miss_threshold: float = 0.9):
        """bvh: a Bvh, or a Batch (crt_batch_predictor_create: one network over
        every scene of the batch, created after the batch's first build)."""
        cfg = PredictorConfig()
        lib().crt_predictor_default_config(C.byref(cfg))
        cfg.seed, cfg.lr, cfg.train_stride, cfg.batch = seed, lr, train_stride, batch
        cfg.miss_threshold = miss_threshold
        h = C.c_void_p()
        create = lib().crt_batch_predictor_create if isinstance(bvh, Batch) else lib().crt_predictor_create
        _check(create(ctx.handle, bvh.handle, C.byref(cfg), C.byref(h)))
        self.ctx, self.bvh, self.handle = ctx, bvh, h

    def info(self) -> dict:
        out = np.zeros(4, np.uint32)
        _check(lib().crt_predictor_info(self.handle, _ptr(out)))
        return {"params": int(out[0]), "classes": int(out[1]), "treelets": int(out[2]), "steps": int(out[3])}

    def retarget(self):
        _check(lib().crt_predictor_retarget(self.ctx.handle, self.handle))

    def train(self, rays, hits, offset: int = 0) -> float:
        self.ctx._after_torch()
        loss = C.c_float()
        _check(lib().crt_predictor_train(self.ctx.handle, self.handle, _ptr(rays), _ptr(hits), _rows(rays), offset,
                                         C.byref(loss)))
        return loss.value

    def infer(self, rays, out=None):
        self.ctx._after_torch()
        out = np.empty(_rows(rays), np.uint16) if out is None else out
        _check(lib().crt_predictor_infer(self.ctx.handle, self.handle, _ptr(rays), _rows(rays), _ptr(out)))
        return out

    def classes_of_hits(self, hits, out=None):
        self.ctx._after_torch()
        out = np.empty(_rows(hits), np.uint16) if out is None else out
        _check(lib().crt_predictor_classes_of_hits(self.ctx.handle, self.handle, _ptr(hits), _rows(hits), _ptr(out)))
        return out

    def gradients(self, rays, targets):
        self.ctx._after_torch()
        grad = np.empty(PREDICTOR_PARAMS, np.float32)
        loss = C.c_float()
        targets = np.ascontiguousarray(targets, np.uint16)
        _check(lib().crt_predictor_gradients(self.ctx.handle, self.handle, _ptr(rays), _ptr(targets), _rows(rays),
                                             _ptr(grad), C.byref(loss)))
        return grad, loss.value

    def params(self):
        out = np.empty(PREDICTOR_PARAMS, np.float32)
        _check(lib().crt_predictor_params(self.ctx.handle, self.handle, _ptr(out), 0))
        return out

    def set_params(self, params):
        params = np.ascontiguousarray(params, np.float32)
        assert params.shape == (PREDICTOR_PARAMS,)
        _check(lib().crt_predictor_params(self.ctx.handle, self.handle, _ptr(params), 1))

    def free(self):
        if self.handle:
            lib().crt_predictor_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Many scenes built and traced with one launch per stage (crt_batch).
    Triangles, rays and hits are concatenated in scene order on the device."""

    def __init__(self, ctx: "Context", tri_counts, ray_counts, models=None):
        tc = np.ascontiguousarray(tri_counts, np.uint32)
        rc = np.ascontiguousarray(ray_counts, np.uint32)
        assert tc.shape == rc.shape
        h = C.c_void_p()
        _check(lib().crt_batch_create(ctx.handle, _ptr(tc), _ptr(rc), tc.shape[0], C.byref(h)))
        self.ctx, self.handle, self.n_scenes = ctx, h, int(tc.shape[0])
        self.tri_counts, self.ray_counts = tc, rc
        if models is not None:
            self.set_models(models)

    def set_models(self, models):
        self.ctx._after_torch()
        m = np.ascontiguousarray(models, np.float32)
        _check(lib().crt_batch_set_models(self.ctx.handle, self.handle, _ptr(m), m.shape[0]))

    def config(self) -> dict:
        c = Config()
        _check(lib().crt_batch_get_config(self.handle, C.byref(c)))
        return {f: getattr(c, f) for f, _ in Config._fields_}

    def set_config(self, ploc_radius=16, sort_digit_bits=8, trace_block=128, stack_depth=64):
        c = Config()
        lib().crt_default_config(C.byref(c))
        c.ploc_radius, c.sort_digit_bits, c.trace_block, c.stack_depth = ploc_radius, sort_digit_bits, trace_block, stack_depth
        _check(lib().crt_batch_set_config(self.handle, C.byref(c)))

    def build(self, tris):
        self.ctx._after_torch()
        _check(lib().crt_batch_build(self.ctx.handle, self.handle, _ptr(tris)))

    def trace(self, rays, hits, flags: int = 0):
        self.ctx._after_torch()
        _check(lib().crt_batch_trace(self.ctx.handle, self.handle, _ptr(rays), flags, _ptr(hits)))
        return hits

    def run(self, tris, rays, hits, flags: int = 0, graph: bool = True) -> bool:
        self.ctx._after_torch()
        used = C.c_int()
        _check(lib().crt_batch_run(self.ctx.handle, self.handle, _ptr(tris), _ptr(rays), flags, _ptr(hits),
                                   1 if graph else 0, C.byref(used)))
        return bool(used.value)

    def set_ray_counts(self, ray_counts):
        """Per-scene ray counts for the following traces (at most the batch's
        rays in total); a captured graph replays only with its own counts."""
        rc = np.ascontiguousarray(ray_counts, np.uint32)
        assert rc.shape == (self.n_scenes,)
        _check(lib().crt_batch_set_ray_counts(self.ctx.handle, self.handle, _ptr(rc)))
        self.ray_counts = rc

    def bounce_rays(self, scene: int, primary, hits, n_out: int, seed: int = 7, out=None):
        """crt_batch_bounce_rays: n_out cosine bounce rays from scene's primary hits."""
        self.ctx._after_torch()
        if out is None:
            import torch
            out = torch.empty((n_out, 8), dtype=torch.float32, device=primary.device)
        _check(lib().crt_batch_bounce_rays(self.ctx.handle, self.handle, scene, _ptr(primary), _ptr(hits),
                                           int(primary.shape[0]), n_out, seed, _ptr(out)))
        return out

    def nodes(self, scene: int):
        n = int(self.tri_counts[scene])
        out = np.empty((2 * n - 1, 12), np.float32)
        _check(lib().crt_batch_copy_nodes(self.ctx.handle, self.handle, scene, _ptr(out)))
        return out

    def scene_info(self, scene: int) -> dict:
        out = np.zeros(4, np.uint32)
        _check(lib().crt_batch_scene_info(self.handle, scene, _ptr(out)))
        return {"tris": int(out[0]), "rays": int(out[1]), "iterations": int(out[2]), "tri_off": int(out[3])}

    def autotune(self, tris, rays, hits, flags: int = 0):
        self.ctx._after_torch()
        c = Config()
        ms = C.c_float()
        _check(lib().crt_batch_autotune(self.ctx.handle, self.handle, _ptr(tris), _ptr(rays), flags, _ptr(hits),
                                        C.byref(c), C.byref(ms)))
        return {f: getattr(c, f) for f, _ in Config._fields_}, ms.value

    def free(self):
        if self.handle:
            lib().crt_batch_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Bvh:
    """A built BVH (crt_bvh): nodes in the reference's DFS layout, sorted
    Morton codes and the sorted-position -> triangle permutation."""

    def __init__(self, ctx: "Context", handle: C.c_void_p):
        self.ctx = ctx
        self.handle = handle

    @property
    def n_tris(self) -> int:
        return lib().crt_bvh_triangle_count(self.handle)

    @property
    def n_nodes(self) -> int:
        return lib().crt_bvh_node_count(self.handle)

    def nodes(self, out=None):
        out = np.empty((self.n_nodes, 12), np.float32) if out is None else out
        _check(lib().crt_bvh_copy_nodes(self.ctx.handle, self.handle, _ptr(out)))
        return out

    def codes(self, out=None):
        out = np.empty(self.n_tris, np.uint32) if out is None else out
        _check(lib().crt_bvh_copy_codes(self.ctx.handle, self.handle, _ptr(out)))
        return out

    def perm(self, out=None):
        out = np.empty(self.n_tris, np.uint32) if out is None else out
        _check(lib().crt_bvh_copy_perm(self.ctx.handle, self.handle, _ptr(out)))
        return out

    def rebuild(self, tris, n_tris=None, models=None, n_buffer=None):
        self.ctx._after_torch()
        models = _models(models)
        n_buffer = _rows(tris) if n_buffer is None else n_buffer
        n_tris = n_buffer if n_tris is None else n_tris
        _check(lib().crt_rebuild(self.ctx.handle, self.handle, _ptr(tris), n_buffer, n_tris, _ptr(models),
                                 0 if models is None else _rows(models)))
        return self

    def refit(self, tris, models=None):
        """crt_refit: the first n_tris triangles moved (same order), same tree
        topology, every box recomputed bottom-up."""
        self.ctx._after_torch()
        models = _models(models)
        _check(lib().crt_refit(self.ctx.handle, self.handle, _ptr(tris), self.n_tris, _ptr(models),
                               0 if models is None else _rows(models)))
        return self

    def optimize(self, passes: int = 2):
        """crt_optimize: treelet restructuring, `passes` passes (0 = boxes
        recomputed and the tree laid out again)."""
        self.ctx._after_torch()
        _check(lib().crt_optimize(self.ctx.handle, self.handle, passes))
        return self

    def free(self):
        if self.handle:
            lib().crt_bvh_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _models(models):
    if models is None:
        return None
    if isinstance(models, np.ndarray):
        return np.ascontiguousarray(models, np.float32)
    return models


class Context:
    """crt_ctx: one CUDA stream and the device scratch of the build."""

    def __init__(self, device: int = 0, ploc_radius: int = 16, sort_digit_bits: int = 8, trace_block: int = 128,
                 stack_depth: int = 64, spin_limit: int = 0, multi_launch_build: bool = False):
        cfg = Config()
        lib().crt_default_config(C.byref(cfg))
        cfg.device, cfg.ploc_radius, cfg.sort_digit_bits = device, ploc_radius, sort_digit_bits
        cfg.trace_block, cfg.stack_depth, cfg.spin_limit = trace_block, stack_depth, spin_limit
        cfg.build_flags = 1 if multi_launch_build else 0
        h = C.c_void_p()
        _check(lib().crt_create(C.byref(h), C.byref(cfg)))
        self.handle = h
        self.device = device
        self._ext = None

    def _after_torch(self):
        """Orders the library's stream after the work torch has queued on its
        current stream, so device inputs torch produced are complete before
        the library reads them (an event wait on the GPU, no host sync).  The
        library's calls return with their outputs complete."""
        t = sys.modules.get("torch")
        if t is None or not t.cuda.is_available() or not t.cuda.is_initialized():
            return
        dev = t.device("cuda", self.device)
        cur = t.cuda.current_stream(dev)
        if cur.cuda_stream == self.stream:
            return
        if self._ext is None:
            self._ext = t.cuda.ExternalStream(self.stream, device=dev)
        self._ext.wait_stream(cur)

    def close(self):
        if getattr(self, "handle", None):
            lib().crt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib().crt_stream(self.handle) or 0

    def sync(self):
        _check(lib().crt_sync(self.handle))

    def selftest_wait(self, set_flag: bool, spin_limit: int = 0):
        """crt_selftest_wait: one bounded device wait on a flag (set or never set)."""
        _check(lib().crt_selftest_wait(self.handle, 1 if set_flag else 0, spin_limit))

    def selftest_tc_wait(self, complete: bool, spin_limit: int = 0):
        """crt_selftest_tc_wait: one MMA commit wait (completed, or never completed)."""
        _check(lib().crt_selftest_tc_wait(self.handle, 1 if complete else 0, spin_limit))

    def radix_digit_counts(self, keys, digit_bits: int):
        """crt_radix_digit_counts: (places, 2^digit_bits) counts of 32-bit keys."""
        keys = np.ascontiguousarray(keys, np.uint32) if isinstance(keys, np.ndarray) else keys
        places = (32 + digit_bits - 1) // digit_bits
        out = np.zeros((places, 1 << digit_bits), np.uint32)
        _check(lib().crt_radix_digit_counts(self.handle, _ptr(keys), _rows(keys), digit_bits, _ptr(out)))
        return out

    def radix_digit_offsets(self, counts, digit_bits: int):
        """crt_radix_digit_offsets: per place (row), the exclusive scan of its digit counts."""
        counts = np.ascontiguousarray(counts, np.uint32).reshape(-1, 1 << digit_bits)
        out = np.zeros_like(counts)
        _check(lib().crt_radix_digit_offsets(self.handle, _ptr(counts), counts.shape[0], digit_bits, _ptr(out)))
        return out

    def build(self, tris, n_tris=None, models=None, n_buffer=None) -> Bvh:
        """cr::BVH::BVH(nbTriangles, unsortedTriangles, meshesInTheScene)."""
        self._after_torch()
        models = _models(models)
        n_buffer = _rows(tris) if n_buffer is None else n_buffer
        n_tris = n_buffer if n_tris is None else n_tris
        h = C.c_void_p()
        _check(lib().crt_build(self.handle, _ptr(tris), n_buffer, n_tris, _ptr(models),
                               0 if models is None else _rows(models), C.byref(h)))
        return Bvh(self, h)

    def bvh_from_nodes(self, nodes, tris, models=None) -> Bvh:
        """crt_bvh_from_nodes: a traceable BVH from a DFS node array in the
        reference's layout ((2n-1, 12) float32 records) and its n triangles."""
        self._after_torch()
        models = _models(models)
        if isinstance(nodes, np.ndarray):
            nodes = np.ascontiguousarray(nodes, np.float32)
        h = C.c_void_p()
        _check(lib().crt_bvh_from_nodes(self.handle, _ptr(nodes), _rows(nodes), _ptr(tris), _rows(tris), _ptr(models),
                                        0 if models is None else _rows(models), C.byref(h)))
        return Bvh(self, h)

    def last_build_stats(self) -> dict:
        s = BuildStats()
        _check(lib().crt_last_build_stats(self.handle, C.byref(s)))
        return s.as_dict()

    def raygen(self, cam, width: int, height: int, out=None):
        self._after_torch()
        cam = np.ascontiguousarray(cam, np.float32) if isinstance(cam, np.ndarray) else cam
        out = np.empty((width * height, 8), np.float32) if out is None else out
        _check(lib().crt_raygen_pinhole(self.handle, _ptr(cam), width, height, _ptr(out)))
        return out

    def shadow_rays(self, primary, hits, light, out=None):
        self._after_torch()
        n = _rows(primary)
        out = np.empty((n, 8), np.float32) if out is None else out
        light = np.ascontiguousarray(light, np.float32)
        _check(lib().crt_shadow_rays(self.handle, _ptr(primary), _ptr(hits), n, _ptr(light), _ptr(out)))
        return out

    def trace(self, bvh: Bvh, rays, flags: int = 0, out=None):
        self._after_torch()
        n = _rows(rays)
        out = np.empty((n, 4), np.float32) if out is None else out
        _check(lib().crt_trace(self.handle, bvh.handle, _ptr(rays), n, flags, _ptr(out)))
        return out

    def bounce_rays(self, bvh: "Bvh", primary, hits, n_out: int, seed: int = 7, out=None):
        self._after_torch()
        out = np.empty((n_out, 8), np.float32) if out is None else out
        _check(lib().crt_bounce_rays(self.handle, bvh.handle, _ptr(primary), _ptr(hits), _rows(primary), n_out, seed,
                                     _ptr(out)))
        return out

    def trace_seeded(self, bvh: "Bvh", rays, classes, flags: int = 0, out=None):
        """Trace with the treelet of classes[i] searched first (device arrays)."""
        self._after_torch()
        _check(lib().crt_trace_seeded(self.handle, bvh.handle, _ptr(rays), _rows(rays), flags, _ptr(classes),
                                      _ptr(out)))
        return out

    def last_trace_stats(self):
        """(node boxes tested, triangles tested) of the last trace issued with TRACE_STATS."""
        out = np.zeros(2, np.uint64)
        _check(lib().crt_last_trace_stats(self.handle, _ptr(out)))
        return int(out[0]), int(out[1])

    def last_trace_timing(self):
        """(ms before the traversal kernel, traversal kernel ms) of the last trace, from CUDA events."""
        out = np.zeros(2, np.float32)
        _check(lib().crt_last_trace_timing(self.handle, _ptr(out)))
        return float(out[0]), float(out[1])

    def trace_frame(self, bvh: Bvh, cam, width: int, height: int, light=None, flags: int = 0,
                    hits_primary=None, hits_shadow=None):
        """Application::drawOneFrame's compute pass: primary closest hits and,
        with a light, shadow any-hits.  Returns (hits_primary, hits_shadow)."""
        self._after_torch()
        n = width * height
        cam = np.ascontiguousarray(cam, np.float32) if isinstance(cam, np.ndarray) else cam
        hp = np.empty((n, 4), np.float32) if hits_primary is None else hits_primary
        hs = None
        lp = None
        if light is not None:
            hs = np.empty((n, 4), np.float32) if hits_shadow is None else hits_shadow
            light = np.ascontiguousarray(light, np.float32)
            lp = _ptr(light)
        _check(lib().crt_trace_frame(self.handle, bvh.handle, _ptr(cam), width, height, lp, flags, _ptr(hp),
                                     _ptr(hs)))
        return hp, hs

    def triangles_from_indexed(self, vertices, indices, model_id: int = 0, out=None):
        """crt_triangles_from_indexed: (m, 16) float32 TriangleGPU records of an
        indexed mesh, built on the GPU."""
        self._after_torch()
        if isinstance(vertices, np.ndarray):
            vertices = np.ascontiguousarray(vertices, np.float32)
        if isinstance(indices, np.ndarray):
            indices = np.ascontiguousarray(indices, np.uint32)
        n_tri = _rows(indices)
        out = np.empty((n_tri, 16), np.float32) if out is None else out
        _check(lib().crt_triangles_from_indexed(self.handle, _ptr(vertices), _rows(vertices), _ptr(indices), n_tri,
                                                model_id, _ptr(out)))
        return out

    def shade(self, bvh: Bvh, rays, hits, models=None, materials=None, shade_flags: int = 0, bvh_depth: int = 0,
              out=None):
        """getColor + imageStore for each hit: (n, 4) RGBA32F texels.  rays are
        read only with SHADE_BVH (else they may be None)."""
        self._after_torch()
        n = _rows(hits)
        out = np.empty((n, 4), np.float32) if out is None else out
        sh, keep = _shading(models, materials, shade_flags, bvh_depth)
        _check(lib().crt_shade(self.handle, bvh.handle, _ptr(rays), _ptr(hits), n, C.byref(sh), _ptr(out)))
        del keep
        return out

    def render_frame(self, bvh: Bvh, cam, width: int, height: int, models=None, materials=None,
                     shade_flags: int = 0, bvh_depth: int = 0, flags: int = 0, out=None):
        """The reference's compute pass (raytracer.glsl main): camera ray,
        closest hit, getColor and imageStore per texel, (width*height, 4)
        RGBA32F with texel (x, y) at row y * width + x."""
        self._after_torch()
        cam = np.ascontiguousarray(cam, np.float32) if isinstance(cam, np.ndarray) else cam
        out = np.empty((width * height, 4), np.float32) if out is None else out
        sh, keep = _shading(models, materials, shade_flags, bvh_depth)
        _check(lib().crt_render_frame(self.handle, bvh.handle, _ptr(cam), width, height, flags, C.byref(sh),
                                      _ptr(out)))
        del keep
        return out
