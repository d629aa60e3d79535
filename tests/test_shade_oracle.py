"""The oracle's shading restatement on the CPU (getColor + imageStore,
srcCommon/shaders/raytracer.glsl:159-179, 299-331, with the bvhColor of
getClosestHitBVH :246-277 and intersectBVH's border test :182-236).

1. getColor's material and wireframe rules, restated again here in numpy.
2. The BVH display colour: the oracle runs the shader's own walk (right child
   popped first, the last intersected depth-D node wins); the CUDA kernel
   instead stops at the FIRST intersected depth-D node of a left-first walk.
   Both are checked here to give the same texel for every ray.
3. The headless PPM writer.
"""
import numpy as np
import pytest

from oracle import oracle as O
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import image
from realtimeraytracing_gb300 import scenes as S

f32 = np.float32
MATERIALS = S.materials([[0.25, 0.5, 0.75, 1.0], [1.0, 0.0, 0.0, 0.5], [0.0, 0.125, 1.0, 0.25]])


@pytest.fixture(scope="module")
def scene():
    O.build(ref=False)
    tris = S.uniform_soup(300, seed=3, edge_lo=0.02, edge_hi=0.2)
    tris.view(np.uint32)[:, 12] = np.arange(300, dtype=np.uint32) % 4  # model 3 >= n_models: material 0
    models = S.models_with_materials([2, 0, 9])                       # material 9 >= n_materials: (0,0,0,0)
    b = O.build_bvh(tris, 300, models)
    cam = S.camera_gpu_data((0.5, 0.5, -1.5))
    rays = np.concatenate([O.raygen(cam, 24, 24), S.sphere_rays(200, seed=5)])
    hits, _ = O.trace(b["nodes"], tris, models, rays, crt.TRI_REFERENCE)
    return tris, models, b["nodes"], rays, hits


def _get_color(tris, models, hits, wire):
    out = np.zeros((hits.shape[0], 4), np.float32)
    out[:, 3] = 1.0
    mids = models.view(np.uint32)[:, 16]
    for i, h in enumerate(hits):
        tri = h[:1].view(np.uint32)[0]
        if tri == crt.MISS:
            continue
        model = tris.view(np.uint32)[tri, 12]
        mat = mids[model] if model < models.shape[0] else 0
        c = MATERIALS[mat] if mat < MATERIALS.shape[0] else np.zeros(4, np.float32)
        out[i] = out[i] + c
        u, v = f32(h[2]), f32(h[3])
        w = f32(1) - u - v
        if wire and (u < f32(0.02) or v < f32(0.02) or w < f32(0.02)):
            out[i] = (0.0, 0.0, 0.0, 1.0)
    return out


@pytest.mark.parametrize("wire", [False, True])
def test_get_color_materials_and_wireframe(scene, wire):
    tris, models, nodes, rays, hits = scene
    n_hit = int((hits[:, 0].view(np.uint32) != crt.MISS).sum())
    assert 50 < n_hit < hits.shape[0]
    got = O.shade(nodes, tris, models, MATERIALS, rays, hits, crt.SHADE_WIREFRAME if wire else 0)
    np.testing.assert_array_equal(got.view(np.uint32), _get_color(tris, models, hits, wire).view(np.uint32))
    if wire:  # some hits are near an edge, some are not
        black = np.all(got == np.array([0, 0, 0, 1], np.float32), axis=1)
        hit = hits[:, 0].view(np.uint32) != crt.MISS
        assert 0 < (black & hit).sum() < hit.sum()


def _min(a, b):
    return b if b < a else a


def _max(a, b):
    return b if a < b else a


def _display_slab(o, d, mn, mx, line):
    """intersectBVH with its border test, in float32 scalars."""
    with np.errstate(all="ignore"):
        t_min = t_max = None
        for k in range(3):
            inv = f32(1) / d[k]
            t1, t2 = (mn[k] - o[k]) * inv, (mx[k] - o[k]) * inv
            if k == 0:
                t_min, t_max = _min(t1, t2), _max(t1, t2)
            else:
                t_min, t_max = _max(t_min, _min(t1, t2)), _min(t_max, _max(t1, t2))
            if k < 2 and (t_max < 0 or t_min > t_max):
                return 0
        if not (t_max >= 0 and t_min <= t_max):
            return 0
        close = [abs(o[k] + d[k] * t_min - mn[k]) < line or abs(o[k] + d[k] * t_min - mx[k]) < line for k in range(3)]
    return 2 if (close[0] and close[1]) or (close[0] and close[2]) or (close[1] and close[2]) else 1


def _first_left_first(nodes, ray, depth_d):
    """The CUDA kernel's formulation: first intersected depth-D node of a
    left-child-first walk through intersected boxes."""
    line = f32(0.05) / (f32(depth_d) + f32(1))
    u = nodes.view(np.uint32)
    o, d = ray[0:3], ray[4:7]
    stack = [(0, 0)]
    while stack:
        ni, depth = stack.pop()
        hit = _display_slab(o, d, nodes[ni, 0:3], nodes[ni, 4:7], line)
        if hit == 0:
            continue
        if depth == depth_d:
            return hit
        left, right = int(u[ni, 9]), int(u[ni, 10])
        if left or right:
            stack.append((right, depth + 1))
            stack.append((left, depth + 1))
    return 0


def test_bvh_display_first_left_first_equals_shaders_last(scene):
    tris, models, nodes, rays, _ = scene
    misses = np.zeros((rays.shape[0], 4), np.float32)
    misses[:, 0] = np.frombuffer(np.uint32(crt.MISS).tobytes(), np.float32)[0]
    colors = {0: (0.0, 0.0, 0.0, 0.0), 1: (0.5, 0.0, 0.5, 0.1), 2: (0.7, 0.0, 0.7, 0.1)}
    seen = set()
    for depth in (0, 1, 3, 6, 9):
        got = O.shade(nodes, tris, models, MATERIALS, rays, misses, crt.SHADE_BVH, depth)
        want = np.array([colors[_first_left_first(nodes, r, depth)] for r in rays], np.float32)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=f"depth {depth}")
        seen |= {tuple(c) for c in want.tolist()}
    assert len(seen) == 3  # misses, box interiors and box edges all occur


def test_bvh_display_adds_material_and_wireframe_wins(scene):
    tris, models, nodes, rays, hits = scene
    base = O.shade(nodes, tris, models, MATERIALS, rays, hits, 0)
    bvh = O.shade(nodes, tris, models, MATERIALS, rays, hits, crt.SHADE_BVH, 2)
    both = O.shade(nodes, tris, models, MATERIALS, rays, hits, crt.SHADE_BVH | crt.SHADE_WIREFRAME, 2)
    wire = O.shade(nodes, tris, models, MATERIALS, rays, hits, crt.SHADE_WIREFRAME, 2)
    hit = hits[:, 0].view(np.uint32) != crt.MISS
    misses = hits.copy()
    misses[:, 0] = np.frombuffer(np.uint32(crt.MISS).tobytes(), np.float32)[0]
    box = O.shade(nodes, tris, models, MATERIALS, rays, misses, crt.SHADE_BVH, 2)
    mat = base - np.array([0, 0, 0, 1], np.float32)  # the material colour alone (exact: small dyadic values)
    np.testing.assert_array_equal(bvh[hit], box[hit] + mat[hit])
    np.testing.assert_array_equal(bvh[~hit], box[~hit])
    u, v = hits[:, 2], hits[:, 3]
    edge = hit & ((u < f32(0.02)) | (v < f32(0.02)) | ((f32(1) - u - v) < f32(0.02)))  # blacked out by the wireframe
    assert 0 < edge.sum() < hit.sum()
    assert np.all(wire[edge] == np.array([0, 0, 0, 1], np.float32))
    np.testing.assert_array_equal(both[edge], wire[edge])
    np.testing.assert_array_equal(both[hit & ~edge], bvh[hit & ~edge])


def test_ppm_writer(tmp_path):
    w, h = 3, 2
    tex = np.zeros((w * h, 4), np.float32)
    tex[0] = (1.0, 0.5, 0.0, 1.0)     # texel (0, 0): bottom-left of the displayed image
    tex[w * h - 1] = (2.0, -1.0, np.nan, 1.0)
    path = tmp_path / "frame.ppm"
    image.write_ppm(str(path), tex, w, h)
    data = path.read_bytes()
    head = b"P6\n3 2\n255\n"
    assert data.startswith(head)
    px = np.frombuffer(data[len(head):], np.uint8).reshape(h, w, 3)
    assert px[1, 0].tolist() == [255, 128, 0]     # bottom row, first column
    assert px[0, 2].tolist() == [255, 0, 0]       # top row, last column: clamped, NaN -> 0
    assert px.sum() == 255 + 128 + 255
