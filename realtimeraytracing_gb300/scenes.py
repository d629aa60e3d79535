"""Seeded synthetic scenes, cameras and record packing.

The reference loads OBJ meshes (srcCommon/scene/geometry/mesh.cpp:186-263)
and pads them into a 65,536-entry TriangleGPU buffer
(srcOpenGL/scene/scene.cpp:26-40).  These generators make the synthetic
scenes the benchmarks are defined on, with a counter-based SplitMix64 stream
and only IEEE-exact float64 arithmetic (+, -, *, /, sqrt) on the paths that
feed golden fixtures, so the same seed gives the same bytes on x86-64 and
aarch64.

Record layouts (see include/crt.h):
  triangles  (n, 16) float32: p0.xyzw, p1.xyzw, p2.xyzw, model id (uint32 bits), pad
  models     (m, 17) float32: column-major 4x4, material id (uint32 bits)
  rays       (n, 8)  float32: o.xyz, tmin, d.xyz, tmax
  hits       (n, 4)  float32: tri (uint32 bits), t, u, v
  materials  (m, 4)  float32: RGBA colour
  texels     (n, 4)  float32: RGBA, texel (x, y) at row y * width + x
  nodes      (2n-1, 12) float32: min.xyz, pad, max.xyz, pad, tri, left, right, pad (uint32 bits)
"""
from __future__ import annotations

import math

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, stream: int, n: int) -> np.ndarray:
    """n values of SplitMix64 for (seed, stream), counter based."""
    base = np.uint64((seed * 0x632BE59BD9B4E019 + stream * 0x2545F4914F6CDD1D + 1) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        z = base + (np.arange(1, n + 1, dtype=np.uint64) * _GOLD)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, stream: int, n: int) -> np.ndarray:
    """n float64 in [0, 1) with 53 random bits (exact)."""
    return (splitmix64(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def _unit_vectors(seed: int, stream: int, n: int) -> np.ndarray:
    """Uniform directions on S^2 by Marsaglia's disk method (only sqrt)."""
    out = np.empty((n, 3), np.float64)
    todo = np.arange(n)
    rnd = 0
    while todo.size:
        k = 8
        u = uniform01(seed, stream * 64 + rnd, todo.size * 2 * k).reshape(todo.size, k, 2) * 2.0 - 1.0
        s = u[..., 0] ** 2 + u[..., 1] ** 2
        ok = (s < 1.0) & (s > 1e-12)
        first = np.argmax(ok, axis=1)
        got = ok[np.arange(todo.size), first]
        sel = u[np.arange(todo.size), first]
        ss = s[np.arange(todo.size), first]
        r = np.sqrt(np.maximum(1.0 - ss, 0.0))
        v = np.stack([2.0 * sel[:, 0] * r, 2.0 * sel[:, 1] * r, 1.0 - 2.0 * ss], axis=1)
        out[todo[got]] = v[got]
        todo = todo[~got]
        rnd += 1
    return out


def _gaussian(seed: int, stream: int, n: int) -> np.ndarray:
    """Standard normals (Box-Muller; uses log/cos, so not for golden fixtures)."""
    u1 = uniform01(seed, stream, n)
    u2 = uniform01(seed, stream + 7919, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


def pack_triangles(v0: np.ndarray, v1: np.ndarray, v2: np.ndarray, model_id=0) -> np.ndarray:
    n = v0.shape[0]
    t = np.zeros((n, 16), np.float32)
    t[:, 0:3] = v0
    t[:, 4:7] = v1
    t[:, 8:11] = v2
    t[:, 3] = t[:, 7] = t[:, 11] = 1.0
    t.view(np.uint32)[:, 12] = model_id
    return t


def identity_models(n: int = 1) -> np.ndarray:
    m = np.zeros((n, 17), np.float32)
    m[:, [0, 5, 10, 15]] = 1.0
    return m


def models_with_materials(material_ids) -> np.ndarray:
    """Identity model records whose material ids are material_ids."""
    ids = np.asarray(material_ids, np.uint32).reshape(-1)
    m = identity_models(ids.shape[0])
    m.view(np.uint32)[:, 16] = ids
    return m


def materials(colors) -> np.ndarray:
    """crt_material records (m, 4) float32: RGBA colours (Material::_Color)."""
    return np.ascontiguousarray(np.asarray(colors, np.float32).reshape(-1, 4))


def uniform_soup(n: int, seed: int = 0, edge_lo: float = 0.001, edge_hi: float = 0.02) -> np.ndarray:
    """Random soup in the unit cube: centroid ~ U[0,1]^3, each vertex =
    centroid + L * u with L ~ U(edge_lo, edge_hi) and u uniform on S^2."""
    c = uniform01(seed, 1, 3 * n).reshape(n, 3)
    verts = []
    for k in range(3):
        L = edge_lo + uniform01(seed, 10 + k, n) * (edge_hi - edge_lo)
        u = _unit_vectors(seed, 20 + k, n)
        verts.append((c + L[:, None] * u).astype(np.float32))
    return pack_triangles(*verts)


def clustered_soup(n: int, clusters: int, sigma: float, edge_mu: float, edge_sigma: float, seed: int = 0) -> np.ndarray:
    """Gaussian blobs: cluster centres ~ U[0,1]^3, centroid = centre + sigma N(0,1)^3,
    vertex offsets of length lognormal(ln edge_mu, edge_sigma) in uniform directions."""
    centres = uniform01(seed, 101, 3 * clusters).reshape(clusters, 3)
    which = (splitmix64(seed, 102, n) % np.uint64(clusters)).astype(np.int64)
    g = _gaussian(seed, 103, 3 * n).reshape(n, 3)
    c = centres[which] + sigma * g
    verts = []
    for k in range(3):
        L = np.exp(math.log(edge_mu) + edge_sigma * _gaussian(seed, 110 + 2 * k, n))
        u = _unit_vectors(seed, 120 + k, n)
        verts.append((c + L[:, None] * u).astype(np.float32))
    return pack_triangles(*verts)


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere by midpoint subdivision: (vertices float64, faces uint32)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.sqrt((v ** 2).sum(1))[:, None]
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        edges = np.stack([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 1).reshape(-1, 2)
        key = np.minimum(edges[:, 0], edges[:, 1]) * (1 << 32) + np.maximum(edges[:, 0], edges[:, 1])
        uk, inv = np.unique(key, return_inverse=True)
        lo, hi = uk >> 32, uk & 0xFFFFFFFF
        mid = v[lo] + v[hi]
        mid /= np.sqrt((mid ** 2).sum(1))[:, None]
        base = v.shape[0]
        v = np.concatenate([v, mid])
        m = (inv.reshape(-1, 3) + base)
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                            np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return v, f.astype(np.uint32)


def _value_noise(p: np.ndarray, seed: int, octave: int) -> np.ndarray:
    """Value noise in [-1, 1]: hashed lattice values, smoothstep trilinear blend."""
    i0 = np.floor(p)
    fr = p - i0
    w = fr * fr * (3.0 - 2.0 * fr)
    ii = i0.astype(np.int64)
    out = np.zeros(p.shape[0])
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                h = ((ii[:, 0] + dx) * 73856093) ^ ((ii[:, 1] + dy) * 19349663) ^ ((ii[:, 2] + dz) * 83492791)
                h = (h.astype(np.uint64) + np.uint64((seed * 1000003 + octave * 7777) & 0xFFFFFFFF))
                with np.errstate(over="ignore"):
                    z = (h * _GOLD) ^ ((h * _GOLD) >> np.uint64(29))
                    z = z * _M1
                    z = z ^ (z >> np.uint64(32))
                val = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53) * 2.0 - 1.0
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += wx * wy * wz * val
    return out


def displaced_icosphere(level: int = 8, amplitude: float = 0.05, seed: int = 0):
    """Icosphere of radius 1 whose vertices move radially by `amplitude` times
    a 3-octave value noise (octave frequencies 2, 4, 8; weights 1, 1/2, 1/4,
    normalised).  Returns (vertices float32 (V,3), indices uint32 (F,3))."""
    v, f = icosphere(level)
    n = np.zeros(v.shape[0])
    for o, (fq, wgt) in enumerate(((2.0, 1.0), (4.0, 0.5), (8.0, 0.25))):
        n += wgt * _value_noise(v * fq + 17.0, seed, o)
    n /= 1.75
    v = v * (1.0 + amplitude * n)[:, None]
    return v.astype(np.float32), f


def indexed_to_triangles(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    return pack_triangles(verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]])


def camera_gpu_data(eye, yaw: float = -90.0, pitch: float = 0.0, fov: float = 45.0, near: float = 0.1,
                    aspect: float = 1.0, world_up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """crt_camera record (24 float32) following Camera::getGpuData
    (srcCommon/scene/camera.cpp:23-34, 44-66, 110-120): inverse of
    lookAt(eye, eye + at, up), eye (w = 1), plane width/height/near.
    Evaluated in float64; components below 1e-12 are snapped to 0 so the
    default yaw of -90 looks exactly along the z axis."""
    def snap(x):
        x = np.asarray(x, np.float64)
        return np.where(np.abs(x) < 1e-12, 0.0, x)
    yr, pr = math.radians(yaw), math.radians(pitch)
    front = snap([math.cos(yr) * math.cos(pr), math.sin(pr), math.sin(yr) * math.cos(pr)])
    at = front / np.linalg.norm(front)
    up_w = np.asarray(world_up, np.float64)
    right = np.cross(at, up_w); right /= np.linalg.norm(right)
    up = np.cross(right, at); up /= np.linalg.norm(up)
    # lookAt: f = at, s = normalize(cross(f, up)), u = cross(s, f); view rows s, u, -f
    f = at
    s = np.cross(f, up); s /= np.linalg.norm(s)
    u = np.cross(s, f)
    e = np.asarray(eye, np.float64)
    inv = np.zeros((4, 4))  # inverse view: columns s, u, -f, eye
    inv[:3, 0], inv[:3, 1], inv[:3, 2], inv[:3, 3], inv[3, 3] = s, u, -f, e, 1.0
    inv = snap(inv)
    rec = np.zeros(24, np.float32)
    rec[0:16] = inv.T.reshape(-1)  # column-major
    rec[16:19] = e
    rec[19] = 1.0
    ph = 2.0 * near * math.tan(0.5 * math.radians(fov))
    rec[20] = np.float32(ph * aspect)
    rec[21] = np.float32(ph)
    rec[22] = np.float32(near)
    return rec


# ---------------------------------------------------------------- workloads
def config0_scene(seed: int = 0):
    """65,536-triangle uniform soup, 512x512 camera at (0.5, 0.5, -1.5) toward +z."""
    tris = uniform_soup(65536, seed)
    cam = camera_gpu_data((0.5, 0.5, -1.5), aspect=1.0)
    return tris, identity_models(1), cam, (512, 512)


def config1_scene(seed: int = 0, level: int = 8):
    """Displaced icosphere (level 8: 1,310,720 triangles), 1920x1080 camera 3
    units out on -z looking toward +z, point light at (2, 2, -2)."""
    v, f = displaced_icosphere(level, 0.05, seed)
    tris = indexed_to_triangles(v, f)
    cam = camera_gpu_data((0.0, 0.0, -3.0), aspect=1920.0 / 1080.0)
    return tris, identity_models(1), cam, (1920, 1080), np.array([2.0, 2.0, -2.0], np.float32)


def config3_scene(seed: int = 0, n: int = 4194304):
    """4M-triangle clustered soup: 256 clusters, sigma 0.02, edges lognormal(ln 0.003, 0.6)."""
    return clustered_soup(n, 256, 0.02, 0.003, 0.6, seed), identity_models(1)


def sphere_rays(n: int, seed: int = 0, radius: float = 2.0, center=(0.5, 0.5, 0.5)) -> np.ndarray:
    """Rays from points uniform on a sphere toward points uniform in the unit cube."""
    o = np.asarray(center, np.float64) + radius * _unit_vectors(seed, 301, n)
    target = uniform01(seed, 302, 3 * n).reshape(n, 3)
    d = target - o
    d /= np.sqrt((d ** 2).sum(1))[:, None]
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 4:7] = d
    r[:, 7] = np.inf
    return r


def bounce_rays(prim: np.ndarray, hits: np.ndarray, tris: np.ndarray, n_out: int, seed: int = 0,
                chunk: int = 1 << 20) -> np.ndarray:
    """Cosine-weighted diffuse bounce rays from closest hits, on the host.

    Ray j leaves hit number (j * 2654435761 + seed) mod n_hits of the
    primary hits in ray order (so consecutive rays come from scattered
    pixels: an incoherent batch).  Its origin is the hit point o + t d, its
    direction normalize(n + u) with n the hit triangle's unit geometric
    normal turned toward the incoming ray and u uniform on S^2 (a
    cosine-weighted direction about n), and [tmin, tmax] = [1e-4, inf].
    Only IEEE-exact float64 arithmetic (+, -, *, /, sqrt) and the SplitMix64
    stream, so equal inputs give equal rays on every machine.  Triangles are
    (n, 16) records with identity models (their vertices as stored)."""
    tri = np.ascontiguousarray(hits[:, 0]).view(np.uint32)
    src = np.nonzero(tri != 0xFFFFFFFF)[0]
    out = np.zeros((n_out, 8), np.float32)
    if src.size == 0:
        out[:, 3] = 1.0  # empty rays: tmin 1 > tmax 0
        return out
    j = np.arange(n_out, dtype=np.uint64)
    with np.errstate(over="ignore"):
        pick = ((j * np.uint64(2654435761) + np.uint64(seed)) % np.uint64(src.size)).astype(np.int64)
    for c0 in range(0, n_out, chunk):
        c1 = min(n_out, c0 + chunk)
        k = src[pick[c0:c1]]
        o = prim[k, 0:3].astype(np.float64)
        d = prim[k, 4:7].astype(np.float64)
        t = hits[k, 1].astype(np.float64)
        p = (o + t[:, None] * d).astype(np.float32).astype(np.float64)
        tv = tris[tri[k]]
        a, b, cc = tv[:, 0:3].astype(np.float64), tv[:, 4:7].astype(np.float64), tv[:, 8:11].astype(np.float64)
        e1, e2 = b - a, cc - a
        nrm = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1],
                        e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                        e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], axis=1)
        ln = np.sqrt((nrm ** 2).sum(1))
        nrm /= np.where(ln > 0.0, ln, 1.0)[:, None]
        flip = (nrm * d).sum(1) > 0.0
        nrm[flip] = -nrm[flip]
        u = _unit_vectors(seed, 5000 + 8 * (c0 // chunk), c1 - c0)
        v = nrm + u
        lv = np.sqrt((v ** 2).sum(1))
        bad = lv < 1e-9
        v[bad] = nrm[bad]
        lv[bad] = 1.0
        v /= lv[:, None]
        out[c0:c1, 0:3] = p
        out[c0:c1, 3] = 1e-4
        out[c0:c1, 4:7] = v
        out[c0:c1, 7] = np.inf
    return out


def config3_rays(tris, models, primary_hits_fn, seed: int = 11, width: int = 2048, n_out: int = 8 * 1024 * 1024):
    """The incoherent-bounce rays of the hit-predictor workload: 2048x2048
    primary rays from (0.5, 0.5, -1.5) toward +z, their closest hits
    (watertight) from primary_hits_fn(rays) -> (n, 4) hits, then n_out
    cosine bounce rays (bounce_rays).  Returns (primary rays, primary hits,
    bounce rays)."""
    cam = camera_gpu_data((0.5, 0.5, -1.5))
    prim = pinhole_rays(cam, width, width)
    ph = primary_hits_fn(prim)
    return prim, ph, bounce_rays(prim, ph, tris, n_out, seed)


def pinhole_rays(cam: np.ndarray, width: int, height: int) -> np.ndarray:
    """getRay (raytracer.glsl:92-100) on the host in float32, operation for
    operation as the library's raygen (float32 division, glm mat*vec order,
    1/sqrt): ray (x, y) at row y * width + x."""
    f = np.float32
    cam = np.asarray(cam, np.float32)
    m = cam[0:16]
    eye = cam[16:20]
    pw_, ph_, pn_ = cam[20], cam[21], cam[22]
    xs = np.arange(width, dtype=np.float32) / f(width)
    ys = np.arange(height, dtype=np.float32) / f(height)
    px, py = np.meshgrid(xs, ys)
    v0 = (px - f(0.5)) * pw_
    v1 = (py - f(0.5)) * ph_
    v2 = np.full_like(v0, f(1.0) * pn_)
    v3 = np.full_like(v0, f(1.0))
    comp = []
    for r in range(4):
        a = m[0 + r] * v0 + m[4 + r] * v1
        b = m[8 + r] * v2 + m[12 + r] * v3
        comp.append(a + b)
    dx, dy, dz, dw = comp[0] - eye[0], comp[1] - eye[1], comp[2] - eye[2], comp[3] - eye[3]
    inv = f(1.0) / np.sqrt(((dx * dx + dy * dy) + dz * dz) + dw * dw)
    rays = np.zeros((height * width, 8), np.float32)
    rays[:, 0:3] = eye[0:3]
    rays[:, 4] = (dx * inv).reshape(-1)
    rays[:, 5] = (dy * inv).reshape(-1)
    rays[:, 6] = (dz * inv).reshape(-1)
    rays[:, 7] = np.inf
    return rays


def config2_sizes(n_scenes: int = 64, seed: int = 0, tri_range=(1000, 2_000_000), ray_range=(65536, 4_194_304)):
    """Log-uniform triangle and ray counts of the batched workload."""
    u = uniform01(seed, 401, n_scenes)
    v = uniform01(seed, 402, n_scenes)
    lt, ht = np.log(tri_range[0]), np.log(tri_range[1])
    lr, hr = np.log(ray_range[0]), np.log(ray_range[1])
    tris = np.floor(np.exp(lt + u * (ht - lt))).astype(np.int64)
    rays = np.floor(np.exp(lr + v * (hr - lr))).astype(np.int64)
    return tris, rays


def config2_scene(k: int, n_tris: int, seed: int = 0) -> np.ndarray:
    """Scene k of the batched workload: even k uniform soups (as config 0),
    odd k clustered soups (32 blobs, sigma 0.03, edges lognormal(ln 0.005, 0.5))."""
    if k % 2 == 0:
        return uniform_soup(int(n_tris), seed=seed * 1000 + k)
    return clustered_soup(int(n_tris), 32, 0.03, 0.005, 0.5, seed=seed * 1000 + k)


# ------------------------------------------------- on-device generators (torch)
# Same distributions as the numpy generators above, drawn on the GPU with a
# seeded torch generator (reproducible on the same device type); used where
# host generation of tens of millions of records would dominate a benchmark.
def _torch():
    import torch
    return torch


def device_soup(n: int, gen, clustered: bool = False, clusters: int = 32, sigma: float = 0.03,
                edge_mu: float = 0.005, edge_sigma: float = 0.5):
    torch = _torch()
    dev = gen.device
    if clustered:
        centres = torch.rand((clusters, 3), generator=gen, device=dev, dtype=torch.float64)
        which = torch.randint(0, clusters, (n,), generator=gen, device=dev)
        c = centres[which] + sigma * torch.randn((n, 3), generator=gen, device=dev, dtype=torch.float64)
    else:
        c = torch.rand((n, 3), generator=gen, device=dev, dtype=torch.float64)
    out = torch.zeros((n, 16), dtype=torch.float32, device=dev)
    for k in range(3):
        if clustered:
            L = torch.exp(np.log(edge_mu) + edge_sigma * torch.randn(n, generator=gen, device=dev, dtype=torch.float64))
        else:
            L = 0.001 + 0.019 * torch.rand(n, generator=gen, device=dev, dtype=torch.float64)
        u = torch.randn((n, 3), generator=gen, device=dev, dtype=torch.float64)
        u /= u.norm(dim=1, keepdim=True).clamp_min(1e-12)
        out[:, 4 * k:4 * k + 3] = (c + L[:, None] * u).float()
        out[:, 4 * k + 3] = 1.0
    return out


def device_sphere_rays(n: int, gen, radius: float = 2.0, center=(0.5, 0.5, 0.5)):
    torch = _torch()
    dev = gen.device
    u = torch.randn((n, 3), generator=gen, device=dev, dtype=torch.float64)
    u /= u.norm(dim=1, keepdim=True).clamp_min(1e-12)
    o = torch.tensor(center, dtype=torch.float64, device=dev) + radius * u
    d = torch.rand((n, 3), generator=gen, device=dev, dtype=torch.float64) - o
    d /= d.norm(dim=1, keepdim=True)
    r = torch.zeros((n, 8), dtype=torch.float32, device=dev)
    r[:, 0:3] = o.float()
    r[:, 4:7] = d.float()
    r[:, 7] = float("inf")
    return r
