// ORACLE — test infrastructure, never part of the product path.
//
// A CPU restatement of the reference's hot path, used by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg to check (and
// time beside) the CUDA library.  Nothing in realtimeraytracing_gb300/ links
// or calls it.
//
// Build side restates srcCommon/scene/geometry/bvh.cpp for any N (the
// reference caps N at 65,536, triangle.hpp:21):
//   scene box            bvh.cpp:235-251   (scans all n_buffer records)
//   circumscribed cube   bvh.cpp:253-303   (incl. the if/else-if axis pick)
//   centroids            bvh.cpp:305-312 -> triangle.cpp:31-33
//   normalised centroids bvh.cpp:314-328
//   Morton codes         bvh.cpp:330-372
//   (code, index) sort   bvh.cpp:214-232
//   leaf clusters        bvh.cpp:26-46, AABB::buildFromTriangle bvh.cpp:383-399
//   PLOC loop            bvh.cpp:48-123; NN search :193-210; merge :159-191;
//                        scan :125-148; compaction :150-156
//   surface area         bvh.cpp:378-381;  box merge bvh.cpp:401-413
//   DFS node layout      srcOpenGL/scene/scene.cpp:189-208
// Trace side restates srcCommon/shaders/raytracer.glsl:
//   getRay               raytracer.glsl:92-100
//   triangle test        raytracer.glsl:102-147 (GLSL field order _P0,_P2,_P1)
//   slab test            raytracer.glsl:182-221 (display border code dropped)
//   closest-hit DFS      raytracer.glsl:246-295 (right child popped first)
//   brute force          raytracer.glsl:149-157
// plus the watertight predicate (Woop, Benthin, Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013) the product also offers.
//
// Floating point: every expression is written in the reference's evaluation
// order and the file is compiled with -ffp-contract=off, so each operation
// rounds once (IEEE binary32, round to nearest).  min/max follow std::min /
// std::max and GLSL min/max: max(a,b) = a < b ? b : a, min(a,b) = b < a ? b : a.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#include "crt.h"

namespace {

inline float fmax_std(float a, float b) { return (a < b) ? b : a; }
inline float fmin_std(float a, float b) { return (b < a) ? b : a; }

struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };
struct Box { V3 mn, mx; };

const float kInf = std::numeric_limits<float>::infinity();

// glm mat4 * vec4: (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w), column-major m.
inline V4 mat_vec(const float* m, const V4& v) {
    V4 r;
    r.x = (m[0] * v.x + m[4] * v.y) + (m[8] * v.z + m[12] * v.w);
    r.y = (m[1] * v.x + m[5] * v.y) + (m[9] * v.z + m[13] * v.w);
    r.z = (m[2] * v.x + m[6] * v.y) + (m[10] * v.z + m[14] * v.w);
    r.w = (m[3] * v.x + m[7] * v.y) + (m[11] * v.z + m[15] * v.w);
    return r;
}

inline V4 load4(const float* p) { return V4{p[0], p[1], p[2], p[3]}; }

// Model matrices: 64 entries, ids >= n_models identity (scene.cpp:17-23).
struct Models {
    float m[64][16];
    Models(const crt_mesh_model* models, uint32_t n) {
        for (int i = 0; i < 64; ++i) {
            for (int k = 0; k < 16; ++k) m[i][k] = (k % 5 == 0) ? 1.f : 0.f;
            if (models && static_cast<uint32_t>(i) < n) std::memcpy(m[i], models[i].m, 64);
        }
    }
    const float* of(const crt_triangle& t) const { return m[t.model_id & 63u]; }
};

// AABB::buildFromTriangle (bvh.cpp:383-399)
inline Box leaf_box(const crt_triangle& t, const float* M) {
    const V4 p0 = mat_vec(M, load4(t.p0));
    const V4 p1 = mat_vec(M, load4(t.p1));
    const V4 p2 = mat_vec(M, load4(t.p2));
    Box b;
    b.mn.x = fmin_std(p0.x, fmin_std(p1.x, p2.x));
    b.mn.y = fmin_std(p0.y, fmin_std(p1.y, p2.y));
    b.mn.z = fmin_std(p0.z, fmin_std(p1.z, p2.z));
    b.mx.x = fmax_std(p0.x, fmax_std(p1.x, p2.x));
    b.mx.y = fmax_std(p0.y, fmax_std(p1.y, p2.y));
    b.mx.z = fmax_std(p0.z, fmax_std(p1.z, p2.z));
    return b;
}

// AABB::merge (bvh.cpp:401-413)
inline Box merge(const Box& a, const Box& b) {
    Box r;
    r.mn.x = fmin_std(a.mn.x, b.mn.x); r.mn.y = fmin_std(a.mn.y, b.mn.y); r.mn.z = fmin_std(a.mn.z, b.mn.z);
    r.mx.x = fmax_std(a.mx.x, b.mx.x); r.mx.y = fmax_std(a.mx.y, b.mx.y); r.mx.z = fmax_std(a.mx.z, b.mx.z);
    return r;
}

// AABB::getSurfaceArea (bvh.cpp:378-381): 2 * ((dx*dy + dy*dz) + dz*dx)
inline float surface_area(const Box& b) {
    const float dx = b.mx.x - b.mn.x, dy = b.mx.y - b.mn.y, dz = b.mx.z - b.mn.z;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

uint32_t expand_bits(uint32_t v) {  // bvh.cpp:350-356
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

inline uint32_t to_u10(float x) {  // bvh.cpp:363-367 incl. the float->uint cast
    x = fmin_std(fmax_std(x * 1024.0f, 0.0f), 1023.0f);
    if (x != x) return 0u;  // NaN: cvt to unsigned gives 0 on x86-64, aarch64 and CUDA
    return static_cast<uint32_t>(x);
}

uint32_t morton3d(V3 p) {  // bvh.cpp:358-372
    return (expand_bits(to_u10(p.x)) << 2) | (expand_bits(to_u10(p.y)) << 1) | expand_bits(to_u10(p.z));
}

// Scene box over all n_buffer records (bvh.cpp:235-251).
Box scene_box(const crt_triangle* tris, uint32_t n_buffer, const Models& M) {
    Box s{{kInf, kInf, kInf}, {-kInf, -kInf, -kInf}};
    for (uint32_t i = 0; i < n_buffer; ++i) {
        const float* m = M.of(tris[i]);
        const V4 p0 = mat_vec(m, load4(tris[i].p0));
        const V4 p1 = mat_vec(m, load4(tris[i].p1));
        const V4 p2 = mat_vec(m, load4(tris[i].p2));
        s.mx.x = fmax_std(s.mx.x, fmax_std(p0.x, fmax_std(p1.x, p2.x)));
        s.mx.y = fmax_std(s.mx.y, fmax_std(p0.y, fmax_std(p1.y, p2.y)));
        s.mx.z = fmax_std(s.mx.z, fmax_std(p0.z, fmax_std(p1.z, p2.z)));
        s.mn.x = fmin_std(s.mn.x, fmin_std(p0.x, fmin_std(p1.x, p2.x)));
        s.mn.y = fmin_std(s.mn.y, fmin_std(p0.y, fmin_std(p1.y, p2.y)));
        s.mn.z = fmin_std(s.mn.z, fmin_std(p0.z, fmin_std(p1.z, p2.z)));
    }
    return s;
}

// bvh.cpp:253-303, including the if / else-if axis choice that takes X
// whenever distX > 0.
Box circumscribed_cube(const Box& b) {
    Box c = b;
    const float dX = b.mx.x - b.mn.x, dY = b.mx.y - b.mn.y, dZ = b.mx.z - b.mn.z;
    float maxDist = 0.f;
    int axis = 0;
    if (dX > maxDist) { maxDist = dX; axis = 0; }
    else if (dY > maxDist) { maxDist = dY; axis = 1; }
    else { maxDist = dZ; axis = 2; }
    float delta;
    switch (axis) {
        case 0:
            delta = (maxDist - dY) / 2.f; c.mx.y += delta; c.mn.y -= delta;
            delta = (maxDist - dZ) / 2.f; c.mx.z += delta; c.mn.z -= delta;
            break;
        case 1:
            delta = (maxDist - dX) / 2.f; c.mx.x += delta; c.mn.x -= delta;
            delta = (maxDist - dZ) / 2.f; c.mx.z += delta; c.mn.z -= delta;
            break;
        default:
            delta = (maxDist - dX) / 2.f; c.mx.x += delta; c.mn.x -= delta;
            delta = (maxDist - dY) / 2.f; c.mx.y += delta; c.mn.y -= delta;
            break;
    }
    return c;
}

// Triangle::getCentroid(tri, M) (triangle.cpp:31-33):
// vec3(((1/3) * M) * ((P0 + P1) + P2)).
inline V3 centroid(const crt_triangle& t, const float* M) {
    const float third = 1.f / 3.f;
    float m3[16];
    for (int k = 0; k < 16; ++k) m3[k] = third * M[k];
    V4 s;
    s.x = t.p0[0] + t.p1[0] + t.p2[0];
    s.y = t.p0[1] + t.p1[1] + t.p2[1];
    s.z = t.p0[2] + t.p1[2] + t.p2[2];
    s.w = t.p0[3] + t.p1[3] + t.p2[3];
    const V4 c = mat_vec(m3, s);
    return V3{c.x, c.y, c.z};
}

struct BuildNode {
    Box box;
    uint32_t tri;       // leaf: triangle index
    uint32_t left, right;
    bool leaf;
};

}  // namespace

extern "C" {

// Morton codes of the first n_tris triangles, with the scene box and cube the
// reference derives on the way (bvh.cpp:330-348).
void oracle_morton(const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                   const crt_mesh_model* models, uint32_t n_models,
                   uint32_t* codes, float* scene6, float* cube6) {
    const Models M(models, n_models);
    const Box sb = scene_box(tris, n_buffer, M);
    const Box cube = circumscribed_cube(sb);
    if (scene6) { float v[6] = {sb.mn.x, sb.mn.y, sb.mn.z, sb.mx.x, sb.mx.y, sb.mx.z}; std::memcpy(scene6, v, 24); }
    if (cube6) { float v[6] = {cube.mn.x, cube.mn.y, cube.mn.z, cube.mx.x, cube.mx.y, cube.mx.z}; std::memcpy(cube6, v, 24); }
    for (uint32_t i = 0; i < n_tris; ++i) {
        const V3 c = centroid(tris[i], M.of(tris[i]));
        const float lx = cube.mx.x - cube.mn.x, ly = cube.mx.y - cube.mn.y, lz = cube.mx.z - cube.mn.z;
        const V3 nc{(c.x - cube.mn.x) / lx, (c.y - cube.mn.y) / ly, (c.z - cube.mn.z) / lz};
        codes[i] = morton3d(nc);
    }
}

// Full build.  Outputs (any may be null except nodes): sorted codes, the
// permutation, the node array (2*n_tris-1 records) and the PLOC iteration
// count.  faithful != 0 runs the PLOC scan as the reference's O(n log n)
// Hillis-Steele passes with OpenMP (bvh.cpp:125-148) and the merge counter in
// an omp critical section (bvh.cpp:175-179) — used when the oracle is timed as
// the CPU baseline; the output is identical either way.  Returns 0, or -1 on
// bad sizes.  ms[4] (optional) receives wall ms of morton / sort / ploc / layout.
int oracle_build(const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                 const crt_mesh_model* models, uint32_t n_models, uint32_t radius, int faithful,
                 uint32_t* codes_sorted, uint32_t* perm_out, crt_bvh_node* nodes,
                 uint32_t* iterations, double* ms) {
    using clk = std::chrono::steady_clock;
    if (n_tris == 0 || n_buffer < n_tris || n_models > 64 || nodes == nullptr) return -1;
    for (uint32_t i = 0; i < n_buffer; ++i)
        if (tris[i].model_id >= 64) return -1;
    const Models M(models, n_models);
    const auto t0 = clk::now();

    // --- Morton codes + sort (bvh.cpp:214-232) ---
    std::vector<uint32_t> codes(n_tris);
    oracle_morton(tris, n_buffer, n_tris, models, n_models, codes.data(), nullptr, nullptr);
    const auto t1 = clk::now();
    std::vector<std::pair<uint32_t, uint32_t>> pairs(n_tris);
    for (uint32_t i = 0; i < n_tris; ++i) pairs[i] = {codes[i], i};
    std::sort(pairs.begin(), pairs.end());
    const auto t2 = clk::now();
    if (codes_sorted) for (uint32_t i = 0; i < n_tris; ++i) codes_sorted[i] = pairs[i].first;
    if (perm_out) for (uint32_t i = 0; i < n_tris; ++i) perm_out[i] = pairs[i].second;

    // --- leaf clusters (bvh.cpp:26-46) ---
    const size_t total = 2 * static_cast<size_t>(n_tris) - 1;
    std::vector<BuildNode> cl(total);
    std::vector<uint32_t> cin(n_tris), cout(n_tris), nn(n_tris, 0), scan(n_tris, 0);
    std::vector<uint8_t> valid(n_tris, 1);
    for (uint32_t i = 0; i < n_tris; ++i) {
        const uint32_t ti = pairs[i].second;
        cl[i].box = leaf_box(tris[ti], M.of(tris[ti]));
        cl[i].tri = ti; cl[i].left = cl[i].right = 0; cl[i].leaf = true;
        cin[i] = i;
    }
    uint32_t n = n_tris, next_id = n_tris, iters = 0;
    std::vector<uint32_t> temp;

    // --- PLOC loop (bvh.cpp:62-122) ---
    while (n > 1) {
        ++iters;
        // nearest neighbour search (bvh.cpp:193-210)
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ++ii) {
            const uint32_t i = static_cast<uint32_t>(ii);
            float minDist = kInf;
            const Box bi = cl[cin[i]].box;
            const uint32_t s = static_cast<uint32_t>(std::max<int64_t>(0, static_cast<int64_t>(i) - radius));
            const uint32_t e = std::min<uint32_t>(i + radius + 1, n);
            for (uint32_t j = s; j < e; ++j) {
                if (j == i) continue;
                const float d = surface_area(merge(bi, cl[cin[j]].box));
                if (d < minDist) { minDist = d; nn[i] = j; }
            }
        }
        // merging (bvh.cpp:159-191): mutual pairs merge at the lower position
        std::fill(valid.begin(), valid.begin() + n, 1);
        if (faithful) {
#pragma omp parallel for schedule(static)
            for (int64_t ii = 0; ii < static_cast<int64_t>(n); ++ii) {
                const uint32_t i = static_cast<uint32_t>(ii), j = nn[i];
                if (nn[j] == i && i < j) {
                    uint32_t id;
#pragma omp critical
                    { id = next_id++; }
                    BuildNode& m = cl[id];
                    m.box = merge(cl[cin[i]].box, cl[cin[j]].box);
                    m.tri = 0; m.left = cin[i]; m.right = cin[j]; m.leaf = false;
                    valid[j] = 0;
                    cin[i] = id;
                }
            }
        } else {
            for (uint32_t i = 0; i < n; ++i) {
                const uint32_t j = nn[i];
                if (nn[j] == i && i < j) {
                    const uint32_t id = next_id++;
                    BuildNode& m = cl[id];
                    m.box = merge(cl[cin[i]].box, cl[cin[j]].box);
                    m.tri = 0; m.left = cin[i]; m.right = cin[j]; m.leaf = false;
                    valid[j] = 0;
                    cin[i] = id;
                }
            }
        }
        // exclusive scan of validity (bvh.cpp:125-148)
        if (faithful) {
            scan[0] = 0;
#pragma omp parallel for schedule(static)
            for (int64_t i = 1; i < static_cast<int64_t>(n); ++i) scan[i] = valid[i - 1];
            temp.assign(n, 0);
            for (int64_t step = 1; step < static_cast<int64_t>(n); step *= 2) {
#pragma omp parallel for schedule(static)
                for (int64_t i = step; i < static_cast<int64_t>(n); ++i) temp[i] = scan[i] + scan[i - step];
#pragma omp parallel for schedule(static)
                for (int64_t i = step; i < static_cast<int64_t>(n); ++i) { scan[i] = temp[i]; temp[i] = 0; }
            }
        } else {
            uint32_t acc = 0;
            for (uint32_t i = 0; i < n; ++i) { scan[i] = acc; acc += valid[i]; }
        }
        // compaction (bvh.cpp:150-156) and loop update (bvh.cpp:105-113)
        for (uint32_t i = 0; i < n; ++i)
            if (valid[i]) cout[scan[i]] = cin[i];
        n = scan[n - 1] + (valid[n - 1] ? 1u : 0u);
        std::swap(cin, cout);
    }
    const auto t3 = clk::now();

    // --- DFS pre-order, left first (scene.cpp:189-208); root = last node ---
    {
        struct Fr { uint32_t id, pos; int st; };
        std::vector<Fr> st;
        size_t w = 0;
        auto emit = [&](uint32_t id) -> uint32_t {
            crt_bvh_node o{};
            const BuildNode& b = cl[id];
            o.mn[0] = b.box.mn.x; o.mn[1] = b.box.mn.y; o.mn[2] = b.box.mn.z;
            o.mx[0] = b.box.mx.x; o.mx[1] = b.box.mx.y; o.mx[2] = b.box.mx.z;
            o.tri = b.leaf ? b.tri : 0u;
            o.left = 0; o.right = 0;
            nodes[w] = o;
            return static_cast<uint32_t>(w++);
        };
        const uint32_t root = static_cast<uint32_t>(total - 1);
        st.push_back({root, emit(root), 0});
        while (!st.empty()) {
            Fr& f = st.back();
            if (cl[f.id].leaf || f.st == 2) { st.pop_back(); continue; }
            const uint32_t c = (f.st == 0) ? cl[f.id].left : cl[f.id].right;
            const uint32_t p = emit(c);
            if (f.st == 0) nodes[f.pos].left = p; else nodes[f.pos].right = p;
            f.st += 1;
            st.push_back({c, p, 0});
        }
        if (w != total) return -2;
    }
    const auto t4 = clk::now();
    if (iterations) *iterations = iters;
    if (ms) {
        ms[0] = std::chrono::duration<double, std::milli>(t1 - t0).count();
        ms[1] = std::chrono::duration<double, std::milli>(t2 - t1).count();
        ms[2] = std::chrono::duration<double, std::milli>(t3 - t2).count();
        ms[3] = std::chrono::duration<double, std::milli>(t4 - t3).count();
    }
    return 0;
}

}  // extern "C"

// ===================================================================== trace
namespace {

inline V3 sub3(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }  // glm/GLSL dot order
inline V3 cross3(V3 a, V3 b) {
    return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
inline V3 normalize3(V3 v) {  // v * inversesqrt(dot(v, v)), inversesqrt = 1 / sqrt
    const float inv = 1.0f / std::sqrt(dot3(v, v));
    return V3{v.x * inv, v.y * inv, v.z * inv};
}

struct XTri { V3 a, b, c; };  // vertices after the model matrix, C++ field order P0, P1, P2

inline XTri xform(const crt_triangle& t, const Models& M) {
    const float* m = M.of(t);
    const V4 p0 = mat_vec(m, load4(t.p0)), p1 = mat_vec(m, load4(t.p1)), p2 = mat_vec(m, load4(t.p2));
    return XTri{{p0.x, p0.y, p0.z}, {p1.x, p1.y, p1.z}, {p2.x, p2.y, p2.z}};
}

struct Hit { bool did; float t, u, v; };

// raytracer.glsl:102-147.  The GLSL struct lists the vec4s as _P0, _P2, _P1,
// so the shader's p1 is the C++ P2 and its p2 is the C++ P1.
inline Hit tri_reference(const crt_ray& r, const XTri& x) {
    Hit h{false, 0.f, 0.f, 0.f};
    const V3 p0 = x.a, p1 = x.c, p2 = x.b;
    const V3 d{r.d[0], r.d[1], r.d[2]};
    const V3 e0 = sub3(p1, p0);
    const V3 e1 = sub3(p2, p0);
    const V3 n = normalize3(cross3(e1, e0));
    const V3 q = cross3(d, e1);
    const float a = dot3(e0, q);
    const float eps = 1e-4f;
    if (dot3(n, d) >= 0.f || std::fabs(a) < eps) return h;
    const V3 s{(r.o[0] - p0.x) / a, (r.o[1] - p0.y) / a, (r.o[2] - p0.z) / a};
    const V3 rr = cross3(s, e0);
    const float u = dot3(s, q);
    const float v = dot3(rr, d);
    const float w = 1.0f - u - v;
    if (u < 0.f || v < 0.f || w < 0.f) return h;
    const float t = dot3(e1, rr);
    if (t < r.tmin || t > r.tmax) return h;  // t < 0 in the shader; [tmin, tmax] generalises it
    h.did = true; h.t = t; h.u = u; h.v = v;
    return h;
}

struct WRay { int kx, ky, kz; float Sx, Sy, Sz; };

inline WRay wt_setup(const crt_ray& r) {
    const float ax = std::fabs(r.d[0]), ay = std::fabs(r.d[1]), az = std::fabs(r.d[2]);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (r.d[kz] < 0.f) std::swap(kx, ky);
    WRay w;
    w.kx = kx; w.ky = ky; w.kz = kz;
    w.Sx = r.d[kx] / r.d[kz];
    w.Sy = r.d[ky] / r.d[kz];
    w.Sz = 1.0f / r.d[kz];
    return w;
}

inline float comp(const V3& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Watertight test, two-sided, with the double-precision fallback for zero
// edge functions (JCGT 2013, section 3).
inline Hit tri_watertight(const crt_ray& r, const WRay& w, const XTri& x) {
    Hit h{false, 0.f, 0.f, 0.f};
    const V3 o{r.o[0], r.o[1], r.o[2]};
    const V3 A = sub3(x.a, o), B = sub3(x.b, o), C = sub3(x.c, o);
    const float Ax = comp(A, w.kx) - w.Sx * comp(A, w.kz);
    const float Ay = comp(A, w.ky) - w.Sy * comp(A, w.kz);
    const float Bx = comp(B, w.kx) - w.Sx * comp(B, w.kz);
    const float By = comp(B, w.ky) - w.Sy * comp(B, w.kz);
    const float Cx = comp(C, w.kx) - w.Sx * comp(C, w.kz);
    const float Cy = comp(C, w.ky) - w.Sy * comp(C, w.kz);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = static_cast<float>(static_cast<double>(Cx) * By - static_cast<double>(Cy) * Bx);
        V = static_cast<float>(static_cast<double>(Ax) * Cy - static_cast<double>(Ay) * Cx);
        W = static_cast<float>(static_cast<double>(Bx) * Ay - static_cast<double>(By) * Ax);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return h;
    const float det = U + V + W;
    if (det == 0.f) return h;
    const float Az = w.Sz * comp(A, w.kz);
    const float Bz = w.Sz * comp(B, w.kz);
    const float Cz = w.Sz * comp(C, w.kz);
    const float T = U * Az + V * Bz + W * Cz;
    const float t = T / det;
    if (!(t >= r.tmin) || !(t <= r.tmax)) return h;
    h.did = true; h.t = t; h.u = V / det; h.v = W / det;
    return h;
}

// raytracer.glsl:182-221 with GLSL min/max semantics and its early exits.
inline bool slab_reference(const crt_ray& r, const crt_bvh_node& n) {
    const float ix = 1.0f / r.d[0];
    const float tx1 = (n.mn[0] - r.o[0]) * ix, tx2 = (n.mx[0] - r.o[0]) * ix;
    float tMin = fmin_std(tx1, tx2), tMax = fmax_std(tx1, tx2);
    if (tMax < 0.f || tMin > tMax) return false;
    const float iy = 1.0f / r.d[1];
    const float ty1 = (n.mn[1] - r.o[1]) * iy, ty2 = (n.mx[1] - r.o[1]) * iy;
    tMin = fmax_std(tMin, fmin_std(ty1, ty2));
    tMax = fmin_std(tMax, fmax_std(ty1, ty2));
    if (tMax < 0.f || tMin > tMax) return false;
    const float iz = 1.0f / r.d[2];
    const float tz1 = (n.mn[2] - r.o[2]) * iz, tz2 = (n.mx[2] - r.o[2]) * iz;
    tMin = fmax_std(tMin, fmin_std(tz1, tz2));
    tMax = fmin_std(tMax, fmax_std(tz1, tz2));
    return tMax >= 0.f && tMin <= tMax;
}

// Generous box test for the watertight oracle: double precision, box grown
// by 1e-5 of its own scale, so every triangle the float test can hit is reached.
// *enter (optional) receives the entry distance along d.
inline bool slab_loose(const crt_ray& r, const crt_bvh_node& n, double* enter = nullptr) {
    double t0 = -1e300, t1 = 1e300;
    for (int k = 0; k < 3; ++k) {
        const double pad = 1e-5 * (1.0 + std::fabs(static_cast<double>(n.mn[k])) + std::fabs(static_cast<double>(n.mx[k])));
        const double lo = n.mn[k] - pad, hi = n.mx[k] + pad, o = r.o[k], d = r.d[k];
        if (d == 0.0) {
            if (o < lo || o > hi) return false;
            continue;
        }
        double a = (lo - o) / d, b = (hi - o) / d;
        if (a > b) std::swap(a, b);
        t0 = std::max(t0, a); t1 = std::min(t1, b);
    }
    if (enter) *enter = t0;
    return t1 >= std::min(0.0, static_cast<double>(r.tmin)) - 1e-6 && t0 <= t1 &&
           t0 <= static_cast<double>(r.tmax) * (1.0 + 1e-5) + 1e-6;
}

// Pruned walk of oracle_trace (ORACLE_PRUNED): the nearer child first, and a
// box only when it can hold a hit at t <= the best t so far (the box test
// with tmax = best t keeps every box a tying hit could lie in).  It finds the
// same closest hit (same tie rule) as the full walk; tests pin that, and it
// serves only to make large test inputs (the hits a bounce ray starts from).
constexpr uint32_t kOraclePruned = 0x100u;

}  // namespace

extern "C" {

// getRay (raytracer.glsl:92-100) for a width x height image; pos = texel / size.
void oracle_raygen(const crt_camera* cam, uint32_t width, uint32_t height, crt_ray* rays) {
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x) {
            const float px = static_cast<float>(x) / static_cast<float>(width);
            const float py = static_cast<float>(y) / static_cast<float>(height);
            const V4 pv{(px - 0.5f) * cam->plane_width, (py - 0.5f) * cam->plane_height, 1.0f * cam->plane_near, 1.0f};
            const V4 pw = mat_vec(cam->inv_view, pv);
            const float dx = pw.x - cam->eye[0], dy = pw.y - cam->eye[1], dz = pw.z - cam->eye[2], dw = pw.w - cam->eye[3];
            const float inv = 1.0f / std::sqrt(((dx * dx + dy * dy) + dz * dz) + dw * dw);
            crt_ray& r = rays[static_cast<size_t>(y) * width + x];
            r.o[0] = cam->eye[0]; r.o[1] = cam->eye[1]; r.o[2] = cam->eye[2];
            r.d[0] = dx * inv; r.d[1] = dy * inv; r.d[2] = dz * inv;
            r.tmin = 0.f; r.tmax = kInf;
        }
}

void oracle_shadow_rays(const crt_ray* prim, const crt_hit* hits, uint32_t n, const float* light, crt_ray* out) {
    for (uint32_t i = 0; i < n; ++i) {
        crt_ray& s = out[i];
        if (hits[i].tri == CRT_MISS) {
            std::memset(&s, 0, sizeof(s));
            s.tmin = 1.f; s.tmax = 0.f;
            continue;
        }
        const float t = hits[i].t;
        const float px = prim[i].o[0] + t * prim[i].d[0];
        const float py = prim[i].o[1] + t * prim[i].d[1];
        const float pz = prim[i].o[2] + t * prim[i].d[2];
        const float lx = light[0] - px, ly = light[1] - py, lz = light[2] - pz;
        const float len = std::sqrt((lx * lx + ly * ly) + lz * lz);
        const float inv = 1.0f / len;
        s.o[0] = px; s.o[1] = py; s.o[2] = pz;
        s.d[0] = lx * inv; s.d[1] = ly * inv; s.d[2] = lz * inv;
        s.tmin = 1e-4f; s.tmax = len;
    }
}

// Trace over the node array (reference layout).  flags as in crt.h.
//   CRT_TRI_REFERENCE: the shader's DFS (right child popped first, no t
//     pruning); a hit replaces the closest when none is held or its t is
//     smaller, so equal t keeps the first leaf visited.  A miss never
//     replaces a hit (the shader's :279 compares an unset t there).
//   CRT_TRI_WATERTIGHT: every triangle reachable through a generously grown
//     box is tested; equal t keeps the lower triangle index.
//   0x100 (with CRT_TRI_WATERTIGHT, closest hit): the pruned walk above, for
//     making large test inputs only; same hits, far fewer boxes.
// stats (optional, 2 x uint64): nodes whose box was tested, triangles tested.
void oracle_trace(const crt_bvh_node* nodes, uint32_t n_nodes, const crt_triangle* tris, uint32_t n_tris,
                  const crt_mesh_model* models, uint32_t n_models, const crt_ray* rays, uint32_t n_rays,
                  uint32_t flags, crt_hit* hits, uint64_t* stats) {
    const Models M(models, n_models);
    std::vector<XTri> xt(n_tris);
    for (uint32_t i = 0; i < n_tris; ++i) xt[i] = xform(tris[i], M);
    const bool any = (flags & CRT_TRACE_ANY) != 0;
    const bool wt = (flags & CRT_TRI_WATERTIGHT) != 0;
    const bool pruned = wt && !any && (flags & kOraclePruned) != 0;
    uint64_t visited = 0, tested = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : visited, tested)
    for (int64_t ri = 0; ri < static_cast<int64_t>(n_rays); ++ri) {
        const crt_ray& r = rays[ri];
        crt_hit out{CRT_MISS, 0.f, 0.f, 0.f};
        if (n_nodes == 0 || !(r.tmin <= r.tmax)) { hits[ri] = out; continue; }
        const WRay w = wt ? wt_setup(r) : WRay{};
        bool have = false;
        float bt = 0.f;
        uint32_t bid = 0;
        // one stack per thread, reused across its rays
        static thread_local std::vector<uint32_t> stack;
        stack.clear();
        stack.push_back(0);
        crt_ray rb = r;  // the pruned walk's box-test ray: tmax = best t
        while (!stack.empty()) {
            const uint32_t ni = stack.back();
            stack.pop_back();
            const crt_bvh_node& nd = nodes[ni];
            ++visited;
            if (pruned) {
                if (!slab_loose(rb, nd)) continue;
                if (!(nd.left == 0 && nd.right == 0)) {
                    double el = 0.0, er = 0.0;
                    const bool hl = slab_loose(rb, nodes[nd.left], &el);
                    const bool hr = slab_loose(rb, nodes[nd.right], &er);
                    if (hl && hr) {
                        stack.push_back(el <= er ? nd.right : nd.left);
                        stack.push_back(el <= er ? nd.left : nd.right);
                    } else if (hl) {
                        stack.push_back(nd.left);
                    } else if (hr) {
                        stack.push_back(nd.right);
                    }
                    continue;
                }
            } else if (!(wt ? slab_loose(r, nd) : slab_reference(r, nd))) {
                continue;
            }
            if (nd.left == 0 && nd.right == 0) {
                ++tested;
                const Hit h = wt ? tri_watertight(r, w, xt[nd.tri]) : tri_reference(r, xt[nd.tri]);
                if (!h.did) continue;
                if (any) { have = true; bid = nd.tri; bt = h.t; out.u = h.u; out.v = h.v; break; }
                const bool better = !have || h.t < bt || (wt && h.t == bt && nd.tri < bid);
                if (better) {
                    have = true; bt = h.t; bid = nd.tri; out.u = h.u; out.v = h.v;
                    rb.tmax = bt;
                }
            } else {
                stack.push_back(nd.left);
                stack.push_back(nd.right);
            }
        }
        if (have) { out.tri = bid; out.t = bt; }
        hits[ri] = out;
    }
    if (stats) { stats[0] = visited; stats[1] = tested; }
}

// Brute force over all triangles (raytracer.glsl:149-157): closest hit, equal t
// keeps the lower triangle index; any-hit stops at the first.
void oracle_trace_brute(const crt_triangle* tris, uint32_t n_tris, const crt_mesh_model* models, uint32_t n_models,
                        const crt_ray* rays, uint32_t n_rays, uint32_t flags, crt_hit* hits) {
    const Models M(models, n_models);
    std::vector<XTri> xt(n_tris);
    for (uint32_t i = 0; i < n_tris; ++i) xt[i] = xform(tris[i], M);
    const bool any = (flags & CRT_TRACE_ANY) != 0;
    const bool wt = (flags & CRT_TRI_WATERTIGHT) != 0;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ri = 0; ri < static_cast<int64_t>(n_rays); ++ri) {
        const crt_ray& r = rays[ri];
        crt_hit out{CRT_MISS, 0.f, 0.f, 0.f};
        if (!(r.tmin <= r.tmax)) { hits[ri] = out; continue; }
        const WRay w = wt ? wt_setup(r) : WRay{};
        bool have = false;
        for (uint32_t i = 0; i < n_tris; ++i) {
            const Hit h = wt ? tri_watertight(r, w, xt[i]) : tri_reference(r, xt[i]);
            if (!h.did) continue;
            if (!have || h.t < out.t) { have = true; out.tri = i; out.t = h.t; out.u = h.u; out.v = h.v; }
            if (any) break;
        }
        hits[ri] = out;
    }
}

}  // extern "C"

// ===================================================================== shade
namespace {

// intersectBVH (raytracer.glsl:182-236) with its border test: 0 = miss,
// 1 = hit, 2 = hit whose entry point o + d * tMin lies within `line` of a
// face of the box on at least two axes.
inline int slab_display(const crt_ray& r, const crt_bvh_node& n, float line) {
    const float ix = 1.0f / r.d[0];
    const float tx1 = (n.mn[0] - r.o[0]) * ix, tx2 = (n.mx[0] - r.o[0]) * ix;
    float tMin = fmin_std(tx1, tx2), tMax = fmax_std(tx1, tx2);
    if (tMax < 0.f || tMin > tMax) return 0;
    const float iy = 1.0f / r.d[1];
    const float ty1 = (n.mn[1] - r.o[1]) * iy, ty2 = (n.mx[1] - r.o[1]) * iy;
    tMin = fmax_std(tMin, fmin_std(ty1, ty2));
    tMax = fmin_std(tMax, fmax_std(ty1, ty2));
    if (tMax < 0.f || tMin > tMax) return 0;
    const float iz = 1.0f / r.d[2];
    const float tz1 = (n.mn[2] - r.o[2]) * iz, tz2 = (n.mx[2] - r.o[2]) * iz;
    tMin = fmax_std(tMin, fmin_std(tz1, tz2));
    tMax = fmin_std(tMax, fmax_std(tz1, tz2));
    if (!(tMax >= 0.f && tMin <= tMax)) return 0;
    bool close[3];
    for (int k = 0; k < 3; ++k) {
        const float e = r.o[k] + r.d[k] * tMin;
        close[k] = std::fabs(e - n.mn[k]) < line || std::fabs(e - n.mx[k]) < line;
    }
    return ((close[0] && close[1]) || (close[0] && close[2]) || (close[1] && close[2])) ? 2 : 1;
}

// bvhColor as getClosestHitBVH leaves it (raytracer.glsl:246-277): the
// shader's own walk — pop a node, test its box, on a hit assign bvhColor if
// its depth is D, then push left and right (right popped first) — where the
// last assignment stands.  Nodes below depth D cannot assign, so the walk
// does not push past depth D.
inline V4 bvh_color(const crt_bvh_node* nodes, uint32_t n_nodes, const crt_ray& r, uint32_t D) {
    const float line = 0.05f / (static_cast<float>(D) + 1.f);
    V4 color{0.f, 0.f, 0.f, 0.f};
    if (n_nodes == 0) return color;
    std::vector<std::pair<uint32_t, uint32_t>> stack{{0u, 0u}};
    while (!stack.empty()) {
        const auto [ni, depth] = stack.back();
        stack.pop_back();
        const crt_bvh_node& nd = nodes[ni];
        const int hit = slab_display(r, nd, line);
        if (hit == 0) continue;
        if (depth == D) color = hit == 2 ? V4{0.7f, 0.f, 0.7f, 0.1f} : V4{0.5f, 0.f, 0.5f, 0.1f};
        const bool leaf = nd.left == 0 && nd.right == 0;
        if (!leaf && depth < D) {
            stack.push_back({nd.left, depth + 1});
            stack.push_back({nd.right, depth + 1});
        }
    }
    return color;
}

}  // namespace

extern "C" {

// getColor + imageStore (raytracer.glsl:159-179, 319-330) for hit i of ray i
// into rgba[4i .. 4i+3].  Material of a hit: the triangle's model's
// material_id (model ids >= n_models: 0), colour (0,0,0,0) for material ids
// >= n_materials.  flags: CRT_SHADE_WIREFRAME | CRT_SHADE_BVH; depth =
// uDepthDisplayBVH.
void oracle_shade(const crt_bvh_node* nodes, uint32_t n_nodes, const crt_triangle* tris, uint32_t n_tris,
                  const crt_mesh_model* models, uint32_t n_models, const float* materials, uint32_t n_materials,
                  const crt_ray* rays, const crt_hit* hits, uint32_t n, uint32_t flags, uint32_t depth, float* rgba) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) {
        V4 value{0.f, 0.f, 0.f, 1.f};
        if (flags & CRT_SHADE_BVH) value = bvh_color(nodes, n_nodes, rays[i], depth);
        const crt_hit& h = hits[i];
        if (h.tri != CRT_MISS && h.tri < n_tris) {
            const uint32_t model = tris[h.tri].model_id;
            const uint32_t mat = (models && model < n_models) ? models[model].material_id : 0u;
            V4 c{0.f, 0.f, 0.f, 0.f};
            if (mat < n_materials) c = load4(materials + 4 * static_cast<size_t>(mat));
            value = V4{value.x + c.x, value.y + c.y, value.z + c.z, value.w + c.w};
            if (flags & CRT_SHADE_WIREFRAME) {
                const float w = 1.0f - h.u - h.v;
                if (h.u < 0.02f || h.v < 0.02f || w < 0.02f) value = V4{0.f, 0.f, 0.f, 1.f};
            }
        }
        float* o = rgba + 4 * static_cast<size_t>(i);
        o[0] = value.x; o[1] = value.y; o[2] = value.z; o[3] = value.w;
    }
}

}  // extern "C"

// ===================================================================== refit
extern "C" {

// Refit of a DFS node array (the product's crt_refit): topology kept, boxes
// recomputed from the moved triangles — leaves as AABB::buildFromTriangle
// (bvh.cpp:383-399), internal nodes as AABB::merge(left, right)
// (bvh.cpp:401-413), children before parents (in pre-order every child
// follows its parent, so a reverse sweep suffices).  nodes is updated in place.
void oracle_refit(crt_bvh_node* nodes, uint32_t n_nodes, const crt_triangle* tris, uint32_t n_tris,
                  const crt_mesh_model* models, uint32_t n_models) {
    const Models M(models, n_models);
    for (int64_t d = static_cast<int64_t>(n_nodes) - 1; d >= 0; --d) {
        crt_bvh_node& nd = nodes[d];
        Box b;
        if (nd.left == 0 && nd.right == 0) {
            if (nd.tri >= n_tris) continue;
            b = leaf_box(tris[nd.tri], M.of(tris[nd.tri]));
        } else {
            const crt_bvh_node& l = nodes[nd.left];
            const crt_bvh_node& r = nodes[nd.right];
            b = merge(Box{{l.mn[0], l.mn[1], l.mn[2]}, {l.mx[0], l.mx[1], l.mx[2]}},
                      Box{{r.mn[0], r.mn[1], r.mn[2]}, {r.mx[0], r.mx[1], r.mx[2]}});
        }
        nd.mn[0] = b.mn.x; nd.mn[1] = b.mn.y; nd.mn[2] = b.mn.z;
        nd.mx[0] = b.mx.x; nd.mx[1] = b.mx.y; nd.mx[2] = b.mx.z;
    }
}

}  // extern "C"

// ==================================================== treelet restructuring
// The product's crt_optimize, restated serially: treelet restructuring after
// Karras & Aila, "Fast Parallel Construction of High-Quality Bounding Volume
// Hierarchies" (HPG 2013), with the product's fixed rules so that the result
// is one exact tree.  No counterpart in the reference.
//
// Ids: leaves 0..N-1 in DFS order, internal nodes N + their rank in DFS order
// (the root is N).  Cost model: a leaf costs its box area, an internal node
// kCi * area + (cost(left) + cost(right)).  One pass visits every internal
// node children first; at node R it sets R's box (AABB::merge(left, right)),
// leaf count, height and cost, and if R has at least 7 leaves it forms R's
// treelet and rebuilds it optimally:
//   * treelet leaves start as [left, right]; 5 times the one with the largest
//     area (ordered-key compare; ties: the lowest index) among those that are
//     internal nodes is replaced in place by its left child and its right
//     child appended; the replaced nodes (R first) are the treelet's ids;
//   * area of each subset s of the 7: the union of its members' boxes taken
//     in increasing index, as AABB::merge(union, member);
//   * C[{k}] = cost of member k; C[s] = kCi * A[s] + min over p (C[p] +
//     C[s ^ p]) for p containing the lowest member of s, p != s; the minimum
//     by (ordered key of the sum, p), so the smallest p wins ties; p is the
//     left child;
//   * if C[all] < cost(R) the treelet is rebuilt: internal subsets take the
//     treelet's ids in pre-order (left first), each gets its union box, C[s],
//     leaf count and height.
// Passes repeat over the current tree; the result is laid out in DFS
// pre-order, left first, as the build lays out its tree.
namespace {

constexpr float kOptCi = 1.2f;

inline uint32_t ordered_key_f(float v) {
    uint32_t b;
    std::memcpy(&b, &v, 4);
    if ((b & 0x7FFFFFFFu) == 0u) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

struct OptTree {
    uint32_t N = 0;
    std::vector<Box> box;           // per id
    std::vector<uint32_t> tri;      // per leaf
    std::vector<float> cost;        // per id
    std::vector<uint32_t> nl, height, parent;
    std::vector<uint32_t> kl, kr;   // per internal id - N
};

void opt_treelet(OptTree& t, uint32_t R) {
    const uint32_t N = t.N;
    uint32_t L[7], I[6];
    int n = 2;
    L[0] = t.kl[R - N];
    L[1] = t.kr[R - N];
    I[0] = R;
    for (int e = 0; e < 5; ++e) {
        int best = -1;
        uint32_t bk = 0;
        for (int j = 0; j < n; ++j) {
            if (L[j] < N) continue;
            const uint32_t k = ordered_key_f(surface_area(t.box[L[j]]));
            if (best < 0 || k > bk) { best = j; bk = k; }
        }
        const uint32_t X = L[best];
        L[best] = t.kl[X - N];
        L[n++] = t.kr[X - N];
        I[e + 1] = X;
    }
    Box U[128];
    float A[128], Cs[128];
    uint8_t P[128] = {};
    for (uint32_t s = 1; s < 128; ++s) {
        int k0 = 0;
        while (!((s >> k0) & 1u)) ++k0;
        Box u = t.box[L[k0]];
        for (int k = k0 + 1; k < 7; ++k)
            if ((s >> k) & 1u) u = merge(u, t.box[L[k]]);
        U[s] = u;
        A[s] = surface_area(u);
    }
    for (int k = 0; k < 7; ++k) Cs[1u << k] = t.cost[L[k]];
    for (int size = 2; size <= 7; ++size) {
        for (uint32_t s = 1; s < 128; ++s) {
            if (__builtin_popcount(s) != size) continue;
            const uint32_t low = s & (0u - s), rest = s ^ low;
            uint32_t bp = 0, bkey = 0;
            float bv = 0.f;
            bool first = true;
            for (uint32_t q = 0;; q = (q - rest) & rest) {  // subsets of rest in increasing order
                if (q == rest) break;
                const uint32_t p = low | q;
                const float v = Cs[p] + Cs[s ^ p];
                const uint32_t key = ordered_key_f(v);
                if (first || key < bkey) { bp = p; bkey = key; bv = v; first = false; }
            }
            P[s] = static_cast<uint8_t>(bp);
            Cs[s] = kOptCi * A[s] + bv;
        }
    }
    if (!(Cs[127] < t.cost[R])) return;
    // ids in pre-order, left first
    uint32_t sid[128];
    for (int k = 0; k < 7; ++k) sid[1u << k] = L[k];
    uint32_t order[6];
    int n_int = 0, next = 0;
    uint32_t stack[8];
    int sp = 0;
    stack[sp++] = 127;
    while (sp > 0) {
        const uint32_t s = stack[--sp];
        if (__builtin_popcount(s) < 2) continue;
        sid[s] = I[next++];
        order[n_int++] = s;
        stack[sp++] = s ^ P[s];
        stack[sp++] = P[s];
    }
    for (int j = n_int - 1; j >= 0; --j) {  // children before parents
        const uint32_t s = order[j], p = P[s], id = sid[s];
        const uint32_t a = sid[p], b = sid[s ^ p];
        t.kl[id - N] = a;
        t.kr[id - N] = b;
        t.parent[a] = id;
        t.parent[b] = id;
        t.box[id] = U[s];
        t.cost[id] = Cs[s];
        t.nl[id] = t.nl[a] + t.nl[b];
        t.height[id] = 1 + std::max(t.height[a], t.height[b]);
    }
}

void opt_process(OptTree& t, uint32_t R, bool treelets) {
    const uint32_t N = t.N, a = t.kl[R - N], b = t.kr[R - N];
    t.box[R] = merge(t.box[a], t.box[b]);
    t.nl[R] = t.nl[a] + t.nl[b];
    t.height[R] = 1 + std::max(t.height[a], t.height[b]);
    t.cost[R] = kOptCi * surface_area(t.box[R]) + (t.cost[a] + t.cost[b]);
    if (treelets && t.nl[R] >= 7) opt_treelet(t, R);
}

}  // namespace

extern "C" {

// nodes_in: a DFS node array (crt_bvh_node, 2N-1); nodes_out receives the
// restructured tree in the same layout.  Returns the root's height.
uint32_t oracle_optimize(const crt_bvh_node* nodes_in, uint32_t n_nodes, uint32_t passes, crt_bvh_node* nodes_out) {
    if (n_nodes == 0) return 0;
    const uint32_t N = (n_nodes + 1) / 2;
    if (N == 1) {
        nodes_out[0] = nodes_in[0];
        return 0;
    }
    OptTree t;
    t.N = N;
    t.box.resize(2 * N - 1);
    t.tri.resize(N);
    t.cost.assign(2 * N - 1, 0.f);
    t.nl.assign(2 * N - 1, 0);
    t.height.assign(2 * N - 1, 0);
    t.parent.assign(2 * N - 1, 0xFFFFFFFFu);
    t.kl.resize(N - 1);
    t.kr.resize(N - 1);
    std::vector<uint32_t> id_of(n_nodes);
    uint32_t n_leaf = 0, n_int = 0;
    for (uint32_t d = 0; d < n_nodes; ++d) {
        const crt_bvh_node& nd = nodes_in[d];
        const bool leaf = nd.left == 0 && nd.right == 0;
        id_of[d] = leaf ? n_leaf++ : N + n_int++;
        const uint32_t id = id_of[d];
        t.box[id] = Box{{nd.mn[0], nd.mn[1], nd.mn[2]}, {nd.mx[0], nd.mx[1], nd.mx[2]}};
        if (leaf) {
            t.tri[id] = nd.tri;
            t.cost[id] = surface_area(t.box[id]);
            t.nl[id] = 1;
        }
    }
    for (uint32_t d = 0; d < n_nodes; ++d) {
        const crt_bvh_node& nd = nodes_in[d];
        if (nd.left == 0 && nd.right == 0) continue;
        const uint32_t id = id_of[d];
        t.kl[id - N] = id_of[nd.left];
        t.kr[id - N] = id_of[nd.right];
        t.parent[id_of[nd.left]] = id;
        t.parent[id_of[nd.right]] = id;
    }
    for (uint32_t pass = 0; pass <= passes; ++pass) {
        const bool treelets = pass < passes;  // a last pass without treelets only sets heights
        if (!treelets && passes > 0) break;
        // post-order, iterative: (node, children pushed)
        std::vector<std::pair<uint32_t, bool>> st;
        st.emplace_back(N, false);
        while (!st.empty()) {
            auto [X, expanded] = st.back();
            st.pop_back();
            if (X < N) continue;
            if (expanded) {
                opt_process(t, X, treelets);
                continue;
            }
            st.emplace_back(X, true);
            st.emplace_back(t.kr[X - N], false);
            st.emplace_back(t.kl[X - N], false);
        }
    }
    // DFS pre-order layout, left first
    uint32_t pos = 0;
    std::vector<std::pair<uint32_t, uint32_t>> st;  // (id, position)
    st.emplace_back(N, pos++);
    while (!st.empty()) {
        const auto [X, p] = st.back();
        st.pop_back();
        crt_bvh_node& o = nodes_out[p];
        std::memset(&o, 0, sizeof(o));
        o.mn[0] = t.box[X].mn.x; o.mn[1] = t.box[X].mn.y; o.mn[2] = t.box[X].mn.z;
        o.mx[0] = t.box[X].mx.x; o.mx[1] = t.box[X].mx.y; o.mx[2] = t.box[X].mx.z;
        if (X < N) {
            o.tri = t.tri[X];
            continue;
        }
        const uint32_t a = t.kl[X - N], b = t.kr[X - N];
        o.left = p + 1;
        o.right = p + 2 * t.nl[a];
        st.emplace_back(b, o.right);
        st.emplace_back(a, o.left);
    }
    return t.height[N];
}

}  // extern "C"
