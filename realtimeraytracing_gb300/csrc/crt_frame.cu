// One-launch frames and the shading pass of libcrt: camera ray, closest hit
// and, per option, the shadow ray's any hit and the shaded texel of every
// pixel.  Compiled with -fmad=false: every float operation rounds once, in
// the shader's order, as in the CPU oracle.
//
// Shading restates srcCommon/shaders/raytracer.glsl:
//   getColor                        :159-179
//   intersectBVH with border test   :182-236
//   bvhColor of getClosestHitBVH    :246-277 (the depth-uDepthDisplayBVH box)
//   main's initial value, imageStore :299-331
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"
#include "crt_traverse.cuh"

namespace crt {

// ------------------------------------------------------------- shading
// intersectBVH (raytracer.glsl:182-236): 0 = miss, 1 = hit, 2 = hit whose
// entry point lies within `line` of a face of the box on at least two axes
// (near a box edge).  GLSL min/max, its early exits and its entry point
// o + d * tMin, each operation rounded once.
__device__ __forceinline__ uint32_t display_slab(float3 o, float3 d, float4 mn, float4 mx, float line) {
    const float ix = 1.0f / d.x;
    const float tx1 = (mn.x - o.x) * ix, tx2 = (mx.x - o.x) * ix;
    float tMin = min_std(tx1, tx2), tMax = max_std(tx1, tx2);
    if (tMax < 0.f || tMin > tMax) return 0u;
    const float iy = 1.0f / d.y;
    const float ty1 = (mn.y - o.y) * iy, ty2 = (mx.y - o.y) * iy;
    tMin = max_std(tMin, min_std(ty1, ty2));
    tMax = min_std(tMax, max_std(ty1, ty2));
    if (tMax < 0.f || tMin > tMax) return 0u;
    const float iz = 1.0f / d.z;
    const float tz1 = (mn.z - o.z) * iz, tz2 = (mx.z - o.z) * iz;
    tMin = max_std(tMin, min_std(tz1, tz2));
    tMax = min_std(tMax, max_std(tz1, tz2));
    if (!(tMax >= 0.f && tMin <= tMax)) return 0u;
    const float ex = o.x + d.x * tMin, ey = o.y + d.y * tMin, ez = o.z + d.z * tMin;
    const bool cx = fabsf(ex - mn.x) < line || fabsf(ex - mx.x) < line;
    const bool cy = fabsf(ey - mn.y) < line || fabsf(ey - mx.y) < line;
    const bool cz = fabsf(ez - mn.z) < line || fabsf(ez - mx.z) < line;
    return ((cx && cy) || (cx && cz) || (cy && cz)) ? 2u : 1u;
}

// bvhColor.  The shader's walk pops right children first, enters every box
// the ray intersects and overwrites bvhColor at each intersected node of
// depth D, so the last such node decides.  A left-child-first walk meets the
// nodes of one depth in exactly the reverse order, so that node is the FIRST
// intersected depth-D node of a left-first walk that descends only through
// intersected boxes: this walk stops there and never goes below depth D.
// Returns display_slab's value for that node, 0 when there is none.
__device__ __noinline__ uint32_t bvh_display(const TraceParams& p, uint32_t depth_d, float3 o, float3 d) {
    const float line = 0.05f / (static_cast<float>(depth_d) + 1.f);  // BVH_LINE_WIDTH / (uDepthDisplayBVH + 1)
    uint32_t st_node[kShadeMaxDepth];
    uint32_t st_depth[kShadeMaxDepth];
    int sp = 0;
    uint32_t cur = 0, depth = 0;
    // each node is met at most once, so a walk longer than the tree is a bad tree
    for (uint32_t guard = 0; guard < p.n_nodes; ++guard) {
        if (cur >= p.n_nodes) { raise_corrupt(p.err, 10, cur, p.n_nodes); return 0u; }
        const float4* nd = reinterpret_cast<const float4*>(p.nodes + cur);
        const float4 mn = __ldg(nd), mx = __ldg(nd + 1);
        const uint4 k = __ldg(reinterpret_cast<const uint4*>(nd + 2));  // tri, left, right, pad
        const uint32_t hit = display_slab(o, d, mn, mx, line);
        if (hit != 0u) {
            if (depth == depth_d) return hit;
            if (k.y != 0u || k.z != 0u) {  // internal (isLeafBVH: left == right == 0)
                // pending right siblings have strictly increasing depths < D
                if (sp >= static_cast<int>(kShadeMaxDepth)) { raise_corrupt(p.err, 10, cur, depth); return 0u; }
                st_node[sp] = k.z;
                st_depth[sp] = depth + 1;
                ++sp;
                cur = k.y;
                ++depth;
                continue;
            }
        }
        if (sp == 0) return 0u;
        --sp;
        cur = st_node[sp];
        depth = st_depth[sp];
    }
    if (p.n_nodes != 0) raise_corrupt(p.err, 10, cur, p.n_nodes);
    return 0u;
}

// getColor + main's initial value for hit h of the ray (r0.xyz, r1.xyz).
__device__ __forceinline__ float4 shade_texel(const TraceParams& p, const ShadeParams& sp, uint4 h, float4 r0,
                                              float4 r1) {
    float4 c = make_float4(0.f, 0.f, 0.f, 1.f);
    if (sp.flags & CRT_SHADE_BVH) {
        const uint32_t b = bvh_display(p, sp.bvh_depth, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z));
        c = b == 2u ? make_float4(0.7f, 0.f, 0.7f, 0.1f)      // BVH_AABB_LINE_COLOR
            : b == 1u ? make_float4(0.5f, 0.f, 0.5f, 0.1f)    // BVH_AABB_COLOR
                      : make_float4(0.f, 0.f, 0.f, 0.f);      // bvhColor's initial value
    }
    if (h.x == CRT_MISS) return c;
    if (h.x >= sp.n_tris) { raise_corrupt(p.err, 11, h.x, sp.n_tris); return c; }
    const uint32_t L = __ldg(sp.inv_perm + h.x);
    if (L >= sp.n_tris) { raise_corrupt(p.err, 11, h.x, L); return c; }
    const uint32_t model = __float_as_uint(__ldg(p.xtri + 3 * static_cast<size_t>(L) + 1).w);
    const uint32_t mat = model < sp.n_models ? __ldg(sp.models + 17 * model + 16) : 0u;
    const float4 m = mat < sp.n_materials ? __ldg(sp.materials + mat) : make_float4(0.f, 0.f, 0.f, 0.f);
    c = make_float4(c.x + m.x, c.y + m.y, c.z + m.z, c.w + m.w);
    if (sp.flags & CRT_SHADE_WIREFRAME) {
        const float u = __uint_as_float(h.z), v = __uint_as_float(h.w);
        const float w = 1.0f - u - v;  // _Coords.z as rayTriangleIntersection forms it
        if (u < 0.02f || v < 0.02f || w < 0.02f) c = make_float4(0.f, 0.f, 0.f, 1.f);  // WIREFRAME_LINE_WIDTH
    }
    return c;
}

__global__ void __launch_bounds__(256) shade_kernel(TraceParams p, ShadeParams sp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n_rays) return;
    const uint4 h = __ldg(reinterpret_cast<const uint4*>(p.hits) + i);
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
    if (sp.flags & CRT_SHADE_BVH) {
        r0 = __ldg(reinterpret_cast<const float4*>(p.rays + i));
        r1 = __ldg(reinterpret_cast<const float4*>(p.rays + i) + 1);
    }
    sp.image[i] = shade_texel(p, sp, h, r0, r1);
}

void launch_shade(const TraceParams& p, const ShadeParams& sp, cudaStream_t s) {
    if (p.n_rays == 0) return;
    shade_kernel<<<(p.n_rays + 255) / 256, 256, 0, s>>>(p, sp);
}

// ------------------------------------------------------------- frames
// One frame in one launch (crt_trace_frame, crt_render_frame): thread t
// takes pixel ray_of_thread(t) of the image rows [y0, y0 + rows), generates
// its camera ray, traces it to the closest hit and, with a light, traces
// that hit's shadow ray to any hit at once, while the nodes around the hit
// are still cached; with SHADE it also writes the pixel's texel.  The rays,
// hits and texels are the ones the separate raygen, trace, shadow-ray and
// shade calls produce.
template <bool WT, int STACK, int BLOCK, bool SHADE>
__global__ void __launch_bounds__(BLOCK) frame_kernel(TraceParams p, const crt_camera* __restrict__ cam, uint32_t width,
                                                      uint32_t height, uint32_t y0, uint32_t rows, int shadows,
                                                      float lx, float ly, float lz, crt_hit* __restrict__ hits_shadow,
                                                      ShadeParams sp) {
    const uint32_t t_id = blockIdx.x * BLOCK + threadIdx.x;
    if (t_id >= width * rows) return;
    const uint32_t i = y0 * width + ray_of_thread(t_id, p.tile_width);
    const uint32_t y = i / width, x = i - y * width;
    float4 r0, r1;
    camera_ray(cam, x, y, width, height, r0, r1);
    const uint4 h = trace_one<false, WT, STACK, false, 0>(p, i, r0, r1);
    if (!SHADE || p.hits) reinterpret_cast<uint4*>(p.hits)[i] = h;
    if (SHADE) sp.image[i] = shade_texel(p, sp, h, r0, r1);
    if (!shadows) return;
    uint4 hs = make_uint4(CRT_MISS, 0u, 0u, 0u);
    if (h.x != CRT_MISS) {
        float4 s0, s1;
        shadow_ray(r0, r1, h, lx, ly, lz, s0, s1);
        hs = trace_one<true, WT, STACK, false, 0>(p, i, s0, s1);
    }
    reinterpret_cast<uint4*>(hits_shadow)[i] = hs;
}

template <bool WT, int BLOCK, bool SHADE>
static void launch_frame_s(const TraceParams& p, const crt_camera* cam, uint32_t width, uint32_t height, uint32_t y0,
                           uint32_t rows, const float* light, crt_hit* hits_shadow, bool deep, const ShadeParams& sp,
                           cudaStream_t s) {
    const uint32_t grid = (width * rows + BLOCK - 1) / BLOCK;
    if (grid == 0) return;
    const int sh = light != nullptr;
    const float lx = sh ? light[0] : 0.f, ly = sh ? light[1] : 0.f, lz = sh ? light[2] : 0.f;
    if (deep)
        frame_kernel<WT, 1024, BLOCK, SHADE>
            <<<grid, BLOCK, 0, s>>>(p, cam, width, height, y0, rows, sh, lx, ly, lz, hits_shadow, sp);
    else
        frame_kernel<WT, 64, BLOCK, SHADE>
            <<<grid, BLOCK, 0, s>>>(p, cam, width, height, y0, rows, sh, lx, ly, lz, hits_shadow, sp);
}

template <bool WT, int BLOCK>
static void launch_frame_b(const TraceParams& p, const crt_camera* cam, uint32_t width, uint32_t height, uint32_t y0,
                           uint32_t rows, const float* light, crt_hit* hits_shadow, bool deep, const ShadeParams* shade,
                           cudaStream_t s) {
    if (shade) launch_frame_s<WT, BLOCK, true>(p, cam, width, height, y0, rows, light, hits_shadow, deep, *shade, s);
    else launch_frame_s<WT, BLOCK, false>(p, cam, width, height, y0, rows, light, hits_shadow, deep, ShadeParams{}, s);
}

void launch_frame(const TraceParams& p, const crt_camera* cam, uint32_t width, uint32_t height, uint32_t y0,
                  uint32_t rows, const float* light, crt_hit* hits_shadow, uint32_t flags, int block,
                  const ShadeParams* shade, cudaStream_t s) {
    const bool wt = flags & CRT_TRI_WATERTIGHT;
    const bool deep = (flags >> 16) != 0;
    if (wt) {
        if (block == 256) launch_frame_b<true, 256>(p, cam, width, height, y0, rows, light, hits_shadow, deep, shade, s);
        else if (block == 64) launch_frame_b<true, 64>(p, cam, width, height, y0, rows, light, hits_shadow, deep, shade, s);
        else launch_frame_b<true, 128>(p, cam, width, height, y0, rows, light, hits_shadow, deep, shade, s);
    } else {
        if (block == 256) launch_frame_b<false, 256>(p, cam, width, height, y0, rows, light, hits_shadow, deep, shade, s);
        else if (block == 64) launch_frame_b<false, 64>(p, cam, width, height, y0, rows, light, hits_shadow, deep, shade, s);
        else launch_frame_b<false, 128>(p, cam, width, height, y0, rows, light, hits_shadow, deep, shade, s);
    }
}

}  // namespace crt
