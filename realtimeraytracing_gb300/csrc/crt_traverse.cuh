// BVH2 traversal of libcrt: one ray's closest or any hit, shared by the
// trace kernels (crt_trace.cu) and the one-launch frame kernels (crt_frame.cu).
//
// Reference: srcCommon/shaders/raytracer.glsl — getRay :92-100,
// rayTriangleIntersection :102-147, intersectBVH :182-221,
// getClosestHitBVH :246-295.  Compiled with -fmad=false: every float
// operation rounds once, in the shader's order, as in the CPU oracle.
//
// Traversal (one thread per ray, stack in local memory) over the 64-byte
// binary nodes the layout pass writes (both child boxes + references), or
// with CRT_TRACE_WIDE over 128-byte 4-wide nodes or with CRT_TRACE_COMPRESSED
// over 64-byte compressed 4-wide nodes (half the fetches, more work per
// fetch — slower on GB300 today, kept for comparison):
//   * children are box-tested at their parent, leaves tested at once, the
//     nearer internal child entered without a stack round trip;
//   * a subtree is skipped when its entry distance exceeds the best hit by
//     more than a slack of |t| * 2^-14 + abs_eps (abs_eps = 2^-20 of the scene
//     extent), so no triangle that can tie or beat the best is lost;
//   * CRT_TRI_REFERENCE tests each leaf box with the shader's own slab test
//     (which is monotone: a leaf box passes only if every ancestor box
//     passes) and the triangle with the shader's predicate, so the tested set
//     is the shader's; equal t keeps the leaf the shader visits first — the
//     one with the higher DFS position, since the shader pops right children
//     first;
//   * CRT_TRI_WATERTIGHT grows every box by abs_eps and uses the watertight
//     predicate (Woop, Benthin, Wald, JCGT 2013); equal t keeps the lower
//     triangle index.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {

__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

struct HitRes { bool did; float t, u, v; };

// raytracer.glsl:102-147; the GLSL struct order _P0,_P2,_P1 makes the
// shader's p1 the C++ P2 and its p2 the C++ P1.
__device__ __forceinline__ HitRes tri_reference(float3 o, float3 d, float tmin, float tmax, float3 P0, float3 P1, float3 P2) {
    HitRes h{false, 0.f, 0.f, 0.f};
    const float3 p0 = P0, p1 = P2, p2 = P1;
    const float3 e0 = sub3(p1, p0);
    const float3 e1 = sub3(p2, p0);
    const float3 c = cross3(e1, e0);
    const float inv = 1.0f / sqrtf(dot3(c, c));
    const float3 nrm = make_float3(c.x * inv, c.y * inv, c.z * inv);
    const float3 q = cross3(d, e1);
    const float a = dot3(e0, q);
    if (dot3(nrm, d) >= 0.f || fabsf(a) < 1e-4f) return h;
    const float3 s = make_float3((o.x - p0.x) / a, (o.y - p0.y) / a, (o.z - p0.z) / a);
    const float3 r = cross3(s, e0);
    const float u = dot3(s, q);
    const float v = dot3(r, d);
    const float w = 1.0f - u - v;
    if (u < 0.f || v < 0.f || w < 0.f) return h;
    const float t = dot3(e1, r);
    if (t < tmin || t > tmax) return h;
    h.did = true; h.t = t; h.u = u; h.v = v;
    return h;
}

struct WRay { int kx, ky, kz; float Sx, Sy, Sz; };

__device__ __forceinline__ float comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ WRay wt_setup(float3 d) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (comp(d, kz) < 0.f) { const int t = kx; kx = ky; ky = t; }
    WRay w;
    w.kx = kx; w.ky = ky; w.kz = kz;
    w.Sx = comp(d, kx) / comp(d, kz);
    w.Sy = comp(d, ky) / comp(d, kz);
    w.Sz = 1.0f / comp(d, kz);
    return w;
}

__device__ __forceinline__ HitRes tri_watertight(float3 o, float tmin, float tmax, const WRay& w, float3 a3, float3 b3, float3 c3) {
    HitRes h{false, 0.f, 0.f, 0.f};
    const float3 A = sub3(a3, o), B = sub3(b3, o), C = sub3(c3, o);
    const float Akz = comp(A, w.kz), Bkz = comp(B, w.kz), Ckz = comp(C, w.kz);
    const float Ax = comp(A, w.kx) - w.Sx * Akz;
    const float Ay = comp(A, w.ky) - w.Sy * Akz;
    const float Bx = comp(B, w.kx) - w.Sx * Bkz;
    const float By = comp(B, w.ky) - w.Sy * Bkz;
    const float Cx = comp(C, w.kx) - w.Sx * Ckz;
    const float Cy = comp(C, w.ky) - w.Sy * Ckz;
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
    const float Az = w.Sz * Akz, Bz = w.Sz * Bkz, Cz = w.Sz * Ckz;
    const float T = U * Az + V * Bz + W * Cz;
    const float t = T / det;
    if (!(t >= tmin) || !(t <= tmax)) return h;
    h.did = true; h.t = t; h.u = V / det; h.v = W / det;
    return h;
}

struct RayCtx {
    float3 o, d, inv;
    float3 oi;    // o * inv, rounded: slab distances as one fma per plane (watertight walks)
    bool exact;   // some 1/d component is not finite or zero: use the shader's min/max
};

// Slab test.  exact: raytracer.glsl:182-221 with GLSL min/max and early
// exits.  Otherwise fminf/fmaxf, which decide identically when every 1/d is
// finite and nonzero (no NaN can arise; a zero's sign changes no comparison).
// GROW widens the box by grow on every side (watertight mode); the binary
// traversal nodes of watertight traces already hold grown boxes.
template <bool GROW>
__device__ __forceinline__ bool slab(const RayCtx& r, float4 mn, float4 mx, float grow, float& t_enter) {
    const float mnx = GROW ? mn.x - grow : mn.x, mny = GROW ? mn.y - grow : mn.y, mnz = GROW ? mn.z - grow : mn.z;
    const float mxx = GROW ? mx.x + grow : mx.x, mxy = GROW ? mx.y + grow : mx.y, mxz = GROW ? mx.z + grow : mx.z;
    const float tx1 = (mnx - r.o.x) * r.inv.x, tx2 = (mxx - r.o.x) * r.inv.x;
    const float ty1 = (mny - r.o.y) * r.inv.y, ty2 = (mxy - r.o.y) * r.inv.y;
    const float tz1 = (mnz - r.o.z) * r.inv.z, tz2 = (mxz - r.o.z) * r.inv.z;
    if (!r.exact) {
        const float t0 = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fminf(tz1, tz2));
        const float t1 = fminf(fminf(fmaxf(tx1, tx2), fmaxf(ty1, ty2)), fmaxf(tz1, tz2));
        t_enter = t0;
        return t1 >= 0.f && t0 <= t1;
    }
    float tMin = min_std(tx1, tx2), tMax = max_std(tx1, tx2);
    t_enter = tMin;
    if (tMax < 0.f || tMin > tMax) return false;
    tMin = max_std(tMin, min_std(ty1, ty2));
    tMax = min_std(tMax, max_std(ty1, ty2));
    t_enter = tMin;
    if (tMax < 0.f || tMin > tMax) return false;
    tMin = max_std(tMin, min_std(tz1, tz2));
    tMax = min_std(tMax, max_std(tz1, tz2));
    t_enter = tMin;
    return tMax >= 0.f && tMin <= tMax;
}

// Watertight walks over the pre-grown traversal boxes: t = plane * (1/d) - o * (1/d) as one
// fused multiply-add per plane.  Its error, like the shader form's, is a few ulps of the
// plane's distance from the origin, which stays below the abs_eps the boxes are grown by
// (2^-20 of the scene's largest coordinate or extent) for origins within 8 times that range,
// so no box that the ray crosses is missed.  Rays with an infinite or zero 1/d take the
// shader's form.
__device__ __forceinline__ bool slab_wt(const RayCtx& r, float4 mn, float4 mx, float& t_enter) {
    if (r.exact) return slab<false>(r, mn, mx, 0.f, t_enter);
    const float tx1 = __fmaf_rn(mn.x, r.inv.x, -r.oi.x), tx2 = __fmaf_rn(mx.x, r.inv.x, -r.oi.x);
    const float ty1 = __fmaf_rn(mn.y, r.inv.y, -r.oi.y), ty2 = __fmaf_rn(mx.y, r.inv.y, -r.oi.y);
    const float tz1 = __fmaf_rn(mn.z, r.inv.z, -r.oi.z), tz2 = __fmaf_rn(mx.z, r.inv.z, -r.oi.z);
    const float t0 = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fminf(tz1, tz2));
    const float t1 = fminf(fminf(fmaxf(tx1, tx2), fmaxf(ty1, ty2)), fmaxf(tz1, tz2));
    t_enter = t0;
    return t1 >= 0.f && t0 <= t1;
}

__device__ __forceinline__ float prune_bound(float t, float abs_eps) {
    return t + (fabsf(t) * 6.103515625e-05f + abs_eps);  // 2^-14 relative
}

// Rays of an image (p.tile_width != 0): each warp takes an 8x4 pixel tile
// instead of a 32-pixel row strip, so its rays stay closer together.
__device__ __forceinline__ uint32_t ray_of_thread(uint32_t t, uint32_t width) {
    if (width == 0) return t;
    const uint32_t tile = t >> 5, lane = t & 31u, tiles_x = width >> 3;
    const uint32_t ty = tile / tiles_x, tx = tile - ty * tiles_x;
    return ((ty << 2) + (lane >> 3)) * width + (tx << 3) + (lane & 7u);
}

// Closest hit (or any hit) of the ray r0 = (o, tmin), r1 = (d, tmax) as a
// crt_hit; i is the ray's index (its predicted treelet with SEED).
// WALK: 0 = binary traversal nodes, 1 = 4-wide nodes, 2 = compressed 4-wide nodes.
template <bool ANY, bool WT, int STACK, bool SEED, int WALK>
__device__ __forceinline__ uint4 trace_one(const TraceParams& p, const uint32_t i, const float4 r0, const float4 r1) {
    RayCtx r;
    r.o = make_float3(r0.x, r0.y, r0.z);
    r.d = make_float3(r1.x, r1.y, r1.z);
    const float tmin = r0.w, tmax = r1.w;
    uint4 out = make_uint4(CRT_MISS, 0u, 0u, 0u);
    if (!(tmin <= tmax) || p.n_nodes == 0) return out;
    r.inv = make_float3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
    r.oi = make_float3(r.o.x * r.inv.x, r.o.y * r.inv.y, r.o.z * r.inv.z);
    r.exact = !(isfinite(r.inv.x) && isfinite(r.inv.y) && isfinite(r.inv.z) && r.inv.x != 0.f && r.inv.y != 0.f &&
                r.inv.z != 0.f);
    WRay w{};
    if (WT) w = wt_setup(r.d);
    const float grow = WT ? p.abs_eps : 0.f;
    const uint32_t n_leaves = (p.n_nodes + 1) / 2;

    bool have = false;
    float bt = tmax, bu = 0.f, bv = 0.f;
    float bound = prune_bound(bt, p.abs_eps);  // subtrees entered beyond this cannot hold the closest hit
    uint32_t bkey = 0xFFFFFFFFu, btri = CRT_MISS;
    uint32_t fetched = 0, tested = 0;
    bool overflow = false, corrupt = false;

    // Leaf L (sorted position = left-to-right order): equal t keeps the leaf
    // the shader visits first, the rightmost, so its key is ~L; watertight
    // ties keep the lower triangle id.
    auto test_leaf = [&](uint32_t L) {
        if (L >= n_leaves) { corrupt = true; return; }
        ++tested;
        const float4* t = p.xtri + 3 * static_cast<size_t>(L);
        const float4 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2);
        const float3 A = make_float3(a.x, a.y, a.z), B = make_float3(b.x, b.y, b.z), C = make_float3(c.x, c.y, c.z);
        const HitRes h = WT ? tri_watertight(r.o, tmin, tmax, w, A, B, C) : tri_reference(r.o, r.d, tmin, tmax, A, B, C);
        if (!h.did) return;
        const uint32_t tri = __float_as_uint(a.w);
        const uint32_t key = WT ? tri : ~L;
        if (!have || h.t < bt || (h.t == bt && key < bkey)) {
            have = true; bt = h.t; bu = h.u; bv = h.v; bkey = key; btri = tri;
            bound = prune_bound(bt, p.abs_eps);
        }
    };

    uint2 st[STACK];  // (node, entry distance) per entry: one 8-byte local store / load
    // Depth-first walk below internal node `cur` (children box-tested at
    // their parent, leaves tested at once, nearer child entered directly).
    // `skip` names a subtree already searched exactly (the seeded treelet).
    auto walk = [&](uint32_t cur, uint32_t skip) {
        int sp = 0;
        while (cur != 0xFFFFFFFFu) {
            if (cur >= n_leaves - 1) { corrupt = true; break; }
            ++fetched;
            const float4* nd = p.wide + 4 * static_cast<size_t>(cur);
            const float4 w0 = __ldg(nd), w1 = __ldg(nd + 1), w2 = __ldg(nd + 2), w3 = __ldg(nd + 3);
            const uint32_t ref0 = __float_as_uint(w0.w), ref1 = __float_as_uint(w1.w);
            float t0, t1;
            bool h0, h1;
            if (WT) {
                h0 = ref0 != skip && slab_wt(r, w0, w1, t0);
                h1 = ref1 != skip && slab_wt(r, w2, w3, t1);
            } else {
                h0 = ref0 != skip && slab<false>(r, w0, w1, 0.f, t0);
                h1 = ref1 != skip && slab<false>(r, w2, w3, 0.f, t1);
            }
            const float bnd = bound;
            h0 = h0 && t0 <= bnd;
            h1 = h1 && t1 <= bnd;
            if (h0 && (ref0 & kLeafRef)) { test_leaf(ref0 & ~kLeafRef); h0 = false; }
            if (h1 && (ref1 & kLeafRef)) { test_leaf(ref1 & ~kLeafRef); h1 = false; }
            if (ANY && have) break;
            if (h0 || h1) {
                const float bnd2 = bound;
                h0 = h0 && t0 <= bnd2;
                h1 = h1 && t1 <= bnd2;
            }
            if (h0 && h1) {
                // closest hit: nearer child first; any hit: farther child first (an
                // occluder of a ray leaving a surface is rarely next to its origin)
                const bool near1 = ANY ? !(t1 < t0) : (t1 < t0);
                if (sp < STACK) {
                    st[sp] = make_uint2(near1 ? ref0 : ref1, __float_as_uint(near1 ? t0 : t1));
                    ++sp;
                } else {
                    overflow = true;
                }
                cur = near1 ? ref1 : ref0;
                continue;
            }
            if (h0) { cur = ref0; continue; }
            if (h1) { cur = ref1; continue; }
            cur = 0xFFFFFFFFu;
            const float bnd3 = bound;
            while (sp > 0) {
                --sp;
                const uint2 e = st[sp];
                if (__uint_as_float(e.y) <= bnd3) { cur = e.x; break; }
            }
        }
    };
    // A leaf reached through a compressed node, whose box there only
    // encloses the exact one: with the shader's predicate the leaf's exact box
    // (from its triangle) must pass the shader's slab test first, so that the
    // tested triangles are the shader's.
    auto test_leaf_exact = [&](uint32_t L) {
        if (L >= n_leaves) { corrupt = true; return; }
        const float4* t = p.xtri + 3 * static_cast<size_t>(L);
        const float4 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2);
        const float4 mn = make_float4(min_std(a.x, min_std(b.x, c.x)), min_std(a.y, min_std(b.y, c.y)),
                                      min_std(a.z, min_std(b.z, c.z)), 0.f);
        const float4 mx = make_float4(max_std(a.x, max_std(b.x, c.x)), max_std(a.y, max_std(b.y, c.y)),
                                      max_std(a.z, max_std(b.z, c.z)), 0.f);
        float te;
        if (!slab<false>(r, mn, mx, 0.f, te) || te > bound) return;
        test_leaf(L);
    };
    // Same walk over the 4-wide nodes: up to four children tested per fetch,
    // leaves tested at once, internal hits ordered by entry distance with a
    // 4-input sorting network; the nearest is entered, the rest pushed.
    // Compressed nodes (WALK 2, 64 bytes) hold each child box as 8-bit
    // offsets from the node's origin in steps of a power of two per axis,
    // rounded outward, decoded as origin + q * step (both exact but the add).
    auto walk4 = [&](uint32_t cur) {
        int sp = 0;
        while (cur != 0xFFFFFFFFu) {
            if (cur >= n_leaves - 1) { corrupt = true; break; }
            ++fetched;
            float nx[4], ny[4], nz[4], xx[4], xy[4], xz[4];
            uint32_t rf[4];
            if (WALK == 2) {
                const uint4* nd = p.cwide + 4 * static_cast<size_t>(cur);
                const uint4 h = __ldg(nd), q0 = __ldg(nd + 1), q1 = __ldg(nd + 2), qr = __ldg(nd + 3);
                const float ox = __uint_as_float(h.x), oy = __uint_as_float(h.y), oz = __uint_as_float(h.z);
                // step 2^e per axis, e biased by 127 in the low three bytes of h.w
                const float sx = __uint_as_float((h.w & 0xFFu) << 23), sy = __uint_as_float(((h.w >> 8) & 0xFFu) << 23);
                const float sz = __uint_as_float(((h.w >> 16) & 0xFFu) << 23);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int sh = 8 * c;
                    nx[c] = ox + static_cast<float>((q0.x >> sh) & 0xFFu) * sx;
                    ny[c] = oy + static_cast<float>((q0.y >> sh) & 0xFFu) * sy;
                    nz[c] = oz + static_cast<float>((q0.z >> sh) & 0xFFu) * sz;
                    xx[c] = ox + static_cast<float>((q0.w >> sh) & 0xFFu) * sx;
                    xy[c] = oy + static_cast<float>((q1.x >> sh) & 0xFFu) * sy;
                    xz[c] = oz + static_cast<float>((q1.y >> sh) & 0xFFu) * sz;
                }
                rf[0] = qr.x; rf[1] = qr.y; rf[2] = qr.z; rf[3] = qr.w;
            } else {
                const float4* nd = p.wide4 + 8 * static_cast<size_t>(cur);
                const float4 qnx = __ldg(nd), qny = __ldg(nd + 1), qnz = __ldg(nd + 2);
                const float4 qxx = __ldg(nd + 3), qxy = __ldg(nd + 4), qxz = __ldg(nd + 5);
                const uint4 qr = __ldg(reinterpret_cast<const uint4*>(nd + 6));
                nx[0] = qnx.x; nx[1] = qnx.y; nx[2] = qnx.z; nx[3] = qnx.w;
                ny[0] = qny.x; ny[1] = qny.y; ny[2] = qny.z; ny[3] = qny.w;
                nz[0] = qnz.x; nz[1] = qnz.y; nz[2] = qnz.z; nz[3] = qnz.w;
                xx[0] = qxx.x; xx[1] = qxx.y; xx[2] = qxx.z; xx[3] = qxx.w;
                xy[0] = qxy.x; xy[1] = qxy.y; xy[2] = qxy.z; xy[3] = qxy.w;
                xz[0] = qxz.x; xz[1] = qxz.y; xz[2] = qxz.z; xz[3] = qxz.w;
                rf[0] = qr.x; rf[1] = qr.y; rf[2] = qr.z; rf[3] = qr.w;
            }
            const float kInf = __int_as_float(0x7F800000);
            float ht[4];
            uint32_t hr[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                ht[c] = kInf;
                hr[c] = 0xFFFFFFFFu;
                if (rf[c] == kNoChild) continue;
                float te;
                if (!slab<WT>(r, make_float4(nx[c], ny[c], nz[c], 0.f), make_float4(xx[c], xy[c], xz[c], 0.f), grow, te))
                    continue;
                if (te > bound) continue;
                if (rf[c] & kLeafRef) {
                    if (WALK == 2 && !WT) test_leaf_exact(rf[c] & ~kLeafRef);
                    else test_leaf(rf[c] & ~kLeafRef);
                } else {
                    ht[c] = te;
                    hr[c] = rf[c];
                }
            }
            if (ANY && have) break;
            const float bnd = bound;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (ht[c] > bnd) { ht[c] = kInf; hr[c] = 0xFFFFFFFFu; }
            // sorting network, ascending entry distance (misses sort last)
#define CRT_CSWAP(a, b)                                                           \
    if (ht[b] < ht[a]) {                                                          \
        const float tt = ht[a]; ht[a] = ht[b]; ht[b] = tt;                        \
        const uint32_t rr = hr[a]; hr[a] = hr[b]; hr[b] = rr;                     \
    }
            CRT_CSWAP(0, 1) CRT_CSWAP(2, 3) CRT_CSWAP(0, 2) CRT_CSWAP(1, 3) CRT_CSWAP(1, 2)
#undef CRT_CSWAP
#pragma unroll
            for (int c = 3; c >= 1; --c) {
                if (hr[c] == 0xFFFFFFFFu) continue;
                if (sp < STACK) {
                    st[sp] = make_uint2(hr[c], __float_as_uint(ht[c]));
                    ++sp;
                } else {
                    overflow = true;
                }
            }
            cur = hr[0];
            if (cur != 0xFFFFFFFFu) continue;
            const float bnd3 = bound;
            while (sp > 0) {
                --sp;
                const uint2 e = st[sp];
                if (__uint_as_float(e.y) <= bnd3) { cur = e.x; break; }
            }
        }
    };
    // Enter a subtree whose box (mn, mx) and reference are known.
    auto enter = [&](float4 mn, float4 mx, uint32_t ref, uint32_t skip) {
        float te;
        if (ref == skip || !slab<WT>(r, mn, mx, grow, te) || te > bound) return;
        if (ref & kLeafRef) test_leaf(ref & ~kLeafRef);
        else if (WALK != 0) walk4(ref);   // the root has depth 0, so it is a 4-wide node
        else walk(ref, skip);
    };
    constexpr uint32_t kNoSkip = 0xFFFFFFFFu;  // never a reference: leaf indices stay below 2^30
    uint32_t skip = kNoSkip;

    if (SEED) {
        // Learned seeding: the predicted treelet first (an exact search of
        // that subtree), so t_max starts at a real hit distance; the full
        // walk below then finds the same closest hit with less work.
        const uint32_t k = p.pred_class[i];
        // The full walk then leaves that treelet out: its closest hit is
        // already known exactly.
        if (k < __ldg(p.n_treelets)) {
            const Treelet* T = p.treelets + k;
            const float4 a = __ldg(reinterpret_cast<const float4*>(T)), b = __ldg(reinterpret_cast<const float4*>(T) + 1);
            enter(a, b, __float_as_uint(a.w), kNoSkip);
            skip = __float_as_uint(a.w);
        }
    }
    if (!(ANY && have)) {
        const float4* n4 = reinterpret_cast<const float4*>(p.nodes);
        const uint4 lr = __ldg(reinterpret_cast<const uint4*>(n4 + 2));
        enter(__ldg(n4), __ldg(n4 + 1), (lr.y == 0u && lr.z == 0u) ? kLeafRef : 0u, skip);
    }
    if (have) out = make_uint4(btri, __float_as_uint(bt), __float_as_uint(bu), __float_as_uint(bv));
    if (corrupt) raise_corrupt(p.err, 5, i, 0u);
    else if (overflow) raise_error(p.err, kDevStackOverflow);
    if (p.stats) {
        atomicAdd(p.stats + 0, static_cast<unsigned long long>(fetched));
        atomicAdd(p.stats + 1, static_cast<unsigned long long>(tested));
    }
    return out;
}

// Ray i of p.rays into p.hits[i].
template <bool ANY, bool WT, int STACK, bool SEED, int WALK>
__device__ __forceinline__ void trace_ray(const TraceParams& p, const uint32_t i) {
    const float4 r0 = __ldg(reinterpret_cast<const float4*>(p.rays + i));
    const float4 r1 = __ldg(reinterpret_cast<const float4*>(p.rays + i) + 1);
    reinterpret_cast<uint4*>(p.hits)[i] = trace_one<ANY, WT, STACK, SEED, WALK>(p, i, r0, r1);
}

// getRay (raytracer.glsl:92-100): pos = texel / size, direction =
// normalize(InvView * vec4((pos - 0.5, 1) * (W, H, near), 1) - eye).
__device__ __forceinline__ void camera_ray(const crt_camera* __restrict__ cam, uint32_t x, uint32_t y, uint32_t width,
                                           uint32_t height, float4& r0, float4& r1) {
    const float* m = cam->inv_view;
    const float px = static_cast<float>(x) / static_cast<float>(width);
    const float py = static_cast<float>(y) / static_cast<float>(height);
    const float4 pv = make_float4((px - 0.5f) * cam->plane_width, (py - 0.5f) * cam->plane_height, 1.0f * cam->plane_near, 1.0f);
    const float4 pw = mat_vec(m, pv);
    const float dx = pw.x - cam->eye[0], dy = pw.y - cam->eye[1], dz = pw.z - cam->eye[2], dw = pw.w - cam->eye[3];
    const float inv = 1.0f / sqrtf(((dx * dx + dy * dy) + dz * dz) + dw * dw);
    r0 = make_float4(cam->eye[0], cam->eye[1], cam->eye[2], 0.f);
    r1 = make_float4(dx * inv, dy * inv, dz * inv, __int_as_float(0x7F800000));
}

// Shadow ray of a primary hit toward the point light l: from the hit point
// (o + t d), unit direction, tmin 1e-4, tmax the distance to the light; a
// miss gives an empty ray (tmin 1 > tmax 0).
__device__ __forceinline__ void shadow_ray(float4 r0, float4 r1, uint4 h, float lx, float ly, float lz, float4& s0,
                                           float4& s1) {
    if (h.x == CRT_MISS) {
        s0 = make_float4(0.f, 0.f, 0.f, 1.f);
        s1 = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float t = __uint_as_float(h.y);
    const float px = r0.x + t * r1.x, py = r0.y + t * r1.y, pz = r0.z + t * r1.z;
    const float dx = lx - px, dy = ly - py, dz = lz - pz;
    const float len = sqrtf((dx * dx + dy * dy) + dz * dz);
    const float inv = 1.0f / len;
    s0 = make_float4(px, py, pz, 1e-4f);
    s1 = make_float4(dx * inv, dy * inv, dz * inv, len);
}

}  // namespace crt
