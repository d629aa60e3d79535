// Trace kernels of libcrt: rays from memory to hits (crt_trace, batched
// scenes), ray ordering for CRT_TRACE_SORT_RAYS, ray generation and shadow
// rays.  The traversal itself is in crt_traverse.cuh.  Compiled with
// -fmad=false: every float operation rounds once, in the shader's order.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"
#include "crt_traverse.cuh"

namespace crt {

template <bool ANY, bool WT, int STACK, bool SEED, int WALK, int BLOCK>
__global__ void __launch_bounds__(BLOCK) trace_kernel(TraceParams p) {
    const uint32_t t_id = blockIdx.x * BLOCK + threadIdx.x;
    if (t_id >= p.n_rays) return;
    const uint32_t i = p.order ? __ldg(p.order + t_id) : ray_of_thread(t_id, p.tile_width);
    if (i >= p.n_rays) { raise_corrupt(p.err, 7, t_id, i); return; }
    trace_ray<ANY, WT, STACK, SEED, WALK>(p, i);
}

// ------------------------------------------------ persistent ray pool
// Closest-hit traversal of many incoherent rays.  One ray per lane, walked
// exactly as trace_one's binary walk (children box-tested at their parent,
// leaves tested at once, nearer child entered, pruning by the best hit's
// bound), but the warps are persistent: after every BURST node visits the
// lanes whose ray has finished take the next rays from a global counter (one
// atomic per warp), so a warp no longer runs as long as its slowest ray
// while most of its lanes idle.  Rays are taken in caller order, or in
// p.order.  The hits are those of trace_kernel: a ray's closest hit (and its
// tie rule) does not depend on the order its nodes are visited in.
// The scene a lane's ray is walked in: traversal nodes, leaf triangles, the
// watertight slack and the leaf count (one scene, or the ray's scene of a batch).
struct PoolScene {
    const crt_bvh_node* nodes;
    const float4* wide;
    const float4* xtri;
    float abs_eps;
    uint32_t n_leaves;
};

template <bool WT, int STACK>
struct PoolRay {
    RayCtx r;
    WRay w;
    float tmin, tmax, bt, bu, bv, bound;
    uint32_t bkey, btri, cur;
    int sp;
    bool have;
    // one postponed leaf (kNoLeaf: none) and the entry distance of its box
    uint32_t pend;
    float pend_t;
    static constexpr uint32_t kNoLeaf = 0xFFFFFFFFu;

    __device__ __forceinline__ void test_leaf(const PoolScene& sc, uint32_t L, uint32_t& tested, bool& corrupt) {
        if (L >= sc.n_leaves) { corrupt = true; return; }
        ++tested;
        const float4* t = sc.xtri + 3 * static_cast<size_t>(L);
        const float4 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2);
        const float3 A = make_float3(a.x, a.y, a.z), B = make_float3(b.x, b.y, b.z), C = make_float3(c.x, c.y, c.z);
        const HitRes h = WT ? tri_watertight(r.o, tmin, tmax, w, A, B, C) : tri_reference(r.o, r.d, tmin, tmax, A, B, C);
        if (!h.did) return;
        const uint32_t tri = __float_as_uint(a.w);
        const uint32_t key = WT ? tri : ~L;
        if (!have || h.t < bt || (h.t == bt && key < bkey)) {
            have = true; bt = h.t; bu = h.u; bv = h.v; bkey = key; btri = tri;
            bound = prune_bound(bt, sc.abs_eps);
        }
    }

    // Sets up ray (r0, r1) and enters the root; false when the ray is already finished.
    __device__ __forceinline__ bool start(const PoolScene& sc, float4 r0, float4 r1, uint32_t& tested, bool& corrupt) {
        r.o = make_float3(r0.x, r0.y, r0.z);
        r.d = make_float3(r1.x, r1.y, r1.z);
        tmin = r0.w;
        tmax = r1.w;
        have = false;
        bt = tmax; bu = 0.f; bv = 0.f;
        bkey = 0xFFFFFFFFu; btri = CRT_MISS;
        sp = 0;
        cur = 0xFFFFFFFFu;
        pend = kNoLeaf;
        if (!(tmin <= tmax) || sc.n_leaves == 0) return false;
        r.inv = make_float3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
        r.oi = make_float3(r.o.x * r.inv.x, r.o.y * r.inv.y, r.o.z * r.inv.z);
        r.exact = !(isfinite(r.inv.x) && isfinite(r.inv.y) && isfinite(r.inv.z) && r.inv.x != 0.f && r.inv.y != 0.f &&
                    r.inv.z != 0.f);
        if (WT) w = wt_setup(r.d);
        bound = prune_bound(bt, sc.abs_eps);
        const float4* n4 = reinterpret_cast<const float4*>(sc.nodes);
        const uint4 lr = __ldg(reinterpret_cast<const uint4*>(n4 + 2));
        float te;
        if (!slab<WT>(r, __ldg(n4), __ldg(n4 + 1), WT ? sc.abs_eps : 0.f, te) || te > bound) return false;
        if (lr.y == 0u && lr.z == 0u) {  // a one-leaf tree
            test_leaf(sc, 0u, tested, corrupt);
            return false;
        }
        cur = 0u;
        return true;
    }

    // A hit leaf child: parked in the free slot (PEND), else tested now.
    template <bool PEND>
    __device__ __forceinline__ void leaf(const PoolScene& sc, uint32_t L, float t, uint32_t& tested, bool& corrupt) {
        if (PEND && pend == kNoLeaf) { pend = L; pend_t = t; return; }
        test_leaf(sc, L, tested, corrupt);
    }

    // Tests the parked leaf unless the best hit found since prunes it (the
    // same entry-distance rule a leaf tested at its parent gets).
    __device__ __forceinline__ void flush(const PoolScene& sc, uint32_t& tested, bool& corrupt) {
        if (pend == kNoLeaf) return;
        if (pend_t <= bound) test_leaf(sc, pend, tested, corrupt);
        pend = kNoLeaf;
    }

    // One node visit; false when the walk has finished.  PEND: hit leaf
    // children are parked (one slot) instead of tested at once, so that the
    // warp can test many lanes' leaves together (flush); a ray's closest hit
    // does not depend on when its leaves are tested, and pruning by a bound
    // that is not yet tightened only visits more nodes.
    template <bool PEND>
    __device__ __forceinline__ bool step(const PoolScene& sc, uint2* st, uint32_t& fetched, uint32_t& tested,
                                         bool& corrupt, bool& overflow) {
        if (cur >= sc.n_leaves - 1) { corrupt = true; return false; }
        ++fetched;
        const float4* nd = sc.wide + 4 * static_cast<size_t>(cur);
        const float4 w0 = __ldg(nd), w1 = __ldg(nd + 1), w2 = __ldg(nd + 2), w3 = __ldg(nd + 3);
        const uint32_t ref0 = __float_as_uint(w0.w), ref1 = __float_as_uint(w1.w);
        float t0, t1;
        bool h0, h1;
        if (WT) {
            h0 = slab_wt(r, w0, w1, t0);
            h1 = slab_wt(r, w2, w3, t1);
        } else {
            h0 = slab<false>(r, w0, w1, 0.f, t0);
            h1 = slab<false>(r, w2, w3, 0.f, t1);
        }
        const float bnd = bound;
        h0 = h0 && t0 <= bnd;
        h1 = h1 && t1 <= bnd;
        if (h0 && (ref0 & kLeafRef)) { leaf<PEND>(sc, ref0 & ~kLeafRef, t0, tested, corrupt); h0 = false; }
        if (h1 && (ref1 & kLeafRef)) { leaf<PEND>(sc, ref1 & ~kLeafRef, t1, tested, corrupt); h1 = false; }
        if (h0 || h1) {
            const float bnd2 = bound;
            h0 = h0 && t0 <= bnd2;
            h1 = h1 && t1 <= bnd2;
        }
        if (h0 && h1) {
            const bool near1 = t1 < t0;
            if (sp < STACK) {  // (node, entry distance) as one 8-byte entry
                st[sp] = make_uint2(near1 ? ref0 : ref1, __float_as_uint(near1 ? t0 : t1));
                ++sp;
            } else {
                overflow = true;
            }
            cur = near1 ? ref1 : ref0;
            return true;
        }
        if (h0) { cur = ref0; return true; }
        if (h1) { cur = ref1; return true; }
        const float bnd3 = bound;
        while (sp > 0) {
            --sp;
            const uint2 e = st[sp];
            if (__uint_as_float(e.y) <= bnd3) { cur = e.x; return true; }
        }
        return false;
    }

    __device__ __forceinline__ uint4 hit() const {
        return have ? make_uint4(btri, __float_as_uint(bt), __float_as_uint(bu), __float_as_uint(bv))
                    : make_uint4(CRT_MISS, 0u, 0u, 0u);
    }
};

// CHUNK: the warp takes rays from the counter 32 at a time and hands them to
// its idle lanes as they free up, so that a warp's lanes hold neighbouring
// rays of the (possibly coherence-sorted) order; otherwise it takes exactly
// as many as it has idle lanes.
//
// BATCH: many scenes in one launch (crt_batch_trace): a lane that takes ray i
// finds i's scene by binary search over the scenes' ray offsets and walks
// that scene's tree; p.nodes / p.wide / p.xtri are the batch's arrays.
//
// PEND: leaf tests are postponed (PoolRay::step<true>) and run for the whole
// warp at once when at least FLUSH lanes hold a parked leaf, or when a lane
// whose walk has ended still holds one (it must be tested before the hit is
// written).
template <bool WT, int STACK, int BLOCK, int BURST, bool CHUNK, bool BATCH, bool PEND, int FLUSH>
__global__ void __launch_bounds__(BLOCK) trace_pool_kernel(TraceParams p, uint32_t* __restrict__ next_ray,
                                                           const BatchScene* __restrict__ scenes, uint32_t n_scenes) {
    constexpr uint32_t kIdle = 0xFFFFFFFFu, kDone = 0xFFFFFFFEu;
    __shared__ uint32_t s_ray_off[BATCH ? kMaxBatchScenes + 1 : 1];
    if (BATCH) {
        for (uint32_t k = threadIdx.x; k <= n_scenes; k += BLOCK)
            s_ray_off[k] = k < n_scenes ? scenes[k].ray_off : scenes[n_scenes - 1].ray_off + scenes[n_scenes - 1].n_rays;
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u, lt_mask = (1u << lane) - 1u;
    PoolScene sc{p.nodes, p.wide, p.xtri, p.abs_eps, (p.n_nodes + 1) / 2};
    PoolRay<WT, STACK> ray;
    uint2 st[STACK];
    uint32_t i = kIdle, fetched = 0, tested = 0;
    uint32_t chunk_next = 0, chunk_end = 0;  // CHUNK: the warp's rays not yet handed out (warp-uniform)
    bool corrupt = false, overflow = false;
    while (true) {
        const bool idle = (i == kIdle);
        const uint32_t need = __ballot_sync(0xFFFFFFFFu, idle);
        if (need) {
            uint32_t base = 0;
            uint32_t take = static_cast<uint32_t>(__popc(need));
            if (CHUNK) {
                if (chunk_next == chunk_end) {
                    uint32_t b = 0;
                    if (lane == 0) b = atomicAdd(next_ray, 32u);
                    chunk_next = __shfl_sync(0xFFFFFFFFu, b, 0);
                    chunk_end = chunk_next + 32u;
                }
                base = chunk_next;
                take = min(take, chunk_end - chunk_next);
                chunk_next += take;
            } else {
                const int leader = __ffs(need) - 1;
                if (lane == static_cast<uint32_t>(leader)) base = atomicAdd(next_ray, take);
                base = __shfl_sync(0xFFFFFFFFu, base, leader);
            }
            const uint32_t rank = static_cast<uint32_t>(__popc(need & lt_mask));
            if (idle && rank < take) {
                const uint32_t k = base + rank;
                if (k >= p.n_rays) {
                    i = kDone;
                } else {
                    i = p.order ? __ldg(p.order + k) : k;
                    if (i >= p.n_rays) {
                        raise_corrupt(p.err, 7, k, i);
                        i = kDone;
                    } else {
                        if (BATCH) {
                            uint32_t lo = 0, hi = n_scenes - 1;
                            while (lo < hi) {
                                const uint32_t mid = (lo + hi + 1) >> 1;
                                if (s_ray_off[mid] <= i) lo = mid; else hi = mid - 1;
                            }
                            const BatchScene bs = scenes[lo];
                            sc.nodes = p.nodes + bs.node_off;
                            sc.wide = p.wide + 4 * static_cast<size_t>(bs.wide_off);
                            sc.xtri = p.xtri + 3 * static_cast<size_t>(bs.tri_off);
                            sc.abs_eps = bs.abs_eps;
                            sc.n_leaves = bs.n_tris;
                        }
                        const float4 r0 = __ldg(reinterpret_cast<const float4*>(p.rays + i));
                        const float4 r1 = __ldg(reinterpret_cast<const float4*>(p.rays + i) + 1);
                        if (!ray.start(sc, r0, r1, tested, corrupt)) {
                            reinterpret_cast<uint4*>(p.hits)[i] = ray.hit();
                            i = kIdle;
                        }
                    }
                }
            }
        }
        if (__all_sync(0xFFFFFFFFu, i == kDone)) break;
        if (PEND) {
            bool walking = i < kDone;
#pragma unroll 1
            for (int s = 0; s < BURST; ++s) {
                if (walking) walking = ray.template step<true>(sc, st, fetched, tested, corrupt, overflow);
                const bool parked = i < kDone && ray.pend != PoolRay<WT, STACK>::kNoLeaf;
                const uint32_t pm = __ballot_sync(0xFFFFFFFFu, parked);
                if (__popc(pm) >= FLUSH || __any_sync(0xFFFFFFFFu, parked && !walking)) {
                    if (parked) ray.flush(sc, tested, corrupt);
                }
                if (!__any_sync(0xFFFFFFFFu, walking)) break;
            }
            if (i < kDone && !walking) {
                reinterpret_cast<uint4*>(p.hits)[i] = ray.hit();
                i = kIdle;
            }
        } else if (i < kDone) {
            bool walking = true;
#pragma unroll 1
            for (int s = 0; s < BURST && walking; ++s)
                walking = ray.template step<false>(sc, st, fetched, tested, corrupt, overflow);
            if (!walking) {
                reinterpret_cast<uint4*>(p.hits)[i] = ray.hit();
                i = kIdle;
            }
        }
    }
    if (corrupt) raise_corrupt(p.err, 5, blockIdx.x, threadIdx.x);
    else if (overflow) raise_error(p.err, kDevStackOverflow);
    if (p.stats) {
        atomicAdd(p.stats + 0, static_cast<unsigned long long>(fetched));
        atomicAdd(p.stats + 1, static_cast<unsigned long long>(tested));
    }
}

// Many scenes in one launch: ray i belongs to the scene whose ray range holds
// it and is traced against that scene's BVH (same walk as above).
// SEED: learned seeding in a batch; base.pred_class holds every ray's class,
// base.treelets / base.n_treelets every scene's cut (scene k's at 128 k / k).
template <bool ANY, bool WT, int STACK, bool SEED, int BLOCK>
__global__ void __launch_bounds__(BLOCK) trace_batch_kernel(TraceParams base, const BatchScene* __restrict__ scenes,
                                                            uint32_t n_scenes, uint32_t n_rays_total) {
    __shared__ uint32_t s_ray_off[kMaxBatchScenes + 1];
    for (uint32_t k = threadIdx.x; k <= n_scenes; k += BLOCK) s_ray_off[k] = scenes[k < n_scenes ? k : n_scenes - 1].ray_off +
                                                                            (k < n_scenes ? 0u : scenes[n_scenes - 1].n_rays);
    __syncthreads();
    const uint32_t t = blockIdx.x * BLOCK + threadIdx.x;
    if (t >= n_rays_total) return;
    const uint32_t i = base.order ? __ldg(base.order + t) : t;
    if (i >= n_rays_total) { raise_corrupt(base.err, 7, t, i); return; }
    uint32_t lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (s_ray_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const BatchScene sc = scenes[lo];
    TraceParams p = base;
    p.nodes = base.nodes + sc.node_off;
    p.wide = base.wide + 4 * static_cast<size_t>(sc.wide_off);
    p.xtri = base.xtri + 3 * static_cast<size_t>(sc.tri_off);
    p.n_nodes = 2 * sc.n_tris - 1;
    p.abs_eps = sc.abs_eps;
    if (SEED) {
        p.treelets = base.treelets + 128 * static_cast<size_t>(lo);
        p.n_treelets = base.n_treelets + lo;
    }
    trace_ray<ANY, WT, STACK, SEED, 0>(p, i);
}

// ------------------------------------------------------ ray ordering
// CRT_TRACE_SORT_RAYS: rays are traced in the order of a 24-bit coherence
// key — Morton code of the cell, on a 32^3 grid of the scene box, where the
// ray enters the box (its origin if it starts inside; 15 bits), then an
// octahedral direction bin (32 x 16, 9 bits) — so warps hold rays that
// reach the scene close together and point the same way.  In a batch
// the scene index (8 bits) goes on top, which keeps every ray inside its
// scene's range.  A stable LSD radix sort (the build's digit pass) makes the
// order; every ray still gets its own hit.
__device__ __forceinline__ uint32_t spread5_bits(uint32_t v) {
    v &= 31u;
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6) | ((v & 16u) << 8);
}

__device__ __forceinline__ uint32_t coherence_key(float4 r0, float4 r1, float4 mn, float4 mx) {
    // entry distance into the box (a key only: any rounding is harmless)
    const float ix = 1.f / r1.x, iy = 1.f / r1.y, iz = 1.f / r1.z;
    const float tx1 = (mn.x - r0.x) * ix, tx2 = (mx.x - r0.x) * ix;
    const float ty1 = (mn.y - r0.y) * iy, ty2 = (mx.y - r0.y) * iy;
    const float tz1 = (mn.z - r0.z) * iz, tz2 = (mx.z - r0.z) * iz;
    float te = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fminf(tz1, tz2));
    if (!(te > 0.f) || !isfinite(te)) te = 0.f;
    const float ex = r0.x + te * r1.x, ey = r0.y + te * r1.y, ez = r0.z + te * r1.z;
    const float sx = 32.f / fmaxf(mx.x - mn.x, 1e-20f), sy = 32.f / fmaxf(mx.y - mn.y, 1e-20f);
    const float sz = 32.f / fmaxf(mx.z - mn.z, 1e-20f);
    const int cx = min(max(static_cast<int>(floorf((ex - mn.x) * sx)), 0), 31);
    const int cy = min(max(static_cast<int>(floorf((ey - mn.y) * sy)), 0), 31);
    const int cz = min(max(static_cast<int>(floorf((ez - mn.z) * sz)), 0), 31);
    const uint32_t m = (spread5_bits(cx) << 2) | (spread5_bits(cy) << 1) | spread5_bits(cz);
    const float a = fabsf(r1.x) + fabsf(r1.y) + fabsf(r1.z);
    float px = a > 0.f ? r1.x / a : 0.f, py = a > 0.f ? r1.y / a : 0.f;
    if (r1.z < 0.f) {
        const float qx = (1.f - fabsf(py)) * (px >= 0.f ? 1.f : -1.f);
        const float qy = (1.f - fabsf(px)) * (py >= 0.f ? 1.f : -1.f);
        px = qx;
        py = qy;
    }
    const int bu = min(max(static_cast<int>((px + 1.f) * 16.f), 0), 31);
    const int bv = min(max(static_cast<int>((py + 1.f) * 8.f), 0), 15);
    return (m << 9) | (static_cast<uint32_t>(bu) << 4) | static_cast<uint32_t>(bv);
}

// Keys of all rays and the histograms of their PASSES 8-bit digits; with
// scenes, ray i belongs to the scene whose ray range holds it and is keyed
// on that scene's root box.
template <int PASSES>
__global__ void __launch_bounds__(256) ray_key_kernel(const crt_ray* __restrict__ rays, uint32_t n,
                                                      const crt_bvh_node* __restrict__ nodes,
                                                      const BatchScene* __restrict__ scenes, uint32_t n_scenes,
                                                      uint32_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[PASSES * 256];
    __shared__ uint32_t s_ray_off[kMaxBatchScenes + 1];
    for (int k = threadIdx.x; k < PASSES * 256; k += blockDim.x) h[k] = 0u;
    if (scenes)
        for (uint32_t k = threadIdx.x; k <= n_scenes; k += blockDim.x)
            s_ray_off[k] = k < n_scenes ? scenes[k].ray_off : scenes[n_scenes - 1].ray_off + scenes[n_scenes - 1].n_rays;
    __syncthreads();
    float4 mn = __ldg(reinterpret_cast<const float4*>(nodes)), mx = __ldg(reinterpret_cast<const float4*>(nodes) + 1);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t top = 0;
        if (scenes) {
            uint32_t lo = 0, hi = n_scenes - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (s_ray_off[mid] <= i) lo = mid; else hi = mid - 1;
            }
            const float4* root = reinterpret_cast<const float4*>(nodes + scenes[lo].node_off);
            mn = __ldg(root);
            mx = __ldg(root + 1);
            top = lo << 24;
        }
        const float4 r0 = __ldg(reinterpret_cast<const float4*>(rays + i));
        const float4 r1 = __ldg(reinterpret_cast<const float4*>(rays + i) + 1);
        const uint32_t key = top | coherence_key(r0, r1, mn, mx);
        keys[i] = key;
#pragma unroll
        for (int p = 0; p < PASSES; ++p) atomicAdd(&h[p * 256 + ((key >> (8 * p)) & 255u)], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < PASSES * 256; k += blockDim.x)
        if (h[k]) atomicAdd(&hist[k], h[k]);
}

__global__ void __launch_bounds__(256) raygen_kernel(const crt_camera* __restrict__ cam, uint32_t width, uint32_t height,
                                                     crt_ray* __restrict__ rays) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y;
    if (x >= width) return;
    float4 r0, r1;
    camera_ray(cam, x, y, width, height, r0, r1);
    float4* o = reinterpret_cast<float4*>(rays + static_cast<size_t>(y) * width + x);
    o[0] = r0;
    o[1] = r1;
}


__global__ void __launch_bounds__(256) shadow_kernel(const crt_ray* __restrict__ prim, const crt_hit* __restrict__ hits,
                                                     uint32_t n, float lx, float ly, float lz, crt_ray* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 h = __ldg(reinterpret_cast<const uint4*>(hits) + i);
    const float4 r0 = __ldg(reinterpret_cast<const float4*>(prim + i));
    const float4 r1 = __ldg(reinterpret_cast<const float4*>(prim + i) + 1);
    float4 s0, s1;
    shadow_ray(r0, r1, h, lx, ly, lz, s0, s1);
    float4* o = reinterpret_cast<float4*>(out + i);
    o[0] = s0;
    o[1] = s1;
}


template <bool ANY, bool WT, int BLOCK>
static void launch_trace_b(const TraceParams& p, bool deep, bool seed, int walk, cudaStream_t s) {
    const uint32_t grid = (p.n_rays + BLOCK - 1) / BLOCK;
    if (grid == 0) return;
    if (seed) {
        if (deep) trace_kernel<ANY, WT, 1024, true, 0, BLOCK><<<grid, BLOCK, 0, s>>>(p);
        else trace_kernel<ANY, WT, 64, true, 0, BLOCK><<<grid, BLOCK, 0, s>>>(p);
    } else if (walk == 1) {
        if (deep) trace_kernel<ANY, WT, 1024, false, 1, BLOCK><<<grid, BLOCK, 0, s>>>(p);
        else trace_kernel<ANY, WT, 96, false, 1, BLOCK><<<grid, BLOCK, 0, s>>>(p);
    } else if (walk == 2) {
        if (deep) trace_kernel<ANY, WT, 1024, false, 2, BLOCK><<<grid, BLOCK, 0, s>>>(p);
        else trace_kernel<ANY, WT, 96, false, 2, BLOCK><<<grid, BLOCK, 0, s>>>(p);
    } else {
        if (deep) trace_kernel<ANY, WT, 1024, false, 0, BLOCK><<<grid, BLOCK, 0, s>>>(p);
        else trace_kernel<ANY, WT, 64, false, 0, BLOCK><<<grid, BLOCK, 0, s>>>(p);
    }
}

template <bool ANY, bool WT>
static void launch_trace_t(const TraceParams& p, int block, bool deep, bool seed, int walk, cudaStream_t s) {
    if (block == 256) launch_trace_b<ANY, WT, 256>(p, deep, seed, walk, s);
    else if (block == 64) launch_trace_b<ANY, WT, 64>(p, deep, seed, walk, s);
    else launch_trace_b<ANY, WT, 128>(p, deep, seed, walk, s);
}

// Launch shape of the persistent traversal (measured on GB300 over 8M
// incoherent bounce rays: block, node visits between refills, chunked refill,
// postponed leaf tests and the parked lanes that trigger a warp's flush).
#ifndef CRT_POOL_BLOCK
#define CRT_POOL_BLOCK 128
#endif
#ifndef CRT_POOL_BURST
#define CRT_POOL_BURST 16
#endif
#ifndef CRT_POOL_CHUNK
#define CRT_POOL_CHUNK 0
#endif
#ifndef CRT_POOL_PEND
#define CRT_POOL_PEND 1
#endif
#ifndef CRT_POOL_FLUSH
#define CRT_POOL_FLUSH 6
#endif

template <bool WT, int STACK, bool BATCH>
static void launch_pool_s(const TraceParams& p, uint32_t* next_ray, const BatchScene* scenes, uint32_t n_scenes,
                          cudaStream_t s) {
    constexpr int kBlock = CRT_POOL_BLOCK, kBurst = CRT_POOL_BURST, kFlush = CRT_POOL_FLUSH;
    constexpr bool kChunk = CRT_POOL_CHUNK != 0, kPend = CRT_POOL_PEND != 0;
    static int grid = 0;
    if (grid == 0) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_pool_kernel<WT, STACK, kBlock, kBurst, kChunk, BATCH, kPend, kFlush>,
                                                      kBlock, 0);
        grid = kNumSms * (per_sm > 0 ? per_sm : 1);
    }
    cudaMemsetAsync(next_ray, 0, 4, s);
    const uint32_t want = (p.n_rays + kBlock - 1) / kBlock;
    trace_pool_kernel<WT, STACK, kBlock, kBurst, kChunk, BATCH, kPend, kFlush>
        <<<want < static_cast<uint32_t>(grid) ? want : static_cast<uint32_t>(grid), kBlock, 0, s>>>(p, next_ray, scenes,
                                                                                                   n_scenes);
}

void launch_trace_pool(const TraceParams& p, uint32_t flags, uint32_t* next_ray, cudaStream_t s) {
    const bool wt = flags & CRT_TRI_WATERTIGHT;
    const bool deep = (flags >> 16) != 0;
    if (p.n_rays == 0) return;
    if (wt) {
        if (deep) launch_pool_s<true, 1024, false>(p, next_ray, nullptr, 0, s);
        else launch_pool_s<true, 64, false>(p, next_ray, nullptr, 0, s);
    } else {
        if (deep) launch_pool_s<false, 1024, false>(p, next_ray, nullptr, 0, s);
        else launch_pool_s<false, 64, false>(p, next_ray, nullptr, 0, s);
    }
}

void launch_trace_batch_pool(const TraceParams& p, const BatchScene* scenes, uint32_t n_scenes, uint32_t flags,
                             bool deep, uint32_t* next_ray, cudaStream_t s) {
    const bool wt = flags & CRT_TRI_WATERTIGHT;
    if (p.n_rays == 0 || n_scenes == 0) return;
    if (wt) {
        if (deep) launch_pool_s<true, 1024, true>(p, next_ray, scenes, n_scenes, s);
        else launch_pool_s<true, 64, true>(p, next_ray, scenes, n_scenes, s);
    } else {
        if (deep) launch_pool_s<false, 1024, true>(p, next_ray, scenes, n_scenes, s);
        else launch_pool_s<false, 64, true>(p, next_ray, scenes, n_scenes, s);
    }
}

void launch_trace(const TraceParams& p, uint32_t flags, int block, cudaStream_t s) {
    const bool any = flags & CRT_TRACE_ANY, wt = flags & CRT_TRI_WATERTIGHT;
    const bool deep = (flags >> 16) != 0;  // set by the host when the tree may be deeper than the stacks allow
    const bool seed = p.pred_class != nullptr;
    const int walk = ((flags & CRT_TRACE_COMPRESSED) && p.cwide) ? 2 : ((flags & CRT_TRACE_WIDE) && p.wide4) ? 1 : 0;
    if (any && wt) launch_trace_t<true, true>(p, block, deep, seed, walk, s);
    else if (any) launch_trace_t<true, false>(p, block, deep, seed, walk, s);
    else if (wt) launch_trace_t<false, true>(p, block, deep, seed, walk, s);
    else launch_trace_t<false, false>(p, block, deep, seed, walk, s);
}

template <bool ANY, bool WT, int BLOCK>
static void launch_batch_b(const TraceParams& p, const BatchScene* scenes, uint32_t n_scenes, uint32_t n_rays,
                           bool deep, cudaStream_t s) {
    const uint32_t grid = (n_rays + BLOCK - 1) / BLOCK;
    if (grid == 0) return;
    if (p.pred_class) {
        if (deep) trace_batch_kernel<ANY, WT, 1024, true, BLOCK><<<grid, BLOCK, 0, s>>>(p, scenes, n_scenes, n_rays);
        else trace_batch_kernel<ANY, WT, 64, true, BLOCK><<<grid, BLOCK, 0, s>>>(p, scenes, n_scenes, n_rays);
    } else {
        if (deep) trace_batch_kernel<ANY, WT, 1024, false, BLOCK><<<grid, BLOCK, 0, s>>>(p, scenes, n_scenes, n_rays);
        else trace_batch_kernel<ANY, WT, 64, false, BLOCK><<<grid, BLOCK, 0, s>>>(p, scenes, n_scenes, n_rays);
    }
}

template <bool ANY, bool WT>
static void launch_batch_t(const TraceParams& p, const BatchScene* scenes, uint32_t n_scenes, uint32_t n_rays,
                           int block, bool deep, cudaStream_t s) {
    if (block == 512) launch_batch_b<ANY, WT, 512>(p, scenes, n_scenes, n_rays, deep, s);
    else if (block == 256) launch_batch_b<ANY, WT, 256>(p, scenes, n_scenes, n_rays, deep, s);
    else launch_batch_b<ANY, WT, 128>(p, scenes, n_scenes, n_rays, deep, s);
}

void launch_trace_batch(const TraceParams& p, const BatchScene* scenes, uint32_t n_scenes, uint32_t n_rays,
                        uint32_t flags, int block, bool deep, cudaStream_t s) {
    const bool any = flags & CRT_TRACE_ANY, wt = flags & CRT_TRI_WATERTIGHT;
    if (any && wt) launch_batch_t<true, true>(p, scenes, n_scenes, n_rays, block, deep, s);
    else if (any) launch_batch_t<true, false>(p, scenes, n_scenes, n_rays, block, deep, s);
    else if (wt) launch_batch_t<false, true>(p, scenes, n_scenes, n_rays, block, deep, s);
    else launch_batch_t<false, false>(p, scenes, n_scenes, n_rays, block, deep, s);
}

size_t ray_order_scratch_bytes(uint32_t n) {
    const size_t tiles = (n + sort_tile_keys(8) - 1) / sort_tile_keys(8);
    return 4 * (3 * static_cast<size_t>(n) + 4 * 256 + 4 * (tiles * 256 + 1) + 64);
}

void launch_ray_order(const crt_ray* rays, uint32_t n, const crt_bvh_node* nodes, const BatchScene* scenes,
                      uint32_t n_scenes, uint32_t* order, void* scratch, uint32_t* err, uint32_t spin_limit,
                      cudaStream_t s) {
    if (n == 0) return;
    const int passes = scenes ? 4 : 3;
    uint32_t* ka = static_cast<uint32_t*>(scratch);
    uint32_t* kb = ka + n;
    uint32_t* vt = kb + n;
    uint32_t* hist = vt + n;
    uint32_t* lb = hist + 4 * 256;  // per pass: ticket, then the look-back words
    const size_t tiles = (n + sort_tile_keys(8) - 1) / sort_tile_keys(8);
    const size_t lb_words = tiles * 256 + 1;
    cudaMemsetAsync(hist, 0, 4 * (4 * 256 + 4 * lb_words), s);
    const uint32_t grid = std::min<uint32_t>((n + 255) / 256, kNumSms * 8);
    if (scenes) ray_key_kernel<4><<<grid, 256, 0, s>>>(rays, n, nodes, scenes, n_scenes, ka, hist);
    else ray_key_kernel<3><<<grid, 256, 0, s>>>(rays, n, nodes, nullptr, 0, ka, hist);
    // stable 8-bit passes; the values alternate between order and vt so
    // that the last pass writes order
    const uint32_t* kin = ka;
    const uint32_t* vin = nullptr;
    for (int p = 0; p < passes; ++p) {
        uint32_t* kout = (p & 1) ? ka : kb;
        uint32_t* vout = ((passes - 1 - p) & 1) ? vt : order;
        uint32_t* l = lb + p * lb_words;
        launch_onesweep(kin, vin, kout, vout, n, 8 * p, 8, hist + 256 * p, l + 1, l, err, spin_limit, s);
        kin = kout;
        vin = vout;
    }
}

void launch_raygen(const crt_camera* cam_dev, uint32_t width, uint32_t height, crt_ray* rays, cudaStream_t s) {
    dim3 grid((width + 255) / 256, height);
    raygen_kernel<<<grid, 256, 0, s>>>(cam_dev, width, height, rays);
}

void launch_shadow_rays(const crt_ray* prim, const crt_hit* hits, uint32_t n, float lx, float ly, float lz, crt_ray* out,
                        cudaStream_t s) {
    if (n == 0) return;
    shadow_kernel<<<(n + 255) / 256, 256, 0, s>>>(prim, hits, n, lx, ly, lz, out);
}

}  // namespace crt
