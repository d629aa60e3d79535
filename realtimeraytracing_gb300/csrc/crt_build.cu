// BVH build kernels of libcrt: scene box, Morton codes, Onesweep LSD radix
// sort of (code, index), PLOC iterations and the DFS node layout.
//
// Reference: srcCommon/scene/geometry/bvh.cpp (CPU, OpenMP) and the DFS
// flattening in srcOpenGL/scene/scene.cpp:189-208.  Every float result is
// bit-identical to the reference's (this file is compiled with -fmad=false).
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {

// =========================================================== K1: scene box
// getSceneAABB (bvh.cpp:235-251) folds max(cur, max(p0, max(p1, p2))) over
// all n_buffer records in order.  That fold ignores NaN candidates and keeps
// the earliest of equal values, so it equals the leftmost arg-max over
// non-NaN per-triangle values — an associative reduction.  Each candidate is
// keyed (ordered value, index); the winner's exact value (sign of zero
// included) is recomputed from its triangle.

struct TriExtent { float hi[3], lo[3]; };

__device__ __forceinline__ TriExtent tri_extent(const TriRec& t, const float* __restrict__ models) {
    const float* M = models + 16 * (t.model & (kMaxModels - 1));
    const float4 p0 = mat_vec(M, t.p0), p1 = mat_vec(M, t.p1), p2 = mat_vec(M, t.p2);
    TriExtent e;
    e.hi[0] = max_std(p0.x, max_std(p1.x, p2.x));
    e.hi[1] = max_std(p0.y, max_std(p1.y, p2.y));
    e.hi[2] = max_std(p0.z, max_std(p1.z, p2.z));
    e.lo[0] = min_std(p0.x, min_std(p1.x, p2.x));
    e.lo[1] = min_std(p0.y, min_std(p1.y, p2.y));
    e.lo[2] = min_std(p0.z, min_std(p1.z, p2.z));
    return e;
}

__device__ __forceinline__ unsigned long long shfl_xor_u64(unsigned long long v, int m) {
    return __shfl_xor_sync(0xFFFFFFFFu, v, m);
}

__global__ void __launch_bounds__(256) scene_box_kernel(const crt_triangle* __restrict__ tris, uint32_t n_buffer,
                                                        const float* __restrict__ models, SceneState* st,
                                                        uint32_t* err) {
    unsigned long long kmax[3] = {0ull, 0ull, 0ull};
    unsigned long long kmin[3] = {~0ull, ~0ull, ~0ull};
    bool bad = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_buffer; i += gridDim.x * blockDim.x) {
        const TriRec t = load_tri(tris, i);
        bad |= t.model >= kMaxModels;
        const TriExtent e = tri_extent(t, models);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (e.hi[a] == e.hi[a]) {
                const unsigned long long k = (static_cast<unsigned long long>(ordered_key(e.hi[a])) << 32) | (0xFFFFFFFFu - i);
                kmax[a] = k > kmax[a] ? k : kmax[a];
            }
            if (e.lo[a] == e.lo[a]) {
                const unsigned long long k = (static_cast<unsigned long long>(ordered_key(e.lo[a])) << 32) | i;
                kmin[a] = k < kmin[a] ? k : kmin[a];
            }
        }
    }
    if (bad) raise_error(err, kDevBadModel);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        for (int m = 16; m > 0; m >>= 1) {
            const unsigned long long x = shfl_xor_u64(kmax[a], m), y = shfl_xor_u64(kmin[a], m);
            kmax[a] = x > kmax[a] ? x : kmax[a];
            kmin[a] = y < kmin[a] ? y : kmin[a];
        }
    __shared__ unsigned long long s_k[6][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { s_k[a][warp] = kmax[a]; s_k[3 + a][warp] = kmin[a]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int a = threadIdx.x;
        const int nw = blockDim.x >> 5;
        unsigned long long v = s_k[a][0];
        for (int w = 1; w < nw; ++w) v = (a < 3) ? (s_k[a][w] > v ? s_k[a][w] : v) : (s_k[a][w] < v ? s_k[a][w] : v);
        if (a < 3) atomicMax(&st->key_max[a], v); else atomicMin(&st->key_min[a - 3], v);
    }
    // The last block to finish turns the keys into the box and the cube.
    __shared__ bool s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(&st->blocks_done, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!s_last || threadIdx.x != 0) return;
    __threadfence();
    const float kInf = __int_as_float(0x7F800000);
    float smin[3], smax[3];
    for (int a = 0; a < 3; ++a) {
        const unsigned long long kx = atomicAdd(&st->key_max[a], 0ull);
        const unsigned long long kn = atomicAdd(&st->key_min[a], 0ull);
        smax[a] = -kInf;
        smin[a] = kInf;
        if (kx != 0ull) smax[a] = tri_extent(load_tri(tris, 0xFFFFFFFFu - static_cast<uint32_t>(kx)), models).hi[a];
        if (kn != ~0ull) smin[a] = tri_extent(load_tri(tris, static_cast<uint32_t>(kn)), models).lo[a];
        st->key_max[a] = 0ull;
        st->key_min[a] = ~0ull;
    }
    st->blocks_done = 0u;
    // getCircumscribedCube (bvh.cpp:253-303): X is chosen whenever distX > 0.
    float cmn[3] = {smin[0], smin[1], smin[2]}, cmx[3] = {smax[0], smax[1], smax[2]};
    const float dX = smax[0] - smin[0], dY = smax[1] - smin[1], dZ = smax[2] - smin[2];
    float maxDist = 0.f;
    int axis;
    if (dX > maxDist) { maxDist = dX; axis = 0; }
    else if (dY > maxDist) { maxDist = dY; axis = 1; }
    else { maxDist = dZ; axis = 2; }
    const float dist[3] = {dX, dY, dZ};
    for (int a = 0; a < 3; ++a) {
        if (a == axis) continue;
        const float delta = (maxDist - dist[a]) / 2.f;
        cmx[a] += delta;
        cmn[a] -= delta;
    }
    for (int a = 0; a < 3; ++a) {
        st->scene_min[a] = smin[a];
        st->scene_max[a] = smax[a];
        st->cube_min[a] = cmn[a];
        st->cube_len[a] = cmx[a] - cmn[a];  // getNormalizedCentroids (bvh.cpp:319-321)
    }
    st->abs_eps = scene_abs_eps(smin, smax);
}

// ====================================================== K1: Morton codes
__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {  // bvh.cpp:350-356
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ __forceinline__ uint32_t to_u10(float x) {  // bvh.cpp:363-367
    x = min_std(max_std(x * 1024.0f, 0.0f), 1023.0f);
    return __float2uint_rz(x);  // NaN -> 0, as on the reference's hosts
}

// The digit histograms of the radix passes: for each of PASSES digit places
// of BITS bits, one count per digit value, in shared memory (s_hist[p *
// 2^BITS + d]).  The sort's counting step — with 1-bit digits it is the
// reference's per-bit histogram (histogramOfGlobalDigitCounts.glsl:31-59).
template <int BITS, int PASSES>
__device__ __forceinline__ void add_digit_counts(uint32_t key, uint32_t* s_hist) {
    constexpr uint32_t RADIX = 1u << BITS;
#pragma unroll
    for (int p = 0; p < PASSES; ++p) atomicAdd(&s_hist[p * RADIX + ((key >> (p * BITS)) & (RADIX - 1))], 1u);
}

// Block-wide inclusive scan, in thread order, of one 64-bit value per thread
// (the radix passes pack two 32-bit counts into it); s_wsum holds one entry
// per warp.  Every thread of the block must call it.
template <int BLOCK>
__device__ __forceinline__ unsigned long long block_inclusive_scan_u64(unsigned long long v,
                                                                       unsigned long long* s_wsum) {
    constexpr int WARPS = BLOCK / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) s_wsum[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (int w = 0; w < WARPS; ++w) { const unsigned long long t = s_wsum[w]; s_wsum[w] = run; run += t; }
    }
    __syncthreads();
    return v + s_wsum[warp];
}

// Centroid (triangle.cpp:31-33), normalisation (bvh.cpp:314-328) and code
// (bvh.cpp:358-372), plus the digit histograms of all radix passes.
template <int BITS>
__global__ void __launch_bounds__(256) morton_kernel(const crt_triangle* __restrict__ tris, uint32_t n,
                                                     const float* __restrict__ models_third,
                                                     const SceneState* __restrict__ st,
                                                     uint32_t* __restrict__ codes, uint32_t* __restrict__ hist) {
    constexpr int RADIX = 1 << BITS;
    constexpr int PASSES = (30 + BITS - 1) / BITS;
    __shared__ uint32_t s_hist[PASSES * RADIX];
    for (int i = threadIdx.x; i < PASSES * RADIX; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    const float cmx = st->cube_min[0], cmy = st->cube_min[1], cmz = st->cube_min[2];
    const float lx = st->cube_len[0], ly = st->cube_len[1], lz = st->cube_len[2];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const TriRec t = load_tri(tris, i);
        const float* M3 = models_third + 16 * (t.model & (kMaxModels - 1));
        float4 s;
        s.x = t.p0.x + t.p1.x + t.p2.x;
        s.y = t.p0.y + t.p1.y + t.p2.y;
        s.z = t.p0.z + t.p1.z + t.p2.z;
        s.w = t.p0.w + t.p1.w + t.p2.w;
        const float4 c = mat_vec(M3, s);
        const float nx = (c.x - cmx) / lx, ny = (c.y - cmy) / ly, nz = (c.z - cmz) / lz;
        const uint32_t code = (expand_bits(to_u10(nx)) << 2) | (expand_bits(to_u10(ny)) << 1) | expand_bits(to_u10(nz));
        codes[i] = code;
        add_digit_counts<BITS, PASSES>(code, s_hist);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < PASSES * RADIX; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

// ============================================== K2: Onesweep digit binning
// One stable counting pass over digit (key >> shift) & (RADIX-1) of a tile
// of BLOCK*KPT keys (Adinets & Merrill, "Onesweep", 2022):
//  * warp multisplit: each lane ORs its bit into the warp's shared-memory
//    mask of its digit, so the lanes holding the same digit read their group
//    back (fewer instructions than BITS ballots, and than match.any, on this
//    part); every lane reads the warp's count of its digit, then the highest
//    of the group adds the group's size (no branch to a leader, no shuffle);
//  * chained-scan decoupled look-back across tiles for the global digit
//    offsets; each digit's thread reads a window of LB_WIN predecessor tiles
//    per round trip with relaxed loads (flag and count share one word);
//  * a shared-memory staged scatter, first of the digit-carrying array
//    (keys, or values for SEG) then of the other, so that every warp's
//    global stores fall in a few contiguous runs.
// Pass 0 synthesises the values (iota), which makes the result the
// reference's std::sort of (code, index) pairs (bvh.cpp:214-232).
constexpr uint32_t kLbAgg = 1u << 30, kLbPrefix = 2u << 30, kLbMask = (1u << 30) - 1u;
constexpr int kLbWindow = 4;

// SEG: the digit is not taken from the key but is the segment (scene) whose
// range [seg_off[d], seg_off[d+1]) holds the value — one extra stable pass
// that groups concatenated scenes back together after the code passes.
template <int BITS, int BLOCK, int KPT, bool SEG>
__global__ void __launch_bounds__(BLOCK, 3) onesweep_kernel(const uint32_t* __restrict__ keys_in,
                                                            const uint32_t* __restrict__ vals_in,
                                                            uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                            uint32_t n, int shift, const uint32_t* __restrict__ pass_hist,
                                                            uint32_t* lookback, uint32_t* ticket, uint32_t* err,
                                                            uint32_t spin_limit, const uint32_t* __restrict__ seg_off,
                                                            uint32_t n_seg) {
    constexpr int RADIX = 1 << BITS;
    constexpr int WARPS = BLOCK / 32;
    constexpr int TILE = BLOCK * KPT;
    static_assert(BLOCK >= RADIX, "one thread per digit");
    __shared__ uint32_t s_buf[TILE];            // staging for the scatter
    __shared__ uint32_t s_whist[WARPS][RADIX];  // per-warp digit counters, then per-warp offsets
    __shared__ uint32_t s_match[WARPS][RADIX];  // per-warp lane masks of the key being ranked
    __shared__ uint32_t s_start[RADIX];         // block-local exclusive digit start
    __shared__ uint32_t s_adj[RADIX];           // global destination of sorted slot i is s_adj[d] + i
    __shared__ unsigned long long s_wsum[WARPS];
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_seg[SEG ? RADIX + 1 : 1];
    __shared__ uint32_t s_timeout;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        s_tile = atomicAdd(ticket, 1u);
        s_timeout = 0u;
    }
    for (int i = threadIdx.x; i < WARPS * RADIX; i += BLOCK) {
        (&s_whist[0][0])[i] = 0u;
        (&s_match[0][0])[i] = 0u;
    }
    if (SEG)
        for (int i = threadIdx.x; i <= RADIX; i += BLOCK) s_seg[i] = (static_cast<uint32_t>(i) <= n_seg) ? seg_off[i] : 0xFFFFFFFFu;
    __syncthreads();
    auto digit_of = [&](uint32_t key, uint32_t val) -> uint32_t {
        if (!SEG) return (key >> shift) & (RADIX - 1);
        uint32_t lo = 0, hi = n_seg - 1;  // last segment start <= val
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (s_seg[mid] <= val) lo = mid; else hi = mid - 1;
        }
        return lo;
    };
    const uint32_t tile = s_tile;
    const uint64_t tile_base = static_cast<uint64_t>(tile) * TILE;
    if (tile_base >= n) return;
    const uint64_t rem = n - tile_base;
    const uint32_t tile_n = rem < static_cast<uint64_t>(TILE) ? static_cast<uint32_t>(rem) : static_cast<uint32_t>(TILE);
    // Warp w ranks the contiguous keys [w*32*KPT, (w+1)*32*KPT) of the tile, j-major.
    const uint32_t wofs = static_cast<uint32_t>(warp) * 32u * KPT + lane;
    const uint32_t* kin = keys_in + tile_base;
    const uint32_t* vin = vals_in ? vals_in + tile_base : nullptr;
    const uint32_t ibase = static_cast<uint32_t>(tile_base);

    uint32_t key[KPT], val[KPT], pos[KPT];
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const uint32_t lo = wofs + j * 32u;
        key[j] = lo < tile_n ? __ldg(kin + lo) : 0u;
        val[j] = lo < tile_n ? (vin ? __ldg(vin + lo) : ibase + lo) : 0u;
    }
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t* my_hist = &s_whist[warp][0];
    uint32_t* my_match = &s_match[warp][0];
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const bool ok = wofs + j * 32u < tile_n;
        const uint32_t d = ok ? digit_of(key[j], val[j]) : 0u;
        // the lanes holding digit d: each sets its bit in the warp's mask of d
        if (ok) atomicOr(my_match + d, 1u << lane);
        __syncwarp();
        const uint32_t peers = ok ? my_match[d] : 0u;
        // every lane reads its digit's running count (the lanes of one digit
        // read one word: a broadcast); after the warp has read, the group's
        // highest lane alone adds the group's size and clears the mask
        const uint32_t base = my_hist[d];
        __syncwarp();
        if (ok && (peers >> lane) == 1u) {
            my_hist[d] = base + static_cast<uint32_t>(__popc(peers));
            my_match[d] = 0u;
        }
        pos[j] = base + __popc(peers & lt_mask);
        __syncwarp();
    }
    __syncthreads();

    // Per digit: exclusive over warps, tile total, publication.
    const int d = threadIdx.x;
    uint32_t total = 0, excl = 0;
    if (d < RADIX) {
        for (int w = 0; w < WARPS; ++w) {
            const uint32_t c = s_whist[w][d];
            s_whist[w][d] = total;
            total += c;
        }
        st_relaxed_u32(lookback + static_cast<size_t>(tile) * RADIX + d, (tile == 0 ? kLbPrefix : kLbAgg) | total);
    }
    // Block-wide exclusive scans over digits of (tile totals) and (global
    // histogram), packed as two 32-bit halves of one 64-bit scan.
    const uint32_t gh = (d < RADIX) ? pass_hist[d] : 0u;
    const uint32_t a = (d < RADIX) ? total : 0u;
    const unsigned long long packed =
        block_inclusive_scan_u64<BLOCK>((static_cast<unsigned long long>(gh) << 32) | a, s_wsum);
    if (d < RADIX) {
        if (tile > 0) {
            // Look-back: sum the predecessors' counts of digit d down to the
            // nearest inclusive prefix; tile 0 always publishes one.
            int64_t k = static_cast<int64_t>(tile) - 1;
            SpinBound spin(spin_limit);
            while (true) {
                uint32_t v[kLbWindow];
#pragma unroll
                for (int q = 0; q < kLbWindow; ++q)
                    v[q] = (k - q >= 0) ? ld_relaxed_u32(lookback + static_cast<size_t>(k - q) * RADIX + d) : kLbPrefix;
                int q = 0;
                bool done = false;
#pragma unroll
                for (; q < kLbWindow; ++q) {
                    const uint32_t f = v[q] & ~kLbMask;
                    if (f == 0u) break;
                    excl += v[q] & kLbMask;
                    if (f == kLbPrefix) { done = true; break; }
                }
                if (done) break;
                k -= q;
                if (q < kLbWindow && !spin.step()) {
                    raise_error(err, kDevTimeout);
                    s_timeout = 1u;
                    break;
                }
            }
            st_relaxed_u32(lookback + static_cast<size_t>(tile) * RADIX + d, kLbPrefix | (excl + total));
        }
        const uint32_t incl_a = static_cast<uint32_t>(packed & 0xFFFFFFFFull);
        const uint32_t incl_g = static_cast<uint32_t>(packed >> 32);
        s_start[d] = incl_a - a;
        s_adj[d] = (incl_g - gh) + excl - (incl_a - a);
    }
    __syncthreads();
    if (s_timeout) return;  // the prefix is incomplete: write nothing
    // Tile-local sorted slot of each element.
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const bool ok = wofs + j * 32u < tile_n;
        const uint32_t dd = ok ? digit_of(key[j], val[j]) : 0u;
        pos[j] += s_start[dd] + my_hist[dd];
        if (ok) s_buf[pos[j]] = SEG ? val[j] : key[j];
    }
    __syncthreads();
    uint32_t dst[KPT];
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        const uint32_t i = k * BLOCK + threadIdx.x;
        if (i < tile_n) {
            const uint32_t x = s_buf[i];
            dst[k] = s_adj[SEG ? digit_of(0u, x) : digit_of(x, 0u)] + i;
            if (dst[k] >= n) {  // only a corrupt histogram gets here
                raise_corrupt(err, 17, tile, dst[k]);
                dst[k] = 0xFFFFFFFFu;
                continue;
            }
            if (SEG) vals_out[dst[k]] = x;
            else keys_out[dst[k]] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < KPT; ++j)
        if (wofs + j * 32u < tile_n) s_buf[pos[j]] = SEG ? key[j] : val[j];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        const uint32_t i = k * BLOCK + threadIdx.x;
        if (i < tile_n && dst[k] != 0xFFFFFFFFu) {
            if (SEG) keys_out[dst[k]] = s_buf[i];
            else vals_out[dst[k]] = s_buf[i];
        }
    }
}

// ==================================================== leaf clusters
// plocPreprocessing (bvh.cpp:26-46): sorted position i holds the leaf of
// triangle perm[i] with AABB::buildFromTriangle's box (bvh.cpp:383-399).
// Also stores the model-transformed vertices the traversal tests against,
// in sorted order (the layout moves them into tree order).
__global__ void __launch_bounds__(256) leaf_init_kernel(const crt_triangle* __restrict__ tris, uint32_t n,
                                                        const float* __restrict__ models,
                                                        const uint32_t* __restrict__ perm,
                                                        float4* __restrict__ node_box, float4* __restrict__ clusters,
                                                        float4* __restrict__ xtri, uint2* it, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) it[0] = make_uint2(n, n);
    if (i >= n) return;
    const uint32_t ti = perm[i];
    if (ti >= n) { raise_corrupt(err, 1, i, ti); return; }
    const TriRec t = load_tri(tris, ti);
    const float* M = models + 16 * (t.model & (kMaxModels - 1));
    const float4 p0 = mat_vec(M, t.p0), p1 = mat_vec(M, t.p1), p2 = mat_vec(M, t.p2);
    float4 mn, mx;
    mn.x = min_std(p0.x, min_std(p1.x, p2.x));
    mn.y = min_std(p0.y, min_std(p1.y, p2.y));
    mn.z = min_std(p0.z, min_std(p1.z, p2.z));
    mx.x = max_std(p0.x, max_std(p1.x, p2.x));
    mx.y = max_std(p0.y, max_std(p1.y, p2.y));
    mx.z = max_std(p0.z, max_std(p1.z, p2.z));
    mn.w = __uint_as_float(ti);
    mx.w = 0.f;
    node_box[2 * static_cast<size_t>(i)] = mn;
    node_box[2 * static_cast<size_t>(i) + 1] = mx;
    mn.w = __uint_as_float(i);
    mx.w = __uint_as_float(1u);
    clusters[2 * static_cast<size_t>(i)] = mn;
    clusters[2 * static_cast<size_t>(i) + 1] = mx;
    // sorted order: triangle id in the first .w, model id in the second
    // (read by the shading pass)
    xtri[3 * static_cast<size_t>(i) + 0] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(ti));
    xtri[3 * static_cast<size_t>(i) + 1] = make_float4(p1.x, p1.y, p1.z, __uint_as_float(t.model));
    xtri[3 * static_cast<size_t>(i) + 2] = make_float4(p2.x, p2.y, p2.z, 0.f);
}

// ================================================ K3: one PLOC iteration
// For the n live clusters (Morton order, 32-byte records: min.xyz|node id,
// max.xyz|leaf count) a tile starting at position s with R = radius does:
//   nearest neighbour of the TILE positions [s-R, s-R+TILE) in [i-R, i+R]
//     by surface area of the merged box, first strict minimum = lowest j on
//     ties (bvh.cpp:193-210);
//   merge decisions for its own ploc_own(R) = TILE-2R positions [s, e):
//     mutual pairs merge at the lower position (bvh.cpp:159-191);
//   exclusive scan of survivors and compaction (bvh.cpp:125-156), with the
//     scan across tiles done by decoupled look-back,
// so one launch is one reference iteration.  New nodes get ids it[iter].y +
// (merges before them); the last tile writes it[iter+1] = (live clusters,
// next id).
//
// Boxes of positions [s-2R, e+2R) are staged in shared memory as separate
// min/max coordinate arrays, position s-2R+w at index w; window entries
// outside [0, n) hold an infinite box (area +inf, never chosen under the strict
// minimum, as the reference never considers them).  Each thread keeps the
// boxes of its 4 consecutive positions in registers and walks the 2R+4 boxes
// around them once, reading two consecutive entries per 8-byte shared load
// (an even R keeps them aligned), so one load serves up to 8 area
// evaluations.
//
// The search compares areas computed from fminf/fmaxf boxes; those differ
// from the std::min/max boxes only in the sign of a zero, which changes no
// difference max - min and no comparison, so the chosen neighbour is the
// reference's.  Stored boxes use std::min/max semantics.
constexpr unsigned long long kPlAgg = 1ull << 62, kPlPrefix = 2ull << 62;
constexpr unsigned long long kPlMask31 = (1ull << 31) - 1ull;

__device__ __forceinline__ float sa_merged(float4 amn, float4 amx, float4 bmn, float4 bmx) {
    const float dx = fmaxf(amx.x, bmx.x) - fminf(amn.x, bmn.x);
    const float dy = fmaxf(amx.y, bmx.y) - fminf(amn.y, bmn.y);
    const float dz = fmaxf(amx.z, bmx.z) - fminf(amn.z, bmn.z);
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

template <int TILE, int BLOCK, int MAXR>
struct __align__(16) PlocSmem {
    static_assert(TILE == 4 * BLOCK, "four nearest-neighbour positions per thread");
    static constexpr int kWin = TILE + 2 * MAXR;  // positions [s-2R, e+2R), e - s <= TILE - 2R
    static_assert(kWin % 4 == 0, "aligned coordinate arrays");
    float mnx[kWin], mny[kWin], mnz[kWin], mxx[kWin], mxy[kWin], mxz[kWin];
    uint32_t id[kWin], lc[kWin];
    uint32_t nn[TILE];  // nearest neighbour of position s - R + i
    unsigned long long wsum[BLOCK / 32];
    unsigned long long prefix;
};

__device__ __forceinline__ float2 lds2(const float* a) { return *reinterpret_cast<const float2*>(a); }

// Nearest neighbours of this thread's positions q0..q0+3, q0 = s - R + 4t.
// RC > 0: the radius is the compile-time RC (even); RC == 0:
// runtime radius R, scalar loads.
template <int RC, int TILE, int BLOCK, int MAXR>
__device__ __forceinline__ void ploc_nearest(PlocSmem<TILE, BLOCK, MAXR>& S, int s, int e, int n, int R_rt) {
    const int R = RC > 0 ? RC : R_rt;
    const int q0 = s - R + 4 * static_cast<int>(threadIdx.x);
    if (q0 >= e + R) return;  // none of its positions is stored (no barrier in here)
    const int wq = 4 * static_cast<int>(threadIdx.x) + R;  // window index of q0
    float amnx[4], amny[4], amnz[4], amxx[4], amxy[4], amxz[4], best[4];
    int bj[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        amnx[i] = S.mnx[wq + i]; amny[i] = S.mny[wq + i]; amnz[i] = S.mnz[wq + i];
        amxx[i] = S.mxx[wq + i]; amxy[i] = S.mxy[wq + i]; amxz[i] = S.mxz[wq + i];
        best[i] = __int_as_float(0x7F800000);
        bj[i] = q0 + i;
    }
    // candidate at window offset d (position q0 + d) for own position i
    auto visit = [&](int d, int i, float bnx, float bny, float bnz, float bxx, float bxy, float bxz) {
        const float dx = fmaxf(amxx[i], bxx) - fminf(amnx[i], bnx);
        const float dy = fmaxf(amxy[i], bxy) - fminf(amny[i], bny);
        const float dz = fmaxf(amxz[i], bxz) - fminf(amnz[i], bnz);
        const float v = 2.0f * (dx * dy + dy * dz + dz * dx);
        if (v < best[i]) { best[i] = v; bj[i] = q0 + d; }
    };
    if (RC > 0) {
        static_assert(RC % 2 == 0, "aligned window pairs");
#pragma unroll
        for (int g = -RC; g <= RC + 2; g += 2) {
            const int w = wq + g;  // even: an 8-byte aligned pair of entries
            const float2 nx = lds2(S.mnx + w), ny = lds2(S.mny + w), nz = lds2(S.mnz + w);
            const float2 xx = lds2(S.mxx + w), xy = lds2(S.mxy + w), xz = lds2(S.mxz + w);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int d = g + u;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int k = d - i;
                    if (k != 0 && k >= -RC && k <= RC)
                        visit(d, i, u ? nx.y : nx.x, u ? ny.y : ny.x, u ? nz.y : nz.x, u ? xx.y : xx.x,
                              u ? xy.y : xy.x, u ? xz.y : xz.x);
                }
            }
            // keeps the next pair's loads below this pair's work: without it
            // every load of the unrolled walk is hoisted and the persistent
            // kernels (80 registers at 3 blocks per SM) spill
            asm volatile("" ::: "memory");
        }
    } else {
        for (int d = -R; d <= R + 3; ++d) {
            const int w = wq + d;
            const float bnx = S.mnx[w], bny = S.mny[w], bnz = S.mnz[w], bxx = S.mxx[w], bxy = S.mxy[w], bxz = S.mxz[w];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int k = d - i;
                if (k != 0 && k >= -R && k <= R) visit(d, i, bnx, bny, bnz, bxx, bxy, bxz);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int p = q0 + i;
        if (p >= 0 && p < n && p < e + R) S.nn[4 * threadIdx.x + i] = static_cast<uint32_t>(bj[i]);
    }
}

// Nearest neighbour of position p, whose box is at window index w (window
// entries outside [0, n) infinite): the 2R candidates in increasing j (strict
// minimum: lowest j on ties).  RC > 0: compile-time radius.
template <int RC, int TILE, int BLOCK, int MAXR>
__device__ __forceinline__ uint32_t ploc_nearest_at(const PlocSmem<TILE, BLOCK, MAXR>& S, int p, int w, int R_rt) {
    const int R = RC > 0 ? RC : R_rt;
    const float amnx = S.mnx[w], amny = S.mny[w], amnz = S.mnz[w], amxx = S.mxx[w], amxy = S.mxy[w], amxz = S.mxz[w];
    float best = __int_as_float(0x7F800000);
    int bj = p;
    auto visit = [&](int d) {
        const int wj = w + d;
        const float dx = fmaxf(amxx, S.mxx[wj]) - fminf(amnx, S.mnx[wj]);
        const float dy = fmaxf(amxy, S.mxy[wj]) - fminf(amny, S.mny[wj]);
        const float dz = fmaxf(amxz, S.mxz[wj]) - fminf(amnz, S.mnz[wj]);
        const float v = 2.0f * (dx * dy + dy * dz + dz * dx);
        if (v < best) { best = v; bj = p + d; }
    };
    if (RC > 0) {
#pragma unroll
        for (int d = -RC; d <= RC; ++d)
            if (d != 0) visit(d);
    } else {
        for (int d = -R; d <= R; ++d)
            if (d != 0) visit(d);
    }
    return static_cast<uint32_t>(bj);
}

// One tile of one PLOC iteration (see above).  Reads of data other blocks
// wrote (the cluster array) bypass L1 (__ldcg), so the same code is correct
// inside the persistent kernel, where no launch boundary separates iterations.
// IPT < 4: a tile owns ploc_own_ipt(R) = IPT*BLOCK - 2R positions and each
// thread searches IPT positions (instead of four): for iterations whose tiles
// all run at once, where a tile's latency is the iteration's.
template <int IPT, int BLOCK>
__host__ __device__ constexpr uint32_t ploc_own_ipt(int radius) {
    return static_cast<uint32_t>(IPT * BLOCK) - 2u * static_cast<uint32_t>(radius);
}
template <int TILE, int BLOCK, int MAXR, int IPT = 4>
__device__ __forceinline__ void ploc_tile(PlocSmem<TILE, BLOCK, MAXR>& S, uint32_t tile, const uint2 cur, int iter,
                                          const float4* __restrict__ cin, float4* __restrict__ cout,
                                          float4* __restrict__ node_box, uint4* __restrict__ node_kids, uint2* it,
                                          uint32_t N, int R, unsigned long long* lb_cur, unsigned long long* lb_next,
                                          uint32_t* err, uint32_t spin_limit) {
    static_assert(IPT == 1 || IPT == 2 || IPT == 4, "one, two or four positions per thread");
    constexpr bool SMALL = IPT < 4;
    const int own = static_cast<int>(SMALL ? ploc_own_ipt<IPT, BLOCK>(R) : ploc_own(R));
    const int n = static_cast<int>(cur.x);
    const int s = static_cast<int>(tile) * own;
    __syncthreads();  // the previous tile of this block is done with S
    if (threadIdx.x == 0) st_relaxed_u64(&lb_next[tile], 0ull);
    const int e = min(n, s + own);
    const int wbase = s - 2 * R;  // window index 0
    const int lo = max(0, wbase);
    const int hi = min(n, e + 2 * R);
    for (int p = lo + threadIdx.x; p < hi; p += BLOCK) {
        const float4 a = __ldcg(cin + 2 * static_cast<size_t>(p));
        const float4 b = __ldcg(cin + 2 * static_cast<size_t>(p) + 1);
        const int w = p - wbase;
        S.mnx[w] = a.x; S.mny[w] = a.y; S.mnz[w] = a.z; S.id[w] = __float_as_uint(a.w);
        S.mxx[w] = b.x; S.mxy[w] = b.y; S.mxz[w] = b.z; S.lc[w] = __float_as_uint(b.w);
    }
    {  // window entries of positions outside [0, n): infinite boxes
        const int kWin = SMALL ? IPT * BLOCK + 2 * R : PlocSmem<TILE, BLOCK, MAXR>::kWin;  // the entries the search reads
        const float inf = __int_as_float(0x7F800000);
        const int below = lo - wbase, above = hi - wbase;
        for (int w = threadIdx.x; w < kWin; w += BLOCK) {
            if (w >= below && w < above) continue;
            S.mnx[w] = -inf; S.mny[w] = -inf; S.mnz[w] = -inf;
            S.mxx[w] = inf; S.mxy[w] = inf; S.mxz[w] = inf;
        }
    }
    __syncthreads();
    if (SMALL) {
        // thread t: positions q = s - R + IPT*t + i at window index IPT*t + i + R;
        // [s - R, e + R) fits since e - s <= IPT*BLOCK - 2R
#pragma unroll
        for (int i = 0; i < IPT; ++i) {
            const int t = IPT * static_cast<int>(threadIdx.x) + i, q = s - R + t;
            if (q >= 0 && q < n && q < e + R) {
                uint32_t j;
                switch (R) {
                    case 8: j = ploc_nearest_at<8>(S, q, t + R, R); break;
                    case 16: j = ploc_nearest_at<16>(S, q, t + R, R); break;
                    case 32: j = ploc_nearest_at<32>(S, q, t + R, R); break;
                    default: j = ploc_nearest_at<0>(S, q, t + R, R); break;
                }
                S.nn[t] = j;
            }
        }
    } else {
        switch (R) {
            case 8: ploc_nearest<8>(S, s, e, n, R); break;
            case 16: ploc_nearest<16>(S, s, e, n, R); break;
            case 32: ploc_nearest<32>(S, s, e, n, R); break;
            default: ploc_nearest<0>(S, s, e, n, R); break;
        }
    }
    __syncthreads();

    // Decisions for the tile's own positions: thread t owns [s + t*IPT, +IPT).
    const int nbase = s - R;  // S.nn index 0
    uint32_t flags = 0;       // bit q: valid, bit 16+q: merge head
    uint32_t nv = 0, nm = 0;
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
        const int p = s + static_cast<int>(threadIdx.x) * IPT + q;
        if (p >= e) break;
        const int j = static_cast<int>(S.nn[p - nbase]);
        const bool mutual = (j != p) && (static_cast<int>(S.nn[j - nbase]) == p);
        const bool head = mutual && p < j;
        const bool gone = mutual && p > j;
        if (!gone) { flags |= 1u << q; ++nv; }
        if (head) { flags |= 1u << (16 + q); ++nm; }
    }
    // Block exclusive scan of (nv, nm) packed as 16|16 bits.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t packed = (nv << 16) | nm;
    uint32_t incl = packed;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) S.wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        // Warp 0: exclusive scan of the warp sums, then the look-back over
        // the preceding tiles, 32 status words per round trip.
        uint32_t ws = lane < BLOCK / 32 ? static_cast<uint32_t>(S.wsum[lane]) : 0u, wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < BLOCK / 32) S.wsum[lane] = wi - ws;
        const uint32_t run = __shfl_sync(0xFFFFFFFFu, wi, 31);
        const unsigned long long tv = run >> 16, tm = run & 0xFFFFu;
        unsigned long long ev = 0, em = 0;
        if (tile == 0) {
            if (lane == 0) st_relaxed_u64(&lb_cur[0], kPlPrefix | (tv << 31) | tm);
        } else {
            if (lane == 0) st_relaxed_u64(&lb_cur[tile], kPlAgg | (tv << 31) | tm);
            // Lane l reads the status word of tile k0 - l (32 predecessors per
            // round trip, nearest first); the sum runs down to the nearest
            // inclusive prefix.  (Four words per lane was measured slower:
            // the nearest prefix is usually a few tiles back.)
            long long k0 = static_cast<long long>(tile) - 1;
            SpinBound spin(spin_limit);
            while (true) {
                const long long k = k0 - lane;
                const unsigned long long v = k >= 0 ? ld_relaxed_u64(&lb_cur[k]) : kPlPrefix;
                const unsigned long long f = v & (3ull << 62);
                const uint32_t pm = __ballot_sync(0xFFFFFFFFu, f == kPlPrefix);
                const uint32_t zm = __ballot_sync(0xFFFFFFFFu, f == 0ull);
                const int stop = pm ? __ffs(pm) - 1 : 31;  // lanes 0..stop are summed
                const uint32_t upto = stop == 31 ? 0xFFFFFFFFu : ((2u << stop) - 1u);
                if (zm & upto) {  // a tile before the nearest prefix has not published yet
                    if (!spin.step()) { raise_error(err, kDevTimeout); break; }
                    continue;
                }
                unsigned long long cv = lane <= stop ? ((v >> 31) & kPlMask31) : 0ull;
                unsigned long long cm = lane <= stop ? (v & kPlMask31) : 0ull;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    cv += __shfl_xor_sync(0xFFFFFFFFu, cv, o);
                    cm += __shfl_xor_sync(0xFFFFFFFFu, cm, o);
                }
                ev += cv;
                em += cm;
                if (pm) break;
                k0 -= 32;
            }
            if (lane == 0) st_relaxed_u64(&lb_cur[tile], kPlPrefix | ((ev + tv) << 31) | (em + tm));
        }
        if (lane == 0) {
            S.prefix = (ev << 32) | em;
            if (e == n)  // last tile: size and id base of the next iteration
                it[iter + 1] = make_uint2(static_cast<uint32_t>(ev + tv), cur.y + static_cast<uint32_t>(em + tm));
        }
    }
    __syncthreads();
    const uint32_t excl = static_cast<uint32_t>(S.wsum[warp]) + (incl - packed);
    uint32_t out_v = static_cast<uint32_t>(S.prefix >> 32) + (excl >> 16);
    uint32_t out_m = cur.y + static_cast<uint32_t>(S.prefix & 0xFFFFFFFFull) + (excl & 0xFFFFu);
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
        if (!(flags & (1u << q))) continue;
        const int p = s + static_cast<int>(threadIdx.x) * IPT + q;
        const int wp = p - wbase;
        float4 mn = make_float4(S.mnx[wp], S.mny[wp], S.mnz[wp], __uint_as_float(S.id[wp]));
        float4 mx = make_float4(S.mxx[wp], S.mxy[wp], S.mxz[wp], __uint_as_float(S.lc[wp]));
        if (flags & (1u << (16 + q))) {
            const int j = static_cast<int>(S.nn[p - nbase]);
            const int wj = j - wbase;
            const uint32_t id = out_m++;
            if (id >= 2 * N - 1 || id < N) { raise_corrupt(err, 2 + (iter << 8), p, id); continue; }
            float4 m0, m1;  // AABB::merge (bvh.cpp:401-413), first argument = lower position
            m0.x = min_std(mn.x, S.mnx[wj]); m0.y = min_std(mn.y, S.mny[wj]); m0.z = min_std(mn.z, S.mnz[wj]);
            m1.x = max_std(mx.x, S.mxx[wj]); m1.y = max_std(mx.y, S.mxy[wj]); m1.z = max_std(mx.z, S.mxz[wj]);
            m0.w = mn.w;                      // left child id
            m1.w = __uint_as_float(S.id[wj]); // right child id
            node_box[2 * static_cast<size_t>(id)] = m0;
            node_box[2 * static_cast<size_t>(id) + 1] = m1;
            const uint32_t lc = S.lc[wp] + S.lc[wj];
            // children and their leaf counts, read by the DFS layout
            node_kids[id - N] = make_uint4(S.id[wp], S.id[wj], S.lc[wp], S.lc[wj]);
            mn = make_float4(m0.x, m0.y, m0.z, __uint_as_float(id));
            mx = make_float4(m1.x, m1.y, m1.z, __uint_as_float(lc));
        }
        if (out_v >= static_cast<uint32_t>(n)) { raise_corrupt(err, 3 + (iter << 8), p, out_v); continue; }
        cout[2 * static_cast<size_t>(out_v)] = mn;
        cout[2 * static_cast<size_t>(out_v) + 1] = mx;
        ++out_v;
    }
}

// The same for a whole-array window (position q at window index q + 2R).
template <int RC, int TILE, int BLOCK, int MAXR>
__device__ __forceinline__ uint32_t ploc_nearest_one(const PlocSmem<TILE, BLOCK, MAXR>& S, int p, int R_rt) {
    return ploc_nearest_at<RC>(S, p, p + 2 * (RC > 0 ? RC : R_rt), R_rt);
}

// The last PLOC iterations, once every live cluster fits in one tile (n <=
// ploc_own(R)): one block runs them with the clusters held in shared memory,
// in the window layout of a single tile starting at position 0 (position q at
// index q + 2R, infinite boxes outside [0, n)), so an iteration costs no
// global round trip; only the new nodes and the iteration records are written
// out.  Each iteration is the same reference iteration as ploc_tile's: the
// same nearest-neighbour search (ploc_nearest over the whole array while n >
// BLOCK, one position per thread below), mutual pairs merged at the lower
// position (AABB::merge), new ids in position order, survivors compacted in
// order.  Thread t decides positions [k t, k t + k), k = ceil(n / BLOCK) <=
// TILE / BLOCK; the compaction is in place, after a barrier that ends every
// read of the iteration's clusters.  Returns the iteration count.
template <int RC, int TILE, int BLOCK, int MAXR>
__device__ __noinline__ int ploc_tail_r(PlocSmem<TILE, BLOCK, MAXR>& S, int iter, int n, uint32_t idb,
                                           float4* __restrict__ node_box, uint4* __restrict__ node_kids, uint2* it,
                                           uint32_t N, int R_rt, uint32_t* err) {
    constexpr int PMAX = TILE / BLOCK;
    const int R = RC > 0 ? RC : R_rt;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float inf = __int_as_float(0x7F800000);
    while (n > 1) {
        if (static_cast<uint32_t>(iter) + 1 >= N) {
            if (threadIdx.x == 0) raise_error(err, kDevIterLimit);
            break;
        }
        if (n > BLOCK) {
            ploc_nearest<RC>(S, 0, n, n, R);  // S.nn[p + R] for p < n
        } else if (static_cast<int>(threadIdx.x) < n) {
            S.nn[threadIdx.x + R] = ploc_nearest_one<RC>(S, static_cast<int>(threadIdx.x), R);
        }
        __syncthreads();
        const int k = (n + BLOCK - 1) / BLOCK;
        const int p0 = k * static_cast<int>(threadIdx.x);
        uint32_t flags = 0, nv = 0, nm = 0;
#pragma unroll
        for (int q = 0; q < PMAX; ++q) {
            const int p = p0 + q;
            if (q >= k || p >= n) continue;
            const int j = static_cast<int>(S.nn[p + R]);
            const bool mutual = (j != p) && (static_cast<int>(S.nn[j + R]) == p);
            if (!(mutual && p > j)) { flags |= 1u << q; ++nv; }
            if (mutual && p < j) { flags |= 1u << (16 + q); ++nm; }
        }
        // exclusive scan of (survivors, merges) in position order, 16|16 bits
        const uint32_t packed = (nv << 16) | nm;
        uint32_t incl = packed;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) S.wsum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t ws = lane < BLOCK / 32 ? static_cast<uint32_t>(S.wsum[lane]) : 0u;
            uint32_t wi = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
                if (lane >= o) wi += y;
            }
            if (lane < BLOCK / 32) S.wsum[lane] = wi - ws;
            if (lane == 31) S.prefix = wi;  // block totals
        }
        __syncthreads();
        const uint32_t excl = static_cast<uint32_t>(S.wsum[warp]) + (incl - packed);
        const uint32_t total = static_cast<uint32_t>(S.prefix);
        uint32_t out_v = excl >> 16;
        uint32_t out_m = idb + (excl & 0xFFFFu);
        float4 omn[PMAX], omx[PMAX];
#pragma unroll
        for (int q = 0; q < PMAX; ++q) {
            if (!(flags & (1u << q))) continue;
            const int p = p0 + q, wp = p + 2 * R;
            float4 mn = make_float4(S.mnx[wp], S.mny[wp], S.mnz[wp], __uint_as_float(S.id[wp]));
            float4 mx = make_float4(S.mxx[wp], S.mxy[wp], S.mxz[wp], __uint_as_float(S.lc[wp]));
            if (flags & (1u << (16 + q))) {
                const int wj = static_cast<int>(S.nn[p + R]) + 2 * R;
                const uint32_t id = out_m++;
                if (id >= 2 * N - 1 || id < N) {
                    raise_corrupt(err, 13 + (iter << 8), p, id);
                    flags &= ~(1u << q);
                    continue;
                }
                float4 m0, m1;  // AABB::merge (bvh.cpp:401-413), first argument = lower position
                m0.x = min_std(mn.x, S.mnx[wj]); m0.y = min_std(mn.y, S.mny[wj]); m0.z = min_std(mn.z, S.mnz[wj]);
                m1.x = max_std(mx.x, S.mxx[wj]); m1.y = max_std(mx.y, S.mxy[wj]); m1.z = max_std(mx.z, S.mxz[wj]);
                m0.w = mn.w;                      // left child id
                m1.w = __uint_as_float(S.id[wj]); // right child id
                node_box[2 * static_cast<size_t>(id)] = m0;
                node_box[2 * static_cast<size_t>(id) + 1] = m1;
                node_kids[id - N] = make_uint4(S.id[wp], S.id[wj], S.lc[wp], S.lc[wj]);
                mn = make_float4(m0.x, m0.y, m0.z, __uint_as_float(id));
                mx = make_float4(m1.x, m1.y, m1.z, __uint_as_float(S.lc[wp] + S.lc[wj]));
            }
            omn[q] = mn;
            omx[q] = mx;
        }
        __syncthreads();  // every read of this iteration's clusters is done: compact in place
        const int n_next = static_cast<int>(total >> 16);
        const uint32_t merges = total & 0xFFFFu;
#pragma unroll
        for (int q = 0; q < PMAX; ++q) {
            if (!(flags & (1u << q))) continue;
            if (out_v >= static_cast<uint32_t>(n_next)) {
                raise_corrupt(err, 14 + (iter << 8), p0 + q, out_v);
                continue;
            }
            const int w = static_cast<int>(out_v) + 2 * R;
            S.mnx[w] = omn[q].x; S.mny[w] = omn[q].y; S.mnz[w] = omn[q].z; S.id[w] = __float_as_uint(omn[q].w);
            S.mxx[w] = omx[q].x; S.mxy[w] = omx[q].y; S.mxz[w] = omx[q].z; S.lc[w] = __float_as_uint(omx[q].w);
            ++out_v;
        }
        for (int q = n_next + static_cast<int>(threadIdx.x); q < n; q += BLOCK) {  // vacated positions
            const int w = q + 2 * R;
            S.mnx[w] = -inf; S.mny[w] = -inf; S.mnz[w] = -inf;
            S.mxx[w] = inf; S.mxy[w] = inf; S.mxz[w] = inf;
        }
        if (threadIdx.x == 0) it[iter + 1] = make_uint2(static_cast<uint32_t>(n_next), idb + merges);
        n = n_next;
        idb += merges;
        ++iter;
        __syncthreads();
    }
    return iter;
}

// Stages the tail's clusters (input of iteration iter) and runs ploc_tail_r
// with the compile-time radius when there is one.
template <int TILE, int BLOCK, int MAXR>
__device__ __forceinline__ int ploc_tail(PlocSmem<TILE, BLOCK, MAXR>& S, int iter, const float4* __restrict__ cin,
                                         float4* __restrict__ node_box, uint4* __restrict__ node_kids, uint2* it,
                                         uint32_t N, int R, uint32_t* err) {
    constexpr int kWin = PlocSmem<TILE, BLOCK, MAXR>::kWin;
    __syncthreads();
    const uint2 cur = __ldcg(it + iter);
    const int n = static_cast<int>(cur.x);
    if (n + 4 * R > kWin || n > TILE) {  // the caller checked n <= ploc_own(R); only corruption gets here
        if (threadIdx.x == 0) raise_corrupt(err, 12, static_cast<uint32_t>(iter), static_cast<uint32_t>(n));
        return iter;
    }
    const float inf = __int_as_float(0x7F800000);
    for (int w = threadIdx.x; w < kWin; w += BLOCK) {
        const int p = w - 2 * R;
        if (p >= 0 && p < n) {
            const float4 a = __ldcg(cin + 2 * static_cast<size_t>(p));
            const float4 b = __ldcg(cin + 2 * static_cast<size_t>(p) + 1);
            S.mnx[w] = a.x; S.mny[w] = a.y; S.mnz[w] = a.z; S.id[w] = __float_as_uint(a.w);
            S.mxx[w] = b.x; S.mxy[w] = b.y; S.mxz[w] = b.z; S.lc[w] = __float_as_uint(b.w);
        } else {
            S.mnx[w] = -inf; S.mny[w] = -inf; S.mnz[w] = -inf;
            S.mxx[w] = inf; S.mxy[w] = inf; S.mxz[w] = inf;
        }
    }
    __syncthreads();
    switch (R) {
        case 8: return ploc_tail_r<8>(S, iter, n, cur.y, node_box, node_kids, it, N, R, err);
        case 16: return ploc_tail_r<16>(S, iter, n, cur.y, node_box, node_kids, it, N, R, err);
        case 32: return ploc_tail_r<32>(S, iter, n, cur.y, node_box, node_kids, it, N, R, err);
        default: return ploc_tail_r<0>(S, iter, n, cur.y, node_box, node_kids, it, N, R, err);
    }
}

template <int TILE, int BLOCK, int MAXR>
__global__ void __launch_bounds__(BLOCK) ploc_iteration_kernel(const float4* __restrict__ cin, float4* __restrict__ cout,
                                                               float4* __restrict__ node_box, uint4* __restrict__ node_kids,
                                                               uint2* it, int iter, uint32_t N,
                                                               int R, unsigned long long* lookback, uint32_t* tickets,
                                                               uint32_t n_tiles_cap, uint32_t* err, uint32_t spin_limit) {
    __shared__ PlocSmem<TILE, BLOCK, MAXR> S;
    __shared__ uint32_t s_tile;
    const uint2 cur = it[iter];
    const uint32_t n = cur.x;
    if (n <= 1u) {
        // Finished: carry the state forward so a later launch of this build
        // never reads an entry left over from an earlier build.
        if (blockIdx.x == 0 && threadIdx.x == 0) it[iter + 1] = cur;
        return;
    }
    unsigned long long* lb_cur = lookback + static_cast<size_t>(iter & 1) * n_tiles_cap;
    unsigned long long* lb_next = lookback + static_cast<size_t>((iter + 1) & 1) * n_tiles_cap;
    if (threadIdx.x == 0) s_tile = atomicAdd(&tickets[iter & 1], 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile * ploc_own(R) >= n) return;
    if (tile == 0 && threadIdx.x == 0) tickets[(iter + 1) & 1] = 0u;
    ploc_tile<TILE, BLOCK, MAXR>(S, tile, cur, iter, cin, cout, node_box, node_kids, it, N, R, lb_cur, lb_next, err,
                                 spin_limit);
}

// ================================================== K4: DFS node layout
// Scene::recursiveTopDownTraversalBVH (scene.cpp:189-201): pre-order, left
// subtree first, root (the last merge, id 2N-2) at 0.  A node at position p
// puts its left child at p+1 and its right child at p + 2*leaves(left).
//
// Two passes.  (a) Top-down: nodes created in PLOC iteration k only have
// parents from later iterations, so levels run from the last iteration
// down; a node reads its (DFS position, first leaf below, depth parity),
// passes them to its children and records dfs[p] = node id for itself and
// for its leaf children.  Only these few words move per node.  (b) One
// parallel pass over the DFS positions in order writes every output record
// once, so the node array and the traversal nodes are written coalesced.
//
// Output (b) also writes the traversal's own node format: one 64-byte record
// per internal node holding both children's boxes and references, indexed by
// the node's rank among internal nodes in DFS order (position minus the
// leaves before it, i.e. minus its first leaf).  Leaves are referenced by
// their position in the tree's left-to-right leaf order (the number of
// leaves before them in DFS order) — which is not their sorted position:
// PLOC merges clusters that are not adjacent in Morton order, so subtrees
// interleave there — and the parent of each leaf moves that leaf's
// transformed triangle into that order.  The traversal's tie rule (equal t:
// the leaf later in DFS order, which the shader visits first) and every
// subtree's leaves forming one contiguous range rest on this order.
constexpr uint32_t kLayoutUnset = 0xFFFFFFFFu;  // a position not yet published (dataflow layout)

__device__ __forceinline__ uint2 layout_place(uint32_t X, const uint2* __restrict__ pf, uint32_t N) {
    // (DFS position, first leaf below | depth parity << 31) of X; the root sits at (0, 0)
    return (X == 2 * N - 2) ? make_uint2(0u, 0u) : __ldcg(pf + (X - N));
}

// Position pass for internal node X placed at me = (position, first leaf |
// parity << 31).  PUBLISH: each internal child's record goes out as one
// 64-bit relaxed store, which a thread polling for it (the dataflow layout
// below) reads whole; the record is all it needs from the parent.
// kids: X's node_kids record (left id, right id, their leaf counts), which the
// dataflow pass loads before it waits for X's position.
template <bool PUBLISH>
__device__ __forceinline__ void layout_down_at(uint32_t X, uint2 me, const uint4 kids, uint2* __restrict__ pf,
                                               uint32_t N, uint32_t* __restrict__ dfs, uint32_t* err) {
    const uint32_t p = me.x, f = me.y & 0x7FFFFFFFu, odd = me.y >> 31;
    const uint32_t a = kids.x, b = kids.y, lca = kids.z;
    const uint32_t pl = p + 1, pr = p + 2 * lca;
    if (pr >= 2 * N - 1 || p < f || p - f >= N - 1 || (b >= N && b - N >= N - 1) || (a >= N && a - N >= N - 1)) {
        raise_corrupt(err, 4, X, pr);
        return;
    }
    dfs[p] = X;
    const uint32_t nodd = (odd ^ 1u) << 31;
    if (PUBLISH) {
        auto word = [](uint32_t pos, uint32_t first) {
            return (static_cast<unsigned long long>(first) << 32) | pos;
        };
        if (a < N) dfs[pl] = a;
        else st_relaxed_u64(reinterpret_cast<unsigned long long*>(pf + (a - N)), word(pl, f | nodd));
        if (b < N) dfs[pr] = b;
        else st_relaxed_u64(reinterpret_cast<unsigned long long*>(pf + (b - N)), word(pr, (f + lca) | nodd));
        return;
    }
    if (a < N) dfs[pl] = a; else pf[a - N] = make_uint2(pl, f | nodd);
    if (b < N) dfs[pr] = b; else pf[b - N] = make_uint2(pr, (f + lca) | nodd);
}

// The dataflow pass also publishes the places of X's grandchildren (from its
// children's node_kids records kc[0], kc[1], loaded while X waited), so
// places travel two levels per round trip through L2.  X's internal child
// later publishes the same words (the same arithmetic on the same inputs);
// whichever store lands first, the word is the same.  Out-of-range records
// are skipped here: the child's own pass reports them.
__device__ __forceinline__ void layout_publish_grandchildren(uint2 me, const uint4 kids, const uint4 kc[2],
                                                            uint2* __restrict__ pf, uint32_t N) {
    const uint32_t p = me.x, f = me.y & 0x7FFFFFFFu, odd = me.y >> 31;
    const uint32_t cp[2] = {p + 1, p + 2 * kids.z}, cf[2] = {f, f + kids.z};
    const uint32_t gpar = odd << 31;  // two levels down: X's own depth parity
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const uint32_t id = c ? kids.y : kids.x;
        if (id < N || id - N >= N - 1) continue;  // a leaf child (or corrupt)
        const uint32_t ga = kc[c].x, gb = kc[c].y, lga = kc[c].z;
        const uint32_t gpl = cp[c] + 1, gpr = cp[c] + 2 * lga;
        if (gpr >= 2 * N - 1) continue;
        if (ga >= N && ga - N < N - 1)
            st_relaxed_u64(reinterpret_cast<unsigned long long*>(pf + (ga - N)),
                           (static_cast<unsigned long long>(cf[c] | gpar) << 32) | gpl);
        if (gb >= N && gb - N < N - 1)
            st_relaxed_u64(reinterpret_cast<unsigned long long*>(pf + (gb - N)),
                           (static_cast<unsigned long long>((cf[c] + lga) | gpar) << 32) | gpr);
    }
}

__device__ __forceinline__ void layout_down(uint32_t X, const uint4* __restrict__ node_kids, uint2* __restrict__ pf,
                                            uint32_t N, uint32_t* __restrict__ dfs, uint32_t* err) {
    layout_down_at<false>(X, layout_place(X, pf, N), __ldcg(node_kids + (X - N)), pf, N, dfs, err);
}

// grow: the scene's abs_eps; wide_wt receives the traversal nodes with every
// child box grown by it (min - grow, max + grow, rounded as the traversal's
// own box growth would round them), for watertight traces.
__device__ __forceinline__ void layout_emit(uint32_t p, const float4* __restrict__ node_box,
                                            const uint4* __restrict__ node_kids, const uint2* __restrict__ pf,
                                            uint32_t N, const uint32_t* __restrict__ dfs, crt_bvh_node* __restrict__ out,
                                            float4* __restrict__ wide, float4* __restrict__ wide_wt,
                                            uint8_t* __restrict__ depth_odd, const LeafOut& lv, float grow,
                                            uint32_t* err) {
    const uint32_t X = __ldcg(dfs + p);
    if (X >= 2 * N - 1) { raise_corrupt(err, 5, p, X); return; }
    const float4 mn = __ldcg(node_box + 2 * static_cast<size_t>(X)), mx = __ldcg(node_box + 2 * static_cast<size_t>(X) + 1);
    float4* o = reinterpret_cast<float4*>(out + p);
    o[0] = make_float4(mn.x, mn.y, mn.z, 0.f);
    o[1] = make_float4(mx.x, mx.y, mx.z, 0.f);
    if (X < N) {  // leaf: its triangle
        reinterpret_cast<uint4*>(o)[2] = make_uint4(__float_as_uint(mn.w), 0u, 0u, 0u);
        return;
    }
    const uint2 me = layout_place(X, pf, N);
    const uint32_t f = me.y & 0x7FFFFFFFu, odd = me.y >> 31;
    const uint4 kids = __ldcg(node_kids + (X - N));
    const uint32_t a = kids.x, b = kids.y, lca = kids.z, lcb = kids.w;
    const uint32_t pl = p + 1, pr = p + 2 * lca;
    if (p < f || p - f >= N - 1) { raise_corrupt(err, 6, p, f); return; }
    reinterpret_cast<uint4*>(o)[2] = make_uint4(0u, pl, pr, 0u);
    const uint32_t ch[2] = {a, b}, cp[2] = {pl, pr}, cf[2] = {f, f + lca};
    float4 cmn[2], cmx[2];
    uint32_t cref[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        cmn[c] = __ldcg(node_box + 2 * static_cast<size_t>(ch[c]));
        cmx[c] = __ldcg(node_box + 2 * static_cast<size_t>(ch[c]) + 1);
        cref[c] = (ch[c] < N) ? (kLeafRef | cf[c])  // leaf: its position in tree order
                              : (cp[c] - cf[c]);    // internal: its rank among internal nodes in DFS order
        if (ch[c] < N) {  // move the leaf's triangle from sorted to tree order
            if (cf[c] >= N) { raise_corrupt(err, 6, p, cf[c]); continue; }
            const float4* src = lv.xtri_sorted + 3 * static_cast<size_t>(ch[c]);
            float4* dst = lv.xtri + 3 * static_cast<size_t>(cf[c]);
            const float4 t0 = __ldcg(src), t1 = __ldcg(src + 1), t2 = __ldcg(src + 2);
            dst[0] = t0;
            dst[1] = t1;
            dst[2] = t2;
            const uint32_t ti = __float_as_uint(t0.w);
            if (ti < N) lv.leaf_of_tri[ti] = cf[c];
            else raise_corrupt(err, 6, p, ti);
        }
    }
    if (depth_odd) depth_odd[p - f] = static_cast<uint8_t>(odd);
    float4* w = wide + 4 * static_cast<size_t>(p - f);
    w[0] = make_float4(cmn[0].x, cmn[0].y, cmn[0].z, __uint_as_float(cref[0]));
    w[1] = make_float4(cmx[0].x, cmx[0].y, cmx[0].z, __uint_as_float(cref[1]));
    w[2] = make_float4(cmn[1].x, cmn[1].y, cmn[1].z, __uint_as_float(lca));  // leaf counts of the children
    w[3] = make_float4(cmx[1].x, cmx[1].y, cmx[1].z, __uint_as_float(lcb));
    float4* g = wide_wt + 4 * static_cast<size_t>(p - f);
    g[0] = make_float4(cmn[0].x - grow, cmn[0].y - grow, cmn[0].z - grow, __uint_as_float(cref[0]));
    g[1] = make_float4(cmx[0].x + grow, cmx[0].y + grow, cmx[0].z + grow, __uint_as_float(cref[1]));
    g[2] = make_float4(cmn[1].x - grow, cmn[1].y - grow, cmn[1].z - grow, __uint_as_float(lca));
    g[3] = make_float4(cmx[1].x + grow, cmx[1].y + grow, cmx[1].z + grow, __uint_as_float(lcb));
}

__global__ void __launch_bounds__(256) layout_level_kernel(const uint4* __restrict__ node_kids,
                                                           uint2* __restrict__ pf, uint32_t id_begin, uint32_t id_end,
                                                           uint32_t N, uint32_t* __restrict__ dfs, uint32_t* err) {
    const uint32_t X = id_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (X >= id_end) return;
    layout_down(X, node_kids, pf, N, dfs, err);
}

__global__ void __launch_bounds__(256) layout_emit_kernel(const float4* __restrict__ node_box,
                                                          const uint4* __restrict__ node_kids,
                                                          const uint2* __restrict__ pf, uint32_t N,
                                                          const uint32_t* __restrict__ dfs, crt_bvh_node* __restrict__ out,
                                                          float4* __restrict__ wide, float4* __restrict__ wide_wt,
                                                          uint8_t* __restrict__ depth_odd, LeafOut lv,
                                                          const SceneState* __restrict__ st, uint32_t* err) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= 2 * N - 1) return;
    layout_emit(p, node_box, node_kids, pf, N, dfs, out, wide, wide_wt, depth_odd, lv, st->abs_eps, err);
}

// ================================== K3+K4 fused: one persistent launch
// All PLOC iterations, then all layout levels, separated by a grid-wide
// barrier (co-residency guaranteed by a cooperative launch; every wait is
// bounded and a timeout ends every block).  Saves the per-iteration launch
// and the host round trips the multi-launch path needs.
__device__ __forceinline__ bool grid_barrier(unsigned long long* bar, unsigned long long& target, uint32_t* err,
                                             uint32_t spin_limit) {
    // A 64-bit arrival counter that only grows (zeroed before the launch):
    // barrier k is complete when it reaches k * gridDim, so a block needs one
    // fence and one atomic, then polls; no reset and no release step.
    // `target` is this block's running count (thread 0's copy is used).
    __syncthreads();
    if (threadIdx.x == 0) {
        target += gridDim.x;
        __threadfence();
        atomicAdd(bar, 1ull);
        SpinBound spin(spin_limit);
        while (ld_acquire_u64(bar) < target)
            if (!spin.step()) { raise_error(err, kDevTimeout); break; }
    }
    __syncthreads();
    return (ld_acquire_u32(err) & kDevTimeout) == 0u;
}

template <int TILE, int BLOCK, int MAXR>
__global__ void __launch_bounds__(BLOCK, kPlocBlocksPerSm) ploc_persistent_kernel(float4* ca, float4* cb, float4* __restrict__ node_box,
                                                                uint4* __restrict__ node_kids, uint2* it, uint32_t N,
                                                                int R, unsigned long long* lookback, uint32_t* tickets,
                                                                uint32_t n_tiles_cap, uint2* pf, crt_bvh_node* out,
                                                                float4* wide, float4* wide_wt, uint8_t* depth_odd,
                                                                LeafOut lv, const SceneState* st, unsigned long long* bar,
                                                                uint32_t* iters_out, uint32_t* err, uint32_t spin_limit) {
    __shared__ PlocSmem<TILE, BLOCK, MAXR> S;
    __shared__ uint32_t s_tile;
    unsigned long long bar_target = 0;  // grid barriers passed x gridDim (thread 0)
    // iters_out[0]: iterations; [1]: blocks finished; then 64-bit globaltimer
    // stamps: start, end of the PLOC loop, end of the layout.
    unsigned long long* stamp = reinterpret_cast<unsigned long long*>(iters_out + 2);
    if (blockIdx.x == 0 && threadIdx.x == 0) stamp[0] = global_ns();
    // The layout's records start unset: a node's position arrives from its
    // parent (pf is not touched by the PLOC iterations, whose grid barriers
    // order this reset before the layout).
    for (uint32_t j = blockIdx.x * BLOCK + threadIdx.x; j + 1 < N; j += gridDim.x * BLOCK)
        pf[j] = make_uint2(kLayoutUnset, 0u);
    int iter = 0;
    bool tail = false;
    for (;; ++iter) {
        const uint2 cur = __ldcg(it + iter);
        if (cur.x <= 1u) break;
        if (cur.x <= ploc_own(R)) { tail = true; break; }  // every block reads the same record
        const float4* cin = (iter & 1) ? cb : ca;
        float4* cout = (iter & 1) ? ca : cb;
        unsigned long long* lb_cur = lookback + static_cast<size_t>(iter & 1) * n_tiles_cap;
        unsigned long long* lb_next = lookback + static_cast<size_t>((iter + 1) & 1) * n_tiles_cap;
        const uint32_t n_tiles = (cur.x + ploc_own(R) - 1) / ploc_own(R);
        const uint32_t n_t1 = (cur.x + ploc_own_ipt<1, BLOCK>(R) - 1) / ploc_own_ipt<1, BLOCK>(R);
        const uint32_t n_t2 = (cur.x + ploc_own_ipt<2, BLOCK>(R) - 1) / ploc_own_ipt<2, BLOCK>(R);
        // one (two) positions per thread while those smaller tiles number at
        // most kPlocSmallTiles1 (kPlocSmallTiles2) per SM and fit the look-back
        // arrays: the iteration then costs one short tile's latency
        const uint32_t per_sm = gridDim.x / kPlocBlocksPerSm;
        const int ipt = (n_t1 <= kPlocSmallTiles1 * per_sm && n_t1 <= n_tiles_cap)   ? 1
                        : (n_t2 <= kPlocSmallTiles2 * per_sm && n_t2 <= n_tiles_cap) ? 2
                                                                                      : 4;
        const bool small = ipt < 4;
        if (small || n_tiles <= gridDim.x) {
            // One wave: block b runs tile b (all tiles are co-resident, so
            // every look-back wait ends), with no ticket round trips.
            if (blockIdx.x == 0 && threadIdx.x == 0) tickets[(iter + 1) & 1] = 0u;
            // Every block clears its word of the next iteration's look-back
            // array: the next iteration may cut its (fewer) clusters into more,
            // smaller tiles than this one has, and a tile clears only its own
            // word (the grid barrier below orders these stores before any read).
            if (threadIdx.x == 0 && blockIdx.x < n_tiles_cap) st_relaxed_u64(&lb_next[blockIdx.x], 0ull);
            if (ipt == 1) {
                if (blockIdx.x < n_t1)
                    ploc_tile<TILE, BLOCK, MAXR, 1>(S, blockIdx.x, cur, iter, cin, cout, node_box, node_kids, it, N, R,
                                                    lb_cur, lb_next, err, spin_limit);
            } else if (ipt == 2) {
                if (blockIdx.x < n_t2)
                    ploc_tile<TILE, BLOCK, MAXR, 2>(S, blockIdx.x, cur, iter, cin, cout, node_box, node_kids, it, N, R,
                                                    lb_cur, lb_next, err, spin_limit);
            } else if (blockIdx.x < n_tiles) {
                ploc_tile<TILE, BLOCK, MAXR>(S, blockIdx.x, cur, iter, cin, cout, node_box, node_kids, it, N, R, lb_cur,
                                             lb_next, err, spin_limit);
            }
            if (!grid_barrier(bar, bar_target, err, spin_limit)) return;
            if (static_cast<uint32_t>(iter) + 1 >= N) { raise_error(err, kDevIterLimit); return; }
            continue;
        }
        // More tiles than blocks: a block takes its next ticket only when it
        // has finished a tile, so tickets follow completion order and a
        // tile's look-back finds its predecessors already published.
        for (;;) {
            __syncthreads();
            if (threadIdx.x == 0) s_tile = atomicAdd(&tickets[iter & 1], 1u);
            __syncthreads();
            const uint32_t tile = s_tile;
            if (tile * ploc_own(R) >= cur.x) break;
            if (tile == 0 && threadIdx.x == 0) tickets[(iter + 1) & 1] = 0u;
            ploc_tile<TILE, BLOCK, MAXR>(S, tile, cur, iter, cin, cout, node_box, node_kids, it, N, R, lb_cur, lb_next,
                                         err, spin_limit);
        }
        if (!grid_barrier(bar, bar_target, err, spin_limit)) return;
        if (static_cast<uint32_t>(iter) + 1 >= N) { raise_error(err, kDevIterLimit); return; }
    }
    if (tail) {
        // The remaining iterations fit in one tile each (the last few hundred
        // clusters, which merge a few pairs per iteration): block 0 runs them
        // alone on shared memory, while the others wait once.
        if (blockIdx.x == 0) {
            iter = ploc_tail<TILE, BLOCK, MAXR>(S, iter, (iter & 1) ? cb : ca, node_box, node_kids, it, N, R, err);
            if (threadIdx.x == 0) iters_out[0] = static_cast<uint32_t>(iter);
        }
        if (!grid_barrier(bar, bar_target, err, spin_limit)) return;
        iter = static_cast<int>(__ldcg(iters_out));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        iters_out[0] = static_cast<uint32_t>(iter);
        stamp[1] = global_ns();
    }
    // DFS layout, position pass as dataflow: internal node ids grow with the
    // PLOC iteration that made them, so a parent's id is larger than its
    // children's and decreasing ids are a top-down order.  Every thread takes
    // the ids 2N-2, 2N-3, ... in grid-stride order and, before laying node X
    // out, waits (bounded) until X's parent has published X's position.  The
    // unfinished node with the largest id never waits (its parent is done), so
    // the co-resident grid always progresses; one grid barrier before the
    // emit pass replaces one barrier per PLOC level.
    uint32_t* dfs = reinterpret_cast<uint32_t*>(ca);
    bool gave_up = false;
    for (uint32_t t = blockIdx.x * BLOCK + threadIdx.x; t + 1 < N && !gave_up; t += gridDim.x * BLOCK) {
        const uint32_t X = 2 * N - 2 - t;
        // X's record (and, for the grid's first round of nodes, the top of the
        // tree, where the chain of places is the latency that counts, its
        // internal children's), in flight while X's place is awaited
        const bool top = t < gridDim.x * BLOCK;
        const uint4 kids = __ldcg(node_kids + (X - N));
        uint4 kc[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
        if (top && kids.x >= N && kids.x - N < N - 1) kc[0] = __ldcg(node_kids + (kids.x - N));
        if (top && kids.y >= N && kids.y - N < N - 1) kc[1] = __ldcg(node_kids + (kids.y - N));
        uint2 me = make_uint2(0u, 0u);  // the root's place
        if (X != 2 * N - 2) {
            const unsigned long long* w = reinterpret_cast<const unsigned long long*>(pf + (X - N));
            unsigned long long v = ld_relaxed_u64(w);
            SpinBound spin(spin_limit);
            while (static_cast<uint32_t>(v) == kLayoutUnset) {
                if (!spin.step()) {
                    raise_error(err, kDevTimeout);
                    gave_up = true;
                    break;
                }
                v = ld_relaxed_u64(w);
            }
            if (gave_up) break;
            me = make_uint2(static_cast<uint32_t>(v), static_cast<uint32_t>(v >> 32));
        }
        if (top) layout_publish_grandchildren(me, kids, kc, pf, N);
        layout_down_at<true>(X, me, kids, pf, N, dfs, err);
    }
    if (!grid_barrier(bar, bar_target, err, spin_limit)) return;
    const float grow = st->abs_eps;
    for (uint32_t p = blockIdx.x * BLOCK + threadIdx.x; p < 2 * N - 1; p += gridDim.x * BLOCK)
        layout_emit(p, node_box, node_kids, pf, N, dfs, out, wide, wide_wt, depth_odd, lv, grow, err);
    __syncthreads();
    if (threadIdx.x == 0 && atomicAdd(iters_out + 1, 1u) + 1u == gridDim.x) stamp[2] = global_ns();
}

__global__ void single_leaf_kernel(const float4* __restrict__ node_box, crt_bvh_node* __restrict__ out, LeafOut lv) {
    const float4 mn = node_box[0], mx = node_box[1];
    float4* o = reinterpret_cast<float4*>(out);
    o[0] = make_float4(mn.x, mn.y, mn.z, 0.f);
    o[1] = make_float4(mx.x, mx.y, mx.z, 0.f);
    reinterpret_cast<uint4*>(o)[2] = make_uint4(__float_as_uint(mn.w), 0u, 0u, 0u);
    for (int k = 0; k < 3; ++k) lv.xtri[k] = lv.xtri_sorted[k];
    lv.leaf_of_tri[0] = 0u;
}

// ========================================== K4b: 4-wide traversal nodes
// Every internal node at even depth becomes a 128-byte 4-wide node holding
// its children's children (a leaf child stays itself): SoA boxes (min x of
// the four, min y, ..., max z) and the four references; empty slots carry
// kNoChild and an empty box.  Nodes keep the binary node's index (odd-depth
// slots stay unused), so references are unchanged and exact boxes stay exact.
__global__ void __launch_bounds__(256) wide4_kernel(const float4* __restrict__ wide, const uint8_t* __restrict__ depth_odd,
                                                    uint32_t n_internal, float4* __restrict__ wide4) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_internal || depth_odd[i]) return;
    float mnx[4], mny[4], mnz[4], mxx[4], mxy[4], mxz[4];
    uint32_t ref[4];
    int k = 0;
    const float4* w = wide + 4 * static_cast<size_t>(i);
    const float4 w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3];
    const float4 cmn[2] = {w0, w2}, cmx[2] = {w1, w3};
    const uint32_t cref[2] = {__float_as_uint(w0.w), __float_as_uint(w1.w)};
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        if (cref[c] & kLeafRef) {
            mnx[k] = cmn[c].x; mny[k] = cmn[c].y; mnz[k] = cmn[c].z;
            mxx[k] = cmx[c].x; mxy[k] = cmx[c].y; mxz[k] = cmx[c].z;
            ref[k++] = cref[c];
        } else {
            const float4* g = wide + 4 * static_cast<size_t>(cref[c]);
            const float4 g0 = g[0], g1 = g[1], g2 = g[2], g3 = g[3];
            mnx[k] = g0.x; mny[k] = g0.y; mnz[k] = g0.z; mxx[k] = g1.x; mxy[k] = g1.y; mxz[k] = g1.z;
            ref[k++] = __float_as_uint(g0.w);
            mnx[k] = g2.x; mny[k] = g2.y; mnz[k] = g2.z; mxx[k] = g3.x; mxy[k] = g3.y; mxz[k] = g3.z;
            ref[k++] = __float_as_uint(g1.w);
        }
    }
    const float inf = __int_as_float(0x7F800000);
    for (; k < 4; ++k) {
        mnx[k] = mny[k] = mnz[k] = inf;
        mxx[k] = mxy[k] = mxz[k] = -inf;
        ref[k] = kNoChild;
    }
    float4* o = wide4 + 8 * static_cast<size_t>(i);
    o[0] = make_float4(mnx[0], mnx[1], mnx[2], mnx[3]);
    o[1] = make_float4(mny[0], mny[1], mny[2], mny[3]);
    o[2] = make_float4(mnz[0], mnz[1], mnz[2], mnz[3]);
    o[3] = make_float4(mxx[0], mxx[1], mxx[2], mxx[3]);
    o[4] = make_float4(mxy[0], mxy[1], mxy[2], mxy[3]);
    o[5] = make_float4(mxz[0], mxz[1], mxz[2], mxz[3]);
    reinterpret_cast<uint4*>(o)[6] = make_uint4(ref[0], ref[1], ref[2], ref[3]);
    o[7] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ================================= K4c: compressed 4-wide traversal nodes
// The same four children as wide4_kernel, in 64 bytes: the node's origin
// (the minimum corner over its children), one power-of-two step per axis
// (the least with 255 steps covering the node's extent, biased exponent in a
// byte) and each child box as 8-bit step counts, the minimum rounded down
// and the maximum up.  The traversal decodes origin + q * step; rounding to
// nearest is monotone, so the decoded box encloses the exact one.  Record:
// (origin xyz, exponents | child count << 24), (qlo x, y, z, qhi x), (qhi y,
// z, 0, 0), four child references; byte c of each q word belongs to child c.
__device__ __forceinline__ uint32_t quant_step_exp(double extent) {
    int e = -126;
    if (extent > 0.0) {
        int k = 0;
        frexp(extent / 255.0, &k);  // extent / 255 < 2^k
        e = k < -126 ? -126 : k;
    }
    return static_cast<uint32_t>(e + 127);
}

__global__ void __launch_bounds__(256) cwide_kernel(const float4* __restrict__ wide, const uint8_t* __restrict__ depth_odd,
                                                    uint32_t n_internal, uint4* __restrict__ cwide, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_internal || depth_odd[i]) return;
    float mn[4][3], mx[4][3];
    uint32_t ref[4];
    int k = 0;
    const float4* w = wide + 4 * static_cast<size_t>(i);
    const float4 w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3];
    const float4 cmn[2] = {w0, w2}, cmx[2] = {w1, w3};
    const uint32_t cref[2] = {__float_as_uint(w0.w), __float_as_uint(w1.w)};
    auto put = [&](float4 a, float4 b, uint32_t r) {
        mn[k][0] = a.x; mn[k][1] = a.y; mn[k][2] = a.z;
        mx[k][0] = b.x; mx[k][1] = b.y; mx[k][2] = b.z;
        ref[k++] = r;
    };
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        if (cref[c] & kLeafRef) {
            put(cmn[c], cmx[c], cref[c]);
        } else {
            const float4* g = wide + 4 * static_cast<size_t>(cref[c]);
            const float4 g0 = g[0], g1 = g[1], g2 = g[2], g3 = g[3];
            put(g0, g1, __float_as_uint(g0.w));
            put(g2, g3, __float_as_uint(g1.w));
        }
    }
    const int n = k;
    float o[3];
    uint32_t ex[3];
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float lo = mn[0][a], hi = mx[0][a];
        for (int c = 1; c < n; ++c) {
            lo = min_std(lo, mn[c][a]);
            hi = max_std(hi, mx[c][a]);
        }
        ok = ok && isfinite(lo) && isfinite(hi) && lo <= hi;
        o[a] = lo;
        ex[a] = quant_step_exp(static_cast<double>(hi) - static_cast<double>(lo));
        ok = ok && ex[a] <= 254u;
    }
    uint32_t q[6] = {0u, 0u, 0u, 0u, 0u, 0u};  // lo x, y, z, hi x, y, z; byte c = child c
    if (ok) {
        for (int c = 0; c < n; ++c)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const double step = ldexp(1.0, static_cast<int>(ex[a]) - 127);
                const float fstep = __uint_as_float(ex[a] << 23);
                double dl = floor((static_cast<double>(mn[c][a]) - o[a]) / step);
                double dh = ceil((static_cast<double>(mx[c][a]) - o[a]) / step);
                int ql = dl < 0.0 ? 0 : (dl > 255.0 ? 255 : static_cast<int>(dl));
                int qh = dh < 0.0 ? 0 : (dh > 255.0 ? 255 : static_cast<int>(dh));
                // settle the counts against the decoder's own float arithmetic
                while (ql > 0 && o[a] + static_cast<float>(ql) * fstep > mn[c][a]) --ql;
                while (qh < 255 && o[a] + static_cast<float>(qh) * fstep < mx[c][a]) ++qh;
                ok = ok && !(o[a] + static_cast<float>(ql) * fstep > mn[c][a]) &&
                     !(o[a] + static_cast<float>(qh) * fstep < mx[c][a]);
                q[a] |= static_cast<uint32_t>(ql) << (8 * c);
                q[3 + a] |= static_cast<uint32_t>(qh) << (8 * c);
            }
    }
    if (!ok) raise_corrupt(err, 16, i, 0u);
    for (int c = n; c < 4; ++c) ref[c] = kNoChild;
    uint4* out = cwide + 4 * static_cast<size_t>(i);
    out[0] = make_uint4(__float_as_uint(o[0]), __float_as_uint(o[1]), __float_as_uint(o[2]),
                        ex[0] | (ex[1] << 8) | (ex[2] << 16) | (static_cast<uint32_t>(n) << 24));
    out[1] = make_uint4(q[0], q[1], q[2], q[3]);
    out[2] = make_uint4(q[4], q[5], 0u, 0u);
    out[3] = make_uint4(ref[0], ref[1], ref[2], ref[3]);
}

void launch_cwide(const float4* wide, const uint8_t* depth_odd, uint32_t n_internal, uint4* cwide, uint32_t* err,
                  cudaStream_t s) {
    if (n_internal == 0) return;
    cwide_kernel<<<(n_internal + 255) / 256, 256, 0, s>>>(wide, depth_odd, n_internal, cwide, err);
}

void launch_wide4(const float4* wide, const uint8_t* depth_odd, uint32_t n_internal, float4* wide4, cudaStream_t s) {
    if (n_internal == 0) return;
    wide4_kernel<<<(n_internal + 255) / 256, 256, 0, s>>>(wide, depth_odd, n_internal, wide4);
}

// ============================================================ launchers
void launch_scene_box(const crt_triangle* tris, uint32_t n_buffer, const float* models, SceneState* st, uint32_t* err,
                      cudaStream_t s) {
    const uint32_t want = (n_buffer + 255) / 256;
    const uint32_t grid = want < static_cast<uint32_t>(kNumSms * 8) ? (want ? want : 1u) : kNumSms * 8;
    scene_box_kernel<<<grid, 256, 0, s>>>(tris, n_buffer, models, st, err);
}

void launch_morton(const crt_triangle* tris, uint32_t n, const float* models_third, const SceneState* st,
                   uint32_t* codes, uint32_t* hist, int bits, cudaStream_t s) {
    const uint32_t want = (n + 255) / 256;
    const uint32_t grid = want < static_cast<uint32_t>(kNumSms * 8) ? (want ? want : 1u) : kNumSms * 8;
    if (bits == 4) morton_kernel<4><<<grid, 256, 0, s>>>(tris, n, models_third, st, codes, hist);
    else morton_kernel<8><<<grid, 256, 0, s>>>(tris, n, models_third, st, codes, hist);
}

uint32_t sort_tile_keys(int bits) { return bits == 4 ? 256u * 16u : 256u * 16u; }

void launch_onesweep(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, uint32_t n,
                     int shift, int bits, const uint32_t* pass_hist, uint32_t* lookback, uint32_t* ticket, uint32_t* err,
                     uint32_t spin_limit, cudaStream_t s) {
    const uint32_t tiles = (n + sort_tile_keys(bits) - 1) / sort_tile_keys(bits);
    if (bits == 4)
        onesweep_kernel<4, 256, 16, false><<<tiles, 256, 0, s>>>(keys_in, vals_in, keys_out, vals_out, n, shift,
                                                                  pass_hist, lookback, ticket, err, spin_limit, nullptr, 0);
    else
        onesweep_kernel<8, 256, 16, false><<<tiles, 256, 0, s>>>(keys_in, vals_in, keys_out, vals_out, n, shift,
                                                                  pass_hist, lookback, ticket, err, spin_limit, nullptr, 0);
}

void launch_onesweep_segments(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                              uint32_t n, const uint32_t* seg_off, uint32_t n_seg, const uint32_t* seg_hist,
                              uint32_t* lookback, uint32_t* ticket, uint32_t* err, uint32_t spin_limit, cudaStream_t s) {
    const uint32_t tiles = (n + sort_tile_keys(8) - 1) / sort_tile_keys(8);
    onesweep_kernel<8, 256, 16, true><<<tiles, 256, 0, s>>>(keys_in, vals_in, keys_out, vals_out, n, 0, seg_hist,
                                                             lookback, ticket, err, spin_limit, seg_off, n_seg);
}

// The sort's counting and digit-offset steps alone, on caller keys and
// counts (the reference's sort-shader known-answer tests drive them).
template <int BITS>
__global__ void __launch_bounds__(256) digit_counts_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                           uint32_t* __restrict__ counts) {
    constexpr int RADIX = 1 << BITS;
    constexpr int PASSES = (32 + BITS - 1) / BITS;
    __shared__ uint32_t s_hist[PASSES * RADIX];
    for (int i = threadIdx.x; i < PASSES * RADIX; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        add_digit_counts<BITS, PASSES>(keys[i], s_hist);
    __syncthreads();
    for (int i = threadIdx.x; i < PASSES * RADIX; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&counts[i], s_hist[i]);
}

// One block per digit place: where each digit's keys start in the pass's
// output, the exclusive scan over digits that the radix pass takes of its
// global histogram (the same packed block scan, the global counts in the
// high half).
template <int BITS, int BLOCK>
__global__ void __launch_bounds__(BLOCK) digit_offsets_kernel(const uint32_t* __restrict__ counts,
                                                              uint32_t* __restrict__ offsets) {
    constexpr int RADIX = 1 << BITS;
    static_assert(BLOCK >= RADIX, "one thread per digit");
    __shared__ unsigned long long s_wsum[BLOCK / 32];
    const int d = threadIdx.x;
    const size_t base = static_cast<size_t>(blockIdx.x) * RADIX;
    const uint32_t gh = d < RADIX ? counts[base + d] : 0u;
    const unsigned long long incl = block_inclusive_scan_u64<BLOCK>(static_cast<unsigned long long>(gh) << 32, s_wsum);
    if (d < RADIX) offsets[base + d] = static_cast<uint32_t>(incl >> 32) - gh;
}

bool launch_digit_counts(const uint32_t* keys, uint32_t n, int bits, uint32_t* counts, cudaStream_t s) {
    const uint32_t want = (n + 255) / 256;
    const uint32_t grid = want < static_cast<uint32_t>(kNumSms * 8) ? (want ? want : 1u) : kNumSms * 8;
    switch (bits) {
        case 1: digit_counts_kernel<1><<<grid, 256, 0, s>>>(keys, n, counts); return true;
        case 2: digit_counts_kernel<2><<<grid, 256, 0, s>>>(keys, n, counts); return true;
        case 4: digit_counts_kernel<4><<<grid, 256, 0, s>>>(keys, n, counts); return true;
        case 8: digit_counts_kernel<8><<<grid, 256, 0, s>>>(keys, n, counts); return true;
        default: return false;
    }
}

bool launch_digit_offsets(const uint32_t* counts, uint32_t places, int bits, uint32_t* offsets, cudaStream_t s) {
    if (places == 0) return true;
    switch (bits) {
        case 1: digit_offsets_kernel<1, 32><<<places, 32, 0, s>>>(counts, offsets); return true;
        case 2: digit_offsets_kernel<2, 32><<<places, 32, 0, s>>>(counts, offsets); return true;
        case 4: digit_offsets_kernel<4, 32><<<places, 32, 0, s>>>(counts, offsets); return true;
        case 8: digit_offsets_kernel<8, 256><<<places, 256, 0, s>>>(counts, offsets); return true;
        default: return false;
    }
}

void launch_leaf_init(const crt_triangle* tris, uint32_t n, const float* models, const uint32_t* perm, float4* node_box,
                      float4* clusters, float4* xtri_sorted, uint2* it, uint32_t* err, cudaStream_t s) {
    leaf_init_kernel<<<(n + 255) / 256, 256, 0, s>>>(tris, n, models, perm, node_box, clusters, xtri_sorted, it, err);
}

void launch_ploc_iteration(const float4* cin, float4* cout, float4* node_box, uint4* node_kids, uint2* it,
                           int iter, uint32_t N, int radius, uint32_t n_upper,
                           unsigned long long* lookback, uint32_t* tickets, uint32_t n_tiles_cap, uint32_t* err,
                           uint32_t spin_limit, cudaStream_t s) {
    const uint32_t tiles = (n_upper + ploc_own(radius) - 1) / ploc_own(radius);
    ploc_iteration_kernel<kPlocSpan, 256, kPlocMaxRadius><<<tiles ? tiles : 1u, 256, 0, s>>>(
        cin, cout, node_box, node_kids, it, iter, N, radius, lookback, tickets, n_tiles_cap, err, spin_limit);
}

void launch_layout_level(const uint4* node_kids, uint2* pf, uint32_t id_begin,
                         uint32_t id_end, uint32_t N, uint32_t* dfs, uint32_t* err, cudaStream_t s) {
    if (id_end <= id_begin || id_end > 2 * N - 1) return;
    const uint32_t cnt = id_end - id_begin;
    layout_level_kernel<<<(cnt + 255) / 256, 256, 0, s>>>(node_kids, pf, id_begin, id_end, N, dfs, err);
}

void launch_layout_emit(const float4* node_box, const uint4* node_kids, const uint2* pf, uint32_t N,
                        const uint32_t* dfs, crt_bvh_node* out, float4* wide, float4* wide_wt, uint8_t* depth_odd,
                        LeafOut lv, const SceneState* st, uint32_t* err, cudaStream_t s) {
    const uint32_t cnt = 2 * N - 1;
    layout_emit_kernel<<<(cnt + 255) / 256, 256, 0, s>>>(node_box, node_kids, pf, N, dfs, out, wide, wide_wt, depth_odd,
                                                         lv, st, err);
}

int ploc_persistent_grid() {
    static int grid = -1;
    if (grid < 0) {
        int per_sm = 0, dev = 0, sms = kNumSms, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &per_sm, ploc_persistent_kernel<kPlocSpan, 256, kPlocMaxRadius>, 256, 0) == cudaSuccess &&
            per_sm > 0)
            grid = (per_sm < kPlocBlocksPerSm ? per_sm : kPlocBlocksPerSm) * sms;
        else
            grid = 0;
        cudaGetLastError();
    }
    return grid;
}

cudaError_t launch_ploc_persistent(float4* ca, float4* cb, float4* node_box, uint4* node_kids, uint2* it, uint32_t N,
                                   int radius, unsigned long long* lookback, uint32_t* tickets, uint32_t n_tiles_cap,
                                   uint2* pf, crt_bvh_node* out, float4* wide, float4* wide_wt, uint8_t* depth_odd,
                                   LeafOut lv, const SceneState* st, unsigned long long* bar, uint32_t* iters_out,
                                   uint32_t* err, uint32_t spin_limit, cudaStream_t s) {
    const int grid = ploc_persistent_grid();
    if (grid <= 0) return cudaErrorNotSupported;
    void* args[] = {&ca, &cb, &node_box, &node_kids, &it, &N, &radius, &lookback, &tickets, &n_tiles_cap, &pf, &out,
                    &wide, &wide_wt, &depth_odd, &lv, &st, &bar, &iters_out, &err, &spin_limit};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(ploc_persistent_kernel<kPlocSpan, 256, kPlocMaxRadius>),
                                       dim3(grid), dim3(256), args, 0, s);
}

// A wait on a flag, bounded like every look-back and grid-barrier wait: on
// exhaustion the error word records the timeout and the kernel returns.
__global__ void wait_probe_kernel(const unsigned int* flag, uint32_t spin_limit, uint32_t* err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    SpinBound spin(spin_limit);
    while (ld_acquire_u32(flag) == 0u)
        if (!spin.step()) { raise_error(err, kDevTimeout); return; }
}

void launch_wait_probe(const unsigned int* flag, uint32_t spin_limit, uint32_t* err, cudaStream_t s) {
    wait_probe_kernel<<<1, 32, 0, s>>>(flag, spin_limit, err);
}

void launch_single_leaf(const float4* node_box, crt_bvh_node* out, LeafOut lv, cudaStream_t s) {
    single_leaf_kernel<<<1, 1, 0, s>>>(node_box, out, lv);
}

}  // namespace crt

#include "crt_batch_kernels.cuh"
