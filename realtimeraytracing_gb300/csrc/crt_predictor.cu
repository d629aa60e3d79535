// Learned hit predictor: an FP16 MLP on tcgen05 tensor cores that guesses,
// per ray, which treelet (subtree of a fixed BVH cut) holds its closest hit.
// The traversal tests that treelet exactly first and uses the hit to seed
// t_max (crt_trace.cu), so a wrong guess costs time, never correctness.
//
// Network (per ray):
//   features  origin cell on a 64^3 grid over the scene box -> 16 learned fp16
//             values; direction in 32x32 octahedral bins -> 16 learned values
//   MLP       32 -> 64 (ReLU) -> 64 (ReLU) -> 128 logits (127 treelets + miss)
// Every layer is one CTA-wide tcgen05.mma chain over a 128-ray tile: fp16
// operands in shared memory (K-major, no swizzle), FP32 accumulators in TMEM,
// read back with tcgen05.ld for the bias/ReLU/softmax epilogues.  Training
// runs the forward pass, the softmax cross-entropy gradient and the backward
// GEMMs (weight and input gradients) on the tensor cores as well, sums the
// gradients into FP32 buffers, and an Adam kernel updates FP32 master
// weights and refreshes the fp16 copies (and the transposed copies the
// backward GEMMs read).
#include <cmath>
#include <algorithm>
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"
#include "crt_predictor.cuh"
#include "crt_tc.cuh"

namespace crt {
namespace pred {

using tc::kmajor_offset;

// ------------------------------------------------------------ features
struct SceneFrame {
    float mnx, mny, mnz, sx, sy, sz;  // cell = (o - mn) * s
};

__device__ __forceinline__ SceneFrame scene_frame(const crt_bvh_node* nodes) {
    const float4 mn = __ldg(reinterpret_cast<const float4*>(nodes));
    const float4 mx = __ldg(reinterpret_cast<const float4*>(nodes) + 1);
    SceneFrame f;
    f.mnx = mn.x; f.mny = mn.y; f.mnz = mn.z;
    const float ex = fmaxf(mx.x - mn.x, 1e-20f), ey = fmaxf(mx.y - mn.y, 1e-20f), ez = fmaxf(mx.z - mn.z, 1e-20f);
    f.sx = kGrid / ex; f.sy = kGrid / ey; f.sz = kGrid / ez;
    return f;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ void ray_keys(const float4 r0, const float4 r1, const SceneFrame& f, uint32_t& cell,
                                         uint32_t& bin) {
    const int cx = clampi(static_cast<int>(floorf((r0.x - f.mnx) * f.sx)), 0, kGrid - 1);
    const int cy = clampi(static_cast<int>(floorf((r0.y - f.mny) * f.sy)), 0, kGrid - 1);
    const int cz = clampi(static_cast<int>(floorf((r0.z - f.mnz) * f.sz)), 0, kGrid - 1);
    cell = (static_cast<uint32_t>(cx) * kGrid + cy) * kGrid + cz;
    // octahedral map of the direction to [-1, 1]^2
    const float s = fabsf(r1.x) + fabsf(r1.y) + fabsf(r1.z);
    float px = s > 0.f ? r1.x / s : 0.f, py = s > 0.f ? r1.y / s : 0.f;
    if (r1.z < 0.f) {
        const float qx = (1.f - fabsf(py)) * (px >= 0.f ? 1.f : -1.f);
        const float qy = (1.f - fabsf(px)) * (py >= 0.f ? 1.f : -1.f);
        px = qx; py = qy;
    }
    const int bu = clampi(static_cast<int>((px + 1.f) * (0.5f * kDirBins)), 0, kDirBins - 1);
    const int bv = clampi(static_cast<int>((py + 1.f) * (0.5f * kDirBins)), 0, kDirBins - 1);
    bin = static_cast<uint32_t>(bu) * kDirBins + bv;
}

// The scene of global ray i in a batch (the last scene whose first ray is <= i).
__device__ __forceinline__ uint32_t scene_of_ray(const BatchScene* sc, uint32_t n_scenes, uint32_t i) {
    uint32_t lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&sc[mid].ray_off) <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Features of ray i: its origin cell and direction bin; in a batch, on its
// scene's box, with the cell index moved by a per-scene hash so that the
// scenes share the cell embeddings without sharing cells.  *scene: the
// ray's scene (0 for one BVH).
// *cell_raw: the cell before that move (the one the trace order key uses).
__device__ __forceinline__ void ray_features(const PredictorDev& P, const crt_bvh_node* nodes, const SceneFrame& fr,
                                             uint32_t i, float4 r0, float4 r1, uint32_t& cell, uint32_t& bin,
                                             uint32_t& scene, uint32_t& cell_raw) {
    if (P.n_scenes == 0) {
        scene = 0;
        ray_keys(r0, r1, fr, cell, bin);
        cell_raw = cell;
        return;
    }
    scene = scene_of_ray(P.scenes, P.n_scenes, i);
    ray_keys(r0, r1, scene_frame(nodes + __ldg(&P.scenes[scene].node_off)), cell, bin);
    cell_raw = cell;
    cell = (cell + scene * 0x9E3779B1u) & static_cast<uint32_t>(kEo - 1);
}

// Trace order of a ray: predicted class (7 bits) | Morton code of its origin
// cell on a 32^3 grid of the scene box (15 bits) | direction bin (10 bits).
// Rays of one class go together, and within a class nearby origins and
// similar directions.  In a batch: (scene, class, origin cell on a 16^3 grid
// of the scene's box, the direction bin's first coordinate), 8 + 7 + 12 + 5
// bits.  cell: the unmoved origin cell (ray_keys).
__device__ __forceinline__ uint32_t spread5(uint32_t v) {
    v &= 31u;
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6) | ((v & 16u) << 8);
}

__device__ __forceinline__ uint32_t order_key(uint32_t n_scenes, uint32_t cell, uint32_t bin, uint32_t scene,
                                              uint32_t cls) {
    const uint32_t cx = cell / (kGrid * kGrid), cy = (cell / kGrid) % kGrid, cz = cell % kGrid;
    cls &= 0x7Fu;
    if (n_scenes == 0) {
        const uint32_t m = (spread5(cx >> 1) << 2) | (spread5(cy >> 1) << 1) | spread5(cz >> 1);
        return (cls << 25) | (m << 10) | (bin & 1023u);
    }
    const uint32_t m = (spread5(cx >> 2) << 2) | (spread5(cy >> 2) << 1) | spread5(cz >> 2);
    return ((scene & 0xFFu) << 24) | (cls << 17) | ((m & 0xFFFu) << 5) | ((bin >> 5) & 31u);
}

// Class of the closest hit `tri` (scene-local id in a batch) of a ray of `scene`.
__device__ __forceinline__ int hit_class(const PredictorDev& P, uint32_t scene, uint32_t tri) {
    if (tri == CRT_MISS) return kMissClass;
    if (P.n_scenes == 0) return tri < P.n_tris ? P.tri_class[tri] : kMissClass;
    const uint32_t off = __ldg(&P.scenes[scene].tri_off), n = __ldg(&P.scenes[scene].n_tris);
    return tri < n ? P.tri_class[off + tri] : kMissClass;
}

// ---------------------------------------------------- smem tile helpers
// Copy a row-major fp16 matrix (rows x cols) into the K-major core layout.
__device__ __forceinline__ void load_kmajor(unsigned char* dst, const __half* src, int rows, int cols) {
    for (int i = threadIdx.x; i < rows * cols / 8; i += blockDim.x) {
        const int r = (i * 8) / cols, k = (i * 8) % cols;
        *reinterpret_cast<uint4*>(dst + kmajor_offset(r, k, cols)) = __ldg(reinterpret_cast<const uint4*>(src) + i);
    }
}

__device__ __forceinline__ void zero_bytes(unsigned char* dst, int bytes) {
    for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) reinterpret_cast<uint4*>(dst)[i] = make_uint4(0, 0, 0, 0);
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Row `row` of a K-major tile with Kd columns, 8 values starting at column k (k % 8 == 0).
__device__ __forceinline__ void store_row8(unsigned char* tile, int Kd, int row, int k, const float* v) {
    uint4 q;
    q.x = pack2(v[0], v[1]); q.y = pack2(v[2], v[3]); q.z = pack2(v[4], v[5]); q.w = pack2(v[6], v[7]);
    *reinterpret_cast<uint4*>(tile + kmajor_offset(row, k, Kd)) = q;
}

__device__ __forceinline__ void store_h(unsigned char* tile, int Kd, int row, int k, float v) {
    *reinterpret_cast<__half*>(tile + kmajor_offset(row, k, Kd)) = __float2half_rn(v);
}

__device__ __forceinline__ float load_h(const unsigned char* tile, int Kd, int row, int k) {
    return __half2float(*reinterpret_cast<const __half*>(tile + kmajor_offset(row, k, Kd)));
}

// Issue D = A * B^T over Kd columns (Kd / 16 MMAs) from one thread.
__device__ __forceinline__ void gemm(uint32_t d_tmem, const unsigned char* A, const unsigned char* B, int Kd, int M,
                                     int N) {
    const uint32_t sbo = static_cast<uint32_t>(Kd / 8) * 128u;
    const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(B);
    const uint32_t id = tc::idesc_f16_f32(M, N);
    for (int kk = 0; kk < Kd / 16; ++kk)
        tc::mma_f16(d_tmem, tc::smem_desc(a0 + kk * 256, tc::kLbo, sbo), tc::smem_desc(b0 + kk * 256, tc::kLbo, sbo),
                    id, kk > 0);
}

constexpr uint32_t kMmaWaitLimit = 1u << 26;  // try_wait rounds before a tile gives up

struct Sync {
    uint64_t* mbar;
    uint32_t phase = 0;
    uint32_t* err;
    uint32_t limit = kMmaWaitLimit;
    // Publish generic smem writes to the tensor core and order tcgen05 work.
    __device__ __forceinline__ void before_mma() {
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
    // Commit the MMAs thread 0 issued and wait for them (issue = false waits
    // on a phase nothing will complete: the self-test's way to make the wait
    // run out).  Block-uniform result: false when any thread's bounded wait
    // gave up.  Then the error word is set and every thread waits once more,
    // again bounded, so that MMAs still in flight finish writing TMEM before
    // the caller frees it; the caller must leave its tile loop without
    // reading TMEM or issuing more MMAs.
    __device__ __forceinline__ bool commit_and_wait(bool issue = true) {
        if (issue && threadIdx.x == 0) tc::mma_commit(mbar);
        const bool ok = tc::mbar_wait(mbar, phase, limit);
        if (__syncthreads_and(ok)) {
            phase ^= 1u;
            tc::fence_after_sync();
            return true;
        }
        if (threadIdx.x == 0) raise_error(err, kDevTimeout);
        tc::mbar_wait(mbar, phase, limit);
        tc::fence_after_sync();
        __syncthreads();
        return false;
    }
};

__device__ __forceinline__ uint32_t lane_addr(uint32_t tbase, uint32_t col) {
    const uint32_t warp = threadIdx.x >> 5;
    return tbase + ((32u * warp) << 16) + col;
}

// ---------------------------------------------------------- inference
// Persistent: each CTA (128 threads, one ray per thread) loads the weights
// once and walks 128-ray tiles.  TMEM (128 columns): D1 cols 0-63, D2 64-127,
// then the logits over both once H2 is out of D2.  Shared memory: weights, X,
// and one activation buffer that holds H1 and then H2 (H1 is dead once the
// second GEMM has completed).
// The last 2 KB: the CTA's trace order key histograms (4 digits x 256
// values, 16-bit counters in pairs), when the kernel writes order keys.
constexpr int kInferSmemUsed = 64 * 32 * 2 + 64 * 64 * 2 + 128 * 64 * 2 + 128 * 32 * 2 + 128 * 64 * 2 +
                               (64 + 64 + 128) * 4 + 64 + 2048;
// Requested size caps residency at four CTAs per SM, the number whose
// 128-column TMEM allocations fit the SM's 512 columns together.
constexpr int kInferSmem = 56 * 1024;
// tiles of 128 rays between flushes of the 16-bit key histograms (< 65536 rays)
constexpr uint32_t kHistFlushTiles = 256;
constexpr int kInferCtasPerSm = 4;
static_assert(kInferSmemUsed <= kInferSmem && kInferCtasPerSm * kInferSmem <= 228 * 1024 &&
              (kInferCtasPerSm + 1) * kInferSmem > 228 * 1024, "inference tile layout and residency");

// ARGMAX: the class is the likeliest of all 128 (miss included), which is all
// that ordering rays by class needs; otherwise the likeliest treelet unless
// the miss class holds at least miss_threshold of the probability mass (the
// seeding rule), which needs the softmax sum.  KEYS (with ARGMAX): the kernel
// also writes each ray's trace order key (order_key) to keys[i] and adds the
// keys' four 8-bit digit histograms into hist (4 x 256), so that the ordering
// needs no second pass over the rays.  rays_copy (optional): ray i is also
// stored to rays_copy[i] (rays in page-locked host memory are read across the
// CPU-GPU link once, by this kernel, and the trace reads the device copy).
template <bool ARGMAX, bool KEYS>
__global__ void __launch_bounds__(128) infer_kernel(PredictorDev P, const crt_bvh_node* nodes, const crt_ray* rays,
                                                    uint32_t n, uint16_t* classes, float miss_threshold,
                                                    uint32_t* keys, uint32_t* hist, crt_ray* rays_copy,
                                                    uint32_t* err) {
    static_assert(ARGMAX || !KEYS, "order keys come with the argmax class");
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sW1 = smem;
    unsigned char* sW2 = sW1 + 64 * 32 * 2;
    unsigned char* sW3 = sW2 + 64 * 64 * 2;
    unsigned char* sX = sW3 + 128 * 64 * 2;
    unsigned char* sH1 = sX + 128 * 32 * 2;
    unsigned char* sH2 = sH1;  // H1 is dead once the second GEMM has completed
    float* sB = reinterpret_cast<float*>(sH1 + 128 * 64 * 2);
    uint32_t* sT = reinterpret_cast<uint32_t*>(sB + 256);
    uint64_t* sM = reinterpret_cast<uint64_t*>(sT + 2);
    uint32_t* sHist = sT + 16;  // 512 words: counter k in half (k & 1) of word k >> 1

    load_kmajor(sW1, P.w16 + hW1, 64, 32);
    load_kmajor(sW2, P.w16 + hW2, 64, 64);
    load_kmajor(sW3, P.w16 + hW3, 128, 64);
    for (int i = threadIdx.x; i < 256; i += 128) {
        const float b = i < 64 ? P.master[oB1 + i] : (i < 128 ? P.master[oB2 + i - 64] : P.master[oB3 + i - 128]);
        sB[i] = b;
    }
    if (KEYS)
        for (int w = threadIdx.x; w < 512; w += 128) sHist[w] = 0u;
    // adds the CTA's counts into hist and clears them (every thread calls it)
    auto flush_hist = [&]() {
        __syncthreads();
        for (int w = threadIdx.x; w < 512; w += 128) {
            const uint32_t v = sHist[w];
            if (v & 0xFFFFu) atomicAdd(hist + 2 * w, v & 0xFFFFu);
            if (v >> 16) atomicAdd(hist + 2 * w + 1, v >> 16);
            sHist[w] = 0u;
        }
        __syncthreads();
    };
    uint32_t tiles_done = 0;
    if (threadIdx.x < 32) { tc::tmem_alloc(sT, 128); tc::tmem_relinquish(); }
    if (threadIdx.x == 0) tc::mbar_init(sM, 1);
    Sync sy{sM, 0, err};
    sy.before_mma();
    const uint32_t tb = *sT;
    const SceneFrame fr = scene_frame(nodes);
    const int tid = threadIdx.x;

    for (uint32_t tile = blockIdx.x; static_cast<uint64_t>(tile) * 128 < n; tile += gridDim.x) {
        const uint32_t i = tile * 128 + tid;
        const bool valid = i < n;
        uint4 e[4] = {};
        uint32_t key_cell = 0, key_bin = 0, key_scene = 0;
        if (valid) {
            const float4 r0 = __ldg(reinterpret_cast<const float4*>(rays + i));
            const float4 r1 = __ldg(reinterpret_cast<const float4*>(rays + i) + 1);
            if (rays_copy) {
                float4* c = reinterpret_cast<float4*>(rays_copy + i);
                c[0] = r0;
                c[1] = r1;
            }
            uint32_t cell, bin, scene;
            ray_features(P, nodes, fr, i, r0, r1, cell, bin, scene, key_cell);
            key_bin = bin;
            key_scene = scene;
            const uint4* eo = reinterpret_cast<const uint4*>(P.w16 + hEo + static_cast<size_t>(cell) * kEmb);
            const uint4* ed = reinterpret_cast<const uint4*>(P.w16 + hEd + static_cast<size_t>(bin) * kEmb);
            e[0] = __ldg(eo); e[1] = __ldg(eo + 1); e[2] = __ldg(ed); e[3] = __ldg(ed + 1);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) *reinterpret_cast<uint4*>(sX + kmajor_offset(tid, 8 * c, 32)) = e[c];
        sy.before_mma();
        if (tid == 0) gemm(tb + 0, sX, sW1, 32, 128, 64);
        if (!sy.commit_and_wait()) break;
        for (int c = 0; c < 64; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + sB[c + j], 0.f);
            store_row8(sH1, 64, tid, c, v);
            store_row8(sH1, 64, tid, c + 8, v + 8);
        }
        sy.before_mma();
        if (tid == 0) gemm(tb + 64, sH1, sW2, 64, 128, 64);
        if (!sy.commit_and_wait()) break;
        for (int c = 0; c < 64; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 64 + c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + sB[64 + c + j], 0.f);
            store_row8(sH2, 64, tid, c, v);
            store_row8(sH2, 64, tid, c + 8, v + 8);
        }
        sy.before_mma();
        if (tid == 0) gemm(tb + 0, sH2, sW3, 64, 128, 128);  // logits over D1 and D2, both read out
        if (!sy.commit_and_wait()) break;
        // Seed the most likely treelet unless the miss class holds at least
        // `miss_threshold` of the probability mass.
        float best = -INFINITY, lmax = -INFINITY, lmiss = 0.f;
        int bc = 0;
        static_assert(kMissClass == 127, "the miss class is the last logit");
        for (int c = 0; c < 112; c += 16) {  // the first 112 logits: treelets only
            float v[16];
            tc::tmem_ld16(lane_addr(tb, c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float l = v[j] + sB[128 + c + j];
                if (!ARGMAX) lmax = fmaxf(lmax, l);
                if (l > best) { best = l; bc = c + j; }
            }
        }
        {  // the last 16, the miss class among them
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 112), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float l = v[j] + sB[128 + 112 + j];
                if (!ARGMAX) lmax = fmaxf(lmax, l);
                if (112 + j == kMissClass) lmiss = l;
                else if (l > best) { best = l; bc = 112 + j; }
            }
        }
        if (ARGMAX) {
            const uint32_t cls = lmiss >= best ? kMissClass : static_cast<uint32_t>(bc);
            if (valid) classes[i] = static_cast<uint16_t>(cls);
            if (KEYS && valid) {
                const uint32_t key = order_key(P.n_scenes, key_cell, key_bin, key_scene, cls);
                keys[i] = key;
#pragma unroll
                for (int d = 0; d < 4; ++d) {
                    const uint32_t k = static_cast<uint32_t>(d) * 256u + ((key >> (8 * d)) & 255u);
                    atomicAdd(sHist + (k >> 1), 1u << (16u * (k & 1u)));
                }
            }
        } else {
            float sum = 0.f;
            for (int c = 0; c < 128; c += 16) {
                float v[16];
                tc::tmem_ld16(lane_addr(tb, c), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) sum += __expf(v[j] + sB[128 + c + j] - lmax);
            }
            const float p_miss = __expf(lmiss - lmax) / sum;
            if (valid) classes[i] = static_cast<uint16_t>(p_miss >= miss_threshold ? kMissClass : bc);
        }
        tc::fence_before_sync();
        __syncthreads();
        if (KEYS && ++tiles_done == kHistFlushTiles) {  // block-uniform
            flush_hist();
            tiles_done = 0;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tb, 128);
    // counts of tiles that gave up (an error is raised) are flushed too; the
    // caller reports the error and ignores the order
    if (KEYS) flush_hist();
}

// ------------------------------------------------------------ training
// One 128-sample tile per CTA: forward, softmax cross-entropy gradient
// (p - onehot, unscaled; the optimiser divides by the sample count), backward
// GEMMs, FP32 atomics into the gradient buffers.  Shared memory:
//   weights  W1 W1T W2 W2T W3 W3T                       56 KB
//   acts     X XT H1 H1T H2 H2T                         80 KB
//   grads    G3 G3T, then G2 G2T(padded to 128 rows),
//            then G1 G1T(padded)                       64 KB
// TMEM (256 cols): D1 0-63, D2 64-127, logits 128-255; then dW3 0-63,
// dH2 64-127; dW2 128-191, dH1 192-255; dW1 0-31, dX 32-63.
constexpr int kTrainSmem = 56 * 1024 + 80 * 1024 + 64 * 1024 + 256 * 4 + 64;

__global__ void __launch_bounds__(128) train_kernel(PredictorDev P, const crt_bvh_node* nodes, const crt_ray* rays,
                                                    uint32_t n_rays, const crt_hit* hits, const uint16_t* targets,
                                                    uint32_t n_samples, uint32_t stride, uint32_t offset,
                                                    float* grad, float* loss_sum, uint32_t* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sW1 = smem;
    unsigned char* sW1T = sW1 + 4096;
    unsigned char* sW2 = sW1T + 4096;
    unsigned char* sW2T = sW2 + 8192;
    unsigned char* sW3 = sW2T + 8192;
    unsigned char* sW3T = sW3 + 16384;
    unsigned char* sX = sW3T + 16384;
    unsigned char* sXT = sX + 8192;
    unsigned char* sH1 = sXT + 8192;
    unsigned char* sH1T = sH1 + 16384;
    unsigned char* sH2 = sH1T + 16384;
    unsigned char* sH2T = sH2 + 16384;
    unsigned char* sGA = sH2T + 16384;
    float* sB = reinterpret_cast<float*>(sGA + 65536);
    uint32_t* sT = reinterpret_cast<uint32_t*>(sB + 256);
    uint64_t* sM = reinterpret_cast<uint64_t*>(sT + 2);
    unsigned char* sG3 = sGA;
    unsigned char* sG3T = sGA + 32768;
    unsigned char* sG = sGA;            // G2 / G1: 128 x 64
    unsigned char* sGT = sGA + 16384;   // G2T / G1T padded: 128 x 128

    load_kmajor(sW1, P.w16 + hW1, 64, 32);
    load_kmajor(sW1T, P.w16 + hW1T, 32, 64);
    load_kmajor(sW2, P.w16 + hW2, 64, 64);
    load_kmajor(sW2T, P.w16 + hW2T, 64, 64);
    load_kmajor(sW3, P.w16 + hW3, 128, 64);
    load_kmajor(sW3T, P.w16 + hW3T, 64, 128);
    for (int i = threadIdx.x; i < 256; i += 128)
        sB[i] = i < 64 ? P.master[oB1 + i] : (i < 128 ? P.master[oB2 + i - 64] : P.master[oB3 + i - 128]);
    if (threadIdx.x < 32) { tc::tmem_alloc(sT, 256); tc::tmem_relinquish(); }
    if (threadIdx.x == 0) tc::mbar_init(sM, 1);
    const int tid = threadIdx.x;
    const uint32_t s = blockIdx.x * 128 + tid;
    const uint64_t ri = static_cast<uint64_t>(s) * stride + offset;
    const bool valid = s < n_samples && ri < n_rays;
    uint32_t cell = 0, bin = 0;
    int target = -1;
    uint4 e[4] = {};
    if (valid) {
        const float4 r0 = __ldg(reinterpret_cast<const float4*>(rays + ri));
        const float4 r1 = __ldg(reinterpret_cast<const float4*>(rays + ri) + 1);
        uint32_t scene, cell_raw;
        ray_features(P, nodes, scene_frame(nodes), static_cast<uint32_t>(ri), r0, r1, cell, bin, scene, cell_raw);
        const uint4* eo = reinterpret_cast<const uint4*>(P.w16 + hEo + static_cast<size_t>(cell) * kEmb);
        const uint4* ed = reinterpret_cast<const uint4*>(P.w16 + hEd + static_cast<size_t>(bin) * kEmb);
        e[0] = __ldg(eo); e[1] = __ldg(eo + 1); e[2] = __ldg(ed); e[3] = __ldg(ed + 1);
        if (targets) {
            target = targets[ri];
        } else {
            target = hit_class(P, scene, __ldg(reinterpret_cast<const uint32_t*>(hits + ri)));
        }
        if (target < 0 || target >= kClasses) target = kMissClass;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        *reinterpret_cast<uint4*>(sX + kmajor_offset(tid, 8 * c, 32)) = e[c];
        const __half* hv = reinterpret_cast<const __half*>(&e[c]);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            *reinterpret_cast<__half*>(sXT + kmajor_offset(8 * c + j, tid, 128)) = hv[j];
    }
    Sync sy{sM, 0, err};
    sy.before_mma();
    const uint32_t tb = *sT;

    // One pass through the tile; a timed-out MMA wait leaves it (break) to
    // the TMEM release below.
    do {
        // ---- forward
        if (tid == 0) gemm(tb + 0, sX, sW1, 32, 128, 64);
        if (!sy.commit_and_wait()) break;
        for (int c = 0; c < 64; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                v[j] = __half2float(__float2half_rn(fmaxf(v[j] + sB[c + j], 0.f)));
                store_h(sH1T, 128, c + j, tid, v[j]);
            }
            store_row8(sH1, 64, tid, c, v);
            store_row8(sH1, 64, tid, c + 8, v + 8);
        }
        sy.before_mma();
        if (tid == 0) gemm(tb + 64, sH1, sW2, 64, 128, 64);
        if (!sy.commit_and_wait()) break;
        for (int c = 0; c < 64; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 64 + c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                v[j] = __half2float(__float2half_rn(fmaxf(v[j] + sB[64 + c + j], 0.f)));
                store_h(sH2T, 128, c + j, tid, v[j]);
            }
            store_row8(sH2, 64, tid, c, v);
            store_row8(sH2, 64, tid, c + 8, v + 8);
        }
        sy.before_mma();
        if (tid == 0) gemm(tb + 128, sH2, sW3, 64, 128, 128);
        if (!sy.commit_and_wait()) break;

        // ---- softmax cross-entropy: G3 = p - onehot(target)
        float mx = -INFINITY;
        for (int c = 0; c < 128; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 128 + c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) mx = fmaxf(mx, v[j] + sB[128 + c + j]);
        }
        float sum = 0.f;
        for (int c = 0; c < 128; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 128 + c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) sum += __expf(v[j] + sB[128 + c + j] - mx);
        }
        const float inv = 1.f / sum;
        for (int c = 0; c < 128; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 128 + c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float l = v[j] + sB[128 + c + j];
                const float p = __expf(l - mx) * inv;
                float g = p - ((c + j) == target ? 1.f : 0.f);
                if (!valid) g = 0.f;
                if (valid && (c + j) == target) atomicAdd(loss_sum, -(l - mx - __logf(sum)));
                v[j] = __half2float(__float2half_rn(g));
                store_h(sG3T, 128, c + j, tid, v[j]);
            }
            store_row8(sG3, 128, tid, c, v);
            store_row8(sG3, 128, tid, c + 8, v + 8);
        }
        // ---- dW3 = G3^T H2 and dH2 = G3 W3
        sy.before_mma();
        if (tid == 0) {
            gemm(tb + 0, sG3T, sH2T, 128, 128, 64);
            gemm(tb + 64, sG3, sW3T, 128, 128, 64);
        }
        if (!sy.commit_and_wait()) break;
        {
            float acc = 0.f;  // db3[tid] = sum over samples of G3[:, tid]
            for (int b = 0; b < 128; ++b) acc += load_h(sG3T, 128, tid, b);
            atomicAdd(grad + oB3 + tid, acc);
        }
        for (int c = 0; c < 64; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, c), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) atomicAdd(grad + oW3 + tid * 64 + c + j, v[j]);
        }
        float dh[64];
        for (int c = 0; c < 64; c += 16) tc::tmem_ld16(lane_addr(tb, 64 + c), dh + c);
        tc::fence_before_sync();
        __syncthreads();  // G3 / G3T fully consumed
        zero_bytes(sGT + 64 * 128 * 2, 64 * 128 * 2);  // padding rows 64..127 of G2T
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            dh[j] = (load_h(sH2, 64, tid, j) > 0.f) ? __half2float(__float2half_rn(dh[j])) : 0.f;
            store_h(sGT, 128, j, tid, dh[j]);
        }
        for (int c = 0; c < 64; c += 8) store_row8(sG, 64, tid, c, dh + c);
        // ---- dW2 = G2^T H1 and dH1 = G2 W2
        sy.before_mma();
        if (tid == 0) {
            gemm(tb + 128, sGT, sH1T, 128, 128, 64);
            gemm(tb + 192, sG, sW2T, 64, 128, 64);
        }
        if (!sy.commit_and_wait()) break;
        if (tid < 64) {
            float acc = 0.f;
            for (int b = 0; b < 128; ++b) acc += load_h(sGT, 128, tid, b);
            atomicAdd(grad + oB2 + tid, acc);
        }
        for (int c = 0; c < 64; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 128 + c), v);
            if (tid < 64) {
#pragma unroll
                for (int j = 0; j < 16; ++j) atomicAdd(grad + oW2 + tid * 64 + c + j, v[j]);
            }
        }
        for (int c = 0; c < 64; c += 16) tc::tmem_ld16(lane_addr(tb, 192 + c), dh + c);
        tc::fence_before_sync();
        __syncthreads();
        zero_bytes(sGT + 64 * 128 * 2, 64 * 128 * 2);
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            dh[j] = (load_h(sH1, 64, tid, j) > 0.f) ? __half2float(__float2half_rn(dh[j])) : 0.f;
            store_h(sGT, 128, j, tid, dh[j]);
        }
        for (int c = 0; c < 64; c += 8) store_row8(sG, 64, tid, c, dh + c);
        // ---- dW1 = G1^T X and dX = G1 W1
        sy.before_mma();
        if (tid == 0) {
            gemm(tb + 0, sGT, sXT, 128, 128, 32);
            gemm(tb + 32, sG, sW1T, 64, 128, 32);
        }
        if (!sy.commit_and_wait()) break;
        if (tid < 64) {
            float acc = 0.f;
            for (int b = 0; b < 128; ++b) acc += load_h(sGT, 128, tid, b);
            atomicAdd(grad + oB1 + tid, acc);
        }
        for (int c = 0; c < 32; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, c), v);
            if (tid < 64) {
#pragma unroll
                for (int j = 0; j < 16; ++j) atomicAdd(grad + oW1 + tid * 32 + c + j, v[j]);
            }
        }
        for (int c = 0; c < 32; c += 16) {
            float v[16];
            tc::tmem_ld16(lane_addr(tb, 32 + c), v);
            if (valid) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int ee = c + j;
                    float* dst = ee < kEmb ? grad + oEo + static_cast<size_t>(cell) * kEmb + ee
                                           : grad + oEd + static_cast<size_t>(bin) * kEmb + (ee - kEmb);
                    atomicAdd(dst, v[j]);
                }
            }
        }
    } while (false);
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tb, 256);
}

// ---------------------------------------------- failure-detection probe
// The MMA wait of the kernels above, alone: one CTA allocates 32 TMEM
// columns, then either issues one 128 x 32 x 16 MMA of all-ones tiles and
// commits it (complete != 0; every output is 16) or waits on a phase that
// nothing completes.  In the second case the bounded wait gives up, the error
// word gets kDevTimeout, TMEM is not read, and the CTA still frees its TMEM
// and returns, so later tcgen05 kernels on the device can allocate again.
__global__ void __launch_bounds__(128) tc_wait_probe_kernel(int complete, uint32_t limit, uint32_t* err, float* out) {
    __shared__ __align__(1024) unsigned char sA[128 * 16 * 2];
    __shared__ __align__(1024) unsigned char sB[32 * 16 * 2];
    __shared__ uint32_t sT[2];
    __shared__ __align__(8) uint64_t sM[1];
    for (int i = threadIdx.x; i < 128 * 16; i += 128) reinterpret_cast<__half*>(sA)[i] = __float2half_rn(1.f);
    for (int i = threadIdx.x; i < 32 * 16; i += 128) reinterpret_cast<__half*>(sB)[i] = __float2half_rn(1.f);
    if (threadIdx.x < 32) { tc::tmem_alloc(sT, 32); tc::tmem_relinquish(); }
    if (threadIdx.x == 0) tc::mbar_init(sM, 1);
    Sync sy{sM, 0, err, limit};
    sy.before_mma();
    const uint32_t tb = *sT;
    if (complete && threadIdx.x == 0) gemm(tb, sA, sB, 16, 128, 32);
    if (sy.commit_and_wait(complete != 0)) {
        float v[16];
        tc::tmem_ld16(lane_addr(tb, 0), v);
        out[threadIdx.x] = v[0];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tb, 32);
}

// ------------------------------------------------------------ optimiser
// The fp16 copy (and, for the weight matrices, the transposed copy) of
// master parameter i, as the forward and backward kernels read them.
__device__ __forceinline__ void store_fp16(const PredictorDev& P, size_t i, __half h) {
    if (i < oB1) {                       // W1 [64][32]
        P.w16[hW1 + i] = h;
        P.w16[hW1T + (i % 32) * 64 + i / 32] = h;
    } else if (i >= oW2 && i < oB2) {    // W2 [64][64]
        const size_t k = i - oW2;
        P.w16[hW2 + k] = h;
        P.w16[hW2T + (k % 64) * 64 + k / 64] = h;
    } else if (i >= oW3 && i < oB3) {    // W3 [128][64]
        const size_t k = i - oW3;
        P.w16[hW3 + k] = h;
        P.w16[hW3T + (k % 64) * 128 + k / 64] = h;
    }
}

// Adam on every parameter, then its fp16 copies, four parameters per thread
// (the parameter blocks all start at multiples of 4, so no group straddles
// two): one pass over the FP32 state instead of an update pass and a
// conversion pass.  Adam (Kingma & Ba 2015) with b1 = 0.9, b2 = 0.999,
// eps = 1e-8 and bias corrections b1t = 1 - b1^t, b2t = 1 - b2^t; the
// gradient is scaled by 1 / batch and cleared for the next step.
__global__ void __launch_bounds__(256) adam_fp16_kernel(PredictorDev P, float scale, float lr, float b1t, float b2t) {
    static_assert(kParams % 4 == 0 && oB1 % 4 == 0 && oW2 % 4 == 0 && oB2 % 4 == 0 && oW3 % 4 == 0 &&
                  oB3 % 4 == 0 && oEo % 4 == 0 && oEd % 4 == 0, "parameter blocks on float4 boundaries");
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float4* g4 = reinterpret_cast<float4*>(P.grad);
    float4* m4 = reinterpret_cast<float4*>(P.m);
    float4* v4 = reinterpret_cast<float4*>(P.v);
    float4* w4 = reinterpret_cast<float4*>(P.master);
    for (size_t q = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; q < kParams / 4;
         q += static_cast<size_t>(gridDim.x) * blockDim.x) {
        float g[4], m[4], v[4], w[4];
        *reinterpret_cast<float4*>(g) = g4[q];
        *reinterpret_cast<float4*>(m) = m4[q];
        *reinterpret_cast<float4*>(v) = v4[q];
        *reinterpret_cast<float4*>(w) = w4[q];
        g4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        __half h[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float gk = g[k] * scale;
            m[k] = b1 * m[k] + (1.f - b1) * gk;
            v[k] = b2 * v[k] + (1.f - b2) * gk * gk;
            w[k] = w[k] - lr * (m[k] / b1t) / (sqrtf(v[k] / b2t) + eps);
            h[k] = __float2half_rn(w[k]);
        }
        m4[q] = *reinterpret_cast<float4*>(m);
        v4[q] = *reinterpret_cast<float4*>(v);
        w4[q] = *reinterpret_cast<float4*>(w);
        const size_t i = 4 * q;
        if (i >= oEo) {                  // embeddings: one 8-byte store of four halves
            __half* dst = P.w16 + (i < oEd ? hEo + (i - oEo) : hEd + (i - oEd));
            *reinterpret_cast<uint2*>(dst) = *reinterpret_cast<const uint2*>(h);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) store_fp16(P, i + k, h[k]);
        }
    }
}

// fp16 copies of the master weights, plus the transposed copies.
__global__ void convert_kernel(PredictorDev P) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < kParams;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const __half h = __float2half_rn(P.master[i]);
        if (i < oB1) {                       // W1 [64][32]
            P.w16[hW1 + i] = h;
            const size_t r = i / 32, c = i % 32;
            P.w16[hW1T + c * 64 + r] = h;
        } else if (i >= oW2 && i < oB2) {    // W2 [64][64]
            const size_t k = i - oW2, r = k / 64, c = k % 64;
            P.w16[hW2 + k] = h;
            P.w16[hW2T + c * 64 + r] = h;
        } else if (i >= oW3 && i < oB3) {    // W3 [128][64]
            const size_t k = i - oW3, r = k / 64, c = k % 64;
            P.w16[hW3 + k] = h;
            P.w16[hW3T + c * 128 + r] = h;
        } else if (i >= oEo && i < oEd) {
            P.w16[hEo + (i - oEo)] = h;
        } else if (i >= oEd) {
            P.w16[hEd + (i - oEd)] = h;
        }
    }
}

__device__ __forceinline__ float hash_uniform(uint64_t x) {  // SplitMix64 -> [0, 1)
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return static_cast<float>(x >> 40) * (1.0f / 16777216.0f);
}

// Kaiming-uniform weights, zero biases, embeddings U(-0.1, 0.1); zero moments.
__global__ void init_kernel(PredictorDev P, uint32_t seed) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < kParams;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const float u = hash_uniform((static_cast<uint64_t>(seed) << 32) ^ i) * 2.f - 1.f;
        float w = 0.f;
        if (i < oB1) w = u * sqrtf(6.f / kIn);
        else if (i >= oW2 && i < oB2) w = u * sqrtf(6.f / kHid);
        else if (i >= oW3 && i < oB3) w = u * sqrtf(6.f / kHid);
        else if (i >= oEo) w = 0.1f * u;
        P.master[i] = w;
        P.m[i] = 0.f;
        P.v[i] = 0.f;
        P.grad[i] = 0.f;
    }
}

// ------------------------------------------------------------- treelets
// Cut the BVH into at most kClasses-1 subtrees: starting from the root,
// repeatedly split the frontier subtree with the most leaves (its children
// come from the 64-byte traversal node).  Single thread; <= 127 splits.
__device__ void treelet_cut(const crt_bvh_node* nodes, const float4* wide, uint32_t n_leaves, Treelet* out,
                            uint32_t* n_out) {
    const float4 rmn = reinterpret_cast<const float4*>(nodes)[0];
    const float4 rmx = reinterpret_cast<const float4*>(nodes)[1];
    const uint4 lr = reinterpret_cast<const uint4*>(nodes)[2];
    uint32_t cnt = 1;
    out[0].mn[0] = rmn.x; out[0].mn[1] = rmn.y; out[0].mn[2] = rmn.z;
    out[0].mx[0] = rmx.x; out[0].mx[1] = rmx.y; out[0].mx[2] = rmx.z;
    out[0].ref = (lr.y == 0u && lr.z == 0u) ? kLeafRef : 0u;
    out[0].first = 0;
    out[0].count = n_leaves;
    while (cnt < static_cast<uint32_t>(kMissClass)) {
        int best = -1;
        uint32_t bc = 1;
        for (uint32_t k = 0; k < cnt; ++k)
            if (!(out[k].ref & kLeafRef) && out[k].count > bc) { bc = out[k].count; best = static_cast<int>(k); }
        if (best < 0) break;
        const Treelet t = out[best];
        const float4* w = wide + 4 * static_cast<size_t>(t.ref);
        const float4 w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3];
        Treelet a, b;
        a.mn[0] = w0.x; a.mn[1] = w0.y; a.mn[2] = w0.z; a.mx[0] = w1.x; a.mx[1] = w1.y; a.mx[2] = w1.z;
        a.ref = __float_as_uint(w0.w); a.first = t.first; a.count = __float_as_uint(w2.w);
        b.mn[0] = w2.x; b.mn[1] = w2.y; b.mn[2] = w2.z; b.mx[0] = w3.x; b.mx[1] = w3.y; b.mx[2] = w3.z;
        b.ref = __float_as_uint(w1.w); b.first = t.first + a.count; b.count = __float_as_uint(w3.w);
        out[best] = a;
        out[cnt++] = b;
    }
    // sort by first leaf (insertion sort, <= 127 entries)
    for (uint32_t k = 1; k < cnt; ++k) {
        const Treelet t = out[k];
        int j = static_cast<int>(k) - 1;
        while (j >= 0 && out[j].first > t.first) { out[j + 1] = out[j]; --j; }
        out[j + 1] = t;
    }
    *n_out = cnt;
}

__global__ void treelet_cut_kernel(const crt_bvh_node* nodes, const float4* wide, uint32_t n_leaves, Treelet* out,
                                   uint32_t* n_out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    treelet_cut(nodes, wide, n_leaves, out, n_out);
}

// One block per scene of a batch: that scene's cut at out + 128 k.
__global__ void treelet_cut_batch_kernel(const BatchScene* scenes, const crt_bvh_node* nodes, const float4* wide,
                                         Treelet* out, uint32_t* n_out) {
    if (threadIdx.x != 0) return;
    const BatchScene sc = scenes[blockIdx.x];
    treelet_cut(nodes + sc.node_off, wide + 4 * static_cast<size_t>(sc.wide_off), sc.n_tris,
                out + 128 * static_cast<size_t>(blockIdx.x), n_out + blockIdx.x);
}

// Class of every triangle: the treelet whose leaf range (in the tree's
// left-to-right leaf order, the order of the leaf records) holds its leaf.
__device__ __forceinline__ void label_leaf(const Treelet* tl, uint32_t n, const float4* xtri, uint32_t L,
                                           uint32_t n_leaves, uint8_t* tri_class) {
    int lo = 0, hi = static_cast<int>(n) - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (tl[mid].first <= L) lo = mid; else hi = mid - 1;
    }
    const uint32_t tri = __float_as_uint(xtri[3 * static_cast<size_t>(L)].w);
    if (tri < n_leaves) tri_class[tri] = static_cast<uint8_t>(lo);
}

__global__ void treelet_label_kernel(const Treelet* tl, const uint32_t* n_tl, const float4* xtri, uint32_t n_leaves,
                                     uint8_t* tri_class) {
    const uint32_t L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= n_leaves) return;
    label_leaf(tl, *n_tl, xtri, L, n_leaves, tri_class);
}

// Leaf g of the concatenated scenes (scene k's leaves from its tri_off).
__global__ void treelet_label_batch_kernel(const BatchScene* scenes, uint32_t n_scenes, uint32_t n_total,
                                           const Treelet* tl, const uint32_t* n_tl, const float4* xtri,
                                           uint8_t* tri_class) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_total) return;
    uint32_t lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&scenes[mid].tri_off) <= g) lo = mid; else hi = mid - 1;
    }
    const BatchScene sc = scenes[lo];
    label_leaf(tl + 128 * static_cast<size_t>(lo), n_tl[lo], xtri + 3 * static_cast<size_t>(sc.tri_off), g - sc.tri_off,
               sc.n_tris, tri_class + sc.tri_off);
}

// Class of the hit of each ray (a batch's rays, or one BVH's).
__global__ void classes_of_hits_kernel(PredictorDev P, const crt_hit* hits, uint32_t n, uint16_t* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t scene = P.n_scenes ? scene_of_ray(P.scenes, P.n_scenes, i) : 0u;
    out[i] = static_cast<uint16_t>(hit_class(P, scene, hits[i].tri));
}

// ------------------------------------------------------------ bounce rays
// Stable compaction of the primary hits (block counts, one-block scan,
// ordered writes), then cosine-weighted diffuse bounce rays: ray j starts at
// hit list entry (j * 2654435761 + seed) mod n_hits, so consecutive rays come
// from unrelated pixels (incoherent).
constexpr int kCompactBlock = 1024;

__global__ void __launch_bounds__(kCompactBlock) hit_count_kernel(const crt_hit* hits, uint32_t n, uint32_t n_tris,
                                                                 uint32_t* counts) {
    const uint32_t i = blockIdx.x * kCompactBlock + threadIdx.x;
    const bool h = i < n && hits[i].tri != CRT_MISS && hits[i].tri < n_tris;
    const int c = __syncthreads_count(h);
    if (threadIdx.x == 0) counts[blockIdx.x] = static_cast<uint32_t>(c);
}

__global__ void __launch_bounds__(1024) hit_scan_kernel(uint32_t* counts, uint32_t nb, uint32_t* total) {
    __shared__ uint32_t s_part[1024];
    const uint32_t per = (nb + 1023) / 1024, lo = threadIdx.x * per, hi = min(nb, lo + per);
    uint32_t acc = 0;
    for (uint32_t b = lo; b < hi; ++b) acc += counts[b];
    s_part[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int k = 0; k < 1024; ++k) { const uint32_t t = s_part[k]; s_part[k] = run; run += t; }
        *total = run;
    }
    __syncthreads();
    uint32_t run = s_part[threadIdx.x];
    for (uint32_t b = lo; b < hi; ++b) { const uint32_t t = counts[b]; counts[b] = run; run += t; }
}

__global__ void __launch_bounds__(kCompactBlock) hit_write_kernel(const crt_hit* hits, uint32_t n, uint32_t n_tris,
                                                                 const uint32_t* offsets, uint32_t* list) {
    __shared__ uint32_t s_warp[kCompactBlock / 32];
    const uint32_t i = blockIdx.x * kCompactBlock + threadIdx.x;
    const bool h = i < n && hits[i].tri != CRT_MISS && hits[i].tri < n_tris;
    const uint32_t ball = __ballot_sync(0xFFFFFFFFu, h);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) s_warp[warp] = __popc(ball);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int w = 0; w < kCompactBlock / 32; ++w) { const uint32_t t = s_warp[w]; s_warp[w] = run; run += t; }
    }
    __syncthreads();
    if (h) list[offsets[blockIdx.x] + s_warp[warp] + __popc(ball & ((1u << lane) - 1u))] = i;
}

__global__ void bounce_kernel(const crt_ray* prim, const crt_hit* hits, const uint32_t* list, const uint32_t* n_list,
                              const float4* xtri, const uint32_t* inv_perm, uint32_t n_tris, uint32_t n_out,
                              uint32_t seed, crt_ray* out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_out) return;
    float4* o = reinterpret_cast<float4*>(out + j);
    const uint32_t nh = *n_list;
    if (nh == 0) {
        o[0] = make_float4(0.f, 0.f, 0.f, 1.f);
        o[1] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const uint32_t s = list[static_cast<uint32_t>((static_cast<uint64_t>(j) * 2654435761ull + seed) % nh)];
    const uint32_t tri = hits[s].tri;
    const float t = hits[s].t;
    const float4 r0 = reinterpret_cast<const float4*>(prim + s)[0], r1 = reinterpret_cast<const float4*>(prim + s)[1];
    const float px = r0.x + t * r1.x, py = r0.y + t * r1.y, pz = r0.z + t * r1.z;
    const uint32_t L = inv_perm[tri];
    const float4 a = xtri[3 * static_cast<size_t>(L)], b = xtri[3 * static_cast<size_t>(L) + 1],
                 c = xtri[3 * static_cast<size_t>(L) + 2];
    float nx = (b.y - a.y) * (c.z - a.z) - (b.z - a.z) * (c.y - a.y);
    float ny = (b.z - a.z) * (c.x - a.x) - (b.x - a.x) * (c.z - a.z);
    float nz = (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
    const float nl = rsqrtf(fmaxf(nx * nx + ny * ny + nz * nz, 1e-30f));
    nx *= nl; ny *= nl; nz *= nl;
    if (nx * r1.x + ny * r1.y + nz * r1.z > 0.f) { nx = -nx; ny = -ny; nz = -nz; }
    // orthonormal basis (Duff et al. 2017)
    const float sg = nz >= 0.f ? 1.f : -1.f;
    const float aa = -1.f / (sg + nz), bb = nx * ny * aa;
    const float tx = 1.f + sg * nx * nx * aa, ty = sg * bb, tz = -sg * nx;
    const float bx = bb, by = sg + ny * ny * aa, bz = -ny;
    const float u1 = hash_uniform((static_cast<uint64_t>(seed) << 33) ^ (2ull * j));
    const float u2 = hash_uniform((static_cast<uint64_t>(seed) << 33) ^ (2ull * j + 1));
    const float r = sqrtf(u1), phi = 6.28318530718f * u2;
    const float lx = r * __cosf(phi), ly = r * __sinf(phi), lz = sqrtf(fmaxf(1.f - u1, 0.f));
    const float dx = lx * tx + ly * bx + lz * nx, dy = lx * ty + ly * by + lz * ny, dz = lx * tz + ly * bz + lz * nz;
    const float dl = rsqrtf(dx * dx + dy * dy + dz * dz);
    o[0] = make_float4(px, py, pz, 1e-4f);
    o[1] = make_float4(dx * dl, dy * dl, dz * dl, __int_as_float(0x7F800000));
}

// Trace order keys (order_key) with the histograms of their four 8-bit
// digits, for classes computed without them.
__global__ void __launch_bounds__(256) order_keys_kernel(PredictorDev P, const crt_bvh_node* nodes,
                                                         const crt_ray* __restrict__ rays,
                                                         const uint16_t* __restrict__ classes, uint32_t n,
                                                         uint32_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[4 * 256];
    for (int k = threadIdx.x; k < 4 * 256; k += blockDim.x) h[k] = 0u;
    __syncthreads();
    const SceneFrame fr = scene_frame(nodes);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 r0 = __ldg(reinterpret_cast<const float4*>(rays + i));
        const float4 r1 = __ldg(reinterpret_cast<const float4*>(rays + i) + 1);
        uint32_t cell, bin, scene, cell_raw;
        ray_features(P, nodes, fr, i, r0, r1, cell, bin, scene, cell_raw);
        const uint32_t key = order_key(P.n_scenes, cell_raw, bin, scene, classes[i]);
        keys[i] = key;
#pragma unroll
        for (int p = 0; p < 4; ++p) atomicAdd(&h[p * 256 + ((key >> (8 * p)) & 255u)], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 4 * 256; k += blockDim.x)
        if (h[k]) atomicAdd(&hist[k], h[k]);
}

}  // namespace pred

// ------------------------------------------------------------ launchers
size_t pred_order_scratch_bytes(uint32_t n) {
    const size_t tiles = (n + sort_tile_keys(8) - 1) / sort_tile_keys(8);
    return 4 * (3 * static_cast<size_t>(n) + 4 * 256 + 4 * (tiles * 256 + 1) + 64);
}

void pred_order_begin(void* scratch, uint32_t n, uint32_t** keys, uint32_t** hist, cudaStream_t s) {
    uint32_t* ka = static_cast<uint32_t*>(scratch);
    uint32_t* h = ka + 3 * static_cast<size_t>(n);
    const size_t tiles = (n + sort_tile_keys(8) - 1) / sort_tile_keys(8);
    const size_t lb_words = tiles * 256 + 1;
    cudaMemsetAsync(h, 0, 4 * (4 * 256 + 4 * lb_words), s);
    *keys = ka;
    *hist = h;
}

void pred_order(const PredictorDev& P, const crt_bvh_node* nodes, const crt_ray* rays, const uint16_t* classes,
                uint32_t n, uint32_t* order, void* scratch, uint32_t* err, uint32_t spin_limit, cudaStream_t s,
                bool keys_ready) {
    if (n == 0) return;
    uint32_t* ka = static_cast<uint32_t*>(scratch);
    uint32_t* kb = ka + n;
    uint32_t* vt = kb + n;
    uint32_t* hist = vt + n;
    uint32_t* lb = hist + 4 * 256;  // per pass: ticket, then the look-back words
    const size_t tiles = (n + sort_tile_keys(8) - 1) / sort_tile_keys(8);
    const size_t lb_words = tiles * 256 + 1;
    if (!keys_ready) {
        cudaMemsetAsync(hist, 0, 4 * (4 * 256 + 4 * lb_words), s);
        const uint32_t grid = std::min<uint32_t>((n + 255) / 256, kNumSms * 8);
        pred::order_keys_kernel<<<grid, 256, 0, s>>>(P, nodes, rays, classes, n, ka, hist);
    }
    // four stable 8-bit passes; pass 0 synthesises the ray indices
    const uint32_t* kin[4] = {ka, kb, ka, kb};
    uint32_t* kout[4] = {kb, ka, kb, ka};
    const uint32_t* vin[4] = {nullptr, vt, order, vt};
    uint32_t* vout[4] = {vt, order, vt, order};
    for (int p = 0; p < 4; ++p) {
        uint32_t* l = lb + p * lb_words;
        launch_onesweep(kin[p], vin[p], kout[p], vout[p], n, 8 * p, 8, hist + 256 * p, l + 1, l, err, spin_limit, s);
    }
}
cudaError_t tc_wait_probe(int complete, uint32_t limit, uint32_t* err, float* out, cudaStream_t s) {
    pred::tc_wait_probe_kernel<<<1, 128, 0, s>>>(complete, limit ? limit : pred::kMmaWaitLimit, err, out);
    return cudaGetLastError();
}

void pred_init(const PredictorDev& P, uint32_t seed, cudaStream_t s) {
    pred::init_kernel<<<kNumSms * 8, 256, 0, s>>>(P, seed);
    pred::convert_kernel<<<kNumSms * 8, 256, 0, s>>>(P);
}

static cudaError_t infer_attributes() {
    cudaError_t e = cudaFuncSetAttribute(pred::infer_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         pred::kInferSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pred::infer_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 pred::kInferSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pred::infer_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 pred::kInferSmem);
    return e;
}

cudaError_t pred_prepare() {
    cudaError_t e = infer_attributes();
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pred::train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, pred::kTrainSmem);
    return e;
}

cudaError_t pred_infer(const PredictorDev& P, const crt_bvh_node* nodes, const crt_ray* rays, uint32_t n,
                       uint16_t* classes, float miss_threshold, bool argmax, uint32_t* err, cudaStream_t s,
                       uint32_t* order_keys, uint32_t* order_hist, crt_ray* rays_copy) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = infer_attributes();
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const uint32_t tiles = (n + 127) / 128;
    const uint32_t cap = static_cast<uint32_t>(pred::kInferCtasPerSm) * kNumSms;
    const uint32_t grid = tiles < cap ? tiles : cap;
    if (grid == 0) return cudaSuccess;
    if (!argmax)
        pred::infer_kernel<false, false><<<grid, 128, pred::kInferSmem, s>>>(P, nodes, rays, n, classes, miss_threshold,
                                                                             nullptr, nullptr, rays_copy, err);
    else if (!order_keys)
        pred::infer_kernel<true, false><<<grid, 128, pred::kInferSmem, s>>>(P, nodes, rays, n, classes, miss_threshold,
                                                                            nullptr, nullptr, rays_copy, err);
    else
        pred::infer_kernel<true, true><<<grid, 128, pred::kInferSmem, s>>>(P, nodes, rays, n, classes, miss_threshold,
                                                                           order_keys, order_hist, rays_copy, err);
    return cudaGetLastError();
}

cudaError_t pred_train_step(const PredictorDev& P, const crt_bvh_node* nodes, const crt_ray* rays, uint32_t n_rays,
                            const crt_hit* hits, const uint16_t* targets, uint32_t n_samples, uint32_t stride,
                            uint32_t offset, float* loss_sum, uint32_t* err, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(pred::train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             pred::kTrainSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const uint32_t grid = (n_samples + 127) / 128;
    if (grid == 0) return cudaSuccess;
    pred::train_kernel<<<grid, 128, pred::kTrainSmem, s>>>(P, nodes, rays, n_rays, hits, targets, n_samples, stride,
                                                          offset, P.grad, loss_sum, err);
    return cudaGetLastError();
}

void pred_adam(const PredictorDev& P, float scale, float lr, uint32_t step, cudaStream_t s) {
    const float b1t = 1.f - std::pow(0.9f, static_cast<float>(step));
    const float b2t = 1.f - std::pow(0.999f, static_cast<float>(step));
    pred::adam_fp16_kernel<<<kNumSms * 8, 256, 0, s>>>(P, scale, lr, b1t, b2t);
}

void pred_refresh_fp16(const PredictorDev& P, cudaStream_t s) {
    pred::convert_kernel<<<kNumSms * 8, 256, 0, s>>>(P);
}

void pred_treelets(const crt_bvh_node* nodes, const float4* wide, const float4* xtri, uint32_t n_leaves,
                   Treelet* tl, uint32_t* n_tl, uint8_t* tri_class, cudaStream_t s) {
    pred::treelet_cut_kernel<<<1, 1, 0, s>>>(nodes, wide, n_leaves, tl, n_tl);
    pred::treelet_label_kernel<<<(n_leaves + 255) / 256, 256, 0, s>>>(tl, n_tl, xtri, n_leaves, tri_class);
}

void pred_treelets_batch(const BatchScene* scenes, uint32_t n_scenes, uint32_t n_tris, const crt_bvh_node* nodes,
                         const float4* wide, const float4* xtri, Treelet* tl, uint32_t* n_tl, uint8_t* tri_class,
                         cudaStream_t s) {
    if (n_scenes == 0) return;
    pred::treelet_cut_batch_kernel<<<n_scenes, 32, 0, s>>>(scenes, nodes, wide, tl, n_tl);
    pred::treelet_label_batch_kernel<<<(n_tris + 255) / 256, 256, 0, s>>>(scenes, n_scenes, n_tris, tl, n_tl, xtri,
                                                                          tri_class);
}

void pred_classes_of_hits(const PredictorDev& P, const crt_hit* hits, uint32_t n, uint16_t* out, cudaStream_t s) {
    if (n == 0) return;
    pred::classes_of_hits_kernel<<<(n + 255) / 256, 256, 0, s>>>(P, hits, n, out);
}

size_t bounce_scratch_bytes(uint32_t n_prim) {
    const size_t nb = (n_prim + pred::kCompactBlock - 1) / pred::kCompactBlock;
    return 4 * (nb + 4 + static_cast<size_t>(n_prim));
}

void launch_bounce(const crt_ray* prim, const crt_hit* hits, uint32_t n_prim, const float4* xtri,
                   const uint32_t* inv_perm, uint32_t n_tris, uint32_t n_out, uint32_t seed, crt_ray* out,
                   uint32_t* scratch, cudaStream_t s) {
    if (n_out == 0 || n_prim == 0) return;
    const uint32_t nb = (n_prim + pred::kCompactBlock - 1) / pred::kCompactBlock;
    uint32_t* counts = scratch;
    uint32_t* total = scratch + nb;
    uint32_t* list = scratch + nb + 4;
    pred::hit_count_kernel<<<nb, pred::kCompactBlock, 0, s>>>(hits, n_prim, n_tris, counts);
    pred::hit_scan_kernel<<<1, 1024, 0, s>>>(counts, nb, total);
    pred::hit_write_kernel<<<nb, pred::kCompactBlock, 0, s>>>(hits, n_prim, n_tris, counts, list);
    pred::bounce_kernel<<<(n_out + 255) / 256, 256, 0, s>>>(prim, hits, list, total, xtri, inv_perm, n_tris, n_out,
                                                           seed, out);
}

}  // namespace crt
