// Refit of a built BVH (crt_refit): the triangles move, the tree keeps its
// topology, and every box is recomputed bottom-up.  No counterpart in the
// reference, which rebuilds the whole tree (srcOpenGL/scene/scene.cpp:148);
// the boxes follow its rules: a leaf box is AABB::buildFromTriangle of the
// transformed triangle (srcCommon/scene/geometry/bvh.cpp:383-399), an
// internal box AABB::merge(left, right) (bvh.cpp:401-413) in the order the
// PLOC merge applies it (bvh.cpp:169-172), so a refit of unmoved triangles
// reproduces the built node array bit for bit.  Compiled with -fmad=false.
//
// Kernels:
//   refit_topo / refit_scan / refit_rank  once per build: parent of every
//       node, DFS index of every leaf, and the rank of every internal node
//       among internal nodes in DFS order (its traversal-node index);
//   refit_leaves  new transformed triangles (traversal leaf records) and the
//       scene box, for the traversal slack;
//   refit_up      one thread per leaf walks up; at each parent the second
//       child to arrive (an atomic counter per node) merges both boxes and
//       continues, so every node is finished once, after both children.
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {

constexpr uint32_t kNoParent = 0xFFFFFFFFu;

__device__ __forceinline__ float from_ordered_key(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k ^ 0x80000000u) : ~k);
}

__global__ void __launch_bounds__(256) refit_topo_kernel(const crt_bvh_node* __restrict__ nodes, uint32_t n_nodes,
                                                         const uint32_t* __restrict__ inv_perm, uint32_t N,
                                                         uint32_t* __restrict__ parent, uint32_t* __restrict__ leaf_dfs,
                                                         uint32_t* __restrict__ block_count, uint32_t* err) {
    const uint32_t d = blockIdx.x * 256 + threadIdx.x;
    bool internal = false;
    if (d < n_nodes) {
        const uint4 k = __ldg(reinterpret_cast<const uint4*>(nodes + d) + 2);  // tri, left, right, pad
        internal = (k.y | k.z) != 0u;
        if (d == 0) parent[0] = kNoParent;
        if (internal) {
            // DFS pre-order: the left child follows its parent
            if (k.y != d + 1 || k.z <= k.y || k.z >= n_nodes) raise_corrupt(err, 12, d, k.z);
            else {
                parent[k.y] = d;
                parent[k.z] = d;
            }
        } else {
            const uint32_t L = k.x < N ? __ldg(inv_perm + k.x) : 0xFFFFFFFFu;
            if (L >= N) raise_corrupt(err, 12, d, k.x);
            else leaf_dfs[L] = d;
        }
    }
    const uint32_t c = static_cast<uint32_t>(__syncthreads_count(internal));
    if (threadIdx.x == 0) block_count[blockIdx.x] = c;
}

// Exclusive scan of the per-block internal-node counts, in place (one block).
__global__ void __launch_bounds__(1024) refit_scan_kernel(uint32_t* __restrict__ block_count, uint32_t n_blocks) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0u;
    __syncthreads();
    for (uint32_t base = 0; base < n_blocks; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < n_blocks ? block_count[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= static_cast<uint32_t>(o)) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= static_cast<uint32_t>(o)) w += y;
            }
            s_warp[lane] = w;
        }
        __syncthreads();
        const uint32_t excl = s_carry + (warp ? s_warp[warp - 1] : 0u) + x - v;
        if (i < n_blocks) block_count[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) s_carry = excl + v;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) refit_rank_kernel(const crt_bvh_node* __restrict__ nodes, uint32_t n_nodes,
                                                         const uint32_t* __restrict__ block_offset,
                                                         uint32_t* __restrict__ rank) {
    __shared__ uint32_t s_w[8];
    const uint32_t d = blockIdx.x * 256 + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    bool internal = false;
    if (d < n_nodes) {
        const uint4 k = __ldg(reinterpret_cast<const uint4*>(nodes + d) + 2);
        internal = (k.y | k.z) != 0u;
    }
    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, internal);
    if (lane == 0) s_w[warp] = __popc(ballot);
    __syncthreads();
    uint32_t before = __ldg(block_offset + blockIdx.x) + __popc(ballot & ((1u << lane) - 1u));
    for (uint32_t w = 0; w < warp; ++w) before += s_w[w];
    if (d < n_nodes) rank[d] = internal ? before : 0xFFFFFFFFu;
}

// New leaf records (sorted order: transformed p0 | triangle id, p1 | model
// id, p2) and the scene box of the moved triangles.
__global__ void __launch_bounds__(256) refit_leaves_kernel(const crt_triangle* __restrict__ tris, uint32_t N,
                                                           const float* __restrict__ models,
                                                           const uint32_t* __restrict__ perm, float4* __restrict__ xtri,
                                                           RefitState* st, uint32_t* err) {
    uint32_t kmax[3] = {0u, 0u, 0u}, kmin_inv[3] = {0u, 0u, 0u};  // max of keys, max of complemented keys
    bool bad = false;
    for (uint32_t L = blockIdx.x * blockDim.x + threadIdx.x; L < N; L += gridDim.x * blockDim.x) {
        const uint32_t ti = __ldg(perm + L);
        if (ti >= N) { raise_corrupt(err, 13, L, ti); continue; }
        const TriRec t = load_tri(tris, ti);
        bad |= t.model >= kMaxModels;
        const float* M = models + 16 * (t.model & (kMaxModels - 1));
        const float4 p0 = mat_vec(M, t.p0), p1 = mat_vec(M, t.p1), p2 = mat_vec(M, t.p2);
        xtri[3 * static_cast<size_t>(L) + 0] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(ti));
        xtri[3 * static_cast<size_t>(L) + 1] = make_float4(p1.x, p1.y, p1.z, __uint_as_float(t.model));
        xtri[3 * static_cast<size_t>(L) + 2] = make_float4(p2.x, p2.y, p2.z, 0.f);
        const float lo[3] = {min_std(p0.x, min_std(p1.x, p2.x)), min_std(p0.y, min_std(p1.y, p2.y)),
                             min_std(p0.z, min_std(p1.z, p2.z))};
        const float hi[3] = {max_std(p0.x, max_std(p1.x, p2.x)), max_std(p0.y, max_std(p1.y, p2.y)),
                             max_std(p0.z, max_std(p1.z, p2.z))};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (hi[a] == hi[a]) kmax[a] = max(kmax[a], ordered_key(hi[a]));
            if (lo[a] == lo[a]) kmin_inv[a] = max(kmin_inv[a], ~ordered_key(lo[a]));
        }
    }
    if (bad) raise_error(err, kDevBadModel);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o > 0; o >>= 1) {
            kmax[a] = max(kmax[a], __shfl_xor_sync(0xFFFFFFFFu, kmax[a], o));
            kmin_inv[a] = max(kmin_inv[a], __shfl_xor_sync(0xFFFFFFFFu, kmin_inv[a], o));
        }
    if ((threadIdx.x & 31u) == 0u)
        for (int a = 0; a < 3; ++a) {
            if (kmax[a]) atomicMax(&st->key_max[a], kmax[a]);
            if (kmin_inv[a]) atomicMax(&st->key_min_inv[a], kmin_inv[a]);
        }
}

__global__ void __launch_bounds__(256) refit_up_kernel(const float4* __restrict__ xtri, uint32_t N,
                                                       const uint32_t* __restrict__ leaf_dfs,
                                                       const uint32_t* __restrict__ parent,
                                                       const uint32_t* __restrict__ rank, uint32_t* __restrict__ cnt,
                                                       crt_bvh_node* __restrict__ nodes, float4* __restrict__ wide,
                                                       float4* __restrict__ wide_wt, RefitState* st, uint32_t* err) {
    __shared__ float s_grow;
    if (threadIdx.x == 0) {
        float smin[3], smax[3];
        for (int a = 0; a < 3; ++a) {
            smax[a] = from_ordered_key(st->key_max[a]);
            smin[a] = from_ordered_key(~st->key_min_inv[a]);
        }
        const float g = scene_abs_eps(smin, smax);
        s_grow = g;
        if (blockIdx.x == 0) st->abs_eps = g;
    }
    __syncthreads();
    const float grow = s_grow;
    const uint32_t L = blockIdx.x * 256 + threadIdx.x;
    if (L >= N) return;
    const uint32_t n_nodes = 2 * N - 1;
    uint32_t cur = __ldg(leaf_dfs + L);
    if (cur >= n_nodes) { raise_corrupt(err, 14, L, cur); return; }
    const float4 a = __ldg(xtri + 3 * static_cast<size_t>(L)), b = __ldg(xtri + 3 * static_cast<size_t>(L) + 1),
                 c = __ldg(xtri + 3 * static_cast<size_t>(L) + 2);
    float3 mn = make_float3(min_std(a.x, min_std(b.x, c.x)), min_std(a.y, min_std(b.y, c.y)), min_std(a.z, min_std(b.z, c.z)));
    float3 mx = make_float3(max_std(a.x, max_std(b.x, c.x)), max_std(a.y, max_std(b.y, c.y)), max_std(a.z, max_std(b.z, c.z)));
    float4* nb = reinterpret_cast<float4*>(nodes + cur);
    nb[0] = make_float4(mn.x, mn.y, mn.z, 0.f);
    nb[1] = make_float4(mx.x, mx.y, mx.z, 0.f);
    for (uint32_t guard = 0; guard < n_nodes; ++guard) {
        const uint32_t p = __ldg(parent + cur);
        if (p == kNoParent) return;  // cur is the root
        const uint32_t k = p < n_nodes ? __ldg(rank + p) : 0xFFFFFFFFu;
        if (k >= N - 1) { raise_corrupt(err, 14, cur, p); return; }
        const uint32_t slot = (cur == p + 1) ? 0u : 1u;  // left child follows its parent
        // this child's box in the parent's traversal record; the .w words
        // (child references, leaf counts) stay as the build wrote them
        float4* w = wide + 4 * static_cast<size_t>(k) + 2 * slot;
        float4* g = wide_wt + 4 * static_cast<size_t>(k) + 2 * slot;
        const float w0 = w[0].w, w1 = w[1].w;
        w[0] = make_float4(mn.x, mn.y, mn.z, w0);
        w[1] = make_float4(mx.x, mx.y, mx.z, w1);
        g[0] = make_float4(mn.x - grow, mn.y - grow, mn.z - grow, w0);
        g[1] = make_float4(mx.x + grow, mx.y + grow, mx.z + grow, w1);
        __threadfence();
        if (atomicAdd(cnt + k, 1u) == 0u) return;  // the sibling's thread finishes the parent
        __threadfence();
        const uint32_t sib = slot == 0u ? __ldg(reinterpret_cast<const uint4*>(nodes + p) + 2).z : p + 1;
        if (sib >= n_nodes) { raise_corrupt(err, 14, p, sib); return; }
        const float4 smn = __ldcg(reinterpret_cast<const float4*>(nodes + sib));
        const float4 smx = __ldcg(reinterpret_cast<const float4*>(nodes + sib) + 1);
        if (slot == 0u) {  // AABB::merge(left = this, right = sibling)
            mn = make_float3(min_std(mn.x, smn.x), min_std(mn.y, smn.y), min_std(mn.z, smn.z));
            mx = make_float3(max_std(mx.x, smx.x), max_std(mx.y, smx.y), max_std(mx.z, smx.z));
        } else {           // AABB::merge(left = sibling, right = this)
            mn = make_float3(min_std(smn.x, mn.x), min_std(smn.y, mn.y), min_std(smn.z, mn.z));
            mx = make_float3(max_std(smx.x, mx.x), max_std(smx.y, mx.y), max_std(smx.z, mx.z));
        }
        float4* pb = reinterpret_cast<float4*>(nodes + p);
        pb[0] = make_float4(mn.x, mn.y, mn.z, 0.f);
        pb[1] = make_float4(mx.x, mx.y, mx.z, 0.f);
        cur = p;
    }
    raise_corrupt(err, 14, L, cur);
}

uint32_t refit_topo_blocks(uint32_t N) { return (2 * N - 1 + 255) / 256; }

void launch_refit_topology(const crt_bvh_node* nodes, const uint32_t* inv_perm, uint32_t N, uint32_t* parent,
                           uint32_t* leaf_dfs, uint32_t* rank, uint32_t* block_count, uint32_t* err, cudaStream_t s) {
    const uint32_t n_nodes = 2 * N - 1, blocks = refit_topo_blocks(N);
    refit_topo_kernel<<<blocks, 256, 0, s>>>(nodes, n_nodes, inv_perm, N, parent, leaf_dfs, block_count, err);
    refit_scan_kernel<<<1, 1024, 0, s>>>(block_count, blocks);
    refit_rank_kernel<<<blocks, 256, 0, s>>>(nodes, n_nodes, block_count, rank);
}

void launch_refit(const crt_triangle* tris, uint32_t N, const float* models, const uint32_t* perm,
                  const uint32_t* leaf_dfs, const uint32_t* parent, const uint32_t* rank, uint32_t* cnt,
                  crt_bvh_node* nodes, float4* xtri, float4* wide, float4* wide_wt, RefitState* st, uint32_t* err,
                  cudaStream_t s) {
    const uint32_t want = (N + 255) / 256;
    const uint32_t grid = want < static_cast<uint32_t>(kNumSms * 8) ? want : kNumSms * 8;
    refit_leaves_kernel<<<grid, 256, 0, s>>>(tris, N, models, perm, xtri, st, err);
    refit_up_kernel<<<want, 256, 0, s>>>(xtri, N, leaf_dfs, parent, rank, cnt, nodes, wide, wide_wt, st, err);
}

}  // namespace crt
