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
//   refit_count / refit_scan / refit_link  once per build: for every leaf
//       (indexed by its place in the tree's left-to-right leaf order) and
//       every internal node (indexed by its rank among internal nodes in DFS
//       order, which is also its traversal-node index) a link to its parent:
//       the parent's rank, which child it is, and the parent's leaf range;
//       plus the DFS position of every internal node;
//   refit_up      one thread per leaf: the moved triangle (traversal leaf
//       record) and its box, then up the tree: at each parent the two
//       children count in and the second to arrive merges both boxes, writes
//       the parent's traversal node and goes on, so every node is finished
//       once, after both children;
//   refit_grow    the watertight copy of the traversal nodes, every box grown
//       by the slack of the new root box (coalesced, one float4 per thread);
//   refit_nodes   on demand (copy-out, box display): the boxes of the
//       reference-layout node array from the traversal nodes.
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {

constexpr uint32_t kNoParent = 0xFFFFFFFFu;

__device__ __forceinline__ bool is_internal_node(const crt_bvh_node* nodes, uint32_t d) {
    const uint4 k = __ldg(reinterpret_cast<const uint4*>(nodes + d) + 2);  // tri, left, right, pad
    return (k.y | k.z) != 0u;
}

__global__ void __launch_bounds__(256) refit_count_kernel(const crt_bvh_node* __restrict__ nodes, uint32_t n_nodes,
                                                          uint32_t* __restrict__ block_count) {
    const uint32_t d = blockIdx.x * 256 + threadIdx.x;
    const bool internal = d < n_nodes && is_internal_node(nodes, d);
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

// For internal node d of rank k: its first leaf is the number of leaves
// before it in DFS order (d - k) and its children's leaf counts are in its
// traversal node; its left child sits at d + 1 (rank k + 1 if internal, leaf
// index first if a leaf), its right child at the node's right index (rank
// right - (first + left count) if internal, leaf index first + left count if
// a leaf).  Links are (parent rank << 1 | child slot, parent's first leaf,
// parent's leaf end, 0); the root's is (kNoParent, 0, N, 0).
__global__ void __launch_bounds__(256) refit_link_kernel(const crt_bvh_node* __restrict__ nodes, uint32_t n_nodes,
                                                         const uint32_t* __restrict__ block_offset,
                                                         const float4* __restrict__ wide, uint4* __restrict__ leaf_link,
                                                         uint4* __restrict__ int_link, uint32_t* __restrict__ int_dfs,
                                                         uint32_t* err) {
    __shared__ uint32_t s_w[8];
    const uint32_t d = blockIdx.x * 256 + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint4 k = make_uint4(0u, 0u, 0u, 0u);
    if (d < n_nodes) k = __ldg(reinterpret_cast<const uint4*>(nodes + d) + 2);
    const bool internal = d < n_nodes && (k.y | k.z) != 0u;
    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, internal);
    if (lane == 0) s_w[warp] = __popc(ballot);
    __syncthreads();
    uint32_t rank = __ldg(block_offset + blockIdx.x) + __popc(ballot & ((1u << lane) - 1u));
    for (uint32_t w = 0; w < warp; ++w) rank += s_w[w];
    const uint32_t N = (n_nodes + 1) / 2;
    if (d == 0) {
        if (internal) int_link[0] = make_uint4(kNoParent, 0u, N, 0u);
        else leaf_link[0] = make_uint4(kNoParent, 0u, N, 0u);
    }
    if (!internal) return;
    // DFS pre-order: the left child follows its parent
    if (k.y != d + 1 || k.z <= k.y || k.z >= n_nodes || rank >= N - 1 || d < rank) {
        raise_corrupt(err, 12, d, k.z);
        return;
    }
    const uint32_t first = d - rank;
    const uint32_t lca = __float_as_uint(__ldg(wide + 4 * static_cast<size_t>(rank) + 2).w);
    const uint32_t lcb = __float_as_uint(__ldg(wide + 4 * static_cast<size_t>(rank) + 3).w);
    if (first >= N || lca == 0u || lcb == 0u || static_cast<uint64_t>(first) + lca + lcb > N) {
        raise_corrupt(err, 12, d, lca);
        return;
    }
    int_dfs[rank] = d;
    const uint32_t end = first + lca + lcb;
    const uint32_t ch[2] = {k.y, k.z}, chf[2] = {first, first + lca};
#pragma unroll
    for (uint32_t slot = 0; slot < 2; ++slot) {
        const uint4 l = make_uint4((rank << 1) | slot, first, end, 0u);
        if (is_internal_node(nodes, ch[slot])) {
            if (ch[slot] < chf[slot] || ch[slot] - chf[slot] >= N - 1) { raise_corrupt(err, 12, d, ch[slot]); continue; }
            int_link[ch[slot] - chf[slot]] = l;  // the child's rank
        } else {
            leaf_link[chf[slot]] = l;
        }
    }
}

__device__ __forceinline__ void store_xyz(float4* p, float x, float y, float z) {
    reinterpret_cast<float2*>(p)[0] = make_float2(x, y);
    reinterpret_cast<float*>(p)[2] = z;
}

// One block per kRefitLeaves consecutive leaves of the tree's left-to-right
// leaf order (the order of the leaf records), in which every subtree's
// leaves form one range.  A parent whose whole leaf range lies in the
// block's range has both arriving threads in the block: they meet in shared
// memory (box and reference per side, slot indexed by the parent's split
// leaf — the first leaf of its right subtree, unique per internal node — and
// a counter) with block-scope fences, and the second writes the parent's
// whole traversal node (boxes, references, leaf counts: 64 full bytes).
// Parents spanning blocks meet in global memory: each child writes its box
// into its half of the parent's traversal node (whose references and leaf
// counts stay as the build wrote them), then counts in with an
// acquire-release atomic.
constexpr int kRefitLeaves = 512;

__global__ void __launch_bounds__(kRefitLeaves) refit_up_kernel(const crt_triangle* __restrict__ tris, uint32_t N,
                                                                const float* __restrict__ models,
                                                                const uint4* __restrict__ leaf_link,
                                                                const uint4* __restrict__ int_link,
                                                                uint32_t* __restrict__ cnt,
                                                                crt_bvh_node* __restrict__ nodes,
                                                                float4* __restrict__ xtri, float4* __restrict__ wide,
                                                                uint32_t* err) {
    __shared__ uint32_t s_cnt[kRefitLeaves];
    __shared__ float s_box[kRefitLeaves][2][6];
    __shared__ uint32_t s_ref[kRefitLeaves][2];
    s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t lo = blockIdx.x * kRefitLeaves;
    const uint32_t hi = min(lo + kRefitLeaves, N);
    const uint32_t L = lo + threadIdx.x;
    if (L >= N) return;
    const uint32_t ti = __float_as_uint(xtri[3 * static_cast<size_t>(L)].w);  // the leaf's triangle stays
    if (ti >= N) { raise_corrupt(err, 13, L, ti); return; }
    // the moved triangle: leaf record (p0 | triangle id, p1 | model id, p2) and box
    const TriRec t = load_tri(tris, ti);
    if (t.model >= kMaxModels) raise_error(err, kDevBadModel);
    const float* M = models + 16 * (t.model & (kMaxModels - 1));
    const float4 p0 = mat_vec(M, t.p0), p1 = mat_vec(M, t.p1), p2 = mat_vec(M, t.p2);
    xtri[3 * static_cast<size_t>(L) + 0] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(ti));
    xtri[3 * static_cast<size_t>(L) + 1] = make_float4(p1.x, p1.y, p1.z, __uint_as_float(t.model));
    xtri[3 * static_cast<size_t>(L) + 2] = make_float4(p2.x, p2.y, p2.z, 0.f);
    float b[6] = {min_std(p0.x, min_std(p1.x, p2.x)), min_std(p0.y, min_std(p1.y, p2.y)),
                  min_std(p0.z, min_std(p1.z, p2.z)), max_std(p0.x, max_std(p1.x, p2.x)),
                  max_std(p0.y, max_std(p1.y, p2.y)), max_std(p0.z, max_std(p1.z, p2.z))};
    uint32_t ref = kLeafRef | L;            // this node's reference in its parent's traversal node
    uint32_t my_first = L, my_end = L + 1;  // its leaf range
    uint4 up = __ldg(leaf_link + L);
    for (uint32_t guard = 0; guard < N; ++guard) {
        if (up.x == kNoParent) {  // the root: its box goes to the node array (the slack is read from it)
            float4* nb = reinterpret_cast<float4*>(nodes);
            nb[0] = make_float4(b[0], b[1], b[2], 0.f);
            nb[1] = make_float4(b[3], b[4], b[5], 0.f);
            return;
        }
        const uint32_t k = up.x >> 1, slot = up.x & 1u;
        if (k >= N - 1) { raise_corrupt(err, 14, L, k); return; }
        float4* w = wide + 4 * static_cast<size_t>(k);
        float sb[6];
        uint32_t sref = 0;
        const bool in_block = up.y >= lo && up.z <= hi;
        if (in_block) {
            const uint32_t j = (slot == 0u ? my_end : my_first) - lo;  // the parent's split leaf, in [1, hi - lo)
            if (j == 0u || j >= kRefitLeaves) { raise_corrupt(err, 14, L, j); return; }
#pragma unroll
            for (int c = 0; c < 6; ++c) s_box[j][slot][c] = b[c];
            s_ref[j][slot] = ref;
            __threadfence_block();
            if (atomicAdd(&s_cnt[j], 1u) == 0u) return;  // the sibling's thread finishes the parent
            __threadfence_block();
#pragma unroll
            for (int c = 0; c < 6; ++c) sb[c] = s_box[j][slot ^ 1u][c];
            sref = s_ref[j][slot ^ 1u];
        } else {
            store_xyz(w + 2 * slot, b[0], b[1], b[2]);
            store_xyz(w + 2 * slot + 1, b[3], b[4], b[5]);
            if (atomic_add_acq_rel_u32(cnt + k, 1u) == 0u) return;
            const float4 smn = __ldcg(w + 2 * (slot ^ 1u)), smx = __ldcg(w + 2 * (slot ^ 1u) + 1);
            sb[0] = smn.x; sb[1] = smn.y; sb[2] = smn.z;
            sb[3] = smx.x; sb[4] = smx.y; sb[5] = smx.z;
        }
        float lb[6], rb[6];  // left and right child's boxes
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            lb[c] = slot == 0u ? b[c] : sb[c];
            rb[c] = slot == 0u ? sb[c] : b[c];
        }
        if (in_block) {
            const uint32_t lref = slot == 0u ? ref : sref, rref = slot == 0u ? sref : ref;
            const uint32_t mine = my_end - my_first, other = (up.z - up.y) - mine;
            const uint32_t lcnt = slot == 0u ? mine : other, rcnt = slot == 0u ? other : mine;
            w[0] = make_float4(lb[0], lb[1], lb[2], __uint_as_float(lref));
            w[1] = make_float4(lb[3], lb[4], lb[5], __uint_as_float(rref));
            w[2] = make_float4(rb[0], rb[1], rb[2], __uint_as_float(lcnt));
            w[3] = make_float4(rb[3], rb[4], rb[5], __uint_as_float(rcnt));
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {  // AABB::merge(left, right)
            b[c] = min_std(lb[c], rb[c]);
            b[3 + c] = max_std(lb[3 + c], rb[3 + c]);
        }
        ref = k;
        my_first = up.y;
        my_end = up.z;
        up = __ldg(int_link + k);
    }
    raise_corrupt(err, 14, L, ref);
}

// wide_wt = wide with every box grown by the slack of the new root box
// (min - grow, max + grow, as the build's layout pass rounds them).
__global__ void __launch_bounds__(256) refit_grow_kernel(const crt_bvh_node* __restrict__ nodes,
                                                         const float4* __restrict__ wide, uint32_t n_vec,
                                                         float4* __restrict__ wide_wt, RefitState* st) {
    __shared__ float s_grow;
    if (threadIdx.x == 0) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(nodes)), b = __ldg(reinterpret_cast<const float4*>(nodes) + 1);
        const float smin[3] = {a.x, a.y, a.z}, smax[3] = {b.x, b.y, b.z};
        s_grow = scene_abs_eps(smin, smax);
        if (blockIdx.x == 0) st->abs_eps = s_grow;
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n_vec) return;
    const float g = (i & 1u) ? s_grow : -s_grow;  // float4s alternate min, max
    const float4 v = __ldg(wide + i);
    wide_wt[i] = make_float4(v.x + g, v.y + g, v.z + g, v.w);
}

// Node-array boxes from the traversal nodes: internal node k (DFS position
// int_dfs[k]) holds its children's boxes; its left child sits right after
// it, its right child at its right index.  The root's box is already there.
__global__ void __launch_bounds__(256) refit_nodes_kernel(const float4* __restrict__ wide,
                                                          const uint32_t* __restrict__ int_dfs, uint32_t N,
                                                          crt_bvh_node* __restrict__ nodes, uint32_t* err) {
    const uint32_t k = blockIdx.x * 256 + threadIdx.x;
    if (k + 1 >= N) return;
    const uint32_t n_nodes = 2 * N - 1;
    const uint32_t d = __ldg(int_dfs + k);
    if (d + 1 >= n_nodes) { raise_corrupt(err, 15, k, d); return; }
    const uint32_t right = __ldg(reinterpret_cast<const uint4*>(nodes + d) + 2).z;
    if (right >= n_nodes) { raise_corrupt(err, 15, k, right); return; }
    const float4* w = wide + 4 * static_cast<size_t>(k);
    const float4 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2), w3 = __ldg(w + 3);
    float4* l = reinterpret_cast<float4*>(nodes + d + 1);
    float4* r = reinterpret_cast<float4*>(nodes + right);
    l[0] = make_float4(w0.x, w0.y, w0.z, 0.f);
    l[1] = make_float4(w1.x, w1.y, w1.z, 0.f);
    r[0] = make_float4(w2.x, w2.y, w2.z, 0.f);
    r[1] = make_float4(w3.x, w3.y, w3.z, 0.f);
}

uint32_t refit_topo_blocks(uint32_t N) { return (2 * N - 1 + 255) / 256; }

void launch_refit_topology(const crt_bvh_node* nodes, const float4* wide, uint32_t N, uint4* leaf_link, uint4* int_link,
                           uint32_t* int_dfs, uint32_t* block_count, uint32_t* err, cudaStream_t s) {
    const uint32_t n_nodes = 2 * N - 1, blocks = refit_topo_blocks(N);
    refit_count_kernel<<<blocks, 256, 0, s>>>(nodes, n_nodes, block_count);
    refit_scan_kernel<<<1, 1024, 0, s>>>(block_count, blocks);
    refit_link_kernel<<<blocks, 256, 0, s>>>(nodes, n_nodes, block_count, wide, leaf_link, int_link, int_dfs, err);
}

void launch_refit(const crt_triangle* tris, uint32_t N, const float* models, const uint4* leaf_link,
                  const uint4* int_link, uint32_t* cnt, crt_bvh_node* nodes, float4* xtri, float4* wide,
                  float4* wide_wt, RefitState* st, uint32_t* err, cudaStream_t s) {
    refit_up_kernel<<<(N + kRefitLeaves - 1) / kRefitLeaves, kRefitLeaves, 0, s>>>(tris, N, models, leaf_link, int_link,
                                                                                  cnt, nodes, xtri, wide, err);
    const uint32_t n_vec = 4 * (N - 1);
    refit_grow_kernel<<<n_vec ? (n_vec + 255) / 256 : 1u, 256, 0, s>>>(nodes, wide, n_vec, wide_wt, st);
}

void launch_refit_nodes(const float4* wide, const uint32_t* int_dfs, uint32_t N, crt_bvh_node* nodes, uint32_t* err,
                        cudaStream_t s) {
    if (N < 2) return;
    refit_nodes_kernel<<<(N - 1 + 255) / 256, 256, 0, s>>>(wide, int_dfs, N, nodes, err);
}

}  // namespace crt
