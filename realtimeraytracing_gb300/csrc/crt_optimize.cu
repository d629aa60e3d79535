// Treelet restructuring of a built or refit BVH (crt_optimize): the tree
// keeps its leaves and gets a lower surface-area cost, after Karras & Aila,
// "Fast Parallel Construction of High-Quality Bounding Volume Hierarchies"
// (HPG 2013).  No counterpart in the reference, which builds once per scene
// change (srcOpenGL/scene/scene.cpp:148); boxes follow its rules —
// AABB::merge(left, right) (srcCommon/scene/geometry/bvh.cpp:401-413), areas
// AABB::getSurfaceArea (bvh.cpp:378-381) — and the result is laid out by the
// build's own DFS layout pass (scene.cpp:189-208 order).  Compiled with
// -fmad=false: every value is one exact function of the input tree.
//
// Ids: leaves 0..N-1 (their place in the tree's left-to-right leaf order),
// internal nodes N + rank (rank among internal nodes in DFS order; the root
// is N).  Cost: a leaf costs its area, an internal node
// kOptCi * area + (cost(left) + cost(right)).
//
// Kernels:
//   opt_init     one thread per internal node: ids, parents and child boxes
//                from the traversal nodes, leaf costs;
//   opt_pass     one thread per leaf climbing to the root; at each internal
//                node the second child to arrive (acquire-release counter)
//                finishes it: box, leaf count, height, cost — in its own
//                lane, unless the node has at least 7 leaves and treelets are
//                on: then the whole warp takes it, one node at a time, and
//                runs the treelet step:
//                  formation: treelet leaves [left, right]; 5 times the
//                    internal one of largest area (ordered-key compare, ties
//                    to the lowest index) is replaced by its left child and
//                    its right child appended;
//                  areas of all 127 subsets (union of the members' boxes in
//                    increasing index, AABB::merge(union, member));
//                  dynamic programme over subset sizes 2..7: C[s] = kOptCi *
//                    A[s] + min over splits p (p holds the lowest member of s,
//                    p != s) of C[p] + C[s ^ p], minimum by (ordered key,
//                    p); sizes up to 5 one lane per subset, size 6 four lanes
//                    per subset, size 7 the whole warp;
//                  if C[all] < cost(R): the treelet's internal subsets take
//                    its ids in pre-order (left first) and get their union
//                    boxes, costs, leaf counts and heights;
//   opt_hist / opt_relabel / opt_remap  internal nodes renumbered by height
//                (children below parents, the root last: the id order the
//                build's layout levels need), children and boxes moved to
//                the new ids;
// then the build's layout_level (one launch per height, root first) and
// layout_emit write the node array, the traversal nodes (exact and grown) and
// the leaf records in the new tree order.
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {

namespace {

constexpr uint32_t kOptNone = 0xFFFFFFFFu;
constexpr float kOptCi = 1.2f;
constexpr int kOptBlock = 256;
constexpr int kOptWarps = kOptBlock / 32;

__device__ __forceinline__ float box_area(float4 mn, float4 mx) {
    const float dx = mx.x - mn.x, dy = mx.y - mn.y, dz = mx.z - mn.z;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

// AABB::merge(a, b) with std::min / std::max semantics; w of a is kept.
__device__ __forceinline__ void box_merge(float4& amn, float4& amx, float4 bmn, float4 bmx) {
    amn.x = min_std(amn.x, bmn.x); amn.y = min_std(amn.y, bmn.y); amn.z = min_std(amn.z, bmn.z);
    amx.x = max_std(amx.x, bmx.x); amx.y = max_std(amx.y, bmx.y); amx.z = max_std(amx.z, bmx.z);
}

__device__ __forceinline__ unsigned long long shfl_xor_u64(unsigned long long v, int m) {
    const uint32_t lo = __shfl_xor_sync(0xFFFFFFFFu, static_cast<uint32_t>(v), m);
    const uint32_t hi = __shfl_xor_sync(0xFFFFFFFFu, static_cast<uint32_t>(v >> 32), m);
    return (static_cast<unsigned long long>(hi) << 32) | lo;
}

// j-th subset (in increasing order) of the bits of mask
__device__ __forceinline__ uint32_t nth_subset(uint32_t j, uint32_t mask) {
    uint32_t q = 0;
    for (uint32_t m = mask; m; m &= m - 1u, j >>= 1)
        if (j & 1u) q |= m & (0u - m);
    return q;
}

// The subsets of 7 treelet leaves with at least 2 members, by size then value.
struct SubsetTable {
    uint8_t s[120];
};
__constant__ SubsetTable c_subsets;
// first table index of the subsets with `size` members (2..8; 8 = the end)
__host__ __device__ constexpr int size_off(int size) {
    return size <= 2 ? 0 : size == 3 ? 21 : size == 4 ? 56 : size == 5 ? 91 : size == 6 ? 112 : size == 7 ? 119 : 120;
}

struct TreeletSmem {
    float u[6][128];  // union box of each subset: min x, y, z, max x, y, z
    float A[128];     // its area
    float C[128];     // its optimal cost
    uint32_t sid[128];  // rebuild: node id of each subset in the new treelet
    float cost1[7];
    uint32_t nl1[7], h1[7];
    uint32_t L[7], I[6];
    uint32_t order[6];  // rebuild: internal subsets in pre-order
    uint32_t n_int;
    uint8_t P[128];     // its best split (the left part)
};

}  // namespace

__global__ void __launch_bounds__(256) opt_init_kernel(const float4* __restrict__ wide, const float4* __restrict__ xtri,
                                                       OptView t, uint32_t* err) {
    const uint32_t k = blockIdx.x * 256 + threadIdx.x;
    const uint32_t N = t.N;
    if (k + 1 >= N) return;
    const float4* w = wide + 4 * static_cast<size_t>(k);
    const float4 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2), w3 = __ldg(w + 3);
    const uint32_t ref[2] = {__float_as_uint(w0.w), __float_as_uint(w1.w)};
    const float4 cmn[2] = {w0, w2}, cmx[2] = {w1, w3};
    uint32_t id[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        if (ref[c] & kLeafRef) {
            const uint32_t l = ref[c] & ~kLeafRef;
            if (l >= N) { raise_corrupt(err, 20, k, ref[c]); return; }
            id[c] = l;
            const uint32_t tri = __float_as_uint(__ldg(xtri + 3 * static_cast<size_t>(l)).w);
            const float4 mn = make_float4(cmn[c].x, cmn[c].y, cmn[c].z, __uint_as_float(tri));
            const float4 mx = make_float4(cmx[c].x, cmx[c].y, cmx[c].z, 0.f);
            t.box[2 * static_cast<size_t>(l)] = mn;
            t.box[2 * static_cast<size_t>(l) + 1] = mx;
            t.cost[l] = box_area(mn, mx);
            t.nl[l] = 1u;
            t.height[l] = 0u;
        } else {
            if (ref[c] == 0u || ref[c] + 1 >= N) { raise_corrupt(err, 20, k, ref[c]); return; }
            id[c] = N + ref[c];
        }
        t.parent[id[c]] = N + k;
    }
    t.kids[k] = make_uint4(id[0], id[1], 0u, 0u);
    if (k == 0) t.parent[N] = kOptNone;
}

// Finish internal node R (uniform over the warp) and, with TREELETS, run its
// treelet step.  Every lane takes part.
template <bool TREELETS>
__device__ __forceinline__ void opt_node(const OptView& t, uint32_t R, TreeletSmem& sm, uint32_t lane, uint32_t* err) {
    const uint32_t N = t.N;
    const uint4 kd = __ldcg(t.kids + (R - N));
    const uint32_t a = kd.x, b = kd.y;
    if (a >= 2 * N - 1 || b >= 2 * N - 1) {
        if (lane == 0) raise_corrupt(err, 21, R, a);
        return;
    }
    float4 mn = __ldcg(t.box + 2 * static_cast<size_t>(a)), mx = __ldcg(t.box + 2 * static_cast<size_t>(a) + 1);
    const float4 bmn = __ldcg(t.box + 2 * static_cast<size_t>(b)), bmx = __ldcg(t.box + 2 * static_cast<size_t>(b) + 1);
    const float area_a = box_area(mn, mx), area_b = box_area(bmn, bmx);
    box_merge(mn, mx, bmn, bmx);
    mn.w = 0.f;
    mx.w = 0.f;
    const uint32_t nla = __ldcg(t.nl + a), nlb = __ldcg(t.nl + b);
    const uint32_t nlR = nla + nlb;
    const uint32_t hR = 1u + max(__ldcg(t.height + a), __ldcg(t.height + b));
    const float costR = kOptCi * box_area(mn, mx) + (__ldcg(t.cost + a) + __ldcg(t.cost + b));
    bool rebuilt = false;
    if (TREELETS && nlR >= 7u) {
        // ---- formation: lane j < n holds treelet leaf j
        uint32_t my = lane == 0 ? a : (lane == 1 ? b : kOptNone);
        float my_area = lane == 0 ? area_a : area_b;  // areas travel with the child ids
        if (lane == 0) sm.I[0] = R;
        bool ok = true;
        for (uint32_t e = 0; e < 5; ++e) {
            const uint32_t n = 2u + e;
            const bool cand = lane < n && my >= N;
            const uint32_t key = cand ? ordered_key(my_area) : 0u;
            const uint32_t kmax = __reduce_max_sync(0xFFFFFFFFu, key);
            const uint32_t win = __ballot_sync(0xFFFFFFFFu, cand && key == kmax);
            if (win == 0u) { ok = false; break; }  // fewer leaves than counted: a corrupt tree
            const uint32_t j = __ffs(win) - 1u;
            const uint32_t X = __shfl_sync(0xFFFFFFFFu, my, j);
            const uint4 xk = __ldcg(t.kids + (X - N));
            const float2 xa = __ldcg(t.karea + (X - N));
            if (lane == 0) sm.I[e + 1] = X;
            if (lane == j || lane == n) {
                my = lane == j ? xk.x : xk.y;
                my_area = lane == j ? xa.x : xa.y;
                if (my >= 2 * N - 1) { raise_corrupt(err, 22, R, my); my = 0u; }
            }
        }
        if (!ok) {
            if (lane == 0) raise_corrupt(err, 23, R, nlR);
        } else {
            if (lane < 7) {
                const uint32_t s1 = 1u << lane;
                const float4 bmn = __ldcg(t.box + 2 * static_cast<size_t>(my));
                const float4 bmx = __ldcg(t.box + 2 * static_cast<size_t>(my) + 1);
                sm.L[lane] = my;
                sm.sid[s1] = my;
                sm.u[0][s1] = bmn.x; sm.u[1][s1] = bmn.y; sm.u[2][s1] = bmn.z;
                sm.u[3][s1] = bmx.x; sm.u[4][s1] = bmx.y; sm.u[5][s1] = bmx.z;
                sm.A[s1] = box_area(bmn, bmx);
                sm.C[s1] = __ldcg(t.cost + my);
                sm.nl1[lane] = __ldcg(t.nl + my);
                sm.h1[lane] = __ldcg(t.height + my);
            }
            __syncwarp();
            // ---- subset unions by highest member: U(s) = merge(U(s - top), box(top)),
            // i.e. the members merged in increasing index
            for (uint32_t top = 1; top < 7; ++top) {
                const uint32_t tb = 1u << top;
                for (uint32_t r = lane + 1; r < tb; r += 32) {
                    const uint32_t sx = tb | r;
                    float4 umn = make_float4(sm.u[0][r], sm.u[1][r], sm.u[2][r], 0.f);
                    float4 umx = make_float4(sm.u[3][r], sm.u[4][r], sm.u[5][r], 0.f);
                    box_merge(umn, umx, make_float4(sm.u[0][tb], sm.u[1][tb], sm.u[2][tb], 0.f),
                              make_float4(sm.u[3][tb], sm.u[4][tb], sm.u[5][tb], 0.f));
                    sm.u[0][sx] = umn.x; sm.u[1][sx] = umn.y; sm.u[2][sx] = umn.z;
                    sm.u[3][sx] = umx.x; sm.u[4][sx] = umx.y; sm.u[5][sx] = umx.z;
                    sm.A[sx] = box_area(umn, umx);
                }
                __syncwarp();
            }
            // ---- dynamic programme, sizes 2..5: one lane per subset; splits in
            // increasing order, so the first strict minimum is the smallest split
            for (int size = 2; size <= 5; ++size) {
                const int off = size_off(size), cnt = size_off(size + 1) - off;
                for (int i = static_cast<int>(lane); i < cnt; i += 32) {
                    const uint32_t sx = c_subsets.s[off + i];
                    const uint32_t low = sx & (0u - sx), rest = sx ^ low;
                    uint32_t bkey = 0xFFFFFFFFu, bp = low;
                    float bv = sm.C[low] + sm.C[sx ^ low];
                    bkey = ordered_key(bv);
                    for (uint32_t q = (0u - rest) & rest; q != rest; q = (q - rest) & rest) {
                        const uint32_t p = low | q;
                        const float v = sm.C[p] + sm.C[sx ^ p];
                        const uint32_t key = ordered_key(v);
                        if (key < bkey) { bkey = key; bp = p; bv = v; }
                    }
                    sm.P[sx] = static_cast<uint8_t>(bp);
                    sm.C[sx] = kOptCi * sm.A[sx] + bv;
                }
                __syncwarp();
            }
            // ---- size 6: 7 subsets x 31 splits, four lanes per subset
            {
                const uint32_t si = lane >> 2, g = lane & 3u;
                unsigned long long best = ~0ull;
                uint32_t sx = 0;
                if (si < 7) {
                    sx = c_subsets.s[size_off(6) + si];
                    const uint32_t low = sx & (0u - sx), rest = sx ^ low;
                    for (uint32_t j = g; j < 31u; j += 4u) {
                        const uint32_t p = low | nth_subset(j, rest);
                        const float v = sm.C[p] + sm.C[sx ^ p];
                        const unsigned long long kv = (static_cast<unsigned long long>(ordered_key(v)) << 32) | p;
                        best = kv < best ? kv : best;
                    }
                }
#pragma unroll
                for (int m = 1; m <= 2; m <<= 1) {
                    const unsigned long long o = shfl_xor_u64(best, m);
                    best = o < best ? o : best;
                }
                if (si < 7 && g == 0) {
                    const uint32_t p = static_cast<uint32_t>(best);
                    sm.P[sx] = static_cast<uint8_t>(p);
                    sm.C[sx] = kOptCi * sm.A[sx] + (sm.C[p] + sm.C[sx ^ p]);
                }
                __syncwarp();
            }
            // ---- size 7: 63 splits over the warp
            {
                unsigned long long best = ~0ull;
                for (uint32_t j = lane; j < 63u; j += 32u) {
                    const uint32_t p = 1u | (j << 1);
                    const float v = sm.C[p] + sm.C[127u ^ p];
                    const unsigned long long kv = (static_cast<unsigned long long>(ordered_key(v)) << 32) | p;
                    best = kv < best ? kv : best;
                }
#pragma unroll
                for (int m = 1; m < 32; m <<= 1) {
                    const unsigned long long o = shfl_xor_u64(best, m);
                    best = o < best ? o : best;
                }
                if (lane == 0) {
                    const uint32_t p = static_cast<uint32_t>(best);
                    sm.P[127] = static_cast<uint8_t>(p);
                    sm.C[127] = kOptCi * sm.A[127] + (sm.C[p] + sm.C[127u ^ p]);
                }
                __syncwarp();
            }
            rebuilt = sm.C[127] < costR;
            // ---- rebuild: the internal subsets take the treelet's ids in
            // pre-order (lane 0), then one lane per internal subset writes its node
            if (rebuilt) {
                if (lane == 0) {
                    uint32_t stack[8];
                    int sp = 0, next = 0;
                    stack[sp++] = 127u;
                    while (sp > 0) {
                        const uint32_t sx = stack[--sp];
                        if (__popc(sx) < 2) continue;
                        if (next >= 6) { raise_corrupt(err, 24, R, sx); break; }
                        sm.sid[sx] = sm.I[next];
                        sm.order[next++] = sx;
                        stack[sp++] = sx ^ sm.P[sx];
                        stack[sp++] = sm.P[sx];
                    }
                    sm.n_int = static_cast<uint32_t>(next);
                }
                __syncwarp();
                if (lane < sm.n_int) {
                    const uint32_t sx = sm.order[lane], p = sm.P[sx], id = sm.sid[sx];
                    const uint32_t ca = sm.sid[p], cb = sm.sid[sx ^ p];
                    // leaf counts add up over members; the height is the deepest member's
                    // height plus the internal subsets on its path (the family is nested)
                    uint32_t nl_p = 0, nl_q = 0, h = 0;
                    for (uint32_t k = 0; k < 7; ++k) {
                        const uint32_t bit = 1u << k;
                        if (!(sx & bit)) continue;
                        if (p & bit) nl_p += sm.nl1[k]; else nl_q += sm.nl1[k];
                        uint32_t depth = 0;
                        for (uint32_t j = 0; j < sm.n_int; ++j) {
                            const uint32_t o = sm.order[j];
                            depth += ((o & bit) && (o & ~sx) == 0u) ? 1u : 0u;
                        }
                        h = max(h, sm.h1[k] + depth);
                    }
                    t.kids[id - N] = make_uint4(ca, cb, nl_p, nl_q);
                    t.karea[id - N] = make_float2(sm.A[p], sm.A[sx ^ p]);
                    t.parent[ca] = id;
                    t.parent[cb] = id;
                    t.box[2 * static_cast<size_t>(id)] = make_float4(sm.u[0][sx], sm.u[1][sx], sm.u[2][sx], 0.f);
                    t.box[2 * static_cast<size_t>(id) + 1] = make_float4(sm.u[3][sx], sm.u[4][sx], sm.u[5][sx], 0.f);
                    t.cost[id] = sm.C[sx];
                    t.nl[id] = nl_p + nl_q;
                    t.height[id] = h;
                }
            }
            __syncwarp();
        }
    }
    if (!rebuilt && lane == 0) {
        t.box[2 * static_cast<size_t>(R)] = mn;
        t.box[2 * static_cast<size_t>(R) + 1] = mx;
        t.cost[R] = costR;
        t.nl[R] = nlR;
        t.height[R] = hR;
        t.kids[R - N] = make_uint4(a, b, nla, nlb);
        t.karea[R - N] = make_float2(area_a, area_b);
    }
}

// Finish internal node R in the calling lane alone when it gets no treelet
// step (fewer than 7 leaves, or treelets off); false leaves it to the warp.
template <bool TREELETS>
__device__ __forceinline__ bool opt_finish_lane(const OptView& t, uint32_t R, uint32_t* err) {
    const uint32_t N = t.N;
    const uint4 kd = __ldcg(t.kids + (R - N));
    const uint32_t a = kd.x, b = kd.y;
    if (a >= 2 * N - 1 || b >= 2 * N - 1) {
        raise_corrupt(err, 21, R, a);
        return true;
    }
    const uint32_t nla = __ldcg(t.nl + a), nlb = __ldcg(t.nl + b);
    if (TREELETS && nla + nlb >= 7u) return false;
    float4 mn = __ldcg(t.box + 2 * static_cast<size_t>(a)), mx = __ldcg(t.box + 2 * static_cast<size_t>(a) + 1);
    const float4 bmn = __ldcg(t.box + 2 * static_cast<size_t>(b)), bmx = __ldcg(t.box + 2 * static_cast<size_t>(b) + 1);
    const float area_a = box_area(mn, mx), area_b = box_area(bmn, bmx);
    box_merge(mn, mx, bmn, bmx);
    mn.w = 0.f;
    mx.w = 0.f;
    t.box[2 * static_cast<size_t>(R)] = mn;
    t.box[2 * static_cast<size_t>(R) + 1] = mx;
    t.cost[R] = kOptCi * box_area(mn, mx) + (__ldcg(t.cost + a) + __ldcg(t.cost + b));
    t.nl[R] = nla + nlb;
    t.height[R] = 1u + max(__ldcg(t.height + a), __ldcg(t.height + b));
    t.kids[R - N] = make_uint4(a, b, nla, nlb);
    t.karea[R - N] = make_float2(area_a, area_b);
    return true;
}

template <bool TREELETS>
__global__ void __launch_bounds__(kOptBlock, 4) opt_pass_kernel(OptView t, uint32_t* err) {
    __shared__ TreeletSmem s_tree[TREELETS ? kOptWarps : 1];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    TreeletSmem& sm = s_tree[TREELETS ? warp : 0];
    const uint32_t N = t.N;
    const uint32_t leaf = blockIdx.x * kOptBlock + threadIdx.x;
    bool active = leaf < N;
    uint32_t cur = leaf;
    // every step takes each active lane one level up: 2N steps bound any tree
    for (uint32_t guard = 0; __any_sync(0xFFFFFFFFu, active); ++guard) {
        if (guard > 2 * N) {
            if (active) raise_corrupt(err, 25, leaf, cur);
            break;
        }
        bool proc = false;
        uint32_t node = 0;
        if (active) {
            node = __ldcg(t.parent + cur);
            if (node == kOptNone) {
                active = false;
            } else if (node < N || node >= 2 * N - 1) {
                raise_corrupt(err, 26, cur, node);
                active = false;
            } else if (atomic_add_acq_rel_u32(t.cnt + (node - N), 1u) == 0u) {
                active = false;  // the sibling's climb finishes the node
            } else {
                proc = true;
            }
        }
        // small nodes: each lane finishes its own (its acquire covers its reads,
        // its next acquire-release atomic releases its writes)
        const bool coop = proc && !opt_finish_lane<TREELETS>(t, node, err);
        uint32_t todo = __ballot_sync(0xFFFFFFFFu, coop);
        if (todo) {
            fence_acq_rel_gpu();  // every lane reads what the acquiring lanes acquired
            while (todo) {
                const uint32_t src = __ffs(todo) - 1u;
                todo &= todo - 1u;
                const uint32_t R = __shfl_sync(0xFFFFFFFFu, node, src);
                opt_node<TREELETS>(t, R, sm, lane, err);
            }
            fence_acq_rel_gpu();  // this warp's writes before any lane's next release
            __syncwarp();
        }
        if (proc) cur = node;
    }
}

// Internal nodes of equal height in a warp count in with one atomic.
__global__ void __launch_bounds__(256) opt_hist_kernel(const uint32_t* __restrict__ height, uint32_t N, uint32_t H,
                                                       uint32_t* __restrict__ hist, uint32_t* err) {
    const uint32_t k = blockIdx.x * 256 + threadIdx.x;
    uint32_t h = k + 1 < N ? __ldg(height + N + k) : 0u;
    if (k + 1 < N && (h == 0u || h > H)) {
        raise_corrupt(err, 27, k, h);
        h = 0u;
    }
    const uint32_t valid = __ballot_sync(0xFFFFFFFFu, h != 0u);
    if (h == 0u) return;
    const uint32_t peers = __match_any_sync(valid, h);
    if ((threadIdx.x & 31u) == static_cast<uint32_t>(__ffs(peers) - 1)) atomicAdd(hist + h, __popc(peers));
}

// cursor: exclusive offsets per height on entry; a warp's nodes of one height
// take consecutive slots with one atomic.
__global__ void __launch_bounds__(256) opt_relabel_kernel(const uint32_t* __restrict__ height, uint32_t N, uint32_t H,
                                                          uint32_t* __restrict__ cursor, uint32_t* __restrict__ newid) {
    const uint32_t k = blockIdx.x * 256 + threadIdx.x;
    uint32_t h = k + 1 < N ? __ldg(height + N + k) : 0u;
    if (h > H) h = 0u;
    const uint32_t valid = __ballot_sync(0xFFFFFFFFu, h != 0u);
    if (h == 0u) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t peers = __match_any_sync(valid, h);
    const uint32_t leader = __ffs(peers) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cursor + h, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    newid[k] = N + base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(256) opt_remap_kernel(const OptView t, const uint32_t* __restrict__ newid,
                                                        uint4* __restrict__ kids2, float4* __restrict__ box2,
                                                        uint32_t* err) {
    const uint32_t id = blockIdx.x * 256 + threadIdx.x;
    const uint32_t N = t.N;
    if (id >= 2 * N - 1) return;
    const float4 mn = __ldg(t.box + 2 * static_cast<size_t>(id)), mx = __ldg(t.box + 2 * static_cast<size_t>(id) + 1);
    if (id < N) {
        box2[2 * static_cast<size_t>(id)] = mn;
        box2[2 * static_cast<size_t>(id) + 1] = mx;
        return;
    }
    const uint32_t nid = __ldg(newid + (id - N));
    if (nid < N || nid >= 2 * N - 1) { raise_corrupt(err, 28, id, nid); return; }
    uint4 k = __ldg(t.kids + (id - N));
    if (k.x >= 2 * N - 1 || k.y >= 2 * N - 1) { raise_corrupt(err, 28, id, k.x); return; }
    if (k.x >= N) k.x = __ldg(newid + (k.x - N));
    if (k.y >= N) k.y = __ldg(newid + (k.y - N));
    kids2[nid - N] = k;
    box2[2 * static_cast<size_t>(nid)] = mn;
    box2[2 * static_cast<size_t>(nid) + 1] = mx;
}

void opt_init_subsets() {
    static bool done = false;
    if (done) return;
    SubsetTable tab{};
    int o = 0;
    for (int size = 2; size <= 7; ++size)
        for (uint32_t s = 1; s < 128; ++s)
            if (__builtin_popcount(s) == size) tab.s[o++] = static_cast<uint8_t>(s);
    cudaMemcpyToSymbol(c_subsets, &tab, sizeof(tab));
    done = true;
}

void launch_opt_init(const float4* wide, const float4* xtri, const OptView& t, uint32_t* err, cudaStream_t s) {
    opt_init_subsets();
    if (t.N < 2) return;
    opt_init_kernel<<<(t.N - 1 + 255) / 256, 256, 0, s>>>(wide, xtri, t, err);
}

void launch_opt_pass(const OptView& t, bool treelets, uint32_t* err, cudaStream_t s) {
    if (t.N < 2) return;
    cudaMemsetAsync(t.cnt, 0, 4ull * (t.N - 1), s);
    const uint32_t blocks = (t.N + kOptBlock - 1) / kOptBlock;
    if (treelets) opt_pass_kernel<true><<<blocks, kOptBlock, 0, s>>>(t, err);
    else opt_pass_kernel<false><<<blocks, kOptBlock, 0, s>>>(t, err);
}

void launch_opt_hist(const OptView& t, uint32_t H, uint32_t* hist, uint32_t* err, cudaStream_t s) {
    if (t.N < 2) return;
    opt_hist_kernel<<<(t.N - 1 + 255) / 256, 256, 0, s>>>(t.height, t.N, H, hist, err);
}

void launch_opt_relabel(const OptView& t, uint32_t H, uint32_t* cursor, uint32_t* newid, uint4* kids2, float4* box2,
                        uint32_t* err, cudaStream_t s) {
    if (t.N < 2) return;
    opt_relabel_kernel<<<(t.N - 1 + 255) / 256, 256, 0, s>>>(t.height, t.N, H, cursor, newid);
    opt_remap_kernel<<<(2 * t.N - 1 + 255) / 256, 256, 0, s>>>(t, newid, kids2, box2, err);
}

}  // namespace crt
