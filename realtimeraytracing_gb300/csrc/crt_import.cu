// A BVH from a node array the caller already has (crt_bvh_from_nodes): the
// reference's own SSBO content — Scene::getBVH_NodesToGPUData's DFS
// pre-order BVH_NodeGPU array (srcOpenGL/scene/scene.cpp:189-208), which
// raytracer.glsl reads from binding 5 — plus the triangles it indexes.  The
// host checks the array's structure and numbers its nodes; these kernels
// derive the traversal's own records from it, as the build's layout pass does
// for a tree it made:
//   import_wide    one thread per internal node (rank in DFS order): both
//                  children's boxes as the array holds them, their references
//                  (leaf: its place in the left-to-right leaf order; internal:
//                  its rank) and leaf counts, once exact and once with every
//                  box grown by the tree's slack (watertight traces);
//   import_leaves  one thread per leaf (left-to-right order): its triangle
//                  transformed by its model matrix (glm mat4 * vec4 order, as
//                  the build's leaf pass) and the triangle -> leaf map.
// Compiled with -fmad=false.
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {

__device__ __forceinline__ bool import_is_leaf(const crt_bvh_node* nodes, uint32_t d) {
    const uint4 k = __ldg(reinterpret_cast<const uint4*>(nodes + d) + 2);  // tri, left, right, pad
    return (k.y | k.z) == 0u;
}

__global__ void __launch_bounds__(256) import_wide_kernel(const crt_bvh_node* __restrict__ nodes, uint32_t n_nodes,
                                                          const uint32_t* __restrict__ idx,
                                                          const uint32_t* __restrict__ int_pos,
                                                          const uint2* __restrict__ leaf_counts, uint32_t N, float grow,
                                                          float4* __restrict__ wide, float4* __restrict__ wide_wt,
                                                          uint32_t* err) {
    const uint32_t k = blockIdx.x * 256 + threadIdx.x;
    if (k + 1 >= N) return;
    const uint32_t d = __ldg(int_pos + k);
    if (d + 1 >= n_nodes) { raise_corrupt(err, 30, k, d); return; }
    const uint4 kd = __ldg(reinterpret_cast<const uint4*>(nodes + d) + 2);
    const uint32_t ch[2] = {kd.y, kd.z};
    float4 cmn[2], cmx[2];
    uint32_t ref[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        if (ch[c] >= n_nodes) { raise_corrupt(err, 30, k, ch[c]); return; }
        const float4* q = reinterpret_cast<const float4*>(nodes + ch[c]);
        cmn[c] = __ldg(q);
        cmx[c] = __ldg(q + 1);
        const uint32_t i = __ldg(idx + ch[c]);
        ref[c] = import_is_leaf(nodes, ch[c]) ? (kLeafRef | i) : i;
    }
    const uint2 lc = __ldg(leaf_counts + k);
    float4* w = wide + 4 * static_cast<size_t>(k);
    w[0] = make_float4(cmn[0].x, cmn[0].y, cmn[0].z, __uint_as_float(ref[0]));
    w[1] = make_float4(cmx[0].x, cmx[0].y, cmx[0].z, __uint_as_float(ref[1]));
    w[2] = make_float4(cmn[1].x, cmn[1].y, cmn[1].z, __uint_as_float(lc.x));
    w[3] = make_float4(cmx[1].x, cmx[1].y, cmx[1].z, __uint_as_float(lc.y));
    float4* g = wide_wt + 4 * static_cast<size_t>(k);
    g[0] = make_float4(cmn[0].x - grow, cmn[0].y - grow, cmn[0].z - grow, __uint_as_float(ref[0]));
    g[1] = make_float4(cmx[0].x + grow, cmx[0].y + grow, cmx[0].z + grow, __uint_as_float(ref[1]));
    g[2] = make_float4(cmn[1].x - grow, cmn[1].y - grow, cmn[1].z - grow, __uint_as_float(lc.x));
    g[3] = make_float4(cmx[1].x + grow, cmx[1].y + grow, cmx[1].z + grow, __uint_as_float(lc.y));
}

__global__ void __launch_bounds__(256) import_leaves_kernel(const crt_bvh_node* __restrict__ nodes, uint32_t n_nodes,
                                                            const uint32_t* __restrict__ leaf_pos,
                                                            const crt_triangle* __restrict__ tris,
                                                            const float* __restrict__ models, uint32_t N,
                                                            float4* __restrict__ xtri, uint32_t* __restrict__ leaf_of_tri,
                                                            uint32_t* err) {
    const uint32_t l = blockIdx.x * 256 + threadIdx.x;
    if (l >= N) return;
    const uint32_t d = __ldg(leaf_pos + l);
    if (d >= n_nodes) { raise_corrupt(err, 31, l, d); return; }
    const uint32_t ti = __ldg(reinterpret_cast<const uint32_t*>(nodes + d) + 8);  // _TriangleId
    if (ti >= N) { raise_corrupt(err, 31, l, ti); return; }
    const TriRec t = load_tri(tris, ti);
    if (t.model >= kMaxModels) raise_error(err, kDevBadModel);
    const float* M = models + 16 * (t.model & (kMaxModels - 1));
    const float4 p0 = mat_vec(M, t.p0), p1 = mat_vec(M, t.p1), p2 = mat_vec(M, t.p2);
    xtri[3 * static_cast<size_t>(l) + 0] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(ti));
    xtri[3 * static_cast<size_t>(l) + 1] = make_float4(p1.x, p1.y, p1.z, __uint_as_float(t.model));
    xtri[3 * static_cast<size_t>(l) + 2] = make_float4(p2.x, p2.y, p2.z, 0.f);
    leaf_of_tri[ti] = l;
}

void launch_import(const crt_bvh_node* nodes, uint32_t N, const uint32_t* idx, const uint32_t* int_pos,
                   const uint2* leaf_counts, const uint32_t* leaf_pos, const crt_triangle* tris, const float* models,
                   float grow, float4* wide, float4* wide_wt, float4* xtri, uint32_t* leaf_of_tri, uint32_t* err,
                   cudaStream_t s) {
    const uint32_t n_nodes = 2 * N - 1;
    if (N > 1)
        import_wide_kernel<<<(N - 1 + 255) / 256, 256, 0, s>>>(nodes, n_nodes, idx, int_pos, leaf_counts, N, grow, wide,
                                                               wide_wt, err);
    import_leaves_kernel<<<(N + 255) / 256, 256, 0, s>>>(nodes, n_nodes, leaf_pos, tris, models, N, xtri, leaf_of_tri,
                                                         err);
}

}  // namespace crt
