// Internal interface between the build kernels (crt_build.cu), the refit
// (crt_refit.cu), the trace and frame kernels (crt_trace.cu, crt_frame.cu)
// and the C ABI (crt_api.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <string>

#include "crt.h"
#include "crt_predictor.cuh"

namespace crt {

// A PLOC tile: one 256-thread block finds the nearest neighbours of
// kPlocSpan consecutive positions (4 per thread) and decides the merges of
// the ploc_own(R) = kPlocSpan - 2R positions in their middle.
constexpr uint32_t kPlocSpan = 1024;
constexpr int kPlocMaxRadius = 32;        // largest supported PLOC radius
// Co-resident blocks per SM of the persistent (cooperative) PLOC launches.
constexpr int kPlocBlocksPerSm = 3;
// One-wave PLOC iterations search one (two) positions per thread once those
// smaller tiles number at most this many per SM (all co-resident).
constexpr uint32_t kPlocSmallTiles1 = 3;  // measured best of 1-3 (1.31 M build: PLOC 0.72 -> 0.67 ms)
constexpr uint32_t kPlocSmallTiles2 = 3;
static_assert(kPlocSmallTiles1 <= kPlocBlocksPerSm && kPlocSmallTiles2 <= kPlocBlocksPerSm, "co-resident tiles");
constexpr uint32_t kPlocMinOwn = kPlocSpan - 2u * kPlocMaxRadius;  // sizes look-back arrays for any radius
__host__ __device__ constexpr uint32_t ploc_own(int radius) { return kPlocSpan - 2u * static_cast<uint32_t>(radius); }
constexpr uint32_t kLeafRef = 0x80000000u;  // traversal child reference: leaf flag | sorted position
constexpr uint32_t kNoChild = 0xFFFFFFFFu;  // empty slot of a 4-wide node

// Scene box reduction state (device memory, zeroed keys at creation; the
// finishing block resets it) and its results for the Morton pass.
struct SceneState {
    unsigned long long key_max[3];
    unsigned long long key_min[3];
    unsigned int blocks_done;
    unsigned int pad;
    float scene_min[3];
    float scene_max[3];
    float cube_min[3];
    float cube_len[3];
    float abs_eps;  // traversal slack of the scene, scene_abs_eps(scene_min, scene_max)
};

// Absolute slack of traversal pruning and of the watertight box growth:
// 2^-20 of the largest finite extent or coordinate magnitude of the scene box.
__host__ __device__ inline float scene_abs_eps(const float* smin, const float* smax) {
    float ext = 0.f;
    for (int a = 0; a < 3; ++a) {
        const float e = smax[a] - smin[a];
        if (isfinite(e) && e > ext) ext = e;
        const float m = fmaxf(fabsf(smin[a]), fabsf(smax[a]));
        if (isfinite(m) && m > ext) ext = m;
    }
    return ldexpf(ext > 0.f ? ext : 1.f, -20);
}

void launch_scene_box(const crt_triangle* tris, uint32_t n_buffer, const float* models, SceneState* st, uint32_t* err,
                      cudaStream_t s);
void launch_morton(const crt_triangle* tris, uint32_t n, const float* models_third, const SceneState* st,
                   uint32_t* codes, uint32_t* hist, int bits, cudaStream_t s);
uint32_t sort_tile_keys(int bits);
// The sort's counting step (digit histograms of 32-bit keys, bits in {1, 2,
// 4, 8}: counts[p * 2^bits + d], counts zeroed by the caller) and its
// digit-offset step (per place, exclusive scan over its 2^bits counts), for
// the known-answer tests of the reference's sort shaders.  False on an
// unsupported width.
bool launch_digit_counts(const uint32_t* keys, uint32_t n, int bits, uint32_t* counts, cudaStream_t s);
bool launch_digit_offsets(const uint32_t* counts, uint32_t places, int bits, uint32_t* offsets, cudaStream_t s);
void launch_onesweep(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, uint32_t n,
                     int shift, int bits, const uint32_t* pass_hist, uint32_t* lookback, uint32_t* ticket, uint32_t* err,
                     uint32_t spin_limit, cudaStream_t s);
// One stable pass whose digit is the segment holding each value (n_seg <= 256).
void launch_onesweep_segments(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                              uint32_t n, const uint32_t* seg_off, uint32_t n_seg, const uint32_t* seg_hist,
                              uint32_t* lookback, uint32_t* ticket, uint32_t* err, uint32_t spin_limit, cudaStream_t s);
// xtri_sorted: the leaves' transformed triangles in sorted (Morton) order;
// the layout moves them into tree order.
void launch_leaf_init(const crt_triangle* tris, uint32_t n, const float* models, const uint32_t* perm, float4* node_box,
                      float4* clusters, float4* xtri_sorted, uint2* it, uint32_t* err, cudaStream_t s);
void launch_ploc_iteration(const float4* cin, float4* cout, float4* node_box, uint4* node_kids, uint2* it,
                           int iter, uint32_t N, int radius, uint32_t n_upper,
                           unsigned long long* lookback, uint32_t* tickets, uint32_t n_tiles_cap, uint32_t* err,
                           uint32_t spin_limit, cudaStream_t s);
// Leaf records moved by the layout: leaf L (sorted position) goes to its
// position in the tree's left-to-right (DFS) leaf order, leaf_of_tri
// receives triangle -> that position.
struct LeafOut {
    const float4* xtri_sorted;
    float4* xtri;
    uint32_t* leaf_of_tri;
};
// DFS layout as separate launches: one top-down level (nodes [id_begin,
// id_end)) recording dfs[position] = node, then the emit pass over all
// positions.
void launch_layout_level(const uint4* node_kids, uint2* pf, uint32_t id_begin,
                         uint32_t id_end, uint32_t N, uint32_t* dfs, uint32_t* err, cudaStream_t s);
void launch_layout_emit(const float4* node_box, const uint4* node_kids, const uint2* pf, uint32_t N,
                        const uint32_t* dfs, crt_bvh_node* out, float4* wide, float4* wide_wt, uint8_t* depth_odd,
                        LeafOut leaves, const SceneState* st, uint32_t* err, cudaStream_t s);
void launch_wide4(const float4* wide, const uint8_t* depth_odd, uint32_t n_internal, float4* wide4, cudaStream_t s);
// 64-byte compressed 4-wide nodes (CRT_TRACE_COMPRESSED) from the binary
// traversal nodes; raises kDevCorrupt where a box cannot be quantized
// (non-finite coordinates).
void launch_cwide(const float4* wide, const uint8_t* depth_odd, uint32_t n_internal, uint4* cwide, uint32_t* err,
                  cudaStream_t s);
void launch_single_leaf(const float4* node_box, crt_bvh_node* out, LeafOut leaves, cudaStream_t s);
// All PLOC iterations and the DFS layout in one cooperative launch; returns
// cudaErrorNotSupported when a cooperative launch is unavailable.
cudaError_t launch_ploc_persistent(float4* ca, float4* cb, float4* node_box, uint4* node_kids, uint2* it, uint32_t N,
                                   int radius, unsigned long long* lookback, uint32_t* tickets, uint32_t n_tiles_cap,
                                   uint2* pf, crt_bvh_node* out, float4* wide, float4* wide_wt, uint8_t* depth_odd,
                                   LeafOut leaves, const SceneState* st, unsigned long long* bar, uint32_t* iters_out,
                                   uint32_t* err, uint32_t spin_limit, cudaStream_t s);

// Refit (crt_refit.cu).  The slack of the refit tree's root box goes to
// abs_eps for the host.
struct RefitState {
    float abs_eps;
    unsigned int pad[3];
};
uint32_t refit_topo_blocks(uint32_t N);
// Once per build: links to the parent (parent's rank << 1 | child slot,
// parent's leaf range [first, end)) for every leaf (leaf_link, by place in
// the tree's leaf order, N entries) and internal node (int_link, by rank,
// N - 1 entries), and every internal node's DFS position (int_dfs).
// block_count: refit_topo_blocks(N) words of scratch.
void launch_refit_topology(const crt_bvh_node* nodes, const float4* wide, uint32_t N, uint4* leaf_link, uint4* int_link,
                           uint32_t* int_dfs, uint32_t* block_count, uint32_t* err, cudaStream_t s);
// New leaf records, both traversal node arrays and the root box of the node
// array; cnt (N - 1 words) zeroed before.
void launch_refit(const crt_triangle* tris, uint32_t N, const float* models, const uint4* leaf_link,
                  const uint4* int_link, uint32_t* cnt, crt_bvh_node* nodes, float4* xtri, float4* wide,
                  float4* wide_wt, RefitState* st, uint32_t* err, cudaStream_t s);
// The other boxes of the node array, from the traversal nodes.
void launch_refit_nodes(const float4* wide, const uint32_t* int_dfs, uint32_t N, crt_bvh_node* nodes, uint32_t* err,
                        cudaStream_t s);

// Trace side (crt_trace.cu).
struct TraceParams {
    const crt_bvh_node* nodes;  // reference layout (root box read from nodes[0])
    const float4* wide;      // 64-B traversal nodes: child boxes + child references (watertight
                             // traces: boxes already grown by abs_eps)
    const float4* wide4;     // 128-B 4-wide traversal nodes (even-depth internal nodes)
    const uint4* cwide = nullptr;  // 64-B compressed 4-wide traversal nodes (same indices)
    const float4* xtri;      // 3 float4 per leaf (tree order): transformed p0 | tri id, p1 | model id, p2
    const crt_ray* rays;
    crt_hit* hits;
    uint32_t n_rays;
    uint32_t n_nodes;
    float abs_eps;           // absolute slack of pruning, from the scene extent
    uint32_t* err;
    uint32_t tile_width = 0;    // image width when rays are pixels (multiple of 8, height multiple of 4)
    unsigned long long* stats;  // optional: nodes visited, triangles tested
    // learned seeding (CRT_TRACE_USE_PREDICTOR): per-ray predicted treelet
    const uint16_t* pred_class = nullptr;
    const Treelet* treelets = nullptr;
    const uint32_t* n_treelets = nullptr;
    // optional order of the rays (thread t traces ray order[t]), e.g. grouped
    // by predicted treelet (CRT_TRACE_PREDICTOR_ORDER)
    const uint32_t* order = nullptr;
};
void launch_trace(const TraceParams& p, uint32_t flags, int block, cudaStream_t s);
// Closest hit of many rays by persistent warps that refill finished lanes from
// a ray counter (next_ray: one device word, reset here); binary nodes, no
// seeding, rays in caller order or p.order.
void launch_trace_pool(const TraceParams& p, uint32_t flags, uint32_t* next_ray, cudaStream_t s);

// Shading (getColor + imageStore) inputs; the BVH, leaf records and error
// word come from the TraceParams it runs with.
constexpr uint32_t kShadeMaxDepth = 64;   // display-walk stack: CRT_SHADE_MAX_BVH_DEPTH + 1
struct ShadeParams {
    const uint32_t* models = nullptr;     // crt_mesh_model records as 32-bit words, 17 per model (word 16: material id)
    uint32_t n_models = 0;
    const float4* materials = nullptr;    // crt_material colours
    uint32_t n_materials = 0;
    uint32_t flags = 0;                   // CRT_SHADE_*
    uint32_t bvh_depth = 0;
    const uint32_t* inv_perm = nullptr;   // triangle -> leaf position in tree order (its xtri record holds the model id)
    uint32_t n_tris = 0;
    float4* image = nullptr;              // RGBA32F texels
};
// Texels of p.n_rays hits p.hits of rays p.rays (rays read with CRT_SHADE_BVH only).
void launch_shade(const TraceParams& p, const ShadeParams& sp, cudaStream_t s);

// Camera rays of image rows [y0, y0 + rows) traced to the closest hit into
// p.hits (may be null with shading) and, with a light, their shadow rays to
// any hit into hits_shadow, and with shade, their texels into shade->image,
// in one launch (p.tile_width: width for 8x4 pixel tiles, or 0).
void launch_frame(const TraceParams& p, const crt_camera* cam, uint32_t width, uint32_t height, uint32_t y0,
                  uint32_t rows, const float* light, crt_hit* hits_shadow, uint32_t flags, int block,
                  const ShadeParams* shade, cudaStream_t s);

// Batched scenes: per-scene offsets into the concatenated arrays.
constexpr uint32_t kMaxBatchScenes = 256;
struct BatchScene {
    uint32_t tri_off;     // first triangle / leaf / cluster of the scene
    uint32_t n_tris;
    uint32_t node_off;    // 2 * tri_off - scene index: first reference-layout node
    uint32_t wide_off;    // tri_off - scene index: first binary traversal node
    uint32_t ray_off;
    uint32_t n_rays;
    uint32_t it_off;      // tri_off + 2 * scene index: first PLOC iteration record
    uint32_t lb_off;      // first PLOC look-back word (per parity)
    float abs_eps;
    uint32_t iters;       // PLOC iterations (0 while running)
    uint32_t n_chunks;    // scene-box chunks of the scene
    uint32_t pad;
};
static_assert(sizeof(BatchScene) == 48, "batch scene record");
void launch_trace_batch(const TraceParams& p, const BatchScene* scenes, uint32_t n_scenes, uint32_t n_rays,
                        uint32_t flags, int block, bool deep, cudaStream_t s);
// The persistent ray pool over a batch: closest hit, no seeding; p holds the
// batch's node arrays and p.n_rays the batch's ray count.
void launch_trace_batch_pool(const TraceParams& p, const BatchScene* scenes, uint32_t n_scenes, uint32_t flags,
                             bool deep, uint32_t* next_ray, cudaStream_t s);
// CRT_TRACE_SORT_RAYS: order[k] = k-th ray by coherence key (origin cell,
// direction; with scenes, scene first).  scratch: ray_order_scratch_bytes(n).
size_t ray_order_scratch_bytes(uint32_t n);
void launch_ray_order(const crt_ray* rays, uint32_t n, const crt_bvh_node* nodes, const BatchScene* scenes,
                      uint32_t n_scenes, uint32_t* order, void* scratch, uint32_t* err, uint32_t spin_limit,
                      cudaStream_t s);
// Batched build stages (crt_batch_kernels.cuh).
size_t batch_box_state_bytes();
size_t batch_chunk_bytes();
uint32_t batch_box_chunk();
void launch_batch_box(const crt_triangle* tris, const void* chunks, uint32_t n_chunks, const float* models, void* states,
                      BatchScene* scenes, uint32_t* err, cudaStream_t s);
void launch_batch_morton(const crt_triangle* tris, const void* chunks, uint32_t n_chunks, const float* models_third,
                         const void* states, uint32_t* codes, uint32_t* hist, int bits, cudaStream_t s);
void launch_batch_leaf_init(const crt_triangle* tris, uint32_t n_total, BatchScene* scenes, uint32_t n_scenes,
                            const float* models, const uint32_t* perm_global, uint32_t* perm_local, float4* node_box,
                            float4* clusters, float4* xtri_sorted, float4* xtri, uint32_t* leaf_of_tri, uint2* it,
                            crt_bvh_node* nodes, uint32_t* err, cudaStream_t s);
cudaError_t launch_batch_ploc(BatchScene* scenes, uint32_t n_scenes, float4* ca, float4* cb, float4* node_box,
                              uint4* node_kids, uint2* it, int radius, unsigned long long* lookback, uint32_t lb_cap,
                              uint32_t* tickets, uint2* pf, crt_bvh_node* nodes, float4* wide, float4* wide_wt,
                              uint8_t* depth_odd, LeafOut leaves, unsigned long long* bar, uint32_t max_iters, uint32_t* err,
                              uint32_t spin_limit, cudaStream_t s);
// Treelet restructuring (crt_optimize.cu).  Ids: leaves 0..N-1 in tree
// leaf order, internal nodes N + DFS rank (root N).
struct OptView {
    float4* box;  // 2 per id: (min | triangle id for leaves), (max | 0)
    float* cost;
    uint32_t* nl;      // leaves below
    uint32_t* height;  // leaves 0
    uint32_t* parent;
    uint4* kids;  // per internal node: left id, right id, leaves(left), leaves(right)
    float2* karea;  // per internal node: its children's box areas
    uint32_t* cnt;
    uint32_t N;
};
void launch_opt_init(const float4* wide, const float4* xtri, const OptView& t, uint32_t* err, cudaStream_t s);
// One bottom-up pass: every internal node's box, cost, leaf count and height;
// with treelets, the treelet step at nodes with at least 7 leaves.
void launch_opt_pass(const OptView& t, bool treelets, uint32_t* err, cudaStream_t s);
// hist[h] += internal nodes of height h (1 <= h <= H)
void launch_opt_hist(const OptView& t, uint32_t H, uint32_t* hist, uint32_t* err, cudaStream_t s);
// cursor: exclusive offsets per height; new ids N + offset (root last), then
// children and boxes (leaves too) moved to kids2 / box2 under the new ids.
void launch_opt_relabel(const OptView& t, uint32_t H, uint32_t* cursor, uint32_t* newid, uint4* kids2, float4* box2,
                        uint32_t* err, cudaStream_t s);
// A BVH from a caller's DFS node array (crt_import.cu): idx[d] = leaf index
// or internal rank of position d; int_pos[k] = position of internal rank k;
// leaf_counts[k] = leaves under its children; leaf_pos[l] = position of leaf l.
void launch_import(const crt_bvh_node* nodes, uint32_t N, const uint32_t* idx, const uint32_t* int_pos,
                   const uint2* leaf_counts, const uint32_t* leaf_pos, const crt_triangle* tris, const float* models,
                   float grow, float4* wide, float4* wide_wt, float4* xtri, uint32_t* leaf_of_tri, uint32_t* err,
                   cudaStream_t s);
// Mesh input (crt_mesh.cu).  obj_parse reads OBJ text into at most vert_cap
// vertices (3 floats each) and tri_cap triangles (3 vertex indices each) —
// either may be null to count only — and returns the full counts, or false
// with *error set.
bool obj_parse(const char* text, size_t len, float* vertices, uint64_t vert_cap, uint32_t* indices, uint64_t tri_cap,
               uint64_t* n_vertices, uint64_t* n_triangles, std::string* error);
// TriangleGPU records of an indexed mesh (vertices: 3 floats each).
void launch_indexed(const float* vertices, uint32_t n_vertices, const uint32_t* indices, uint32_t n_triangles,
                    uint32_t model_id, crt_triangle* out, uint32_t* err, cudaStream_t s);

// One bounded wait on *flag (crt_selftest_wait); a timeout sets kDevTimeout.
void launch_wait_probe(const unsigned int* flag, uint32_t spin_limit, uint32_t* err, cudaStream_t s);

// Sets the message crt_last_error_string() returns on the calling thread.
void set_last_error(const char* msg);

void launch_raygen(const crt_camera* cam_dev, uint32_t width, uint32_t height, crt_ray* rays, cudaStream_t s);
void launch_shadow_rays(const crt_ray* prim, const crt_hit* hits, uint32_t n, float lx, float ly, float lz, crt_ray* out,
                        cudaStream_t s);

}  // namespace crt
