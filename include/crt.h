/*
 * crt.h — C ABI of the GB300 ray-tracing core (libcrt.so).
 *
 * The library replaces one data-parallel path of MrBigoudi/RealTimeRaytracing:
 * the BVH build that Scene::bindSSBO runs on the CPU
 *     cr::BVH::BVH(nbTriangles, unsortedTriangles, meshesInTheScene)
 *         srcCommon/scene/geometry/bvh.hpp:89-91, bvh.cpp:11-24
 *     called at srcOpenGL/scene/scene.cpp:148, flattened at scene.cpp:189-208
 * and the closest-hit traversal the compute shader runs per pixel
 *     glDispatchCompute(W/16, H/16, 1)       srcOpenGL/application.cpp:245
 *     raytracer.glsl main / getRay / getClosestHitBVH / rayTriangleIntersection
 *         srcCommon/shaders/raytracer.glsl:92-147, 182-295, 299-331
 * Every stage runs as hand-written CUDA kernels for sm_103a on one GPU.
 *
 * Conventions
 *   - Plain pointers and sizes only.  The single-scene calls accept each
 *     pointer in host or device memory; the library checks with
 *     cudaPointerGetAttributes and copies host data in and out on the
 *     context's stream.  The batched calls (crt_batch_*) and
 *     crt_morton_sort_noalloc take device memory for their triangles, rays,
 *     hits and outputs and refuse host pointers (CRT_ERR_INVALID_ARG).
 *   - Calls are ordered on the context's stream.  Functions that return data
 *     to host memory synchronise that stream before returning.
 *   - Errors come back as crt_status; crt_last_error_string() describes the
 *     last failure on the calling thread.  Nothing here calls exit().
 *   - One context per host thread.  A context owns its device buffers; a
 *     crt_bvh owns the node array until crt_bvh_free.
 */
#ifndef CRT_H
#define CRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CRT_ABI_VERSION 1u

typedef enum crt_status {
    CRT_OK = 0,
    CRT_ERR_INVALID_ARG = 1,      /* bad pointer, size or flag */
    CRT_ERR_OOM = 2,              /* device allocation failed */
    CRT_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    CRT_ERR_DEVICE_TIMEOUT = 4,   /* a bounded device-side wait gave up */
    CRT_ERR_STACK_OVERFLOW = 5,   /* a ray's traversal stack overflowed */
    CRT_ERR_UNSUPPORTED = 6,      /* no sm_103a device, or feature absent */
    CRT_ERR_BAD_INPUT = 7         /* input data the path cannot handle (e.g. model id >= 64) */
} crt_status;

/* cr::TriangleGPU (srcCommon/scene/geometry/triangle.hpp:9-14): three vec4
 * vertices (w = 1) and a model index, 64 bytes.  Note: the GLSL mirror of this
 * struct names the 2nd and 3rd vec4 _P2 and _P1 (raytracer.glsl:20-25). */
typedef struct crt_triangle {
    float p0[4];
    float p1[4];
    float p2[4];
    uint32_t model_id;
    uint32_t pad[3];
} crt_triangle;

/* cr::MeshModelGPU (srcCommon/scene/geometry/mesh.hpp:12-15): a column-major
 * 4x4 model matrix and a material id, 68 bytes. */
typedef struct crt_mesh_model {
    float m[16];
    uint32_t material_id;
} crt_mesh_model;

/* cr::BVH_NodeGPU (srcCommon/scene/geometry/bvh.hpp:22-26, 36-42), 48 bytes:
 * a leaf has left == right == 0 and tri = triangle index; an internal node
 * has tri = 0.  The node array is in DFS pre-order, left subtree first, root
 * at index 0 (srcOpenGL/scene/scene.cpp:189-208). */
typedef struct crt_bvh_node {
    float mn[3];
    float pad0;
    float mx[3];
    float pad1;
    uint32_t tri;
    uint32_t left;
    uint32_t right;
    uint32_t pad2;
} crt_bvh_node;

/* A ray (raytracer.glsl:15-18 carries origin/direction as vec4 with w = 1/0).
 * Hits are accepted for tmin <= t <= tmax; primary rays use [0, +inf]. */
typedef struct crt_ray {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} crt_ray;

/* Result of a trace.  tri == CRT_MISS on a miss.  For closest-hit, t is the
 * hit distance in units of |d|; (u, v) are the reference predicate's
 * (_Coords.x, _Coords.y) or the watertight predicate's weights of p1 and p2.
 * For any-hit, tri is the id of some occluder (which one is unspecified). */
typedef struct crt_hit {
    uint32_t tri;
    float t;
    float u;
    float v;
} crt_hit;
#define CRT_MISS 0xFFFFFFFFu

/* The part of cr::CameraGPU (srcCommon/scene/camera.hpp:21-30) that getRay
 * reads (raytracer.glsl:92-100): column-major inverse view matrix, eye
 * position (w = 1) and the image-plane size. */
typedef struct crt_camera {
    float inv_view[16];
    float eye[4];
    float plane_width;
    float plane_height;
    float plane_near;
    float pad;
} crt_camera;

/* Trace flags. */
#define CRT_TRACE_CLOSEST     0x0u  /* closest hit */
#define CRT_TRACE_ANY         0x1u  /* any hit (shadow rays); stops at the first */
#define CRT_TRI_REFERENCE     0x0u  /* raytracer.glsl:102-147 predicate, bit for bit */
#define CRT_TRI_WATERTIGHT    0x2u  /* Woop/Benthin/Wald 2013 watertight predicate, two-sided */
#define CRT_TRACE_USE_PREDICTOR 0x4u /* seed t_max from the learned hit predictor */
#define CRT_TRACE_STATS       0x8u  /* count visited nodes / tested triangles (slower) */
#define CRT_TRACE_WIDE        0x10u /* walk the 4-wide nodes instead of the binary ones (same hits) */
#define CRT_TRACE_PREDICTOR_ORDER 0x20u /* trace the rays grouped by the predictor's likeliest class (a treelet,
                                           or miss) (same hits) */
#define CRT_TRACE_SORT_RAYS   0x40u /* trace the rays ordered by origin cell and direction (same hits) */
#define CRT_TRACE_COMPRESSED  0x80u /* walk 64-byte compressed 4-wide nodes: 8-bit child boxes rounded
                                       outward, exact leaf boxes re-checked (same hits); the reference
                                       layout stays the export format */
#define CRT_TRACE_PER_RAY_THREADS 0x100u /* closest-hit crt_trace of >= 65,536 rays normally runs on
                                       persistent warps whose lanes take a new ray as soon as theirs
                                       is done; this flag keeps one thread per ray for its whole walk
                                       instead (same hits) */

typedef struct crt_config {
    int device;                 /* CUDA device ordinal, default 0 */
    uint32_t ploc_radius;       /* PLOC search radius, default 16 (bvh.hpp:66) */
    uint32_t sort_digit_bits;   /* radix digit width: 4 or 8, default 8 */
    uint32_t trace_block;       /* threads per traversal block, default 128 */
    uint32_t stack_depth;       /* traversal stack entries per ray, default 64 */
    uint32_t spin_limit;        /* bound on every device-side wait loop, 0 = default */
    uint32_t build_flags;       /* CRT_BUILD_MULTI_LAUNCH: one launch per PLOC iteration and layout level */
} crt_config;
#define CRT_BUILD_MULTI_LAUNCH 0x1u

typedef struct crt_ctx crt_ctx;
typedef struct crt_bvh crt_bvh;

/* Build statistics of the last crt_build on a context (device-timed). */
typedef struct crt_build_stats {
    uint32_t n_tris;
    uint32_t ploc_iterations;
    float ms_morton;     /* scene box + Morton codes */
    float ms_sort;       /* radix sort of (code, index) */
    float ms_ploc;       /* PLOC iterations */
    float ms_layout;     /* DFS node layout (inside the one-launch path: from its own timer stamps) */
    float ms_total;
    float scene_box[6];  /* min xyz, max xyz over the scanned buffer */
} crt_build_stats;

/* ---- context ---------------------------------------------------------- */
uint32_t crt_abi_version(void);
void crt_default_config(crt_config* cfg);
crt_status crt_create(crt_ctx** ctx, const crt_config* cfg /* may be NULL */);
crt_status crt_destroy(crt_ctx* ctx);
crt_status crt_sync(crt_ctx* ctx);
const char* crt_last_error_string(void);
/* The CUDA stream (cudaStream_t) the context orders its work on. */
void* crt_stream(crt_ctx* ctx);

/* ---- mesh input: replaces Mesh::load (srcCommon/scene/geometry/mesh.cpp:186-263) and
 * the TriangleGPU assembly of Scene::getTriangleToGPUData (srcOpenGL/scene/scene.cpp:26-40).
 * crt_obj_parse reads Wavefront OBJ text (len bytes) on the host: "v x y z" vertices and
 * "f" faces ("v", "v/vt", "v//vn", "v/vt/vn" corners, 1-based or negative relative
 * indices; faces of more than 3 corners become the fan (0, i, i+1)); everything else is
 * skipped.  It writes up to vert_cap vertices (3 floats each) and tri_cap triangles (3
 * vertex indices each) — pass NULL / 0 to count only — and returns the full counts in
 * counts[0] (vertices) and counts[1] (triangles).  Malformed lines give CRT_ERR_BAD_INPUT
 * naming the line. */
crt_status crt_obj_parse(const char* text, size_t len, float* vertices, uint32_t vert_cap, uint32_t* indices,
                         uint32_t tri_cap, uint32_t counts[2]);
/* TriangleGPU records of an indexed mesh on the GPU: out[i] holds the vertices of
 * indices[3i..3i+2] as (x, y, z, 1) and model_id (Triangle's constructor,
 * triangle.cpp:18-25).  Several meshes form one scene buffer by writing to out + offset
 * with each mesh's id.  Indices past n_vertices give CRT_ERR_BAD_INPUT. */
crt_status crt_triangles_from_indexed(crt_ctx* ctx, const float* vertices, uint32_t n_vertices, const uint32_t* indices,
                                      uint32_t n_triangles, uint32_t model_id, crt_triangle* out);

/* ---- build: replaces cr::BVH::BVH (bvh.cpp:11-24) + Scene::getBVH_NodesToGPUData
 * (scene.cpp:203-208).
 *   tris      n_buffer triangles; the reference scans all n_buffer of them for
 *             the scene box (bvh.cpp:235-251; Scene pads to 65,536 with zero
 *             records, scene.cpp:26-40) and builds over the first n_tris.
 *   models    n_models <= 64 mesh models; ids >= n_models use identity, as
 *             Scene::getMeshModelToGPUData pads (scene.cpp:17-23).
 *   out       receives a new BVH handle (free with crt_bvh_free). */
crt_status crt_build(crt_ctx* ctx, const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                     const crt_mesh_model* models, uint32_t n_models, crt_bvh** out);
/* Rebuild into an existing handle (same or smaller capacity is reused). */
crt_status crt_rebuild(crt_ctx* ctx, crt_bvh* bvh, const crt_triangle* tris, uint32_t n_buffer,
                       uint32_t n_tris, const crt_mesh_model* models, uint32_t n_models);
/* Refit instead of rebuild, for moving geometry (no counterpart in the
 * reference, which rebuilds).  The n_tris triangles (the count of the last
 * build, same order and tree positions) carry new vertices and/or models; the
 * tree keeps the last build's topology and every box is recomputed bottom-up
 * with the build's rules — AABB::buildFromTriangle for leaves, AABB::merge(left,
 * right) for internal nodes (bvh.cpp:383-413) — so unmoved triangles give the
 * built node array bit for bit.  Traces afterwards are exact for the moved
 * geometry (with CRT_TRI_REFERENCE, equal-t ties follow this tree's DFS
 * order; watertight hits equal those of a rebuild).  The tree gets slower to
 * trace as the motion grows: rebuild when it does.  A bound predictor needs
 * crt_predictor_retarget afterwards, as after a rebuild. */
crt_status crt_refit(crt_ctx* ctx, crt_bvh* bvh, const crt_triangle* tris, uint32_t n_tris,
                     const crt_mesh_model* models, uint32_t n_models);
/* Treelet restructuring of a built or refit tree (no counterpart in the
 * reference; Karras & Aila, "Fast Parallel Construction of High-Quality
 * BVHs", HPG 2013): the same leaves under a tree of lower surface-area cost
 * (a leaf costs its box area, an internal node 1.2 x its area plus its
 * children's costs), for faster traces of a tree that is traced many times,
 * or of a refit tree whose boxes have grown.  Each pass visits every internal
 * node after its children and rebuilds the 7-leaf treelet under each node
 * with at least 7 leaves optimally when that lowers its cost; every box is
 * recomputed with AABB::merge (bvh.cpp:401-413), so the result is one exact
 * function of the input tree.  passes = 0 only recomputes the boxes and lays
 * the tree out again.  The node array and the traversal nodes are rewritten
 * in DFS order (leaf positions change; crt_bvh_copy_perm keeps the build's
 * sorted order); with CRT_TRI_REFERENCE equal-t ties follow the new tree's
 * DFS order, watertight hits are unchanged.  A bound predictor needs
 * crt_predictor_retarget afterwards. */
#define CRT_OPTIMIZE_MAX_PASSES 16u
crt_status crt_optimize(crt_ctx* ctx, crt_bvh* bvh, uint32_t passes);
/* A BVH from a node array the caller already has: the reference's own
 * Scene::getBVH_NodesToGPUData output (scene.cpp:203-208; BVH_NodeGPU in DFS
 * pre-order, left child first, leaves with both children 0 — the array
 * raytracer.glsl reads from binding 5) and the n_tris triangles it indexes,
 * with their models.  Keeps the caller's tree (for example the reference's
 * own CPU build) and makes it traceable here: crt_trace, crt_trace_frame,
 * crt_shade, crt_render_frame, crt_refit and crt_optimize accept the result;
 * crt_bvh_copy_codes / _perm do not (there is no Morton sort).  nodes and
 * tris may be host or device memory.  The array must have 2 n_tris - 1
 * records in that order, each triangle in exactly one leaf; anything else is
 * CRT_ERR_INVALID_ARG.  Boxes are used as given and must contain their
 * triangles (AABB::buildFromTriangle, bvh.cpp:383-399, makes such boxes); the
 * watertight slack is derived from the root box. */
crt_status crt_bvh_from_nodes(crt_ctx* ctx, const crt_bvh_node* nodes, uint32_t n_nodes, const crt_triangle* tris,
                              uint32_t n_tris, const crt_mesh_model* models, uint32_t n_models, crt_bvh** out);
/* The structure check of crt_bvh_from_nodes alone, on the host, without a
 * context (nodes in host memory, or device memory when a GPU is present):
 * CRT_OK for a well-formed array, with info[0] = leaves, [1] = internal nodes,
 * [2] = height (edges on the longest root-leaf path), [3] = 0; otherwise
 * CRT_ERR_INVALID_ARG, and crt_last_error_string() names the first problem. */
crt_status crt_validate_nodes(const crt_bvh_node* nodes, uint32_t n_nodes, uint32_t n_tris, uint32_t info[4]);
crt_status crt_bvh_free(crt_bvh* bvh);
uint32_t crt_bvh_node_count(const crt_bvh* bvh);       /* 2 * n_tris - 1 */
uint32_t crt_bvh_triangle_count(const crt_bvh* bvh);
const crt_bvh_node* crt_bvh_nodes_device(const crt_bvh* bvh);
/* Copy out: node array (reference layout), sorted Morton codes, permutation
 * (sorted position -> triangle index).  dst may be host or device memory. */
crt_status crt_bvh_copy_nodes(crt_ctx* ctx, const crt_bvh* bvh, crt_bvh_node* dst);
crt_status crt_bvh_copy_codes(crt_ctx* ctx, const crt_bvh* bvh, uint32_t* dst);
crt_status crt_bvh_copy_perm(crt_ctx* ctx, const crt_bvh* bvh, uint32_t* dst);
crt_status crt_last_build_stats(crt_ctx* ctx, crt_build_stats* stats);

/* Failure detection check: one bounded device-side wait on a flag in context
 * memory, the same bounded spin every look-back and grid barrier uses.  With
 * set_flag != 0 the flag is set before the wait (CRT_OK); with set_flag == 0
 * nothing sets it and the wait gives up after spin_limit rounds
 * (CRT_ERR_DEVICE_TIMEOUT, the context stays usable).  spin_limit 0 = the
 * context's limit. */
crt_status crt_selftest_wait(crt_ctx* ctx, int set_flag, uint32_t spin_limit);
/* Failure detection check of the tensor-core wait the predictor kernels use
 * (an mbarrier that an MMA commit completes): one CTA allocates tensor
 * memory, then with complete != 0 issues and commits one MMA and reads the
 * result back (CRT_OK when it is right); with complete == 0 it waits on a
 * phase nothing completes, gives up after spin_limit rounds
 * (CRT_ERR_DEVICE_TIMEOUT), frees its tensor memory without reading it and
 * returns, so the context and later predictor calls stay usable.  spin_limit
 * 0 = the predictor kernels' own limit. */
crt_status crt_selftest_tc_wait(crt_ctx* ctx, int complete, uint32_t spin_limit);

/* The radix sort's two counting steps alone, the parts the reference's GPU
 * sort shaders implement (srcCommon/shaders/ploc/preprocessing/sort/
 * histogramOfGlobalDigitCounts.glsl:31-59, prefixSumOfGlobalDigitCounts.glsl:
 * 24-69) and its sort tests check (tests/testsSortGPU/testHistogramCreation.cpp,
 * testHistogramCreationHard.cpp, testHistogramPrefixSum.cpp).  Both run the
 * device functions the sort passes themselves use.  digit_bits: 1, 2, 4 or 8.
 *   crt_radix_digit_counts: counts[p * 2^digit_bits + d] = keys whose digit p
 *     (bits p*digit_bits and up) is d, for the ceil(32 / digit_bits) digit
 *     places of 32-bit keys.  With 1-bit digits, counts[2b + 1] is the
 *     reference's per-bit histogram entry b.
 *   crt_radix_digit_offsets: for each of n_places places, the exclusive scan
 *     of its 2^digit_bits counts (where each digit's keys start in that
 *     pass's output).  With 2-bit digits this is the reference's scan inside
 *     each group of 4 histogram entries.
 * Pointers may be host or device memory; both return after their stream
 * synchronises. */
crt_status crt_radix_digit_counts(crt_ctx* ctx, const uint32_t* keys, uint32_t n, uint32_t digit_bits,
                                  uint32_t* counts);
crt_status crt_radix_digit_offsets(crt_ctx* ctx, const uint32_t* counts, uint32_t n_places, uint32_t digit_bits,
                                   uint32_t* offsets);

/* ---- rays ------------------------------------------------------------- */
/* Primary rays of getRay (raytracer.glsl:92-100) for a width x height image:
 * ray (x, y) is stored at y * width + x and uses pos = (x / width, y / height). */
crt_status crt_raygen_pinhole(crt_ctx* ctx, const crt_camera* cam, uint32_t width, uint32_t height,
                              crt_ray* rays);
/* One shadow ray per primary hit toward a point light: origin = o + t d,
 * direction = normalize(light - origin), [tmin, tmax] = [1e-4, |light - origin|].
 * Primary misses give an empty ray (tmin = 1, tmax = 0) that never hits. */
crt_status crt_shadow_rays(crt_ctx* ctx, const crt_ray* primary, const crt_hit* hits, uint32_t n_rays,
                           const float light[3], crt_ray* shadow);

/* ---- trace: replaces getClosestHitBVH (raytracer.glsl:246-295) ---------- */
crt_status crt_trace(crt_ctx* ctx, const crt_bvh* bvh, const crt_ray* rays, uint32_t n_rays,
                     uint32_t flags, crt_hit* hits);
/* Counters of the last crt_trace issued with CRT_TRACE_STATS:
 * out[0] = traversal nodes fetched (64-byte binary, or 128-byte 4-wide with
 * CRT_TRACE_WIDE), out[1] = triangles tested. */
crt_status crt_last_trace_stats(crt_ctx* ctx, uint64_t out[2]);
/* Device time of the last traversal issued through crt_trace,
 * crt_trace_seeded or the multi-launch frame paths, from CUDA events on the
 * context's stream: ms[0] = the work before the traversal kernel (predictor
 * inference, ray keys and their radix sort; 0 for a plain trace), ms[1] =
 * the traversal kernel itself.  With host rays and predictor ordering the
 * inference runs while the rays come in, before the first event, so ms[0]
 * is the sort alone.  Waits for that work to finish. */
crt_status crt_last_trace_timing(crt_ctx* ctx, float ms[2]);

/* One frame of the reference's compute pass (Application::drawOneFrame,
 * srcOpenGL/application.cpp:220-262, minus shading): getRay for every texel
 * of a width x height image, closest hit with `flags`, then — when light is
 * not NULL — one any-hit shadow ray per primary hit toward the point light.
 * Rays live in context memory; only the camera goes in and the hits come out
 * (hits_primary[width*height], hits_shadow[width*height] or NULL; host or
 * device memory).  Shadow misses on primary misses are reported as CRT_MISS.
 * Plain frames (no CRT_TRACE_USE_PREDICTOR / CRT_TRACE_WIDE) run in one
 * launch: each pixel's camera ray, closest hit, shadow ray and any hit; with
 * CRT_TRACE_STATS the counts cover the primary and the shadow traversals. */
crt_status crt_trace_frame(crt_ctx* ctx, const crt_bvh* bvh, const crt_camera* cam, uint32_t width,
                           uint32_t height, const float* light, uint32_t flags, crt_hit* hits_primary,
                           crt_hit* hits_shadow);

/* ---- shading: replaces getColor + imageStore (raytracer.glsl:159-179, 319-330) ----
 * cr::MaterialGPU (srcCommon/scene/pbr/material.hpp:9-11): an RGBA colour, 16 bytes. */
typedef struct crt_material {
    float color[4];
} crt_material;

#define CRT_SHADE_WIREFRAME 0x1u  /* uIsWireframeModeOn: hits with a barycentric coordinate < 0.02 are black */
#define CRT_SHADE_BVH       0x2u  /* uIsBVHDisplayed: texels start from the colour of the BVH boxes at bvh_depth */
#define CRT_SHADE_MAX_BVH_DEPTH 63u

/* What getColor reads besides the hit: the shader's uniforms
 * (srcOpenGL/application.cpp:229-232) and its model and material buffers
 * (srcOpenGL/scene/scene.cpp:17-23, 42-48, 110-121).  Only material_id of a
 * model is read; model ids >= n_models use material 0 (the default records of
 * the shader's 64-entry model buffer), and material ids >= n_materials read
 * (0, 0, 0, 0) (the never-uploaded part of its material buffer). */
typedef struct crt_shading {
    const crt_mesh_model* models;    /* uModels; may be NULL when n_models == 0 */
    uint32_t n_models;               /* <= 64 */
    const crt_material* materials;   /* uMaterials; may be NULL when n_materials == 0 */
    uint32_t n_materials;
    uint32_t flags;                  /* CRT_SHADE_* */
    uint32_t bvh_depth;              /* uDepthDisplayBVH, <= CRT_SHADE_MAX_BVH_DEPTH */
} crt_shading;

/* Texel i of n (rgba[4i .. 4i+3], RGBA32F) for hit i of ray i, as main and
 * getColor compute it:
 *   value = (0, 0, 0, 1);
 *   with CRT_SHADE_BVH, value = bvhColor: (0.5, 0, 0.5, 0.1) for the box at
 *     depth bvh_depth that the shader's walk (getClosestHitBVH, right child
 *     popped first, every intersected box entered) meets last, (0.7, 0, 0.7,
 *     0.1) if the ray enters that box within 0.05 / (bvh_depth + 1) of its
 *     faces on two axes (intersectBVH returns 2), (0, 0, 0, 0) if no box at
 *     that depth is met;
 *   on a hit, value += the colour of the hit triangle's model's material, then
 *     with CRT_SHADE_WIREFRAME value = (0, 0, 0, 1) where u, v or 1 - u - v
 *     is below 0.02.
 * rays are read only with CRT_SHADE_BVH (else they may be NULL); hits come
 * from a trace of those rays on bvh.  Every pointer may be host or device
 * memory; device rgba must be 16-byte aligned. */
crt_status crt_shade(crt_ctx* ctx, const crt_bvh* bvh, const crt_ray* rays, const crt_hit* hits, uint32_t n,
                     const crt_shading* shading, float* rgba);
/* The reference's whole compute pass for one frame (raytracer.glsl main,
 * dispatched at srcOpenGL/application.cpp:245): getRay for every texel,
 * closest hit with `flags` (as crt_trace_frame), getColor and imageStore into
 * rgba[4 * (y * width + x)] (row y = 0 is the texture's first row, the bottom
 * of the displayed image).  Plain frames (no CRT_TRACE_USE_PREDICTOR /
 * CRT_TRACE_WIDE) run in one launch. */
crt_status crt_render_frame(crt_ctx* ctx, const crt_bvh* bvh, const crt_camera* cam, uint32_t width, uint32_t height,
                            uint32_t flags, const crt_shading* shading, float* rgba);

/* ---- learned hit predictor (no counterpart in the reference) --------------
 * An FP16 MLP on tcgen05 tensor cores maps a ray (origin cell on a 64^3 grid,
 * direction in 32x32 octahedral bins, each through a learned 16-wide
 * embedding) through 32 -> 64 -> 64 -> 128 to a treelet of the BVH (the BVH
 * cut into <= 127 subtrees, class 127 = miss).  crt_trace with
 * CRT_TRACE_USE_PREDICTOR first searches the predicted treelet exactly and
 * seeds t_max with that hit, then runs the full traversal: results are
 * identical to the plain traversal; only the work changes.  Training is
 * online on the tracer's own exact hits (softmax cross-entropy, Adam with
 * FP32 master weights).  A predictor is bound to one BVH; call
 * crt_predictor_retarget after rebuilding that BVH. */
typedef struct crt_predictor crt_predictor;
typedef struct crt_predictor_config {
    uint32_t seed;          /* weight initialisation seed */
    float lr;               /* Adam learning rate, default 1e-3 */
    uint32_t train_stride;  /* train on every train_stride-th ray (20 = 5%) */
    uint32_t batch;         /* samples per Adam step, default 16384 */
    float miss_threshold;   /* seed the likeliest treelet unless P(miss) >= this, default 0.9 */
} crt_predictor_config;
#define CRT_PREDICTOR_CLASSES 128u
#define CRT_PREDICTOR_PARAMS 4225280u   /* floats in the flat parameter / gradient vector */

void crt_predictor_default_config(crt_predictor_config* cfg);
crt_status crt_predictor_create(crt_ctx* ctx, crt_bvh* bvh, const crt_predictor_config* cfg, crt_predictor** out);
crt_status crt_predictor_destroy(crt_predictor* pred);
/* Recompute the treelet cut and classes after the bound BVH was rebuilt. */
crt_status crt_predictor_retarget(crt_ctx* ctx, crt_predictor* pred);
/* Train on rays offset, offset + stride, ... of (rays, hits) — hits from the
 * exact tracer — in Adam steps of `batch` samples; mean loss to *loss. */
crt_status crt_predictor_train(crt_ctx* ctx, crt_predictor* pred, const crt_ray* rays, const crt_hit* hits,
                               uint32_t n_rays, uint32_t offset, float* loss);
/* crt_trace seeded from caller-given classes instead of the network's (for
 * measuring a given prediction quality, e.g. the true classes). */
crt_status crt_trace_seeded(crt_ctx* ctx, const crt_bvh* bvh, const crt_ray* rays, uint32_t n_rays, uint32_t flags,
                            const uint16_t* classes, crt_hit* hits);
/* Predicted class per ray: the likeliest treelet, or 127 when the network
 * gives a miss at least miss_threshold probability. */
crt_status crt_predictor_infer(crt_ctx* ctx, crt_predictor* pred, const crt_ray* rays, uint32_t n, uint16_t* classes);
/* The class an exact hit belongs to (treelet of its triangle, or 127). */
crt_status crt_predictor_classes_of_hits(crt_ctx* ctx, crt_predictor* pred, const crt_hit* hits, uint32_t n,
                                         uint16_t* classes);
/* Forward + backward only, on explicit target classes: gradient sums (not
 * averaged) over the n rays into grad[CRT_PREDICTOR_PARAMS], summed loss. */
crt_status crt_predictor_gradients(crt_ctx* ctx, crt_predictor* pred, const crt_ray* rays, const uint16_t* targets,
                                   uint32_t n, float* grad, float* loss);
/* Copy the FP32 master parameters out (set = 0) or in (set = 1). */
crt_status crt_predictor_params(crt_ctx* ctx, crt_predictor* pred, float* params, int set);
/* info[0] = parameters, [1] = classes, [2] = treelets, [3] = Adam steps taken. */
crt_status crt_predictor_info(const crt_predictor* pred, uint32_t info[4]);

/* Cosine-weighted diffuse bounce rays about the geometric normal of primary
 * hits: ray j starts at entry (j * 2654435761 + seed) mod n_hits of the
 * ordered list of primary hits (incoherent order); [tmin, tmax] =
 * [1e-4, +inf].  With no primary hit every output ray is empty. */
crt_status crt_bounce_rays(crt_ctx* ctx, const crt_bvh* bvh, const crt_ray* primary, const crt_hit* hits,
                           uint32_t n_primary, uint32_t n_out, uint32_t seed, crt_ray* out);

/* ---- batched scenes (many scenes, one launch per stage) -----------------
 * n_scenes <= 256 scenes whose triangles and rays are concatenated in scene
 * order (scene s owns tri_counts[s] triangles and ray_counts[s] rays).  Every
 * stage runs as one launch over all scenes (per-scene scene boxes and Morton
 * codes, one radix sort with a final pass that regroups the scenes, all
 * scenes' PLOC iterations in one persistent launch, one trace launch), and
 * crt_batch_run can capture build + trace into a CUDA graph and replay it.
 * Each scene's node array equals crt_build on that scene alone.  Hits carry
 * scene-local triangle indices. */
typedef struct crt_batch crt_batch;
crt_status crt_batch_create(crt_ctx* ctx, const uint32_t* tri_counts, const uint32_t* ray_counts, uint32_t n_scenes,
                            crt_batch** out);
crt_status crt_batch_free(crt_batch* batch);
/* Model matrices shared by all scenes (host memory, <= 64). */
crt_status crt_batch_set_models(crt_ctx* ctx, crt_batch* batch, const crt_mesh_model* models, uint32_t n_models);
/* Build parameters (ploc_radius, sort_digit_bits) and trace parameters
 * (trace_block 128/256/512, stack_depth 64 or 1024) of this batch. */
crt_status crt_batch_set_config(crt_batch* batch, const crt_config* cfg);
crt_status crt_batch_get_config(const crt_batch* batch, crt_config* cfg);
/* tris, rays, hits: device memory. */
crt_status crt_batch_build(crt_ctx* ctx, crt_batch* batch, const crt_triangle* tris);
crt_status crt_batch_trace(crt_ctx* ctx, crt_batch* batch, const crt_ray* rays, uint32_t flags, crt_hit* hits);
/* Build + trace; use_graph != 0 captures the sequence into a CUDA graph on
 * first use (per argument set) and replays it.  *graph_used (optional)
 * reports whether the graph path ran. */
crt_status crt_batch_run(crt_ctx* ctx, crt_batch* batch, const crt_triangle* tris, const crt_ray* rays, uint32_t flags,
                         crt_hit* hits, int use_graph, int* graph_used);
/* New per-scene ray counts for the following traces (no counterpart in the
 * reference): ray_counts[n_scenes], in total at most the rays the batch was
 * created with; the scenes' rays stay concatenated in scene order.  A graph
 * that crt_batch_run captured replays only with the counts it was captured
 * with (other counts capture a new one), so a frame can switch between a
 * fixed primary ray set (build + trace replayed) and a varying secondary one
 * (crt_batch_trace). */
crt_status crt_batch_set_ray_counts(crt_ctx* ctx, crt_batch* batch, const uint32_t* ray_counts);
/* crt_bounce_rays over one scene of a built batch: primary rays and their
 * hits (scene-local triangle ids) in, n_out cosine bounce rays out; device
 * memory. */
crt_status crt_batch_bounce_rays(crt_ctx* ctx, crt_batch* batch, uint32_t scene, const crt_ray* primary,
                                 const crt_hit* hits, uint32_t n_primary, uint32_t n_out, uint32_t seed, crt_ray* out);
crt_status crt_batch_copy_nodes(crt_ctx* ctx, const crt_batch* batch, uint32_t scene, crt_bvh_node* dst);
/* info[0] = triangles, [1] = rays, [2] = PLOC iterations, [3] = first triangle (concatenated index). */
crt_status crt_batch_scene_info(const crt_batch* batch, uint32_t scene, uint32_t info[4]);
/* Project-written autotuner: times build + trace for PLOC radius {8, 16, 32}
 * x digit width {4, 8}, then the trace for block {128, 256, 512} x stack
 * {64 when the trees allow, 1024}; keeps the fastest in the batch and
 * returns it (and its build + trace ms). */
crt_status crt_batch_autotune(crt_ctx* ctx, crt_batch* batch, const crt_triangle* tris, const crt_ray* rays,
                              uint32_t flags, crt_hit* hits, crt_config* best, float* best_ms);

/* A predictor over every scene of a batch (no counterpart in the reference):
 * one network for all scenes; a ray's class is a treelet of its own scene
 * (each scene's BVH cut into <= 127 subtrees) or "miss", its features its
 * origin cell on its scene's box (the cell index moved by a hash of the scene
 * index) and its direction bin.  Create it after the batch's first build and
 * call crt_predictor_retarget after every rebuild.  crt_predictor_train,
 * _infer, _classes_of_hits and _gradients take the batch's concatenated rays
 * and hits (ray i belongs to the scene whose ray range holds it; hits carry
 * scene-local triangle ids).  crt_batch_trace and crt_batch_run then accept
 * CRT_TRACE_PREDICTOR_ORDER (rays ordered by scene, predicted treelet, origin
 * cell, direction) and CRT_TRACE_USE_PREDICTOR (each ray first searches its
 * predicted treelet exactly), with the same hits as without them; a captured
 * graph includes the inference and reads the current weights. */
crt_status crt_batch_predictor_create(crt_ctx* ctx, crt_batch* batch, const crt_predictor_config* cfg,
                                      crt_predictor** out);

/* ---- allocation-free Morton + sort ------------------------------------
 * No counterpart in the reference (its build allocates std::vectors freely).
 * For callers that must not have this library allocate device memory — e.g.
 * an engine that gives all device memory to its own pool and forbids the
 * libraries it embeds from calling cudaMalloc, whose allocations would escape
 * its budget and can stall the device mid-frame.  Computes what crt_build
 * computes first: Morton codes of the first n_tris of n_buffer triangles,
 * sorted with their indices; codes_out / perm_out match crt_bvh_copy_codes /
 * crt_bvh_copy_perm of crt_build on the same input.
 *   tris, codes_out, perm_out  device memory; models: host memory (or NULL
 *   when n_models == 0); stream: a cudaStream_t, NULL for the default stream.
 * It calls no cudaMalloc/cudaFree: its scratch is one fixed array of about
 * 4.5 MB compiled into the library and kept on every GPU that loads it until
 * the process exits, which caps n_tris at CRT_NOALLOC_MAX_TRIANGLES (larger
 * inputs return CRT_ERR_INVALID_ARG).  All calls share that array: calls whose
 * work overlaps on the GPU race and must be serialised by the caller.  The
 * first call on a device looks up the array's device address.  Returns after
 * the stream synchronises. */
#define CRT_NOALLOC_MAX_TRIANGLES 262144u
crt_status crt_morton_sort_noalloc(const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                                   const crt_mesh_model* models, uint32_t n_models, uint32_t* codes_out,
                                   uint32_t* perm_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CRT_H */
