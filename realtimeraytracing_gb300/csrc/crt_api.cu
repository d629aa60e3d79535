// C ABI of libcrt (include/crt.h): contexts, device buffers, the build
// pipeline (scene box -> Morton -> radix sort -> PLOC -> DFS layout) and the
// trace entry points.  No compute happens on the host: a call that cannot
// run its kernels returns an error instead of falling back.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>
#include <vector>

#include "crt.h"
#include "crt_build.cuh"
#include "crt_common.cuh"

namespace {

thread_local char g_err[512] = "no error";

crt_status fail(crt_status s, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return s;
}

#define CRT_CUDA(call)                                                                                  \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            return fail(e_ == cudaErrorMemoryAllocation ? CRT_ERR_OOM : CRT_ERR_CUDA, "%s failed: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                             \
        }                                                                                               \
    } while (0)

#define CRT_TRY(expr)                  \
    do {                               \
        crt_status s_ = (expr);        \
        if (s_ != CRT_OK) return s_;   \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    crt_status reserve(size_t bytes) {
        if (bytes <= cap) return CRT_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = bytes + bytes / 8 + 256;
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(CRT_ERR_OOM, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
        }
        cap = want;
        return CRT_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

bool is_device_ptr(const void* ptr) {
    if (!ptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The device address of page-locked host memory the GPU can write directly
// (cudaMallocHost / cudaHostRegister, mapped under unified addressing), or
// null for device, pageable or unknown memory.
void* mapped_host_ptr(void* ptr) {
    if (!ptr) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    // the kernels read and write records as 16-byte vectors: other page-locked
    // buffers take the copy path
    if (a.type != cudaMemoryTypeHost || (reinterpret_cast<uintptr_t>(a.devicePointer) & 15u) != 0) return nullptr;
    return a.devicePointer;
}

// A caller's device buffer the kernels read or write as 16-byte vectors.
crt_status check_aligned16(const void* p, const char* what) {
    if ((reinterpret_cast<uintptr_t>(p) & 15u) != 0)
        return fail(CRT_ERR_INVALID_ARG, "%s: device memory must be 16-byte aligned", what);
    return CRT_OK;
}

// The batch pipeline reads its triangles and rays and writes its hits in
// device memory only (graph replays reuse the pointers).
crt_status check_batch_buffers(const void* tris, const void* rays, const void* hits, const char* fn) {
    if (!is_device_ptr(tris) || !is_device_ptr(rays) || !is_device_ptr(hits))
        return fail(CRT_ERR_INVALID_ARG, "%s: triangles, rays and hits must be device memory", fn);
    if (((reinterpret_cast<uintptr_t>(tris) | reinterpret_cast<uintptr_t>(rays) | reinterpret_cast<uintptr_t>(hits)) & 15u) != 0)
        return fail(CRT_ERR_INVALID_ARG, "%s: device memory must be 16-byte aligned", fn);
    return CRT_OK;
}

constexpr uint32_t kDefaultSpin = 1u << 22;   // ~0.3 s with back-off; far above any normal wait

}  // namespace

namespace crt {
void set_last_error(const char* msg) { std::snprintf(g_err, sizeof(g_err), "%s", msg); }
}  // namespace crt

struct crt_bvh {
    crt_ctx* ctx = nullptr;
    uint32_t n = 0;
    // Bound on the traversal stack's depth: the PLOC iteration count after a
    // build (tree height <= iterations + 1), the tree's height after crt_optimize.
    uint32_t depth_bound = 0;
    float abs_eps = 0.f;
    // wide_wt: boxes grown by abs_eps; xtri: transformed triangles in the tree's
    // left-to-right leaf order; inv_perm: triangle -> its position in that order
    DevBuf nodes, wide, wide_wt, depth_odd, xtri, codes, perm, inv_perm;
    mutable DevBuf wide4, cwide;
    crt_predictor* predictor = nullptr;
    // The 4-wide traversal nodes are derived on the first CRT_TRACE_WIDE
    // trace after a build, so builds whose trees are never walked 4-wide
    // neither compute nor store them.
    mutable bool wide4_ready = false;
    mutable bool cwide_ready = false;  // the compressed 4-wide nodes, derived likewise
    // Refit topology of the last build (crt_refit, derived on its first call).
    DevBuf refit_link, refit_leaf, refit_dfs, refit_cnt;
    bool refit_ready = false;
    // After a refit only the root box of the node array is current; the
    // others are derived from the traversal nodes when the array is read.
    mutable bool node_boxes_stale = false;
    // Sorted Morton codes and permutation exist (a tree from crt_bvh_from_nodes has none).
    bool has_sort = false;
};

struct crt_predictor {
    crt_bvh* bvh = nullptr;        // bound to one BVH ...
    crt_batch* batch = nullptr;    // ... or to every scene of a batch
    // a batch's device scene table, node array and triangle count (fixed at crt_batch_create)
    const crt::BatchScene* batch_scenes = nullptr;
    const crt_bvh_node* batch_nodes = nullptr;
    uint32_t batch_n_scenes = 0, batch_n_tris = 0;
    crt_predictor_config cfg{};
    DevBuf params;      // master | m | v | grad, CRT_PREDICTOR_PARAMS floats each
    DevBuf w16;         // fp16 copies
    DevBuf tri_class;   // triangle -> class
    DevBuf treelets;    // Treelet[127] + count
    DevBuf classes;     // per-ray predicted classes (trace scratch)
    DevBuf order, order_scratch;  // rays grouped by predicted class (CRT_TRACE_PREDICTOR_ORDER)
    DevBuf scratch;     // loss accumulator
    DevBuf rays_in, hits_in, targets_in;
    uint32_t step = 0;
    uint32_t n_treelets = 0;
    crt::PredictorDev dev() const {
        crt::PredictorDev d;
        float* base = params.as<float>();
        d.master = base;
        d.m = base + crt::pred::kParams;
        d.v = base + 2 * crt::pred::kParams;
        d.grad = base + 3 * crt::pred::kParams;
        d.w16 = w16.as<__half>();
        d.tri_class = tri_class.as<uint8_t>();
        d.n_tris = bvh ? bvh->n : batch_n_tris;
        d.scenes = batch_scenes;
        d.n_scenes = batch ? batch_n_scenes : 0u;
        return d;
    }
    bool bound() const { return bvh != nullptr || batch != nullptr; }
    const crt_bvh_node* nodes() const { return bvh ? bvh->nodes.as<crt_bvh_node>() : batch_nodes; }
};

struct crt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    crt_config cfg{};
    // build scratch
    DevBuf tris_in, models, scene_state, err, hist, sort_lb, codes_a, codes_b, vals_a, vals_b;
    DevBuf node_box, node_kids, pos, clus_a, clus_b, iters, ploc_lb;
    DevBuf cam, rays_in, hits_out, rays_out, trace_stats, frame_rays, frame_hits, frame_shadow, frame_shits;
    DevBuf ray_order, ray_order_scratch;  // CRT_TRACE_SORT_RAYS
    DevBuf shade_models, shade_materials, shade_rays, shade_hits, image;  // crt_shade / crt_render_frame
    DevBuf refit_state;  // crt::RefitState
    DevBuf xtri_sorted;  // leaf records in sorted order until the layout moves them
    DevBuf mesh_vertices, mesh_indices, mesh_out;  // crt_triangles_from_indexed staging
    DevBuf probe_flag;                             // crt_selftest_wait
    DevBuf step_in, step_out;                      // crt_radix_digit_counts / _offsets
    DevBuf pool_counter;                           // persistent traversal: next ray to take
    DevBuf opt_scratch;                            // crt_optimize
    uint64_t last_trace_stats[2] = {0, 0};
    // pinned host staging
    void* pinned = nullptr;
    size_t pinned_cap = 0;
    cudaEvent_t ev[6] = {};
    // crt_trace timing: start, traversal kernel launch, end (on the stream)
    cudaEvent_t tev[3] = {};
    // host rays copied in chunks on a second stream so that each chunk's
    // predictor inference runs while the next chunk is in flight
    static constexpr int kCopyChunks = 8;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ev[kCopyChunks + 1] = {};
    bool tev_valid = false;
    crt_build_stats stats{};
    std::vector<uint2> it_host;
    bool force_multi_launch = false;  // testing: run PLOC/layout as one launch per iteration

    crt_status pinned_reserve(size_t bytes) {
        if (bytes <= pinned_cap) return CRT_OK;
        if (pinned) cudaFreeHost(pinned);
        pinned = nullptr;
        pinned_cap = 0;
        CRT_CUDA(cudaMallocHost(&pinned, bytes));
        pinned_cap = bytes;
        return CRT_OK;
    }
    crt_status check_device_error() {
        uint32_t ew[4] = {0, 0, 0, 0};
        CRT_CUDA(cudaMemcpyAsync(ew, err.p, 16, cudaMemcpyDeviceToHost, stream));
        CRT_CUDA(cudaStreamSynchronize(stream));
        const uint32_t e = ew[0];
        if (e & crt::kDevTimeout) return fail(CRT_ERR_DEVICE_TIMEOUT, "a bounded device wait gave up (err=0x%x)", e);
        if (e & crt::kDevBadModel) return fail(CRT_ERR_BAD_INPUT, "a triangle references model id >= 64");
        if (e & crt::kDevBadIndex) return fail(CRT_ERR_BAD_INPUT, "a triangle references a vertex past the end");
        if (e & crt::kDevStackOverflow) return fail(CRT_ERR_STACK_OVERFLOW, "a ray overflowed its traversal stack");
        if (e & crt::kDevCorrupt)
            return fail(CRT_ERR_CUDA, "a device index check failed (err=0x%x site=%u iter=%u values=%u,%u)", e,
                        ew[1] & 0xFFu, ew[1] >> 8, ew[2], ew[3]);
        if (e) return fail(CRT_ERR_CUDA, "device error word 0x%x", e);
        return CRT_OK;
    }
};

extern "C" {

uint32_t crt_abi_version(void) { return CRT_ABI_VERSION; }

const char* crt_last_error_string(void) { return g_err; }

void crt_default_config(crt_config* cfg) {
    if (!cfg) return;
    cfg->device = 0;
    cfg->ploc_radius = 16;
    cfg->sort_digit_bits = 8;
    cfg->trace_block = 128;
    cfg->stack_depth = 64;
    cfg->spin_limit = 0;
    cfg->build_flags = 0;
}

crt_status crt_create(crt_ctx** out, const crt_config* cfg) {
    if (!out) return fail(CRT_ERR_INVALID_ARG, "crt_create: null output pointer");
    *out = nullptr;
    crt_config c;
    crt_default_config(&c);
    if (cfg) c = *cfg;
    if (c.ploc_radius == 0 || c.ploc_radius > static_cast<uint32_t>(crt::kPlocMaxRadius))
        return fail(CRT_ERR_INVALID_ARG, "ploc_radius must be in [1, %d]", crt::kPlocMaxRadius);
    if (c.sort_digit_bits != 4 && c.sort_digit_bits != 8)
        return fail(CRT_ERR_INVALID_ARG, "sort_digit_bits must be 4 or 8");
    if (c.trace_block != 64 && c.trace_block != 128 && c.trace_block != 256)
        return fail(CRT_ERR_INVALID_ARG, "trace_block must be 64, 128 or 256");
    if (c.spin_limit == 0) c.spin_limit = kDefaultSpin;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CRT_ERR_UNSUPPORTED, "no CUDA device");
    }
    if (c.device < 0 || c.device >= ndev) return fail(CRT_ERR_INVALID_ARG, "device %d out of range", c.device);
    cudaDeviceProp prop;
    CRT_CUDA(cudaGetDeviceProperties(&prop, c.device));
    if (prop.major * 10 + prop.minor != 103)
        return fail(CRT_ERR_UNSUPPORTED, "libcrt is built for sm_103a; device is sm_%d%d", prop.major, prop.minor);
    CRT_CUDA(cudaSetDevice(c.device));
    crt_ctx* x = new crt_ctx();
    x->device = c.device;
    x->cfg = c;
    x->force_multi_launch = (c.build_flags & CRT_BUILD_MULTI_LAUNCH) != 0;
    crt_status s = CRT_OK;
    if (cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking) != cudaSuccess) s = fail(CRT_ERR_CUDA, "stream");
    for (auto& e : x->ev)
        if (s == CRT_OK && cudaEventCreate(&e) != cudaSuccess) s = fail(CRT_ERR_CUDA, "event");
    for (auto& e : x->tev)
        if (s == CRT_OK && cudaEventCreate(&e) != cudaSuccess) s = fail(CRT_ERR_CUDA, "event");
    if (s == CRT_OK && cudaStreamCreateWithFlags(&x->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
        s = fail(CRT_ERR_CUDA, "stream");
    for (auto& e : x->copy_ev)
        if (s == CRT_OK && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) s = fail(CRT_ERR_CUDA, "event");
    if (s == CRT_OK) s = x->scene_state.reserve(sizeof(crt::SceneState));
    if (s == CRT_OK) s = x->err.reserve(16);
    if (s == CRT_OK) s = x->models.reserve(2 * 64 * 16 * sizeof(float));
    if (s == CRT_OK) s = x->cam.reserve(sizeof(crt_camera));
    if (s == CRT_OK) s = x->trace_stats.reserve(16);
    if (s == CRT_OK) s = x->pinned_reserve(1 << 16);
    if (s == CRT_OK) {
        crt::SceneState init{};
        for (int a = 0; a < 3; ++a) { init.key_max[a] = 0ull; init.key_min[a] = ~0ull; }
        if (cudaMemcpy(x->scene_state.p, &init, sizeof(init), cudaMemcpyHostToDevice) != cudaSuccess)
            s = fail(CRT_ERR_CUDA, "scene state init");
    }
    if (s != CRT_OK) {
        crt_destroy(x);
        return s;
    }
    *out = x;
    return CRT_OK;
}

crt_status crt_destroy(crt_ctx* x) {
    if (!x) return CRT_OK;
    cudaSetDevice(x->device);
    if (x->stream) cudaStreamSynchronize(x->stream);
    DevBuf* bufs[] = {&x->tris_in, &x->models, &x->scene_state, &x->err, &x->hist, &x->sort_lb, &x->codes_a,
                      &x->codes_b, &x->vals_a, &x->vals_b, &x->node_box, &x->node_kids, &x->pos, &x->clus_a,
                      &x->clus_b, &x->iters, &x->ploc_lb, &x->cam, &x->rays_in, &x->hits_out, &x->rays_out,
                      &x->trace_stats, &x->frame_rays, &x->frame_hits, &x->frame_shadow, &x->frame_shits,
                      &x->ray_order, &x->ray_order_scratch, &x->shade_models, &x->shade_materials,
                      &x->shade_rays, &x->shade_hits, &x->image, &x->refit_state, &x->xtri_sorted,
                      &x->mesh_vertices, &x->mesh_indices, &x->mesh_out, &x->probe_flag, &x->step_in,
                      &x->step_out, &x->pool_counter};
    for (DevBuf* b : bufs) b->release();
    for (auto& e : x->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : x->tev)
        if (e) cudaEventDestroy(e);
    for (auto& e : x->copy_ev)
        if (e) cudaEventDestroy(e);
    if (x->pinned) cudaFreeHost(x->pinned);
    if (x->copy_stream) {
        cudaStreamSynchronize(x->copy_stream);
        cudaStreamDestroy(x->copy_stream);
    }
    if (x->stream) cudaStreamDestroy(x->stream);
    delete x;
    return CRT_OK;
}

crt_status crt_selftest_wait(crt_ctx* x, int set_flag, uint32_t spin_limit) {
    if (!x) return fail(CRT_ERR_INVALID_ARG, "null context");
    CRT_CUDA(cudaSetDevice(x->device));
    CRT_TRY(x->probe_flag.reserve(4));
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    CRT_CUDA(cudaMemsetAsync(x->probe_flag.p, set_flag ? 0xFF : 0, 4, x->stream));
    crt::launch_wait_probe(x->probe_flag.as<unsigned int>(), spin_limit ? spin_limit : x->cfg.spin_limit,
                           x->err.as<uint32_t>(), x->stream);
    CRT_CUDA(cudaGetLastError());
    return x->check_device_error();
}

crt_status crt_selftest_tc_wait(crt_ctx* x, int complete, uint32_t spin_limit) {
    if (!x) return fail(CRT_ERR_INVALID_ARG, "null context");
    CRT_CUDA(cudaSetDevice(x->device));
    CRT_TRY(x->probe_flag.reserve(128 * sizeof(float)));
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    CRT_CUDA(cudaMemsetAsync(x->probe_flag.p, 0, 128 * sizeof(float), x->stream));
    CRT_CUDA(crt::tc_wait_probe(complete, spin_limit, x->err.as<uint32_t>(), x->probe_flag.as<float>(), x->stream));
    const crt_status st = x->check_device_error();
    if (st != CRT_OK || !complete) return st;
    float got[128];
    CRT_CUDA(cudaMemcpyAsync(got, x->probe_flag.p, sizeof(got), cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    for (int i = 0; i < 128; ++i)
        if (got[i] != 16.f) return fail(CRT_ERR_CUDA, "MMA probe: lane %d read %g, expected 16", i, got[i]);
    return CRT_OK;
}

// The radix sort's counting and digit-offset steps on caller data (host or
// device memory), each through the library's own device functions.
crt_status crt_radix_digit_counts(crt_ctx* x, const uint32_t* keys, uint32_t n, uint32_t digit_bits, uint32_t* counts) {
    if (!x || (!keys && n) || !counts) return fail(CRT_ERR_INVALID_ARG, "crt_radix_digit_counts: null argument");
    if (digit_bits != 1 && digit_bits != 2 && digit_bits != 4 && digit_bits != 8)
        return fail(CRT_ERR_INVALID_ARG, "crt_radix_digit_counts: digit_bits must be 1, 2, 4 or 8");
    CRT_CUDA(cudaSetDevice(x->device));
    const size_t n_counts = static_cast<size_t>((32 + digit_bits - 1) / digit_bits) << digit_bits;
    const uint32_t* d_keys = keys;
    if (n && !is_device_ptr(keys)) {
        CRT_TRY(x->step_in.reserve(4ull * n));
        CRT_CUDA(cudaMemcpyAsync(x->step_in.p, keys, 4ull * n, cudaMemcpyHostToDevice, x->stream));
        d_keys = x->step_in.as<uint32_t>();
    }
    const bool dev_out = is_device_ptr(counts);
    uint32_t* d_counts = counts;
    if (!dev_out) {
        CRT_TRY(x->step_out.reserve(4 * n_counts));
        d_counts = x->step_out.as<uint32_t>();
    }
    CRT_CUDA(cudaMemsetAsync(d_counts, 0, 4 * n_counts, x->stream));
    if (n) crt::launch_digit_counts(d_keys, n, static_cast<int>(digit_bits), d_counts, x->stream);
    CRT_CUDA(cudaGetLastError());
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(counts, d_counts, 4 * n_counts, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status crt_radix_digit_offsets(crt_ctx* x, const uint32_t* counts, uint32_t n_places, uint32_t digit_bits,
                                   uint32_t* offsets) {
    if (!x || !counts || !offsets) return fail(CRT_ERR_INVALID_ARG, "crt_radix_digit_offsets: null argument");
    if (digit_bits != 1 && digit_bits != 2 && digit_bits != 4 && digit_bits != 8)
        return fail(CRT_ERR_INVALID_ARG, "crt_radix_digit_offsets: digit_bits must be 1, 2, 4 or 8");
    if (n_places == 0 || n_places > 65536) return fail(CRT_ERR_INVALID_ARG, "crt_radix_digit_offsets: bad n_places");
    CRT_CUDA(cudaSetDevice(x->device));
    const size_t n_counts = static_cast<size_t>(n_places) << digit_bits;
    const uint32_t* d_in = counts;
    if (!is_device_ptr(counts)) {
        CRT_TRY(x->step_in.reserve(4 * n_counts));
        CRT_CUDA(cudaMemcpyAsync(x->step_in.p, counts, 4 * n_counts, cudaMemcpyHostToDevice, x->stream));
        d_in = x->step_in.as<uint32_t>();
    }
    const bool dev_out = is_device_ptr(offsets);
    uint32_t* d_out = offsets;
    if (!dev_out) {
        CRT_TRY(x->step_out.reserve(4 * n_counts));
        d_out = x->step_out.as<uint32_t>();
    }
    crt::launch_digit_offsets(d_in, n_places, static_cast<int>(digit_bits), d_out, x->stream);
    CRT_CUDA(cudaGetLastError());
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(offsets, d_out, 4 * n_counts, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status crt_sync(crt_ctx* x) {
    if (!x) return fail(CRT_ERR_INVALID_ARG, "null context");
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

void* crt_stream(crt_ctx* x) { return x ? static_cast<void*>(x->stream) : nullptr; }

}  // extern "C"

namespace {

// Models: 64 column-major matrices (identity past n_models) and the same
// matrices scaled by 1/3 for the centroid (triangle.cpp:32), into x->models.
crt_status stage_model_matrices(crt_ctx* x, const crt_mesh_model* models, uint32_t n_models) {
    float* hm = static_cast<float*>(x->pinned);
    CRT_CUDA(cudaStreamSynchronize(x->stream));  // the pinned staging area may still feed an earlier copy
    const bool dev = n_models > 0 && is_device_ptr(models);
    for (uint32_t m = 0; m < 64; ++m) {
        for (int k = 0; k < 16; ++k) hm[16 * m + k] = (k % 5 == 0) ? 1.f : 0.f;
        if (m < n_models) {
            crt_mesh_model mm;
            if (dev) {
                CRT_CUDA(cudaMemcpy(&mm, models + m, sizeof(mm), cudaMemcpyDeviceToHost));
            } else {
                std::memcpy(&mm, models + m, sizeof(mm));
            }
            std::memcpy(hm + 16 * m, mm.m, 64);
        }
    }
    const volatile float third = 1.f / 3.f;
    for (int k = 0; k < 64 * 16; ++k) hm[64 * 16 + k] = third * hm[k];
    CRT_CUDA(cudaMemcpyAsync(x->models.p, hm, 2 * 64 * 16 * sizeof(float), cudaMemcpyHostToDevice, x->stream));
    return CRT_OK;
}

crt_status build_impl(crt_ctx* x, crt_bvh* b, const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                      const crt_mesh_model* models, uint32_t n_models) {
    if (!tris) return fail(CRT_ERR_INVALID_ARG, "crt_build: null triangles");
    if (n_tris == 0) return fail(CRT_ERR_INVALID_ARG, "crt_build: n_tris must be >= 1");
    if (n_buffer < n_tris) return fail(CRT_ERR_INVALID_ARG, "crt_build: n_buffer < n_tris");
    if (n_tris > (1u << 30)) return fail(CRT_ERR_INVALID_ARG, "crt_build: n_tris above 2^30");
    if (n_models > crt::kMaxModels) return fail(CRT_ERR_INVALID_ARG, "crt_build: more than 64 models");
    if (n_models > 0 && !models) return fail(CRT_ERR_INVALID_ARG, "crt_build: null models");
    CRT_CUDA(cudaSetDevice(x->device));
    cudaStream_t s = x->stream;
    const uint32_t N = n_tris;
    const int bits = static_cast<int>(x->cfg.sort_digit_bits);
    const int passes = (30 + bits - 1) / bits;
    const uint32_t radix = 1u << bits;
    const uint32_t sort_tiles = (N + crt::sort_tile_keys(bits) - 1) / crt::sort_tile_keys(bits);
    const uint32_t ploc_tiles = (N + crt::kPlocMinOwn - 1) / crt::kPlocMinOwn;

    // ---- buffers
    const crt_triangle* d_tris = tris;
    if (!is_device_ptr(tris)) {
        CRT_TRY(x->tris_in.reserve(sizeof(crt_triangle) * static_cast<size_t>(n_buffer)));
        CRT_CUDA(cudaMemcpyAsync(x->tris_in.p, tris, sizeof(crt_triangle) * static_cast<size_t>(n_buffer),
                                 cudaMemcpyHostToDevice, s));
        d_tris = x->tris_in.as<crt_triangle>();
    } else {
        CRT_TRY(check_aligned16(tris, "crt_build: triangles"));
    }
    const size_t hist_words = static_cast<size_t>(passes) * radix;
    const size_t sort_lb_words = static_cast<size_t>(passes) * (sort_tiles * radix + 1);  // + ticket per pass
    CRT_TRY(x->hist.reserve(4 * hist_words));
    CRT_TRY(x->sort_lb.reserve(4 * sort_lb_words));
    CRT_TRY(x->codes_a.reserve(4ull * N));
    CRT_TRY(x->codes_b.reserve(4ull * N));
    CRT_TRY(x->vals_a.reserve(4ull * N));
    CRT_TRY(x->vals_b.reserve(4ull * N));
    CRT_TRY(x->node_box.reserve(32ull * (2ull * N - 1)));
    CRT_TRY(x->node_kids.reserve(16ull * N));
    CRT_TRY(x->pos.reserve(8ull * N));
    CRT_TRY(x->clus_a.reserve(32ull * N));
    CRT_TRY(x->clus_b.reserve(32ull * N));
    CRT_TRY(x->iters.reserve(8ull * (N + 2)));
    // + tail: tickets[2], barrier[2], iteration count, finished blocks, 3 timer stamps
    CRT_TRY(x->ploc_lb.reserve(8ull * (2ull * ploc_tiles) + 64));
    CRT_TRY(b->nodes.reserve(sizeof(crt_bvh_node) * (2ull * N - 1)));
    CRT_TRY(b->xtri.reserve(48ull * N));
    CRT_TRY(x->xtri_sorted.reserve(48ull * N));
    CRT_TRY(b->wide.reserve(64ull * N));
    CRT_TRY(b->wide_wt.reserve(64ull * N));
    b->wide4_ready = false;
    b->cwide_ready = false;
    b->refit_ready = false;
    b->node_boxes_stale = false;
    CRT_TRY(b->depth_odd.reserve(N));
    CRT_TRY(b->inv_perm.reserve(4ull * N));
    CRT_TRY(b->codes.reserve(4ull * N));
    CRT_TRY(b->perm.reserve(4ull * N));

    CRT_TRY(stage_model_matrices(x, models, n_models));
    const float* d_models = x->models.as<float>();
    const float* d_models3 = d_models + 64 * 16;

    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, s));
    CRT_CUDA(cudaMemsetAsync(x->hist.p, 0, 4 * hist_words, s));
    CRT_CUDA(cudaMemsetAsync(x->sort_lb.p, 0, 4 * sort_lb_words, s));
    CRT_CUDA(cudaMemsetAsync(x->ploc_lb.p, 0, 8ull * (2ull * ploc_tiles) + 64, s));
    uint32_t* err = x->err.as<uint32_t>();
    auto* st = x->scene_state.as<crt::SceneState>();

    CRT_CUDA(cudaEventRecord(x->ev[0], s));
    // ---- K1: scene box + Morton codes + digit histograms
    crt::launch_scene_box(d_tris, n_buffer, d_models, st, err, s);
    crt::launch_morton(d_tris, N, d_models3, st, x->codes_a.as<uint32_t>(), x->hist.as<uint32_t>(), bits, s);
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaEventRecord(x->ev[1], s));

    // ---- K2: LSD radix sort, one Onesweep pass per digit
    {
        uint32_t* kin = x->codes_a.as<uint32_t>();
        uint32_t* vin = nullptr;
        for (int p = 0; p < passes; ++p) {
            const bool last = (p == passes - 1);
            uint32_t* kout = last ? b->codes.as<uint32_t>() : ((p & 1) ? x->codes_a.as<uint32_t>() : x->codes_b.as<uint32_t>());
            uint32_t* vout = last ? b->perm.as<uint32_t>() : ((p & 1) ? x->vals_a.as<uint32_t>() : x->vals_b.as<uint32_t>());
            uint32_t* lb = x->sort_lb.as<uint32_t>() + static_cast<size_t>(p) * (sort_tiles * radix + 1);
            crt::launch_onesweep(kin, vin, kout, vout, N, p * bits, bits, x->hist.as<uint32_t>() + p * radix, lb + 1, lb,
                                 err, x->cfg.spin_limit, s);
            kin = kout;
            vin = vout;
        }
    }
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaEventRecord(x->ev[2], s));

    // ---- K3: leaf clusters + PLOC iterations
    uint2* d_it = x->iters.as<uint2>();
    crt::launch_leaf_init(d_tris, N, d_models, b->perm.as<uint32_t>(), x->node_box.as<float4>(), x->clus_a.as<float4>(),
                          x->xtri_sorted.as<float4>(), d_it, err, s);
    const crt::LeafOut leaves{x->xtri_sorted.as<float4>(), b->xtri.as<float4>(), b->inv_perm.as<uint32_t>()};
    CRT_CUDA(cudaGetLastError());
    x->it_host.assign(1, make_uint2(N, N));
    uint32_t iters = 0;
    bool laid_out = false;
    float layout_in_kernel_ms = 0.f;  // the persistent launch's layout phase, from its timer stamps
    if (N > 1 && !x->force_multi_launch) {
        // one cooperative launch: every PLOC iteration, then the DFS layout
        unsigned long long* lb = x->ploc_lb.as<unsigned long long>();
        uint32_t* tail = reinterpret_cast<uint32_t*>(lb + 2ull * ploc_tiles);
        const cudaError_t e = crt::launch_ploc_persistent(
            x->clus_a.as<float4>(), x->clus_b.as<float4>(), x->node_box.as<float4>(), x->node_kids.as<uint4>(), d_it, N,
            static_cast<int>(x->cfg.ploc_radius), lb, tail, ploc_tiles, x->pos.as<uint2>(), b->nodes.as<crt_bvh_node>(),
            b->wide.as<float4>(), b->wide_wt.as<float4>(), b->depth_odd.as<uint8_t>(), leaves, st,
            reinterpret_cast<unsigned long long*>(tail + 2), tail + 4,
            err, x->cfg.spin_limit, s);
        if (e == cudaSuccess) {
            CRT_CUDA(cudaEventRecord(x->ev[3], s));
            uint32_t* hp = static_cast<uint32_t*>(x->pinned);
            CRT_CUDA(cudaMemcpyAsync(hp, tail + 4, 32, cudaMemcpyDeviceToHost, s));
            CRT_CUDA(cudaStreamSynchronize(s));
            iters = hp[0];
            unsigned long long stamp[3];
            std::memcpy(stamp, hp + 2, sizeof(stamp));
            if (stamp[2] > stamp[1]) layout_in_kernel_ms = static_cast<float>(static_cast<double>(stamp[2] - stamp[1]) * 1e-6);
            laid_out = true;
        } else if (e != cudaErrorNotSupported && e != cudaErrorCooperativeLaunchTooLarge) {
            return fail(CRT_ERR_CUDA, "PLOC launch failed: %s", cudaGetErrorString(e));
        } else {
            cudaGetLastError();
        }
    }
    if (N > 1 && !laid_out) {
        uint32_t n_known = N;
        int iter = 0;
        double rate = 0.6;
        float4* ca = x->clus_a.as<float4>();
        float4* cb = x->clus_b.as<float4>();
        unsigned long long* lb = x->ploc_lb.as<unsigned long long>();
        uint32_t* tickets = reinterpret_cast<uint32_t*>(lb + 2ull * ploc_tiles);
        uint2* hpin = static_cast<uint2*>(x->pinned);
        bool done = false;
        while (!done) {
            // enough launches to likely finish, estimated from the observed shrink rate
            int chunk = static_cast<int>(std::ceil(std::log(static_cast<double>(n_known)) / -std::log(rate))) + 2;
            if (chunk < 4) chunk = 4;
            if (chunk > 64) chunk = 64;
            if (static_cast<uint32_t>(iter + chunk) > N) chunk = static_cast<int>(N) - iter;
            if (chunk <= 0) return fail(CRT_ERR_CUDA, "PLOC did not converge");
            for (int c = 0; c < chunk; ++c, ++iter) {
                const float4* cin = (iter & 1) ? cb : ca;
                float4* cout = (iter & 1) ? ca : cb;
                crt::launch_ploc_iteration(cin, cout, x->node_box.as<float4>(), x->node_kids.as<uint4>(), d_it, iter, N,
                                           static_cast<int>(x->cfg.ploc_radius), n_known, lb, tickets, ploc_tiles, err,
                                           x->cfg.spin_limit, s);
            }
            CRT_CUDA(cudaGetLastError());
            const int first = iter - chunk + 1;
            CRT_CUDA(cudaMemcpyAsync(hpin, d_it + first, sizeof(uint2) * chunk, cudaMemcpyDeviceToHost, s));
            CRT_CUDA(cudaStreamSynchronize(s));
            const uint32_t prev = n_known;
            for (int c = 0; c < chunk; ++c) {
                x->it_host.push_back(hpin[c]);
                n_known = hpin[c].x;
                if (n_known <= 1) {
                    iters = static_cast<uint32_t>(first + c);
                    done = true;
                    break;
                }
                if (n_known > prev || n_known == 0) return fail(CRT_ERR_CUDA, "PLOC state corrupt (n=%u)", n_known);
            }
            if (!done) {
                const double r = std::pow(static_cast<double>(n_known) / prev, 1.0 / chunk);
                rate = std::min(0.95, std::max(0.3, r));
                uint32_t e = 0;
                CRT_CUDA(cudaMemcpy(&e, err, 4, cudaMemcpyDeviceToHost));
                if (e) break;
            }
        }
    }
    if (!laid_out) CRT_CUDA(cudaEventRecord(x->ev[3], s));

    // ---- K4: DFS layout, last PLOC iteration first (done above on the persistent path)
    if (N == 1) {
        crt::launch_single_leaf(x->node_box.as<float4>(), b->nodes.as<crt_bvh_node>(), leaves, s);
    } else if (!laid_out) {
        uint32_t* dfs = x->clus_a.as<uint32_t>();  // the cluster buffers are free after PLOC
        for (int k = static_cast<int>(iters) - 1; k >= 0; --k)
            crt::launch_layout_level(x->node_kids.as<uint4>(), x->pos.as<uint2>(),
                                     x->it_host[k].y, x->it_host[k + 1].y, N, dfs, err, s);
        crt::launch_layout_emit(x->node_box.as<float4>(), x->node_kids.as<uint4>(), x->pos.as<uint2>(), N, dfs,
                                b->nodes.as<crt_bvh_node>(), b->wide.as<float4>(), b->wide_wt.as<float4>(),
                                b->depth_odd.as<uint8_t>(), leaves, st, err, s);
    }
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaEventRecord(x->ev[4], s));
    CRT_TRY(x->check_device_error());

    crt::SceneState hs;
    CRT_CUDA(cudaMemcpy(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost));
    float ms[4];
    for (int k = 0; k < 4; ++k) CRT_CUDA(cudaEventElapsedTime(&ms[k], x->ev[k], x->ev[k + 1]));
    x->stats.n_tris = N;
    x->stats.ploc_iterations = iters;
    x->stats.ms_morton = ms[0];
    x->stats.ms_sort = ms[1];
    x->stats.ms_ploc = ms[2] - layout_in_kernel_ms;
    x->stats.ms_layout = ms[3] + layout_in_kernel_ms;
    x->stats.ms_total = ms[0] + ms[1] + ms[2] + ms[3];
    for (int a = 0; a < 3; ++a) {
        x->stats.scene_box[a] = hs.scene_min[a];
        x->stats.scene_box[3 + a] = hs.scene_max[a];
    }
    b->n = N;
    b->depth_bound = iters;
    b->has_sort = true;
    b->abs_eps = hs.abs_eps;  // the value the layout grew the watertight nodes by
    b->ctx = x;
    return CRT_OK;
}

crt_status copy_out(crt_ctx* x, void* dst, const void* src, size_t bytes) {
    if (!dst) return fail(CRT_ERR_INVALID_ARG, "null destination");
    CRT_CUDA(cudaMemcpyAsync(dst, src, bytes, is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status check_trace_flags(const crt_bvh* b, uint32_t flags) {
    if (flags & ~(CRT_TRACE_ANY | CRT_TRI_WATERTIGHT | CRT_TRACE_USE_PREDICTOR | CRT_TRACE_STATS | CRT_TRACE_WIDE |
                  CRT_TRACE_PREDICTOR_ORDER | CRT_TRACE_SORT_RAYS | CRT_TRACE_COMPRESSED | CRT_TRACE_PER_RAY_THREADS))
        return fail(CRT_ERR_INVALID_ARG, "crt_trace: unknown flags 0x%x", flags);
    if ((flags & (CRT_TRACE_USE_PREDICTOR | CRT_TRACE_PREDICTOR_ORDER)) && !b->predictor)
        return fail(CRT_ERR_UNSUPPORTED, "crt_trace: no predictor bound to this bvh (crt_predictor_create)");
    if (b->n == 0) return fail(CRT_ERR_INVALID_ARG, "crt_trace: empty bvh");
    return CRT_OK;
}

// Derives the 4-wide traversal nodes of b on x's stream if the last build
// has not yet done so.
crt_status ensure_wide4(crt_ctx* x, const crt_bvh* b) {
    if (b->wide4_ready || b->n <= 1) return CRT_OK;
    CRT_TRY(b->wide4.reserve(128ull * b->n));
    crt::launch_wide4(b->wide.as<float4>(), b->depth_odd.as<uint8_t>(), b->n - 1, b->wide4.as<float4>(), x->stream);
    CRT_CUDA(cudaGetLastError());
    b->wide4_ready = true;
    return CRT_OK;
}

// Derives the compressed 4-wide traversal nodes of b on x's stream if the
// last build (or refit) has not yet done so.
crt_status ensure_cwide(crt_ctx* x, const crt_bvh* b) {
    if (b->cwide_ready || b->n <= 1) return CRT_OK;
    CRT_TRY(b->cwide.reserve(64ull * b->n));
    crt::launch_cwide(b->wide.as<float4>(), b->depth_odd.as<uint8_t>(), b->n - 1, b->cwide.as<uint4>(),
                      x->err.as<uint32_t>(), x->stream);
    CRT_CUDA(cudaGetLastError());
    b->cwide_ready = true;
    return CRT_OK;
}

// Enqueues one traversal launch on device-resident rays/hits (no sync).
constexpr uint32_t kPoolMinRays = 65536;  // below this a launch of one thread per ray fills the GPU as well
constexpr uint32_t kChunkedCopyMinRays = 1u << 20;  // crt_trace: smaller host batches copy in one piece

// classes_ready: the predictor's classes of these rays are already in its
// class buffer, and with CRT_TRACE_PREDICTOR_ORDER their order keys in its
// order scratch (crt_trace's chunked copy ran the inference per chunk).
crt_status trace_device(crt_ctx* x, const crt_bvh* b, const crt_ray* d_rays, uint32_t n_rays, uint32_t flags,
                        crt_hit* d_hits, const uint16_t* seed_classes = nullptr, uint32_t tile_width = 0,
                        bool classes_ready = false) {
    if (n_rays == 0) return CRT_OK;
    if (flags & CRT_TRACE_WIDE) CRT_TRY(ensure_wide4(x, b));
    if (flags & CRT_TRACE_COMPRESSED) CRT_TRY(ensure_cwide(x, b));
    x->tev_valid = false;
    CRT_CUDA(cudaEventRecord(x->tev[0], x->stream));
    crt::TraceParams p{};
    p.nodes = b->nodes.as<crt_bvh_node>();
    p.xtri = b->xtri.as<float4>();
    p.wide = (flags & CRT_TRI_WATERTIGHT) ? b->wide_wt.as<float4>() : b->wide.as<float4>();
    p.wide4 = (b->n > 1) ? b->wide4.as<float4>() : nullptr;
    p.cwide = (b->n > 1 && (flags & CRT_TRACE_COMPRESSED)) ? b->cwide.as<uint4>() : nullptr;
    p.rays = d_rays;
    p.hits = d_hits;
    p.n_rays = n_rays;
    p.n_nodes = 2 * b->n - 1;
    p.abs_eps = b->abs_eps;
    p.err = x->err.as<uint32_t>();
    p.stats = nullptr;
    p.tile_width = tile_width;
    if (flags & CRT_TRACE_STATS) {
        CRT_CUDA(cudaMemsetAsync(x->trace_stats.p, 0, 16, x->stream));
        p.stats = x->trace_stats.as<unsigned long long>();
    }
    if (seed_classes) {
        p.pred_class = seed_classes;
        p.treelets = b->predictor->treelets.as<crt::Treelet>();
        p.n_treelets = reinterpret_cast<const uint32_t*>(b->predictor->treelets.as<crt::Treelet>() + 128);
    } else if (flags & (CRT_TRACE_USE_PREDICTOR | CRT_TRACE_PREDICTOR_ORDER)) {
        crt_predictor* pr = b->predictor;
        CRT_TRY(pr->classes.reserve(2ull * n_rays));
        // ordering alone needs only the likeliest class, and then the inference
        // also writes the trace order keys; seeding needs the miss rule
        const bool fuse = (flags & CRT_TRACE_PREDICTOR_ORDER) && !(flags & CRT_TRACE_USE_PREDICTOR);
        if (flags & CRT_TRACE_PREDICTOR_ORDER) {
            CRT_TRY(pr->order.reserve(4ull * n_rays));
            CRT_TRY(pr->order_scratch.reserve(crt::pred_order_scratch_bytes(n_rays)));
        }
        if (!classes_ready) {
            uint32_t *okeys = nullptr, *ohist = nullptr;
            if (fuse) crt::pred_order_begin(pr->order_scratch.p, n_rays, &okeys, &ohist, x->stream);
            CRT_CUDA(crt::pred_infer(pr->dev(), b->nodes.as<crt_bvh_node>(), d_rays, n_rays, pr->classes.as<uint16_t>(),
                                     pr->cfg.miss_threshold, !(flags & CRT_TRACE_USE_PREDICTOR), x->err.as<uint32_t>(),
                                     x->stream, okeys, ohist));
        }
        if (flags & CRT_TRACE_USE_PREDICTOR) {
            p.pred_class = pr->classes.as<uint16_t>();
            p.treelets = pr->treelets.as<crt::Treelet>();
            p.n_treelets = reinterpret_cast<const uint32_t*>(pr->treelets.as<crt::Treelet>() + 128);
        }
        if (flags & CRT_TRACE_PREDICTOR_ORDER) {  // includes the coherence order of CRT_TRACE_SORT_RAYS
            crt::pred_order(pr->dev(), b->nodes.as<crt_bvh_node>(), d_rays, pr->classes.as<uint16_t>(), n_rays,
                            pr->order.as<uint32_t>(), pr->order_scratch.p, x->err.as<uint32_t>(), x->cfg.spin_limit,
                            x->stream, fuse);
            CRT_CUDA(cudaGetLastError());
            p.order = pr->order.as<uint32_t>();
        }
    }
    if ((flags & CRT_TRACE_SORT_RAYS) && !p.order && n_rays > 1) {
        CRT_TRY(x->ray_order.reserve(4ull * n_rays));
        CRT_TRY(x->ray_order_scratch.reserve(crt::ray_order_scratch_bytes(n_rays)));
        crt::launch_ray_order(d_rays, n_rays, b->nodes.as<crt_bvh_node>(), nullptr, 0, x->ray_order.as<uint32_t>(),
                              x->ray_order_scratch.p, x->err.as<uint32_t>(), x->cfg.spin_limit, x->stream);
        CRT_CUDA(cudaGetLastError());
        p.order = x->ray_order.as<uint32_t>();
    }
    // binary walk: stack <= tree height <= PLOC iterations + 1; 4-wide walk: <= 3 per two levels
    const bool deep = (b->depth_bound + 2 > 64) || (3 * ((b->depth_bound + 2) / 2) + 3 > 96);
    const uint32_t launch_flags =
        (flags & (CRT_TRACE_ANY | CRT_TRI_WATERTIGHT | CRT_TRACE_WIDE | CRT_TRACE_COMPRESSED)) | (deep ? (1u << 16) : 0u);
    // Large closest-hit batches over the binary nodes: persistent warps that
    // refill finished lanes (the rays of a batch differ widely in walk
    // length); pixels in 8x4 tiles, any-hit, seeded and wide walks keep one
    // thread per ray, which shares node fetches between a tile's rays.
    const bool pool = !(flags & (CRT_TRACE_ANY | CRT_TRACE_WIDE | CRT_TRACE_COMPRESSED | CRT_TRACE_PER_RAY_THREADS)) &&
                      !p.pred_class && tile_width == 0 && n_rays >= kPoolMinRays;
    if (pool) CRT_TRY(x->pool_counter.reserve(16));
    CRT_CUDA(cudaEventRecord(x->tev[1], x->stream));
    if (pool) crt::launch_trace_pool(p, launch_flags, x->pool_counter.as<uint32_t>(), x->stream);
    else crt::launch_trace(p, launch_flags, static_cast<int>(x->cfg.trace_block), x->stream);
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaEventRecord(x->tev[2], x->stream));
    x->tev_valid = true;
    return CRT_OK;
}

}  // namespace

extern "C" {

crt_status crt_build(crt_ctx* x, const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                     const crt_mesh_model* models, uint32_t n_models, crt_bvh** out) {
    if (!x || !out) return fail(CRT_ERR_INVALID_ARG, "crt_build: null context or output");
    *out = nullptr;
    crt_bvh* b = new crt_bvh();
    const crt_status s = build_impl(x, b, tris, n_buffer, n_tris, models, n_models);
    if (s != CRT_OK) {
        crt_bvh_free(b);
        return s;
    }
    *out = b;
    return CRT_OK;
}

crt_status crt_rebuild(crt_ctx* x, crt_bvh* b, const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                       const crt_mesh_model* models, uint32_t n_models) {
    if (!x || !b) return fail(CRT_ERR_INVALID_ARG, "crt_rebuild: null context or bvh");
    return build_impl(x, b, tris, n_buffer, n_tris, models, n_models);
}

// Brings the node array's boxes up to date after a refit (on x's stream).
static crt_status ensure_node_boxes(crt_ctx* x, const crt_bvh* b) {
    if (!b->node_boxes_stale) return CRT_OK;
    crt::launch_refit_nodes(b->wide.as<float4>(), b->refit_dfs.as<uint32_t>(), b->n,
                            const_cast<crt_bvh_node*>(b->nodes.as<crt_bvh_node>()), x->err.as<uint32_t>(), x->stream);
    CRT_CUDA(cudaGetLastError());
    b->node_boxes_stale = false;
    return CRT_OK;
}

crt_status crt_refit(crt_ctx* x, crt_bvh* b, const crt_triangle* tris, uint32_t n_tris, const crt_mesh_model* models,
                     uint32_t n_models) {
    if (!x || !b || !tris) return fail(CRT_ERR_INVALID_ARG, "crt_refit: null argument");
    if (b->n == 0 || n_tris != b->n)
        return fail(CRT_ERR_INVALID_ARG, "crt_refit: %u triangles for a bvh built over %u", n_tris, b->n);
    if (n_models > crt::kMaxModels) return fail(CRT_ERR_INVALID_ARG, "crt_refit: more than 64 models");
    if (n_models > 0 && !models) return fail(CRT_ERR_INVALID_ARG, "crt_refit: null models");
    CRT_CUDA(cudaSetDevice(x->device));
    cudaStream_t s = x->stream;
    const uint32_t N = b->n;
    const crt_triangle* d_tris = tris;
    if (!is_device_ptr(tris)) {
        CRT_TRY(x->tris_in.reserve(sizeof(crt_triangle) * static_cast<size_t>(N)));
        CRT_CUDA(cudaMemcpyAsync(x->tris_in.p, tris, sizeof(crt_triangle) * static_cast<size_t>(N), cudaMemcpyHostToDevice, s));
        d_tris = x->tris_in.as<crt_triangle>();
    } else {
        CRT_TRY(check_aligned16(tris, "crt_refit: triangles"));
    }
    CRT_TRY(stage_model_matrices(x, models, n_models));
    CRT_TRY(x->refit_state.reserve(sizeof(crt::RefitState)));
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, s));
    if (!b->refit_ready) {
        const size_t n_int = std::max<size_t>(N - 1, 1);
        CRT_TRY(b->refit_leaf.reserve(16ull * N));
        CRT_TRY(b->refit_link.reserve(16ull * n_int));
        CRT_TRY(b->refit_dfs.reserve(4ull * n_int));
        CRT_TRY(b->refit_cnt.reserve(4ull * std::max<size_t>(n_int, crt::refit_topo_blocks(N))));
        // the counters' buffer holds the per-block counts of the topology pass first
        crt::launch_refit_topology(b->nodes.as<crt_bvh_node>(), b->wide.as<float4>(), N, b->refit_leaf.as<uint4>(),
                                   b->refit_link.as<uint4>(), b->refit_dfs.as<uint32_t>(), b->refit_cnt.as<uint32_t>(),
                                   x->err.as<uint32_t>(), s);
        CRT_CUDA(cudaGetLastError());
        b->refit_ready = true;
    }
    if (N > 1) CRT_CUDA(cudaMemsetAsync(b->refit_cnt.p, 0, 4ull * (N - 1), s));
    crt::launch_refit(d_tris, N, x->models.as<float>(), b->refit_leaf.as<uint4>(), b->refit_link.as<uint4>(),
                      b->refit_cnt.as<uint32_t>(), b->nodes.as<crt_bvh_node>(), b->xtri.as<float4>(),
                      b->wide.as<float4>(), b->wide_wt.as<float4>(), x->refit_state.as<crt::RefitState>(),
                      x->err.as<uint32_t>(), s);
    CRT_CUDA(cudaGetLastError());
    float* h_eps = static_cast<float*>(x->pinned);
    CRT_CUDA(cudaMemcpyAsync(h_eps, &x->refit_state.as<crt::RefitState>()->abs_eps, sizeof(float),
                             cudaMemcpyDeviceToHost, s));
    b->wide4_ready = false;
    b->cwide_ready = false;
    b->node_boxes_stale = N > 1;
    const crt_status st = x->check_device_error();
    if (st != CRT_OK) {
        b->refit_ready = false;  // derive the topology again next time
        return st;
    }
    b->abs_eps = *h_eps;
    return CRT_OK;
}

// The structure check and numbering of a caller's DFS node array (host copy
// h of n_nodes records over N triangles), shared by crt_validate_nodes and
// crt_bvh_from_nodes.  DFS pre-order, left child first (scene.cpp:189-208):
// an internal node at d has its left child at d + 1 and its right child
// after the left subtree; a leaf (both children 0, raytracer.glsl:239-244)
// names one triangle, each triangle once.  Leaves and internal nodes are
// numbered in order of position.
struct NodeNumbering {
    std::vector<uint32_t> idx, int_pos, leaf_pos;
    std::vector<uint2> lc;
    std::vector<uint8_t> odd;
    uint32_t max_depth = 0;
};

static crt_status number_nodes(const crt_bvh_node* h, uint32_t n_nodes, uint32_t N, const char* fn, NodeNumbering* out) {
    if (N == 0 || N > (1u << 30)) return fail(CRT_ERR_INVALID_ARG, "%s: n_tris must be in [1, 2^30]", fn);
    if (n_nodes != 2 * N - 1) return fail(CRT_ERR_INVALID_ARG, "%s: %u nodes for %u triangles (need 2n-1)", fn, n_nodes, N);
    NodeNumbering& o = *out;
    o.idx.assign(n_nodes, 0);
    o.int_pos.assign(N > 1 ? N - 1 : 1, 0);
    o.leaf_pos.assign(N, 0);
    o.lc.assign(N > 1 ? N - 1 : 1, make_uint2(0u, 0u));
    o.odd.assign(N > 1 ? N - 1 : 1, 0);
    o.max_depth = 0;
    std::vector<uint32_t> leaves(n_nodes, 0), dep(n_nodes, 0);
    std::vector<uint8_t> seen(N, 0), referenced(n_nodes, 0);
    uint32_t n_leaf = 0, n_int = 0;
    for (uint32_t d = 0; d < n_nodes; ++d) {
        const crt_bvh_node& nd = h[d];
        if (d > 0 && !referenced[d]) return fail(CRT_ERR_INVALID_ARG, "%s: node %u is no node's child", fn, d);
        if (nd.left == 0 && nd.right == 0) {
            if (nd.tri >= N) return fail(CRT_ERR_INVALID_ARG, "%s: leaf %u names triangle %u", fn, d, nd.tri);
            if (seen[nd.tri]) return fail(CRT_ERR_INVALID_ARG, "%s: triangle %u in two leaves", fn, nd.tri);
            seen[nd.tri] = 1;
            if (n_leaf >= N) return fail(CRT_ERR_INVALID_ARG, "%s: more than %u leaves", fn, N);
            o.idx[d] = n_leaf;
            o.leaf_pos[n_leaf++] = d;
        } else {
            if (nd.left != d + 1 || nd.right <= nd.left || nd.right >= n_nodes || referenced[nd.left] ||
                referenced[nd.right])
                return fail(CRT_ERR_INVALID_ARG, "%s: node %u is not in DFS pre-order (children %u, %u)", fn, d, nd.left,
                            nd.right);
            if (n_int + 1 >= N) return fail(CRT_ERR_INVALID_ARG, "%s: more than %u internal nodes", fn, N - 1);
            referenced[nd.left] = referenced[nd.right] = 1;
            dep[nd.left] = dep[nd.right] = dep[d] + 1;
            o.max_depth = std::max(o.max_depth, dep[d] + 1);
            o.idx[d] = n_int;
            o.int_pos[n_int++] = d;
        }
    }
    if (n_leaf != N || n_int != N - 1)
        return fail(CRT_ERR_INVALID_ARG, "%s: %u leaves and %u internal nodes for %u triangles", fn, n_leaf, n_int, N);
    for (uint32_t d = n_nodes; d-- > 0;) {  // children follow their parent: a reverse sweep counts leaves
        const crt_bvh_node& nd = h[d];
        if (nd.left == 0 && nd.right == 0) {
            leaves[d] = 1;
            continue;
        }
        leaves[d] = leaves[nd.left] + leaves[nd.right];
        if (nd.right != nd.left + 2 * leaves[nd.left] - 1)
            return fail(CRT_ERR_INVALID_ARG, "%s: node %u's right child does not follow its left subtree", fn, d);
        o.lc[o.idx[d]] = make_uint2(leaves[nd.left], leaves[nd.right]);
        o.odd[o.idx[d]] = static_cast<uint8_t>(dep[d] & 1u);
    }
    if (leaves[0] != N) return fail(CRT_ERR_INVALID_ARG, "%s: the root holds %u of %u leaves", fn, leaves[0], N);
    return CRT_OK;
}

// A host copy of the caller's node array (host or device memory).
static crt_status host_nodes(const crt_bvh_node* nodes, uint32_t n_nodes, std::vector<crt_bvh_node>* h) {
    h->resize(n_nodes);
    if (is_device_ptr(nodes)) {
        CRT_CUDA(cudaMemcpy(h->data(), nodes, sizeof(crt_bvh_node) * n_nodes, cudaMemcpyDeviceToHost));
    } else {
        std::memcpy(h->data(), nodes, sizeof(crt_bvh_node) * n_nodes);
    }
    return CRT_OK;
}

crt_status crt_validate_nodes(const crt_bvh_node* nodes, uint32_t n_nodes, uint32_t n_tris, uint32_t info[4]) {
    if (!nodes) return fail(CRT_ERR_INVALID_ARG, "crt_validate_nodes: null nodes");
    if (n_tris == 0 || n_nodes != 2 * n_tris - 1)
        return fail(CRT_ERR_INVALID_ARG, "crt_validate_nodes: %u nodes for %u triangles (need 2n-1)", n_nodes, n_tris);
    std::vector<crt_bvh_node> h;
    CRT_TRY(host_nodes(nodes, n_nodes, &h));
    NodeNumbering num;
    CRT_TRY(number_nodes(h.data(), n_nodes, n_tris, "crt_validate_nodes", &num));
    if (info) {
        info[0] = n_tris;
        info[1] = n_tris - 1;
        info[2] = num.max_depth;
        info[3] = 0;
    }
    return CRT_OK;
}

crt_status crt_bvh_from_nodes(crt_ctx* x, const crt_bvh_node* nodes, uint32_t n_nodes, const crt_triangle* tris,
                              uint32_t n_tris, const crt_mesh_model* models, uint32_t n_models, crt_bvh** out) {
    if (!x || !nodes || !tris || !out) return fail(CRT_ERR_INVALID_ARG, "crt_bvh_from_nodes: null argument");
    *out = nullptr;
    if (n_tris == 0 || n_tris > (1u << 30))
        return fail(CRT_ERR_INVALID_ARG, "crt_bvh_from_nodes: n_tris must be in [1, 2^30]");
    if (n_nodes != 2 * n_tris - 1)
        return fail(CRT_ERR_INVALID_ARG, "crt_bvh_from_nodes: %u nodes for %u triangles (need 2n-1)", n_nodes, n_tris);
    if (n_models > crt::kMaxModels) return fail(CRT_ERR_INVALID_ARG, "crt_bvh_from_nodes: more than 64 models");
    if (n_models > 0 && !models) return fail(CRT_ERR_INVALID_ARG, "crt_bvh_from_nodes: null models");
    CRT_CUDA(cudaSetDevice(x->device));
    cudaStream_t s = x->stream;
    const uint32_t N = n_tris;
    if (is_device_ptr(tris)) CRT_TRY(check_aligned16(tris, "crt_bvh_from_nodes: triangles"));
    // the array on the host, for the structure check and the numbering
    std::vector<crt_bvh_node> h;
    CRT_TRY(host_nodes(nodes, n_nodes, &h));
    NodeNumbering num;
    CRT_TRY(number_nodes(h.data(), n_nodes, N, "crt_bvh_from_nodes", &num));
    const std::vector<uint32_t>& idx = num.idx;
    const std::vector<uint32_t>& int_pos = num.int_pos;
    const std::vector<uint32_t>& leaf_pos = num.leaf_pos;
    const std::vector<uint2>& lc = num.lc;
    const std::vector<uint8_t>& odd = num.odd;
    const uint32_t max_depth = num.max_depth;

    crt_bvh* b = new crt_bvh();
    auto fail_free = [&](crt_status st) {
        crt_bvh_free(b);
        return st;
    };
    const size_t n_int_alloc = std::max<size_t>(N - 1, 1);
    crt_status st = CRT_OK;
    if ((st = b->nodes.reserve(sizeof(crt_bvh_node) * n_nodes)) != CRT_OK || (st = b->xtri.reserve(48ull * N)) != CRT_OK ||
        (st = b->wide.reserve(64ull * n_int_alloc)) != CRT_OK || (st = b->wide_wt.reserve(64ull * n_int_alloc)) != CRT_OK ||
        (st = b->depth_odd.reserve(n_int_alloc)) != CRT_OK || (st = b->inv_perm.reserve(4ull * N)) != CRT_OK)
        return fail_free(st);
    // staging: idx (n_nodes) | int_pos (N-1) | leaf counts (N-1, uint2) | leaf_pos (N), each part
    // starting on a 256-byte boundary (the uint2 loads need 8-byte alignment)
    auto up256 = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t o_int = up256(4ull * n_nodes), o_lc = up256(o_int + 4ull * n_int_alloc),
                 o_leaf = up256(o_lc + 8ull * n_int_alloc), bytes = o_leaf + 4ull * N;
    if ((st = x->opt_scratch.reserve(bytes)) != CRT_OK) return fail_free(st);
    char* base = x->opt_scratch.as<char>();
    if ((st = stage_model_matrices(x, models, n_models)) != CRT_OK) return fail_free(st);
    const crt_triangle* d_tris = tris;
    if (!is_device_ptr(tris)) {
        if ((st = x->tris_in.reserve(sizeof(crt_triangle) * static_cast<size_t>(N))) != CRT_OK) return fail_free(st);
        if (cudaMemcpyAsync(x->tris_in.p, tris, sizeof(crt_triangle) * static_cast<size_t>(N), cudaMemcpyHostToDevice, s) !=
            cudaSuccess)
            return fail_free(fail(CRT_ERR_CUDA, "crt_bvh_from_nodes: triangle upload failed"));
        d_tris = x->tris_in.as<crt_triangle>();
    }
    const cudaError_t ce[6] = {
        cudaMemcpyAsync(b->nodes.p, h.data(), sizeof(crt_bvh_node) * n_nodes, cudaMemcpyHostToDevice, s),
        cudaMemcpyAsync(base, idx.data(), 4ull * n_nodes, cudaMemcpyHostToDevice, s),
        cudaMemcpyAsync(base + o_int, int_pos.data(), 4ull * n_int_alloc, cudaMemcpyHostToDevice, s),
        cudaMemcpyAsync(base + o_lc, lc.data(), 8ull * n_int_alloc, cudaMemcpyHostToDevice, s),
        cudaMemcpyAsync(base + o_leaf, leaf_pos.data(), 4ull * N, cudaMemcpyHostToDevice, s),
        cudaMemcpyAsync(b->depth_odd.p, odd.data(), n_int_alloc, cudaMemcpyHostToDevice, s)};
    for (cudaError_t e : ce)
        if (e != cudaSuccess) return fail_free(fail(CRT_ERR_CUDA, "crt_bvh_from_nodes: upload failed: %s", cudaGetErrorString(e)));
    // the traversal slack of the root box, as a refit derives it
    const float smin[3] = {h[0].mn[0], h[0].mn[1], h[0].mn[2]}, smax[3] = {h[0].mx[0], h[0].mx[1], h[0].mx[2]};
    const float grow = crt::scene_abs_eps(smin, smax);
    if (cudaMemsetAsync(x->err.p, 0, 16, s) != cudaSuccess) return fail_free(fail(CRT_ERR_CUDA, "crt_bvh_from_nodes: memset"));
    crt::launch_import(b->nodes.as<crt_bvh_node>(), N, reinterpret_cast<const uint32_t*>(base),
                       reinterpret_cast<const uint32_t*>(base + o_int), reinterpret_cast<const uint2*>(base + o_lc),
                       reinterpret_cast<const uint32_t*>(base + o_leaf), d_tris, x->models.as<float>(), grow,
                       b->wide.as<float4>(), b->wide_wt.as<float4>(), b->xtri.as<float4>(), b->inv_perm.as<uint32_t>(),
                       x->err.as<uint32_t>(), s);
    if (cudaGetLastError() != cudaSuccess) return fail_free(fail(CRT_ERR_CUDA, "crt_bvh_from_nodes: launch failed"));
    if ((st = x->check_device_error()) != CRT_OK) return fail_free(st);  // synchronises: the host arrays may go
    b->n = N;
    b->depth_bound = max_depth;
    b->abs_eps = grow;
    b->has_sort = false;
    b->ctx = x;
    *out = b;
    return CRT_OK;
}

crt_status crt_optimize(crt_ctx* x, crt_bvh* b, uint32_t passes) {
    if (!x || !b) return fail(CRT_ERR_INVALID_ARG, "crt_optimize: null context or bvh");
    if (b->n == 0) return fail(CRT_ERR_INVALID_ARG, "crt_optimize: empty bvh");
    if (passes > CRT_OPTIMIZE_MAX_PASSES)
        return fail(CRT_ERR_INVALID_ARG, "crt_optimize: %u passes (at most %u)", passes, CRT_OPTIMIZE_MAX_PASSES);
    const uint32_t N = b->n;
    if (N < 2) return CRT_OK;
    CRT_CUDA(cudaSetDevice(x->device));
    cudaStream_t s = x->stream;
    uint32_t* err = x->err.as<uint32_t>();
    // scratch: per id (2N-1) two boxes, cost, leaf count, height, parent; per
    // internal node (N-1) children twice, child areas, counter, new id, layout position;
    // DFS table (2N-1); leaf records (N); scene slack
    const size_t n_id = 2ull * N - 1, n_int = N - 1;
    size_t off = 0;
    auto carve = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    const size_t o_box = carve(32 * n_id), o_box2 = carve(32 * n_id), o_cost = carve(4 * n_id), o_nl = carve(4 * n_id),
                 o_h = carve(4 * n_id), o_par = carve(4 * n_id), o_kids = carve(16 * n_int), o_kids2 = carve(16 * n_int),
                 o_karea = carve(8 * n_int), o_cnt = carve(4 * n_int), o_new = carve(4 * n_int), o_pf = carve(8 * n_int),
                 o_dfs = carve(4 * n_id), o_xtri = carve(48ull * N), o_st = carve(sizeof(crt::SceneState)),
                 o_hist = carve(4 * (n_id + 1));
    CRT_TRY(x->opt_scratch.reserve(off));
    char* base = x->opt_scratch.as<char>();
    crt::OptView v;
    v.box = reinterpret_cast<float4*>(base + o_box);
    v.cost = reinterpret_cast<float*>(base + o_cost);
    v.nl = reinterpret_cast<uint32_t*>(base + o_nl);
    v.height = reinterpret_cast<uint32_t*>(base + o_h);
    v.parent = reinterpret_cast<uint32_t*>(base + o_par);
    v.kids = reinterpret_cast<uint4*>(base + o_kids);
    v.karea = reinterpret_cast<float2*>(base + o_karea);
    v.cnt = reinterpret_cast<uint32_t*>(base + o_cnt);
    v.N = N;
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, s));
    crt::launch_opt_init(b->wide.as<float4>(), b->xtri.as<float4>(), v, err, s);
    for (uint32_t k = 0; k < passes; ++k) crt::launch_opt_pass(v, true, err, s);
    if (passes == 0) crt::launch_opt_pass(v, false, err, s);
    CRT_CUDA(cudaGetLastError());
    uint32_t H = 0;
    CRT_CUDA(cudaMemcpyAsync(&H, v.height + N, 4, cudaMemcpyDeviceToHost, s));
    CRT_TRY(x->check_device_error());  // synchronises: H is read
    if (H == 0 || H > N - 1) return fail(CRT_ERR_CUDA, "crt_optimize: root height %u for %u leaves", H, N);
    // internal nodes bucketed by height, the root (unique at height H) last
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + o_hist);
    CRT_CUDA(cudaMemsetAsync(hist, 0, 4ull * (H + 1), s));
    crt::launch_opt_hist(v, H, hist, err, s);
    std::vector<uint32_t> h_hist(H + 2, 0);
    CRT_CUDA(cudaMemcpyAsync(h_hist.data(), hist, 4ull * (H + 1), cudaMemcpyDeviceToHost, s));
    CRT_TRY(x->check_device_error());
    std::vector<uint32_t> h_off(H + 2, 0);
    for (uint32_t h = 1; h <= H + 1; ++h) h_off[h] = h_off[h - 1] + h_hist[h - 1];
    if (h_off[H + 1] != N - 1 || h_hist[H] != 1u || h_hist[0] != 0u)
        return fail(CRT_ERR_CUDA, "crt_optimize: height histogram inconsistent (%u of %u nodes)", h_off[H + 1], N - 1);
    CRT_CUDA(cudaMemcpyAsync(hist, h_off.data(), 4ull * (H + 1), cudaMemcpyHostToDevice, s));
    uint4* kids2 = reinterpret_cast<uint4*>(base + o_kids2);
    float4* box2 = reinterpret_cast<float4*>(base + o_box2);
    crt::launch_opt_relabel(v, H, hist, reinterpret_cast<uint32_t*>(base + o_new), kids2, box2, err, s);
    // the leaf records move from the current tree order to the new one
    float4* xtri_old = reinterpret_cast<float4*>(base + o_xtri);
    CRT_CUDA(cudaMemcpyAsync(xtri_old, b->xtri.p, 48ull * N, cudaMemcpyDeviceToDevice, s));
    crt::SceneState hst{};
    hst.abs_eps = b->abs_eps;  // the slack the watertight nodes are grown by stays the tree's own
    crt::SceneState* st = reinterpret_cast<crt::SceneState*>(base + o_st);
    CRT_CUDA(cudaMemcpyAsync(st, &hst, sizeof(hst), cudaMemcpyHostToDevice, s));
    uint2* pf = reinterpret_cast<uint2*>(base + o_pf);
    uint32_t* dfs = reinterpret_cast<uint32_t*>(base + o_dfs);
    for (uint32_t h = H; h >= 1; --h)
        crt::launch_layout_level(kids2, pf, N + h_off[h], N + h_off[h + 1], N, dfs, err, s);
    crt::LeafOut leaves{xtri_old, b->xtri.as<float4>(), b->inv_perm.as<uint32_t>()};
    crt::launch_layout_emit(box2, kids2, pf, N, dfs, b->nodes.as<crt_bvh_node>(), b->wide.as<float4>(),
                            b->wide_wt.as<float4>(), b->depth_odd.as<uint8_t>(), leaves, st, err, s);
    CRT_CUDA(cudaGetLastError());
    b->wide4_ready = false;
    b->cwide_ready = false;
    b->refit_ready = false;
    b->node_boxes_stale = false;
    b->depth_bound = H;
    return x->check_device_error();  // also keeps the host staging alive until the copies ran
}

crt_status crt_bvh_free(crt_bvh* b) {
    if (!b) return CRT_OK;
    b->nodes.release();
    b->xtri.release();
    b->wide.release();
    b->wide_wt.release();
    b->wide4.release();
    b->cwide.release();
    b->depth_odd.release();
    b->inv_perm.release();
    if (b->predictor) b->predictor->bvh = nullptr;
    b->codes.release();
    b->perm.release();
    b->refit_link.release();
    b->refit_leaf.release();
    b->refit_dfs.release();
    b->refit_cnt.release();
    delete b;
    return CRT_OK;
}

uint32_t crt_bvh_node_count(const crt_bvh* b) { return (b && b->n) ? 2 * b->n - 1 : 0; }
uint32_t crt_bvh_triangle_count(const crt_bvh* b) { return b ? b->n : 0; }
const crt_bvh_node* crt_bvh_nodes_device(const crt_bvh* b) {
    if (!b) return nullptr;
    if (b->ctx && ensure_node_boxes(b->ctx, b) != CRT_OK) return nullptr;
    if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
    return b->nodes.as<crt_bvh_node>();
}

crt_status crt_bvh_copy_nodes(crt_ctx* x, const crt_bvh* b, crt_bvh_node* dst) {
    if (!x || !b) return fail(CRT_ERR_INVALID_ARG, "null context or bvh");
    CRT_TRY(ensure_node_boxes(x, b));
    return copy_out(x, dst, b->nodes.p, sizeof(crt_bvh_node) * (2ull * b->n - 1));
}
crt_status crt_bvh_copy_codes(crt_ctx* x, const crt_bvh* b, uint32_t* dst) {
    if (!x || !b) return fail(CRT_ERR_INVALID_ARG, "null context or bvh");
    if (!b->has_sort) return fail(CRT_ERR_INVALID_ARG, "crt_bvh_copy_codes: this tree was not built here (no Morton sort)");
    return copy_out(x, dst, b->codes.p, 4ull * b->n);
}
crt_status crt_bvh_copy_perm(crt_ctx* x, const crt_bvh* b, uint32_t* dst) {
    if (!x || !b) return fail(CRT_ERR_INVALID_ARG, "null context or bvh");
    if (!b->has_sort) return fail(CRT_ERR_INVALID_ARG, "crt_bvh_copy_perm: this tree was not built here (no Morton sort)");
    return copy_out(x, dst, b->perm.p, 4ull * b->n);
}

crt_status crt_last_build_stats(crt_ctx* x, crt_build_stats* st) {
    if (!x || !st) return fail(CRT_ERR_INVALID_ARG, "null context or stats");
    *st = x->stats;
    return CRT_OK;
}

crt_status crt_raygen_pinhole(crt_ctx* x, const crt_camera* cam, uint32_t width, uint32_t height, crt_ray* rays) {
    if (!x || !cam || !rays) return fail(CRT_ERR_INVALID_ARG, "crt_raygen_pinhole: null argument");
    if (width == 0 || height == 0 || height > 65535) return fail(CRT_ERR_INVALID_ARG, "bad image size");
    CRT_CUDA(cudaSetDevice(x->device));
    const size_t n = static_cast<size_t>(width) * height;
    const crt_camera* d_cam = cam;
    if (!is_device_ptr(cam)) {
        CRT_CUDA(cudaMemcpyAsync(x->cam.p, cam, sizeof(crt_camera), cudaMemcpyHostToDevice, x->stream));
        d_cam = x->cam.as<crt_camera>();
    } else {
        CRT_TRY(check_aligned16(cam, "crt_raygen_pinhole: camera"));
    }
    const bool dev_out = is_device_ptr(rays);
    if (dev_out) CRT_TRY(check_aligned16(rays, "crt_raygen_pinhole: rays"));
    crt_ray* d_rays = rays;
    if (!dev_out) {
        CRT_TRY(x->rays_out.reserve(sizeof(crt_ray) * n));
        d_rays = x->rays_out.as<crt_ray>();
    }
    crt::launch_raygen(d_cam, width, height, d_rays, x->stream);
    CRT_CUDA(cudaGetLastError());
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(rays, d_rays, sizeof(crt_ray) * n, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status crt_shadow_rays(crt_ctx* x, const crt_ray* primary, const crt_hit* hits, uint32_t n, const float light[3],
                           crt_ray* shadow) {
    if (!x || !primary || !hits || !light || !shadow) return fail(CRT_ERR_INVALID_ARG, "crt_shadow_rays: null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    if (n == 0) return CRT_OK;
    const crt_ray* d_prim = primary;
    const crt_hit* d_hits = hits;
    if (is_device_ptr(primary)) CRT_TRY(check_aligned16(primary, "crt_shadow_rays: primary rays"));
    if (is_device_ptr(hits)) CRT_TRY(check_aligned16(hits, "crt_shadow_rays: hits"));
    if (is_device_ptr(shadow)) CRT_TRY(check_aligned16(shadow, "crt_shadow_rays: shadow rays"));
    if (!is_device_ptr(primary)) {
        CRT_TRY(x->rays_in.reserve(sizeof(crt_ray) * n));
        CRT_CUDA(cudaMemcpyAsync(x->rays_in.p, primary, sizeof(crt_ray) * n, cudaMemcpyHostToDevice, x->stream));
        d_prim = x->rays_in.as<crt_ray>();
    }
    if (!is_device_ptr(hits)) {
        CRT_TRY(x->hits_out.reserve(sizeof(crt_hit) * n));
        CRT_CUDA(cudaMemcpyAsync(x->hits_out.p, hits, sizeof(crt_hit) * n, cudaMemcpyHostToDevice, x->stream));
        d_hits = x->hits_out.as<crt_hit>();
    }
    const bool dev_out = is_device_ptr(shadow);
    crt_ray* d_out = shadow;
    if (!dev_out) {
        CRT_TRY(x->rays_out.reserve(sizeof(crt_ray) * n));
        d_out = x->rays_out.as<crt_ray>();
    }
    crt::launch_shadow_rays(d_prim, d_hits, n, light[0], light[1], light[2], d_out, x->stream);
    CRT_CUDA(cudaGetLastError());
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(shadow, d_out, sizeof(crt_ray) * n, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status crt_trace(crt_ctx* x, const crt_bvh* b, const crt_ray* rays, uint32_t n_rays, uint32_t flags, crt_hit* hits) {
    if (!x || !b || !rays || !hits) return fail(CRT_ERR_INVALID_ARG, "crt_trace: null argument");
    CRT_TRY(check_trace_flags(b, flags));
    CRT_CUDA(cudaSetDevice(x->device));
    if (n_rays == 0) return CRT_OK;
    if (is_device_ptr(rays)) CRT_TRY(check_aligned16(rays, "crt_trace: rays"));
    if (is_device_ptr(hits)) CRT_TRY(check_aligned16(hits, "crt_trace: hits"));
    const crt_ray* d_rays = rays;
    bool classes_ready = false;
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    if (!is_device_ptr(rays)) {
        // Page-locked host rays are read in place by the trace kernel when it
        // reads each ray once, in order; reordered or predicted traces read
        // them more than once and out of order, so those copy them in first.
        const bool once = !(flags & (CRT_TRACE_SORT_RAYS | CRT_TRACE_PREDICTOR_ORDER | CRT_TRACE_USE_PREDICTOR));
        const bool learned_order = (flags & CRT_TRACE_PREDICTOR_ORDER) && !(flags & CRT_TRACE_USE_PREDICTOR) &&
                                   b->predictor;
        const bool chunked = learned_order && n_rays >= kChunkedCopyMinRays;
        if (void* m = once ? mapped_host_ptr(const_cast<crt_ray*>(rays)) : nullptr) {
            d_rays = static_cast<const crt_ray*>(m);
        } else if (void* mi = learned_order ? mapped_host_ptr(const_cast<crt_ray*>(rays)) : nullptr) {
            // Ordering by the predictor over page-locked host rays: the inference
            // kernel reads them across the CPU-GPU link itself, once, on every
            // SM under its own work, and stores the device copy the ordering and
            // the trace read (the copy engines alone moved them at about 200 GB/s
            // ahead of the inference).
            crt_predictor* pr = b->predictor;
            CRT_TRY(x->rays_in.reserve(sizeof(crt_ray) * n_rays));
            CRT_TRY(pr->classes.reserve(2ull * n_rays));
            CRT_TRY(pr->order.reserve(4ull * n_rays));
            CRT_TRY(pr->order_scratch.reserve(crt::pred_order_scratch_bytes(n_rays)));
            uint32_t *okeys = nullptr, *ohist = nullptr;
            crt::pred_order_begin(pr->order_scratch.p, n_rays, &okeys, &ohist, x->stream);
            CRT_CUDA(crt::pred_infer(pr->dev(), b->nodes.as<crt_bvh_node>(), static_cast<const crt_ray*>(mi), n_rays,
                                     pr->classes.as<uint16_t>(), pr->cfg.miss_threshold, true, x->err.as<uint32_t>(),
                                     x->stream, okeys, ohist, x->rays_in.as<crt_ray>()));
            d_rays = x->rays_in.as<crt_ray>();
            classes_ready = true;
        } else if (chunked) {
            // Ordering by the predictor over pageable host rays: copy the rays in
            // kCopyChunks pieces on the copy stream and run each piece's inference on the context's
            // stream as soon as it has landed, so the inference hides behind the
            // copy; the ordering and the trace then wait for the last piece.
            crt_predictor* pr = b->predictor;
            CRT_TRY(x->rays_in.reserve(sizeof(crt_ray) * n_rays));
            CRT_TRY(pr->classes.reserve(2ull * n_rays));
            CRT_TRY(pr->order.reserve(4ull * n_rays));
            CRT_TRY(pr->order_scratch.reserve(crt::pred_order_scratch_bytes(n_rays)));
            uint32_t *okeys = nullptr, *ohist = nullptr;  // every piece's order keys, one histogram
            crt::pred_order_begin(pr->order_scratch.p, n_rays, &okeys, &ohist, x->stream);
            crt_ray* dst = x->rays_in.as<crt_ray>();
            CRT_CUDA(cudaEventRecord(x->copy_ev[crt_ctx::kCopyChunks], x->stream));  // earlier readers of rays_in
            CRT_CUDA(cudaStreamWaitEvent(x->copy_stream, x->copy_ev[crt_ctx::kCopyChunks], 0));
            const uint32_t per = ((n_rays + crt_ctx::kCopyChunks - 1) / crt_ctx::kCopyChunks + 127u) & ~127u;
            for (int c = 0; c < crt_ctx::kCopyChunks; ++c) {
                const uint32_t off = static_cast<uint32_t>(c) * per;
                if (off >= n_rays) break;
                const uint32_t cnt = std::min(per, n_rays - off);
                CRT_CUDA(cudaMemcpyAsync(dst + off, rays + off, sizeof(crt_ray) * cnt, cudaMemcpyHostToDevice,
                                         x->copy_stream));
                CRT_CUDA(cudaEventRecord(x->copy_ev[c], x->copy_stream));
                CRT_CUDA(cudaStreamWaitEvent(x->stream, x->copy_ev[c], 0));
                CRT_CUDA(crt::pred_infer(pr->dev(), b->nodes.as<crt_bvh_node>(), dst + off, cnt,
                                         pr->classes.as<uint16_t>() + off, pr->cfg.miss_threshold, true,
                                         x->err.as<uint32_t>(), x->stream, okeys + off, ohist));
            }
            d_rays = dst;
            classes_ready = true;
        } else {
            CRT_TRY(x->rays_in.reserve(sizeof(crt_ray) * n_rays));
            CRT_CUDA(cudaMemcpyAsync(x->rays_in.p, rays, sizeof(crt_ray) * n_rays, cudaMemcpyHostToDevice, x->stream));
            d_rays = x->rays_in.as<crt_ray>();
        }
    }
    bool dev_out = is_device_ptr(hits);
    crt_hit* d_hits = hits;
    if (!dev_out) {  // page-locked host hits: written by the trace kernel itself
        if (void* m = mapped_host_ptr(hits)) {
            d_hits = static_cast<crt_hit*>(m);
            dev_out = true;
        }
    }
    if (!dev_out) {
        CRT_TRY(x->hits_out.reserve(sizeof(crt_hit) * n_rays));
        d_hits = x->hits_out.as<crt_hit>();
    }
    CRT_TRY(trace_device(x, b, d_rays, n_rays, flags, d_hits, nullptr, 0, classes_ready));
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(hits, d_hits, sizeof(crt_hit) * n_rays, cudaMemcpyDeviceToHost, x->stream));
    CRT_TRY(x->check_device_error());
    if (flags & CRT_TRACE_STATS)
        CRT_CUDA(cudaMemcpy(x->last_trace_stats, x->trace_stats.p, 16, cudaMemcpyDeviceToHost));
    return CRT_OK;
}

crt_status crt_trace_seeded(crt_ctx* x, const crt_bvh* b, const crt_ray* rays, uint32_t n_rays, uint32_t flags,
                            const uint16_t* classes, crt_hit* hits) {
    if (!x || !b || !rays || !hits || !classes) return fail(CRT_ERR_INVALID_ARG, "crt_trace_seeded: null argument");
    if (!b->predictor) return fail(CRT_ERR_UNSUPPORTED, "crt_trace_seeded: the bvh has no treelet cut (crt_predictor_create)");
    CRT_TRY(check_trace_flags(b, flags & ~CRT_TRACE_USE_PREDICTOR));
    CRT_CUDA(cudaSetDevice(x->device));
    if (n_rays == 0) return CRT_OK;
    if (!is_device_ptr(rays) || !is_device_ptr(hits) || !is_device_ptr(classes))
        return fail(CRT_ERR_INVALID_ARG, "crt_trace_seeded: rays, classes and hits must be device memory");
    CRT_TRY(check_aligned16(rays, "crt_trace_seeded: rays"));
    CRT_TRY(check_aligned16(hits, "crt_trace_seeded: hits"));
    if (reinterpret_cast<uintptr_t>(classes) & 1u)
        return fail(CRT_ERR_INVALID_ARG, "crt_trace_seeded: classes must be 2-byte aligned");
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    CRT_TRY(trace_device(x, b, rays, n_rays, flags & ~CRT_TRACE_USE_PREDICTOR, hits, classes));
    CRT_TRY(x->check_device_error());
    if (flags & CRT_TRACE_STATS)
        CRT_CUDA(cudaMemcpy(x->last_trace_stats, x->trace_stats.p, 16, cudaMemcpyDeviceToHost));
    return CRT_OK;
}

crt_status crt_last_trace_timing(crt_ctx* x, float ms[2]) {
    if (!x || !ms) return fail(CRT_ERR_INVALID_ARG, "null argument");
    if (!x->tev_valid) return fail(CRT_ERR_INVALID_ARG, "crt_last_trace_timing: no traversal recorded yet");
    CRT_CUDA(cudaEventSynchronize(x->tev[2]));
    CRT_CUDA(cudaEventElapsedTime(&ms[0], x->tev[0], x->tev[1]));
    CRT_CUDA(cudaEventElapsedTime(&ms[1], x->tev[1], x->tev[2]));
    return CRT_OK;
}

crt_status crt_last_trace_stats(crt_ctx* x, uint64_t out[2]) {
    if (!x || !out) return fail(CRT_ERR_INVALID_ARG, "null argument");
    out[0] = x->last_trace_stats[0];
    out[1] = x->last_trace_stats[1];
    return CRT_OK;
}

crt_status crt_trace_frame(crt_ctx* x, const crt_bvh* b, const crt_camera* cam, uint32_t width, uint32_t height,
                           const float* light, uint32_t flags, crt_hit* hits_primary, crt_hit* hits_shadow) {
    if (!x || !b || !cam || !hits_primary) return fail(CRT_ERR_INVALID_ARG, "crt_trace_frame: null argument");
    if (width == 0 || height == 0 || height > 65535) return fail(CRT_ERR_INVALID_ARG, "bad image size");
    if (light && !hits_shadow) return fail(CRT_ERR_INVALID_ARG, "crt_trace_frame: light without shadow output");
    CRT_TRY(check_trace_flags(b, flags));
    if (flags & CRT_TRACE_ANY) return fail(CRT_ERR_INVALID_ARG, "crt_trace_frame: primary rays are closest-hit");
    CRT_CUDA(cudaSetDevice(x->device));
    const uint32_t n = width * height;
    const bool fused = !(flags & (CRT_TRACE_USE_PREDICTOR | CRT_TRACE_WIDE | CRT_TRACE_COMPRESSED));
    bool dev_p = is_device_ptr(hits_primary);
    if (dev_p) CRT_TRY(check_aligned16(hits_primary, "crt_trace_frame: primary hits"));
    if (light && hits_shadow && is_device_ptr(hits_shadow))
        CRT_TRY(check_aligned16(hits_shadow, "crt_trace_frame: shadow hits"));
    crt_hit* d_hp = hits_primary;
    if (!dev_p && fused) {  // page-locked host output: the frame kernel writes it over the CPU-GPU link
        if (void* m = mapped_host_ptr(hits_primary)) {
            d_hp = static_cast<crt_hit*>(m);
            dev_p = true;
        }
    }
    if (!dev_p) {
        CRT_TRY(x->frame_hits.reserve(sizeof(crt_hit) * static_cast<size_t>(n)));
        d_hp = x->frame_hits.as<crt_hit>();
    }
    const crt_camera* d_cam = cam;
    if (!is_device_ptr(cam)) {
        CRT_CUDA(cudaMemcpyAsync(x->cam.p, cam, sizeof(crt_camera), cudaMemcpyHostToDevice, x->stream));
        d_cam = x->cam.as<crt_camera>();
    } else {
        CRT_TRY(check_aligned16(cam, "camera"));
    }
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    const uint32_t tw = (width % 8 == 0 && height % 4 == 0) ? width : 0u;  // 8x4 pixel tiles per warp
    if (fused) {
        // one launch: camera ray, closest hit, shadow ray, any hit per pixel.
        // Page-locked host outputs are written by the kernel itself over the
        // CPU-GPU link while it runs; only pageable ones go through a copy.
        crt_hit* d_hs = nullptr;
        bool dev_s = true;
        if (light) {
            dev_s = is_device_ptr(hits_shadow);
            d_hs = hits_shadow;
            if (!dev_s) {
                if (void* m = mapped_host_ptr(hits_shadow)) {
                    d_hs = static_cast<crt_hit*>(m);
                    dev_s = true;
                } else {
                    CRT_TRY(x->frame_shits.reserve(sizeof(crt_hit) * static_cast<size_t>(n)));
                    d_hs = x->frame_shits.as<crt_hit>();
                }
            }
        }
        crt::TraceParams p{};
        p.nodes = b->nodes.as<crt_bvh_node>();
        p.xtri = b->xtri.as<float4>();
        p.wide = (flags & CRT_TRI_WATERTIGHT) ? b->wide_wt.as<float4>() : b->wide.as<float4>();
        p.hits = d_hp;
        p.n_rays = n;
        p.n_nodes = 2 * b->n - 1;
        p.abs_eps = b->abs_eps;
        p.err = x->err.as<uint32_t>();
        p.tile_width = tw;
        if (flags & CRT_TRACE_STATS) {
            CRT_CUDA(cudaMemsetAsync(x->trace_stats.p, 0, 16, x->stream));
            p.stats = x->trace_stats.as<unsigned long long>();
        }
        const bool deep = b->depth_bound + 2 > 64;
        const uint32_t kflags = (flags & CRT_TRI_WATERTIGHT) | (deep ? (1u << 16) : 0u);
        // One launch for the whole image.  Splitting it into row bands whose
        // hits are copied out on a second stream while the next band runs was
        // measured slower at every band count (2, 4, 8) on GB300.
        crt::launch_frame(p, d_cam, width, height, 0, height, light, d_hs, kflags, static_cast<int>(x->cfg.trace_block),
                          nullptr, x->stream);
        CRT_CUDA(cudaGetLastError());
        if (!dev_p)
            CRT_CUDA(cudaMemcpyAsync(hits_primary, d_hp, sizeof(crt_hit) * static_cast<size_t>(n), cudaMemcpyDeviceToHost,
                                     x->stream));
        if (light && !dev_s)
            CRT_CUDA(cudaMemcpyAsync(hits_shadow, d_hs, sizeof(crt_hit) * static_cast<size_t>(n), cudaMemcpyDeviceToHost,
                                     x->stream));
        if (flags & CRT_TRACE_STATS) {
            CRT_CUDA(cudaStreamSynchronize(x->stream));
            CRT_CUDA(cudaMemcpy(x->last_trace_stats, x->trace_stats.p, 16, cudaMemcpyDeviceToHost));
        }
        return x->check_device_error();
    }
    CRT_TRY(x->frame_rays.reserve(sizeof(crt_ray) * static_cast<size_t>(n)));
    crt_ray* rays = x->frame_rays.as<crt_ray>();
    crt::launch_raygen(d_cam, width, height, rays, x->stream);
    CRT_TRY(trace_device(x, b, rays, n, flags, d_hp, nullptr, tw));
    if (!dev_p) CRT_CUDA(cudaMemcpyAsync(hits_primary, d_hp, sizeof(crt_hit) * static_cast<size_t>(n), cudaMemcpyDeviceToHost, x->stream));
    if (light) {
        CRT_TRY(x->frame_shadow.reserve(sizeof(crt_ray) * static_cast<size_t>(n)));
        const bool dev_s = is_device_ptr(hits_shadow);
        crt_hit* d_hs = hits_shadow;
        if (!dev_s) {
            CRT_TRY(x->frame_shits.reserve(sizeof(crt_hit) * static_cast<size_t>(n)));
            d_hs = x->frame_shits.as<crt_hit>();
        }
        crt_ray* sh = x->frame_shadow.as<crt_ray>();
        crt::launch_shadow_rays(rays, d_hp, n, light[0], light[1], light[2], sh, x->stream);
        CRT_TRY(trace_device(x, b, sh, n, (flags & ~CRT_TRACE_STATS) | CRT_TRACE_ANY, d_hs, nullptr, tw));
        if (!dev_s) CRT_CUDA(cudaMemcpyAsync(hits_shadow, d_hs, sizeof(crt_hit) * static_cast<size_t>(n), cudaMemcpyDeviceToHost, x->stream));
    }
    return x->check_device_error();
}

}  // extern "C"

// ===================================================================== predictor
namespace {

crt_status stage_in(crt_ctx* x, DevBuf& buf, const void* src, size_t bytes, const void** dev) {
    if (is_device_ptr(src)) {
        CRT_TRY(check_aligned16(src, "ray or hit input"));
        *dev = src;
        return CRT_OK;
    }
    CRT_TRY(buf.reserve(bytes));
    CRT_CUDA(cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, x->stream));
    *dev = buf.p;
    return CRT_OK;
}

// As stage_in, for inputs a kernel reads once, in order: page-locked host
// memory is then read in place over the CPU-GPU link instead of copied.
crt_status stage_in_once(crt_ctx* x, DevBuf& buf, const void* src, size_t bytes, const void** dev) {
    if (!is_device_ptr(src)) {
        if (void* m = mapped_host_ptr(const_cast<void*>(src))) {
            *dev = m;
            return CRT_OK;
        }
    }
    return stage_in(x, buf, src, bytes, dev);
}

// The batch's traversal nodes and leaf records, and dropping its predictor
// (defined with crt_batch below).
const float4* batch_wide(const crt_batch* bt);
const float4* batch_xtri(const crt_batch* bt);
void batch_unbind(crt_batch* bt);

crt_status predictor_targets(crt_ctx* x, crt_predictor* pr) {
    if (pr->batch) {  // every scene cut into its own treelets
        const uint32_t ns = pr->batch_n_scenes;
        CRT_TRY(pr->tri_class.reserve(pr->batch_n_tris));
        CRT_TRY(pr->treelets.reserve(sizeof(crt::Treelet) * 128 * ns + 4ull * ns + 16));
        CRT_CUDA(cudaMemsetAsync(pr->tri_class.p, crt::pred::kMissClass, pr->batch_n_tris, x->stream));
        uint32_t* n_tl = reinterpret_cast<uint32_t*>(pr->treelets.as<crt::Treelet>() + 128 * ns);
        crt::pred_treelets_batch(pr->batch_scenes, ns, pr->batch_n_tris, pr->batch_nodes,
                                 batch_wide(pr->batch), batch_xtri(pr->batch), pr->treelets.as<crt::Treelet>(), n_tl,
                                 pr->tri_class.as<uint8_t>(), x->stream);
        CRT_CUDA(cudaGetLastError());
        std::vector<uint32_t> counts(ns);
        CRT_CUDA(cudaMemcpyAsync(counts.data(), n_tl, 4ull * ns, cudaMemcpyDeviceToHost, x->stream));
        CRT_CUDA(cudaStreamSynchronize(x->stream));
        pr->n_treelets = 0;
        for (uint32_t c : counts) pr->n_treelets += c;
        return CRT_OK;
    }
    crt_bvh* b = pr->bvh;
    CRT_TRY(pr->tri_class.reserve(b->n));
    CRT_TRY(pr->treelets.reserve(sizeof(crt::Treelet) * 128 + 16));
    CRT_CUDA(cudaMemsetAsync(pr->tri_class.p, crt::pred::kMissClass, b->n, x->stream));
    uint32_t* n_tl = reinterpret_cast<uint32_t*>(pr->treelets.as<crt::Treelet>() + 128);
    crt::pred_treelets(b->nodes.as<crt_bvh_node>(), b->wide.as<float4>(), b->xtri.as<float4>(), b->n,
                       pr->treelets.as<crt::Treelet>(), n_tl, pr->tri_class.as<uint8_t>(), x->stream);
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaMemcpyAsync(&pr->n_treelets, n_tl, 4, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

}  // namespace

extern "C" {

void crt_predictor_default_config(crt_predictor_config* cfg) {
    if (!cfg) return;
    cfg->seed = 1;
    cfg->lr = 1e-3f;
    cfg->train_stride = 20;
    cfg->batch = 16384;
    cfg->miss_threshold = 0.9f;
}

crt_status crt_predictor_create(crt_ctx* x, crt_bvh* b, const crt_predictor_config* cfg, crt_predictor** out) {
    if (!x || !b || !out) return fail(CRT_ERR_INVALID_ARG, "crt_predictor_create: null argument");
    if (b->n < 2) return fail(CRT_ERR_INVALID_ARG, "crt_predictor_create: the bvh needs at least 2 triangles");
    if (b->predictor) return fail(CRT_ERR_INVALID_ARG, "crt_predictor_create: the bvh already has a predictor");
    static_assert(crt::pred::kParams == CRT_PREDICTOR_PARAMS, "parameter count");
    CRT_CUDA(cudaSetDevice(x->device));
    crt_predictor* pr = new crt_predictor();
    crt_predictor_default_config(&pr->cfg);
    if (cfg) pr->cfg = *cfg;
    if (pr->cfg.train_stride == 0) pr->cfg.train_stride = 1;
    if (pr->cfg.batch == 0) pr->cfg.batch = 16384;
    pr->bvh = b;
    crt_status s = pr->params.reserve(4 * sizeof(float) * crt::pred::kParams);
    if (s == CRT_OK) s = pr->w16.reserve(sizeof(__half) * crt::pred::kHalfs);
    if (s == CRT_OK) s = pr->scratch.reserve(16);
    if (s == CRT_OK) {
        crt::pred_init(pr->dev(), pr->cfg.seed, x->stream);
        s = predictor_targets(x, pr);
    }
    if (s != CRT_OK) {
        crt_predictor_destroy(pr);
        return s;
    }
    b->predictor = pr;
    *out = pr;
    return CRT_OK;
}

crt_status crt_predictor_destroy(crt_predictor* pr) {
    if (!pr) return CRT_OK;
    if (pr->bvh) pr->bvh->predictor = nullptr;
    if (pr->batch) batch_unbind(pr->batch);
    DevBuf* bufs[] = {&pr->params, &pr->w16, &pr->tri_class, &pr->treelets, &pr->classes, &pr->scratch,
                      &pr->rays_in, &pr->hits_in, &pr->targets_in, &pr->order, &pr->order_scratch};
    for (DevBuf* d : bufs) d->release();
    delete pr;
    return CRT_OK;
}

crt_status crt_predictor_retarget(crt_ctx* x, crt_predictor* pr) {
    if (!x || !pr || !pr->bound()) return fail(CRT_ERR_INVALID_ARG, "crt_predictor_retarget: null or unbound predictor");
    CRT_CUDA(cudaSetDevice(x->device));
    return predictor_targets(x, pr);
}

crt_status crt_predictor_train(crt_ctx* x, crt_predictor* pr, const crt_ray* rays, const crt_hit* hits,
                               uint32_t n_rays, uint32_t offset, float* loss) {
    if (!x || !pr || !pr->bound() || !rays || !hits) return fail(CRT_ERR_INVALID_ARG, "crt_predictor_train: null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    const void* d_rays;
    const void* d_hits;
    CRT_TRY(stage_in(x, pr->rays_in, rays, sizeof(crt_ray) * static_cast<size_t>(n_rays), &d_rays));
    CRT_TRY(stage_in(x, pr->hits_in, hits, sizeof(crt_hit) * static_cast<size_t>(n_rays), &d_hits));
    const uint32_t stride = pr->cfg.train_stride;
    const uint32_t total = offset < n_rays ? (n_rays - offset + stride - 1) / stride : 0;
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    CRT_CUDA(cudaMemsetAsync(pr->scratch.p, 0, 16, x->stream));
    for (uint32_t done = 0; done < total; done += pr->cfg.batch) {
        const uint32_t nb = std::min(pr->cfg.batch, total - done);
        CRT_CUDA(crt::pred_train_step(pr->dev(), pr->nodes(),
                                      static_cast<const crt_ray*>(d_rays), n_rays, static_cast<const crt_hit*>(d_hits),
                                      nullptr, nb, stride, offset + done * stride, pr->scratch.as<float>(),
                                      x->err.as<uint32_t>(), x->stream));
        ++pr->step;
        crt::pred_adam(pr->dev(), 1.f / static_cast<float>(nb), pr->cfg.lr, pr->step, x->stream);
        CRT_CUDA(cudaGetLastError());
    }
    float ls = 0.f;
    CRT_CUDA(cudaMemcpyAsync(&ls, pr->scratch.p, 4, cudaMemcpyDeviceToHost, x->stream));
    CRT_TRY(x->check_device_error());
    if (loss) *loss = total ? ls / static_cast<float>(total) : 0.f;
    return CRT_OK;
}

crt_status crt_predictor_infer(crt_ctx* x, crt_predictor* pr, const crt_ray* rays, uint32_t n, uint16_t* classes) {
    if (!x || !pr || !pr->bound() || !rays || !classes) return fail(CRT_ERR_INVALID_ARG, "crt_predictor_infer: null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    if (n == 0) return CRT_OK;
    const void* d_rays;
    CRT_TRY(stage_in(x, pr->rays_in, rays, sizeof(crt_ray) * static_cast<size_t>(n), &d_rays));
    const bool dev_out = is_device_ptr(classes);
    if (dev_out && (reinterpret_cast<uintptr_t>(classes) & 1u))
        return fail(CRT_ERR_INVALID_ARG, "classes: device memory must be 2-byte aligned");
    uint16_t* d_out = classes;
    if (!dev_out) {
        CRT_TRY(pr->classes.reserve(2ull * n));
        d_out = pr->classes.as<uint16_t>();
    }
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    CRT_CUDA(crt::pred_infer(pr->dev(), pr->nodes(), static_cast<const crt_ray*>(d_rays), n,
                             d_out, pr->cfg.miss_threshold, false, x->err.as<uint32_t>(), x->stream));
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(classes, d_out, 2ull * n, cudaMemcpyDeviceToHost, x->stream));
    return x->check_device_error();
}

crt_status crt_predictor_classes_of_hits(crt_ctx* x, crt_predictor* pr, const crt_hit* hits, uint32_t n,
                                         uint16_t* classes) {
    if (!x || !pr || !pr->bound() || !hits || !classes) return fail(CRT_ERR_INVALID_ARG, "null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    if (n == 0) return CRT_OK;
    const void* d_hits;
    CRT_TRY(stage_in(x, pr->hits_in, hits, sizeof(crt_hit) * static_cast<size_t>(n), &d_hits));
    const bool dev_out = is_device_ptr(classes);
    if (dev_out && (reinterpret_cast<uintptr_t>(classes) & 1u))
        return fail(CRT_ERR_INVALID_ARG, "classes: device memory must be 2-byte aligned");
    uint16_t* d_out = classes;
    if (!dev_out) {
        CRT_TRY(pr->targets_in.reserve(2ull * n));
        d_out = pr->targets_in.as<uint16_t>();
    }
    crt::pred_classes_of_hits(pr->dev(), static_cast<const crt_hit*>(d_hits), n, d_out, x->stream);
    CRT_CUDA(cudaGetLastError());
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(classes, d_out, 2ull * n, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status crt_predictor_gradients(crt_ctx* x, crt_predictor* pr, const crt_ray* rays, const uint16_t* targets,
                                   uint32_t n, float* grad, float* loss) {
    if (!x || !pr || !pr->bound() || !rays || !targets || !grad) return fail(CRT_ERR_INVALID_ARG, "null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    const void* d_rays;
    const void* d_t;
    CRT_TRY(stage_in(x, pr->rays_in, rays, sizeof(crt_ray) * static_cast<size_t>(n), &d_rays));
    CRT_TRY(stage_in(x, pr->targets_in, targets, 2ull * n, &d_t));
    const crt::PredictorDev d = pr->dev();
    CRT_CUDA(cudaMemsetAsync(d.grad, 0, sizeof(float) * crt::pred::kParams, x->stream));
    CRT_CUDA(cudaMemsetAsync(pr->scratch.p, 0, 16, x->stream));
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    CRT_CUDA(crt::pred_train_step(d, pr->nodes(), static_cast<const crt_ray*>(d_rays), n, nullptr,
                                  static_cast<const uint16_t*>(d_t), n, 1, 0, pr->scratch.as<float>(),
                                  x->err.as<uint32_t>(), x->stream));
    CRT_CUDA(cudaMemcpyAsync(grad, d.grad, sizeof(float) * crt::pred::kParams,
                             is_device_ptr(grad) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, x->stream));
    float ls = 0.f;
    CRT_CUDA(cudaMemcpyAsync(&ls, pr->scratch.p, 4, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaMemsetAsync(d.grad, 0, sizeof(float) * crt::pred::kParams, x->stream));
    CRT_TRY(x->check_device_error());
    if (loss) *loss = ls;
    return CRT_OK;
}

crt_status crt_predictor_params(crt_ctx* x, crt_predictor* pr, float* params, int set) {
    if (!x || !pr || !params) return fail(CRT_ERR_INVALID_ARG, "null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    const size_t bytes = sizeof(float) * crt::pred::kParams;
    const bool dev = is_device_ptr(params);
    if (set) {
        CRT_CUDA(cudaMemcpyAsync(pr->params.p, params, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 x->stream));
        crt::pred_refresh_fp16(pr->dev(), x->stream);
        CRT_CUDA(cudaGetLastError());
    } else {
        CRT_CUDA(cudaMemcpyAsync(params, pr->params.p, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                 x->stream));
    }
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status crt_predictor_info(const crt_predictor* pr, uint32_t info[4]) {
    if (!pr || !info) return fail(CRT_ERR_INVALID_ARG, "null argument");
    info[0] = static_cast<uint32_t>(crt::pred::kParams);
    info[1] = crt::pred::kClasses;
    info[2] = pr->n_treelets;
    info[3] = pr->step;
    return CRT_OK;
}

crt_status crt_bounce_rays(crt_ctx* x, const crt_bvh* b, const crt_ray* primary, const crt_hit* hits,
                           uint32_t n_primary, uint32_t n_out, uint32_t seed, crt_ray* out) {
    if (!x || !b || !primary || !hits || !out) return fail(CRT_ERR_INVALID_ARG, "crt_bounce_rays: null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    if (n_out == 0) return CRT_OK;
    const void* d_prim;
    const void* d_hits;
    CRT_TRY(stage_in(x, x->rays_in, primary, sizeof(crt_ray) * static_cast<size_t>(n_primary), &d_prim));
    CRT_TRY(stage_in(x, x->hits_out, hits, sizeof(crt_hit) * static_cast<size_t>(n_primary), &d_hits));
    const bool dev_out = is_device_ptr(out);
    if (dev_out) CRT_TRY(check_aligned16(out, "crt_bounce_rays: rays"));
    crt_ray* d_out = out;
    if (!dev_out) {
        CRT_TRY(x->rays_out.reserve(sizeof(crt_ray) * static_cast<size_t>(n_out)));
        d_out = x->rays_out.as<crt_ray>();
    }
    CRT_TRY(x->pos.reserve(crt::bounce_scratch_bytes(n_primary)));  // build scratch, idle between builds
    crt::launch_bounce(static_cast<const crt_ray*>(d_prim), static_cast<const crt_hit*>(d_hits), n_primary,
                       b->xtri.as<float4>(), b->inv_perm.as<uint32_t>(), b->n, n_out, seed, d_out,
                       x->pos.as<uint32_t>(), x->stream);
    CRT_CUDA(cudaGetLastError());
    if (!dev_out) CRT_CUDA(cudaMemcpyAsync(out, d_out, sizeof(crt_ray) * static_cast<size_t>(n_out), cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

}  // extern "C"

// ===================================================================== batches
struct crt_batch {
    crt_ctx* ctx = nullptr;
    crt_predictor* predictor = nullptr;  // crt_batch_predictor_create
    bool built = false;                  // a build has completed
    uint32_t n_scenes = 0;
    uint32_t n_tris = 0, n_rays = 0;
    uint32_t ray_cap = 0;                // rays reserved at creation; crt_batch_set_ray_counts stays within it
    std::vector<crt::BatchScene> hs;
    std::vector<uint32_t> tri_off;
    uint32_t n_chunks = 0, lb_cap = 0, max_n = 0, max_iters = 0;
    crt_config cfg{};
    DevBuf scenes, seg_off, seg_hist, chunks, states, models, err;
    DevBuf codes_a, codes_b, vals_a, vals_b, codes, perm_global, perm_local;
    DevBuf node_box, node_kids, pf, clus_a, clus_b, it, ploc_lb, hist, sort_lb;
    DevBuf nodes, wide, wide_wt, depth_odd, xtri, xtri_sorted, inv_perm;
    DevBuf ray_order, ray_order_scratch;  // CRT_TRACE_SORT_RAYS
    DevBuf pool_counter;                  // the persistent trace's ray counter
    bool models_set = false;
    cudaGraphExec_t graph = nullptr;
    const void* g_tris = nullptr;
    const void* g_rays = nullptr;
    const void* g_hits = nullptr;
    uint32_t g_flags = 0;
    crt_config g_cfg{};
    std::vector<uint32_t> g_counts;      // per-scene ray counts the graph was captured with
    std::vector<uint32_t> ray_counts() const {
        std::vector<uint32_t> c(n_scenes);
        for (uint32_t k = 0; k < n_scenes; ++k) c[k] = hs[k].n_rays;
        return c;
    }
    void drop_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
};

namespace {

const float4* batch_wide(const crt_batch* bt) { return bt->wide.as<float4>(); }
const float4* batch_xtri(const crt_batch* bt) { return bt->xtri.as<float4>(); }
void batch_unbind(crt_batch* bt) { bt->predictor = nullptr; bt->drop_graph(); }

crt_status batch_upload_models(crt_ctx* x, crt_batch* bt, const crt_mesh_model* models, uint32_t n_models) {
    std::vector<float> hm(2 * 64 * 16);
    for (uint32_t m = 0; m < 64; ++m) {
        for (int k = 0; k < 16; ++k) hm[16 * m + k] = (k % 5 == 0) ? 1.f : 0.f;
        if (models && m < n_models) std::memcpy(&hm[16 * m], models[m].m, 64);
    }
    const volatile float third = 1.f / 3.f;
    for (int k = 0; k < 64 * 16; ++k) hm[64 * 16 + k] = third * hm[k];
    CRT_CUDA(cudaMemcpy(bt->models.p, hm.data(), hm.size() * 4, cudaMemcpyHostToDevice));
    bt->models_set = true;
    (void)x;
    return CRT_OK;
}

// Enqueue build (and trace when rays != null) without synchronising.
// The trace of every scene's rays, one launch (after the ordering or learned
// steps the flags ask for), on x's stream; no allocation, so it can be
// captured into the batch's graph.
crt_status batch_trace_enqueue(crt_ctx* x, crt_batch* bt, const crt_ray* rays, uint32_t flags, crt_hit* hits,
                               bool deep) {
    cudaStream_t s = x->stream;
    uint32_t* err = bt->err.as<uint32_t>();
    crt::TraceParams p{};
    p.nodes = bt->nodes.as<crt_bvh_node>();
    p.wide = (flags & CRT_TRI_WATERTIGHT) ? bt->wide_wt.as<float4>() : bt->wide.as<float4>();
    p.xtri = bt->xtri.as<float4>();
    p.rays = rays;
    p.hits = hits;
    p.n_rays = bt->n_rays;
    p.err = err;
    if ((flags & (CRT_TRACE_USE_PREDICTOR | CRT_TRACE_PREDICTOR_ORDER)) && bt->n_rays > 0) {
        crt_predictor* pr = bt->predictor;
        const bool fuse = (flags & CRT_TRACE_PREDICTOR_ORDER) && !(flags & CRT_TRACE_USE_PREDICTOR) && bt->n_rays > 1;
        uint32_t *okeys = nullptr, *ohist = nullptr;  // the inference writes the order keys too
        if (fuse) crt::pred_order_begin(pr->order_scratch.p, bt->n_rays, &okeys, &ohist, s);
        CRT_CUDA(crt::pred_infer(pr->dev(), pr->nodes(), rays, bt->n_rays, pr->classes.as<uint16_t>(),
                                 pr->cfg.miss_threshold, !(flags & CRT_TRACE_USE_PREDICTOR), err, s, okeys, ohist));
        if (flags & CRT_TRACE_USE_PREDICTOR) {
            p.pred_class = pr->classes.as<uint16_t>();
            p.treelets = pr->treelets.as<crt::Treelet>();
            p.n_treelets = reinterpret_cast<const uint32_t*>(pr->treelets.as<crt::Treelet>() + 128 * bt->n_scenes);
        }
        if ((flags & CRT_TRACE_PREDICTOR_ORDER) && bt->n_rays > 1) {
            crt::pred_order(pr->dev(), pr->nodes(), rays, pr->classes.as<uint16_t>(), bt->n_rays, pr->order.as<uint32_t>(),
                            pr->order_scratch.p, err, x->cfg.spin_limit, s, fuse);
            p.order = pr->order.as<uint32_t>();
        }
    }
    if ((flags & CRT_TRACE_SORT_RAYS) && !p.order && bt->n_rays > 1) {
        crt::launch_ray_order(rays, bt->n_rays, bt->nodes.as<crt_bvh_node>(), bt->scenes.as<crt::BatchScene>(),
                              bt->n_scenes, bt->ray_order.as<uint32_t>(), bt->ray_order_scratch.p, err, x->cfg.spin_limit,
                              s);
        p.order = bt->ray_order.as<uint32_t>();
    }
    // large closest-hit batches: the persistent ray pool, each lane walking
    // its ray's scene (as trace_device does for one scene)
    if (!(flags & CRT_TRACE_ANY) && !p.pred_class && bt->n_rays >= kPoolMinRays)
        crt::launch_trace_batch_pool(p, bt->scenes.as<crt::BatchScene>(), bt->n_scenes, flags & CRT_TRI_WATERTIGHT, deep,
                                     bt->pool_counter.as<uint32_t>(), s);
    else
        crt::launch_trace_batch(p, bt->scenes.as<crt::BatchScene>(), bt->n_scenes, bt->n_rays,
                                flags & (CRT_TRACE_ANY | CRT_TRI_WATERTIGHT), static_cast<int>(bt->cfg.trace_block), deep,
                                s);
    CRT_CUDA(cudaGetLastError());
    return CRT_OK;
}

// Flags a batch trace accepts: the learned ones need the batch's predictor.
crt_status batch_trace_flags(const crt_batch* bt, uint32_t flags, const char* who) {
    if (flags & ~(CRT_TRACE_ANY | CRT_TRI_WATERTIGHT | CRT_TRACE_SORT_RAYS | CRT_TRACE_USE_PREDICTOR |
                  CRT_TRACE_PREDICTOR_ORDER))
        return fail(CRT_ERR_INVALID_ARG, "%s: unsupported flags 0x%x", who, flags);
    if ((flags & (CRT_TRACE_USE_PREDICTOR | CRT_TRACE_PREDICTOR_ORDER)) && !bt->predictor)
        return fail(CRT_ERR_UNSUPPORTED, "%s: the batch has no predictor (crt_batch_predictor_create)", who);
    return CRT_OK;
}

crt_status batch_enqueue(crt_ctx* x, crt_batch* bt, const crt_triangle* tris, const crt_ray* rays, uint32_t flags,
                         crt_hit* hits, cudaEvent_t ev_built) {
    cudaStream_t s = x->stream;
    const int bits = static_cast<int>(bt->cfg.sort_digit_bits);
    const int passes = (30 + bits - 1) / bits;
    const uint32_t radix = 1u << bits;
    const uint32_t tiles = (bt->n_tris + crt::sort_tile_keys(bits) - 1) / crt::sort_tile_keys(bits);
    const size_t lb_words = static_cast<size_t>(tiles) * 256 + 1;  // per pass (room for 256-digit scene pass)
    uint32_t* err = bt->err.as<uint32_t>();
    CRT_CUDA(cudaMemsetAsync(bt->err.p, 0, 16, s));
    CRT_CUDA(cudaMemsetAsync(bt->states.p, 0, crt::batch_box_state_bytes() * bt->n_scenes, s));
    CRT_CUDA(cudaMemsetAsync(bt->hist.p, 0, 4ull * passes * radix, s));
    CRT_CUDA(cudaMemsetAsync(bt->sort_lb.p, 0, 4ull * (passes + 1) * lb_words, s));
    CRT_CUDA(cudaMemsetAsync(bt->ploc_lb.p, 0, 8ull * 2 * bt->lb_cap + 32, s));
    crt::launch_batch_box(tris, bt->chunks.p, bt->n_chunks, bt->models.as<float>(), bt->states.p,
                          bt->scenes.as<crt::BatchScene>(), err, s);
    crt::launch_batch_morton(tris, bt->chunks.p, bt->n_chunks, bt->models.as<float>() + 64 * 16, bt->states.p,
                             bt->codes_a.as<uint32_t>(), bt->hist.as<uint32_t>(), bits, s);
    uint32_t* kin = bt->codes_a.as<uint32_t>();
    uint32_t* vin = nullptr;
    for (int p = 0; p < passes; ++p) {
        uint32_t* kout = (p & 1) ? bt->codes_a.as<uint32_t>() : bt->codes_b.as<uint32_t>();
        uint32_t* vout = (p & 1) ? bt->vals_a.as<uint32_t>() : bt->vals_b.as<uint32_t>();
        uint32_t* lb = bt->sort_lb.as<uint32_t>() + static_cast<size_t>(p) * lb_words;
        crt::launch_onesweep(kin, vin, kout, vout, bt->n_tris, p * bits, bits, bt->hist.as<uint32_t>() + p * radix, lb + 1,
                             lb, err, x->cfg.spin_limit, s);
        kin = kout;
        vin = vout;
    }
    {
        uint32_t* lb = bt->sort_lb.as<uint32_t>() + static_cast<size_t>(passes) * lb_words;
        crt::launch_onesweep_segments(kin, vin, bt->codes.as<uint32_t>(), bt->perm_global.as<uint32_t>(), bt->n_tris,
                                      bt->seg_off.as<uint32_t>(), bt->n_scenes, bt->seg_hist.as<uint32_t>(), lb + 1, lb,
                                      err, x->cfg.spin_limit, s);
    }
    crt::launch_batch_leaf_init(tris, bt->n_tris, bt->scenes.as<crt::BatchScene>(), bt->n_scenes, bt->models.as<float>(),
                                bt->perm_global.as<uint32_t>(), bt->perm_local.as<uint32_t>(), bt->node_box.as<float4>(),
                                bt->clus_a.as<float4>(), bt->xtri_sorted.as<float4>(), bt->xtri.as<float4>(),
                                bt->inv_perm.as<uint32_t>(), bt->it.as<uint2>(), bt->nodes.as<crt_bvh_node>(), err, s);
    {
        unsigned long long* lb = bt->ploc_lb.as<unsigned long long>();
        uint32_t* tail = reinterpret_cast<uint32_t*>(lb + 2ull * bt->lb_cap);
        const cudaError_t e = crt::launch_batch_ploc(
            bt->scenes.as<crt::BatchScene>(), bt->n_scenes, bt->clus_a.as<float4>(), bt->clus_b.as<float4>(),
            bt->node_box.as<float4>(), bt->node_kids.as<uint4>(), bt->it.as<uint2>(), static_cast<int>(bt->cfg.ploc_radius),
            lb, bt->lb_cap, tail, bt->pf.as<uint2>(), bt->nodes.as<crt_bvh_node>(), bt->wide.as<float4>(),
            bt->wide_wt.as<float4>(), bt->depth_odd.as<uint8_t>(),
            crt::LeafOut{bt->xtri_sorted.as<float4>(), bt->xtri.as<float4>(), bt->inv_perm.as<uint32_t>()},
            reinterpret_cast<unsigned long long*>(tail + 2),
            bt->max_n + 1, err, x->cfg.spin_limit, s);
        if (e != cudaSuccess) return fail(CRT_ERR_UNSUPPORTED, "batched PLOC launch failed: %s", cudaGetErrorString(e));
    }
    CRT_CUDA(cudaGetLastError());
    if (ev_built) CRT_CUDA(cudaEventRecord(ev_built, s));
    if (rays) CRT_TRY(batch_trace_enqueue(x, bt, rays, flags, hits, bt->cfg.stack_depth > 64));
    return CRT_OK;
}

// Scratch of CRT_TRACE_SORT_RAYS for a batch, reserved outside graph capture.
crt_status batch_order_buffers(crt_batch* bt, uint32_t flags) {
    // sized for the batch's ray capacity, so a later crt_batch_set_ray_counts
    // never moves a buffer that a captured graph points at
    if (!(flags & CRT_TRACE_SORT_RAYS) || bt->ray_cap <= 1) return CRT_OK;
    CRT_TRY(bt->ray_order.reserve(4ull * bt->ray_cap));
    CRT_TRY(bt->ray_order_scratch.reserve(crt::ray_order_scratch_bytes(bt->ray_cap)));
    return CRT_OK;
}

crt_status batch_check(crt_ctx* x, crt_batch* bt) {
    uint32_t ew[4] = {0, 0, 0, 0};
    CRT_CUDA(cudaMemcpyAsync(ew, bt->err.p, 16, cudaMemcpyDeviceToHost, x->stream));
    CRT_CUDA(cudaMemcpyAsync(bt->hs.data(), bt->scenes.p, sizeof(crt::BatchScene) * bt->n_scenes, cudaMemcpyDeviceToHost,
                             x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    bt->max_iters = 0;
    for (const auto& sc : bt->hs) bt->max_iters = std::max(bt->max_iters, sc.iters);
    if (ew[0] & crt::kDevTimeout) return fail(CRT_ERR_DEVICE_TIMEOUT, "batch: a bounded device wait gave up");
    if (ew[0] & crt::kDevBadModel) return fail(CRT_ERR_BAD_INPUT, "batch: a triangle references model id >= 64");
    if (ew[0] & crt::kDevStackOverflow)
        return fail(CRT_ERR_STACK_OVERFLOW, "batch: a ray overflowed its traversal stack (use stack_depth 1024)");
    if (ew[0]) return fail(CRT_ERR_CUDA, "batch: device error word 0x%x (site %u, %u, %u)", ew[0], ew[1], ew[2], ew[3]);
    return CRT_OK;
}

}  // namespace

extern "C" {

crt_status crt_batch_create(crt_ctx* x, const uint32_t* tri_counts, const uint32_t* ray_counts, uint32_t n_scenes,
                            crt_batch** out) {
    if (!x || !tri_counts || !ray_counts || !out) return fail(CRT_ERR_INVALID_ARG, "crt_batch_create: null argument");
    if (n_scenes == 0 || n_scenes > crt::kMaxBatchScenes)
        return fail(CRT_ERR_INVALID_ARG, "crt_batch_create: 1 to %u scenes", crt::kMaxBatchScenes);
    CRT_CUDA(cudaSetDevice(x->device));
    crt_batch* bt = new crt_batch();
    bt->ctx = x;
    bt->n_scenes = n_scenes;
    bt->cfg = x->cfg;
    bt->cfg.stack_depth = 64;
    uint64_t nt = 0, nr = 0, lb = 0;
    std::vector<crt::BatchScene> hs(n_scenes);
    std::vector<uint32_t> chunks;
    for (uint32_t k = 0; k < n_scenes; ++k) {
        if (tri_counts[k] == 0) { delete bt; return fail(CRT_ERR_INVALID_ARG, "crt_batch_create: empty scene %u", k); }
        hs[k] = crt::BatchScene{};
        hs[k].tri_off = static_cast<uint32_t>(nt);
        hs[k].n_tris = tri_counts[k];
        hs[k].node_off = static_cast<uint32_t>(2 * nt - k);
        hs[k].wide_off = static_cast<uint32_t>(nt - k);
        hs[k].ray_off = static_cast<uint32_t>(nr);
        hs[k].n_rays = ray_counts[k];
        hs[k].it_off = static_cast<uint32_t>(nt + 2ull * k);
        hs[k].lb_off = static_cast<uint32_t>(lb);
        lb += (tri_counts[k] + crt::kPlocMinOwn - 1) / crt::kPlocMinOwn;
        const uint32_t ck = crt::batch_box_chunk();
        hs[k].n_chunks = static_cast<uint32_t>((tri_counts[k] + ck - 1) / ck);
        for (uint64_t b = 0; b < tri_counts[k]; b += ck) {
            chunks.push_back(k);
            chunks.push_back(static_cast<uint32_t>(nt + b));
            chunks.push_back(static_cast<uint32_t>(nt + std::min<uint64_t>(tri_counts[k], b + ck)));
            chunks.push_back(0);
        }
        bt->max_n = std::max(bt->max_n, tri_counts[k]);
        nt += tri_counts[k];
        nr += ray_counts[k];
    }
    if (nt >= (1ull << 30) || nr >= (1ull << 31)) { delete bt; return fail(CRT_ERR_INVALID_ARG, "crt_batch_create: too large"); }
    bt->n_tris = static_cast<uint32_t>(nt);
    bt->n_rays = static_cast<uint32_t>(nr);
    bt->ray_cap = bt->n_rays;
    bt->hs = hs;
    bt->n_chunks = static_cast<uint32_t>(chunks.size() / 4);
    bt->lb_cap = static_cast<uint32_t>(lb);
    const uint32_t N = bt->n_tris;
    const uint32_t max_tiles = (N + crt::sort_tile_keys(4) - 1) / crt::sort_tile_keys(4);
    crt_status st = CRT_OK;
    auto R = [&](DevBuf& b, size_t bytes) { if (st == CRT_OK) st = b.reserve(bytes); };
    R(bt->scenes, sizeof(crt::BatchScene) * n_scenes);
    R(bt->seg_off, 4ull * (n_scenes + 1));
    R(bt->seg_hist, 4ull * 256);
    R(bt->chunks, crt::batch_chunk_bytes() * bt->n_chunks);
    R(bt->states, crt::batch_box_state_bytes() * n_scenes);
    R(bt->models, 2 * 64 * 16 * 4);
    R(bt->err, 16);
    for (DevBuf* b : {&bt->codes_a, &bt->codes_b, &bt->vals_a, &bt->vals_b, &bt->codes, &bt->perm_global, &bt->perm_local,
                      &bt->inv_perm})
        R(*b, 4ull * N);
    R(bt->node_kids, 16ull * N);
    R(bt->node_box, 32ull * (2ull * N));
    R(bt->pf, 8ull * N);
    R(bt->clus_a, 32ull * N);
    R(bt->clus_b, 32ull * N);
    R(bt->it, 8ull * (N + 2ull * n_scenes + 2));
    R(bt->ploc_lb, 8ull * 2 * bt->lb_cap + 32);
    R(bt->hist, 4ull * 8 * 256);
    R(bt->sort_lb, 4ull * 9 * (static_cast<size_t>(max_tiles) * 256 + 1));
    R(bt->nodes, sizeof(crt_bvh_node) * 2ull * N);
    R(bt->wide, 64ull * N);
    R(bt->wide_wt, 64ull * N);
    R(bt->depth_odd, N);
    R(bt->xtri, 48ull * N);
    R(bt->xtri_sorted, 48ull * N);
    R(bt->pool_counter, 16);
    if (st != CRT_OK) { crt_batch_free(bt); return st; }
    std::vector<uint32_t> seg(n_scenes + 1), segh(256, 0);
    for (uint32_t k = 0; k < n_scenes; ++k) { seg[k] = hs[k].tri_off; segh[k] = hs[k].n_tris; }
    seg[n_scenes] = N;
    bt->tri_off = seg;
    st = CRT_OK;
    if (cudaMemcpy(bt->scenes.p, hs.data(), sizeof(crt::BatchScene) * n_scenes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(bt->seg_off.p, seg.data(), 4ull * seg.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(bt->seg_hist.p, segh.data(), 4ull * 256, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(bt->chunks.p, chunks.data(), 4ull * chunks.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        crt_batch_free(bt);
        return fail(CRT_ERR_CUDA, "crt_batch_create: upload failed");
    }
    CRT_TRY(batch_upload_models(x, bt, nullptr, 0));
    bt->models_set = false;
    *out = bt;
    return CRT_OK;
}

crt_status crt_batch_free(crt_batch* bt) {
    if (!bt) return CRT_OK;
    bt->drop_graph();
    if (bt->predictor) {  // the predictor stays valid but unbound
        bt->predictor->batch = nullptr;
        bt->predictor->batch_scenes = nullptr;
        bt->predictor->batch_nodes = nullptr;
    }
    DevBuf* bufs[] = {&bt->scenes, &bt->seg_off, &bt->seg_hist, &bt->chunks, &bt->states, &bt->models, &bt->err,
                      &bt->codes_a, &bt->codes_b, &bt->vals_a, &bt->vals_b, &bt->codes, &bt->perm_global,
                      &bt->perm_local, &bt->node_box, &bt->node_kids, &bt->pf, &bt->clus_a, &bt->clus_b, &bt->it,
                      &bt->ploc_lb, &bt->hist, &bt->sort_lb, &bt->nodes, &bt->wide, &bt->wide_wt, &bt->depth_odd, &bt->xtri, &bt->ray_order, &bt->ray_order_scratch,
                      &bt->inv_perm, &bt->xtri_sorted, &bt->pool_counter};
    for (DevBuf* b : bufs) b->release();
    delete bt;
    return CRT_OK;
}

crt_status crt_batch_set_models(crt_ctx* x, crt_batch* bt, const crt_mesh_model* models, uint32_t n_models) {
    if (!x || !bt) return fail(CRT_ERR_INVALID_ARG, "null argument");
    if (n_models > 64 || (n_models && !models)) return fail(CRT_ERR_INVALID_ARG, "crt_batch_set_models: bad models");
    bt->drop_graph();
    return batch_upload_models(x, bt, models, n_models);
}

crt_status crt_batch_set_config(crt_batch* bt, const crt_config* cfg) {
    if (!bt || !cfg) return fail(CRT_ERR_INVALID_ARG, "null argument");
    if (cfg->ploc_radius == 0 || cfg->ploc_radius > static_cast<uint32_t>(crt::kPlocMaxRadius) ||
        (cfg->sort_digit_bits != 4 && cfg->sort_digit_bits != 8) ||
        (cfg->trace_block != 128 && cfg->trace_block != 256 && cfg->trace_block != 512))
        return fail(CRT_ERR_INVALID_ARG, "crt_batch_set_config: unsupported parameters");
    bt->cfg.ploc_radius = cfg->ploc_radius;
    bt->cfg.sort_digit_bits = cfg->sort_digit_bits;
    bt->cfg.trace_block = cfg->trace_block;
    bt->cfg.stack_depth = cfg->stack_depth > 64 ? 1024 : 64;
    bt->drop_graph();
    return CRT_OK;
}

crt_status crt_batch_get_config(const crt_batch* bt, crt_config* cfg) {
    if (!bt || !cfg) return fail(CRT_ERR_INVALID_ARG, "null argument");
    *cfg = bt->cfg;
    return CRT_OK;
}

crt_status crt_batch_build(crt_ctx* x, crt_batch* bt, const crt_triangle* tris) {
    if (!x || !bt || !tris) return fail(CRT_ERR_INVALID_ARG, "crt_batch_build: null argument");
    if (!is_device_ptr(tris)) return fail(CRT_ERR_INVALID_ARG, "crt_batch_build: triangles must be device memory");
    CRT_TRY(check_aligned16(tris, "crt_batch_build: triangles"));
    CRT_CUDA(cudaSetDevice(x->device));
    CRT_TRY(batch_enqueue(x, bt, tris, nullptr, 0, nullptr, nullptr));
    CRT_TRY(batch_check(x, bt));
    bt->built = true;
    return CRT_OK;
}

crt_status crt_batch_predictor_create(crt_ctx* x, crt_batch* bt, const crt_predictor_config* cfg, crt_predictor** out) {
    if (!x || !bt || !out) return fail(CRT_ERR_INVALID_ARG, "crt_batch_predictor_create: null argument");
    if (bt->predictor) return fail(CRT_ERR_INVALID_ARG, "crt_batch_predictor_create: the batch already has a predictor");
    if (!bt->built) return fail(CRT_ERR_INVALID_ARG, "crt_batch_predictor_create: build the batch first");
    CRT_CUDA(cudaSetDevice(x->device));
    crt_predictor* pr = new crt_predictor();
    crt_predictor_default_config(&pr->cfg);
    if (cfg) pr->cfg = *cfg;
    if (pr->cfg.train_stride == 0) pr->cfg.train_stride = 1;
    if (pr->cfg.batch == 0) pr->cfg.batch = 16384;
    pr->batch = bt;
    pr->batch_scenes = bt->scenes.as<crt::BatchScene>();
    pr->batch_nodes = bt->nodes.as<crt_bvh_node>();
    pr->batch_n_scenes = bt->n_scenes;
    pr->batch_n_tris = bt->n_tris;
    const size_t n_rays = bt->ray_cap;
    crt_status s = pr->params.reserve(4 * sizeof(float) * crt::pred::kParams);
    if (s == CRT_OK) s = pr->w16.reserve(sizeof(__half) * crt::pred::kHalfs);
    if (s == CRT_OK) s = pr->scratch.reserve(16);
    // the trace's inference and ordering buffers, sized now so that a captured graph allocates nothing
    if (s == CRT_OK) s = pr->classes.reserve(2 * n_rays + 16);
    if (s == CRT_OK) s = pr->order.reserve(4 * n_rays + 16);
    if (s == CRT_OK) s = pr->order_scratch.reserve(crt::pred_order_scratch_bytes(static_cast<uint32_t>(n_rays)));
    if (s == CRT_OK && crt::pred_prepare() != cudaSuccess) s = fail(CRT_ERR_CUDA, "predictor kernel attributes");
    if (s == CRT_OK) {
        crt::pred_init(pr->dev(), pr->cfg.seed, x->stream);
        s = predictor_targets(x, pr);
    }
    if (s != CRT_OK) {
        pr->batch = nullptr;
        crt_predictor_destroy(pr);
        return s;
    }
    bt->predictor = pr;
    bt->drop_graph();
    *out = pr;
    return CRT_OK;
}

crt_status crt_batch_trace(crt_ctx* x, crt_batch* bt, const crt_ray* rays, uint32_t flags, crt_hit* hits) {
    if (!x || !bt || !rays || !hits) return fail(CRT_ERR_INVALID_ARG, "crt_batch_trace: null argument");
    CRT_TRY(batch_trace_flags(bt, flags, "crt_batch_trace"));
    if (!is_device_ptr(rays) || !is_device_ptr(hits)) return fail(CRT_ERR_INVALID_ARG, "crt_batch_trace: device memory only");
    CRT_TRY(check_aligned16(rays, "crt_batch_trace: rays"));
    CRT_TRY(check_aligned16(hits, "crt_batch_trace: hits"));
    CRT_CUDA(cudaSetDevice(x->device));
    CRT_TRY(batch_order_buffers(bt, flags));
    CRT_CUDA(cudaMemsetAsync(bt->err.p, 0, 16, x->stream));
    const bool deep = bt->cfg.stack_depth > 64 || bt->max_iters + 2 > 64;
    CRT_TRY(batch_trace_enqueue(x, bt, rays, flags, hits, deep));
    return batch_check(x, bt);
}

crt_status crt_batch_run(crt_ctx* x, crt_batch* bt, const crt_triangle* tris, const crt_ray* rays, uint32_t flags,
                         crt_hit* hits, int use_graph, int* graph_used) {
    if (!x || !bt || !tris || !rays || !hits) return fail(CRT_ERR_INVALID_ARG, "crt_batch_run: null argument");
    CRT_TRY(batch_trace_flags(bt, flags, "crt_batch_run"));
    CRT_TRY(check_batch_buffers(tris, rays, hits, "crt_batch_run"));
    CRT_CUDA(cudaSetDevice(x->device));
    CRT_TRY(batch_order_buffers(bt, flags));  // before any graph capture: no allocation inside it
    if (graph_used) *graph_used = 0;
    if (bt->max_iters + 2 > 64) bt->cfg.stack_depth = 1024;
    if (use_graph) {
        // the graph bakes in the ray count of every launch; the scene table it
        // reads holds the current counts, so it replays only with the counts
        // it was captured with
        const bool same = bt->graph && bt->g_tris == tris && bt->g_rays == rays && bt->g_hits == hits &&
                          bt->g_flags == flags && std::memcmp(&bt->g_cfg, &bt->cfg, sizeof(crt_config)) == 0 &&
                          bt->g_counts == bt->ray_counts();
        if (!same) {
            bt->drop_graph();
            cudaGraph_t g = nullptr;
            bool ok = cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            crt_status es = CRT_OK;
            if (ok) es = batch_enqueue(x, bt, tris, rays, flags, hits, nullptr);
            cudaError_t ce = cudaStreamEndCapture(x->stream, &g);
            ok = ok && es == CRT_OK && ce == cudaSuccess && g != nullptr;
            if (ok) ok = cudaGraphInstantiate(&bt->graph, g, 0) == cudaSuccess;
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            if (!ok) {
                bt->graph = nullptr;
            } else {
                bt->g_tris = tris; bt->g_rays = rays; bt->g_hits = hits; bt->g_flags = flags; bt->g_cfg = bt->cfg;
                bt->g_counts = bt->ray_counts();
            }
        }
        if (bt->graph) {
            CRT_CUDA(cudaGraphLaunch(bt->graph, x->stream));
            if (graph_used) *graph_used = 1;
            CRT_TRY(batch_check(x, bt));
            bt->built = true;
            return CRT_OK;
        }
    }
    CRT_TRY(batch_enqueue(x, bt, tris, rays, flags, hits, nullptr));
    CRT_TRY(batch_check(x, bt));
    bt->built = true;
    return CRT_OK;
}

crt_status crt_batch_set_ray_counts(crt_ctx* x, crt_batch* bt, const uint32_t* ray_counts) {
    if (!x || !bt || !ray_counts) return fail(CRT_ERR_INVALID_ARG, "crt_batch_set_ray_counts: null argument");
    uint64_t total = 0;
    for (uint32_t k = 0; k < bt->n_scenes; ++k) total += ray_counts[k];
    if (total > bt->ray_cap)
        return fail(CRT_ERR_INVALID_ARG, "crt_batch_set_ray_counts: %llu rays exceed the batch's %u",
                    static_cast<unsigned long long>(total), bt->ray_cap);
    CRT_CUDA(cudaSetDevice(x->device));
    // the device table also holds what the last build wrote (slack, iterations): take it, change the ray fields
    CRT_CUDA(cudaMemcpyAsync(bt->hs.data(), bt->scenes.p, sizeof(crt::BatchScene) * bt->n_scenes, cudaMemcpyDeviceToHost,
                             x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    uint32_t off = 0;
    for (uint32_t k = 0; k < bt->n_scenes; ++k) {
        bt->hs[k].ray_off = off;
        bt->hs[k].n_rays = ray_counts[k];
        off += ray_counts[k];
    }
    CRT_CUDA(cudaMemcpyAsync(bt->scenes.p, bt->hs.data(), sizeof(crt::BatchScene) * bt->n_scenes, cudaMemcpyHostToDevice,
                             x->stream));
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    bt->n_rays = off;
    return CRT_OK;
}

crt_status crt_batch_bounce_rays(crt_ctx* x, crt_batch* bt, uint32_t scene, const crt_ray* primary, const crt_hit* hits,
                                 uint32_t n_primary, uint32_t n_out, uint32_t seed, crt_ray* out) {
    if (!x || !bt || !primary || !hits || !out || scene >= bt->n_scenes)
        return fail(CRT_ERR_INVALID_ARG, "crt_batch_bounce_rays: bad argument");
    if (!bt->built) return fail(CRT_ERR_INVALID_ARG, "crt_batch_bounce_rays: build the batch first");
    if (!is_device_ptr(primary) || !is_device_ptr(hits) || !is_device_ptr(out))
        return fail(CRT_ERR_INVALID_ARG, "crt_batch_bounce_rays: device memory only");
    CRT_TRY(check_aligned16(primary, "crt_batch_bounce_rays: primary rays"));
    CRT_TRY(check_aligned16(hits, "crt_batch_bounce_rays: hits"));
    CRT_TRY(check_aligned16(out, "crt_batch_bounce_rays: rays"));
    CRT_CUDA(cudaSetDevice(x->device));
    if (n_out == 0) return CRT_OK;
    const crt::BatchScene& sc = bt->hs[scene];
    CRT_TRY(x->pos.reserve(crt::bounce_scratch_bytes(n_primary)));
    crt::launch_bounce(primary, hits, n_primary, bt->xtri.as<float4>() + 3 * static_cast<size_t>(sc.tri_off),
                       bt->inv_perm.as<uint32_t>() + sc.tri_off, sc.n_tris, n_out, seed, out, x->pos.as<uint32_t>(),
                       x->stream);
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaStreamSynchronize(x->stream));
    return CRT_OK;
}

crt_status crt_batch_copy_nodes(crt_ctx* x, const crt_batch* bt, uint32_t scene, crt_bvh_node* dst) {
    if (!x || !bt || !dst || scene >= bt->n_scenes) return fail(CRT_ERR_INVALID_ARG, "crt_batch_copy_nodes: bad argument");
    const crt::BatchScene& sc = bt->hs[scene];
    return copy_out(x, dst, bt->nodes.as<crt_bvh_node>() + sc.node_off, sizeof(crt_bvh_node) * (2ull * sc.n_tris - 1));
}

crt_status crt_batch_scene_info(const crt_batch* bt, uint32_t scene, uint32_t info[4]) {
    if (!bt || !info || scene >= bt->n_scenes) return fail(CRT_ERR_INVALID_ARG, "crt_batch_scene_info: bad argument");
    const crt::BatchScene& sc = bt->hs[scene];
    info[0] = sc.n_tris;
    info[1] = sc.n_rays;
    info[2] = sc.n_tris > 1 ? sc.iters : 0;
    info[3] = sc.tri_off;
    return CRT_OK;
}

crt_status crt_batch_autotune(crt_ctx* x, crt_batch* bt, const crt_triangle* tris, const crt_ray* rays, uint32_t flags,
                              crt_hit* hits, crt_config* best, float* best_ms) {
    if (!x || !bt || !tris || !rays || !hits) return fail(CRT_ERR_INVALID_ARG, "crt_batch_autotune: null argument");
    CRT_TRY(check_batch_buffers(tris, rays, hits, "crt_batch_autotune"));
    CRT_CUDA(cudaSetDevice(x->device));
    CRT_TRY(batch_order_buffers(bt, flags));
    cudaEvent_t e0, e1, e2;
    CRT_CUDA(cudaEventCreate(&e0));
    CRT_CUDA(cudaEventCreate(&e1));
    CRT_CUDA(cudaEventCreate(&e2));
    const crt_config start = bt->cfg;
    crt_config bestc = start;
    float best_total = 1e30f, best_build = 0.f;
    auto run = [&](float* ms_build, float* ms_total) -> crt_status {
        CRT_CUDA(cudaEventRecord(e0, x->stream));
        CRT_TRY(batch_enqueue(x, bt, tris, rays, flags, hits, e1));
        CRT_CUDA(cudaEventRecord(e2, x->stream));
        CRT_TRY(batch_check(x, bt));
        CRT_CUDA(cudaEventElapsedTime(ms_build, e0, e1));
        CRT_CUDA(cudaEventElapsedTime(ms_total, e0, e2));
        return CRT_OK;
    };
    // build parameters (with the default trace shape)
    for (uint32_t radius : {8u, 16u, 32u})
        for (uint32_t bits : {4u, 8u}) {
            bt->cfg = start;
            bt->cfg.ploc_radius = radius;
            bt->cfg.sort_digit_bits = bits;
            bt->cfg.trace_block = 128;
            bt->cfg.stack_depth = 1024;
            float b = 0.f, t = 0.f;
            CRT_TRY(run(&b, &t));  // warm-up (also sizes the trees)
            CRT_TRY(run(&b, &t));
            if (t < best_total) { best_total = t; best_build = b; bestc = bt->cfg; }
        }
    // trace parameters on the chosen build
    bt->cfg = bestc;
    float b = 0.f, t = 0.f;
    CRT_TRY(run(&b, &t));
    const bool shallow = bt->max_iters + 2 <= 64;
    float best_trace = 1e30f;
    crt_config bt_cfg = bestc;
    for (uint32_t block : {128u, 256u, 512u})
        for (uint32_t stack : {64u, 1024u}) {
            if (stack == 64 && !shallow) continue;
            bt->cfg.trace_block = block;
            bt->cfg.stack_depth = stack;
            CRT_TRY(run(&b, &t));
            CRT_TRY(run(&b, &t));
            if (t - b < best_trace) { best_trace = t - b; bt_cfg = bt->cfg; }
        }
    bt->cfg = bt_cfg;
    bt->drop_graph();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (best) *best = bt->cfg;
    if (best_ms) *best_ms = best_build + best_trace;
    return CRT_OK;
}

}  // extern "C"

// ===================================================================== shading
namespace {

static_assert(sizeof(crt_mesh_model) == 17 * 4, "crt_mesh_model: 16 floats + material id");
static_assert(sizeof(crt_material) == 16, "crt_material: one RGBA colour");

bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

// Checks a crt_shading and stages what getColor reads (model material ids,
// material colours) in device memory.
crt_status shade_setup(crt_ctx* x, const crt_bvh* b, const crt_shading* sh, crt::ShadeParams* sp) {
    if (!sh) return fail(CRT_ERR_INVALID_ARG, "shading: null crt_shading");
    if (sh->flags & ~(CRT_SHADE_WIREFRAME | CRT_SHADE_BVH))
        return fail(CRT_ERR_INVALID_ARG, "shading: unknown flags 0x%x", sh->flags);
    if (sh->bvh_depth > CRT_SHADE_MAX_BVH_DEPTH)
        return fail(CRT_ERR_INVALID_ARG, "shading: bvh_depth %u > %u", sh->bvh_depth, CRT_SHADE_MAX_BVH_DEPTH);
    if (sh->n_models > crt::kMaxModels) return fail(CRT_ERR_INVALID_ARG, "shading: n_models %u > 64", sh->n_models);
    if ((sh->n_models && !sh->models) || (sh->n_materials && !sh->materials))
        return fail(CRT_ERR_INVALID_ARG, "shading: null models or materials");
    *sp = crt::ShadeParams{};
    sp->flags = sh->flags;
    sp->bvh_depth = sh->bvh_depth;
    sp->inv_perm = b->inv_perm.as<uint32_t>();
    sp->n_tris = b->n;
    if (sh->flags & CRT_SHADE_BVH) CRT_TRY(ensure_node_boxes(x, b));  // the box display walks the node array
    if (sh->n_models) {
        const void* d = nullptr;
        CRT_TRY(stage_in(x, x->shade_models, sh->models, sizeof(crt_mesh_model) * sh->n_models, &d));
        if (!aligned(d, 4)) return fail(CRT_ERR_INVALID_ARG, "shading: models must be 4-byte aligned");
        sp->models = static_cast<const uint32_t*>(d);
        sp->n_models = sh->n_models;
    }
    if (sh->n_materials) {
        const void* d = nullptr;
        CRT_TRY(stage_in(x, x->shade_materials, sh->materials, sizeof(crt_material) * sh->n_materials, &d));
        if (!aligned(d, 16)) return fail(CRT_ERR_INVALID_ARG, "shading: materials must be 16-byte aligned");
        sp->materials = static_cast<const float4*>(d);
        sp->n_materials = sh->n_materials;
    }
    return CRT_OK;
}

// Where the kernel writes n texels for the caller's rgba: device memory,
// page-locked host memory (written by the kernel over the CPU-GPU link), or
// a context buffer that is copied out afterwards (*copy_out).
crt_status image_target(crt_ctx* x, float* rgba, size_t n, float4** dev, bool* copy_out) {
    *copy_out = false;
    void* d = is_device_ptr(rgba) ? static_cast<void*>(rgba) : mapped_host_ptr(rgba);
    if (d) {
        if (!aligned(d, 16)) return fail(CRT_ERR_INVALID_ARG, "rgba must be 16-byte aligned");
        *dev = static_cast<float4*>(d);
        return CRT_OK;
    }
    CRT_TRY(x->image.reserve(16 * n));
    *dev = x->image.as<float4>();
    *copy_out = true;
    return CRT_OK;
}

crt::TraceParams bvh_params(crt_ctx* x, const crt_bvh* b, uint32_t flags) {
    crt::TraceParams p{};
    p.nodes = b->nodes.as<crt_bvh_node>();
    p.xtri = b->xtri.as<float4>();
    p.wide = (flags & CRT_TRI_WATERTIGHT) ? b->wide_wt.as<float4>() : b->wide.as<float4>();
    p.n_nodes = 2 * b->n - 1;
    p.abs_eps = b->abs_eps;
    p.err = x->err.as<uint32_t>();
    return p;
}

}  // namespace

extern "C" {

crt_status crt_shade(crt_ctx* x, const crt_bvh* b, const crt_ray* rays, const crt_hit* hits, uint32_t n,
                     const crt_shading* sh, float* rgba) {
    if (!x || !b || !hits || !rgba) return fail(CRT_ERR_INVALID_ARG, "crt_shade: null argument");
    if (sh && (sh->flags & CRT_SHADE_BVH) && !rays)
        return fail(CRT_ERR_INVALID_ARG, "crt_shade: CRT_SHADE_BVH reads the rays");
    if (b->n == 0) return fail(CRT_ERR_INVALID_ARG, "crt_shade: empty bvh");
    CRT_CUDA(cudaSetDevice(x->device));
    crt::ShadeParams sp;
    CRT_TRY(shade_setup(x, b, sh, &sp));
    if (n == 0) return CRT_OK;
    const void* d_hits = nullptr;
    CRT_TRY(stage_in_once(x, x->shade_hits, hits, sizeof(crt_hit) * n, &d_hits));
    const void* d_rays = nullptr;
    if (sp.flags & CRT_SHADE_BVH) CRT_TRY(stage_in_once(x, x->shade_rays, rays, sizeof(crt_ray) * n, &d_rays));
    if (!aligned(d_hits, 16) || !aligned(d_rays, 16))
        return fail(CRT_ERR_INVALID_ARG, "crt_shade: rays and hits must be 16-byte aligned");
    bool copy_out = false;
    CRT_TRY(image_target(x, rgba, n, &sp.image, &copy_out));
    crt::TraceParams p = bvh_params(x, b, 0);
    p.rays = static_cast<const crt_ray*>(d_rays);
    p.hits = static_cast<crt_hit*>(const_cast<void*>(d_hits));
    p.n_rays = n;
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    crt::launch_shade(p, sp, x->stream);
    CRT_CUDA(cudaGetLastError());
    if (copy_out) CRT_CUDA(cudaMemcpyAsync(rgba, sp.image, 16 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, x->stream));
    return x->check_device_error();
}

crt_status crt_render_frame(crt_ctx* x, const crt_bvh* b, const crt_camera* cam, uint32_t width, uint32_t height,
                            uint32_t flags, const crt_shading* sh, float* rgba) {
    if (!x || !b || !cam || !rgba) return fail(CRT_ERR_INVALID_ARG, "crt_render_frame: null argument");
    if (width == 0 || height == 0 || height > 65535 || static_cast<uint64_t>(width) * height > (1ull << 31))
        return fail(CRT_ERR_INVALID_ARG, "bad image size");
    CRT_TRY(check_trace_flags(b, flags));
    if (flags & CRT_TRACE_ANY) return fail(CRT_ERR_INVALID_ARG, "crt_render_frame: primary rays are closest-hit");
    CRT_CUDA(cudaSetDevice(x->device));
    crt::ShadeParams sp;
    CRT_TRY(shade_setup(x, b, sh, &sp));
    const uint32_t n = width * height;
    bool copy_out = false;
    CRT_TRY(image_target(x, rgba, n, &sp.image, &copy_out));
    const crt_camera* d_cam = cam;
    if (!is_device_ptr(cam)) {
        CRT_CUDA(cudaMemcpyAsync(x->cam.p, cam, sizeof(crt_camera), cudaMemcpyHostToDevice, x->stream));
        d_cam = x->cam.as<crt_camera>();
    } else {
        CRT_TRY(check_aligned16(cam, "camera"));
    }
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    const uint32_t tw = (width % 8 == 0 && height % 4 == 0) ? width : 0u;  // 8x4 pixel tiles per warp
    if (!(flags & (CRT_TRACE_USE_PREDICTOR | CRT_TRACE_WIDE | CRT_TRACE_COMPRESSED))) {
        // one launch: camera ray, closest hit and texel per pixel
        crt::TraceParams p = bvh_params(x, b, flags);
        p.n_rays = n;
        p.tile_width = tw;
        if (flags & CRT_TRACE_STATS) {
            CRT_CUDA(cudaMemsetAsync(x->trace_stats.p, 0, 16, x->stream));
            p.stats = x->trace_stats.as<unsigned long long>();
        }
        const bool deep = b->depth_bound + 2 > 64;
        const uint32_t kflags = (flags & CRT_TRI_WATERTIGHT) | (deep ? (1u << 16) : 0u);
        crt::launch_frame(p, d_cam, width, height, 0, height, nullptr, nullptr, kflags,
                          static_cast<int>(x->cfg.trace_block), &sp, x->stream);
        CRT_CUDA(cudaGetLastError());
    } else {
        CRT_TRY(x->frame_rays.reserve(sizeof(crt_ray) * static_cast<size_t>(n)));
        CRT_TRY(x->frame_hits.reserve(sizeof(crt_hit) * static_cast<size_t>(n)));
        crt_ray* rays = x->frame_rays.as<crt_ray>();
        crt_hit* hits = x->frame_hits.as<crt_hit>();
        crt::launch_raygen(d_cam, width, height, rays, x->stream);
        CRT_TRY(trace_device(x, b, rays, n, flags, hits, nullptr, tw));
        crt::TraceParams p = bvh_params(x, b, flags);
        p.rays = rays;
        p.hits = hits;
        p.n_rays = n;
        crt::launch_shade(p, sp, x->stream);
        CRT_CUDA(cudaGetLastError());
    }
    if (copy_out) CRT_CUDA(cudaMemcpyAsync(rgba, sp.image, 16 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, x->stream));
    CRT_TRY(x->check_device_error());
    if (flags & CRT_TRACE_STATS) CRT_CUDA(cudaMemcpy(x->last_trace_stats, x->trace_stats.p, 16, cudaMemcpyDeviceToHost));
    return CRT_OK;
}

}  // extern "C"

// ===================================================================== mesh input
extern "C" {

crt_status crt_obj_parse(const char* text, size_t len, float* vertices, uint32_t vert_cap, uint32_t* indices,
                         uint32_t tri_cap, uint32_t counts[2]) {
    if (!text || !counts) return fail(CRT_ERR_INVALID_ARG, "crt_obj_parse: null text or counts");
    uint64_t nv = 0, nt = 0;
    std::string err;
    if (!crt::obj_parse(text, len, vertices, vertices ? vert_cap : 0, indices, indices ? tri_cap : 0, &nv, &nt, &err))
        return fail(CRT_ERR_BAD_INPUT, "crt_obj_parse: %s", err.c_str());
    if (nv > 0xFFFFFFFFull || nt > 0xFFFFFFFFull) return fail(CRT_ERR_BAD_INPUT, "crt_obj_parse: more than 2^32 elements");
    counts[0] = static_cast<uint32_t>(nv);
    counts[1] = static_cast<uint32_t>(nt);
    return CRT_OK;
}

crt_status crt_triangles_from_indexed(crt_ctx* x, const float* vertices, uint32_t n_vertices, const uint32_t* indices,
                                      uint32_t n_triangles, uint32_t model_id, crt_triangle* out) {
    if (!x || !out || (n_triangles && (!vertices || !indices)))
        return fail(CRT_ERR_INVALID_ARG, "crt_triangles_from_indexed: null argument");
    CRT_CUDA(cudaSetDevice(x->device));
    if (n_triangles == 0) return CRT_OK;
    const void* d_v = nullptr;
    const void* d_i = nullptr;
    CRT_TRY(stage_in(x, x->mesh_vertices, vertices, 12ull * n_vertices, &d_v));
    CRT_TRY(stage_in(x, x->mesh_indices, indices, 12ull * n_triangles, &d_i));
    if (!aligned(d_v, 4) || !aligned(d_i, 4))
        return fail(CRT_ERR_INVALID_ARG, "crt_triangles_from_indexed: vertices and indices must be 4-byte aligned");
    const bool dev_out = is_device_ptr(out);
    crt_triangle* d_out = out;
    if (!dev_out) {
        CRT_TRY(x->mesh_out.reserve(sizeof(crt_triangle) * static_cast<size_t>(n_triangles)));
        d_out = x->mesh_out.as<crt_triangle>();
    } else if (!aligned(out, 16)) {
        return fail(CRT_ERR_INVALID_ARG, "crt_triangles_from_indexed: out must be 16-byte aligned");
    }
    CRT_CUDA(cudaMemsetAsync(x->err.p, 0, 16, x->stream));
    crt::launch_indexed(static_cast<const float*>(d_v), n_vertices, static_cast<const uint32_t*>(d_i), n_triangles,
                        model_id, d_out, x->err.as<uint32_t>(), x->stream);
    CRT_CUDA(cudaGetLastError());
    if (!dev_out)
        CRT_CUDA(cudaMemcpyAsync(out, d_out, sizeof(crt_triangle) * static_cast<size_t>(n_triangles),
                                 cudaMemcpyDeviceToHost, x->stream));
    return x->check_device_error();
}

}  // extern "C"
