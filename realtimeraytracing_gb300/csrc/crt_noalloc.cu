// crt_morton_sort_noalloc: the Morton-code + radix-sort stage of the build
// for callers that cannot allocate device memory.
//
// Who needs it: a host engine that hands all device memory to its own pool
// and forbids the libraries it embeds from calling cudaMalloc (allocation
// would bypass its budget and can synchronise the device mid-frame), or code
// that runs where allocation is not allowed at all.  crt_build keeps its
// scratch in per-context cudaMalloc'd buffers; this entry point instead uses
// one fixed scratch array compiled into the library, so it calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// Scratch: g_noalloc_scratch, a file-scope __device__ array of
// kNoAllocScratchBytes (about 4.5 MB), present on every GPU that loads the
// library until the process exits.  It limits a call to
// CRT_NOALLOC_MAX_TRIANGLES triangles.  Every call shares it and it keeps the
// previous call's contents, so each call first clears what must start from
// zero; two calls whose work overlaps on the GPU (different streams, or
// different host threads on the same device) race on it and must be
// serialised by the caller.
//
// Host code cannot use the array's name as a device address, so the first
// call on each device looks the address up with cudaGetSymbolAddress while
// that device is current.
// The address is kept per device together with the unique id of the CUDA
// context it was looked up in (cuCtxGetId): after cudaDeviceReset the device
// gets a new primary context, the library's device code is loaded again and
// the array may move, so a call that finds a different context id looks the
// address up again instead of using the stale one.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cuda.h>
#include <cuda_runtime.h>
#include <mutex>

#include "crt.h"
#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {
namespace {

constexpr int kBits = 8;
constexpr int kPasses = (30 + kBits - 1) / kBits;
constexpr uint32_t kRadix = 1u << kBits;
constexpr uint32_t kMaxKeys = CRT_NOALLOC_MAX_TRIANGLES;
constexpr uint32_t kTileKeys = 256u * 16u;   // keys per Onesweep tile (sort_tile_keys(8))
constexpr uint32_t kMaxTiles = (kMaxKeys + kTileKeys - 1) / kTileKeys;

constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }
constexpr size_t kOffState = 0;
constexpr size_t kOffErr = align256(kOffState + sizeof(SceneState));
constexpr size_t kOffModels = align256(kOffErr + 16);
constexpr size_t kOffHist = align256(kOffModels + 2 * 64 * 16 * sizeof(float));
constexpr size_t kLbWordsPerPass = static_cast<size_t>(kMaxTiles) * kRadix + 1;  // + ticket
constexpr size_t kOffLookback = align256(kOffHist + static_cast<size_t>(kPasses) * kRadix * 4);
constexpr size_t kOffKeys = align256(kOffLookback + kPasses * kLbWordsPerPass * 4);
constexpr size_t kKeyBytes = static_cast<size_t>(kMaxKeys) * 4;
constexpr size_t kNoAllocScratchBytes = kOffKeys + 4 * kKeyBytes;  // keys a/b, values a/b

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Resets the parts of the scratch that a call must find cleared: scene-box
// keys, error word, digit histograms, look-back words and tile tickets.
__global__ void noalloc_clear_kernel(unsigned char* scratch) {
    SceneState* st = reinterpret_cast<SceneState*>(scratch + kOffState);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0) {
        for (int a = 0; a < 3; ++a) {
            st->key_max[a] = 0ull;
            st->key_min[a] = ~0ull;
        }
        st->blocks_done = 0u;
        uint32_t* err = reinterpret_cast<uint32_t*>(scratch + kOffErr);
        err[0] = err[1] = err[2] = err[3] = 0u;
    }
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + kOffHist);
    for (uint32_t i = tid; i < kPasses * kRadix; i += gridDim.x * blockDim.x) hist[i] = 0u;
    uint32_t* lb = reinterpret_cast<uint32_t*>(scratch + kOffLookback);
    for (size_t i = tid; i < kPasses * kLbWordsPerPass; i += static_cast<size_t>(gridDim.x) * blockDim.x) lb[i] = 0u;
}

std::mutex g_setup_mu;
// Per device ordinal: the scratch array's device address and the id of the
// context it belongs to (0 = not looked up yet).
struct ScratchSlot {
    unsigned long long ctx_id;
    void* addr;
};
ScratchSlot g_scratch_slot[64] = {};

// Unique id of the calling thread's current CUDA context (never reused
// within a process), through the driver entry points the runtime exposes, so
// that the library needs no link to the driver library.  False when the
// driver cannot tell (no current context yet, or an old driver).
bool current_context_id(unsigned long long* id) {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
        cudaGetLastError();
        resolved = true;
    }
    if (!get_current || !get_id) return false;
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || c == nullptr) return false;
    return get_id(c, id) == CUDA_SUCCESS && *id != 0;
}

crt_status nerr(crt_status s, const char* msg, cudaError_t e = cudaSuccess) {
    char buf[256];
    if (e != cudaSuccess)
        std::snprintf(buf, sizeof(buf), "%s: %s", msg, cudaGetErrorString(e));
    else
        std::snprintf(buf, sizeof(buf), "%s", msg);
    set_last_error(buf);  // read back through crt_last_error_string()
    return s;
}

// Device (or managed) memory of device `dev`: every launch runs on the
// current device, so buffers of another GPU are refused rather than reached
// through peer access.
bool on_device(const void* p, int dev) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}

bool is_device_memory(const void* p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace
}  // namespace crt

extern "C" {

crt_status crt_morton_sort_noalloc(const crt_triangle* tris, uint32_t n_buffer, uint32_t n_tris,
                                   const crt_mesh_model* models, uint32_t n_models, uint32_t* codes_out,
                                   uint32_t* perm_out, void* stream) {
    using namespace crt;
    if (!tris || !codes_out || !perm_out) return nerr(CRT_ERR_INVALID_ARG, "crt_morton_sort_noalloc: null pointer");
    if (n_tris == 0) return nerr(CRT_ERR_INVALID_ARG, "crt_morton_sort_noalloc: n_tris must be >= 1");
    if (n_tris > kMaxKeys)
        return nerr(CRT_ERR_INVALID_ARG,
                    "crt_morton_sort_noalloc: n_tris exceeds CRT_NOALLOC_MAX_TRIANGLES (262144); use crt_build");
    if (n_buffer < n_tris) return nerr(CRT_ERR_INVALID_ARG, "crt_morton_sort_noalloc: n_buffer < n_tris");
    if (n_models > kMaxModels) return nerr(CRT_ERR_INVALID_ARG, "crt_morton_sort_noalloc: more than 64 models");
    if (n_models > 0 && !models) return nerr(CRT_ERR_INVALID_ARG, "crt_morton_sort_noalloc: null models");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return nerr(CRT_ERR_CUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= 64) return nerr(CRT_ERR_UNSUPPORTED, "crt_morton_sort_noalloc: device ordinal above 63");
    if (!on_device(tris, dev) || !on_device(codes_out, dev) || !on_device(perm_out, dev))
        return nerr(CRT_ERR_INVALID_ARG,
                    "crt_morton_sort_noalloc: tris, codes_out and perm_out must be device memory of the current device");
    if (n_models > 0 && is_device_memory(models))
        return nerr(CRT_ERR_INVALID_ARG, "crt_morton_sort_noalloc: models must be host memory");

    unsigned char* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        ScratchSlot& slot = g_scratch_slot[dev];
        unsigned long long id = 0;
        const bool have_id = current_context_id(&id);
        if (!slot.addr || !have_id || slot.ctx_id != id) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return nerr(CRT_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch)", e);
            // the lookup makes the device's primary context current if it was not yet
            if (!have_id && !current_context_id(&id)) id = 0;
            slot.addr = p;
            slot.ctx_id = id;
        }
        scratch = static_cast<unsigned char*>(slot.addr);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // Model table (64 matrices, identity past n_models) and its 1/3-scaled
    // copy for the centroid, staged from the host stack.
    float hm[2 * 64 * 16];
    for (uint32_t m = 0; m < 64; ++m) {
        for (int k = 0; k < 16; ++k) hm[16 * m + k] = (k % 5 == 0) ? 1.f : 0.f;
        if (m < n_models) std::memcpy(hm + 16 * m, models[m].m, 64);
    }
    const volatile float third = 1.f / 3.f;
    for (int k = 0; k < 64 * 16; ++k) hm[64 * 16 + k] = third * hm[k];
    e = cudaMemcpyAsync(scratch + kOffModels, hm, sizeof(hm), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return nerr(CRT_ERR_CUDA, "model upload", e);

    noalloc_clear_kernel<<<kNumSms, 256, 0, s>>>(scratch);
    SceneState* st = reinterpret_cast<SceneState*>(scratch + kOffState);
    uint32_t* err = reinterpret_cast<uint32_t*>(scratch + kOffErr);
    const float* d_models = reinterpret_cast<const float*>(scratch + kOffModels);
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + kOffHist);
    uint32_t* keys_a = reinterpret_cast<uint32_t*>(scratch + kOffKeys);
    uint32_t* keys_b = reinterpret_cast<uint32_t*>(scratch + kOffKeys + kKeyBytes);
    uint32_t* vals_a = reinterpret_cast<uint32_t*>(scratch + kOffKeys + 2 * kKeyBytes);
    uint32_t* vals_b = reinterpret_cast<uint32_t*>(scratch + kOffKeys + 3 * kKeyBytes);

    launch_scene_box(tris, n_buffer, d_models, st, err, s);
    launch_morton(tris, n_tris, d_models + 64 * 16, st, keys_a, hist, kBits, s);
    uint32_t* kin = keys_a;
    uint32_t* vin = nullptr;
    for (int p = 0; p < kPasses; ++p) {
        const bool last = (p == kPasses - 1);
        uint32_t* kout = last ? codes_out : ((p & 1) ? keys_a : keys_b);
        uint32_t* vout = last ? perm_out : ((p & 1) ? vals_a : vals_b);
        uint32_t* lb = reinterpret_cast<uint32_t*>(scratch + kOffLookback) + static_cast<size_t>(p) * kLbWordsPerPass;
        launch_onesweep(kin, vin, kout, vout, n_tris, p * kBits, kBits, hist + p * kRadix, lb + 1, lb, err,
                        1u << 22, s);
        kin = kout;
        vin = vout;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return nerr(CRT_ERR_CUDA, "kernel launch", e);
    uint32_t ew = 0;
    e = cudaMemcpyAsync(&ew, err, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return nerr(CRT_ERR_CUDA, "crt_morton_sort_noalloc", e);
    if (ew & kDevTimeout) return nerr(CRT_ERR_DEVICE_TIMEOUT, "crt_morton_sort_noalloc: a bounded device wait gave up");
    if (ew & kDevBadModel) return nerr(CRT_ERR_BAD_INPUT, "crt_morton_sort_noalloc: a triangle references model id >= 64");
    if (ew) return nerr(CRT_ERR_CUDA, "crt_morton_sort_noalloc: device error word set");
    return CRT_OK;
}

}  // extern "C"
