// Shared device helpers of libcrt (sm_103a).
//
// Exactness rules (the build and trace translation units are compiled with
// -fmad=false and IEEE division/sqrt, so every float operation below rounds
// once, in the order written — the order the reference evaluates it in):
//   * min/max follow std::min/std::max (srcCommon/scene/geometry/bvh.cpp) and
//     GLSL min/max (srcCommon/shaders/raytracer.glsl):
//         max(a, b) = a < b ? b : a,   min(a, b) = b < a ? b : a;
//   * mat4 * vec4 follows glm: (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "crt.h"

namespace crt {

constexpr int kNumSms = 152;             // GB300: 2 dies x 76 SMs
constexpr uint32_t kMaxModels = 64;      // Mesh::MAX_NB_MESHES (mesh.hpp:26)

__device__ __forceinline__ float max_std(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float min_std(float a, float b) { return (b < a) ? b : a; }

// glm mat4 * vec4 on a column-major matrix.
__device__ __forceinline__ float4 mat_vec(const float* __restrict__ m, float4 v) {
    float4 r;
    r.x = (m[0] * v.x + m[4] * v.y) + (m[8] * v.z + m[12] * v.w);
    r.y = (m[1] * v.x + m[5] * v.y) + (m[9] * v.z + m[13] * v.w);
    r.z = (m[2] * v.x + m[6] * v.y) + (m[10] * v.z + m[14] * v.w);
    r.w = (m[3] * v.x + m[7] * v.y) + (m[11] * v.z + m[15] * v.w);
    return r;
}

// Triangle record (crt_triangle, 64 bytes) read as four 16-byte vectors.
struct TriRec {
    float4 p0, p1, p2;
    uint32_t model;
};

__device__ __forceinline__ TriRec load_tri(const crt_triangle* __restrict__ t, uint64_t i) {
    const float4* p = reinterpret_cast<const float4*>(t + i);
    TriRec r;
    r.p0 = __ldg(p + 0);
    r.p1 = __ldg(p + 1);
    r.p2 = __ldg(p + 2);
    r.model = __ldg(reinterpret_cast<const uint32_t*>(p + 3));
    return r;
}

// Order-preserving map of a float to uint32 (NaN excluded by callers);
// -0 and +0 map to the same key.
__device__ __forceinline__ uint32_t ordered_key(float v) {
    uint32_t b = __float_as_uint(v);
    if ((b & 0x7FFFFFFFu) == 0u) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Bounded spin with back-off; returns false when the bound is exhausted.
struct SpinBound {
    uint32_t left;
    __device__ explicit SpinBound(uint32_t limit) : left(limit) {}
    __device__ __forceinline__ bool step() {
        if (left == 0) return false;
        --left;
        if ((left & 63u) == 0u) __nanosleep(64);
        return true;
    }
};

__device__ __forceinline__ uint64_t ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned int* p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Relaxed (not ordering) gpu-scope accesses: for a status word whose flag and
// payload share one 32-bit word, so no other data has to be made visible.
// Unlike acquire loads, several of these can be in flight at once.
__device__ __forceinline__ uint32_t ld_relaxed_u32(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u32(unsigned int* p, unsigned int v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Atomic add with acquire-release semantics at gpu scope: the caller's
// earlier writes are visible to a thread that later observes this add, and
// writes released before any add this one observes are visible afterwards.
__device__ __forceinline__ uint32_t atomic_add_acq_rel_u32(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Nanoseconds of the GPU's global timer.
// Acquire-release fence at device scope (lighter than __threadfence's
// sequentially consistent one).
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Device-side error word, set by any kernel whose bounded wait ran out or
// whose input is unusable; read by the host after each stage.
enum DevError : uint32_t {
    kDevOk = 0,
    kDevTimeout = 1u << 0,
    kDevBadModel = 1u << 1,
    kDevStackOverflow = 1u << 2,
    kDevIterLimit = 1u << 3,
    kDevCorrupt = 1u << 4,   // an index check failed; the access was skipped
    kDevBadIndex = 1u << 5,  // an input triangle names a vertex past the end
};

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t code) { atomicOr(err, code); }

// Records the first failed index check: err[1] = site, err[2..3] = values.
__device__ __forceinline__ void raise_corrupt(uint32_t* err, uint32_t site, uint32_t v0, uint32_t v1) {
    atomicOr(err, static_cast<uint32_t>(kDevCorrupt));
    if (atomicCAS(err + 1, 0u, site) == 0u) {
        err[2] = v0;
        err[3] = v1;
    }
}

}  // namespace crt
