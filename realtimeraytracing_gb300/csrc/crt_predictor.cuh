// Learned hit predictor: parameter layout and the device view shared by the
// predictor kernels (crt_predictor.cu), the seeded traversal (crt_trace.cu)
// and the C ABI (crt_api.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "crt.h"

namespace crt {
namespace pred {

constexpr int kIn = 32;            // input features: 16 origin-cell + 16 direction-bin embedding values
constexpr int kHid = 64;           // hidden width
constexpr int kClasses = 128;      // 127 treelets + "miss"
constexpr int kMissClass = kClasses - 1;
constexpr int kGrid = 64;          // origin cells per axis
constexpr int kDirBins = 32;       // octahedral direction bins per axis
constexpr int kEmb = 16;           // embedding width per table
constexpr size_t kEo = static_cast<size_t>(kGrid) * kGrid * kGrid;
constexpr size_t kEd = static_cast<size_t>(kDirBins) * kDirBins;

// FP32 master parameters (and Adam moments, gradients) in one flat array.
constexpr size_t oW1 = 0;                        // [64][32]  (out, in)
constexpr size_t oB1 = oW1 + kHid * kIn;         // [64]
constexpr size_t oW2 = oB1 + kHid;               // [64][64]
constexpr size_t oB2 = oW2 + kHid * kHid;        // [64]
constexpr size_t oW3 = oB2 + kHid;               // [128][64]
constexpr size_t oB3 = oW3 + kClasses * kHid;    // [128]
constexpr size_t oEo = oB3 + kClasses;           // [64^3][16]
constexpr size_t oEd = oEo + kEo * kEmb;         // [32*32][16]
constexpr size_t kParams = oEd + kEd * kEmb;

// fp16 copies read by the kernels (row-major), incl. transposes for backward.
constexpr size_t hW1 = 0;                        // [64][32]
constexpr size_t hW2 = hW1 + kHid * kIn;         // [64][64]
constexpr size_t hW3 = hW2 + kHid * kHid;        // [128][64]
constexpr size_t hW1T = hW3 + kClasses * kHid;   // [32][64]
constexpr size_t hW2T = hW1T + kIn * kHid;       // [64][64]
constexpr size_t hW3T = hW2T + kHid * kHid;      // [64][128]
constexpr size_t hEo = hW3T + kHid * kClasses;   // [64^3][16]
constexpr size_t hEd = hEo + kEo * kEmb;         // [1024][16]
constexpr size_t kHalfs = hEd + kEd * kEmb;

}  // namespace pred

struct BatchScene;

struct PredictorDev {
    float* master = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    __half* w16 = nullptr;
    const uint8_t* tri_class = nullptr;   // triangle id -> treelet class (a batch: concatenated scenes)
    uint32_t n_tris = 0;
    // A predictor over a batch of scenes: the batch's scene table.  A ray
    // belongs to the scene whose ray range holds it; its features are taken
    // on that scene's box, with the origin cell hashed by the scene index;
    // its class is a treelet of that scene (or miss).  n_scenes 0: one BVH.
    const BatchScene* scenes = nullptr;
    uint32_t n_scenes = 0;
};

// A subtree of the BVH cut: its box, traversal reference and leaf range.
struct Treelet {
    float mn[3];
    uint32_t ref;
    float mx[3];
    uint32_t first;
    uint32_t count;
    uint32_t pad[3];
};
static_assert(sizeof(Treelet) == 48, "treelet record");

void pred_init(const PredictorDev& P, uint32_t seed, cudaStream_t s);
// Sets the kernels' shared-memory attributes (done again on first use; call
// before capturing predictor work into a graph).
cudaError_t pred_prepare();
// classes[i]: with argmax the likeliest of the 128 classes (treelets and
// miss), used to order rays; otherwise the likeliest treelet unless P(miss) >=
// miss_threshold (then the miss class), the seeding rule.
// order_keys (with argmax): also each ray's trace order key (see pred_order)
// at order_keys[i], and the keys' digit histograms added into order_hist,
// both from pred_order_begin; rays in several calls (pieces of one array)
// pass order_keys + the piece's offset and the same order_hist.  rays_copy
// (device, optional): receives a copy of the rays, which may then be read from
// page-locked host memory (its device-mapped address, 16-byte aligned).
cudaError_t pred_infer(const PredictorDev& P, const crt_bvh_node* nodes, const crt_ray* rays, uint32_t n,
                       uint16_t* classes, float miss_threshold, bool argmax, uint32_t* err, cudaStream_t s,
                       uint32_t* order_keys = nullptr, uint32_t* order_hist = nullptr, crt_ray* rays_copy = nullptr);
cudaError_t pred_train_step(const PredictorDev& P, const crt_bvh_node* nodes, const crt_ray* rays, uint32_t n_rays,
                            const crt_hit* hits, const uint16_t* targets, uint32_t n_samples, uint32_t stride,
                            uint32_t offset, float* loss_sum, uint32_t* err, cudaStream_t s);
void pred_adam(const PredictorDev& P, float scale, float lr, uint32_t step, cudaStream_t s);
void pred_refresh_fp16(const PredictorDev& P, cudaStream_t s);
// Trace order of rays: by predicted class, then the Morton code of the origin
// cell (32^3 grid of the root box), then the direction bin (a stable radix
// sort of 32-bit keys); order[k] = index of the k-th ray.  scratch holds
// pred_order_scratch_bytes(n).
size_t pred_order_scratch_bytes(uint32_t n);
// With P.n_scenes != 0 (a batch) the key is (scene, predicted class, origin
// cell on a 16^3 grid of the scene's box, direction bin's first coordinate).
// keys_ready: the keys and histograms are already in scratch (pred_order_begin,
// then pred_infer with them); otherwise they are computed from the classes.
void pred_order(const PredictorDev& P, const crt_bvh_node* nodes, const crt_ray* rays, const uint16_t* classes,
                uint32_t n, uint32_t* order, void* scratch, uint32_t* err, uint32_t spin_limit, cudaStream_t s,
                bool keys_ready = false);
// Clears the ordering's histograms and look-back words in scratch (sized for
// n rays) and returns where pred_infer writes the keys and histograms.
void pred_order_begin(void* scratch, uint32_t n, uint32_t** keys, uint32_t** hist, cudaStream_t s);
void pred_treelets(const crt_bvh_node* nodes, const float4* wide, const float4* xtri, uint32_t n_leaves,
                   Treelet* tl, uint32_t* n_tl, uint8_t* tri_class, cudaStream_t s);
// Every scene of a batch cut into <= 127 treelets: scene k's at tl + 128 k,
// their count at n_tl[k]; tri_class of the concatenated triangles.
void pred_treelets_batch(const BatchScene* scenes, uint32_t n_scenes, uint32_t n_tris, const crt_bvh_node* nodes,
                         const float4* wide, const float4* xtri, Treelet* tl, uint32_t* n_tl, uint8_t* tri_class,
                         cudaStream_t s);
// Class of each hit of a batch's rays (treelet of its triangle in the ray's scene, or miss).
void pred_classes_of_hits(const PredictorDev& P, const crt_hit* hits, uint32_t n, uint16_t* out, cudaStream_t s);
// Failure-detection probe of the predictor kernels' MMA wait (one CTA, one
// MMA or none): out[128] receives 16.0 per thread when complete != 0.
cudaError_t tc_wait_probe(int complete, uint32_t limit, uint32_t* err, float* out, cudaStream_t s);
size_t bounce_scratch_bytes(uint32_t n_prim);
void launch_bounce(const crt_ray* prim, const crt_hit* hits, uint32_t n_prim, const float4* xtri,
                   const uint32_t* inv_perm, uint32_t n_tris, uint32_t n_out, uint32_t seed, crt_ray* out,
                   uint32_t* scratch, cudaStream_t s);

}  // namespace crt
