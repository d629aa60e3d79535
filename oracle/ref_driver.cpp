// Oracle (test infrastructure only): a C-ABI driver around the reference's
// own BVH builder.
//
// Compiled together with the reference's UNMODIFIED
//   srcCommon/scene/geometry/bvh.cpp       (BVH::BVH, bvh.cpp:11-24; PLOC bvh.cpp:48-210)
//   srcCommon/scene/geometry/triangle.cpp  (Triangle::getCentroid, triangle.cpp:31-33)
// read in place from the reference checkout, against the project-written glm
// shim in oracle/glm_shim.  The recipe is oracle/Makefile; the library lands
// in oracle/_ref/ and is never shipped with the product.
//
// What the driver adds on top of the reference classes:
//   * the DFS pre-order flattening of Scene::recursiveTopDownTraversalBVH /
//     Scene::getBVH_NodesToGPUData (srcOpenGL/scene/scene.cpp:189-208),
//     restated here because scene.cpp needs OpenGL;
//   * read-out of the Morton codes, which the reference keeps private
//     (BVH::getMortonCodes bvh.cpp:330-348 and
//     BVH::sortMortonCodesAndTriangleIndices bvh.cpp:214-232).
// The reference caps scenes at Triangle::MAX_NB_TRIANGLES = 65,536 triangles
// (triangle.hpp:21) and Mesh::MAX_NB_MESHES = 64 meshes (mesh.hpp:26).
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <numeric>
#include <optional>
#include <string>
#include <vector>

#include <glm/glm.hpp>

#define private public
#include "bvh.hpp"
#undef private

namespace {

struct NodeOut {  // byte image of cr::BVH_NodeGPU (bvh.hpp:36-42), 48 bytes
    float mn[3];
    float pad0;
    float mx[3];
    float pad1;
    uint32_t tri, left, right, pad2;
};
static_assert(sizeof(NodeOut) == 48, "node image");
static_assert(sizeof(cr::BVH_NodeGPU) == 48, "reference node size");
static_assert(sizeof(cr::TriangleGPU) == 64, "reference triangle size");

// scene.cpp:189-201 restated: pre-order, left subtree first.
void flatten(const cr::BVH& bvh, uint32_t root, std::vector<NodeOut>& out) {
    struct Frame { uint32_t id; uint32_t pos; int state; };
    std::vector<Frame> st;
    auto emit = [&](uint32_t id) -> uint32_t {
        const cr::BVH_NodeGPU n = bvh._InternalStruct._Clusters[id].value();
        NodeOut o{};
        o.mn[0] = n._BoundingBox._Min.x; o.mn[1] = n._BoundingBox._Min.y; o.mn[2] = n._BoundingBox._Min.z;
        o.mx[0] = n._BoundingBox._Max.x; o.mx[1] = n._BoundingBox._Max.y; o.mx[2] = n._BoundingBox._Max.z;
        o.tri = n._TriangleId; o.left = n._LeftChild; o.right = n._RightChild;
        out.push_back(o);
        return static_cast<uint32_t>(out.size() - 1);
    };
    st.push_back({root, emit(root), 0});
    while (!st.empty()) {
        Frame& f = st.back();
        const bool leaf = bvh._InternalStruct._IsLeaf[f.id].has_value();  // `!_IsLeaf[id]` in scene.cpp:193
        if (leaf || f.state == 2) { st.pop_back(); continue; }
        if (f.state == 0) {
            f.state = 1;
            const uint32_t c = bvh._InternalStruct._LeftChild[f.id].value();
            out[f.pos].left = static_cast<uint32_t>(out.size());
            const uint32_t p = emit(c);
            st.push_back({c, p, 0});
        } else {
            f.state = 2;
            const uint32_t c = bvh._InternalStruct._RightChild[f.id].value();
            out[f.pos].right = static_cast<uint32_t>(out.size());
            const uint32_t p = emit(c);
            st.push_back({c, p, 0});
        }
    }
}

}  // namespace

extern "C" {

uint32_t ref_max_triangles(void) { return static_cast<uint32_t>(cr::Triangle::MAX_NB_TRIANGLES); }
uint32_t ref_max_meshes(void) { return static_cast<uint32_t>(cr::Mesh::MAX_NB_MESHES); }

// Builds the BVH with the reference's constructor and writes:
//   codes_unsorted[n_tris]  Morton code of triangle i (may be null)
//   codes_sorted[n_tris], perm[n_tris]   the sorted (code, index) pairs
//   nodes[2*n_tris-1]       the DFS node array Scene::getBVH_NodesToGPUData uploads
//   ctor_ms                 wall time of cr::BVH::BVH (may be null)
// tris: n_buffer TriangleGPU records (the reference scans all of them for the
// scene box); models: n_models MeshModelGPU records (68 bytes each), padded
// with identity matrices to 64 as Scene::getMeshModelToGPUData does.
// Returns 0 on success, -1 on an unsupported size.
int ref_bvh_build(const void* tris, uint32_t n_buffer, uint32_t n_tris,
                  const void* models, uint32_t n_models,
                  uint32_t* codes_unsorted, uint32_t* codes_sorted, uint32_t* perm,
                  void* nodes, double* ctor_ms) {
    if (n_tris == 0 || n_tris > cr::Triangle::MAX_NB_TRIANGLES || n_buffer < n_tris ||
        n_models > cr::Mesh::MAX_NB_MESHES)
        return -1;
    std::vector<cr::TriangleGPU> tv(n_buffer);
    std::memcpy(tv.data(), tris, sizeof(cr::TriangleGPU) * n_buffer);
    for (const auto& t : tv)
        if (t._ModelId >= cr::Mesh::MAX_NB_MESHES) return -1;
    std::vector<cr::MeshModelGPU> mv(cr::Mesh::MAX_NB_MESHES);
    const unsigned char* mb = static_cast<const unsigned char*>(models);
    for (uint32_t m = 0; m < n_models; ++m) {
        std::memcpy(&mv[m]._ModelMatrix, mb + 68 * m, 64);
        std::memcpy(&mv[m]._MaterialId, mb + 68 * m + 64, 4);
    }

    const auto t0 = std::chrono::steady_clock::now();
    auto bvh = std::make_unique<cr::BVH>(n_tris, tv, mv);
    const auto t1 = std::chrono::steady_clock::now();
    if (ctor_ms) *ctor_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();

    if (codes_unsorted) {
        const std::vector<uint32_t> c = bvh->getMortonCodes();
        std::memcpy(codes_unsorted, c.data(), sizeof(uint32_t) * n_tris);
    }
    {
        std::vector<uint32_t> idx(cr::Triangle::MAX_NB_TRIANGLES), codes;
        bvh->sortMortonCodesAndTriangleIndices(idx, codes);
        std::memcpy(codes_sorted, codes.data(), sizeof(uint32_t) * n_tris);
        std::memcpy(perm, idx.data(), sizeof(uint32_t) * n_tris);
    }
    std::vector<NodeOut> out;
    out.reserve(2 * static_cast<size_t>(n_tris) - 1);
    flatten(*bvh, 2 * n_tris - 2, out);
    if (out.size() != 2 * static_cast<size_t>(n_tris) - 1) return -2;
    std::memcpy(nodes, out.data(), sizeof(NodeOut) * out.size());
    return 0;
}

}  // extern "C"
