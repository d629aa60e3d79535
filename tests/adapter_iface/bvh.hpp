// Test-only stand-in for the reference's srcCommon/scene/geometry/bvh.hpp
// (with the parts of triangle.hpp and mesh.hpp it pulls in), written for
// this project so that adapter/bvh_cuda.cpp can be compiled and run where
// the reference checkout is absent (the GPU machines).  It declares only what
// the adapter and the test driver touch, with the reference's names, member
// types and record layouts: TriangleGPU (triangle.hpp:9-14), MeshModelGPU
// (mesh.hpp:12-15), AABB_GPU and BVH_NodeGPU (bvh.hpp:22-42), the
// BVH_Params vectors (bvh.hpp:44-63) and BVH's constructor (bvh.hpp:89-91).
// tests/test_abi.py compares its record sizes and member offsets with the
// real header's, where that header exists.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <optional>
#include <vector>

#include <glm/glm.hpp>

namespace cr {

struct TriangleGPU {
    glm::vec4 _P0;
    glm::vec4 _P1;
    glm::vec4 _P2;
    alignas(16) uint32_t _ModelId;
};

struct Triangle {
    static const uint32_t MAX_NB_TRIANGLES = 2 << 15;
};

struct MeshModelGPU {
    glm::mat4 _ModelMatrix = glm::mat4(1);
    uint32_t _MaterialId = 0;
};

struct Mesh {
    static const size_t MAX_NB_MESHES = 2 << 5;
};

struct AABB_GPU {
    glm::vec3 _Min = INFINITY * glm::vec3(1.f, 1.f, 1.f);
    alignas(16) glm::vec3 _Max = -INFINITY * glm::vec3(1.f, 1.f, 1.f);
};

struct BVH_NodeGPU {
    AABB_GPU _BoundingBox;
    uint32_t _TriangleId;
    uint32_t _LeftChild;
    uint32_t _RightChild;
};

struct BVH_Params {
    template <class T>
    using Slots = std::vector<std::optional<T>>;
    static constexpr size_t kClusters = 2 * Triangle::MAX_NB_TRIANGLES - 1;
    size_t _NbTriangles = 0;
    std::vector<TriangleGPU> _UnsortedTriangles = std::vector<TriangleGPU>(Triangle::MAX_NB_TRIANGLES);
    std::vector<MeshModelGPU> _MeshesInTheScene = std::vector<MeshModelGPU>(Mesh::MAX_NB_MESHES);
    Slots<BVH_NodeGPU> _Clusters = Slots<BVH_NodeGPU>(kClusters);
    Slots<bool> _IsLeaf = Slots<bool>(kClusters);
    Slots<uint32_t> _Parent = Slots<uint32_t>(kClusters);
    Slots<uint32_t> _LeftChild = Slots<uint32_t>(kClusters);
    Slots<uint32_t> _RightChild = Slots<uint32_t>(kClusters);
    std::vector<uint32_t> _TriangleIndices = std::vector<uint32_t>(Triangle::MAX_NB_TRIANGLES, 0);
};

class BVH {
  public:
    BVH_Params _InternalStruct = {};
    BVH(uint32_t nbTriangles, const std::vector<TriangleGPU>& unsortedTriangles,
        const std::vector<MeshModelGPU>& meshesInTheScene);
};

}  // namespace cr
