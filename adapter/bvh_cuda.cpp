// Drop-in replacement for the reference's cr::BVH constructor
// (srcCommon/scene/geometry/bvh.hpp:89-91, bvh.cpp:11-24), backed by libcrt.
//
// Link this file instead of srcCommon/scene/geometry/bvh.cpp.  It compiles
// against the reference's own bvh.hpp, builds the BVH on the GPU with
// crt_build and fills BVH_Params (_Clusters, _IsLeaf, _LeftChild,
// _RightChild, _Parent, _TriangleIndices) so that the unchanged
// Scene::getBVH_NodesToGPUData (srcOpenGL/scene/scene.cpp:189-208), which
// starts from cluster 2N-2 and walks the tree left first, reproduces the node
// array crt_build returned, bit for bit.
//
// Cluster numbering: leaves keep the reference's ids 0..N-1 in sorted
// (Morton) order; internal nodes are numbered 2N-2 downward in DFS order, so
// the root is 2N-2 as Scene expects.  The reference numbers internal nodes in
// an OpenMP critical section (bvh.cpp:175-179), so its numbering is not
// reproducible either; only the tree and the flattened array are.
//
// The reference's fixed-size vectors (bvh.hpp:46-55) cap N at
// Triangle::MAX_NB_TRIANGLES; larger scenes call crt_build directly.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bvh.hpp"
#include "crt.h"

namespace {

crt_ctx* shared_context() {
    static crt_ctx* ctx = nullptr;
    if (!ctx && crt_create(&ctx, nullptr) != CRT_OK) {
        std::fprintf(stderr, "libcrt: %s\n", crt_last_error_string());
        std::exit(EXIT_FAILURE);  // the reference's ErrorHandler also exits on FATAL
    }
    return ctx;
}

void check(crt_status s) {
    if (s != CRT_OK) {
        std::fprintf(stderr, "libcrt: %s\n", crt_last_error_string());
        std::exit(EXIT_FAILURE);
    }
}

}  // namespace

namespace cr {

BVH::BVH(uint32_t nbTriangles, const std::vector<TriangleGPU>& unsortedTriangles,
         const std::vector<MeshModelGPU>& meshesInTheScene) {
    static_assert(sizeof(TriangleGPU) == sizeof(crt_triangle), "TriangleGPU layout");
    static_assert(sizeof(BVH_NodeGPU) == sizeof(crt_bvh_node), "BVH_NodeGPU layout");
    _InternalStruct._NbTriangles = nbTriangles;
    _InternalStruct._UnsortedTriangles = unsortedTriangles;
    _InternalStruct._MeshesInTheScene = meshesInTheScene;
    if (nbTriangles == 0 || nbTriangles > Triangle::MAX_NB_TRIANGLES) return;

    std::vector<crt_mesh_model> models(meshesInTheScene.size());
    for (size_t m = 0; m < meshesInTheScene.size() && m < 64; ++m) {
        const float* src = &meshesInTheScene[m]._ModelMatrix[0][0];
        for (int k = 0; k < 16; ++k) models[m].m[k] = src[k];
        models[m].material_id = meshesInTheScene[m]._MaterialId;
    }
    crt_ctx* ctx = shared_context();
    crt_bvh* bvh = nullptr;
    check(crt_build(ctx, reinterpret_cast<const crt_triangle*>(unsortedTriangles.data()),
                    static_cast<uint32_t>(unsortedTriangles.size()), nbTriangles, models.data(),
                    static_cast<uint32_t>(models.size() < 64 ? models.size() : 64), &bvh));
    const uint32_t n_nodes = 2 * nbTriangles - 1;
    std::vector<crt_bvh_node> nodes(n_nodes);
    std::vector<uint32_t> perm(nbTriangles);
    check(crt_bvh_copy_nodes(ctx, bvh, nodes.data()));
    check(crt_bvh_copy_perm(ctx, bvh, perm.data()));
    crt_bvh_free(bvh);

    // DFS position -> cluster id
    std::vector<uint32_t> id(n_nodes);
    uint32_t next_leaf = 0, next_internal = 2 * nbTriangles - 2;
    for (uint32_t p = 0; p < n_nodes; ++p) {
        const bool leaf = nodes[p].left == 0 && nodes[p].right == 0;
        id[p] = leaf ? next_leaf++ : next_internal--;
    }
    BVH_Params& S = _InternalStruct;
    for (uint32_t i = 0; i < nbTriangles; ++i) S._TriangleIndices[i] = perm[i];
    for (uint32_t p = 0; p < n_nodes; ++p) {
        BVH_NodeGPU c{};
        c._BoundingBox._Min = glm::vec3(nodes[p].mn[0], nodes[p].mn[1], nodes[p].mn[2]);
        c._BoundingBox._Max = glm::vec3(nodes[p].mx[0], nodes[p].mx[1], nodes[p].mx[2]);
        c._TriangleId = nodes[p].tri;
        const uint32_t me = id[p];
        S._Clusters[me] = c;
        if (nodes[p].left == 0 && nodes[p].right == 0) {
            S._IsLeaf[me] = true;
        } else {
            const uint32_t l = id[nodes[p].left], r = id[nodes[p].right];
            S._LeftChild[me] = l;
            S._RightChild[me] = r;
            S._Parent[l] = me;
            S._Parent[r] = me;
        }
    }
}

}  // namespace cr
