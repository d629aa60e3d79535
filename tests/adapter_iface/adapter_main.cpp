// Test driver for adapter/bvh_cuda.cpp: runs the reference's build entry
// cr::BVH::BVH (bvh.hpp:89-91), which the adapter implements on the GPU, and
// flattens the resulting cluster graph the way the reference's renderer does
// before upload — Scene::getBVH_NodesToGPUData / recursiveTopDownTraversalBVH
// (srcOpenGL/scene/scene.cpp:189-208): pre-order from cluster 2N-2, left
// subtree first, children addressed by their position in the array, leaves
// with both children 0.  That file needs OpenGL, so its walk is restated here.
//
// Usage: adapter_main <in.bin> <out.bin>
//   in:  uint32 n_tris, uint32 n_buffer, uint32 n_models, then n_buffer
//        64-byte TriangleGPU records and n_models 68-byte MeshModelGPU records
//   out: the 2 n_tris - 1 48-byte BVH_NodeGPU records
#include <cstdio>
#include <cstring>
#include <vector>

#include "bvh.hpp"

namespace {

struct Frame {
    uint32_t id;
    uint32_t pos;
    int state;
};

// scene.cpp:189-201, iteratively: emit a cluster, then its left subtree, then
// its right subtree, patching the parent's child positions as they are known.
std::vector<cr::BVH_NodeGPU> flatten(const cr::BVH& bvh, uint32_t root) {
    const cr::BVH_Params& S = bvh._InternalStruct;
    std::vector<cr::BVH_NodeGPU> out;
    std::vector<Frame> st;
    auto emit = [&](uint32_t id) {  // the cluster's record as stored; internal nodes' children are patched below
        out.push_back(S._Clusters[id].value());
        return static_cast<uint32_t>(out.size() - 1);
    };
    st.push_back({root, emit(root), 0});
    while (!st.empty()) {
        Frame& f = st.back();
        if (S._IsLeaf[f.id].has_value() || f.state == 2) {  // `!_IsLeaf[id]` (an empty optional) marks internal nodes
            st.pop_back();
            continue;
        }
        const bool left = f.state == 0;
        f.state += 1;
        const uint32_t c = left ? S._LeftChild[f.id].value() : S._RightChild[f.id].value();
        const uint32_t parent = f.pos;
        const uint32_t p = emit(c);
        if (left) out[parent]._LeftChild = p; else out[parent]._RightChild = p;
        st.push_back({c, p, 0});
    }
    return out;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    uint32_t hdr[3];
    if (std::fread(hdr, 4, 3, f) != 3) return 4;
    const uint32_t n_tris = hdr[0], n_buffer = hdr[1], n_models = hdr[2];
    std::vector<cr::TriangleGPU> tris(n_buffer);
    std::vector<cr::MeshModelGPU> models(n_models);
    if (std::fread(tris.data(), sizeof(cr::TriangleGPU), n_buffer, f) != n_buffer) return 5;
    for (uint32_t m = 0; m < n_models; ++m) {
        unsigned char rec[68];
        if (std::fread(rec, 1, 68, f) != 68) return 6;
        std::memcpy(&models[m]._ModelMatrix, rec, 64);
        std::memcpy(&models[m]._MaterialId, rec + 64, 4);
    }
    std::fclose(f);
    cr::BVH bvh(n_tris, tris, models);
    const std::vector<cr::BVH_NodeGPU> nodes = flatten(bvh, 2 * n_tris - 2);
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 7;
    std::fwrite(nodes.data(), sizeof(cr::BVH_NodeGPU), nodes.size(), o);
    std::fclose(o);
    return 0;
}
