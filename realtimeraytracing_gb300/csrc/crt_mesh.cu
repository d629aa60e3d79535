// Mesh input: Wavefront OBJ text to an indexed triangle mesh (host), and an
// indexed mesh to TriangleGPU records (GPU).
//
// Reference: Mesh::load (srcCommon/scene/geometry/mesh.cpp:186-263) reads the
// file with tinyobjloader and makes one Triangle(v0, v1, v2, meshId) per face,
// shape after shape, in file order, each vertex as vec4(p, 1)
// (triangle.cpp:18-25); Scene::getTriangleToGPUData (srcOpenGL/scene/
// scene.cpp:26-40) concatenates the meshes' triangles into the TriangleGPU
// buffer.  Here the OBJ subset the reference's assets use is read directly:
//   v x y z [w]        a vertex (w ignored); numbers read as double, then
//                      rounded to float, as tinyobjloader stores real_t
//   f i j k ...        a face; each corner "v", "v/vt", "v//vn" or
//                      "v/vt/vn"; indices 1-based, negative ones relative
//                      to the vertices read so far
// Other statements (vn, vt, g, o, s, usemtl, mtllib, comments) carry nothing
// the path uses and are skipped.  Faces with more than three corners become
// the fan (0, i, i+1); tinyobjloader, whose version the reference does not
// pin, triangulates them itself and may split them differently (the
// reference's teapot and bunny are all triangles).
#include <charconv>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>
#include <string>
#include <system_error>

#include "crt_build.cuh"
#include "crt_common.cuh"

namespace crt {

namespace {

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Next whitespace-separated token of [p, end) starting at *p, or false.
bool next_token(const char*& p, const char* end, const char*& tb, const char*& te) {
    while (p < end && is_space(*p)) ++p;
    if (p >= end) return false;
    tb = p;
    while (p < end && !is_space(*p)) ++p;
    te = p;
    return true;
}

bool parse_float(const char* b, const char* e, float& out) {
    double v = 0.0;
    if (b < e && *b == '+') ++b;  // from_chars takes no leading '+'
    const auto r = std::from_chars(b, e, v);
    if (r.ec != std::errc() || r.ptr != e) return false;
    out = static_cast<float>(v);
    return true;
}

// Vertex index of a face corner ("v", "v/vt", "v//vn", "v/vt/vn"), made
// 0-based against n_seen vertices read so far.
bool parse_corner(const char* b, const char* e, uint64_t n_seen, uint32_t& out) {
    const char* slash = static_cast<const char*>(std::memchr(b, '/', static_cast<size_t>(e - b)));
    const char* ve = slash ? slash : e;
    long long v = 0;
    if (b < ve && *b == '+') ++b;
    const auto r = std::from_chars(b, ve, v);
    if (r.ec != std::errc() || r.ptr != ve || v == 0) return false;
    const long long idx = v > 0 ? v - 1 : static_cast<long long>(n_seen) + v;
    if (idx < 0 || idx > 0xFFFFFFFELL) return false;
    out = static_cast<uint32_t>(idx);
    return true;
}

}  // namespace

bool obj_parse(const char* text, size_t len, float* vertices, uint64_t vert_cap, uint32_t* indices,
               uint64_t tri_cap, uint64_t* n_vertices, uint64_t* n_triangles, std::string* error) {
    uint64_t nv = 0, nt = 0, line_no = 0;
    const char* p = text;
    const char* end = text + len;
    auto bad = [&](const char* what) {
        if (error) *error = "OBJ line " + std::to_string(line_no) + ": " + what;
        return false;
    };
    while (p < end) {
        ++line_no;
        const char* eol = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(end - p)));
        const char* le = eol ? eol : end;
        const char* q = p;
        p = eol ? eol + 1 : end;
        const char *tb, *te;
        if (!next_token(q, le, tb, te)) continue;
        const size_t tl = static_cast<size_t>(te - tb);
        if (tl == 1 && *tb == 'v') {
            float xyz[3];
            for (int k = 0; k < 3; ++k) {
                const char *nb, *ne;
                if (!next_token(q, le, nb, ne) || !parse_float(nb, ne, xyz[k])) return bad("bad vertex");
            }
            if (vertices && nv < vert_cap) std::memcpy(vertices + 3 * nv, xyz, sizeof(xyz));
            ++nv;
        } else if (tl == 1 && *tb == 'f') {
            uint32_t first = 0, prev = 0;
            int corners = 0;
            const char *cb, *ce;
            while (next_token(q, le, cb, ce)) {
                uint32_t v;
                if (!parse_corner(cb, ce, nv, v)) return bad("bad face corner");
                if (v >= nv) return bad("face corner past the vertices read so far");
                if (corners == 0) {
                    first = v;
                } else if (corners >= 2) {  // fan (first, prev, v)
                    if (indices && nt < tri_cap) {
                        indices[3 * nt + 0] = first;
                        indices[3 * nt + 1] = prev;
                        indices[3 * nt + 2] = v;
                    }
                    ++nt;
                }
                prev = v;
                ++corners;
            }
            if (corners < 3) return bad("face with fewer than 3 corners");
        }
    }
    *n_vertices = nv;
    *n_triangles = nt;
    return true;
}

// TriangleGPU record of triangle i: its three vertices as (x, y, z, 1) and
// the model id (the Triangle constructor, triangle.cpp:18-25).
__global__ void __launch_bounds__(256) indexed_kernel(const float* __restrict__ vertices, uint32_t n_vertices,
                                                      const uint32_t* __restrict__ indices, uint32_t n_triangles,
                                                      uint32_t model_id, crt_triangle* __restrict__ out,
                                                      uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_triangles) return;
    const uint32_t a = __ldg(indices + 3 * static_cast<size_t>(i)), b = __ldg(indices + 3 * static_cast<size_t>(i) + 1),
                   c = __ldg(indices + 3 * static_cast<size_t>(i) + 2);
    float4* o = reinterpret_cast<float4*>(out + i);
    if (a >= n_vertices || b >= n_vertices || c >= n_vertices) {
        raise_error(err, kDevBadIndex);
        const float4 z = make_float4(0.f, 0.f, 0.f, 1.f);
        o[0] = z; o[1] = z; o[2] = z;
        reinterpret_cast<uint4*>(o)[3] = make_uint4(model_id, 0u, 0u, 0u);
        return;
    }
    const float* pa = vertices + 3 * static_cast<size_t>(a);
    const float* pb = vertices + 3 * static_cast<size_t>(b);
    const float* pc = vertices + 3 * static_cast<size_t>(c);
    o[0] = make_float4(__ldg(pa), __ldg(pa + 1), __ldg(pa + 2), 1.f);
    o[1] = make_float4(__ldg(pb), __ldg(pb + 1), __ldg(pb + 2), 1.f);
    o[2] = make_float4(__ldg(pc), __ldg(pc + 1), __ldg(pc + 2), 1.f);
    reinterpret_cast<uint4*>(o)[3] = make_uint4(model_id, 0u, 0u, 0u);
}

void launch_indexed(const float* vertices, uint32_t n_vertices, const uint32_t* indices, uint32_t n_triangles,
                    uint32_t model_id, crt_triangle* out, uint32_t* err, cudaStream_t s) {
    if (n_triangles == 0) return;
    indexed_kernel<<<(n_triangles + 255) / 256, 256, 0, s>>>(vertices, n_vertices, indices, n_triangles, model_id, out,
                                                             err);
}

}  // namespace crt
