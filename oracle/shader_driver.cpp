// Oracle (test infrastructure only): a C-ABI driver around the reference's
// own compute shader srcCommon/shaders/raytracer.glsl, compiled as C++.
//
// oracle/glsl_to_cpp.py rewrites the shader's declarations (layout, uniform,
// buffer blocks, inout, main) into oracle/_ref/raytracer_glsl.inc; the
// function bodies are the shader's own.  They compile here against the
// project-written GLSL shim (oracle/glsl_shim/glsl.hpp).  The recipe is
// oracle/Makefile (target "shader"); the library lands in oracle/_ref/ and is
// never shipped with the product.  There is no graphics stack on these
// machines, so this is the one way the shader's code runs at all.
//
// Entry points:
//   glsl_closest_hits  getClosestHitBVH (raytracer.glsl:246-295) per ray, root 0
//   glsl_all_hits      getAllHits (raytracer.glsl:149-157) per ray
//   glsl_frame         main (raytracer.glsl:299-331) for every texel of an
//                      image of (width / 16) x (height / 16) work groups
// Inputs use the library's record layouts (include/crt.h): TriangleGPU is the
// shader's Triangle byte for byte (its vec4s named _P0, _P2, _P1); node
// records are BVH_Node byte for byte; models are copied into the shader's
// 80-byte Model records (64 of them, identity past n_models, as
// Scene::getMeshModelToGPUData pads).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "crt.h"

namespace glsl_ref {
#include "glsl.hpp"
#include "raytracer_glsl.inc"
}  // namespace glsl_ref

namespace {

using namespace glsl_ref;

static_assert(sizeof(Triangle) == sizeof(crt_triangle), "Triangle record");
static_assert(sizeof(BVH_Node) == sizeof(crt_bvh_node), "BVH_Node record");
static_assert(sizeof(Model) == 80, "std430 Model record");
static_assert(sizeof(Material) == 16, "Material record");

std::vector<Model> g_models;

void bind(const crt_bvh_node* nodes, const crt_triangle* tris, uint32_t n_tris, const crt_mesh_model* models,
          uint32_t n_models, const crt_material* materials, uint32_t n_materials) {
    uBVH_Nodes = reinterpret_cast<BVH_Node*>(const_cast<crt_bvh_node*>(nodes));
    uTriangles = reinterpret_cast<Triangle*>(const_cast<crt_triangle*>(tris));
    g_models.assign(64, Model{});
    for (uint32_t m = 0; m < 64; ++m) {
        for (int c = 0; c < 4; ++c)
            g_models[m]._ModelMatrix.c[c] = vec4(c == 0 ? 1.f : 0.f, c == 1 ? 1.f : 0.f, c == 2 ? 1.f : 0.f,
                                                 c == 3 ? 1.f : 0.f);
        g_models[m]._MaterialId = 0;
        if (m < n_models) {
            for (int c = 0; c < 4; ++c)
                g_models[m]._ModelMatrix.c[c] = vec4(models[m].m[4 * c], models[m].m[4 * c + 1],
                                                     models[m].m[4 * c + 2], models[m].m[4 * c + 3]);
            g_models[m]._MaterialId = models[m].material_id;
        }
    }
    uModels = g_models.data();
    uMaterials = reinterpret_cast<Material*>(const_cast<crt_material*>(materials));
    uNbTriangles = n_tris;
    uNbModels = 64;
    uNbMaterials = n_materials;
}

Ray make_ray(const crt_ray& r) {
    Ray ray{};
    ray._Origin = vec4(r.o[0], r.o[1], r.o[2], 1.f);
    ray._Direction = vec4(r.d[0], r.d[1], r.d[2], 0.f);
    return ray;
}

crt_hit to_hit(const Hit& h) {
    crt_hit o{CRT_MISS, 0.f, 0.f, 0.f};
    if (h._DidHit != 0) {
        o.tri = h._TriangleId;
        o.t = h._Coords.w;
        o.u = h._Coords.x;
        o.v = h._Coords.y;
    }
    return o;
}

}  // namespace

extern "C" {

void glsl_closest_hits(const crt_bvh_node* nodes, const crt_triangle* tris, uint32_t n_tris,
                       const crt_mesh_model* models, uint32_t n_models, const crt_ray* rays, uint32_t n_rays,
                       crt_hit* hits) {
    bind(nodes, tris, n_tris, models, n_models, nullptr, 0);
    uDepthDisplayBVH = -1;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < static_cast<int64_t>(n_rays); ++i) {
        vec4 bvh_color(0.f, 0.f, 0.f, 0.f);
        hits[i] = to_hit(getClosestHitBVH(make_ray(rays[i]), 0u, bvh_color));
    }
}

void glsl_all_hits(const crt_triangle* tris, uint32_t n_tris, const crt_mesh_model* models, uint32_t n_models,
                   const crt_ray* rays, uint32_t n_rays, crt_hit* hits) {
    bind(nullptr, tris, n_tris, models, n_models, nullptr, 0);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < static_cast<int64_t>(n_rays); ++i) {
        Hit closest{};
        closest._DidHit = 0;
        getAllHits(make_ray(rays[i]), n_tris, closest);
        hits[i] = to_hit(closest);
    }
}

// cam: the crt_camera record (inverse view, eye, plane sizes) that getRay reads
// from uCamera.  flags: CRT_SHADE_WIREFRAME / CRT_SHADE_BVH.  rgba: width x
// height texels, row y at y * width.
void glsl_frame(const crt_camera* cam, uint32_t width, uint32_t height, const crt_bvh_node* nodes,
                const crt_triangle* tris, uint32_t n_tris, const crt_mesh_model* models, uint32_t n_models,
                const crt_material* materials, uint32_t n_materials, uint32_t flags, int bvh_depth, float* rgba) {
    bind(nodes, tris, n_tris, models, n_models, materials, n_materials);
    for (int c = 0; c < 4; ++c)
        uCamera._InvView.c[c] = vec4(cam->inv_view[4 * c], cam->inv_view[4 * c + 1], cam->inv_view[4 * c + 2],
                                     cam->inv_view[4 * c + 3]);
    uCamera._Eye = vec4(cam->eye[0], cam->eye[1], cam->eye[2], cam->eye[3]);
    uCamera._PlaneWidth = cam->plane_width;
    uCamera._PlaneHeight = cam->plane_height;
    uCamera._PlaneNear = cam->plane_near;
    uIsWireframeModeOn = (flags & CRT_SHADE_WIREFRAME) != 0;
    uIsBVHDisplayed = (flags & CRT_SHADE_BVH) != 0;
    uDepthDisplayBVH = bvh_depth;
    oImage.texels = reinterpret_cast<vec4*>(rgba);
    oImage.width = static_cast<int>(width);
    oImage.height = static_cast<int>(height);
    gl_NumWorkGroups = uvec3(width / gl_WorkGroupSize.x, height / gl_WorkGroupSize.y, 1u);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t y = 0; y < static_cast<int64_t>(height); ++y)
        for (uint32_t x = 0; x < width; ++x) {
            gl_GlobalInvocationID = uvec3(x, static_cast<uint32_t>(y), 0u);
            shader_main();
        }
}

}  // extern "C"
