/*
 * C entry points around the reference's own CPU code, compiled in place from
 * the reference checkout (OpenCL_PathTracer/Equivalent/sim_*.hpp and
 * OpenCL_PathTracer/BVH.hpp) with the stand-in headers in oracle/ref_stubs.
 *
 * TEST INFRASTRUCTURE ONLY: it is used to pin the oracle restatement
 * (oracle/lbvh_oracle.c) against the reference itself and to generate the
 * golden fixtures under tests/golden.  It is built only where the reference
 * sources are present (oracle/build_oracle.py), into oracle/_ref/.
 *
 * Compiled twice: with -D__USE_LBVH (LBVH traversal + path tracer) and
 * without (the reference's CPU midpoint BVH and its traversal), because the
 * reference selects between the two with that macro.
 */
#include <cstdint>
#include <cstring>
#include <vector>

#ifndef CLR_REF_PIPED_PATHTRACER  // else its text was piped ahead of this file
#include "sim_pathtracer.hpp"
#endif
#ifdef __USE_LBVH
#include "sim_bvh_visualizer.hpp"
#endif
#ifndef __USE_LBVH
#include "BVH.hpp"
#endif

namespace {
sim::Scene make_scene(const float* verts, const float* normals, const float* tangents, const float* uvs,
                      const uint8_t* faces, const uint8_t* lights, const uint8_t* materials,
                      const uint8_t* textures, const uint8_t* others, const uint8_t* nodes0,
                      const uint8_t* nodes1) {
    sim::Scene s;
    std::memset(&s, 0, sizeof(s));
    s.vertices = (sim::point3*)verts;
    s.normals = (sim::vector3*)normals;
    s.tangents = (sim::vector3*)tangents;
    s.uvs = (sim::float2*)uvs;
    s.faces = (sim::Face*)faces;
    s.lights = (sim::LightInfo*)lights;
    s.materialsData = (sim::uchar*)materials;
    s.texturesData = (sim::uchar*)textures;
    s.otherResourcesData = (sim::uchar*)others;
#ifdef __USE_LBVH
    s.LBVHInternalNodes = (sim::LBVHInternalNode*)nodes0;
    s.LBVHLeafNodes = (sim::LBVHLeafNode*)nodes1;
#else
    (void)nodes1;
    s.BVHNodes = (sim::BVHNode*)nodes0;
#endif
    return s;
}

/* rays: 8 floats {ox,oy,oz,tmax,dx,dy,dz,-}; the reference's traversal always
 * starts at t = INFINITY, so tmax is ignored here. */
void trace(const sim::Scene& scene, const float* rays, uint32_t nrays, uint32_t* hit_id, float* hit_t) {
    for (uint32_t r = 0; r < nrays; ++r) {
        const float* R = rays + 8u * r;
        sim::point3 org(R[0], R[1], R[2]);
        sim::vector3 dir(R[4], R[5], R[6]);
        sim::SurfacePoint sp;
        bool hit = sim::rayIntersection(&scene, &org, &dir, &sp);
        if (!hit) {
            hit_id[r] = 0xFFFFFFFFu;
            hit_t[r] = INFINITY;
            continue;
        }
        /* the reference returns the hit point, not t: re-run its own
         * triangle test on the winning face to read t back */
        float t = INFINITY;
        sim::Intersection is;
        sim::rayTriangleIntersection(&scene, &org, &dir, (sim::ushort)sp.faceID, &t, &is);
        hit_id[r] = sp.faceID;
        hit_t[r] = t;
    }
}
}  // namespace

extern "C" {

#ifdef __USE_LBVH
/* sim::rayIntersection over reference-layout LBVH nodes (48 B each). */
int ref_trace_closest_lbvh(const float* verts, const uint8_t* faces, const uint8_t* inodes,
                           const uint8_t* lnodes, const float* rays, uint32_t nrays, uint32_t* hit_id,
                           float* hit_t) {
    sim::Scene scene = make_scene(verts, nullptr, nullptr, nullptr, faces, nullptr, nullptr, nullptr,
                                  nullptr, inodes, lnodes);
    trace(scene, rays, nrays, hit_id, hit_t);
    return 0;
}

/* sim::pathtracing for rows [y0, y1) of a width x height image, spp passes.
 * The whole image is one NDRange (offset 0), so the reference's RNG state
 * index 4*(gsize0*tileY + tileX) is the per-pixel index. */
int ref_render(const float* verts, const float* normals, const float* tangents, const float* uvs,
               const uint8_t* faces, const uint8_t* lights, const uint8_t* materials,
               const uint8_t* textures, const uint8_t* others, const uint8_t* inodes,
               const uint8_t* lnodes, uint32_t* rand_states, float* pixels, uint32_t width,
               uint32_t height, uint32_t y0, uint32_t y1, uint32_t spp) {
    sim::global_sizes[0] = width;
    sim::global_sizes[1] = height;
    sim::global_offsets[0] = 0;
    sim::global_offsets[1] = 0;
    for (uint32_t s = 0; s < spp; ++s)
        for (uint32_t y = y0; y < y1; ++y)
            for (uint32_t x = 0; x < width; ++x) {
                sim::global_ids[0] = x;
                sim::global_ids[1] = y;
                sim::pathtracing((sim::float3*)verts, (sim::float3*)normals, (sim::float3*)tangents,
                                 (sim::float2*)uvs, (sim::uchar*)faces, (sim::uint*)lights,
                                 (sim::uchar*)materials, (sim::uchar*)textures, (sim::uchar*)others,
                                 (sim::uchar*)inodes, (sim::uchar*)lnodes, rand_states,
                                 (sim::float3*)pixels);
            }
    return 0;
}

#ifdef CLR_REF_PIPED_PATHTRACER
/* The depth cap of the piped renderer: a path stops after max_depth bounces
 * (the reference's constant, ray.depth > 99, is max_depth = 100). */
int ref_set_max_depth(uint32_t max_depth) {
    clr_ref_depth_cap = (int)max_depth - 1;
    return 0;
}
#endif

/* sim::bvh_visualizer over a width x height image (one NDRange, offset 0). */
int ref_bvh_visualizer(const float* verts, const float* normals, const float* tangents, const float* uvs,
                       const uint8_t* faces, const uint8_t* lights, const uint8_t* materials,
                       const uint8_t* textures, const uint8_t* others, const uint8_t* inodes,
                       const uint8_t* lnodes, uint32_t* rand_states, float* pixels, uint32_t width,
                       uint32_t height) {
    sim::global_sizes[0] = width;
    sim::global_sizes[1] = height;
    sim::global_offsets[0] = 0;
    sim::global_offsets[1] = 0;
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x) {
            sim::global_ids[0] = x;
            sim::global_ids[1] = y;
            sim::bvh_visualizer((sim::float3*)verts, (sim::float3*)normals, (sim::float3*)tangents,
                                (sim::float2*)uvs, (sim::uchar*)faces, (sim::uint*)lights, (sim::uchar*)materials,
                                (sim::uchar*)textures, (sim::uchar*)others, (sim::uchar*)inodes,
                                (sim::uchar*)lnodes, rand_states, (sim::float3*)pixels);
        }
    return 0;
}
#else
/* The reference's CPU build: Scene::build's leaf loop (Scene.cpp:328-334) and
 * BVH::build (BVH.hpp:172-175).  nodes_out holds 2n-1 48-byte BVHNodes;
 * returns the node count. */
int64_t ref_midbvh_build(const float* verts, const uint32_t* tri, uint32_t n, uint8_t* nodes_out) {
    BVH bvh;
    for (uint32_t i = 0; i < n; ++i) {
        const cl_float3* v = (const cl_float3*)verts;
        BBox bb{v[tri[3 * i + 0]]};
        bb.unionP(v[tri[3 * i + 1]]);
        bb.unionP(v[tri[3 * i + 2]]);
        bvh.addLeaf(bb);
    }
    bvh.build();
    std::memcpy(nodes_out, bvh.nodes.data(), bvh.nodes.size() * sizeof(BVHNode));
    return (int64_t)bvh.nodes.size();
}

/* sim::rayIntersection over the midpoint BVH (bvh_traversal.cl:256-285). */
int ref_trace_closest_mid(const float* verts, const uint8_t* faces, const uint8_t* nodes, const float* rays,
                          uint32_t nrays, uint32_t* hit_id, float* hit_t) {
    sim::Scene scene = make_scene(verts, nullptr, nullptr, nullptr, faces, nullptr, nullptr, nullptr,
                                  nullptr, nodes, nullptr);
    trace(scene, rays, nrays, hit_id, hit_t);
    return 0;
}
#endif
}
