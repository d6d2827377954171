// BVH visualiser: the reference's `bvh_visualizer` kernel
// (OpenCL/bvh_visualizer.cl:25-84).  One camera ray per pixel through the
// lens centre and the pixel centre; the closest-hit search in the reference's
// visiting order counts the boxes it accepts (internal and leaf,
// rayIntersectionVis, bvh_traversal.cl:217-254); the pixel gains the hit
// material's base colour (getBaseColor_fs, reflection.cl:730-774; times the
// camera's sample_We value, which is one, camera.cl:95-115) and 0.025 per
// accepted box.  The per-pixel counts
// also go to `visits` (optional): the traversal work each ray costs.
#include "render_common.cuh"

CLR_DEFINE_STATUS_READER(bvh_vis)

namespace clr {

// getBaseColor_fx (reflection.cl:730-762): R / Rs / Rd of a component, black
// for specular transmission.
__device__ __forceinline__ f3 base_color(const BSDF& f) {
    f3 c = mk(0.f, 0.f, 0.f);
    for (int k = 0; k < f.num; ++k) {
        const BxDF b = load_bx(f, f.off[k]);
        if (b.id != kBxSpecT) c += b.c0;  // c0 is Rd for AshikhminD
    }
    return c;
}

__global__ void __launch_bounds__(128) k_bvh_vis(DScene sc, uint32_t width, uint32_t height,
                                                 float4* __restrict__ pixels, uint32_t* __restrict__ visits) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= width * height) return;
    const uint32_t x = p % width, y = p / width;
    const Camera cam = load_camera(sc);
    f3 org, dir, alpha;  // alpha (|cos| / pdf, the path tracer's weight) is not used here
    float dirPDF;
    camera_ray_at(cam, x, y, 0.5f, 0.5f, 0.5f, 0.5f, org, dir, alpha, dirPDF);
    uint2 stack[kStackSize];
    uint32_t cnt[2] = {0u, 0u};
    Hit h;
    float4 px = pixels[p];
    const bool hit = intersect_impl<false, true>(sc, org, dir, h, stack, cnt);
    const uint32_t boxes = cnt[0] + cnt[1];
    if (hit) {
        SurfPt sp;
        surface_point(sc, org, dir, h, sp);
        const Face face = load_face(sc, sp.faceID);
        BSDF bsdf;
        bsdf_alloc(sc, face.mat, sp, bsdf);
        const f3 c = base_color(bsdf);
        px.x += c.x;
        px.y += c.y;
        px.z += c.z;
    }
    const float v = boxes * 0.025f;
    px.x += v;
    px.y += v;
    px.z += v;
    pixels[p] = px;
    if (visits) visits[p] = boxes;
}

// Closest hit of rays {ox,oy,oz,tmax,dx,dy,dz,0} in the reference's order
// with t unbounded, counting per ray the internal boxes and the leaf boxes
// the search accepts (counts[2r], counts[2r+1]).
__global__ void __launch_bounds__(128) k_trace_counted(DScene sc, const float4* __restrict__ rays, uint32_t n,
                                                       uint32_t* __restrict__ hit_id, uint32_t* __restrict__ counts) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float4 a = rays[2u * r], b = rays[2u * r + 1];
    uint2 stack[kStackSize];
    uint32_t cnt[2] = {0u, 0u};
    Hit h;
    const bool hit = intersect_impl<false, true>(sc, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), h, stack, cnt);
    if (hit_id) hit_id[r] = hit ? h.id : kNone32;
    counts[2u * r] = cnt[0];
    counts[2u * r + 1] = cnt[1];
}

}  // namespace clr

using namespace clr;

extern "C" int clr_trace_closest_counted(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                         uint32_t* counts, void* stream) {
    if (!bvh || !counts || (num_rays && !rays))
        return clr_set_error(CLR_EINVAL, "clr_trace_closest_counted: NULL argument");
    if (reinterpret_cast<uintptr_t>(rays) & 15u)
        return clr_set_error(CLR_EINVAL, "clr_trace_closest_counted: rays must be 16-byte aligned");
    if (num_rays == 0) return CLR_OK;
    DScene sc{};
    sc.nodes = static_cast<const float4*>(bvh->nodes);
    sc.tris = static_cast<const float4*>(bvh->tris);
    sc.root_box = bvh->root_box;
    sc.num_tris = bvh->num_tris;
    k_trace_counted<<<div_up(num_rays, 128u), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        sc, reinterpret_cast<const float4*>(rays), num_rays, hit_id, counts);
    CLR_LAUNCH_CHECK("k_trace_counted");
    return CLR_OK;
}

extern "C" int clr_bvh_visualize(const clr_scene* scene, uint32_t width, uint32_t height, float* pixels,
                                 uint32_t* visits, void* stream) {
    if (!scene || !scene->bvh || !pixels || !scene->vertices || !scene->faces || !scene->materials ||
        !scene->textures || !scene->others)
        return clr_set_error(CLR_EINVAL, "clr_bvh_visualize: NULL argument");
    if (reinterpret_cast<uintptr_t>(pixels) & 15u)
        return clr_set_error(CLR_EINVAL, "clr_bvh_visualize: pixels must be 16-byte aligned");
    if (width == 0 || height == 0) return CLR_OK;
    const DScene sc = make_dscene(scene);
    const uint64_t n = (uint64_t)width * height;
    k_bvh_vis<<<(unsigned)div_up(n, (uint64_t)128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        sc, width, height, reinterpret_cast<float4*>(pixels), visits);
    CLR_LAUNCH_CHECK("k_bvh_vis");
    return CLR_OK;
}
