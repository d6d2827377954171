// Unidirectional path tracer on sm_103a (megakernel form).
//
// Replaces the reference's `pathtracing` kernel (OpenCL/pathtracer.cl:25-271):
// per pixel a thin-lens camera sample, next-event estimation with the power
// heuristic, BSDF sampling over the material's layered BxDFs, implicit-hit
// MIS, Russian roulette on throughput luminance, and the environment light on
// escape.  It reads the reference's scene blobs unchanged (materials,
// textures, other resources, 56-byte faces, 8-byte light infos) and traces
// rays with this project's LBVH (exact reference-order traversal, or
// nearer-child-first with CLR_RENDER_ORDERED).
//
// Differences from the reference, each deliberate:
//   * one NDRange over the whole image, so the RNG state of pixel (x, y) is
//     4*(W*y + x) (the reference indexes it tile-locally, pathtracer.cl:52-54,
//     so all tiles share one 64x64 block of streams);
//   * the depth cap is a parameter (the reference hard-codes depth > 99,
//     pathtracer.cl:166; max_depth = 100 reproduces it);
//   * the shadow test is the reference's, light face carried along the path
//     (shadow_visible), with the values it leaves unset defined: the path's
//     light face starts as no face, and a missed shadow ray never matches
//     (the reference compares an unset hit record, pathtracer.cl:120-122);
//   * samples-per-pixel loop inside the kernel (the reference launches once
//     per sample); each pixel's contributions are added in the same order.
//
// The kernel traces from three sites (camera ray, shadow ray, bounce); one
// out-of-line copy of each search instead of three inlined copies keeps the
// kernel's instruction footprint down, which this instruction-fetch-bound
// kernel turns into speed (13.2 -> 20.1 Msamples/s on the Cornell box).
#define CLR_TRAVERSAL_OUTLINED
#include "render_common.cuh"

CLR_DEFINE_STATUS_READER(render)

namespace clr {

// ----------------------------------------------------------- path tracer

// With kCount, cnt[0] counts the closest-hit rays, cnt[1] the shadow rays,
// cnt[2] the nodes loaded and cnt[3] the triangles tested by both, and cnt[4]
// the surface hits shaded (the visiting counts behind the path's bytes).
// kAlpha: the scene has cutout faces (CLR_SCENE_ALPHA), fixed per launch.
template <bool kOrdered, bool kCount, bool kAlpha>
__device__ void trace_path(const DScene& sc, const Camera& cam, uint32_t gx, uint32_t gy, Rng& rng, f3& pix,
                           uint32_t max_depth, uint2* stack, uint32_t* cnt = nullptr) {
    auto closest = [&](f3 o, f3 d, Hit& hh) {
        const bool hit = intersect_impl<kOrdered, kCount, kAlpha ? 1 : 0>(sc, o, d, hh, stack, kCount ? cnt + 2 : nullptr);
        if (kCount) {
            ++cnt[0];
            cnt[4] += hit ? 1u : 0u;
        }
        return hit;
    };
    f3 org, dir, alpha;
    float dirPDF;
    camera_ray(cam, gx, gy, rng, org, dir, alpha, dirPDF);
    const float initY = luminance(alpha);

    uint32_t depth = 0;
    SurfPt sp;
    LightPt lpos;
    lpos.faceID = kNone32;
    bool traceContinue = true;
    f3 vout;
    uint32_t sampledType = 0;
    float lightPDF = 0.f, MISWeight;
    EDF edf;
    BSDF bsdf;
    Hit h;
    if (closest(org, dir, h)) {
        surface_point(sc, org, dir, h, sp);
        Face face = load_face(sc, sp.faceID);
        vout = -dir;
        if (face.light != kNone16) {
            light_from_surface(sp, lpos);
            edf_alloc(sc, face.light, lpos, edf);
            pix += alpha * edf_le(edf, vout);
        }
        for (;;) {
            bsdf_alloc(sc, face.mat, sp, bsdf);
            float dist2;
            if (bsdf_has_non_specular(bsdf)) {
                const float uL = rng.uniform(), u0 = rng.uniform(), u1 = rng.uniform();
                sample_light(sc, uL, u0, u1, lpos, edf, lightPDF);
                f3 vinL = lpos.p - sp.p;
                dist2 = dot(vinL, vinL);
                vinL = vinL * (1.0f / sqrtf(dist2));
                if (lpos.atInfinity) {
                    vinL = lpos.p;
                    dist2 = 1.0f;
                }
                const f3 sorg = sp.p + vinL * kEpsilon;
                if (kCount) ++cnt[1];
                if (shadow_visible<kOrdered, kCount, kAlpha ? 1 : 0>(sc, sorg, vinL, shadow_light_word(lpos), stack,
                                                                     kCount ? cnt + 2 : nullptr)) {
                    const f3 vinLrev = -vinL;
                    const float fsPDF = bsdf_pdf(bsdf, vout, vinL) * edf_abs_cos(edf, vinL) / dist2;
                    MISWeight = (lightPDF * lightPDF) / (lightPDF * lightPDF + fsPDF * fsPDF);
                    pix += (MISWeight * edf_abs_cos(edf, vinL) * fabsf(dot(bsdf.n, vinL)) / dist2 / lightPDF) *
                           (alpha * edf_le(edf, vinLrev) * bsdf_f(bsdf, vout, vinL));
                }
            }
            traceContinue = true;
            const float uc = rng.uniform(), v0 = rng.uniform(), v1 = rng.uniform();
            const f3 fs = bsdf_sample(bsdf, vout, uc, v0, v1, dir, dirPDF, sampledType);
            if (zero_vec(fs) || dirPDF == 0.0f) {
                traceContinue = false;
                break;
            }
            alpha *= fs * (fabsf(dot(bsdf.n, dir)) / dirPDF);
            org = sp.p + dir * kEpsilon;
            ++depth;
            if (!closest(org, dir, h)) break;
            surface_point(sc, org, dir, h, sp);
            face = load_face(sc, sp.faceID);
            vout = -dir;
            if (face.light != kNone16) {
                light_from_surface(sp, lpos);
                edf_alloc(sc, face.light, lpos, edf);
                MISWeight = 1.0f;
                if (sampledType & kTyNonSingular) {
                    const f3 dd = org - sp.p;
                    const float d2 = (org.x - sp.p.x) * (org.x - sp.p.x) + (org.y - sp.p.y) * (org.y - sp.p.y) +
                                     (org.z - sp.p.z) * (org.z - sp.p.z);
                    (void)dd;
                    lightPDF = area_pdf(sc, lpos) * d2 / edf_abs_cos(edf, vout);
                    MISWeight = (dirPDF * dirPDF) / (lightPDF * lightPDF + dirPDF * dirPDF);
                }
                pix += MISWeight * alpha * edf_le(edf, vout);
            }
            if (depth >= max_depth) {
                traceContinue = false;
                break;
            }
            const float continueProb = fminf(luminance(alpha) * (1.0f / initY), 1.0f);
            if (rng.uniform() < continueProb) {
                alpha *= 1.0f / continueProb;
                dirPDF *= continueProb;
            } else {
                traceContinue = false;
                break;
            }
        }
    }
    if (traceContinue) {
        vout = -dir;
        lpos.atInfinity = true;
        lpos.uv = env_uv(dir);
        edf_alloc(sc, kNone16, lpos, edf);
        MISWeight = 1.0f;
        if ((sampledType & kTyNonSingular) && depth > 0) {
            lightPDF = area_pdf(sc, lpos) * 1.0f / edf_abs_cos(edf, vout);
            MISWeight = (dirPDF * dirPDF) / (lightPDF * lightPDF + dirPDF * dirPDF);
        }
        pix += MISWeight * alpha * edf_le(edf, vout);
    }
}

template <bool kOrdered, bool kCount, bool kAlpha>
__global__ void __launch_bounds__(128) k_render(DScene sc, uint32_t width, uint32_t height,
                                                uint32_t* __restrict__ rand_states, float4* __restrict__ pixels,
                                                uint32_t spp, uint32_t max_depth,
                                                unsigned long long* __restrict__ counts = nullptr) {
    const uint32_t x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (x >= width || y >= height) return;
    const uint32_t idx = y * width + x;
    Rng rng;
    const uint4 s = reinterpret_cast<const uint4*>(rand_states)[idx];
    rng.s[0] = s.x;
    rng.s[1] = s.y;
    rng.s[2] = s.z;
    rng.s[3] = s.w;
    const float4 p = pixels[idx];
    f3 pix = mk(p.x, p.y, p.z);
    const Camera cam = load_camera(sc);
    uint2 stack[kStackSize];
    uint32_t cnt[5] = {0, 0, 0, 0, 0};
    for (uint32_t i = 0; i < spp; ++i)
        trace_path<kOrdered, kCount, kAlpha>(sc, cam, x, y, rng, pix, max_depth, stack, cnt);
    pixels[idx] = make_float4(pix.x, pix.y, pix.z, p.w);
    reinterpret_cast<uint4*>(rand_states)[idx] = make_uint4(rng.s[0], rng.s[1], rng.s[2], rng.s[3]);
    if (kCount)
        for (int k = 0; k < 5; ++k) atomicAdd(counts + k, (unsigned long long)cnt[k]);
}

}  // namespace clr

using namespace clr;

// k_render over the image, instantiated for the traversal order and for
// whether the scene has cutout faces.
template <bool kCount>
static void launch_render(const DScene& sc, uint32_t width, uint32_t height, uint32_t* rand_states, float* pixels,
                          uint32_t spp, uint32_t max_depth, uint32_t flags, unsigned long long* counts,
                          cudaStream_t st) {
    const dim3 grid(div_up(width, 16), div_up(height, 8));
    float4* px = reinterpret_cast<float4*>(pixels);
    const bool ordered = (flags & CLR_RENDER_ORDERED) != 0;
    if (ordered && sc.alpha)
        k_render<true, kCount, true><<<grid, 128, 0, st>>>(sc, width, height, rand_states, px, spp, max_depth, counts);
    else if (ordered)
        k_render<true, kCount, false><<<grid, 128, 0, st>>>(sc, width, height, rand_states, px, spp, max_depth, counts);
    else if (sc.alpha)
        k_render<false, kCount, true><<<grid, 128, 0, st>>>(sc, width, height, rand_states, px, spp, max_depth, counts);
    else
        k_render<false, kCount, false><<<grid, 128, 0, st>>>(sc, width, height, rand_states, px, spp, max_depth, counts);
}

// The wavefront form on the library's own workspace (render_wf.cu).
int clr_render_kept_wavefront(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                              float* pixels, uint32_t spp, uint32_t max_depth, uint32_t flags, void* stream);

extern "C" int clr_render(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                          float* pixels, uint32_t spp, uint32_t max_depth, uint32_t flags, void* stream) {
    int rc = check_render_args(scene, rand_states, pixels);
    if (rc != CLR_OK) return rc;
    if (width == 0 || height == 0 || spp == 0) return CLR_OK;
    if (flags & CLR_RENDER_WAVEFRONT)
        return clr_render_kept_wavefront(scene, width, height, rand_states, pixels, spp, max_depth, flags, stream);
    if (max_depth == 0) max_depth = 100;
    launch_render<false>(make_dscene(scene), width, height, rand_states, pixels, spp, max_depth, flags, nullptr,
                         static_cast<cudaStream_t>(stream));
    CLR_LAUNCH_CHECK("k_render");
    return CLR_OK;
}

extern "C" int clr_render_counted(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                                  float* pixels, uint32_t spp, uint32_t max_depth, uint32_t flags,
                                  unsigned long long* counts, void* stream) {
    int rc = check_render_args(scene, rand_states, pixels);
    if (rc != CLR_OK) return rc;
    if (!counts) return clr_set_error(CLR_EINVAL, "clr_render_counted: counts is NULL");
    if (flags & CLR_RENDER_WAVEFRONT)
        return clr_set_error(CLR_EINVAL, "clr_render_counted: counts are taken by the megakernel form only");
    if (width == 0 || height == 0 || spp == 0) return CLR_OK;
    if (max_depth == 0) max_depth = 100;
    launch_render<true>(make_dscene(scene), width, height, rand_states, pixels, spp, max_depth, flags, counts,
                        static_cast<cudaStream_t>(stream));
    CLR_LAUNCH_CHECK("k_render");
    return CLR_OK;
}
