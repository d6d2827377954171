// Wavefront path tracer: the megakernel (render.cu) split into small kernels
// over path state kept in SoA device buffers (generate / extend / shade /
// shadow-connect).
//
// One path slot per pixel: a pixel's samples are sequential in its own
// XORShift128 stream (the reference's per-pixel stream), so a finished path
// immediately starts the pixel's next sample in the same slot ("path
// regeneration") and the pool stays full until pixels run out of samples.
// Per iteration:
//   extend : closest hit of every active path's ray;
//   shade  : emission with MIS at the hit (or environment on a miss), the
//            depth cap and Russian roulette, BSDF construction, next-event
//            estimation (writes a shadow-ray entry with its contribution),
//            BSDF sampling of the continuation ray; finished paths
//            regenerate (camera ray of the pixel's next sample);
//   shadow : closest hit of every shadow ray; adds the contribution when the
//            sampled light point is visible.
// Random numbers are drawn in the reference's order (camera 4, then per
// bounce NEE 3, BSDF 3, roulette 1) and each pixel's contributions are added
// in the reference's order (a bounce's NEE term lands in the shadow pass,
// before the next bounce's emission term), so results match the megakernel
// path for path.
#include <mutex>

#include "render_common.cuh"

CLR_DEFINE_STATUS_READER(render_wf)

namespace clr {

constexpr int kWfThreads = 128;

struct WfState {
    float4* org;     // xyz ray origin, w the path's light face (bits; shadow_visible)
    float4* dir;     // xyz ray direction, w dirPDF
    float4* alpha;   // xyz throughput, w initY
    uint4* misc;     // x depth, y sampledType, z samples done, w pixel
    float4* hit;     // x id bits, y t, z b1, w b2
    uint32_t* q[2];  // active path queues
    uint32_t* qs;    // the extended paths for shade: escaped first, hits from the end
    float4* sh;      // shadow entries: org (w shadow_light_word), dir (w path), contribution
    unsigned int* count;  // [0],[1] active counts, [2] shadow count, [3] escaped, [4] hits
};

__device__ __forceinline__ Rng load_rng(const uint32_t* rs, uint32_t p) {
    const uint4 s = reinterpret_cast<const uint4*>(rs)[p];
    Rng r;
    r.s[0] = s.x;
    r.s[1] = s.y;
    r.s[2] = s.z;
    r.s[3] = s.w;
    return r;
}
__device__ __forceinline__ void store_rng(uint32_t* rs, uint32_t p, const Rng& r) {
    reinterpret_cast<uint4*>(rs)[p] = make_uint4(r.s[0], r.s[1], r.s[2], r.s[3]);
}

// Warp-aggregated queue append.
__device__ __forceinline__ uint32_t queue_slot(unsigned int* count, bool want) {
    const unsigned int m = __ballot_sync(0xFFFFFFFFu, want);
    if (!m) return 0;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    unsigned int lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    return base + __popc(m & lt);
}

// Pixel p of the rendered rows is image pixel (p % width, row0 + p / width).
__device__ __forceinline__ void start_sample(const Camera& cam, WfState& S, uint32_t p, uint32_t width,
                                             uint32_t row0, Rng& rng, uint32_t done) {
    f3 org, dir, alpha;
    float dirPDF;
    camera_ray(cam, p % width, row0 + p / width, rng, org, dir, alpha, dirPDF);
    S.org[p] = make_float4(org.x, org.y, org.z, __uint_as_float(kNone32));
    S.dir[p] = make_float4(dir.x, dir.y, dir.z, dirPDF);
    S.alpha[p] = make_float4(alpha.x, alpha.y, alpha.z, luminance(alpha));
    S.misc[p] = make_uint4(0u, 0u, done, p);
}

__global__ void __launch_bounds__(kWfThreads) k_wf_init(DScene sc, WfState S, uint32_t npix, uint32_t width,
                                                        uint32_t row0, uint32_t* __restrict__ rand_states) {
    const Camera cam = load_camera(sc);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        Rng rng = load_rng(rand_states, p);
        start_sample(cam, S, p, width, row0, rng, 0u);
        store_rng(rand_states, p, rng);
        S.q[0][p] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S.count[0] = npix;
        S.count[1] = 0;
        S.count[2] = 0;
        S.count[3] = 0;
        S.count[4] = 0;
    }
}

template <bool kOrdered>
__global__ void __launch_bounds__(kWfThreads, 8) k_wf_extend(DScene sc, WfState S, int cur) {
    const uint32_t n = S.count[cur];
    uint2 stack[kStackSize];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = S.q[cur][i];
        const float4 o = S.org[p], d = S.dir[p];
        Hit h;
        if (intersect<kOrdered>(sc, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), h, stack))
            S.hit[p] = make_float4(__uint_as_float(h.id), h.t, h.b1, h.b2);
        else
            S.hit[p] = make_float4(__uint_as_float(kNone32), INFINITY, 0.f, 0.f);
    }
}

// The extended paths partitioned for shade: escaped paths (the environment
// branch) to the front of S.qs, paths that hit something to its end, so that
// shade's warps mostly run one of the two branches instead of both.  The
// order in which paths are shaded changes no path's result.  (A separate pass:
// votes inside the extend loop would hold every lane of a warp to the
// slowest ray's traversal.)
__global__ void __launch_bounds__(kWfThreads) k_wf_partition(WfState S, const uint32_t* __restrict__ q, int cur) {
    const uint32_t n = S.count[cur];
    const uint32_t n_round = (n + 31u) & ~31u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += gridDim.x * blockDim.x) {
        uint32_t p = 0;
        bool hit = false;
        if (i < n) {
            p = q[i];
            hit = __float_as_uint(S.hit[p].x) != kNone32;
        }
        const uint32_t ms = queue_slot(S.count + 3, i < n && !hit);
        const uint32_t hs = queue_slot(S.count + 4, hit);
        if (i < n) S.qs[hit ? n - 1u - hs : ms] = p;
    }
}

// kHit = false shades the escaped paths (S.qs[0, count[3])), kHit = true
// the paths that hit a surface (S.qs[count[3], n)): two kernels, each with
// only its branch's code.
template <bool kHit>
__global__ void __launch_bounds__(kWfThreads) k_wf_shade(DScene sc, WfState S, int cur, uint32_t width, uint32_t row0,
                                                         uint32_t* __restrict__ rand_states,
                                                         float4* __restrict__ pixels, uint32_t spp,
                                                         uint32_t max_depth) {
    const uint32_t n = S.count[cur], nm = S.count[3];
    const uint32_t lo = kHit ? nm : 0u, hi = kHit ? n : nm;
    const Camera cam = load_camera(sc);
    const uint32_t stride = gridDim.x * blockDim.x;
    // whole warps iterate together so the queue appends can use warp votes
    const uint32_t n_round = (hi - lo + 31u) & ~31u;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_round; j += stride) {
        const uint32_t i = lo + j;
        bool cont = false;      // path goes on to the next extend
        bool shadow = false;    // a shadow entry is written
        uint32_t p = 0;
        float4 sh0, sh1, sh2;
        if (i < hi) {
            p = S.qs[i];
            Rng rng = load_rng(rand_states, p);
            const float4 o4 = S.org[p], d4 = S.dir[p], a4 = S.alpha[p];
            uint4 m = S.misc[p];
            const float4 h4 = S.hit[p];
            f3 org = mk(o4.x, o4.y, o4.z), dir = mk(d4.x, d4.y, d4.z), alpha = mk(a4.x, a4.y, a4.z);
            float dirPDF = d4.w;
            const float initY = a4.w;
            uint32_t depth = m.x, sampledType = m.y;
            const float4 px = pixels[p];
            f3 pix = mk(px.x, px.y, px.z);
            bool ended = false;
            uint32_t light_face = __float_as_uint(o4.w);
            const uint32_t hid = __float_as_uint(h4.x);
            if (!kHit) {
                // escaped: environment emission (pathtracer.cl:183-196)
                LightPt lpos;
                lpos.atInfinity = true;
                lpos.uv = env_uv(dir);
                const f3 vout = -dir;
                EDF edf;
                edf_alloc(sc, kNone16, lpos, edf);
                float MISWeight = 1.0f;
                if ((sampledType & kTyNonSingular) && depth > 0) {
                    const float lightPDF = area_pdf(sc, lpos) * 1.0f / edf_abs_cos(edf, vout);
                    MISWeight = (dirPDF * dirPDF) / (lightPDF * lightPDF + dirPDF * dirPDF);
                }
                pix += MISWeight * alpha * edf_le(edf, vout);
                ended = true;
            } else {
                Hit h{hid, h4.y, h4.z, h4.w};
                SurfPt sp;
                surface_point(sc, org, dir, h, sp);
                const Face face = load_face(sc, sp.faceID);
                const f3 vout = -dir;
                LightPt lpos;
                lpos.faceID = light_face;
                if (face.light != kNone16) {
                    light_from_surface(sp, lpos);
                    EDF edf;
                    edf_alloc(sc, face.light, lpos, edf);
                    float MISWeight = 1.0f;
                    if (depth > 0 && (sampledType & kTyNonSingular)) {
                        const float d2 = (org.x - sp.p.x) * (org.x - sp.p.x) + (org.y - sp.p.y) * (org.y - sp.p.y) +
                                         (org.z - sp.p.z) * (org.z - sp.p.z);
                        const float lightPDF = area_pdf(sc, lpos) * d2 / edf_abs_cos(edf, vout);
                        MISWeight = (dirPDF * dirPDF) / (lightPDF * lightPDF + dirPDF * dirPDF);
                    }
                    pix += depth > 0 ? MISWeight * alpha * edf_le(edf, vout) : alpha * edf_le(edf, vout);
                }
                if (depth > 0) {
                    if (depth >= max_depth) ended = true;
                    else {
                        const float continueProb = fminf(luminance(alpha) * (1.0f / initY), 1.0f);
                        if (rng.uniform() < continueProb) {
                            alpha *= 1.0f / continueProb;
                            dirPDF *= continueProb;
                        } else {
                            ended = true;
                        }
                    }
                }
                if (!ended) {
                    BSDF bsdf;
                    bsdf_alloc(sc, face.mat, sp, bsdf);
                    if (bsdf_has_non_specular(bsdf)) {
                        const float uL = rng.uniform(), u0 = rng.uniform(), u1 = rng.uniform();
                        EDF edf;
                        float lightPDF;
                        sample_light(sc, uL, u0, u1, lpos, edf, lightPDF);
                        f3 vinL = lpos.p - sp.p;
                        float dist2 = dot(vinL, vinL);
                        vinL = vinL * (1.0f / sqrtf(dist2));
                        if (lpos.atInfinity) {
                            vinL = lpos.p;
                            dist2 = 1.0f;
                        }
                        const f3 sorg = sp.p + vinL * kEpsilon;
                        const f3 vinLrev = -vinL;
                        const float fsPDF = bsdf_pdf(bsdf, vout, vinL) * edf_abs_cos(edf, vinL) / dist2;
                        const float MISWeight = (lightPDF * lightPDF) / (lightPDF * lightPDF + fsPDF * fsPDF);
                        const f3 c = (MISWeight * edf_abs_cos(edf, vinL) * fabsf(dot(bsdf.n, vinL)) / dist2 / lightPDF) *
                                     (alpha * edf_le(edf, vinLrev) * bsdf_f(bsdf, vout, vinL));
                        sh0 = make_float4(sorg.x, sorg.y, sorg.z, __uint_as_float(shadow_light_word(lpos)));
                        sh1 = make_float4(vinL.x, vinL.y, vinL.z, __uint_as_float(p));
                        sh2 = make_float4(c.x, c.y, c.z, 0.f);
                        shadow = true;
                    }
                    const float uc = rng.uniform(), v0 = rng.uniform(), v1 = rng.uniform();
                    const f3 fs = bsdf_sample(bsdf, vout, uc, v0, v1, dir, dirPDF, sampledType);
                    if (zero_vec(fs) || dirPDF == 0.0f) {
                        ended = true;
                    } else {
                        alpha *= fs * (fabsf(dot(bsdf.n, dir)) / dirPDF);
                        org = sp.p + dir * kEpsilon;
                        ++depth;
                    }
                }
                light_face = lpos.faceID;
            }
            pixels[p] = make_float4(pix.x, pix.y, pix.z, px.w);
            if (ended) {
                const uint32_t done = m.z + 1;
                if (done < spp) {
                    start_sample(cam, S, p, width, row0, rng, done);
                    cont = true;
                } else {
                    S.misc[p] = make_uint4(depth, sampledType, done, p);
                }
            } else {
                S.org[p] = make_float4(org.x, org.y, org.z, __uint_as_float(light_face));
                S.dir[p] = make_float4(dir.x, dir.y, dir.z, dirPDF);
                S.alpha[p] = make_float4(alpha.x, alpha.y, alpha.z, initY);
                S.misc[p] = make_uint4(depth, sampledType, m.z, p);
                cont = true;
            }
            store_rng(rand_states, p, rng);
        }
        const uint32_t qs = queue_slot(S.count + (cur ^ 1), cont);
        if (cont) S.q[cur ^ 1][qs] = p;
        const uint32_t ss = queue_slot(S.count + 2, shadow);
        if (shadow) {
            S.sh[3u * ss] = sh0;
            S.sh[3u * ss + 1] = sh1;
            S.sh[3u * ss + 2] = sh2;
        }
    }
}

template <bool kOrdered>
__global__ void __launch_bounds__(kWfThreads, 8) k_wf_shadow(DScene sc, WfState S, float4* __restrict__ pixels) {
    const uint32_t n = S.count[2];
    uint2 stack[kStackSize];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = S.sh[3u * i], b = S.sh[3u * i + 1], c = S.sh[3u * i + 2];
        const uint32_t p = __float_as_uint(b.w);
        if (shadow_visible<kOrdered>(sc, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), __float_as_uint(a.w), stack)) {
            float4 px = pixels[p];
            px.x += c.x;
            px.y += c.y;
            px.z += c.z;
            pixels[p] = px;
        }
    }
}

// After the extend: the counts the shade kernels append to and the
// partition's counts.
__global__ void k_wf_reset(WfState S, int next) {
    S.count[next] = 0;
    S.count[2] = 0;
    S.count[3] = 0;
    S.count[4] = 0;
}

static size_t wf_layout(uint32_t npix, char* base, WfState* S) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) / 256 * 256;
        return o;
    };
    const size_t o_org = take(16ull * npix), o_dir = take(16ull * npix), o_alpha = take(16ull * npix),
                 o_misc = take(16ull * npix), o_hit = take(16ull * npix), o_q0 = take(4ull * npix),
                 o_q1 = take(4ull * npix), o_qs = take(4ull * npix), o_sh = take(48ull * npix), o_cnt = take(32);
    if (base && S) {
        S->org = reinterpret_cast<float4*>(base + o_org);
        S->dir = reinterpret_cast<float4*>(base + o_dir);
        S->alpha = reinterpret_cast<float4*>(base + o_alpha);
        S->misc = reinterpret_cast<uint4*>(base + o_misc);
        S->hit = reinterpret_cast<float4*>(base + o_hit);
        S->q[0] = reinterpret_cast<uint32_t*>(base + o_q0);
        S->q[1] = reinterpret_cast<uint32_t*>(base + o_q1);
        S->qs = reinterpret_cast<uint32_t*>(base + o_qs);
        S->sh = reinterpret_cast<float4*>(base + o_sh);
        S->count = reinterpret_cast<unsigned int*>(base + o_cnt);
    }
    return off;
}

// One block of kWfBlockIters iterations (the first of parity 0).
constexpr int kWfBlockIters = 8;

struct WfArgs {
    DScene sc;
    WfState S;
    uint32_t width, row0, spp, max_depth;
    uint32_t* rand_states;
    float4* px;
    bool ordered;
    unsigned int grid;        // shade kernels
    unsigned int grid_trace;  // extend and shadow: the resident blocks
};

static void wf_block(const WfArgs& a, cudaStream_t st) {
    for (int k = 0; k < kWfBlockIters; ++k) {
        const int cur = k & 1;
        if (a.ordered) k_wf_extend<true><<<a.grid_trace, kWfThreads, 0, st>>>(a.sc, a.S, cur);
        else k_wf_extend<false><<<a.grid_trace, kWfThreads, 0, st>>>(a.sc, a.S, cur);
        k_wf_reset<<<1, 1, 0, st>>>(a.S, cur ^ 1);
        k_wf_partition<<<a.grid, kWfThreads, 0, st>>>(a.S, a.S.q[cur], cur);
        k_wf_shade<false><<<a.grid, kWfThreads, 0, st>>>(a.sc, a.S, cur, a.width, a.row0, a.rand_states, a.px, a.spp,
                                                         a.max_depth);
        k_wf_shade<true><<<a.grid, kWfThreads, 0, st>>>(a.sc, a.S, cur, a.width, a.row0, a.rand_states, a.px, a.spp,
                                                        a.max_depth);
        if (a.ordered) k_wf_shadow<true><<<a.grid_trace, kWfThreads, 0, st>>>(a.sc, a.S, a.px);
        else k_wf_shadow<false><<<a.grid_trace, kWfThreads, 0, st>>>(a.sc, a.S, a.px);
    }
}

static bool same_args(const WfArgs& x, const WfArgs& y) {
    return same_scene(x.sc, y.sc) && x.S.org == y.S.org && x.S.count == y.S.count && x.S.qs == y.S.qs &&
           x.width == y.width && x.row0 == y.row0 && x.spp == y.spp && x.max_depth == y.max_depth &&
           x.rand_states == y.rand_states && x.px == y.px && x.ordered == y.ordered && x.grid == y.grid &&
           x.grid_trace == y.grid_trace;
}

thread_local BlockGraphCache<WfArgs> t_wf_graphs;

}  // namespace clr

using namespace clr;

extern "C" int clr_render_workspace_bytes(uint32_t width, uint32_t height, uint64_t* bytes) {
    if (!bytes) return clr_set_error(CLR_EINVAL, "clr_render_workspace_bytes: bytes is NULL");
    *bytes = wf_layout(width * height, nullptr, nullptr);
    return CLR_OK;
}

extern "C" int clr_render_wavefront_rows(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t row0,
                                         uint32_t rows, uint32_t* rand_states, float* pixels, uint32_t spp,
                                         uint32_t max_depth, uint32_t flags, void* workspace,
                                         uint64_t workspace_bytes, void* stream) {
    int rc = check_render_args(scene, rand_states, pixels);
    if (rc != CLR_OK) return rc;
    if (row0 > height || rows > height - row0)
        return clr_set_error(CLR_EINVAL, "clr_render_wavefront_rows: rows [%u, %u) outside the image's %u", row0,
                             row0 + rows, height);
    if (width == 0 || rows == 0 || spp == 0) return CLR_OK;
    const uint32_t npix = width * rows;
    if (!workspace || workspace_bytes < wf_layout(npix, nullptr, nullptr))
        return clr_set_error(CLR_ECAPACITY, "clr_render_wavefront: workspace of %llu bytes is smaller than %zu",
                             (unsigned long long)workspace_bytes, wf_layout(npix, nullptr, nullptr));
    if (reinterpret_cast<uintptr_t>(workspace) & 255u)
        return clr_set_error(CLR_EINVAL, "clr_render_wavefront: workspace must be 256-byte aligned");
    if (max_depth == 0) max_depth = 100;
    const DScene sc = make_dscene(scene);
    WfState S;
    wf_layout(npix, static_cast<char*>(workspace), &S);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool ordered = (flags & CLR_RENDER_ORDERED) != 0;
    const unsigned int grid = std::min(div_up(npix, kWfThreads), (unsigned int)clr_sm_count() * 16u);
    float4* px = reinterpret_cast<float4*>(pixels);
    k_wf_init<<<grid, kWfThreads, 0, st>>>(sc, S, npix, width, row0, rand_states);
    CLR_LAUNCH_CHECK("k_wf_init");
    const unsigned int work = div_up(npix, kWfThreads);
    const unsigned int grid_trace =
        ordered ? std::min(resident_grid(k_wf_extend<true>, kWfThreads, 0, work),
                           resident_grid(k_wf_shadow<true>, kWfThreads, 0, work))
                : std::min(resident_grid(k_wf_extend<false>, kWfThreads, 0, work),
                           resident_grid(k_wf_shadow<false>, kWfThreads, 0, work));
    const WfArgs a{sc, S, width, row0, spp, max_depth, rand_states, px, ordered, grid, grid_trace};
    cudaGraphExec_t exec = t_wf_graphs.get(a, wf_block, same_args);
    cudaGetLastError();  // a failed capture leaves no error behind: the kernels are launched directly
    // every iteration advances each unfinished pixel by one path vertex; a
    // block ends with the next iteration's queue count in count[0]
    const uint64_t max_iters = (uint64_t)spp * (max_depth + 1) + 1;
    for (uint64_t it = 0; it < max_iters; it += kWfBlockIters) {
        if (exec && cudaGraphLaunch(exec, st) != cudaSuccess) {
            cudaGetLastError();
            t_wf_graphs.drop();
            exec = nullptr;
        }
        if (!exec) wf_block(a, st);
        CLR_LAUNCH_CHECK("wavefront iterations");
        // stop once no path is left
        unsigned int left = 0;
        CLR_CUDA_TRY(cudaMemcpyAsync(&left, S.count, sizeof(left), cudaMemcpyDeviceToHost, st));
        CLR_CUDA_TRY(cudaStreamSynchronize(st));
        if (left == 0) break;
    }
    return CLR_OK;
}

extern "C" int clr_render_wavefront(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                                    float* pixels, uint32_t spp, uint32_t max_depth, uint32_t flags, void* workspace,
                                    uint64_t workspace_bytes, void* stream) {
    return clr_render_wavefront_rows(scene, width, height, 0u, height, rand_states, pixels, spp, max_depth, flags,
                                     workspace, workspace_bytes, stream);
}

// clr_render with CLR_RENDER_WAVEFRONT: the wavefront form on a workspace the
// library keeps per device until the process exits.  It grows to the largest
// image rendered (freed and reallocated once the renders queued on it are
// done), and every render that uses it waits on the GPU for the previous
// one, so calls on different streams stay correct (they take turns).
namespace {
constexpr int kKeptDevices = 64;
struct KeptWorkspace {
    void* ptr = nullptr;
    uint64_t bytes = 0;
    cudaEvent_t last_use = nullptr;
};
std::mutex g_kept_mutex;
KeptWorkspace g_kept[kKeptDevices];
}  // namespace

int clr_render_kept_wavefront(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                              float* pixels, uint32_t spp, uint32_t max_depth, uint32_t flags, void* stream) {
    int dev = 0;
    CLR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kKeptDevices) return clr_set_error(CLR_EINVAL, "clr_render: device %d out of range", dev);
    uint64_t need = 0;
    int rc = clr_render_workspace_bytes(width, height, &need);
    if (rc != CLR_OK) return rc;
    std::lock_guard<std::mutex> lock(g_kept_mutex);
    KeptWorkspace& w = g_kept[dev];
    if (!w.last_use) CLR_CUDA_TRY(cudaEventCreateWithFlags(&w.last_use, cudaEventDisableTiming));
    if (w.bytes < need) {
        CLR_CUDA_TRY(cudaEventSynchronize(w.last_use));  // no queued render still uses it
        if (w.ptr) cudaFree(w.ptr);
        w.ptr = nullptr;
        w.bytes = 0;
        if (cudaMalloc(&w.ptr, need) != cudaSuccess) {
            cudaGetLastError();
            w.ptr = nullptr;
            return clr_set_error(CLR_ENOMEM, "clr_render: cudaMalloc of a %llu-byte workspace failed",
                                 (unsigned long long)need);
        }
        w.bytes = need;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CLR_CUDA_TRY(cudaStreamWaitEvent(st, w.last_use, 0));
    rc = clr_render_wavefront(scene, width, height, rand_states, pixels, spp, max_depth, flags & ~CLR_RENDER_WAVEFRONT,
                              w.ptr, w.bytes, stream);
    if (rc != CLR_OK) return rc;
    CLR_CUDA_TRY(cudaEventRecord(w.last_use, st));
    return CLR_OK;
}
