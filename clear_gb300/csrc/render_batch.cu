// Batched wavefront path tracer: many scenes (each with its own blobs, BVH,
// camera and resolution) rendered by one wavefront over a fixed pool of path
// slots.
//
// Pixels of all scenes are numbered globally (scene s owns [pix0_s,
// pix0_{s+1})).  A slot renders every sample of one pixel in sequence, in the
// pixel's own XORShift128 stream (as render_wf.cu does), then takes the next
// unrendered pixel from a global counter, so the pool stays full until the
// last pixels; the pool size (the queue capacity) is a tuning parameter.
// Every pixel sees exactly the operations of a per-scene wavefront render, so
// each scene's image is bit-identical to clr_render_wavefront of that scene.
//
// The frame loop (extend / shade / shadow per iteration) can run as one CUDA
// graph: an init kernel followed by a conditional WHILE node whose body holds
// two iterations and a kernel that keeps the loop going while paths remain
// (bounded by an iteration cap), so a whole batch is one graph launch with no
// host synchronisation.
#include <algorithm>
#include <new>
#include <vector>

#include "render_common.cuh"

CLR_DEFINE_STATUS_READER(render_batch)

namespace clr {

constexpr int kBtShadeThreads = 128;
constexpr int kBtTraceMaxThreads = 256;

struct BtScene {
    DScene sc;
    uint32_t width;
    uint32_t pix0;
};

struct BtState {
    float4* org;     // xyz ray origin, w the path's light face (bits; shadow_visible)
    float4* dir;     // xyz direction, w dirPDF
    float4* alpha;   // xyz throughput, w initY
    uint4* misc;     // x depth, y sampledType, z samples done, w scene
    float4* hit;     // x id bits, y t, z b1, w b2
    uint32_t* pix;   // global pixel of the slot
    uint32_t* q[2];  // active slots
    float4* sh;      // shadow entries: org (w shadow_light_word), dir (w pixel), contribution (w scene)
    unsigned int* count;  // [0],[1] active slots, [2] shadow entries, [3] next pixel, [4] iterations run
};

struct BtArgs {
    const BtScene* scenes;
    const uint32_t* pix0;  // num_scenes + 1
    uint32_t num_scenes;
    uint32_t total_pix;
    uint32_t slots;
    uint32_t* rand_states;
    float4* pixels;
    uint32_t spp;
    uint32_t max_depth;
};

__device__ __forceinline__ Rng bt_rng(const uint32_t* rs, uint32_t g) {
    const uint4 s = reinterpret_cast<const uint4*>(rs)[g];
    Rng r;
    r.s[0] = s.x;
    r.s[1] = s.y;
    r.s[2] = s.z;
    r.s[3] = s.w;
    return r;
}
__device__ __forceinline__ void bt_store_rng(uint32_t* rs, uint32_t g, const Rng& r) {
    reinterpret_cast<uint4*>(rs)[g] = make_uint4(r.s[0], r.s[1], r.s[2], r.s[3]);
}

// Warp-aggregated counter increment: lanes with `want` get consecutive values.
__device__ __forceinline__ uint32_t bt_take(unsigned int* ctr, bool want) {
    const unsigned int m = __ballot_sync(0xFFFFFFFFu, want);
    if (!m) return 0;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(ctr, (unsigned int)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    unsigned int lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    return base + __popc(m & lt);
}

// The scene owning global pixel g.
__device__ __forceinline__ uint32_t bt_scene_of(const uint32_t* __restrict__ pix0, uint32_t nscenes, uint32_t g) {
    uint32_t lo = 0, hi = nscenes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(pix0 + mid) <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Camera ray of sample `done` of global pixel g in slot p.
__device__ __forceinline__ void bt_start(const BtArgs& A, const BtState& S, uint32_t p, uint32_t g, uint32_t s,
                                         Rng& rng, uint32_t done) {
    const BtScene& bs = A.scenes[s];
    const Camera cam = load_camera(bs.sc);
    const uint32_t lp = g - bs.pix0;
    f3 org, dir, alpha;
    float dirPDF;
    camera_ray(cam, lp % bs.width, lp / bs.width, rng, org, dir, alpha, dirPDF);
    S.org[p] = make_float4(org.x, org.y, org.z, __uint_as_float(kNone32));
    S.dir[p] = make_float4(dir.x, dir.y, dir.z, dirPDF);
    S.alpha[p] = make_float4(alpha.x, alpha.y, alpha.z, luminance(alpha));
    S.misc[p] = make_uint4(0u, 0u, done, s);
    S.pix[p] = g;
}

__global__ void __launch_bounds__(kBtTraceMaxThreads) k_bt_init(BtArgs A, BtState S) {
    const uint32_t live = min(A.slots, A.total_pix);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < live; p += gridDim.x * blockDim.x) {
        const uint32_t s = bt_scene_of(A.pix0, A.num_scenes, p);
        Rng rng = bt_rng(A.rand_states, p);
        bt_start(A, S, p, p, s, rng, 0u);
        bt_store_rng(A.rand_states, p, rng);
        S.q[0][p] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S.count[0] = live;
        S.count[1] = 0;
        S.count[2] = 0;
        S.count[3] = live;
        S.count[4] = 0;
    }
}

template <bool kOrdered>
__global__ void __launch_bounds__(kBtTraceMaxThreads, 4) k_bt_extend(BtArgs A, BtState S, int cur) {
    const uint32_t n = S.count[cur];
    uint2 stack[kStackSize];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = S.q[cur][i];
        const float4 o = S.org[p], d = S.dir[p];
        const DScene& sc = A.scenes[S.misc[p].w].sc;
        Hit h;
        if (intersect<kOrdered>(sc, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), h, stack))
            S.hit[p] = make_float4(__uint_as_float(h.id), h.t, h.b1, h.b2);
        else
            S.hit[p] = make_float4(__uint_as_float(kNone32), INFINITY, 0.f, 0.f);
    }
}

// One path vertex per active slot (render_wf.cu k_wf_shade, pathtracer.cl:
// 128-262), then sample / pixel succession.
__global__ void __launch_bounds__(kBtShadeThreads) k_bt_shade(BtArgs A, BtState S, int cur) {
    const uint32_t n = S.count[cur];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_round = (n + 31u) & ~31u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        bool cont = false, shadow = false, need_pixel = false;
        uint32_t p = 0;
        float4 sh0, sh1, sh2;
        if (i < n) {
            p = S.q[cur][i];
            const uint32_t g = S.pix[p];
            const uint4 m = S.misc[p];
            const uint32_t s = m.w;
            const DScene& sc = A.scenes[s].sc;
            Rng rng = bt_rng(A.rand_states, g);
            const float4 o4 = S.org[p], d4 = S.dir[p], a4 = S.alpha[p], h4 = S.hit[p];
            f3 org = mk(o4.x, o4.y, o4.z), dir = mk(d4.x, d4.y, d4.z), alpha = mk(a4.x, a4.y, a4.z);
            float dirPDF = d4.w;
            const float initY = a4.w;
            uint32_t depth = m.x, sampledType = m.y;
            const float4 px = A.pixels[g];
            f3 pix = mk(px.x, px.y, px.z);
            bool ended = false;
            uint32_t light_face = __float_as_uint(o4.w);
            const uint32_t hid = __float_as_uint(h4.x);
            if (hid == kNone32) {
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
                    if (depth >= A.max_depth) ended = true;
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
                        sh1 = make_float4(vinL.x, vinL.y, vinL.z, __uint_as_float(g));
                        sh2 = make_float4(c.x, c.y, c.z, __uint_as_float(s));
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
            A.pixels[g] = make_float4(pix.x, pix.y, pix.z, px.w);
            if (ended) {
                const uint32_t done = m.z + 1;
                if (done < A.spp) {
                    bt_start(A, S, p, g, s, rng, done);
                    cont = true;
                } else {
                    need_pixel = true;
                }
            } else {
                S.org[p] = make_float4(org.x, org.y, org.z, __uint_as_float(light_face));
                S.dir[p] = make_float4(dir.x, dir.y, dir.z, dirPDF);
                S.alpha[p] = make_float4(alpha.x, alpha.y, alpha.z, initY);
                S.misc[p] = make_uint4(depth, sampledType, m.z, s);
                cont = true;
            }
            bt_store_rng(A.rand_states, g, rng);
        }
        // a slot whose pixel is done takes the next pixel of the batch
        const uint32_t ng = bt_take(S.count + 3, need_pixel);
        if (need_pixel && ng < A.total_pix) {
            const uint32_t ns = bt_scene_of(A.pix0, A.num_scenes, ng);
            Rng rng = bt_rng(A.rand_states, ng);
            bt_start(A, S, p, ng, ns, rng, 0u);
            bt_store_rng(A.rand_states, ng, rng);
            cont = true;
        }
        const unsigned int m = __ballot_sync(0xFFFFFFFFu, cont);
        if (m) {
            const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(S.count + (cur ^ 1), (unsigned int)__popc(m));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            unsigned int lt;
            asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
            if (cont) S.q[cur ^ 1][base + __popc(m & lt)] = p;
        }
        const unsigned int ms = __ballot_sync(0xFFFFFFFFu, shadow);
        if (ms) {
            const int lane = threadIdx.x & 31, leader = __ffs(ms) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(S.count + 2, (unsigned int)__popc(ms));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            unsigned int lt;
            asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
            if (shadow) {
                const uint32_t ss = base + __popc(ms & lt);
                S.sh[3u * ss] = sh0;
                S.sh[3u * ss + 1] = sh1;
                S.sh[3u * ss + 2] = sh2;
            }
        }
    }
}

template <bool kOrdered>
__global__ void __launch_bounds__(kBtTraceMaxThreads, 4) k_bt_shadow(BtArgs A, BtState S) {
    const uint32_t n = S.count[2];
    uint2 stack[kStackSize];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = S.sh[3u * i], b = S.sh[3u * i + 1], c = S.sh[3u * i + 2];
        const uint32_t g = __float_as_uint(b.w);
        const DScene& sc = A.scenes[__float_as_uint(c.w)].sc;
        if (shadow_visible<kOrdered>(sc, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), __float_as_uint(a.w), stack)) {
            float4 px = A.pixels[g];
            px.x += c.x;
            px.y += c.y;
            px.z += c.z;
            A.pixels[g] = px;
        }
    }
}

__global__ void k_bt_reset(BtState S, int next) {
    S.count[next] = 0;
    S.count[2] = 0;
    S.count[4] += 1;
}

// Keeps the graph's WHILE loop running while paths remain (and below the
// iteration cap: a corrupt count cannot loop forever).
__global__ void k_bt_continue(BtState S, cudaGraphConditionalHandle h, unsigned int max_iters) {
    const bool more = S.count[0] > 0 && S.count[4] < max_iters;
    if (S.count[0] > 0 && !more) clr_raise(CLR_DEVERR_QUEUE);
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

// After a frame loop run without the graph: paths still in flight when the
// iteration bound ran out are reported, as the graph's loop does.
__global__ void k_bt_check_done(BtState S, int next) {
    if (S.count[next] > 0) clr_raise(CLR_DEVERR_QUEUE);
}

static size_t bt_layout(uint32_t slots, char* base, BtState* S) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) / 256 * 256;
        return o;
    };
    const size_t n = slots;
    const size_t o_org = take(16 * n), o_dir = take(16 * n), o_alpha = take(16 * n), o_misc = take(16 * n),
                 o_hit = take(16 * n), o_pix = take(4 * n), o_q0 = take(4 * n), o_q1 = take(4 * n),
                 o_sh = take(48 * n), o_cnt = take(32);
    if (base && S) {
        S->org = reinterpret_cast<float4*>(base + o_org);
        S->dir = reinterpret_cast<float4*>(base + o_dir);
        S->alpha = reinterpret_cast<float4*>(base + o_alpha);
        S->misc = reinterpret_cast<uint4*>(base + o_misc);
        S->hit = reinterpret_cast<float4*>(base + o_hit);
        S->pix = reinterpret_cast<uint32_t*>(base + o_pix);
        S->q[0] = reinterpret_cast<uint32_t*>(base + o_q0);
        S->q[1] = reinterpret_cast<uint32_t*>(base + o_q1);
        S->sh = reinterpret_cast<float4*>(base + o_sh);
        S->count = reinterpret_cast<unsigned int*>(base + o_cnt);
    }
    return off;
}

}  // namespace clr

using namespace clr;

// Batch handle: the scene table on the device, the slot pool and the graph of
// the last configuration it was captured for.
struct clr_batch {
    uint32_t num_scenes = 0;
    uint32_t total_pix = 0;
    clr_batch_config cfg{};
    void* dev = nullptr;  // scene table + pixel offsets
    BtScene* scenes = nullptr;
    uint32_t* pix0 = nullptr;
    void* pool = nullptr;
    size_t pool_bytes = 0;
    uint32_t slots = 0;
    BtState S{};
    // captured graph and the arguments it was captured with
    cudaGraphExec_t exec = nullptr;
    cudaStream_t capture = nullptr;  // private stream the graph is captured on
    uint32_t* g_rs = nullptr;
    float* g_px = nullptr;
    uint32_t g_spp = 0, g_depth = 0, g_flags = 0;
    uint64_t g_cap = 0;  // iteration bound the graph was captured with
    clr_batch_config g_cfg{};
};

static void batch_drop_graph(clr_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
}

static void batch_free(clr_batch* b) {
    batch_drop_graph(b);
    if (b->capture) cudaStreamDestroy(b->capture);
    if (b->pool) cudaFree(b->pool);
    if (b->dev) cudaFree(b->dev);
    delete b;
}

static int batch_configure(clr_batch* b, const clr_batch_config* cfg) {
    clr_batch_config c = cfg ? *cfg : clr_batch_config{};
    if (c.trace_block == 0) c.trace_block = 128;
    if (c.shade_block == 0) c.shade_block = kBtShadeThreads;
    if (c.trace_block % 32 || c.trace_block > kBtTraceMaxThreads || c.shade_block % 32 ||
        c.shade_block > kBtShadeThreads)
        return clr_set_error(CLR_EINVAL, "clr_batch: trace_block %u / shade_block %u (multiples of 32, <= %d / %d)",
                             c.trace_block, c.shade_block, kBtTraceMaxThreads, kBtShadeThreads);
    const uint32_t slots = c.pool_slots == 0 || c.pool_slots > b->total_pix ? b->total_pix : c.pool_slots;
    c.pool_slots = slots;
    const size_t need = bt_layout(slots, nullptr, nullptr);
    if (!b->pool || need > b->pool_bytes) {
        if (b->pool) cudaFree(b->pool);
        b->pool = nullptr;
        b->pool_bytes = 0;
        if (cudaMalloc(&b->pool, need) != cudaSuccess) {
            cudaGetLastError();
            b->pool = nullptr;
            return clr_set_error(CLR_ENOMEM, "clr_batch: cudaMalloc(%zu) for %u path slots failed", need, slots);
        }
        b->pool_bytes = need;
    }
    bt_layout(slots, static_cast<char*>(b->pool), &b->S);
    b->slots = slots;
    b->cfg = c;
    batch_drop_graph(b);
    return CLR_OK;
}

extern "C" int clr_batch_create(const clr_scene* scenes, const uint32_t* widths, const uint32_t* heights,
                                uint32_t num_scenes, const clr_batch_config* cfg, clr_batch** out) {
    if (!scenes || !widths || !heights || !out || num_scenes == 0)
        return clr_set_error(CLR_EINVAL, "clr_batch_create: NULL argument or no scene");
    std::vector<BtScene> tab(num_scenes);
    std::vector<uint32_t> pix0(num_scenes + 1);
    uint64_t total = 0;
    for (uint32_t s = 0; s < num_scenes; ++s) {
        if (!scenes[s].bvh || widths[s] == 0 || heights[s] == 0)
            return clr_set_error(CLR_EINVAL, "clr_batch_create: scene %u has no BVH or an empty image", s);
        tab[s].sc = make_dscene(scenes + s);
        tab[s].width = widths[s];
        tab[s].pix0 = (uint32_t)total;
        pix0[s] = (uint32_t)total;
        total += (uint64_t)widths[s] * heights[s];
    }
    if (total >= (1ull << 31)) return clr_set_error(CLR_EINVAL, "clr_batch_create: %llu pixels exceed 2^31",
                                                    (unsigned long long)total);
    pix0[num_scenes] = (uint32_t)total;
    clr_batch* b = new (std::nothrow) clr_batch{};
    if (!b) return clr_set_error(CLR_ENOMEM, "clr_batch_create: host allocation failed");
    b->num_scenes = num_scenes;
    b->total_pix = (uint32_t)total;
    const size_t tab_bytes = (sizeof(BtScene) * num_scenes + 255) / 256 * 256;
    if (cudaMalloc(&b->dev, tab_bytes + 4ull * (num_scenes + 1)) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return clr_set_error(CLR_ENOMEM, "clr_batch_create: cudaMalloc for the scene table failed");
    }
    b->scenes = static_cast<BtScene*>(b->dev);
    b->pix0 = reinterpret_cast<uint32_t*>(static_cast<char*>(b->dev) + tab_bytes);
    if (cudaMemcpy(b->scenes, tab.data(), sizeof(BtScene) * num_scenes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->pix0, pix0.data(), 4ull * (num_scenes + 1), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(b->dev);
        delete b;
        return clr_set_error(CLR_ECUDA, "clr_batch_create: upload of the scene table failed");
    }
    int rc = batch_configure(b, cfg);
    if (rc != CLR_OK) {
        cudaFree(b->dev);
        delete b;
        return rc;
    }
    *out = b;
    return CLR_OK;
}

extern "C" int clr_batch_destroy(clr_batch* b) {
    if (b) batch_free(b);
    return CLR_OK;
}

extern "C" int clr_batch_set_config(clr_batch* b, const clr_batch_config* cfg) {
    if (!b) return clr_set_error(CLR_EINVAL, "clr_batch_set_config: NULL handle");
    return batch_configure(b, cfg);
}

extern "C" int clr_batch_get_config(const clr_batch* b, clr_batch_config* cfg) {
    if (!b || !cfg) return clr_set_error(CLR_EINVAL, "clr_batch_get_config: NULL argument");
    *cfg = b->cfg;
    return CLR_OK;
}

extern "C" int clr_batch_pixels(const clr_batch* b, uint32_t* total) {
    if (!b || !total) return clr_set_error(CLR_EINVAL, "clr_batch_pixels: NULL argument");
    *total = b->total_pix;
    return CLR_OK;
}

static unsigned int bt_grid(uint32_t work, uint32_t block) {
    return std::max(1u, std::min(div_up(work, block), (unsigned int)clr_sm_count() * (2048u / block)));
}

// One iteration's kernels (parity cur).
static void bt_iteration(const clr_batch* b, const BtArgs& A, int cur, bool ordered, cudaStream_t st) {
    const uint32_t tb = b->cfg.trace_block, sb = b->cfg.shade_block;
    const unsigned int gt = bt_grid(b->slots, tb), gs = bt_grid(b->slots, sb);
    if (ordered) k_bt_extend<true><<<gt, tb, 0, st>>>(A, b->S, cur);
    else k_bt_extend<false><<<gt, tb, 0, st>>>(A, b->S, cur);
    k_bt_reset<<<1, 1, 0, st>>>(b->S, cur ^ 1);
    k_bt_shade<<<gs, sb, 0, st>>>(A, b->S, cur);
    if (ordered) k_bt_shadow<true><<<gt, tb, 0, st>>>(A, b->S);
    else k_bt_shadow<false><<<gt, tb, 0, st>>>(A, b->S);
}

// A lower iteration bound set through clr_debug_set_wait_limits (0 = none), so
// that a test can make the frame loop's bound run out.
static uint32_t g_iteration_cap = 0;

int clr_batch_set_iteration_cap(uint32_t cap) {
    g_iteration_cap = cap;
    return CLR_OK;
}

static uint64_t bt_max_iters(const clr_batch* b, uint32_t spp, uint32_t max_depth) {
    // every iteration advances every busy slot by one vertex; a pixel takes at
    // most spp * (max_depth + 1) vertices and one succession step.  While
    // pixels remain all slots are busy, so that phase lasts at most
    // ceil(pixels / slots) pixel-lengths; the last pixels then finish within
    // one more pixel-length.
    const uint64_t per_pixel = (uint64_t)spp * (max_depth + 1) + 1;
    const uint64_t per_slot = (b->total_pix + b->slots - 1) / b->slots;
    const uint64_t bound = (per_slot + 1) * per_pixel + 4;
    return (g_iteration_cap && g_iteration_cap < bound) ? g_iteration_cap : bound;
}

// Builds the frame graph: init kernel -> WHILE (two iterations + continue
// test).  Captured on the handle's own stream (the caller's may be the legacy
// stream, which cannot capture); launched on the caller's.
static int bt_capture(clr_batch* b, const BtArgs& A, bool ordered, unsigned int max_iters) {
    if (!b->capture) CLR_CUDA_TRY(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
    cudaStream_t st = b->capture;
    cudaGraph_t g = nullptr;
    CLR_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
    cudaGraphNode_t init_node = nullptr;
    if (e == cudaSuccess) {
        cudaGraphNodeParams kp = {};
        kp.type = cudaGraphNodeTypeKernel;
        BtArgs a = A;
        BtState s = b->S;
        void* args[] = {&a, &s};
        kp.kernel.func = reinterpret_cast<void*>(k_bt_init);
        kp.kernel.gridDim = dim3(bt_grid(b->slots, b->cfg.trace_block));
        kp.kernel.blockDim = dim3(b->cfg.trace_block);
        kp.kernel.sharedMemBytes = 0;
        kp.kernel.kernelParams = args;
        e = cudaGraphAddNode(&init_node, g, nullptr, nullptr, 0, &kp);
    }
    cudaGraphNode_t cond = nullptr;
    cudaGraphNodeParams cp = {};
    if (e == cudaSuccess) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        e = cudaGraphAddNode(&cond, g, &init_node, nullptr, 1, &cp);
    }
    if (e == cudaSuccess) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            bt_iteration(b, A, 0, ordered, st);
            bt_iteration(b, A, 1, ordered, st);
            k_bt_continue<<<1, 1, 0, st>>>(b->S, h, max_iters);
            cudaGraph_t out = nullptr;
            e = cudaStreamEndCapture(st, &out);
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b->exec = nullptr;
        return clr_set_error(CLR_ECUDA, "clr_batch_render: graph construction failed: %s", cudaGetErrorString(e));
    }
    return CLR_OK;
}

extern "C" int clr_batch_render(clr_batch* b, uint32_t* rand_states, float* pixels, uint32_t spp, uint32_t max_depth,
                                uint32_t flags, void* stream) {
    if (!b || !rand_states || !pixels) return clr_set_error(CLR_EINVAL, "clr_batch_render: NULL argument");
    if ((reinterpret_cast<uintptr_t>(rand_states) | reinterpret_cast<uintptr_t>(pixels)) & 15u)
        return clr_set_error(CLR_EINVAL, "clr_batch_render: rand_states and pixels must be 16-byte aligned");
    if (spp == 0) return CLR_OK;
    if (max_depth == 0) max_depth = 100;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    BtArgs A{b->scenes, b->pix0, b->num_scenes, b->total_pix, b->slots, rand_states,
             reinterpret_cast<float4*>(pixels), spp, max_depth};
    const bool ordered = (flags & CLR_RENDER_ORDERED) != 0;
    const uint64_t cap = bt_max_iters(b, spp, max_depth);
    if (flags & CLR_BATCH_GRAPH) {
        if (cap >= 0xFFFFFFFFull) return clr_set_error(CLR_EINVAL, "clr_batch_render: iteration bound too large");
        const bool same = b->exec && b->g_rs == rand_states && b->g_px == pixels && b->g_spp == spp && b->g_cap == cap &&
                          b->g_depth == max_depth && b->g_flags == flags && b->g_cfg.trace_block == b->cfg.trace_block &&
                          b->g_cfg.shade_block == b->cfg.shade_block && b->g_cfg.pool_slots == b->cfg.pool_slots;
        if (!same) {
            batch_drop_graph(b);
            int rc = bt_capture(b, A, ordered, (unsigned int)cap);
            if (rc != CLR_OK) return rc;
            b->g_rs = rand_states;
            b->g_px = pixels;
            b->g_spp = spp;
            b->g_cap = cap;
            b->g_depth = max_depth;
            b->g_flags = flags;
            b->g_cfg = b->cfg;
        }
        CLR_CUDA_TRY(cudaGraphLaunch(b->exec, st));
        return CLR_OK;
    }
    k_bt_init<<<bt_grid(b->slots, b->cfg.trace_block), b->cfg.trace_block, 0, st>>>(A, b->S);
    CLR_LAUNCH_CHECK("k_bt_init");
    for (uint64_t it = 0; it < cap; ++it) {
        const int cur = (int)(it & 1);
        bt_iteration(b, A, cur, ordered, st);
        CLR_LAUNCH_CHECK("batched iteration");
        if ((it & 7) == 7) {
            unsigned int left = 0;
            CLR_CUDA_TRY(cudaMemcpyAsync(&left, b->S.count + (cur ^ 1), sizeof(left), cudaMemcpyDeviceToHost, st));
            CLR_CUDA_TRY(cudaStreamSynchronize(st));
            if (left == 0) return CLR_OK;
        }
    }
    k_bt_check_done<<<1, 1, 0, st>>>(b->S, (int)(cap & 1));
    CLR_LAUNCH_CHECK("k_bt_check_done");
    return CLR_OK;
}
