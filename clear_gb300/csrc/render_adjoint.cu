// Adjoint path tracer: path-replay backpropagation in wavefront form.
//
// Gives G = sum_p dLoss/dAccum_p . dAccum_p/dtheta for a per-pixel weight
// dLoss/dAccum (the gradient of an image loss) with respect to constant
// textures of the materials (colour: albedo R / T / Rs / Rd; float: Oren-Nayar
// sigma, Ward ax / ay, Ashikhmin nu / nv) and the texels of the environment's
// image texture.  Sampling is detached: directions, pdfs, MIS weights, light
// selection and Russian-roulette probabilities are constants, so G is the
// derivative of the estimator over the sampled paths (no visibility or
// geometry terms).
//
// Every sample of a pixel runs twice from the same RNG state in the pixel's
// path slot:
//   primal pass : the forward path tracer (render_wf.cu) with the radiance of
//                 the sample summed into L instead of the pixel;
//   replay pass : the same path, same random numbers; each term is subtracted
//                 from L when it is met, so L is the radiance still ahead.
//                 The BSDF value sampled at vertex k scales every later term:
//                 it adds dlog(fs_k)/dtheta * L, taken at vertex k+1 after the
//                 shadow pass has removed vertex k's next-event term.  Emission
//                 and next-event terms add their own BSDF / environment-texel
//                 derivatives.
// Between its passes a path keeps its RNG state and, for its first kAdCache
// vertices, the primal's hit records and next-event visibilities, so that the
// replay traces only what lies deeper (the same rays give the same answers);
// with CLR_ADJOINT_RETRACE (`cached` = 0 in the kernels) it keeps only the
// RNG state and the replay traces every ray again.
//
// Gradients of the material parameters are summed per block in shared memory
// and kept per block in the workspace; one reduction adds them to the caller's
// buffer at the end.  Environment texels (many addresses, little contention)
// take global atomics.
//
// An optional tape records every factor of every replayed path (camera
// weight, emission, roulette, next-event and BSDF-sample records) so that the
// estimator can be re-evaluated on the host with perturbed parameters.
#include "adjoint.cuh"
#include "render_common.cuh"

CLR_DEFINE_STATUS_READER(render_adjoint)

namespace clr {

constexpr int kAdThreads = 128;
constexpr uint32_t kSmemParams = 1024;  // parameters summed in shared memory (K * 16 B)
constexpr int kShWords = 4 + kMaxGrad;  // float4s per shadow entry
// The replay pass traces the primal pass's rays again (same random numbers,
// same arithmetic), so the primal's answers are kept for the replay: the hit
// record of each of a path's first kAdCache vertices, and per vertex whether
// its next-event ray was unoccluded.  A shadow entry's path word carries the
// vertex depth in its top bits (kShDepthShift), for images below 2^27 pixels.
constexpr uint32_t kAdCache = 8;
constexpr uint32_t kShDepthShift = 27;
constexpr uint32_t kShPixMask = (1u << kShDepthShift) - 1u;

// Tape record kinds (word 3, bits 0-7); bit 8 marks a visible next-event record.
enum : uint32_t { kTapeCam = 0, kTapeEmit = 1, kTapeRR = 2, kTapeNee = 3, kTapeSample = 4, kTapeVisible = 0x100 };
constexpr uint32_t kTapeWords = 32;
constexpr uint32_t kTapeSpecular = 0x80000000u;  // BSDF-sample record: specular component index follows

struct AdState {
    float4* org;     // xyz ray origin, w the path's light face (bits; shadow_visible)
    float4* dir;     // xyz direction, w dirPDF
    float4* alpha;   // xyz throughput, w initY
    uint4* misc;     // x depth, y sampledType, z samples done, w pass (0 primal, 1 replay)
    float4* hit;     // x id bits, y t, z b1, w b2
    float4* L;       // xyz radiance of the sample (primal: summed so far; replay: still ahead)
    uint4* rng0;     // RNG state at the start of the current sample
    float4* pd;      // kMaxGrad per path: pending dlog(fs)/dtheta per channel, w = slot bits (-1 = none)
    uint32_t* q[4];  // path queues, [2 * parity + pass]
    float4* sh;      // kShWords float4s per shadow entry
    unsigned int* count;  // [2 * parity + pass] queued paths, [4] shadow entries
    float* partial;  // per-block parameter gradients (grid x K x 4), or null
    float4* hitc;    // kAdCache per path: the primal pass's hit record at each vertex
    uint32_t* visc;  // per path: bit k = the primal's next-event ray at vertex k was unoccluded
};

struct Tape {
    uint32_t* rec;
    uint32_t cap;
    uint32_t* count;
};

struct AdParams {
    ParamTable pt;
    float4* grad;         // K entries: xyz per channel (colour) or x (float)
    uint32_t env_tex;     // textures-blob offset of the differentiated environment texture, kNoTex = none
    float4* grad_env;     // one per texel of that texture
    const float4* dloss;  // dLoss / dAccum per pixel
    Tape tape;
};

__device__ __forceinline__ Rng rng_from(uint4 s) {
    Rng r;
    r.s[0] = s.x;
    r.s[1] = s.y;
    r.s[2] = s.z;
    r.s[3] = s.w;
    return r;
}
__device__ __forceinline__ uint4 rng_bits(const Rng& r) { return make_uint4(r.s[0], r.s[1], r.s[2], r.s[3]); }

__device__ __forceinline__ uint32_t ad_queue_slot(unsigned int* count, bool want) {
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

// d / fs of one channel (0 where fs is 0 or the ratio overflows).
__device__ __forceinline__ float dlog(float d, float fs) {
    const float r = fs != 0.f ? d / fs : 0.f;
    return isfinite(r) ? r : 0.f;
}

// Where a block sums its parameter gradients (the table's size picks it):
//   kSinkPrivate : one private float per thread, parameter and channel in
//                  shared memory (no atomics), summed per block at the end;
//   kSinkShared  : per-block shared-memory atomics;
//   kSinkGlobal  : global atomics straight into the caller's buffer.
// The first two keep per-channel sums in the block's row of the per-block
// buffer; k_ad_reduce folds float parameters' channels together.
enum : int { kSinkNone = 0, kSinkPrivate = 1, kSinkShared = 2, kSinkGlobal = 3 };
constexpr uint32_t kPrivStride = kAdThreads + 1;  // padded: the end-of-block sums read conflict-free
constexpr uint32_t kPrivMaxParams = 31;           // 3 x 31 x 129 floats < 48 KB

__host__ __device__ __forceinline__ int sink_mode(uint32_t k) {
    return k == 0 ? kSinkNone : (k <= kPrivMaxParams ? kSinkPrivate : (k <= kSmemParams ? kSinkShared : kSinkGlobal));
}
__host__ __device__ __forceinline__ uint32_t sink_smem_bytes(uint32_t k) {
    const int m = sink_mode(k);
    return m == kSinkPrivate ? 3u * k * kPrivStride * 4u : (m == kSinkShared ? 4u * k * 4u : 0u);
}

struct GradSink {
    int mode;
    float* s;
    const uint8_t* kind;
    __device__ __forceinline__ void add(int slot, f3 w) const {
        if (slot < 0) return;
        if (mode == kSinkPrivate) {
            float* a = s + (3u * slot) * kPrivStride + threadIdx.x;
            a[0] += w.x;
            a[kPrivStride] += w.y;
            a[2 * kPrivStride] += w.z;
        } else if (mode == kSinkShared) {
            float* g = s + 4 * slot;
            atomicAdd(g, w.x);
            atomicAdd(g + 1, w.y);
            atomicAdd(g + 2, w.z);
        } else {
            float* g = s + 4 * slot;
            if (__ldg(kind + slot) == 1) {
                atomicAdd(g, w.x + w.y + w.z);
            } else {
                atomicAdd(g, w.x);
                atomicAdd(g + 1, w.y);
                atomicAdd(g + 2, w.z);
            }
        }
    }
};

extern __shared__ float s_grad[];

__device__ __forceinline__ GradSink sink_begin(const AdParams& P) {
    GradSink g;
    g.kind = P.pt.kind;
    g.mode = sink_mode(P.pt.k);
    if (g.mode == kSinkPrivate || g.mode == kSinkShared) {
        const uint32_t n = sink_smem_bytes(P.pt.k) / 4u;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) s_grad[i] = 0.f;
        __syncthreads();
        g.s = s_grad;
    } else {
        g.s = reinterpret_cast<float*>(P.grad);
    }
    return g;
}

// Adds the block's sums to its row of the per-block buffer (the row's only
// writer: kernels of one call run in stream order).
__device__ __forceinline__ void sink_end(const AdState& S, const AdParams& P, const GradSink& g) {
    if (g.mode != kSinkPrivate && g.mode != kSinkShared) return;
    __syncthreads();
    float* row = S.partial + (size_t)blockIdx.x * 4u * P.pt.k;
    if (g.mode == kSinkShared) {
        for (uint32_t i = threadIdx.x; i < 4u * P.pt.k; i += blockDim.x) {
            const float v = s_grad[i];
            if (v != 0.f) row[i] += v;
        }
        return;
    }
    for (uint32_t i = threadIdx.x; i < 3u * P.pt.k; i += blockDim.x) {
        const float* a = s_grad + i * kPrivStride;
        float v = 0.f;
        for (uint32_t t = 0; t < kAdThreads; ++t) v += a[t];
        if (v != 0.f) row[4u * (i / 3u) + i % 3u] += v;
    }
}

__device__ __forceinline__ void add_env_grad(const AdParams& P, int texel, f3 g) {
    float4* ge = P.grad_env + texel;
    atomicAdd(&ge->x, g.x);
    atomicAdd(&ge->y, g.y);
    atomicAdd(&ge->z, g.z);
}

// Texel of the differentiated environment texture seen in direction uv
// (image lookup of texture.cl:76-80), with the light's multiplier, or -1
// when the environment's first component does not read that texture.
__device__ __forceinline__ int env_texel(const DScene& sc, const AdParams& P, float2 uv, float& mult) {
    mult = 0.f;
    if (P.env_tex == kNoTex) return -1;
    const uint8_t* l = env_light_property(sc);
    if (l[0] == 0) return -1;
    const uint8_t* e = l + 4;  // ImageBasedEnvLElem {id, idx_Le, multiplier, idx_Dist2D}
    if (e[0] != 0 || ldb<uint32_t>(e + 4) != P.env_tex) return -1;
    mult = ldb<float>(e + 8);
    const uint8_t* t = sc.textures + P.env_tex;
    uint32_t x, y;
    const uint8_t* d;
    image_xy(t, uv, x, y, d);
    return (int)(y * ldb<uint32_t>(t + 4) + x);
}

// ------------------------------------------------------------------ tape

__device__ __forceinline__ uint32_t tape_alloc(const Tape& t) {
    if (!t.rec) return kNone32;
    const uint32_t i = atomicAdd(t.count, 1u);
    return i < t.cap ? i : kNone32;
}

struct TapeRec {
    uint32_t w[kTapeWords];
    __device__ __forceinline__ void head(uint32_t p, uint32_t sample, uint32_t depth, uint32_t kind) {
#pragma unroll
        for (int k = 0; k < (int)kTapeWords; ++k) w[k] = 0;
        w[0] = p;
        w[1] = sample;
        w[2] = depth;
        w[3] = kind;
    }
    __device__ __forceinline__ void f(int k, float v) { w[k] = __float_as_uint(v); }
    __device__ __forceinline__ void f3at(int k, f3 v) {
        f(k, v.x);
        f(k + 1, v.y);
        f(k + 2, v.z);
    }
    __device__ __forceinline__ void store(const Tape& t, uint32_t i) const {
        uint4* dst = reinterpret_cast<uint4*>(t.rec + (size_t)kTapeWords * i);
#pragma unroll
        for (int k = 0; k < (int)kTapeWords / 4; ++k)
            dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    }
};

__device__ __forceinline__ void tape_put(const Tape& t, const TapeRec& r) {
    const uint32_t i = tape_alloc(t);
    if (i != kNone32) r.store(t, i);
}

// ---------------------------------------------------------------- kernels
//
// Queues: q[buf][pass] holds the paths of one pass (0 primal, 1 replay) to
// shade in iteration parity `buf`; count[2 * buf + pass] their number and
// count[4] the shadow entries.  The two passes are shaded by separate kernels
// so that neither carries the other's code or diverges on it.

__device__ __forceinline__ uint32_t* queue(const AdState& S, int buf, int pass) { return S.q[2 * buf + pass]; }

__device__ __forceinline__ void ad_start(const Camera& cam, const AdState& S, uint32_t p, uint32_t width, Rng& rng,
                                         uint32_t done, uint32_t pass) {
    f3 org, dir, alpha;
    float dirPDF;
    camera_ray(cam, p % width, p / width, rng, org, dir, alpha, dirPDF);
    S.org[p] = make_float4(org.x, org.y, org.z, __uint_as_float(kNone32));
    S.dir[p] = make_float4(dir.x, dir.y, dir.z, dirPDF);
    S.alpha[p] = make_float4(alpha.x, alpha.y, alpha.z, luminance(alpha));
    S.misc[p] = make_uint4(0u, 0u, done, pass);
    S.pd[(size_t)kMaxGrad * p] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
}

__global__ void __launch_bounds__(kAdThreads) k_ad_init(DScene sc, AdState S, uint32_t npix, uint32_t width,
                                                        uint32_t* __restrict__ rand_states, uint32_t partial_floats) {
    const Camera cam = load_camera(sc);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const uint4 s = reinterpret_cast<const uint4*>(rand_states)[p];
        Rng rng = rng_from(s);
        S.rng0[p] = s;
        ad_start(cam, S, p, width, rng, 0u, 0u);
        S.L[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        reinterpret_cast<uint4*>(rand_states)[p] = rng_bits(rng);
        queue(S, 0, 0)[p] = p;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < partial_floats; i += gridDim.x * blockDim.x)
        S.partial[i] = 0.f;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S.count[0] = npix;
        for (int k = 1; k < 5; ++k) S.count[k] = 0;
    }
}

// Closest hit of every queued path of both passes.
template <bool kOrdered>
__global__ void __launch_bounds__(kAdThreads, 8) k_ad_extend(DScene sc, AdState S, int cur, int cached) {
    const uint32_t n0 = S.count[2 * cur], n = n0 + S.count[2 * cur + 1];
    const uint32_t* q0 = queue(S, cur, 0);
    const uint32_t* q1 = queue(S, cur, 1);
    uint2 stack[kStackSize];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = i < n0 ? q0[i] : q1[i - n0];
        if (cached && i >= n0) {  // replay pass: the primal found this vertex's hit already
            const uint32_t depth = S.misc[p].x;
            if (depth < kAdCache) {
                S.hit[p] = S.hitc[(size_t)kAdCache * p + depth];
                continue;
            }
        }
        const float4 o = S.org[p], d = S.dir[p];
        Hit h;
        if (intersect<kOrdered>(sc, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), h, stack))
            S.hit[p] = make_float4(__uint_as_float(h.id), h.t, h.b1, h.b2);
        else
            S.hit[p] = make_float4(__uint_as_float(kNone32), INFINITY, 0.f, 0.f);
    }
}

// Reflection / transmission mask of the components fs sums (reflection.cl:679-702).
__device__ __forceinline__ uint32_t side_flags(const BSDF& f, f3 vout, f3 vin) {
    return dot(vin, f.ng) * dot(vout, f.ng) > 0 ? (kTyAll & ~kTyTransmission) : (kTyAll & ~kTyReflection);
}

// Derivative of fs (the sum over the matching components) or, for a sampled
// specular component `spec` (>= 0), of that component's value.  Kept out of
// line: the replay kernel calls it from two places.
static __device__ __noinline__ void bsdf_grad(const BSDF& f, const ParamTable& pt, uint32_t flags, int spec, f3 vl,
                                              f3 il, GradList& g) {
    g.clear();
    if (spec >= 0) {
        const uint32_t off = pick4(f.off, (uint32_t)spec);
        g.add(param_slot(pt, bx_tex(f, off).c0), spec_dc0(load_bx(f, off), vl, il));
        return;
    }
#pragma unroll 1
    for (int k = 0; k < f.num; ++k)
        if (match_type(f.type[k], flags)) bx_grad(f, f.off[k], pt, vl, il, g);
}

// Shadow entry: [0] origin, w light face (0xFFFFFFFF = environment);
// [1] direction, w path; [2] contribution c, w flags (bit 0 add to L, bit 1
// replay, bits 2.. tape record + 1); replay only: [3] dc/d(env texel), w
// texel (-1 = none); [4 + k] dc/dtheta of parameter k, w slot (-1 = end).
struct ShEntry {
    float4 e[kShWords];
};

__device__ __forceinline__ void put_shadow3(const AdState& S, bool want, float4 e0, float4 e1, float4 e2) {
    const uint32_t ss = ad_queue_slot(S.count + 4, want);
    if (!want) return;
    float4* dst = S.sh + (size_t)kShWords * ss;
    dst[0] = e0;
    dst[1] = e1;
    dst[2] = e2;
}

__device__ __forceinline__ void put_shadow(const AdState& S, bool want, const ShEntry& e, bool replay) {
    const uint32_t ss = ad_queue_slot(S.count + 4, want);
    if (!want) return;
    float4* dst = S.sh + (size_t)kShWords * ss;
    dst[0] = e.e[0];
    dst[1] = e.e[1];
    dst[2] = e.e[2];
    if (replay)
#pragma unroll
        for (int k = 3; k < kShWords; ++k) dst[k] = e.e[k];
}

// Emission seen at a path vertex and the MIS weight of the BSDF sample that
// found it (pathtracer.cl:165-204).  Returns the emitted radiance and sets
// `w` to the weight (1 for camera rays).
__device__ __forceinline__ f3 vertex_emission(const DScene& sc, bool escaped, const SurfPt& sp, const Face& face,
                                              f3 org, f3 dir, float dirPDF, uint32_t depth, uint32_t sampledType,
                                              LightPt& lenv, float& w) {
    w = 1.0f;
    const f3 vout = -dir;
    if (escaped) {
        lenv.atInfinity = true;
        lenv.uv = env_uv(dir);
        EDF edf;
        edf_alloc(sc, kNone16, lenv, edf);
        if ((sampledType & kTyNonSingular) && depth > 0) {
            const float lightPDF = area_pdf(sc, lenv) * 1.0f / edf_abs_cos(edf, vout);
            w = (dirPDF * dirPDF) / (lightPDF * lightPDF + dirPDF * dirPDF);
        }
        return edf_le(edf, vout);
    }
    if (face.light == kNone16) return mk(0.f, 0.f, 0.f);
    LightPt lpos;
    light_from_surface(sp, lpos);
    EDF edf;
    edf_alloc(sc, face.light, lpos, edf);
    if (depth > 0 && (sampledType & kTyNonSingular)) {
        const float d2 = (org.x - sp.p.x) * (org.x - sp.p.x) + (org.y - sp.p.y) * (org.y - sp.p.y) +
                         (org.z - sp.p.z) * (org.z - sp.p.z);
        const float lightPDF = area_pdf(sc, lpos) * d2 / edf_abs_cos(edf, vout);
        w = (dirPDF * dirPDF) / (lightPDF * lightPDF + dirPDF * dirPDF);
    }
    return edf_le(edf, vout);
}

// Next-event estimation at a surface point (pathtracer.cl:216-240): samples a
// light, returns false when the BSDF has no non-specular component.  Sets the
// shadow ray, the scalar weight s (MIS * |cos_l| * |cos| / dist^2 / pdf),
// the light's radiance and the BSDF value toward it; light_face is the
// path's light face (shadow_visible), updated when an area light is sampled.
struct Nee {
    f3 org, dir, le, fs;
    float s;
    LightPt lpos;
};

__device__ __forceinline__ void next_event(const DScene& sc, const BSDF& bsdf, const SurfPt& sp, f3 vout, Rng& rng,
                                           Nee& n, uint32_t& light_face) {
    const float uL = rng.uniform(), u0 = rng.uniform(), u1 = rng.uniform();
    EDF edf;
    float lightPDF;
    n.lpos.faceID = light_face;
    sample_light(sc, uL, u0, u1, n.lpos, edf, lightPDF);
    light_face = n.lpos.faceID;
    f3 vinL = n.lpos.p - sp.p;
    float dist2 = dot(vinL, vinL);
    vinL = vinL * (1.0f / sqrtf(dist2));
    if (n.lpos.atInfinity) {
        vinL = n.lpos.p;
        dist2 = 1.0f;
    }
    n.org = sp.p + vinL * kEpsilon;
    n.dir = vinL;
    const float fsPDF = bsdf_pdf(bsdf, vout, vinL) * edf_abs_cos(edf, vinL) / dist2;
    const float MISWeight = (lightPDF * lightPDF) / (lightPDF * lightPDF + fsPDF * fsPDF);
    n.s = MISWeight * edf_abs_cos(edf, vinL) * fabsf(dot(bsdf.n, vinL)) / dist2 / lightPDF;
    n.le = edf_le(edf, -vinL);
    n.fs = bsdf_f(bsdf, vout, vinL);
}

// Primal pass: the forward path tracer (render_wf.cu k_wf_shade) summing the
// sample's radiance into L.  A finished sample is queued for its replay,
// unless its pixel's loss weight is zero: its replay would add nothing to any
// gradient, and the random-number state after the primal pass is the state
// the replay would end in, so the pixel goes on with its next sample.
__global__ void __launch_bounds__(kAdThreads, 4) k_ad_primal(DScene sc, AdState S, int cur, uint32_t width,
                                                          uint32_t* __restrict__ rand_states, uint32_t max_depth,
                                                          const float4* __restrict__ dloss, uint32_t spp,
                                                          int cached) {
    const uint32_t n = S.count[2 * cur];
    const uint32_t* qin = queue(S, cur, 0);
    const Camera cam = load_camera(sc);
    const uint32_t n_round = (n + 31u) & ~31u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += gridDim.x * blockDim.x) {
        bool cont = false, shadow = false;
        int next_pass = 0;
        uint32_t p = 0;
        float4 sh0, sh1, sh2;
        if (i < n) {
            p = qin[i];
            Rng rng = rng_from(reinterpret_cast<const uint4*>(rand_states)[p]);
            const float4 o4 = S.org[p], d4 = S.dir[p], a4 = S.alpha[p], h4 = S.hit[p], L4 = S.L[p];
            const uint4 m = S.misc[p];
            f3 org = mk(o4.x, o4.y, o4.z), dir = mk(d4.x, d4.y, d4.z), alpha = mk(a4.x, a4.y, a4.z);
            f3 L = mk(L4.x, L4.y, L4.z);
            float dirPDF = d4.w;
            const float initY = a4.w;
            uint32_t depth = m.x, sampledType = m.y;
            bool ended = false;
            if (cached && depth < kAdCache) S.hitc[(size_t)kAdCache * p + depth] = h4;  // for the replay pass
            const uint32_t hid = __float_as_uint(h4.x);
            uint32_t light_face = __float_as_uint(o4.w);
            SurfPt sp;
            Face face;
            if (hid != kNone32) {
                Hit h{hid, h4.y, h4.z, h4.w};
                surface_point(sc, org, dir, h, sp);
                face = load_face(sc, sp.faceID);
                if (face.light != kNone16) light_face = sp.faceID;  // LightPointFromSurfacePoint
            }
            LightPt lenv;
            float w;
            const f3 le = vertex_emission(sc, hid == kNone32, sp, face, org, dir, dirPDF, depth, sampledType, lenv, w);
            L += w * alpha * le;
            if (hid == kNone32) {
                ended = true;
            } else {
                const f3 vout = -dir;
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
                        Nee ne;
                        next_event(sc, bsdf, sp, vout, rng, ne, light_face);
                        const f3 c = ne.s * (alpha * ne.le * ne.fs);
                        sh0 = make_float4(ne.org.x, ne.org.y, ne.org.z,
                                              __uint_as_float(shadow_light_word(ne.lpos)));
                        sh1 = make_float4(ne.dir.x, ne.dir.y, ne.dir.z,
                                          __uint_as_float(p | (min(depth, 31u) << kShDepthShift)));
                        sh2 = make_float4(c.x, c.y, c.z, __uint_as_float(1u));  // add to L
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
            }
            cont = true;
            const float4 g = __ldg(dloss + p);
            if (ended && g.x == 0.0f && g.y == 0.0f && g.z == 0.0f) {
                if (m.z + 1 < spp) {
                    S.rng0[p] = rng_bits(rng);
                    ad_start(cam, S, p, width, rng, m.z + 1, 0u);
                } else {
                    S.misc[p] = make_uint4(depth, sampledType, m.z + 1, 1u);
                    cont = false;
                }
            } else if (ended) {
                // replay the sample from its first random number
                rng = rng_from(S.rng0[p]);
                ad_start(cam, S, p, width, rng, m.z, 1u);
                next_pass = 1;
            } else {
                S.org[p] = make_float4(org.x, org.y, org.z, __uint_as_float(light_face));
                S.dir[p] = make_float4(dir.x, dir.y, dir.z, dirPDF);
                S.alpha[p] = make_float4(alpha.x, alpha.y, alpha.z, initY);
                S.misc[p] = make_uint4(depth, sampledType, m.z, 0u);
            }
            S.L[p] = make_float4(L.x, L.y, L.z, 0.f);
            reinterpret_cast<uint4*>(rand_states)[p] = rng_bits(rng);
        }
        const uint32_t s0 = ad_queue_slot(S.count + 2 * (cur ^ 1), cont && next_pass == 0);
        const uint32_t s1 = ad_queue_slot(S.count + 2 * (cur ^ 1) + 1, cont && next_pass == 1);
        if (cont) queue(S, cur ^ 1, next_pass)[next_pass ? s1 : s0] = p;
        put_shadow3(S, shadow, sh0, sh1, sh2);
    }
}

// Replay pass: the same vertex, subtracting each term from L and adding the
// derivatives.  A finished replay starts the pixel's next sample (primal).
template <bool kTape>
__global__ void __launch_bounds__(kAdThreads, 4) k_ad_replay(DScene sc, AdState S, AdParams P, int cur, uint32_t width,
                                                          uint32_t* __restrict__ rand_states, uint32_t spp,
                                                          uint32_t max_depth) {
    const uint32_t n = S.count[2 * cur + 1];
    const uint32_t n_round = (n + 31u) & ~31u;
    if (blockIdx.x * blockDim.x >= n_round) return;  // whole block idle: skip the gradient sink
    const GradSink sink = sink_begin(P);
    const uint32_t* qin = queue(S, cur, 1);
    const Camera cam = load_camera(sc);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += gridDim.x * blockDim.x) {
        bool cont = false, shadow = false;
        int next_pass = 1;
        uint32_t p = 0;
        ShEntry se;
        if (i < n) {
            p = qin[i];
            Rng rng = rng_from(reinterpret_cast<const uint4*>(rand_states)[p]);
            const float4 o4 = S.org[p], d4 = S.dir[p], a4 = S.alpha[p], h4 = S.hit[p], L4 = S.L[p];
            const float4 dl4 = __ldg(P.dloss + p);
            const uint4 m = S.misc[p];
            f3 org = mk(o4.x, o4.y, o4.z), dir = mk(d4.x, d4.y, d4.z), alpha = mk(a4.x, a4.y, a4.z);
            f3 L = mk(L4.x, L4.y, L4.z);
            const f3 dL = mk(dl4.x, dl4.y, dl4.z);
            float dirPDF = d4.w;
            const float initY = a4.w;
            uint32_t depth = m.x, sampledType = m.y;
            const uint32_t done = m.z;
            if (kTape && depth == 0) {
                TapeRec r;
                r.head(p, done, 0, kTapeCam);
                r.f3at(4, alpha);
                tape_put(P.tape, r);
            }
            // the BSDF value sampled at the previous vertex scales all that is ahead
            for (int k = 0; k < kMaxGrad; ++k) {
                const float4 dd = S.pd[(size_t)kMaxGrad * p + k];
                const int slot = __float_as_int(dd.w);
                if (slot < 0) break;
                sink.add(slot, dL * L * mk(dd.x, dd.y, dd.z));
            }
            int npend = 0;
            bool ended = false;
            const uint32_t hid = __float_as_uint(h4.x);
            uint32_t light_face = __float_as_uint(o4.w);
            SurfPt sp;
            Face face;
            if (hid != kNone32) {
                Hit h{hid, h4.y, h4.z, h4.w};
                surface_point(sc, org, dir, h, sp);
                face = load_face(sc, sp.faceID);
                if (face.light != kNone16) light_face = sp.faceID;  // LightPointFromSurfacePoint
            }
            LightPt lenv;
            float w;
            const f3 le = vertex_emission(sc, hid == kNone32, sp, face, org, dir, dirPDF, depth, sampledType, lenv, w);
            const f3 T = w * alpha * le;
            L = mk(L.x - T.x, L.y - T.y, L.z - T.z);
            if (hid == kNone32) {
                float mult;
                const int tx = env_texel(sc, P, lenv.uv, mult);
                if (tx >= 0) add_env_grad(P, tx, dL * (w * alpha) * mult);
                if (kTape) {
                    TapeRec r;
                    r.head(p, done, depth, kTapeEmit);
                    r.f(4, w);
                    r.f3at(5, le);
                    r.w[8] = (uint32_t)tx;
                    r.f(9, mult);
                    tape_put(P.tape, r);
                }
                ended = true;
            } else {
                if (kTape && face.light != kNone16) {
                    TapeRec r;
                    r.head(p, done, depth, kTapeEmit);
                    r.f(4, w);
                    r.f3at(5, le);
                    r.w[8] = kNone32;
                    tape_put(P.tape, r);
                }
                const f3 vout = -dir;
                if (depth > 0) {
                    if (depth >= max_depth) ended = true;
                    else {
                        const float continueProb = fminf(luminance(alpha) * (1.0f / initY), 1.0f);
                        if (rng.uniform() < continueProb) {
                            alpha *= 1.0f / continueProb;
                            dirPDF *= continueProb;
                            if (kTape) {
                                TapeRec r;
                                r.head(p, done, depth, kTapeRR);
                                r.f(4, 1.0f / continueProb);
                                tape_put(P.tape, r);
                            }
                        } else {
                            ended = true;
                        }
                    }
                }
                if (!ended) {
                    BSDF bsdf;
                    bsdf_alloc(sc, face.mat, sp, bsdf);
                    if (bsdf_has_non_specular(bsdf)) {
                        Nee ne;
                        next_event(sc, bsdf, sp, vout, rng, ne, light_face);
                        const f3 c = ne.s * (alpha * ne.le * ne.fs);
                        const uint32_t flags = side_flags(bsdf, vout, ne.dir);
                        const f3 vl = world_to_local(bsdf.s, bsdf.t, bsdf.n, vout);
                        const f3 il = world_to_local(bsdf.s, bsdf.t, bsdf.n, ne.dir);
                        GradList g;
                        bsdf_grad(bsdf, P.pt, flags, -1, vl, il, g);
                        const f3 pre = ne.s * (alpha * ne.le);
#pragma unroll
                        for (int k = 0; k < kMaxGrad; ++k) {
                            const f3 d = k < g.n ? pre * g.d[k] : mk(0.f, 0.f, 0.f);
                            se.e[4 + k] = make_float4(d.x, d.y, d.z, __int_as_float(k < g.n ? g.slot[k] : -1));
                        }
                        float mult = 0.f;
                        const int tx = ne.lpos.atInfinity ? env_texel(sc, P, ne.lpos.uv, mult) : -1;
                        const f3 dt = ne.s * (alpha * ne.fs) * mult;
                        se.e[3] = make_float4(dt.x, dt.y, dt.z, __int_as_float(tx));
                        uint32_t tflag = 0;
                        if (kTape) {
                            const uint32_t ti = tape_alloc(P.tape);
                            if (ti != kNone32) {
                                TapeRec r;
                                r.head(p, done, depth, kTapeNee);
                                r.f(4, ne.s);
                                r.f3at(5, ne.le);
                                r.w[8] = (uint32_t)tx;
                                r.f(9, mult);
                                r.w[10] = face.mat;
                                r.f(11, sp.uv.x);
                                r.f(12, sp.uv.y);
                                r.f3at(13, vl);
                                r.f3at(16, il);
                                r.w[19] = flags;
                                r.store(P.tape, ti);
                                tflag = (ti + 1u) << 2;
                            }
                        }
                        se.e[0] = make_float4(ne.org.x, ne.org.y, ne.org.z,
                                              __uint_as_float(shadow_light_word(ne.lpos)));
                        se.e[1] = make_float4(ne.dir.x, ne.dir.y, ne.dir.z,
                                              __uint_as_float(p | (min(depth, 31u) << kShDepthShift)));
                        se.e[2] = make_float4(c.x, c.y, c.z, __uint_as_float(tflag | 2u));  // bit 0 set below
                        shadow = true;
                    }
                    const float uc = rng.uniform(), v0 = rng.uniform(), v1 = rng.uniform();
                    const f3 fs = bsdf_sample(bsdf, vout, uc, v0, v1, dir, dirPDF, sampledType);
                    if (zero_vec(fs) || dirPDF == 0.0f) {
                        ended = true;
                    } else {
                        // dlog of the sampled value: the summed components for a
                        // non-specular sample, the chosen component for a specular one
                        const f3 vl = world_to_local(bsdf.s, bsdf.t, bsdf.n, vout);
                        const f3 il = world_to_local(bsdf.s, bsdf.t, bsdf.n, dir);
                        GradList g;
                        uint32_t flags;
                        int spec = -1;
                        if (sampledType & kTySpecular) {
                            spec = (int)rand_uint(uc, (uint32_t)bsdf.num);
                            flags = kTapeSpecular | (uint32_t)spec;
                        } else {
                            flags = side_flags(bsdf, vout, dir);
                        }
                        bsdf_grad(bsdf, P.pt, flags, spec, vl, il, g);
                        for (int k = 0; k < g.n; ++k) {
                            const f3 d = mk(dlog(g.d[k].x, fs.x), dlog(g.d[k].y, fs.y), dlog(g.d[k].z, fs.z));
                            S.pd[(size_t)kMaxGrad * p + k] = make_float4(d.x, d.y, d.z, __int_as_float(g.slot[k]));
                        }
                        npend = g.n;
                        if (kTape) {
                            TapeRec r;
                            r.head(p, done, depth, kTapeSample);
                            r.f(4, fabsf(dot(bsdf.n, dir)) / dirPDF);
                            r.w[10] = face.mat;
                            r.f(11, sp.uv.x);
                            r.f(12, sp.uv.y);
                            r.f3at(13, vl);
                            r.f3at(16, il);
                            r.w[19] = flags;
                            tape_put(P.tape, r);
                        }
                        alpha *= fs * (fabsf(dot(bsdf.n, dir)) / dirPDF);
                        org = sp.p + dir * kEpsilon;
                        ++depth;
                    }
                }
            }
            if (ended) {
                // L of this sample is no longer needed: its last next-event term stays out of L
                if (done + 1 < spp) {
                    S.rng0[p] = rng_bits(rng);
                    ad_start(cam, S, p, width, rng, done + 1, 0u);
                    L = mk(0.f, 0.f, 0.f);
                    next_pass = 0;
                    cont = true;
                } else {
                    S.misc[p] = make_uint4(depth, sampledType, done + 1, 1u);
                }
            } else {
                se.e[2].w = __uint_as_float(__float_as_uint(se.e[2].w) | 1u);
                S.org[p] = make_float4(org.x, org.y, org.z, __uint_as_float(light_face));
                S.dir[p] = make_float4(dir.x, dir.y, dir.z, dirPDF);
                S.alpha[p] = make_float4(alpha.x, alpha.y, alpha.z, initY);
                S.misc[p] = make_uint4(depth, sampledType, done, 1u);
                if (npend < kMaxGrad)
                    S.pd[(size_t)kMaxGrad * p + npend] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
                cont = true;
            }
            S.L[p] = make_float4(L.x, L.y, L.z, 0.f);
            reinterpret_cast<uint4*>(rand_states)[p] = rng_bits(rng);
        }
        const uint32_t s0 = ad_queue_slot(S.count + 2 * (cur ^ 1), cont && next_pass == 0);
        const uint32_t s1 = ad_queue_slot(S.count + 2 * (cur ^ 1) + 1, cont && next_pass == 1);
        if (cont) queue(S, cur ^ 1, next_pass)[next_pass ? s1 : s0] = p;
        put_shadow(S, shadow, se, true);
    }
    sink_end(S, P, sink);
}

template <bool kOrdered>
__global__ void __launch_bounds__(kAdThreads, 8) k_ad_shadow(DScene sc, AdState S, AdParams P, int cached) {
    const uint32_t n = S.count[4];
    if (blockIdx.x * blockDim.x >= n) return;
    const GradSink sink = sink_begin(P);
    uint2 stack[kStackSize];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4* e = S.sh + (size_t)kShWords * i;
        const float4 a = e[0], b = e[1], c = e[2];
        const uint32_t pw = __float_as_uint(b.w), flags = __float_as_uint(c.w);
        const uint32_t p = pw & kShPixMask, depth = pw >> kShDepthShift;
        const bool replay = (flags & 2u) != 0;
        bool visible;
        if (cached && replay && depth < kAdCache) {
            visible = (S.visc[p] >> depth) & 1u;  // the primal traced this ray
        } else {
            visible = shadow_visible<kOrdered>(sc, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), __float_as_uint(a.w), stack);
            // one entry per path per launch: this is the bit's only writer
            if (cached && !replay && depth < kAdCache)
                S.visc[p] = (S.visc[p] & ~(1u << depth)) | ((visible ? 1u : 0u) << depth);
        }
        if (!visible) continue;
        if (flags & 1u) {
            float4 L = S.L[p];
            if (replay) {
                L.x -= c.x;
                L.y -= c.y;
                L.z -= c.z;
            } else {
                L.x += c.x;
                L.y += c.y;
                L.z += c.z;
            }
            S.L[p] = L;
        }
        if (!replay) continue;
        if (flags >> 2) P.tape.rec[(size_t)kTapeWords * ((flags >> 2) - 1u) + 3] |= kTapeVisible;
        const float4 dl4 = __ldg(P.dloss + p);
        const f3 dL = mk(dl4.x, dl4.y, dl4.z);
        for (int k = 0; k < kMaxGrad; ++k) {
            const float4 g = e[4 + k];
            const int slot = __float_as_int(g.w);
            if (slot < 0) break;
            sink.add(slot, dL * mk(g.x, g.y, g.z));
        }
        const float4 t = e[3];
        const int tx = __float_as_int(t.w);
        if (tx >= 0) add_env_grad(P, tx, dL * mk(t.x, t.y, t.z));
    }
    sink_end(S, P, sink);
}

__global__ void k_ad_reset(AdState S, int next) {
    S.count[2 * next] = 0;
    S.count[2 * next + 1] = 0;
    S.count[4] = 0;
}

// grad[k] += sum over blocks of partial[b][k] (channels summed for a float
// parameter); one block per parameter.
__global__ void __launch_bounds__(256) k_ad_reduce(const float* __restrict__ partial, uint32_t nblocks, uint32_t k,
                                                   const uint8_t* __restrict__ kind, float* __restrict__ grad) {
    const uint32_t slot = blockIdx.x;
    float acc[3] = {0.f, 0.f, 0.f};
    for (uint32_t b = threadIdx.x; b < nblocks; b += blockDim.x) {
        const float* r = partial + (size_t)b * 4u * k + 4u * slot;
        acc[0] += r[0];
        acc[1] += r[1];
        acc[2] += r[2];
    }
    __shared__ float red[3][8];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xFFFFFFFFu, acc[c], o);
        if ((threadIdx.x & 31) == 0) red[c][threadIdx.x >> 5] = acc[c];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float s[3] = {0.f, 0.f, 0.f};
        for (int c = 0; c < 3; ++c)
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s[c] += red[c][w];
        float* g = grad + 4u * slot;
        if (kind[slot] == 1) {
            g[0] += s[0] + s[1] + s[2];
        } else {
            g[0] += s[0];
            g[1] += s[1];
            g[2] += s[2];
        }
    }
}

static uint32_t ad_grid(uint32_t npix) { return std::min(div_up(npix, kAdThreads), (unsigned int)clr_sm_count() * 16u); }

static size_t ad_layout(uint32_t npix, uint32_t num_params, char* base, AdState* S) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) / 256 * 256;
        return o;
    };
    const size_t n = npix;
    const size_t o_org = take(16 * n), o_dir = take(16 * n), o_alpha = take(16 * n), o_misc = take(16 * n),
                 o_hit = take(16 * n), o_L = take(16 * n), o_rng0 = take(16 * n), o_pd = take(16 * kMaxGrad * n),
                 o_q = take(16 * n), o_sh = take(16 * kShWords * n), o_cnt = take(32),
                 o_hitc = take(16 * kAdCache * n), o_visc = take(4 * n);
    const int mode = sink_mode(num_params);
    const bool use_partial = mode == kSinkPrivate || mode == kSinkShared;
    const size_t o_part = use_partial ? take((size_t)ad_grid(npix) * num_params * 16) : 0;
    if (base && S) {
        S->org = reinterpret_cast<float4*>(base + o_org);
        S->dir = reinterpret_cast<float4*>(base + o_dir);
        S->alpha = reinterpret_cast<float4*>(base + o_alpha);
        S->misc = reinterpret_cast<uint4*>(base + o_misc);
        S->hit = reinterpret_cast<float4*>(base + o_hit);
        S->L = reinterpret_cast<float4*>(base + o_L);
        S->rng0 = reinterpret_cast<uint4*>(base + o_rng0);
        S->pd = reinterpret_cast<float4*>(base + o_pd);
        for (int k = 0; k < 4; ++k) S->q[k] = reinterpret_cast<uint32_t*>(base + o_q) + (size_t)k * n;
        S->sh = reinterpret_cast<float4*>(base + o_sh);
        S->count = reinterpret_cast<unsigned int*>(base + o_cnt);
        S->partial = use_partial ? reinterpret_cast<float*>(base + o_part) : nullptr;
        S->hitc = reinterpret_cast<float4*>(base + o_hitc);
        S->visc = reinterpret_cast<uint32_t*>(base + o_visc);
    }
    return off;
}

// One block of kAdBlockIters iterations (the first of parity 0), launched as a
// CUDA graph kept per thread and device (render_common.cuh BlockGraphCache).
constexpr int kAdBlockIters = 8;

struct AdArgs {
    DScene sc;
    AdState S;
    AdParams P;
    uint32_t width, spp, max_depth;
    uint32_t* rand_states;
    bool ordered, tape, cached;
    unsigned int grid;
    size_t smem;
};

static void ad_block(const AdArgs& a, cudaStream_t st) {
    for (int k = 0; k < kAdBlockIters; ++k) {
        const int cur = k & 1;
        if (a.ordered) k_ad_extend<true><<<a.grid, kAdThreads, 0, st>>>(a.sc, a.S, cur, a.cached);
        else k_ad_extend<false><<<a.grid, kAdThreads, 0, st>>>(a.sc, a.S, cur, a.cached);
        k_ad_reset<<<1, 1, 0, st>>>(a.S, cur ^ 1);
        k_ad_primal<<<a.grid, kAdThreads, 0, st>>>(a.sc, a.S, cur, a.width, a.rand_states, a.max_depth, a.P.dloss,
                                                    a.spp, a.cached);
        if (a.tape)
            k_ad_replay<true><<<a.grid, kAdThreads, a.smem, st>>>(a.sc, a.S, a.P, cur, a.width, a.rand_states, a.spp,
                                                                  a.max_depth);
        else
            k_ad_replay<false><<<a.grid, kAdThreads, a.smem, st>>>(a.sc, a.S, a.P, cur, a.width, a.rand_states, a.spp,
                                                                   a.max_depth);
        if (a.ordered) k_ad_shadow<true><<<a.grid, kAdThreads, a.smem, st>>>(a.sc, a.S, a.P, a.cached);
        else k_ad_shadow<false><<<a.grid, kAdThreads, a.smem, st>>>(a.sc, a.S, a.P, a.cached);
    }
}

static bool same_ad_args(const AdArgs& x, const AdArgs& y) {
    const AdParams &p = x.P, &q = y.P;
    return same_scene(x.sc, y.sc) && x.S.org == y.S.org && x.S.count == y.S.count && x.S.partial == y.S.partial &&
           p.pt.tex == q.pt.tex && p.pt.kind == q.pt.kind && p.pt.k == q.pt.k && p.grad == q.grad &&
           p.env_tex == q.env_tex && p.grad_env == q.grad_env && p.dloss == q.dloss && p.tape.rec == q.tape.rec &&
           p.tape.cap == q.tape.cap && p.tape.count == q.tape.count && x.width == y.width && x.spp == y.spp &&
           x.max_depth == y.max_depth && x.rand_states == y.rand_states && x.ordered == y.ordered &&
           x.tape == y.tape && x.cached == y.cached && x.grid == y.grid && x.smem == y.smem;
}

thread_local BlockGraphCache<AdArgs> t_ad_graphs;

}  // namespace clr

using namespace clr;

extern "C" int clr_render_adjoint_workspace_bytes(uint32_t width, uint32_t height, uint32_t num_params,
                                                  uint64_t* bytes) {
    if (!bytes) return clr_set_error(CLR_EINVAL, "clr_render_adjoint_workspace_bytes: bytes is NULL");
    *bytes = ad_layout(width * height, num_params, nullptr, nullptr);
    return CLR_OK;
}

extern "C" int clr_render_adjoint(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                                  const float* dloss_daccum, uint32_t spp, uint32_t max_depth, uint32_t flags,
                                  const clr_adjoint_params* params, void* workspace, uint64_t workspace_bytes,
                                  void* stream) {
    int rc = check_render_args(scene, rand_states, const_cast<float*>(dloss_daccum));
    if (rc != CLR_OK) return rc;
    if (!params) return clr_set_error(CLR_EINVAL, "clr_render_adjoint: params is NULL");
    const clr_adjoint_params& A = *params;
    if (A.num_params > 0 && (!A.param_tex || !A.param_kind || !A.grad_params))
        return clr_set_error(CLR_EINVAL, "clr_render_adjoint: NULL parameter table or gradient buffer");
    if (A.env_tex != kNoTex && !A.grad_env) return clr_set_error(CLR_EINVAL, "clr_render_adjoint: grad_env is NULL");
    if (A.tape && (!A.tape_count || A.tape_capacity == 0 || A.tape_capacity > (1u << 29)))
        return clr_set_error(CLR_EINVAL, "clr_render_adjoint: a tape needs a counter and 1 .. 2^29 records");
    if ((reinterpret_cast<uintptr_t>(A.grad_params) | reinterpret_cast<uintptr_t>(A.grad_env) |
         reinterpret_cast<uintptr_t>(A.tape)) & 15u)
        return clr_set_error(CLR_EINVAL, "clr_render_adjoint: gradient and tape buffers must be 16-byte aligned");
    if (width == 0 || height == 0 || spp == 0) return CLR_OK;
    if ((uint64_t)width * height > kShPixMask)
        return clr_set_error(CLR_EINVAL, "clr_render_adjoint: %u x %u pixels exceed 2^27 - 1", width, height);
    const uint32_t npix = width * height;
    const size_t need = ad_layout(npix, A.num_params, nullptr, nullptr);
    if (!workspace || workspace_bytes < need)
        return clr_set_error(CLR_ECAPACITY, "clr_render_adjoint: workspace of %llu bytes is smaller than %zu",
                             (unsigned long long)workspace_bytes, need);
    if (reinterpret_cast<uintptr_t>(workspace) & 255u)
        return clr_set_error(CLR_EINVAL, "clr_render_adjoint: workspace must be 256-byte aligned");
    if (max_depth == 0) max_depth = 100;
    const DScene sc = make_dscene(scene);
    AdState S;
    ad_layout(npix, A.num_params, static_cast<char*>(workspace), &S);
    AdParams P;
    P.pt.tex = A.param_tex;
    P.pt.kind = A.param_kind;
    P.pt.k = A.num_params;
    P.grad = reinterpret_cast<float4*>(A.grad_params);
    P.env_tex = A.env_tex;
    P.grad_env = reinterpret_cast<float4*>(A.grad_env);
    P.dloss = reinterpret_cast<const float4*>(dloss_daccum);
    P.tape = Tape{A.tape, A.tape_capacity, A.tape_count};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool ordered = (flags & CLR_RENDER_ORDERED) != 0;
    const unsigned int grid = ad_grid(npix);
    const uint32_t nfloats = 4u * A.num_params;
    const size_t smem = sink_smem_bytes(A.num_params);
    k_ad_init<<<grid, kAdThreads, 0, st>>>(sc, S, npix, width, rand_states, S.partial ? grid * nfloats : 0u);
    CLR_LAUNCH_CHECK("k_ad_init");
    // every iteration advances each unfinished path by one vertex; a sample
    // takes at most (max_depth + 1) vertices per pass
    const uint64_t max_iters = 2ull * spp * (max_depth + 1) + 2;
    AdArgs a{};
    a.sc = sc;
    a.S = S;
    a.P = P;
    a.width = width;
    a.spp = spp;
    a.max_depth = max_depth;
    a.rand_states = rand_states;
    a.ordered = ordered;
    a.tape = A.tape != nullptr;
    a.cached = (flags & CLR_ADJOINT_RETRACE) == 0;
    a.grid = grid;
    a.smem = smem;
    cudaGraphExec_t exec = t_ad_graphs.get(a, ad_block, same_ad_args);
    cudaGetLastError();  // a failed capture leaves no error behind: the kernels are launched directly
    // a block ends with the next iteration's queue counts in count[0..1]
    for (uint64_t it = 0; it < max_iters; it += kAdBlockIters) {
        if (exec && cudaGraphLaunch(exec, st) != cudaSuccess) {
            cudaGetLastError();
            t_ad_graphs.drop();
            exec = nullptr;
        }
        if (!exec) ad_block(a, st);
        CLR_LAUNCH_CHECK("adjoint iterations");
        unsigned int left[2] = {0, 0};
        CLR_CUDA_TRY(cudaMemcpyAsync(left, S.count, sizeof(left), cudaMemcpyDeviceToHost, st));
        CLR_CUDA_TRY(cudaStreamSynchronize(st));
        if (left[0] + left[1] == 0) break;
    }
    if (S.partial) {
        k_ad_reduce<<<A.num_params, 256, 0, st>>>(S.partial, grid, A.num_params, A.param_kind, A.grad_params);
        CLR_LAUNCH_CHECK("k_ad_reduce");
    }
    return CLR_OK;
}
