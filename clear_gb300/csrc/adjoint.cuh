// Derivatives of the BxDF values (reflection.cl:500-583) with respect to the
// scene parameters the adjoint renderer differentiates: the colour texture of
// a component (R, T, Rs, Rd) and its float textures (Oren-Nayar sigma, Ward
// ax/ay, Ashikhmin nu/nv), all read at the shading point's uv.  Sampling
// pdfs are not differentiated (path replay with detached sampling).
#pragma once

#include "shading.cuh"

namespace clr {

constexpr uint32_t kNoTex = 0xFFFFFFFFu;
constexpr int kMaxGrad = 6;  // distinct parameters touched by one BSDF evaluation

// Texture offsets a component reads: colour c0, colour c1, float a, float b.
struct BxTex {
    uint32_t c0, c1, a, b;
};

__device__ __forceinline__ BxTex bx_tex(const BSDF& f, uint32_t off) {
    BxTex t{kNoTex, kNoTex, kNoTex, kNoTex};
    if (off == 0xFFFF) return t;
    const uint8_t* p = f.mat + off;
    switch (p[0]) {
        case kBxDiffuse: t.c0 = ldb<uint32_t>(p + 4); t.a = ldb<uint32_t>(p + 8); break;
        case kBxSpecR: case kBxSpecT: t.c0 = ldb<uint32_t>(p + 4); break;
        case kBxNewWard: case kBxAshS:
            t.c0 = ldb<uint32_t>(p + 4); t.a = ldb<uint32_t>(p + 8); t.b = ldb<uint32_t>(p + 12); break;
        case kBxAshD: t.c0 = ldb<uint32_t>(p + 8); t.c1 = ldb<uint32_t>(p + 4); break;  // Rd, Rs
        default: break;
    }
    return t;
}

// d f / d(c0), d f / d(c1), d f / d(a), d f / d(b): per colour channel (the
// colour derivatives are diagonal: channel c of f depends on channel c of the
// colour only).  `sigma` is the Oren-Nayar roughness texture value.
struct BxDeriv {
    f3 dc0, dc1, da, db;
};

static __device__ __noinline__ BxDeriv bx_f_deriv(const BxDF& b, float sigma, f3 vout, f3 vin) {
    const f3 zero = mk(0, 0, 0);
    BxDeriv d{zero, zero, zero, zero};
    switch (b.id) {
        case kBxDiffuse: {
            if (vin.z * vout.z <= 0.0f) return d;
            if (b.a == 1.0f) {  // sigma == 0: f = R / pi, A and B are flat in sigma there
                d.dc0 = mk(1.0f / kPi, 1.0f / kPi, 1.0f / kPi);
                return d;
            }
            const float sti = sin_theta(vin), sto = sin_theta(vout);
            float maxCos = 0.0f;
            if (sti > 1e-4f && sto > 1e-4f) maxCos = fmaxf(0.0f, cos_phi(vin) * cos_phi(vout) + sin_phi(vin) * sin_phi(vout));
            float sinAlpha, tanBeta;
            if (fabsf(vin.z) > fabsf(vout.z)) {
                sinAlpha = sto;
                tanBeta = sti / fabsf(vin.z);
            } else {
                sinAlpha = sti;
                tanBeta = sto / fabsf(vout.z);
            }
            const float X = maxCos * sinAlpha * tanBeta;
            const float k = (b.a + b.b * X) / kPi;
            d.dc0 = mk(k, k, k);
            // A = 1 - s2 / (2 (s2 + 0.33)), B = 0.45 s2 / (s2 + 0.09), s2 = sigma^2
            const float s2 = sigma * sigma;
            const float dA = -1.32f * sigma / ((2.0f * s2 + 0.66f) * (2.0f * s2 + 0.66f));
            const float dB = 0.081f * sigma / ((s2 + 0.09f) * (s2 + 0.09f));
            d.da = b.c0 * ((dA + dB * X) / kPi);
            return d;
        }
        case kBxNewWard: {
            if (vin.z * vout.z <= 0.0f) return d;
            const f3 h = normalize(vout + vin);
            const float hx = h.x / b.a, hy = h.y / b.b, dotHN = fabsf(h.z), dotHI = dot(h, vin);
            const float k = expf(-(hx * hx + hy * hy) / (dotHN * dotHN)) /
                            (4 * kPi * b.a * b.b * dotHI * dotHI * dotHN * dotHN * dotHN * dotHN);
            d.dc0 = mk(k, k, k);
            if (!(k > 0.0f) || !isfinite(k)) return d;  // underflow: the roughness terms vanish too
            const f3 f = b.c0 * k;
            const float n2 = dotHN * dotHN;
            d.da = f * (2.0f * hx * hx / (b.a * n2) - 1.0f / b.a);
            d.db = f * (2.0f * hy * hy / (b.b * n2) - 1.0f / b.b);
            return d;
        }
        case kBxAshS: {
            if (vin.z * vout.z <= 0.0f) return d;
            const f3 h = normalize(vout + vin);
            const float dotHV = dot(h, vout);
            const float s2 = 1 - h.z * h.z;
            const float e = (b.a * h.x * h.x + b.b * h.y * h.y) / s2;
            const float w5 = powf(1.0f - dotHV, 5);
            const float g = sqrtf((b.a + 1) * (b.b + 1)) / (8 * kPi) * powf(fabsf(h.z), e) /
                            (dotHV * fmaxf(fabsf(vout.z), fabsf(vin.z)));
            const f3 fr = b.c0 + (mk(1, 1, 1) - b.c0) * w5;
            const f3 f = g * fr;
            d.dc0 = mk(g * (1.0f - w5), g * (1.0f - w5), g * (1.0f - w5));
            if (!(g > 0.0f) || !isfinite(g)) return d;
            const float lnz = logf(fabsf(h.z));
            d.da = f * (0.5f / (b.a + 1) + lnz * h.x * h.x / s2);
            d.db = f * (0.5f / (b.b + 1) + lnz * h.y * h.y / s2);
            return d;
        }
        case kBxAshD: {
            if (vin.z * vout.z <= 0.0f) return d;
            const float go = 1.0f - powf(1.0f - fabsf(vout.z) / 2, 5), gi = 1.0f - powf(1.0f - fabsf(vin.z) / 2, 5);
            const float k = 28.0f / (23.0f * kPi) * go * gi;
            d.dc0 = (mk(1, 1, 1) - b.c1) * k;  // d/dRd
            d.dc1 = b.c0 * (-k);               // d/dRs
            return d;
        }
        default:
            return d;
    }
}

// Derivative of the value a sampled specular component returns
// (reflection.cl:404-438): R F / |cos| or (1 - F) T / |cos|, linear in R / T.
__device__ __forceinline__ f3 spec_dc0(const BxDF& b, f3 vout, f3 vin) {
    if (b.id == kBxSpecR) return eval_fresnel(b.fresnel, vout.z) / fabsf(vin.z);
    if (b.id == kBxSpecT) return (mk(1, 1, 1) - eval_fresnel(b.fresnel, vout.z)) / fabsf(vin.z);
    return mk(0, 0, 0);
}

// ------------------------------------------------------------- parameters

// The differentiated parameters: K constant textures, identified by their
// offset in the textures blob.  A colour texture has 3 gradient channels; a
// float texture (kind 1) feeds every colour channel and has one.
struct ParamTable {
    const uint32_t* tex;
    const uint8_t* kind;
    uint32_t k;
};

__device__ __forceinline__ int param_slot(const ParamTable& pt, uint32_t tex_off) {
    if (tex_off == kNoTex) return -1;
    for (uint32_t i = 0; i < pt.k; ++i)
        if (__ldg(pt.tex + i) == tex_off) return (int)i;
    return -1;
}

// Sparse derivative of a BSDF value: (slot, d value / d parameter) pairs.
struct GradList {
    int n;
    int slot[kMaxGrad];
    f3 d[kMaxGrad];
    __device__ __forceinline__ void clear() { n = 0; }
    __device__ __forceinline__ void add(int s, f3 v) {
        if (s < 0) return;
#pragma unroll
        for (int i = 0; i < kMaxGrad; ++i)
            if (i < n && slot[i] == s) {
                d[i] += v;
                return;
            }
        if (n < kMaxGrad) {
            slot[n] = s;
            d[n] = v;
            ++n;
        } else {
            clr_raise(CLR_DEVERR_QUEUE);
        }
    }
};

// Diffuse sigma texture value of a component (needed for its derivative).
__device__ __forceinline__ float bx_sigma(const BSDF& f, uint32_t off) {
    if (off == 0xFFFF) return 0.f;
    const uint8_t* p = f.mat + off;
    return p[0] == kBxDiffuse ? eval_float_texture(f.tex + ldb<uint32_t>(p + 8), f.uv) : 0.f;
}

// Adds d(component value)/d(parameters) of component `off` to g.
__device__ __forceinline__ void bx_grad(const BSDF& f, uint32_t off, const ParamTable& pt, f3 vl, f3 il, GradList& g) {
    const BxDF b = load_bx(f, off);
    const BxTex t = bx_tex(f, off);
    const BxDeriv d = bx_f_deriv(b, bx_sigma(f, off), vl, il);
    g.add(param_slot(pt, t.c0), d.dc0);
    g.add(param_slot(pt, t.c1), d.dc1);
    g.add(param_slot(pt, t.a), d.da);
    g.add(param_slot(pt, t.b), d.db);
}

}  // namespace clr
