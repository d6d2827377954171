// Device-side shading library of the path tracer: vector helpers, RNG,
// sampling distributions, textures, BSDFs, lights and camera, reading the
// reference's byte-blob scene format (materials / textures / other
// resources).  Each function cites the reference kernel code whose result it
// reproduces; float expressions keep the reference CPU equivalent's operation
// order (OpenCL_PathTracer/Equivalent), including its vector conventions
// (v / s is v * (1/s), normalize(v) = v * (1/|v|)).
#pragma once

#include <cuda_fp16.h>

#include "common.cuh"

namespace clr {

// ------------------------------------------------------------------ vectors

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ f3 operator/(f3 a, float s) {
    const float r = 1.0f / s;
    return mk(a.x * r, a.y * r, a.z * r);
}
__device__ __forceinline__ f3 operator/(f3 a, f3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ f3& operator+=(f3& a, f3 b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    return a;
}
__device__ __forceinline__ f3& operator*=(f3& a, f3 b) {
    a.x *= b.x;
    a.y *= b.y;
    a.z *= b.z;
    return a;
}
__device__ __forceinline__ f3& operator*=(f3& a, float s) {
    a.x *= s;
    a.y *= s;
    a.z *= s;
    return a;
}
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(f3 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ f3 normalize(f3 v) { return v / length(v); }
__device__ __forceinline__ bool zero_vec(f3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }
__device__ __forceinline__ float luminance(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fmaxf(fminf(v, hi), lo); }

constexpr float kPi = 3.14159265358979323846f;

// ------------------------------------------------------------- blob reads

template <typename T>
__device__ __forceinline__ T ldb(const uint8_t* p) {
    return *reinterpret_cast<const T*>(p);
}
__device__ __forceinline__ f3 ldf3(const uint8_t* p) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    return mk(v.x, v.y, v.z);
}
__device__ __forceinline__ const uint8_t* align_ptr(const uint8_t* p, uintptr_t a) {
    return reinterpret_cast<const uint8_t*>((reinterpret_cast<uintptr_t>(p) + (a - 1)) & ~(a - 1));
}

// -------------------------------------------------------------------- RNG
// XORShift128 (rng.cl:21-31), state in registers.

struct Rng {
    uint32_t s[4];
    __device__ __forceinline__ uint32_t next() {
        const uint32_t t = s[0] ^ (s[0] << 11);
        s[0] = s[1];
        s[1] = s[2];
        s[2] = s[3];
        s[3] = (s[3] ^ (s[3] >> 19)) ^ (t ^ (t >> 8));
        return s[3];
    }
    __device__ __forceinline__ float uniform() { return __uint_as_float((next() >> 9) | 0x3f800000u) - 1.0f; }
};

__device__ __forceinline__ uint32_t rand_uint(float u, uint32_t maxv) {
    return min((uint32_t)(maxv * u), maxv - 1u);
}

// concentricSampleDisk (rng.cl:38-71)
__device__ __forceinline__ void concentric_disk(float u1, float u2, float& dx, float& dy) {
    const float sx = 2 * u1 - 1, sy = 2 * u2 - 1;
    if (sx == 0.0f && sy == 0.0f) {
        dx = dy = 0.0f;
        return;
    }
    float r, theta;
    if (sx >= -sy) {
        if (sx > sy) {
            r = sx;
            theta = sy / sx;
        } else {
            r = sy;
            theta = 2.0f - sx / sy;
        }
    } else {
        if (sx > sy) {
            r = -sy;
            theta = 6.0f + sx / sy;
        } else {
            r = -sx;
            theta = 4.0f + sy / sx;
        }
    }
    theta *= kPi / 4.0f;
    dx = r * cosf(theta);
    dy = r * sinf(theta);
}

__device__ __forceinline__ f3 cosine_hemisphere(float u1, float u2) {
    float x, y;
    concentric_disk(u1, u2, x, y);
    return mk(x, y, sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y)));
}

// ---------------------------------------------------------- distributions
// distribution.cl:59-129; offsets are relative to each struct's own head.

__device__ __forceinline__ uint32_t sample_discrete_1d(const uint8_t* d, float u, float* prob) {
    const float* cdf = reinterpret_cast<const float*>(d + ldb<int32_t>(d + 12));
    uint32_t start = 0, end = ldb<uint32_t>(d + 4) + 1, i = end / 2;
    for (int guard = 0; guard < 64; ++guard) {
        if (cdf[i] > u) end = i;
        else start = i;
        if (end - start == 1) break;
        i = (end - start) / 2 + start;
    }
    *prob = reinterpret_cast<const float*>(d + ldb<int32_t>(d + 8))[start];
    return start;
}

__device__ __forceinline__ float prob_discrete_1d(const uint8_t* d, uint32_t i) {
    return reinterpret_cast<const float*>(d + ldb<int32_t>(d + 8))[i];
}

// ContinuousConsts1D: type@0, numValues@4, start@8, end@12, width@16, offPDF@20, offCDF@24
__device__ __forceinline__ float sample_cc_1d(const uint8_t* d, float u, float* pdf) {
    const float* cdf = reinterpret_cast<const float*>(d + ldb<int32_t>(d + 24));
    uint32_t start = 0, end = ldb<uint32_t>(d + 4) + 1, i = end / 2;
    for (int guard = 0; guard < 64; ++guard) {
        if (cdf[i] > u) end = i;
        else start = i;
        if (end - start == 1) break;
        i = (end - start) / 2 + start;
    }
    const float t = (u - cdf[start]) / (cdf[end] - cdf[start]);
    *pdf = reinterpret_cast<const float*>(d + ldb<int32_t>(d + 20))[start];
    return ldb<float>(d + 8) + (start + t) * ldb<float>(d + 16);
}

__device__ __forceinline__ float pdf_cc_1d(const uint8_t* d, float x) {
    const float* pdf = reinterpret_cast<const float*>(d + ldb<int32_t>(d + 20));
    return pdf[(uint32_t)((x - ldb<float>(d + 8)) / ldb<float>(d + 16))];
}

// ContinuousConsts2D_H: type@0, offChildren@4, parent ContinuousConsts1D@8
__device__ __forceinline__ float2 sample_cc_2d(const uint8_t* d, float u0, float u1, float* pdf) {
    const uint8_t* parent = d + 8;
    float pdf_top;
    float2 r;
    r.y = sample_cc_1d(parent, u1, &pdf_top);
    const uint32_t child = (uint32_t)((r.y - ldb<float>(parent + 8)) / ldb<float>(parent + 16));
    r.x = sample_cc_1d(d + ldb<int32_t>(d + 4) + 28u * child, u0, pdf);
    *pdf *= pdf_top;
    return r;
}

__device__ __forceinline__ float pdf_cc_2d(const uint8_t* d, float2 p) {
    const uint8_t* parent = d + 8;
    float r = pdf_cc_1d(parent, p.y);
    const uint32_t child = (uint32_t)((p.y - ldb<float>(parent + 8)) / ldb<float>(parent + 16));
    r *= pdf_cc_1d(d + ldb<int32_t>(d + 4) + 28u * child, p.x);
    return r;
}

// --------------------------------------------------------------- textures
// texture.cl:58-204; texture types of texture_structures.cl:18-28.

enum : uint8_t {
    kTexColorConst = 0, kTexRGB8, kTexRGBA8, kTexRGBA16F, kTexColorProc, kTexGray8, kTexFloatConst, kTexFloatImage,
    kTexFloatProc
};

__device__ __forceinline__ void image_xy(const uint8_t* t, float2 uv, uint32_t& x, uint32_t& y, const uint8_t*& data) {
    const uint32_t w = ldb<uint32_t>(t + 4), h = ldb<uint32_t>(t + 8);
    x = min(max((uint32_t)fmodf(w * uv.x, (float)w), 0u), w - 1);
    y = min(max((uint32_t)fmodf(h * uv.y, (float)h), 0u), h - 1);
    data = t + ldb<int32_t>(t + 12);
}

static __device__ __noinline__ f3 eval_color_texture(const uint8_t* t, float2 uv) {
    switch (t[0]) {
        case kTexColorConst:
            return ldf3(t + 16);
        case kTexRGB8:
        case kTexRGBA8: {
            uint32_t x, y;
            const uint8_t* d;
            image_xy(t, uv, x, y, d);
            const uint32_t w = ldb<uint32_t>(t + 4);
            const uint8_t* p = d + 4u * (y * w + x);  // 4-byte texel (uchar3 / uchar4)
            return mk((float)p[0], (float)p[1], (float)p[2]) / 255.0f;
        }
        case kTexRGBA16F: {
            uint32_t x, y;
            const uint8_t* d;
            image_xy(t, uv, x, y, d);
            const uint32_t w = ldb<uint32_t>(t + 4);
            const __half* p = reinterpret_cast<const __half*>(d) + 4u * (y * w + x);
            return mk(__half2float(p[0]), __half2float(p[1]), __half2float(p[2]));
        }
        case kTexColorProc: {
            const uint8_t proc = t[1];
            if (proc == 0) {  // checkerboard
                const uint32_t k = ((uint32_t)(uv.x * 2) + (uint32_t)(uv.y * 2)) % 2;
                return ldf3(t + 16 + 16 * k);
            }
            if (proc == 1) {  // checkerboard bump
                const float halfWidth = ldb<float>(t + 4) * 0.5f;
                const bool reverse = t[8] != 0;
                float uComp = 0.0f, vComp = 0.0f;
                const float absWrapU = fmodf(fabsf(uv.x), 1.0f);
                if (absWrapU < halfWidth * 0.5f || absWrapU > 1.0f - halfWidth * 0.5f) uComp = 1.0f;
                else if (absWrapU > 0.5f - halfWidth * 0.5f && absWrapU < 0.5f + halfWidth * 0.5f) uComp = -1.0f;
                const float absWrapV = fmodf(fabsf(uv.y), 1.0f);
                if (absWrapV < halfWidth * 0.5f || absWrapV > 1.0f - halfWidth * 0.5f) vComp = 1.0f;
                else if (absWrapV > 0.5f - halfWidth * 0.5f && absWrapV < 0.5f + halfWidth * 0.5f) vComp = -1.0f;
                if (absWrapV > 0.5f) uComp *= -1;
                if (absWrapU > 0.5f) vComp *= -1;
                if (reverse) {
                    uComp *= -1;
                    vComp *= -1;
                }
                const f3 n = normalize(mk(uComp, vComp, 1.0f));
                return mk(0.5f * n.x + 0.5f, 0.5f * n.y + 0.5f, 0.5f * n.z + 0.5f);
            }
            return mk(0, 0, 0);
        }
        case kTexGray8: {
            uint32_t x, y;
            const uint8_t* d;
            image_xy(t, uv, x, y, d);
            const float v = d[y * ldb<uint32_t>(t + 4) + x] / 255.0f;
            return mk(v, v, v);
        }
        default:
            return mk(0, 0, 0);
    }
}

static __device__ __noinline__ float eval_float_texture(const uint8_t* t, float2 uv) {
    switch (t[0]) {
        case kTexFloatConst:
            return ldb<float>(t + 4);
        case kTexFloatImage: {
            uint32_t x, y;
            const uint8_t* d;
            image_xy(t, uv, x, y, d);
            return reinterpret_cast<const float*>(d)[y * ldb<uint32_t>(t + 4) + x];
        }
        case kTexFloatProc: {
            if (t[1] == 0) {
                const uint32_t k = ((uint32_t)(uv.x * 2) + (uint32_t)(uv.y * 2)) % 2;
                return ldb<float>(t + 4 + 4 * k);
            }
            return 0.0f;
        }
        default:
            return 0.0f;
    }
}

// --------------------------------------------------------- surface points

struct SurfPt {
    f3 p, gNormal, sNormal, sTangent, uDir;
    float2 uv;
    uint32_t faceID;
    bool hasTangent;
};

__device__ __forceinline__ void make_tangent(f3 n, f3& t) {  // global.cl:417-426
    if (fabsf(n.x) > fabsf(n.y)) {
        const float inv = 1.0f / sqrtf(n.x * n.x + n.z * n.z);
        t = mk(-n.z * inv, 0.0f, n.x * inv);
    } else {
        const float inv = 1.0f / sqrtf(n.y * n.y + n.z * n.z);
        t = mk(0.0f, n.z * inv, -n.y * inv);
    }
}

__device__ __forceinline__ f3 world_to_local(f3 s, f3 t, f3 n, f3 v) { return mk(dot(s, v), dot(t, v), dot(n, v)); }
__device__ __forceinline__ f3 local_to_world(f3 s, f3 t, f3 n, f3 v) {
    return mk(s.x * v.x + t.x * v.y + n.x * v.z, s.y * v.x + t.y * v.y + n.y * v.z, s.z * v.x + t.z * v.y + n.z * v.z);
}

// ------------------------------------------------------------------ BSDF
// reflection.cl:16-776.

enum : uint8_t { kBxDiffuse = 0, kBxSpecR, kBxSpecT, kBxNewWard, kBxAshS, kBxAshD };
enum : uint32_t {
    kTyReflection = 1, kTyTransmission = 2, kTyDiffuse = 4, kTyGlossy = 8, kTySpecular = 16,
    kTyNonSingular = kTyDiffuse | kTyGlossy, kTyAll = 31
};

struct BxDF {
    uint8_t id;
    uint8_t type;
    f3 c0, c1;       // R | T | Rs (AshikhminS) | Rd, Rs (AshikhminD)
    float a, b;      // A,B (Oren-Nayar) | ax,ay | nu,nv | etaExt,etaInt
    const uint8_t* fresnel;
};

constexpr int kMaxBxDFs = 4;

// A BSDF as the reference's BSDFAlloc builds it (reflection.cl:185-342), but
// holding only the shading frame and where each component's parameters live
// in the material blob: a component's textures are evaluated when the
// component is used (the blobs are small and cache resident), so no per-thread
// array of decoded components is kept.
struct BSDF {
    const uint8_t* mat;
    const uint8_t* tex;
    const uint8_t* others;
    float2 uv;
    int num;
    uint16_t off[kMaxBxDFs];   // element offset from `mat`
    uint8_t type[kMaxBxDFs];   // BxDFType of each component
    f3 n, s, t, ng;
};

__device__ __forceinline__ uint8_t elem_type(uint8_t id) {
    switch (id) {
        case kBxDiffuse: return kTyReflection | kTyDiffuse;
        case kBxSpecR: return kTyReflection | kTySpecular;
        case kBxSpecT: return kTyTransmission | kTySpecular;
        case kBxNewWard: return kTyReflection | kTyGlossy;
        case kBxAshS: return kTyReflection | kTyGlossy;
        case kBxAshD: return kTyReflection | kTyDiffuse;
        default: return kTyReflection | kTyDiffuse;
    }
}

__device__ __forceinline__ int elem_size(uint8_t id) {
    switch (id) {
        case kBxSpecT: return 20;
        case kBxNewWard: case kBxAshS: return 16;
        default: return 12;
    }
}

// Component i of the BSDF with its textures evaluated (the BxDF part of
// BSDFAlloc, reflection.cl:230-341).  Unknown element ids decode as black
// diffuse.
static __device__ __noinline__ BxDF load_bx(const BSDF& f, uint32_t off) {
    BxDF b;
    if (off == 0xFFFF) {  // empty material: black diffuse
        b.id = kBxDiffuse;
        b.type = kTyReflection | kTyDiffuse;
        b.c0 = b.c1 = mk(0, 0, 0);
        b.a = 1.0f;
        b.b = 0.0f;
        b.fresnel = nullptr;
        return b;
    }
    const uint8_t* p = f.mat + off;
    b.id = p[0];
    b.type = elem_type(p[0]);
    b.fresnel = nullptr;
    b.a = b.b = 0.f;
    b.c1 = mk(0, 0, 0);
    switch (p[0]) {
        case kBxDiffuse: {  // DiffuseRElem {id, idx_R, idx_sigma}
            b.c0 = eval_color_texture(f.tex + ldb<uint32_t>(p + 4), f.uv);
            float sigma2 = eval_float_texture(f.tex + ldb<uint32_t>(p + 8), f.uv);
            sigma2 *= sigma2;
            b.a = 1.0f - (sigma2 / (2.0f * (sigma2 + 0.33f)));
            b.b = 0.45f * sigma2 / (sigma2 + 0.09f);
            break;
        }
        case kBxSpecR:  // SpecularRElem {id, idx_R, idx_Fresnel}
            b.c0 = eval_color_texture(f.tex + ldb<uint32_t>(p + 4), f.uv);
            b.fresnel = f.others + ldb<uint32_t>(p + 8);
            break;
        case kBxSpecT:  // SpecularTElem {id, idx_T, etaExt, etaInt, idx_Fresnel}
            b.c0 = eval_color_texture(f.tex + ldb<uint32_t>(p + 4), f.uv);
            b.a = ldb<float>(p + 8);
            b.b = ldb<float>(p + 12);
            b.fresnel = f.others + ldb<uint32_t>(p + 16);
            break;
        case kBxNewWard:  // NewWardElem {id, idx_R, idx_anisoX, idx_anisoY}
        case kBxAshS:     // AshikhminSElem {id, idx_Rs, idx_nu, idx_nv}
            b.c0 = eval_color_texture(f.tex + ldb<uint32_t>(p + 4), f.uv);
            b.a = eval_float_texture(f.tex + ldb<uint32_t>(p + 8), f.uv);
            b.b = eval_float_texture(f.tex + ldb<uint32_t>(p + 12), f.uv);
            break;
        case kBxAshD:  // AshikhminDElem {id, idx_Rs, idx_Rd}
            b.c0 = eval_color_texture(f.tex + ldb<uint32_t>(p + 8), f.uv);  // Rd
            b.c1 = eval_color_texture(f.tex + ldb<uint32_t>(p + 4), f.uv);  // Rs
            break;
        default:
            b.id = kBxDiffuse;
            b.c0 = mk(0, 0, 0);
            b.a = 1.0f;
            break;
    }
    return b;
}

template <typename T>
__device__ __forceinline__ T pick4(const T* a, uint32_t i) {
    return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

static __device__ __noinline__ f3 eval_fresnel(const uint8_t* fr, float cosi) {  // reflection.cl:345-390
    switch (fr[0]) {
        case 0:
            return mk(1, 1, 1);
        case 1: {
            const f3 eta = ldf3(fr + 16), k = ldf3(fr + 32);
            cosi = fabsf(cosi);
            const f3 tmp = (eta * eta + k * k) * cosi * cosi;
            const f3 one = mk(1, 1, 1);
            const f3 Rparl2 = (tmp - (2.0f * eta * cosi) + one) / (tmp + (2.0f * eta * cosi) + one);
            const f3 tmp_f = eta * eta + k * k;
            const f3 c2 = mk(cosi * cosi, cosi * cosi, cosi * cosi);
            const f3 Rperp2 = (tmp_f - (2.0f * eta * cosi) + c2) / (tmp_f + (2.0f * eta * cosi) + c2);
            return (Rparl2 + Rperp2) / 2.0f;
        }
        case 2: {
            cosi = clampf(cosi, -1.0f, 1.0f);
            const bool entering = cosi > 0.0f;
            float ei = ldb<float>(fr + 4), et = ldb<float>(fr + 8);
            if (!entering) {
                const float tmp = ei;
                ei = et;
                et = tmp;
            }
            const float sint = ei / et * sqrtf(fmaxf(0.0f, 1.0f - cosi * cosi));
            if (sint >= 1.0f) return mk(1, 1, 1);
            const float cost = sqrtf(fmaxf(0.0f, 1.0f - sint * sint));
            cosi = fabsf(cosi);
            const float Rparl = ((et * cosi) - (ei * cost)) / ((et * cosi) + (ei * cost));
            const float Rperp = ((ei * cosi) - (et * cost)) / ((ei * cosi) + (et * cost));
            const float v = Rparl * Rparl + Rperp * Rperp;
            return mk(v, v, v) / 2.0f;
        }
        default:
            return mk(0, 0, 0);
    }
}

__device__ __forceinline__ float sin_theta2(f3 v) { return fmaxf(1.0f - v.z * v.z, 0.0f); }
__device__ __forceinline__ float sin_theta(f3 v) { return sqrtf(sin_theta2(v)); }
__device__ __forceinline__ float cos_phi(f3 v) {
    const float s = sin_theta(v);
    if (s == 0.0f) return 1.0f;
    return clampf(v.x / s, -1.0f, 1.0f);
}
__device__ __forceinline__ float sin_phi(f3 v) {
    const float s = sin_theta(v);
    if (s == 0.0f) return 0.0f;
    return clampf(v.y / s, -1.0f, 1.0f);
}

static __device__ __noinline__ f3 bx_f(const BxDF& b, f3 vout, f3 vin) {  // fx, reflection.cl:500-583
    const f3 zero = mk(0, 0, 0);
    switch (b.id) {
        case kBxDiffuse: {
            if (vin.z * vout.z <= 0.0f) return zero;
            if (b.a == 1.0f) return b.c0 / kPi;
            const float sti = sin_theta(vin), sto = sin_theta(vout);
            float maxCos = 0.0f;
            if (sti > 1e-4f && sto > 1e-4f) {
                const float dcos = cos_phi(vin) * cos_phi(vout) + sin_phi(vin) * sin_phi(vout);
                maxCos = fmaxf(0.0f, dcos);
            }
            float sinAlpha, tanBeta;
            if (fabsf(vin.z) > fabsf(vout.z)) {
                sinAlpha = sto;
                tanBeta = sti / fabsf(vin.z);
            } else {
                sinAlpha = sti;
                tanBeta = sto / fabsf(vout.z);
            }
            return b.c0 / kPi * (b.a + b.b * maxCos * sinAlpha * tanBeta);
        }
        case kBxSpecR:
        case kBxSpecT:
            return zero;
        case kBxNewWard: {
            if (vin.z * vout.z <= 0.0f) return zero;
            const f3 h = normalize(vout + vin);
            const float hx = h.x / b.a, hy = h.y / b.b, dotHN = fabsf(h.z), dotHI = dot(h, vin);
            return b.c0 * expf(-(hx * hx + hy * hy) / (dotHN * dotHN)) /
                   (4 * kPi * b.a * b.b * dotHI * dotHI * dotHN * dotHN * dotHN * dotHN);
        }
        case kBxAshS: {
            if (vin.z * vout.z <= 0.0f) return zero;
            const f3 h = normalize(vout + vin);
            const float dotHV = dot(h, vout);
            const float e = (b.a * h.x * h.x + b.b * h.y * h.y) / (1 - h.z * h.z);
            const f3 fr = b.c0 + (mk(1, 1, 1) - b.c0) * powf(1.0f - dotHV, 5);
            return sqrtf((b.a + 1) * (b.b + 1)) / (8 * kPi) * powf(fabsf(h.z), e) /
                   (dotHV * fmaxf(fabsf(vout.z), fabsf(vin.z))) * fr;
        }
        case kBxAshD: {
            if (vin.z * vout.z <= 0.0f) return zero;
            return 28 * b.c0 / (23 * kPi) * (mk(1, 1, 1) - b.c1) * (1.0f - powf(1.0f - fabsf(vout.z) / 2, 5)) *
                   (1.0f - powf(1.0f - fabsf(vin.z) / 2, 5));
        }
        default:
            return zero;
    }
}

static __device__ __noinline__ float bx_pdf(const BxDF& b, f3 vout, f3 vin) {  // fx_pdf, reflection.cl:585-626
    switch (b.id) {
        case kBxDiffuse:
        case kBxAshD:
            return fabsf(vin.z) / kPi;
        case kBxNewWard: {
            if (vin.z * vout.z <= 0) return 0.0f;
            const f3 h = normalize(vout + vin);
            const float hx = h.x / b.a, hy = h.y / b.b, dotHN = fabsf(h.z), dotHI = dot(h, vin);
            const float num = expf(-(hx * hx + hy * hy) / (dotHN * dotHN));
            return num / (4 * kPi * b.a * b.b * dotHI * dotHN * dotHN * dotHN);
        }
        case kBxAshS: {
            if (vout.z * vin.z <= 0) return 0.0f;
            const f3 h = normalize(vout + vin);
            const float e = (b.a * h.x * h.x + b.b * h.y * h.y) / (1 - h.z * h.z);
            return sqrtf((b.a + 1) * (b.b + 1)) / (2 * kPi) * powf(fabsf(h.z), e) / (4 * dot(vout, h));
        }
        default:
            return 0.0f;
    }
}

// sample_fx, reflection.cl:393-498.  AshikhminS reads vin->z before it is
// written (reflection.cl:474); vout.z is used instead, as NewWard does at :447.
static __device__ __noinline__ f3 bx_sample(const BxDF& b, f3 vout, float u0, float u1, f3& vin, float& pdf) {
    const f3 zero = mk(0, 0, 0);
    switch (b.id) {
        case kBxDiffuse:
        case kBxAshD: {
            vin = cosine_hemisphere(u0, u1);
            if (vout.z < 0.0f) vin.z *= -1;
            pdf = fabsf(vin.z) / kPi;
            return bx_f(b, vout, vin);
        }
        case kBxSpecR: {
            vin = mk(-vout.x, -vout.y, vout.z);
            pdf = 1.0f;
            return b.c0 * eval_fresnel(b.fresnel, vout.z) / fabsf(vin.z);
        }
        case kBxSpecT: {
            const bool entering = vout.z > 0.0f;
            float ei = b.a, et = b.b;
            if (!entering) {
                ei = b.b;
                et = b.a;
            }
            const float sini2 = sin_theta2(vout);
            const float eta = ei / et;
            const float sint2 = eta * eta * sini2;
            if (sint2 >= 1.0f) return zero;  // pdf left unset, as in the reference
            float cost = sqrtf(fmaxf(0.0f, 1.0f - sint2));
            if (entering) cost = -cost;
            vin = mk(eta * -vout.x, eta * -vout.y, cost);
            pdf = 1.0f;
            const f3 f = eval_fresnel(b.fresnel, vout.z);
            return (mk(1, 1, 1) - f) * b.c0 / fabsf(vin.z);
        }
        case kBxNewWard: {
            const float quad = 2 * kPi * u1;
            const float phi_h = atan2f(b.b * sinf(quad), b.a * cosf(quad));
            const float cpa = cosf(phi_h) / b.a, spa = sinf(phi_h) / b.b;
            float theta_h = atanf(sqrtf(-logf(1 - u0) / (cpa * cpa + spa * spa)));
            if (vout.z < 0) theta_h = kPi - theta_h;
            const f3 h = mk(sinf(theta_h) * cosf(phi_h), sinf(theta_h) * sinf(phi_h), cosf(theta_h));
            vin = 2 * dot(vout, h) * h - vout;
            if (vin.z * vout.z <= 0) {
                pdf = 0.0f;
                return zero;
            }
            const float hx = h.x / b.a, hy = h.y / b.b, dotHN = fabsf(h.z), dotHI = dot(h, vin);
            const float num = expf(-(hx * hx + hy * hy) / (dotHN * dotHN));
            const float den = 4 * kPi * b.a * b.b * dotHI * dotHN * dotHN * dotHN;
            pdf = num / den;
            return b.c0 * (num / (den * dotHI * dotHN));
        }
        case kBxAshS: {
            const float quad = 2 * kPi * u1;
            const float phi_h = atan2f(sqrtf(b.a + 1) * sinf(quad), sqrtf(b.b + 1) * cosf(quad));
            const float cp = cosf(phi_h), sp = sinf(phi_h);
            float theta_h = acosf(powf(1 - u0, 1.0f / (b.a * cp * cp + b.b * sp * sp + 1)));
            if (vout.z < 0) theta_h = kPi - theta_h;
            const f3 h = mk(sinf(theta_h) * cosf(phi_h), sinf(theta_h) * sinf(phi_h), cosf(theta_h));
            vin = 2 * dot(vout, h) * h - vout;
            if (vout.z * vin.z <= 0) {
                pdf = 0.0f;
                return zero;
            }
            pdf = bx_pdf(b, vout, vin);
            return bx_f(b, vout, vin);
        }
        default:
            return zero;
    }
}

__device__ __forceinline__ bool bsdf_has_non_specular(const BSDF& f) {
    bool r = false;
#pragma unroll
    for (int i = 0; i < kMaxBxDFs; ++i)
        if (i < f.num && (f.type[i] & kTyNonSingular)) r = true;
    return r;
}

__device__ __forceinline__ bool match_type(uint8_t type, uint32_t mask) { return (type & mask) == type; }

// sample_fs, reflection.cl:629-677
__device__ __forceinline__ f3 bsdf_sample(const BSDF& f, f3 vout, float uc, float u0, float u1, f3& vin, float& pdf,
                          uint32_t& sampledType) {
    const f3 zero = mk(0, 0, 0);
    uint32_t flags = kTyAll;
    const uint32_t numMatches = (uint32_t)f.num;
    const f3 vl = world_to_local(f.s, f.t, f.n, vout);
    const uint32_t which = rand_uint(uc, (uint32_t)f.num);
    const BxDF b = load_bx(f, pick4(f.off, which));
    f3 vinl = zero;
    f3 ret = bx_sample(b, vl, u0, u1, vinl, pdf);
    if (pdf == 0.0f) {
        sampledType = 0;
        return zero;
    }
    sampledType = b.type;
    vin = local_to_world(f.s, f.t, f.n, vinl);
    if (!(b.type & kTySpecular) && numMatches > 1) {
#pragma unroll 1
        for (int i = 0; i < f.num; ++i)
            if ((uint32_t)i != which && match_type(f.type[i], flags))
                pdf += bx_pdf(load_bx(f, f.off[i]), vl, vinl);
    }
    pdf /= (float)numMatches;
    if (!(b.type & kTySpecular)) {
        ret = zero;
        if (dot(vin, f.ng) * dot(vout, f.ng) > 0) flags &= ~kTyTransmission;
        else flags &= ~kTyReflection;
#pragma unroll 1
        for (int i = 0; i < f.num; ++i)
            if (match_type(f.type[i], flags)) ret += bx_f(load_bx(f, f.off[i]), vl, vinl);
    }
    return ret;
}

// fs, reflection.cl:679-702
__device__ __forceinline__ f3 bsdf_f(const BSDF& f, f3 vout, f3 vin) {
    uint32_t flags = kTyAll;
    const f3 vl = world_to_local(f.s, f.t, f.n, vout), il = world_to_local(f.s, f.t, f.n, vin);
    f3 ret = mk(0, 0, 0);
    if (dot(vin, f.ng) * dot(vout, f.ng) > 0) flags &= ~kTyTransmission;
    else flags &= ~kTyReflection;
#pragma unroll 1
    for (int i = 0; i < f.num; ++i)
        if (match_type(f.type[i], flags)) ret += bx_f(load_bx(f, f.off[i]), vl, il);
    return ret;
}

// fs_pdf, reflection.cl:704-723
__device__ __forceinline__ float bsdf_pdf(const BSDF& f, f3 vout, f3 vin) {
    const f3 vl = world_to_local(f.s, f.t, f.n, vout), il = world_to_local(f.s, f.t, f.n, vin);
    float pdf = 0.0f;
#pragma unroll 1
    for (int i = 0; i < f.num; ++i)
        if (match_type(f.type[i], kTyAll)) pdf += bx_pdf(load_bx(f, f.off[i]), vl, il);
    return pdf / (uint32_t)f.num;
}

// ------------------------------------------------------------------- EDF
// light.cl:46-84, 295-440.  As for the BSDF, only the frame and the blob
// offsets of the emission components are kept; their textures are evaluated
// in Le.

struct EDF {
    bool env;
    int num;
    const uint8_t* prop;   // light property (materials blob)
    const uint8_t* tex;
    float2 uv;
    uint16_t off[kMaxBxDFs];
    f3 n, s, t, ng;
};

__device__ __forceinline__ f3 edf_component(const EDF& e, uint32_t off) {
    const uint8_t* p = e.prop + off;
    if (e.env)  // ImageBasedEnvLElem {id, idx_Le, multiplier, idx_Dist2D}
        return eval_color_texture(e.tex + ldb<uint32_t>(p + 4), e.uv) * ldb<float>(p + 8);
    return eval_color_texture(e.tex + ldb<uint32_t>(p + 4), e.uv);  // DiffuseLElem {id, idx_M}
}

__device__ __forceinline__ f3 edf_le(const EDF& e, f3 vout) {  // Le, light.cl:409-436
    f3 r = mk(0, 0, 0);
    if (!e.env) {
        const f3 vl = world_to_local(e.s, e.t, e.n, vout);
#pragma unroll
        for (int i = 0; i < kMaxBxDFs; ++i)
            if (i < e.num) r += vl.z > 0.0f ? edf_component(e, e.off[i]) / kPi : mk(0, 0, 0);
    } else {
#pragma unroll
        for (int i = 0; i < kMaxBxDFs; ++i)
            if (i < e.num) r += edf_component(e, e.off[i]);
    }
    return r;
}

__device__ __forceinline__ float edf_abs_cos(const EDF& e, f3 v) { return e.env ? 1.0f : fabsf(dot(e.n, v)); }

}  // namespace clr
