/* OpenCL C on the host, for compiling the reference's own LBVH and
 * post-processing kernels (OpenCL_PathTracer/OpenCL/lbvh_construction.cl,
 * post_processing.cl, CommonSources/OpenCL/generic_kernels.cl) as C++ and
 * running them on the CPU (oracle/ref_lbvh_cl.cpp, ref_post_cl.cpp).  TEST
 * INFRASTRUCTURE ONLY.
 *
 * Written from the OpenCL C 1.2 specification for the subset those kernels
 * use: the address-space qualifiers (empty; the build turns the kernels'
 * work-group `local` declarations into `static`, which is the same storage
 * when work-groups run one at a time), the 3-component vector types with 16-
 * byte size and alignment, their component-wise operators with scalar
 * widening, clz / min / max / fmin / fmax, convert_uint3_rtz (round toward
 * zero; NaN and negative inputs, undefined in OpenCL, give 0 as in the
 * oracle's restatement), convert_uchar3(_rtz), as_uint / as_float, exp / pow
 * / clamp, atomic_inc / atomic_cmpxchg, the work-item functions and barrier(),
 * which yields to the next work-item of the group (oracle/ref_cl_exec.cpp
 * runs a group's work-items as coroutines).  Vector literals `(T)(a, b, c)`
 * reach the compiler as `T(a, b, c)` (oracle/build_oracle.py). */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

typedef uint8_t uchar;
typedef uint16_t ushort;
typedef uint32_t uint;
typedef uint64_t ulong;

#define kernel extern "C"
#define global
#define local
#define constant const
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

// ------------------------------------------------------------ work-items
namespace clshim {
struct Ids {  // per dimension 0, 1 (offsets are always 0)
    size_t gid[2], lid[2], grp[2], ngrp[2], lsize[2], gsize[2];
};
extern Ids* g_cur;      // the running work-item's ids
void barrier_yield();   // suspends the running work-item until the group reaches the barrier
// 1-D NDRange of global_size items in groups of local_size (oracle/ref_cl_exec.cpp)
void launch(size_t global_size, size_t local_size, bool barriers, void (*body)(void*), void* arg);
// 2-D NDRange without barriers, one work-item per group
void launch2d(size_t gx, size_t gy, void (*body)(void*), void* arg);
}  // namespace clshim

inline size_t get_global_id(uint d) { return clshim::g_cur->gid[d]; }
inline size_t get_local_id(uint d) { return clshim::g_cur->lid[d]; }
inline size_t get_group_id(uint d) { return clshim::g_cur->grp[d]; }
inline size_t get_num_groups(uint d) { return clshim::g_cur->ngrp[d]; }
inline size_t get_local_size(uint d) { return clshim::g_cur->lsize[d]; }
inline size_t get_global_size(uint d) { return clshim::g_cur->gsize[d]; }
inline size_t get_global_offset(uint) { return 0; }
inline void barrier(int) { clshim::barrier_yield(); }

// ------------------------------------------------------------ vector types
// components by letter (x, y, z, w) or number (s0 .. s3)
struct alignas(16) float3 {
    union {
        struct { float x, y, z, w; };
        struct { float s0, s1, s2, s3; };
    };
    float3() { x = y = z = w = 0.0f; }
    float3(float v) { x = y = z = v; w = 0.0f; }  // (float3)(s): every component s
    float3(float a, float b, float c) { x = a; y = b; z = c; w = 0.0f; }
};
inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
// a scalar operand is converted to the element type first (OpenCL 6.2.6)
inline float3 operator*(float3 a, float s) { return a * float3(s); }
inline float3 operator*(float s, float3 a) { return float3(s) * a; }
inline float3 operator*(float3 a, uint s) { return a * float3((float)s); }
inline float3 fmin(float3 a, float3 b) { return float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
inline float3 fmax(float3 a, float3 b) { return float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
inline float fmin(float a, float b) { return fminf(a, b); }
inline float fmax(float a, float b) { return fmaxf(a, b); }
// float arguments stay in float, as the OpenCL built-ins (the C library's
// expf / powf)
inline float exp(float x) { return expf(x); }
inline float pow(float x, float y) { return powf(x, y); }
inline float3 pow(float3 a, float y) { return float3(powf(a.x, y), powf(a.y, y), powf(a.z, y)); }
// clamp(x, lo, hi) = fmin(fmax(x, lo), hi) for floats
inline float3 clamp(float3 a, float lo, float hi) {
    return float3(fminf(fmaxf(a.x, lo), hi), fminf(fmaxf(a.y, lo), hi), fminf(fmaxf(a.z, lo), hi));
}
inline int clamp(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

struct alignas(16) uint3 {
    union {
        struct { uint x, y, z, w; };
        struct { uint s0, s1, s2, s3; };
    };
    uint3() { x = y = z = w = 0u; }
    uint3(uint v) { x = y = z = v; w = 0u; }
    uint3(uint a, uint b, uint c) { x = a; y = b; z = c; w = 0u; }
};
inline uint3 operator^(uint3 a, uint3 b) { return uint3(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z); }
inline uint3 operator>>(uint3 a, uint s) { return uint3(a.x >> s, a.y >> s, a.z >> s); }
inline uint3 operator&(uint3 a, uint s) { return uint3(a.x & s, a.y & s, a.z & s); }
inline uint3 operator-(uint3 a, uint s) { return uint3(a.x - s, a.y - s, a.z - s); }

struct uchar3 {
    union {
        struct { uchar x, y, z, w; };
        struct { uchar s0, s1, s2, s3; };
    };
};

inline uint clz(uint v) { return v ? (uint)__builtin_clz(v) : 32u; }
inline int clz(int v) { return (int)clz((uint)v); }
inline uint3 clz(uint3 v) { return uint3(clz(v.x), clz(v.y), clz(v.z)); }

template <typename T>
inline T min(T a, T b) { return b < a ? b : a; }
template <typename T>
inline T max(T a, T b) { return a < b ? b : a; }
inline uint3 min(uint3 a, uint s) { return uint3(min(a.x, s), min(a.y, s), min(a.z, s)); }

inline uint convert_uint_rtz(float f) {
    if (!(f > 0.0f)) return 0u;  // NaN, zero, negative
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint)f;  // C conversion truncates toward zero
}
inline uint3 convert_uint3_rtz(float3 v) {
    return uint3(convert_uint_rtz(v.x), convert_uint_rtz(v.y), convert_uint_rtz(v.z));
}
inline uchar3 convert_uchar3(uint3 v) {
    uchar3 r;
    r.x = (uchar)v.x; r.y = (uchar)v.y; r.z = (uchar)v.z; r.w = 0;
    return r;
}
// round toward zero; used on values already clamped to [0, 255]
inline uchar3 convert_uchar3_rtz(float3 v) {
    uchar3 r;
    r.x = (uchar)(uint)v.x; r.y = (uchar)(uint)v.y; r.z = (uchar)(uint)v.z; r.w = 0;
    return r;
}

inline uint as_uint(float f) {
    uint u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float as_float(uint u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// work-items of a group run one at a time on one host thread: a plain
// read-modify-write is atomic with respect to them
inline uint atomic_inc(volatile uint* p) {
    const uint old = *p;
    *p = old + 1u;
    return old;
}
inline uint atomic_cmpxchg(volatile uint* p, uint cmp, uint val) {
    const uint old = *p;
    if (old == cmp) *p = val;
    return old;
}
