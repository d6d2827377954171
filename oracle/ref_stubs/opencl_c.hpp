/* OpenCL C on the host, for compiling the reference's own LBVH kernels
 * (OpenCL_PathTracer/OpenCL/lbvh_construction.cl, CommonSources/OpenCL/
 * generic_kernels.cl) as C++ and running them on the CPU
 * (oracle/ref_lbvh_cl.cpp).  TEST INFRASTRUCTURE ONLY.
 *
 * Written from the OpenCL C 1.2 specification for the subset those kernels
 * use: the address-space qualifiers (empty; the build turns the kernels'
 * work-group `local` declarations into `static`, which is the same storage
 * when work-groups run one at a time), the 3-component vector types with 16-
 * byte size and alignment, their component-wise operators with scalar
 * widening, clz / min / max / fmin / fmax, convert_uint3_rtz (round toward
 * zero; NaN and negative inputs, undefined in OpenCL, give 0 as in the
 * oracle's restatement), convert_uchar3, as_uint / as_float, atomic_inc /
 * atomic_cmpxchg, the work-item functions and barrier(), which yields to the
 * next work-item of the group (oracle/ref_lbvh_cl.cpp runs a group's
 * work-items as coroutines). */
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
struct Ids {
    size_t gid, lid, grp, ngrp, lsize, gsize, goff;
};
extern Ids* g_cur;      // the running work-item's ids
void barrier_yield();   // suspends the running work-item until the group reaches the barrier
}  // namespace clshim

inline size_t get_global_id(uint) { return clshim::g_cur->gid; }
inline size_t get_local_id(uint) { return clshim::g_cur->lid; }
inline size_t get_group_id(uint) { return clshim::g_cur->grp; }
inline size_t get_num_groups(uint) { return clshim::g_cur->ngrp; }
inline size_t get_local_size(uint) { return clshim::g_cur->lsize; }
inline size_t get_global_size(uint) { return clshim::g_cur->gsize; }
inline size_t get_global_offset(uint) { return clshim::g_cur->goff; }
inline void barrier(int) { clshim::barrier_yield(); }

// ------------------------------------------------------------ vector types
struct alignas(16) float3 {
    float x, y, z, w;
    float3() : x(0), y(0), z(0), w(0) {}
    float3(float v) : x(v), y(v), z(v), w(0) {}  // (float3)(s): every component s
    float3(float a, float b, float c) : x(a), y(b), z(c), w(0) {}
};
inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
// a scalar operand is converted to the element type first (OpenCL 6.2.6)
inline float3 operator*(float3 a, float s) { return a * float3(s); }
inline float3 operator*(float3 a, uint s) { return a * float3((float)s); }
inline float3 fmin(float3 a, float3 b) { return float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
inline float3 fmax(float3 a, float3 b) { return float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
inline float fmin(float a, float b) { return fminf(a, b); }
inline float fmax(float a, float b) { return fmaxf(a, b); }

struct alignas(16) uint3 {
    uint x, y, z, w;
    uint3() : x(0), y(0), z(0), w(0) {}
    uint3(uint v) : x(v), y(v), z(v), w(0) {}
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c), w(0) {}
};
inline uint3 operator^(uint3 a, uint3 b) { return uint3(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z); }
inline uint3 operator>>(uint3 a, uint s) { return uint3(a.x >> s, a.y >> s, a.z >> s); }
inline uint3 operator&(uint3 a, uint s) { return uint3(a.x & s, a.y & s, a.z & s); }
inline uint3 operator-(uint3 a, uint s) { return uint3(a.x - s, a.y - s, a.z - s); }

struct uchar3 {
    uchar x, y, z, w;
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
inline uchar3 convert_uchar3(uint3 v) { return uchar3{(uchar)v.x, (uchar)v.y, (uchar)v.z, 0}; }

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
