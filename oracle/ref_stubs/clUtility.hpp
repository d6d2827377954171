/* Stand-in for CommonSources/clUtility.hpp when the reference's CPU code is
 * compiled for the oracle.  The BVH builder (OpenCL_PathTracer/BVH.hpp) needs
 * cl_float3 and the component-wise min/max helpers, which use std::min /
 * std::max in the reference (CommonSources/clUtility.cpp:544-552); the scene
 * encoders (CreateFunctions.cpp, Scene.h) and the .obj loader
 * (ModelLoader.cpp) need the OpenCL scalar/vector typedefs and the three
 * blob helpers, which behave as CommonSources/clUtility.cpp:554-571 does:
 * pad the byte vector with zeros to the alignment, then append. */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
typedef float cl_float;
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint16_t cl_ushort;
typedef uint8_t cl_uchar;
typedef union alignas(16) { struct { float s0, s1, s2, s3; }; float s[4]; } cl_float3;  // cl_float4 layout
typedef union { struct { float s0, s1; }; float s[2]; } cl_float2;
namespace CLUtil {
inline cl_float3 minCLfloat3(const cl_float3& a, const cl_float3& b) {
    cl_float3 r; r.s0 = std::min(a.s0, b.s0); r.s1 = std::min(a.s1, b.s1); r.s2 = std::min(a.s2, b.s2); r.s3 = 0; return r;
}
inline cl_float3 maxCLfloat3(const cl_float3& a, const cl_float3& b) {
    cl_float3 r; r.s0 = std::max(a.s0, b.s0); r.s1 = std::max(a.s1, b.s1); r.s2 = std::max(a.s2, b.s2); r.s3 = 0; return r;
}
inline size_t padding_to(size_t size, uint32_t alignment) {
    const size_t a = alignment ? alignment : 1;
    return (a - size % a) % a;
}
inline uint64_t align(std::vector<uint8_t>* vec, uint32_t alignment) {
    vec->resize(vec->size() + padding_to(vec->size(), alignment), 0);
    return vec->size();
}
inline uint64_t fillZerosAligned(std::vector<uint8_t>* dest, uint32_t bytes, uint32_t alignment) {
    const uint64_t at = align(dest, alignment);
    dest->resize(at + bytes, 0);
    return at;
}
inline uint64_t addDataAligned(std::vector<uint8_t>* dest, const void* data, size_t bytes, uint32_t alignment) {
    const uint64_t at = fillZerosAligned(dest, (uint32_t)bytes, alignment);
    if (bytes) std::memcpy(dest->data() + at, data, bytes);
    return at;
}
template <typename T>
uint64_t addDataAligned(std::vector<uint8_t>* dest, const T& data, uint32_t alignment = sizeof(T)) {
    return addDataAligned(dest, &data, sizeof(T), alignment);
}
}  // namespace CLUtil
