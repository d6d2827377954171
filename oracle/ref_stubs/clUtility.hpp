/* Stand-in for CommonSources/clUtility.hpp when the reference's CPU BVH
 * builder (OpenCL_PathTracer/BVH.hpp) is compiled for the oracle: it needs
 * only cl_float3 and the component-wise min/max helpers, which use
 * std::min/std::max in the reference (CommonSources/clUtility.cpp:544-552). */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
typedef union { struct { float s0, s1, s2, s3; }; float s[4]; } cl_float3;
namespace CLUtil {
inline cl_float3 minCLfloat3(const cl_float3& a, const cl_float3& b) {
    cl_float3 r; r.s0 = std::min(a.s0, b.s0); r.s1 = std::min(a.s1, b.s1); r.s2 = std::min(a.s2, b.s2); r.s3 = 0; return r;
}
inline cl_float3 maxCLfloat3(const cl_float3& a, const cl_float3& b) {
    cl_float3 r; r.s0 = std::max(a.s0, b.s0); r.s1 = std::max(a.s1, b.s1); r.s2 = std::max(a.s2, b.s2); r.s3 = 0; return r;
}
}
