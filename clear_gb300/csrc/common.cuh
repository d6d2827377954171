// Shared device/host helpers for the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "clear_cuda.h"

// ----------------------------------------------------------------- errors

// Thread-local last-error text (capi.cu) and a setter used by entry points.
int clr_set_error(int code, const char* fmt, ...);

#define CLR_CUDA_TRY(expr)                                                              \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return clr_set_error(CLR_ECUDA, "%s failed: %s", #expr, cudaGetErrorString(e_)); \
    } while (0)

#define CLR_LAUNCH_CHECK(name)                                                          \
    do {                                                                                \
        cudaError_t e_ = cudaGetLastError();                                            \
        if (e_ != cudaSuccess)                                                          \
            return clr_set_error(CLR_ECUDA, "launch of %s failed: %s", name, cudaGetErrorString(e_)); \
    } while (0)

// Device error word, CLR_DEVERR_* bits.  Without relocatable device code each
// translation unit has its own copy; CLR_DEFINE_STATUS_READER(tu) gives the
// host a reader for it, and clr_device_status() (capi.cu) ORs them together.
static __device__ unsigned int g_clr_dev_error = 0;

#define CLR_DEFINE_STATUS_READER(tu)                                                 \
    cudaError_t clr_status_##tu(unsigned int* v, int clear) {                       \
        cudaError_t e = cudaMemcpyFromSymbol(v, g_clr_dev_error, sizeof(unsigned int)); \
        if (e != cudaSuccess || !clear) return e;                                    \
        const unsigned int z = 0;                                                    \
        return cudaMemcpyToSymbol(g_clr_dev_error, &z, sizeof(z));                   \
    }

__device__ __forceinline__ void clr_raise(unsigned int bit) { atomicOr(&g_clr_dev_error, bit); }

// --------------------------------------------------- exact float arithmetic
//
// The reference's float expressions are evaluated without contraction; these
// wrappers keep nvcc from fusing a*b+c into one FMA so results round exactly
// as the reference's (and the oracle's) separate operations do.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// OpenCL dot(a,b) as the reference's CPU equivalent evaluates it:
// (a.x*b.x + a.y*b.y) + a.z*b.z, each op rounded.
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return fadd(fadd(fmul(ax, bx), fmul(ay, by)), fmul(az, bz));
}

// ------------------------------------------------------------ relaxed atomics

__device__ __forceinline__ unsigned int ld_relaxed_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_gpu(unsigned int* p, unsigned int v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Order-preserving float <-> uint map: a < b  <=>  enc(a) < enc(b).
__device__ __forceinline__ unsigned int float_to_ordered(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(unsigned int u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

namespace clr {
// Child reference flag: bit 31 set = leaf index, clear = internal node index.
constexpr uint32_t kLeafBit = 0x80000000u;
}  // namespace clr

static inline unsigned int div_up(unsigned int a, unsigned int b) { return (a + b - 1) / b; }

// Streaming multiprocessors of the current device (capi.cu), queried once per
// device; grids that fill the GPU once are sized from it.
int clr_sm_count();
