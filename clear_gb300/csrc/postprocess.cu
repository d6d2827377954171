// Post-processing of the accumulated image: the reference's `scaling` and
// `toneMapping` kernels (OpenCL/post_processing.cl:20-26, 98-117, launched
// back to back by main.cpp:526-536) fused into one pass over the pixels.
//
// Per pixel: v = accum * (1 / spp); each channel saturates at 30; the
// luminance Y = 0.2989 r + 0.5866 g + 0.1144 b and the tone-mapping scale
// (1 - e^-Y) / Y are evaluated in double precision as the reference's double
// literals make them (then rounded to float); the channel value is
// 255 * (scale * v)^(1/2.2), clamped to [0, 255] and truncated to a byte.  The
// output is the reference's BMP pixel array: BGR, rows bottom-up, each row
// 3 * width + width % 4 bytes (BMPExporter.cpp:14-15); the row padding is
// written as zeros (the reference leaves it unset).  HBM-bound: 16 bytes read
// and 3 written per pixel.
//
// Double arithmetic is slow on this part (its FP64 rate is a small fraction of
// its FP32 rate), so Y and the scale are first evaluated in float-float
// arithmetic -- error-free products with fmaf and error-free sums (Dekker,
// Knuth) -- with a relative error below 2^-42 of the exact value.  The double
// evaluation is within 2^-50 of the exact value, so when the float-float
// result lies further than 2^-40 (relative) from a midpoint between two
// floats, both round to the same float and the float-float result is the
// double expression's.  Otherwise (about one value in 2^16, and every NaN,
// negative or tiny input) the double expression itself is evaluated.  The
// result is therefore exactly that of the double expression.
#include "common.cuh"

namespace clr {

constexpr float kToneThreshold = 30.0f;  // post_processing.cl:70

// The double constants as float hi + lo (hi = the nearest float, lo the
// nearest float to the remainder): c - hi - lo is below 2^-48 c.
constexpr double kC0 = 0.2989, kC1 = 0.5866, kC2 = 0.1144;
constexpr float kC0h = (float)kC0, kC1h = (float)kC1, kC2h = (float)kC2;
constexpr float kC0l = (float)(kC0 - (double)kC0h), kC1l = (float)(kC1 - (double)kC1h),
                kC2l = (float)(kC2 - (double)kC2h);

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// With hi = RN(hi + lo): every value within 2^-41 |hi| of hi + lo rounds to
// hi when lo stays clear of the midpoint on its side by 2^-40 |hi|.  The
// midpoint is half an ulp away, a quarter of hi's ulp when hi is a power of
// two and lo points towards zero (the spacing halves below a power of two).
__device__ __forceinline__ bool rounds_clear(float hi, float lo) {
    const uint32_t b = __float_as_uint(hi);
    const uint32_t e = b & 0x7f800000u;
    if (e < (64u << 23) || e >= (254u << 23)) return false;  // near the subnormal or overflow range
    uint32_t half_e = e - (24u << 23);
    if ((b & 0x007fffffu) == 0 && ((__float_as_uint(lo) ^ b) & 0x80000000u)) half_e -= 1u << 23;
    const float half_ulp = __uint_as_float(half_e);
    const float margin = __uint_as_float(e - (40u << 23));
    return fabsf(lo) < __fsub_rn(half_ulp, margin);
}

// Y and the tone-mapping scale of one pixel, exactly as
//   Y = (float)(0.2989 * (double)s0 + 0.5866 * (double)s1 + 0.1144 * (double)s2)
//   scale = Y == 0 ? 1 : (float)((1.0 - (double)expf(-Y)) / (double)Y).
__device__ __forceinline__ void tone_scale(float s0, float s1, float s2, float& Y, float& e, float& scale) {
    bool fast = s0 >= 0.0f && s1 >= 0.0f && s2 >= 0.0f;  // false for NaN
    if (fast) {
        // p_i = s_i (c_ih + c_il) = h_i + e_i + l_i, h_i + e_i exact
        const float h0 = __fmul_rn(s0, kC0h), h1 = __fmul_rn(s1, kC1h), h2 = __fmul_rn(s2, kC2h);
        const float e0 = __fmaf_rn(s0, kC0h, -h0), e1 = __fmaf_rn(s1, kC1h, -h1), e2 = __fmaf_rn(s2, kC2h, -h2);
        const float l0 = __fmul_rn(s0, kC0l), l1 = __fmul_rn(s1, kC1l), l2 = __fmul_rn(s2, kC2l);
        float H, t0, t1;
        two_sum(h0, h1, H, t0);
        two_sum(H, h2, H, t1);
        const float L = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), __fadd_rn(__fadd_rn(e0, e1), e2)),
                                  __fadd_rn(__fadd_rn(l0, l1), l2));
        float Yh, Yl;
        fast_two_sum(H, L, Yh, Yl);
        fast = Yh == 0.0f ? (H == 0.0f && L == 0.0f) : rounds_clear(Yh, Yl);
        Y = Yh;
    }
    if (!fast) Y = (float)(kC0 * (double)s0 + kC1 * (double)s1 + kC2 * (double)s2);
    e = expf(-Y);
    if (Y == 0.0f) {
        scale = 1.0f;
        return;
    }
    bool fastq = fast && Y > 0.0f;
    if (fastq) {
        // N = 1 - e exactly (float-float); q = N / Y = qh + ql
        float Nh, Nl;
        two_sum(1.0f, -e, Nh, Nl);
        const float qh = __fdiv_rn(Nh, Y);
        const float r = __fmaf_rn(-qh, Y, Nh);  // exact remainder of a correctly rounded quotient
        const float ql = __fdiv_rn(__fadd_rn(r, Nl), Y);
        float Qh, Ql;
        fast_two_sum(qh, ql, Qh, Ql);
        fastq = rounds_clear(Qh, Ql);
        scale = Qh;
    }
    if (!fastq) scale = (float)((1.0 - (double)e) / (double)Y);
}

__device__ __forceinline__ unsigned char tone_channel(float v, float scale) {
    const float p = powf(scale * v, 1.0f / 2.2f);
    float r = 255.0f * p;
    r = fminf(fmaxf(r, 0.0f), 255.0f);  // NaN becomes 0 (fmaxf returns the non-NaN operand)
    return (unsigned char)(unsigned int)r;
}

// kScales: write {Y, e^-Y, scale, 0} per pixel to `scales` instead of the
// bytes (the parity check of the precision rules above).
template <bool kScales>
__global__ void __launch_bounds__(256) k_tonemap(const float4* __restrict__ accum, uint32_t width, uint32_t height,
                                                 float inv_spp, uint32_t byte_width, uint8_t* __restrict__ dst,
                                                 float4* __restrict__ scales) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= width) return;
    const float4 a = accum[(size_t)width * y + x];
    // scaling
    const float v0 = a.x * inv_spp, v1 = a.y * inv_spp, v2 = a.z * inv_spp;
    // toneMapping
    const float s0 = v0 > kToneThreshold ? kToneThreshold : v0;
    const float s1 = v1 > kToneThreshold ? kToneThreshold : v1;
    const float s2 = v2 > kToneThreshold ? kToneThreshold : v2;
    float Y, e, scaleTM;
    tone_scale(s0, s1, s2, Y, e, scaleTM);
    if (kScales) {
        scales[(size_t)width * y + x] = make_float4(Y, e, scaleTM, 0.0f);
        return;
    }
    uint8_t* d = dst + (size_t)byte_width * (height - 1 - y) + 3u * x;
    d[0] = tone_channel(s2, scaleTM);
    d[1] = tone_channel(s1, scaleTM);
    d[2] = tone_channel(s0, scaleTM);
    if (x == width - 1)
        for (uint32_t k = 3u * width; k < byte_width; ++k) dst[(size_t)byte_width * (height - 1 - y) + k] = 0;
}

int launch_tonemap(const float* accum, uint32_t width, uint32_t height, uint32_t spp, uint8_t* bgr, float* scales,
                   void* stream, const char* fn) {
    if (width == 0 || height == 0) return CLR_OK;
    if (!accum || (!bgr && !scales)) return clr_set_error(CLR_EINVAL, "%s: NULL buffer", fn);
    if (spp == 0) return clr_set_error(CLR_EINVAL, "%s: spp must be at least 1", fn);
    if (reinterpret_cast<uintptr_t>(accum) & 15u) return clr_set_error(CLR_EINVAL, "%s: accum must be 16-byte aligned", fn);
    if (scales && (reinterpret_cast<uintptr_t>(scales) & 15u))
        return clr_set_error(CLR_EINVAL, "%s: scales must be 16-byte aligned", fn);
    if (height > 65535u) return clr_set_error(CLR_EINVAL, "%s: height %u above 65535", fn, height);
    const uint32_t byte_width = 3u * width + width % 4u;
    const float inv_spp = 1.0f / (float)spp;
    const dim3 grid(div_up(width, 256u), height);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (scales) {
        k_tonemap<true><<<grid, 256, 0, st>>>(reinterpret_cast<const float4*>(accum), width, height, inv_spp,
                                              byte_width, nullptr, reinterpret_cast<float4*>(scales));
    } else {
        k_tonemap<false><<<grid, 256, 0, st>>>(reinterpret_cast<const float4*>(accum), width, height, inv_spp,
                                               byte_width, bgr, nullptr);
    }
    CLR_LAUNCH_CHECK("k_tonemap");
    return CLR_OK;
}

}  // namespace clr

using namespace clr;

extern "C" int clr_postprocess_ldr(const float* accum, uint32_t width, uint32_t height, uint32_t spp, uint8_t* bgr,
                                   void* stream) {
    return launch_tonemap(accum, width, height, spp, bgr, nullptr, stream, "clr_postprocess_ldr");
}

extern "C" int clr_postprocess_scales(const float* accum, uint32_t width, uint32_t height, uint32_t spp,
                                      float* scales, void* stream) {
    return launch_tonemap(accum, width, height, spp, nullptr, scales, stream, "clr_postprocess_scales");
}
