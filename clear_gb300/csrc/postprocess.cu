// Post-processing of the accumulated image: the reference's `scaling` and
// `toneMapping` kernels (OpenCL/post_processing.cl:20-26, 98-117, launched
// back to back by main.cpp:526-536) fused into one pass over the pixels.
//
// Per pixel: v = accum * (1 / spp); each channel saturates at 30; the
// luminance Y = 0.2989 r + 0.5866 g + 0.1144 b and the tone-mapping scale
// (1 - e^-Y) / Y are evaluated in double precision as the reference's
// double literals make them (then rounded to float); the channel value is
// 255 * (scale * v)^(1/2.2), clamped to [0, 255] and truncated to a byte.  The
// output is the reference's BMP pixel array: BGR, rows bottom-up, each row
// 3 * width + width % 4 bytes (BMPExporter.cpp:14-15); the row padding is
// written as zeros (the reference leaves it unset).  HBM-bound: 16 bytes read
// and 3 written per pixel.
#include "common.cuh"

namespace clr {

constexpr float kToneThreshold = 30.0f;  // post_processing.cl:70

__device__ __forceinline__ unsigned char tone_channel(float v, float scale) {
    const float p = powf(scale * v, 1.0f / 2.2f);
    float r = 255.0f * p;
    r = fminf(fmaxf(r, 0.0f), 255.0f);  // NaN becomes 0 (fmaxf returns the non-NaN operand)
    return (unsigned char)(unsigned int)r;
}

__global__ void __launch_bounds__(256) k_tonemap(const float4* __restrict__ accum, uint32_t width, uint32_t height,
                                                 float inv_spp, uint32_t byte_width, uint8_t* __restrict__ dst) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= width) return;
    const float4 a = accum[(size_t)width * y + x];
    // scaling
    const float v0 = a.x * inv_spp, v1 = a.y * inv_spp, v2 = a.z * inv_spp;
    // toneMapping
    const float s0 = v0 > kToneThreshold ? kToneThreshold : v0;
    const float s1 = v1 > kToneThreshold ? kToneThreshold : v1;
    const float s2 = v2 > kToneThreshold ? kToneThreshold : v2;
    const float Y = (float)(0.2989 * (double)s0 + 0.5866 * (double)s1 + 0.1144 * (double)s2);
    float scaleTM = (float)((1.0 - (double)expf(-Y)) / (double)Y);
    if (Y == 0.0f) scaleTM = 1.0f;
    uint8_t* d = dst + (size_t)byte_width * (height - 1 - y) + 3u * x;
    d[0] = tone_channel(s2, scaleTM);
    d[1] = tone_channel(s1, scaleTM);
    d[2] = tone_channel(s0, scaleTM);
    if (x == width - 1)
        for (uint32_t k = 3u * width; k < byte_width; ++k) dst[(size_t)byte_width * (height - 1 - y) + k] = 0;
}

}  // namespace clr

using namespace clr;

extern "C" int clr_postprocess_ldr(const float* accum, uint32_t width, uint32_t height, uint32_t spp, uint8_t* bgr,
                                   void* stream) {
    if (width == 0 || height == 0) return CLR_OK;
    if (!accum || !bgr) return clr_set_error(CLR_EINVAL, "clr_postprocess_ldr: NULL buffer");
    if (spp == 0) return clr_set_error(CLR_EINVAL, "clr_postprocess_ldr: spp must be at least 1");
    if (reinterpret_cast<uintptr_t>(accum) & 15u)
        return clr_set_error(CLR_EINVAL, "clr_postprocess_ldr: accum must be 16-byte aligned");
    if (height > 65535u) return clr_set_error(CLR_EINVAL, "clr_postprocess_ldr: height %u above 65535", height);
    const uint32_t byte_width = 3u * width + width % 4u;
    const float inv_spp = 1.0f / (float)spp;
    const dim3 grid(div_up(width, 256u), height);
    k_tonemap<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(reinterpret_cast<const float4*>(accum), width,
                                                                  height, inv_spp, byte_width, bgr);
    CLR_LAUNCH_CHECK("k_tonemap");
    return CLR_OK;
}
