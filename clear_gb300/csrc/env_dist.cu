// Importance distribution of the image-based environment light, built on the
// device: createContinuousConsts2D_H_FromImageTexture
// (OpenCL_PathTracer/CreateFunctions.cpp:246-349) for one stratum per texel,
// recomputed in place whenever the environment's texels change (adjoint
// optimisation steps, many scenes) without a round trip through the host.
//
// Layout (read from the structure's own headers in the `others` blob):
// ContinuousConsts2D_H {type, offsetChildren, ContinuousConsts1D parent};
// ContinuousConsts1D {type, numValues, start, end, widthStratum, offsetPDF,
// offsetCDF} for the parent (rows) and each child (the texels of a row);
// distribution.cl:85-129 samples it.
//
// Row i (one thread): pdf_j = L * w_i, where L is the reference's
// averageLuminance of a one-texel stratum (CreateFunctions.cpp:159-244): the
// texel's luminance l = 0.2126 r + 0.7152 g + 0.0722 b, in float, added once
// per corner of the stratum, ((l + l) + l) + l, over an area of 1; w_i is the
// row weight, by default the zenith correction cos(pi (0.5 - (i + 0.5) / h))
// with the device cosf (the host passes the C library's for bit-exactness
// with the host encoder); cdf_{j+1} = cdf_j +
// pdf_j * (1 / width) accumulated left to right as the reference's loop does,
// both normalised by the row's mass cdf_w, which becomes the parent's pdf_i;
// then the parent's cdf over rows, normalised the same way (one thread).  The
// running sums are sequential on purpose: their rounding is the reference's.
#include <cuda_fp16.h>

#include "common.cuh"

CLR_DEFINE_STATUS_READER(env_dist)

namespace clr {

constexpr uint32_t kDevErrInput = CLR_DEVERR_INPUT;

struct Cc1d {  // ContinuousConsts1D as laid out in the blob
    uint32_t num;
    float width;
    float* pdf;
    float* cdf;
};

__device__ __forceinline__ Cc1d read_cc1d(uint8_t* p) {
    Cc1d c;
    c.num = *reinterpret_cast<const uint32_t*>(p + 4);
    c.width = *reinterpret_cast<const float*>(p + 16);
    c.pdf = reinterpret_cast<float*>(p + *reinterpret_cast<const int32_t*>(p + 20));
    c.cdf = reinterpret_cast<float*>(p + *reinterpret_cast<const int32_t*>(p + 24));
    return c;
}

__global__ void __launch_bounds__(128) k_env_rows(uint8_t* __restrict__ others, uint32_t dist_off,
                                                  const uint8_t* __restrict__ textures, uint32_t tex_off,
                                                  const float* __restrict__ row_weight, uint32_t rows) {
    uint8_t* head = others + dist_off;
    const Cc1d parent = read_cc1d(head + 8);
    const uint32_t h = parent.num;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= h) return;
    const uint8_t* tex = textures + tex_off;
    const uint32_t tw = *reinterpret_cast<const uint32_t*>(tex + 4), th = *reinterpret_cast<const uint32_t*>(tex + 8);
    uint8_t* child_p = head + *reinterpret_cast<const int32_t*>(head + 4) + 28u * i;
    const Cc1d row = read_cc1d(child_p);
    // a ContinuousConsts2D_H with one stratum per texel of an RGBA16F image
    if (head[0] != 2 || tex[0] != 3 || row.num != tw || h != th || h != rows) {
        clr_raise(kDevErrInput);
        return;
    }
    const __half* texel = reinterpret_cast<const __half*>(tex + *reinterpret_cast<const int32_t*>(tex + 12)) +
                          4ull * tw * i;
    float corr;
    if (row_weight) {
        corr = row_weight[i];
    } else {
        const float a = __fsub_rn(0.5f, __fdiv_rn(__fadd_rn((float)i, 0.5f), (float)h));
        corr = cosf((float)(3.14159265358979323846 * (double)a));
    }
    const uint32_t w = row.num;
    const float wc = row.width;
    float c = 0.0f;
    row.cdf[0] = 0.0f;
    for (uint32_t j = 0; j < w; ++j) {
        const float r = __half2float(texel[4 * j]), g = __half2float(texel[4 * j + 1]), b = __half2float(texel[4 * j + 2]);
        const float lum = __fadd_rn(__fadd_rn(__fmul_rn(0.2126f, r), __fmul_rn(0.7152f, g)), __fmul_rn(0.0722f, b));
        const float l4 = __fadd_rn(__fadd_rn(__fadd_rn(lum, lum), lum), lum);
        const float pdf = __fmul_rn(l4, corr);
        row.pdf[j] = pdf;
        c = __fadd_rn(c, __fmul_rn(pdf, wc));
        row.cdf[j + 1] = c;
    }
    const float mass = c;
    const float norm = mass > 0.0f ? __fdiv_rn(1.0f, mass) : 0.0f;
    for (uint32_t j = 0; j < w; ++j) {
        row.pdf[j] = __fmul_rn(row.pdf[j], norm);
        row.cdf[j + 1] = __fmul_rn(row.cdf[j + 1], norm);
    }
    parent.pdf[i] = mass;
}

__global__ void k_env_parent(uint8_t* __restrict__ others, uint32_t dist_off) {
    const Cc1d parent = read_cc1d(others + dist_off + 8);
    const uint32_t h = parent.num;
    float c = 0.0f;
    parent.cdf[0] = 0.0f;
    for (uint32_t i = 0; i < h; ++i) {
        c = __fadd_rn(c, __fmul_rn(parent.pdf[i], parent.width));
        parent.cdf[i + 1] = c;
    }
    const float norm = __fdiv_rn(1.0f, c);
    for (uint32_t i = 0; i < h; ++i) {
        parent.pdf[i] = __fmul_rn(parent.pdf[i], norm);
        parent.cdf[i + 1] = __fmul_rn(parent.cdf[i + 1], norm);
    }
}

}  // namespace clr

using namespace clr;

extern "C" int clr_env_distribution_update(uint8_t* others, uint32_t dist_offset, const uint8_t* textures,
                                           uint32_t tex_offset, uint32_t height, const float* row_weight,
                                           void* stream) {
    if (!others || !textures) return clr_set_error(CLR_EINVAL, "clr_env_distribution_update: NULL blob");
    if ((dist_offset & 3u) || (tex_offset & 3u))
        return clr_set_error(CLR_EINVAL, "clr_env_distribution_update: offsets must be 4-byte aligned");
    if (height == 0) return CLR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_env_rows<<<div_up(height, 128u), 128, 0, st>>>(others, dist_offset, textures, tex_offset, row_weight, height);
    CLR_LAUNCH_CHECK("k_env_rows");
    k_env_parent<<<1, 1, 0, st>>>(others, dist_offset);
    CLR_LAUNCH_CHECK("k_env_parent");
    return CLR_OK;
}
