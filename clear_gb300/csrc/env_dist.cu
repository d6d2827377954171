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
// Row i: pdf_j = L * w_i, where L is the reference's
// averageLuminance of a one-texel stratum (CreateFunctions.cpp:159-244): the
// texel's luminance l = 0.2126 r + 0.7152 g + 0.0722 b, in float, added once
// per corner of the stratum, ((l + l) + l) + l, over an area of 1; w_i is the
// row weight, by default the zenith correction cos(pi (0.5 - (i + 0.5) / h))
// with the device cosf (the host passes the C library's for bit-exactness
// with the host encoder); cdf_{j+1} = cdf_j +
// pdf_j * (1 / width) accumulated left to right as the reference's loop does,
// both normalised by the row's mass cdf_w, which becomes the parent's pdf_i;
// then the parent's cdf over rows, normalised the same way.  The running sums
// are sequential on purpose (one lane per row): their rounding is the
// reference's.  HBM-bound otherwise: 8 bytes read and 8 written per texel.
#include <cuda_fp16.h>

#include <algorithm>

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

// Rows [r0, r0 + nr) of the distribution, nr <= rows_per_block.  All threads
// read the rows' texels (coalesced) and stage pdf_j in shared memory; one lane
// per row then runs that row's sequential cdf chain from shared memory (the
// lanes of a warp run different rows' chains side by side); all threads write
// the normalised pdf and cdf.  Shared memory: 2 * rows_per_block * (w + 1)
// floats (row stride w + 1: the chain lanes hit different banks) plus the
// per-row records.
struct RowRec {
    float* pdf;
    float* cdf;
    float norm;
    float corr;
};

__global__ void __launch_bounds__(256) k_env_rows(uint8_t* __restrict__ others, uint32_t dist_off,
                                                  const uint8_t* __restrict__ textures, uint32_t tex_off,
                                                  const float* __restrict__ row_weight, uint32_t rows,
                                                  uint32_t width, uint32_t rows_per_block) {
    extern __shared__ float sm[];
    __shared__ int bad;
    uint8_t* head = others + dist_off;
    const Cc1d parent = read_cc1d(head + 8);
    const uint8_t* tex = textures + tex_off;
    const uint32_t h = parent.num;
    const uint32_t r0 = blockIdx.x * rows_per_block;
    const uint32_t nr = min(rows_per_block, rows - r0);
    const uint32_t w = width, stride = w + 1;
    float* spdf = sm;
    float* scdf = sm + (size_t)rows_per_block * stride;
    RowRec* rec = reinterpret_cast<RowRec*>(scdf + (size_t)rows_per_block * stride);
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    const uint32_t tw = *reinterpret_cast<const uint32_t*>(tex + 4), th = *reinterpret_cast<const uint32_t*>(tex + 8);
    if (threadIdx.x < nr) {
        const uint32_t i = r0 + threadIdx.x;
        // a ContinuousConsts2D_H with one stratum per texel of a w x rows RGBA16F
        // image whose texels are 8-byte aligned; the row's record is read only
        // once the head has checked out
        const uintptr_t px = reinterpret_cast<uintptr_t>(tex + *reinterpret_cast<const int32_t*>(tex + 12));
        if (head[0] != 2 || tex[0] != 3 || tw != w || h != th || h != rows || (px & 7u) ||
            read_cc1d(head + *reinterpret_cast<const int32_t*>(head + 4) + 28u * i).num != w) {
            bad = 1;
        } else {
            float corr;
            if (row_weight) {
                corr = row_weight[i];
            } else {
                const float a = __fsub_rn(0.5f, __fdiv_rn(__fadd_rn((float)i, 0.5f), (float)h));
                corr = cosf((float)(3.14159265358979323846 * (double)a));
            }
            const Cc1d row = read_cc1d(head + *reinterpret_cast<const int32_t*>(head + 4) + 28u * i);
            rec[threadIdx.x] = RowRec{row.pdf, row.cdf, 0.0f, corr};
        }
    }
    __syncthreads();
    if (bad) {
        if (threadIdx.x == 0) clr_raise(kDevErrInput);
        return;
    }
    // pdf_j = L_j * corr, L_j the one-texel stratum's averageLuminance
    const uint2* texel = reinterpret_cast<const uint2*>(tex + *reinterpret_cast<const int32_t*>(tex + 12)) +
                         (size_t)w * r0;
    for (uint32_t k = threadIdx.x; k < nr * w; k += blockDim.x) {
        const uint32_t r = k / w, j = k - r * w;
        const uint2 q = __ldg(texel + k);
        const float R = __half2float(__ushort_as_half((unsigned short)(q.x & 0xFFFFu)));
        const float G = __half2float(__ushort_as_half((unsigned short)(q.x >> 16)));
        const float B = __half2float(__ushort_as_half((unsigned short)(q.y & 0xFFFFu)));
        const float lum = __fadd_rn(__fadd_rn(__fmul_rn(0.2126f, R), __fmul_rn(0.7152f, G)), __fmul_rn(0.0722f, B));
        const float l4 = __fadd_rn(__fadd_rn(__fadd_rn(lum, lum), lum), lum);
        spdf[r * stride + j] = __fmul_rn(l4, rec[r].corr);
    }
    __syncthreads();
    // cdf_{j+1} = cdf_j + pdf_j * width_stratum, left to right
    if (threadIdx.x < nr) {
        const uint32_t r = threadIdx.x;
        const float wc = read_cc1d(head + *reinterpret_cast<const int32_t*>(head + 4) + 28u * (r0 + r)).width;
        const float* __restrict__ p = spdf + r * stride;
        float* __restrict__ c = scdf + r * stride;
        float acc = 0.0f;
        c[0] = 0.0f;
        // eight terms loaded ahead of their adds, so the chain waits on the
        // adds alone
        uint32_t j = 0;
        for (; j + 8 <= w; j += 8) {
            float t[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) t[k] = __fmul_rn(p[j + k], wc);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                acc = __fadd_rn(acc, t[k]);
                c[j + k + 1] = acc;
            }
        }
        for (; j < w; ++j) {
            acc = __fadd_rn(acc, __fmul_rn(p[j], wc));
            c[j + 1] = acc;
        }
        rec[r].norm = acc > 0.0f ? __fdiv_rn(1.0f, acc) : 0.0f;
        parent.pdf[r0 + r] = acc;
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < nr * w; k += blockDim.x) {
        const uint32_t r = k / w, j = k - r * w;
        const RowRec rr = rec[r];
        rr.pdf[j] = __fmul_rn(spdf[r * stride + j], rr.norm);
        rr.cdf[j + 1] = __fmul_rn(scdf[r * stride + j + 1], rr.norm);
        if (j == 0) rr.cdf[0] = 0.0f;
    }
}

// The parent over rows: the masses staged in shared memory, one thread's
// sequential chain, then all threads normalise.  Shared memory 2 * (h + 1)
// floats; k_env_parent_global does the same from global memory for maps too
// tall for that.
__global__ void __launch_bounds__(1024) k_env_parent(uint8_t* __restrict__ others, uint32_t dist_off,
                                                     uint32_t rows) {
    extern __shared__ float sm[];
    const Cc1d parent = read_cc1d(others + dist_off + 8);
    const uint32_t h = parent.num;
    if (others[dist_off] != 2 || h != rows) {  // the row pass has raised CLR_DEVERR_INPUT
        return;
    }
    float* mass = sm;
    float* cdf = sm + h + 1;
    for (uint32_t i = threadIdx.x; i < h; i += blockDim.x) mass[i] = parent.pdf[i];
    __syncthreads();
    __shared__ float norm;
    if (threadIdx.x == 0) {
        const float* __restrict__ m = mass;
        float* __restrict__ cd = cdf;
        float c = 0.0f;
        cd[0] = 0.0f;
        uint32_t i = 0;
        for (; i + 8 <= h; i += 8) {
            float t[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) t[k] = __fmul_rn(m[i + k], parent.width);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                c = __fadd_rn(c, t[k]);
                cd[i + k + 1] = c;
            }
        }
        for (; i < h; ++i) {
            c = __fadd_rn(c, __fmul_rn(m[i], parent.width));
            cd[i + 1] = c;
        }
        norm = __fdiv_rn(1.0f, c);
        parent.cdf[0] = 0.0f;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < h; i += blockDim.x) {
        parent.pdf[i] = __fmul_rn(mass[i], norm);
        parent.cdf[i + 1] = __fmul_rn(cdf[i + 1], norm);
    }
}

__global__ void k_env_parent_global(uint8_t* __restrict__ others, uint32_t dist_off, uint32_t rows) {
    const Cc1d parent = read_cc1d(others + dist_off + 8);
    const uint32_t h = parent.num;
    if (others[dist_off] != 2 || h != rows) return;
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
                                           uint32_t tex_offset, uint32_t height, uint32_t width,
                                           const float* row_weight, void* stream) {
    if (!others || !textures) return clr_set_error(CLR_EINVAL, "clr_env_distribution_update: NULL blob");
    if ((dist_offset & 3u) || (tex_offset & 3u))
        return clr_set_error(CLR_EINVAL, "clr_env_distribution_update: offsets must be 4-byte aligned");
    if (height == 0 || width == 0) return CLR_OK;
    constexpr size_t kSmemBudget = 200u * 1024u;
    const size_t per_row = 2u * ((size_t)width + 1u) * sizeof(float) + sizeof(RowRec);
    if (per_row > kSmemBudget)
        return clr_set_error(CLR_EINVAL, "clr_env_distribution_update: width %u above %zu", width,
                             (kSmemBudget - sizeof(RowRec)) / 8u - 1u);
    // rows per block: enough blocks to cover the SMs, at most what fits
    int dev = 0, sms = 0;
    CLR_CUDA_TRY(cudaGetDevice(&dev));
    CLR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    uint32_t rpb = (uint32_t)std::min<size_t>(32u, kSmemBudget / per_row);
    rpb = std::max(1u, std::min(rpb, div_up(height, (uint32_t)std::max(sms, 1))));
    const size_t smem = rpb * per_row;
    CLR_CUDA_TRY(cudaFuncSetAttribute(k_env_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_env_rows<<<div_up(height, rpb), 256, smem, st>>>(others, dist_offset, textures, tex_offset, row_weight, height,
                                                        width, rpb);
    CLR_LAUNCH_CHECK("k_env_rows");
    const size_t psmem = 2u * ((size_t)height + 1u) * sizeof(float);
    if (psmem <= kSmemBudget) {
        CLR_CUDA_TRY(cudaFuncSetAttribute(k_env_parent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
        k_env_parent<<<1, 1024, psmem, st>>>(others, dist_offset, height);
        CLR_LAUNCH_CHECK("k_env_parent");
    } else {
        k_env_parent_global<<<1, 1, 0, st>>>(others, dist_offset, height);
        CLR_LAUNCH_CHECK("k_env_parent_global");
    }
    return CLR_OK;
}
