/*
 * The reference's own post-processing kernels run on the CPU
 * (OpenCL_PathTracer/OpenCL/post_processing.cl: `clear`, `scaling`,
 * `toneMapping`), compiled as C++ through oracle/ref_stubs/opencl_c.hpp and
 * launched as main.cpp:519-537 does (NDRange width x height each, the
 * intermediate buffer cleared first).  exp and pow are the C library's
 * float functions, which is where this can differ from a GPU's.
 *
 * TEST INFRASTRUCTURE ONLY: it pins the post-processing oracle
 * (oracle/postprocess.py) and the device kernel (clr_postprocess_ldr)
 * against the reference's kernels.  Built only where the reference sources
 * are present (oracle/build_oracle.py), into oracle/_ref/libref_post_cl.so.
 */
#include <cstdint>
#include <cstring>
#include <vector>

#include "opencl_c.hpp"

extern "C" {
void clear(uint width, uint height, float3* buffer);
void scaling(uint width, uint height, uint spp, float3* src, float3* output);
void toneMapping(uint width, uint height, uint b_width, float3* src, uchar* dst);
}

namespace {
template <typename F>
void run2d(size_t gx, size_t gy, F f) {
    clshim::launch2d(gx, gy, [](void* p) { (*static_cast<F*>(p))(); }, &f);
}
}  // namespace

extern "C" {

/* accum: float4 per pixel (xyz used, the accumulation buffer); dst: the BMP
 * pixel array, height rows of 3 * width + width % 4 bytes (the row padding
 * is left as the caller set it, as the reference leaves it unset). */
void ref_cl_postprocess(const float* accum, uint32_t width, uint32_t height, uint32_t spp, uint8_t* dst) {
    const size_t n = size_t(width) * height;
    std::vector<float3> pixels(n), inter(n);
    for (size_t i = 0; i < n; ++i) pixels[i] = float3(accum[4 * i], accum[4 * i + 1], accum[4 * i + 2]);
    float3* pp = pixels.data();
    float3* ip = inter.data();
    const uint byte_width = 3u * width + width % 4u;
    run2d(width, height, [=] { clear(width, height, ip); });
    run2d(width, height, [=] { scaling(width, height, spp, pp, ip); });
    run2d(width, height, [=] { toneMapping(width, height, byte_width, ip, dst); });
}

}  // extern "C"
