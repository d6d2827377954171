// Error reporting shared by every C entry point.
#include <stdarg.h>
#include <stdio.h>

#include "common.cuh"

static thread_local char t_last_error[512] = "no error";

int clr_set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_last_error, sizeof(t_last_error), fmt, ap);
    va_end(ap);
    return code;
}

extern "C" const char* clr_last_error_string(void) { return t_last_error; }

int clr_sm_count() {
    constexpr int kMaxDevices = 64;
    static int sms[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
    if (sms[dev] <= 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
        sms[dev] = v;
    }
    return sms[dev];
}

cudaError_t clr_status_lbvh(unsigned int* v, int clear);
cudaError_t clr_status_traverse(unsigned int* v, int clear);
cudaError_t clr_status_render(unsigned int* v, int clear);
cudaError_t clr_status_render_wf(unsigned int* v, int clear);
cudaError_t clr_status_render_adjoint(unsigned int* v, int clear);
cudaError_t clr_status_render_batch(unsigned int* v, int clear);
cudaError_t clr_status_env_dist(unsigned int* v, int clear);
cudaError_t clr_status_bvh_vis(unsigned int* v, int clear);

extern "C" int clr_device_status(uint32_t* bits, int clear) {
    CLR_CUDA_TRY(cudaDeviceSynchronize());
    unsigned int all = 0;
    cudaError_t (*readers[])(unsigned int*, int) = {clr_status_lbvh, clr_status_traverse, clr_status_render,
                                                   clr_status_render_wf, clr_status_render_adjoint,
                                                   clr_status_render_batch, clr_status_env_dist,
                                                   clr_status_bvh_vis};
    for (auto rd : readers) {
        unsigned int v = 0;
        CLR_CUDA_TRY(rd(&v, clear));
        all |= v;
    }
    if (bits) *bits = all;
    return CLR_OK;
}
