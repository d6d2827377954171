// Exercises the C++ facade (include/clear_cuda.hpp): on a machine without a
// GPU the builder's constructor must throw clr::Error with a message; with a
// GPU, a two-triangle soup is built and one ray finds the nearer triangle,
// and the same soup built from host arrays gives the same tree.
// Prints one line per check; exits 0 when all pass.
#include <cstdio>
#include <cstring>
#include <cuda_runtime_api.h>

#include "clear_cuda.hpp"

int main() {
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
        try {
            clr::LBVHBuilder b(16);
            std::puts("FAIL: builder constructed without a GPU");
            return 1;
        } catch (const clr::Error& e) {
            std::printf("no-gpu: clr::Error code %d: %s\n", e.code, e.what());
            return e.code != CLR_OK && std::strlen(e.what()) > 0 ? 0 : 1;
        }
    }
    // two triangles in the z = 1 and z = 2 planes; a ray down +z from the origin
    const float hx[6] = {-1, 1, 0, -1, 1, 0}, hy[6] = {-1, -1, 1, -1, -1, 1}, hz[6] = {1, 1, 1, 2, 2, 2};
    const float hray[8] = {0, 0, 0, 1e30f, 0, 0, 1, 0};
    float *vx, *vy, *vz, *rays, *t;
    uint32_t* id;
    clr_bvh bvh{};
    cudaMalloc((void**)&vx, sizeof(hx)); cudaMalloc((void**)&vy, sizeof(hy)); cudaMalloc((void**)&vz, sizeof(hz));
    cudaMalloc((void**)&rays, sizeof(hray)); cudaMalloc((void**)&t, 4); cudaMalloc((void**)&id, 4);
    cudaMalloc(&bvh.nodes, CLR_NODE_BYTES); cudaMalloc(&bvh.tris, 2 * CLR_TRI_BYTES);
    cudaMalloc((void**)&bvh.root_box, 32);
    cudaMemcpy(vx, hx, sizeof(hx), cudaMemcpyHostToDevice);
    cudaMemcpy(vy, hy, sizeof(hy), cudaMemcpyHostToDevice);
    cudaMemcpy(vz, hz, sizeof(hz), cudaMemcpyHostToDevice);
    cudaMemcpy(rays, hray, sizeof(hray), cudaMemcpyHostToDevice);
    clr::LBVHBuilder b(2);
    b.perform(nullptr, vx, vy, vz, nullptr, 2, 10, bvh, true);
    const auto passes = b.passTimes();
    clr::traceClosest(nullptr, bvh, rays, 1, id, t);
    uint32_t hid = 0;
    float ht = 0;
    cudaMemcpy(&hid, id, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&ht, t, 4, cudaMemcpyDeviceToHost);
    std::printf("gpu: hit %u at t %g, %zu timed passes\n", hid, ht, passes.size());
    bool ok = hid == 0 && ht == 1.0f && !passes.empty();
    // the same query with the rays sorted by origin first
    {
        const uint64_t wsb = clr::traceSortWorkspaceBytes(1);
        void* ws = nullptr;
        cudaMalloc(&ws, wsb);
        cudaMemset(id, 0xFF, 4);
        clr::traceClosestSorted(nullptr, bvh, rays, 1, id, t, ws, wsb);
        uint32_t sid = 1;
        float st = 0;
        cudaMemcpy(&sid, id, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&st, t, 4, cudaMemcpyDeviceToHost);
        std::printf("gpu: sorted query hit %u at t %g\n", sid, st);
        ok = ok && sid == hid && st == ht;
        cudaFree(ws);
    }
    // the same soup uploaded from host arrays: same tree, root record read back
    {
        clr_bvh hb{};
        cudaMalloc(&hb.nodes, CLR_NODE_BYTES); cudaMalloc(&hb.tris, 2 * CLR_TRI_BYTES);
        cudaMalloc((void**)&hb.root_box, 32);
        float root_a[8], root_b[8];
        clr::LBVHBuilder hbld(2);
        hbld.performHost(nullptr, hx, hy, hz, nullptr, 6, 2, 10, hb, root_b);
        hbld.hostCopyWait();
        cudaDeviceSynchronize();
        cudaMemcpy(root_a, bvh.root_box, 32, cudaMemcpyDeviceToHost);
        unsigned char ta[2 * CLR_TRI_BYTES], tb[2 * CLR_TRI_BYTES];
        cudaMemcpy(ta, bvh.tris, sizeof(ta), cudaMemcpyDeviceToHost);
        cudaMemcpy(tb, hb.tris, sizeof(tb), cudaMemcpyDeviceToHost);
        const bool same = std::memcmp(root_a, root_b, 32) == 0 && std::memcmp(ta, tb, sizeof(ta)) == 0;
        std::printf("gpu: host-input build %s\n", same ? "identical" : "DIFFERS");
        ok = ok && same;
    }
    try {
        clr::LBVHBuilder bad(1);
        bad.perform(nullptr, vx, vy, vz, nullptr, 1, 0, bvh);  // bits_per_dim 0 is rejected
        ok = false;
    } catch (const clr::Error& e) {
        std::printf("gpu: invalid argument -> clr::Error %d\n", e.code);
        ok = ok && e.code == CLR_EINVAL;
    }
    return ok ? 0 : 1;
}
