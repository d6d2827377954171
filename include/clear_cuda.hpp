/*
 * clear_cuda.hpp -- C++ facade over the C ABI of clear_cuda.h, mirroring the
 * reference's host classes so that a C++ host swaps them one for one:
 *
 *   LBVHBuilder (OpenCL_PathTracer/LBVHBuilder.h:37-75): the constructor takes
 *   the capacity in triangles, perform() builds (profiling flag included),
 *   exportReference() gives the reference's 48-byte node arrays;
 *   rayIntersection / shadow queries (OpenCL/bvh_traversal.cl:182-215);
 *   the pathtracing launches of main.cpp:477-494 (render / renderWavefront).
 *
 * Errors are thrown as clr::Error, as the reference throws cl::Error
 * (main.cpp:17, 546-551); the status code and clr_last_error_string() are
 * kept.  Device pointers are the caller's; a stream is a cudaStream_t passed
 * as void* (no CUDA header needed here).  Header only.
 */
#ifndef CLEAR_CUDA_HPP
#define CLEAR_CUDA_HPP

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "clear_cuda.h"

namespace clr {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc) {
    if (rc != CLR_OK) throw Error(rc, clr_last_error_string());
}

class LBVHBuilder {
   public:
    explicit LBVHBuilder(uint32_t numFaces) { check(clr_lbvh_create(numFaces, &h_)); }
    ~LBVHBuilder() {
        if (h_) clr_lbvh_destroy(h_);
    }
    LBVHBuilder(const LBVHBuilder&) = delete;
    LBVHBuilder& operator=(const LBVHBuilder&) = delete;
    LBVHBuilder(LBVHBuilder&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    LBVHBuilder& operator=(LBVHBuilder&& o) noexcept {
        std::swap(h_, o.h_);
        return *this;
    }

    // perform(queue, vertices, faces, numFaces, numBitsPerDim, nodes, ..., profiling):
    // vertices as SoA floats, faces as 3 vertex indices per triangle (or
    // nullptr for an unindexed soup); the caller allocates out.nodes,
    // out.tris and out.root_box (sizes in clear_cuda.h).
    void perform(void* stream, const float* vx, const float* vy, const float* vz, const uint32_t* faces,
                 uint32_t numFaces, uint32_t numBitsPerDim, clr_bvh& out, bool profiling = false) {
        check(clr_lbvh_set_profiling(h_, profiling ? 1 : 0));
        check(clr_lbvh_build(h_, vx, vy, vz, faces, numFaces, numBitsPerDim, &out, stream));
    }

    // Upload-and-build from host arrays (the reference host's buffers created
    // from host memory, then perform): numVerts vertices, faces as 3 indices
    // per triangle or nullptr for a soup (numVerts = 3 * numFaces).  The copy
    // of a call overlaps the previous call's build; see clr_lbvh_build_host.
    void performHost(void* stream, const float* hostVx, const float* hostVy, const float* hostVz,
                     const uint32_t* hostFaces, uint32_t numVerts, uint32_t numFaces, uint32_t numBitsPerDim,
                     clr_bvh& out, float* hostRootBox = nullptr) {
        check(clr_lbvh_build_host(h_, hostVx, hostVy, hostVz, hostFaces, numVerts, numFaces, numBitsPerDim, &out,
                                  hostRootBox, stream));
    }
    // Later performHost copies start after the work queued on `stream` so far.
    void hostCopyAfter(void* stream) { check(clr_lbvh_host_copy_after(h_, stream)); }
    // Blocks until the host arrays of every performHost so far may change.
    void hostCopyWait() { check(clr_lbvh_host_copy_wait(h_)); }

    // The per-pass device times of the last profiled perform() (ms), in order.
    std::vector<std::pair<std::string, float>> passTimes() const {
        constexpr int kMax = 64;  // more than the passes of any build
        float ms[kMax];
        const char* names[kMax];
        int n = 0;
        check(clr_lbvh_pass_times(h_, ms, names, kMax, &n));
        std::vector<std::pair<std::string, float>> out;
        for (int i = 0; i < n; ++i) out.emplace_back(names[i], ms[i]);
        return out;
    }

    // The reference's InternalNode / LeafNode arrays (48 B each), parents,
    // sorted triangle order and keys of the last build; any may be nullptr.
    void exportReference(void* stream, const clr_bvh& bvh, void* internalNodes, void* leafNodes,
                         uint32_t* parents = nullptr, uint32_t* sortedIdx = nullptr, uint64_t* keys = nullptr) {
        check(clr_lbvh_export_reference(h_, &bvh, internalNodes, leafNodes, parents, sortedIdx, keys, stream));
    }

    clr_lbvh* handle() const { return h_; }

   private:
    clr_lbvh* h_ = nullptr;
};

// rayIntersection over rays {ox, oy, oz, tmax, dx, dy, dz, 0}: closest hit id
// (0xFFFFFFFF = miss) and distance; ordered = nearer child first.
inline void traceClosest(void* stream, const clr_bvh& bvh, const float* rays, uint32_t numRays, uint32_t* hitId,
                         float* hitT, bool ordered = false) {
    check(ordered ? clr_trace_closest_ordered(&bvh, rays, numRays, hitId, hitT, stream)
                  : clr_trace_closest(&bvh, rays, numRays, hitId, hitT, stream));
}

// Shadow rays: 1 where something blocks [0, tmax].
inline void traceShadow(void* stream, const clr_bvh& bvh, const float* rays, uint32_t numRays, uint8_t* occluded) {
    check(clr_trace_shadow(&bvh, rays, numRays, occluded, stream));
}

// Workspace bytes of the sorted queries below for numRays rays.
inline uint64_t traceSortWorkspaceBytes(uint32_t numRays) {
    uint64_t b = 0;
    check(clr_trace_sort_workspace_bytes(numRays, &b));
    return b;
}

// traceClosest(ordered = true) and traceShadow with the rays searched in the
// order of their origins' Morton codes (for incoherent ray lists): the same
// answers, in the callers' ray order.  `workspace` (256-byte aligned) holds
// traceSortWorkspaceBytes(numRays) bytes.
inline void traceClosestSorted(void* stream, const clr_bvh& bvh, const float* rays, uint32_t numRays,
                               uint32_t* hitId, float* hitT, void* workspace, uint64_t workspaceBytes) {
    check(clr_trace_closest_sorted(&bvh, rays, numRays, hitId, hitT, workspace, workspaceBytes, stream));
}
inline void traceShadowSorted(void* stream, const clr_bvh& bvh, const float* rays, uint32_t numRays,
                              uint8_t* occluded, void* workspace, uint64_t workspaceBytes) {
    check(clr_trace_shadow_sorted(&bvh, rays, numRays, occluded, workspace, workspaceBytes, stream));
}

// The pathtracing launches: spp samples added to every pixel of `pixels`
// (float4 per pixel) from the per-pixel random states.
inline void render(void* stream, const clr_scene& scene, uint32_t width, uint32_t height, uint32_t* randStates,
                   float* pixels, uint32_t spp, uint32_t maxDepth = 100, uint32_t flags = CLR_RENDER_ORDERED) {
    check(clr_render(&scene, width, height, randStates, pixels, spp, maxDepth, flags, stream));
}

inline uint64_t renderWorkspaceBytes(uint32_t width, uint32_t height) {
    uint64_t b = 0;
    check(clr_render_workspace_bytes(width, height, &b));
    return b;
}

// The same samples with the wavefront kernels; `workspace` (256-byte aligned)
// holds renderWorkspaceBytes(width, height) bytes.
inline void renderWavefront(void* stream, const clr_scene& scene, uint32_t width, uint32_t height,
                            uint32_t* randStates, float* pixels, uint32_t spp, void* workspace,
                            uint64_t workspaceBytes, uint32_t maxDepth = 100, uint32_t flags = CLR_RENDER_ORDERED) {
    check(clr_render_wavefront(&scene, width, height, randStates, pixels, spp, maxDepth, flags, workspace,
                               workspaceBytes, stream));
}

inline uint64_t renderAdjointWorkspaceBytes(uint32_t width, uint32_t height, uint32_t numParams) {
    uint64_t b = 0;
    check(clr_render_adjoint_workspace_bytes(width, height, numParams, &b));
    return b;
}

// Gradients of an image loss (dlossDaccum: float4 per pixel) for the samples
// renderWavefront would take from the same randStates (advanced as it would
// advance them); `workspace` (256-byte aligned) holds
// renderAdjointWorkspaceBytes(width, height, params.num_params) bytes.
// flags: CLR_RENDER_ORDERED, CLR_ADJOINT_RETRACE.
inline void renderAdjoint(void* stream, const clr_scene& scene, uint32_t width, uint32_t height,
                          uint32_t* randStates, const float* dlossDaccum, uint32_t spp,
                          const clr_adjoint_params& params, void* workspace, uint64_t workspaceBytes,
                          uint32_t maxDepth = 100, uint32_t flags = CLR_RENDER_ORDERED) {
    check(clr_render_adjoint(&scene, width, height, randStates, dlossDaccum, spp, maxDepth, flags, &params,
                             workspace, workspaceBytes, stream));
}

}  // namespace clr

#endif /* CLEAR_CUDA_HPP */
