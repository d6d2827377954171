// Internal constants and the builder handle of the LBVH build.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <cuda.h>
#include <cuda_runtime.h>

namespace clr {

constexpr int kRadix = 256;          // 8-bit digits
constexpr int kMaxPasses = 8;        // 63-bit keys (21 bits per axis)
constexpr int kSortThreads = 256;
constexpr unsigned int kMinSortTile = 2048;  // smallest tile (64-bit keys)
constexpr unsigned int kFlagAggregate = 1u << 30;
constexpr unsigned int kFlagInclusive = 2u << 30;
constexpr unsigned int kFlagMask = 3u << 30;
constexpr unsigned int kValueMask = (1u << 30) - 1u;
constexpr unsigned int kSpinLimit = 1u << 22;  // look-back polls before giving up
// Depth bound of the Karras tree: every level down adds at least one common
// bit of the (3b + 32)-bit extended key, so depth <= 63 + 32 for b = 21.
constexpr int kMaxDepth = 96;

}  // namespace clr

// Builder handle: the scratch pool and what the last build left in it.
struct clr_lbvh {
    // the staging array as a tensor of n rows x 12 floats, for the tree pass's
    // TMA gathers (encoded for map_base / map_rows; map_ok false = unavailable)
    CUtensorMap stage_map{};
    const void* map_base = nullptr;
    uint32_t map_rows = 0;
    bool map_ok = false;
    uint32_t capacity = 0;
    void* pool = nullptr;
    size_t pool_bytes = 0;
    void* keys[2] = {nullptr, nullptr};     // sort ping-pong (up to 8 B per key)
    uint32_t* vals[2] = {nullptr, nullptr};  // triangle ids riding with the keys
    uint32_t* karras_idx = nullptr;          // node (at its split) -> reference index
    float4* stage = nullptr;                 // 48-byte vertex record per triangle (input order), or null
    unsigned int* counters = nullptr;        // tree-pass arrival counters
    void* zero_region = nullptr;             // cleared per build: hist, tile_ctr, boxw,
    size_t zero_bytes = 0;                   //   then the used part of status
    size_t zero_prefix_bytes = 0;            // hist, tile_ctr and boxw (status follows)
    unsigned int* hist = nullptr;            // [pass][256] digit counts
    unsigned int* status = nullptr;          // [pass][tile][256] look-back words
    size_t status_stride = 0;                // words per pass: the build's tiles x 256
    unsigned int* tile_ctr = nullptr;        // [pass] dynamic tile counter
    unsigned int* boxw = nullptr;            // scene box, ordered-uint encoded
    // batched builds: scene offsets and per-scene boxes (own allocation)
    uint32_t seg_cap = 0;
    void* seg_pool = nullptr;
    uint32_t* seg_off = nullptr;
    unsigned int* seg_box = nullptr;
    uint32_t last_n = 0, last_bits = 0;
    int final_buf = 0;                       // ping-pong side holding sorted data
    // builds from host inputs (clr_lbvh_build_host): two device input buffers
    // used in turn, the copy stream, and per buffer the events "copy done"
    // and "build that read it done"
    void* in_buf[2] = {nullptr, nullptr};
    size_t in_bytes[2] = {0, 0};
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t in_copied[2] = {}, in_consumed[2] = {}, copy_gate = nullptr;
    bool in_used[2] = {false, false};
    uint32_t host_calls = 0;
    // profiling (clr_lbvh_set_profiling)
    static constexpr int kMaxTimed = 16;
    bool profiling = false;
    int num_timed = 0;
    cudaEvent_t ev[kMaxTimed + 1] = {};
    const char* ev_name[kMaxTimed] = {};
};
