// LBVH construction on sm_103a.
//
// Reference pipeline (OpenCL_PathTracer/LBVHBuilder.cpp:160-375) and what
// replaces each step here:
//   calcAABBs + unifyAABBs + host read-back (lbvh_construction.cl:81-162,
//   LBVHBuilder.cpp:189-229)        -> k_scene_box: one pass over the vertices,
//                                      block reduce + ordered-uint atomics; the
//                                      scene box never leaves the device.
//   calcMortonCodes (:169-181)      -> k_morton: per-triangle box/centre and
//                                      quantisation, packed straight into an
//                                      interleaved 3b-bit key whose order is the
//                                      reference's LSD digit order, plus the
//                                      digit histograms of every sort pass.
//   b rounds of blockwiseSort / histograms / global scan / scatter
//   (:231-316, CLGenericKernels.cpp:107-151)
//                                   -> ceil(3b/8) passes of a one-sweep 8-bit LSD
//                                      radix sort (warp match-any ranking,
//                                      decoupled look-back).  Stable, so the
//                                      sorted order is the reference's.
//   constructBinaryRadixTree (:342-410) + calcNodeAABBs (:415-492)
//                                   -> k_build_tree: the same radix tree, emitted
//                                      bottom-up in the atomic-counter climb that
//                                      refits the boxes (with device fences, which
//                                      the reference's refit lacks); each leaf
//                                      thread writes its triangle record.
#include <stdio.h>

#include <mutex>
#include <new>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "lbvh_internal.cuh"

CLR_DEFINE_STATUS_READER(lbvh)

namespace clr {

// -------------------------------------------------------------- key packing

__device__ __forceinline__ uint32_t spread3_10(uint32_t x) {
    x &= 0x3FFu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__device__ __forceinline__ uint64_t spread3_21(uint64_t x) {
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x001F00000000FFFFull;
    x = (x | (x << 16)) & 0x001F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Key whose ascending order is the reference's sort order: the per-bit digit
// is x | y<<1 | z<<2 (lbvh_construction.cl:245-246), least significant bit
// level sorted first (LBVHBuilder.cpp:263).
template <typename KeyT>
__device__ __forceinline__ KeyT make_key(uint32_t qx, uint32_t qy, uint32_t qz);
template <>
__device__ __forceinline__ uint32_t make_key<uint32_t>(uint32_t qx, uint32_t qy, uint32_t qz) {
    return spread3_10(qx) | (spread3_10(qy) << 1) | (spread3_10(qz) << 2);
}
template <>
__device__ __forceinline__ uint64_t make_key<uint64_t>(uint32_t qx, uint32_t qy, uint32_t qz) {
    return spread3_21(qx) | (spread3_21(qy) << 1) | (spread3_21(qz) << 2);
}

// One 64-byte internal node written as two 32-byte stores when the node array
// is 32-byte aligned (whole DRAM sectors per store), else as four 16-byte ones.
__device__ __forceinline__ void st_node(float* nn, bool wide, float4 a, float4 b, float4 c, float4 d) {
    if (wide) {
        asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(nn), "f"(a.x), "f"(a.y), "f"(a.z),
                     "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                     : "memory");
        asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(nn + 8), "f"(c.x), "f"(c.y), "f"(c.z),
                     "f"(c.w), "f"(d.x), "f"(d.y), "f"(d.z), "f"(d.w)
                     : "memory");
    } else {
        float4* n4 = reinterpret_cast<float4*>(nn);
        n4[0] = a;
        n4[1] = b;
        n4[2] = c;
        n4[3] = d;
    }
}

// 48-byte staging record of triangle t in input order: the nine vertex floats
// p0, p1, p2 packed into three float4 (and three zeros), so that the tree
// pass gathers two DRAM sectors per leaf instead of three scattered 12-byte
// runs of the SoA arrays.
__device__ __forceinline__ void stage_tri(float4* stage, uint32_t t, const float P[3][3]) {
    float4* r = stage + 3ull * t;
    r[0] = make_float4(P[0][0], P[0][1], P[0][2], P[1][0]);
    r[1] = make_float4(P[1][1], P[1][2], P[2][0], P[2][1]);
    r[2] = make_float4(P[2][2], 0.f, 0.f, 0.f);
}

__device__ __forceinline__ uint32_t tri_vertex(const uint32_t* tri, uint32_t t, uint32_t k) {
    return tri ? __ldg(tri + 3u * t + k) : 3u * t + k;
}

// ----------------------------------------------------------- scene bounds

__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

// boxw[0..2] hold ~ordered(min) (atomicMax of the complement = atomicMin),
// boxw[3..5] hold ordered(max); all start at 0.
__global__ void __launch_bounds__(256) k_scene_box(const float* __restrict__ vx, const float* __restrict__ vy,
                                                   const float* __restrict__ vz, const uint32_t* __restrict__ tri,
                                                   uint32_t n, unsigned int* __restrict__ boxw) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    const uint32_t stride = gridDim.x * blockDim.x;
    if (tri == nullptr) {
        // unindexed soup: every vertex belongs to a triangle; with 16-byte
        // aligned arrays four vertices per load and array, two loads in
        // flight per array and thread
        const uint64_t nv = 3ull * n;
        const uint64_t first = blockIdx.x * blockDim.x + threadIdx.x;
        uint64_t scalar_from = 0;
        if (((reinterpret_cast<uintptr_t>(vx) | reinterpret_cast<uintptr_t>(vy) | reinterpret_cast<uintptr_t>(vz)) &
             15u) == 0u) {
            const float4* x4 = reinterpret_cast<const float4*>(vx);
            const float4* y4 = reinterpret_cast<const float4*>(vy);
            const float4* z4 = reinterpret_cast<const float4*>(vz);
            const uint64_t nv4 = nv / 4;
            auto take = [&](const float4 x, const float4 y, const float4 z) {
                mn[0] = fminf(mn[0], fminf(fminf(x.x, x.y), fminf(x.z, x.w)));
                mx[0] = fmaxf(mx[0], fmaxf(fmaxf(x.x, x.y), fmaxf(x.z, x.w)));
                mn[1] = fminf(mn[1], fminf(fminf(y.x, y.y), fminf(y.z, y.w)));
                mx[1] = fmaxf(mx[1], fmaxf(fmaxf(y.x, y.y), fmaxf(y.z, y.w)));
                mn[2] = fminf(mn[2], fminf(fminf(z.x, z.y), fminf(z.z, z.w)));
                mx[2] = fmaxf(mx[2], fmaxf(fmaxf(z.x, z.y), fmaxf(z.z, z.w)));
            };
            uint64_t i = first;
            for (; i + stride < nv4; i += 2 * (uint64_t)stride) {
                const float4 xa = __ldg(x4 + i), ya = __ldg(y4 + i), za = __ldg(z4 + i);
                const float4 xb = __ldg(x4 + i + stride), yb = __ldg(y4 + i + stride), zb = __ldg(z4 + i + stride);
                take(xa, ya, za);
                take(xb, yb, zb);
            }
            if (i < nv4) take(__ldg(x4 + i), __ldg(y4 + i), __ldg(z4 + i));
            scalar_from = 4 * nv4;
        }
        for (uint64_t i = scalar_from + first; i < nv; i += stride) {
            float x = __ldg(vx + i), y = __ldg(vy + i), z = __ldg(vz + i);
            mn[0] = fminf(mn[0], x); mx[0] = fmaxf(mx[0], x);
            mn[1] = fminf(mn[1], y); mx[1] = fmaxf(mx[1], y);
            mn[2] = fminf(mn[2], z); mx[2] = fmaxf(mx[2], z);
        }
    } else {
        for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
            for (int k = 0; k < 3; ++k) {
                uint32_t v = __ldg(tri + 3u * t + k);
                float x = __ldg(vx + v), y = __ldg(vy + v), z = __ldg(vz + v);
                mn[0] = fminf(mn[0], x); mx[0] = fmaxf(mx[0], x);
                mn[1] = fminf(mn[1], y); mx[1] = fmaxf(mx[1], y);
                mn[2] = fminf(mn[2], z); mx[2] = fmaxf(mx[2], z);
            }
        }
    }
    __shared__ float s[6][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 3; ++k) {
        float a = warp_min(mn[k]), b = warp_max(mx[k]);
        if (lane == 0) { s[k][warp] = a; s[3 + k][warp] = b; }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        float v = s[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = k < 3 ? fminf(v, s[k][w]) : fmaxf(v, s[k][w]);
        if (v == v) {  // skip NaN (fmin/fmax ignore NaN operands)
            unsigned int e = float_to_ordered(v);
            atomicMax(boxw + k, k < 3 ? ~e : e);
        }
    }
}

__device__ __forceinline__ void load_scene_box(const unsigned int* boxw, float smin[3], float ssize[3]) {
    for (int k = 0; k < 3; ++k) {
        float mn = ordered_to_float(~__ldcg(boxw + k));
        float mx = ordered_to_float(__ldcg(boxw + 3 + k));
        smin[k] = mn;
        ssize[k] = fsub(mx, mn);  // host subtraction in the reference, LBVHBuilder.cpp:236-240
    }
}

// ------------------------------------------------------------ Morton keys

template <typename KeyT>
__global__ void __launch_bounds__(256) k_morton(const float* __restrict__ vx, const float* __restrict__ vy,
                                                const float* __restrict__ vz, const uint32_t* __restrict__ tri,
                                                uint32_t n, uint32_t bits, const unsigned int* __restrict__ boxw,
                                                KeyT* __restrict__ keys, unsigned int* __restrict__ hist,
                                                int npasses, unsigned int* __restrict__ counters,
                                                float4* __restrict__ stage) {
    __shared__ unsigned int sh[kMaxPasses * kRadix];
    for (int i = threadIdx.x; i < npasses * kRadix; i += blockDim.x) sh[i] = 0;
    float smin[3], ssize[3];
    load_scene_box(boxw, smin, ssize);
    const uint32_t numDivs = 1u << bits;
    const float fDivs = (float)numDivs;
    __syncthreads();
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t a = tri_vertex(tri, t, 0), b = tri_vertex(tri, t, 1), c = tri_vertex(tri, t, 2);
        const float P[3][3] = {{__ldg(vx + a), __ldg(vy + a), __ldg(vz + a)},
                               {__ldg(vx + b), __ldg(vy + b), __ldg(vz + b)},
                               {__ldg(vx + c), __ldg(vy + c), __ldg(vz + c)}};
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            // calcAABBs (lbvh_construction.cl:92-94) then calcMortonCodes (:178-179)
            const float mn = fminf(P[0][k], fminf(P[1][k], P[2][k]));
            const float mx = fmaxf(P[0][k], fmaxf(P[1][k], P[2][k]));
            const float center = fmul(fadd(mn, mx), 0.5f);
            const float normPos = fdiv(fsub(center, smin[k]), ssize[k]);
            const uint32_t v = __float2uint_rz(fmul(normPos, fDivs));
            q[k] = min(v, numDivs - 1u);
        }
        const KeyT key = make_key<KeyT>(q[0], q[1], q[2]);
        keys[t] = key;
        if (stage) stage_tri(stage, t, P);
        if (t + 1 < n) counters[t] = 0u;  // arrival counters of the tree pass
        for (int p = 0; p < npasses; ++p) atomicAdd(&sh[p * kRadix + (uint32_t)((key >> (8 * p)) & 0xFFu)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npasses * kRadix; i += blockDim.x)
        if (sh[i]) atomicAdd(hist + i, sh[i]);
}

// ------------------------------------------------------ one-sweep radix pass

__device__ __forceinline__ unsigned int lanemask_lt() {
    unsigned int m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ unsigned int block_excl_scan256(unsigned int v, unsigned int* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    unsigned int off = 0;
    for (int w = 0; w < warp; ++w) off += s_warp[w];
    __syncthreads();
    return off + x - v;
}

template <typename KeyT>
struct SortCfg;
template <>
struct SortCfg<uint32_t> { static constexpr int kItems = 16; };
template <>
struct SortCfg<uint64_t> { static constexpr int kItems = 8; };

// kBits-bit digits (6, 7 or 8); the per-digit arrays keep a 256 stride.
template <typename KeyT, bool kFirst, int kBits = 8>
__global__ void __launch_bounds__(kSortThreads, 4) k_onesweep(const KeyT* __restrict__ kin,
                                                           const uint32_t* __restrict__ vin,
                                                           KeyT* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, uint32_t shift,
                                                           const unsigned int* __restrict__ hist,
                                                           unsigned int* __restrict__ status,
                                                           unsigned int* __restrict__ tile_ctr,
                                                           unsigned int spin_limit) {
    constexpr int kItems = SortCfg<KeyT>::kItems;
    constexpr unsigned int kR = 1u << kBits, kDigitMask = kR - 1u;
    static_assert(kBits >= 1 && kBits <= 8, "digits of 1..8 bits");
    constexpr int kWarps = kSortThreads / 32;
    constexpr int kWarpSpan = 32 * kItems;
    constexpr int kTile = kSortThreads * kItems;
    __shared__ unsigned int s_tile;
    __shared__ unsigned int s_whist[kWarps][kRadix];
    __shared__ unsigned int s_tile_off[kRadix];
    __shared__ unsigned int s_gbase[kRadix];
    __shared__ unsigned int s_scan[kWarps];
    __shared__ KeyT s_keys[kTile];
    __shared__ uint32_t s_vals[kTile];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int i = tid; i < kWarps * kRadix; i += kSortThreads) (&s_whist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)kTile;
    const uint32_t tile_n = min((uint32_t)kTile, n - base);

    // Load: warp w owns the contiguous span [base + w*kWarpSpan, +kWarpSpan),
    // lane-striped so every load instruction is coalesced.
    KeyT k[kItems];
    uint32_t v[kItems];
    uint32_t rank[kItems];
    const uint32_t wbase = base + warp * kWarpSpan;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const uint32_t idx = wbase + i * 32 + lane;
        const bool ok = idx < n;
        k[i] = ok ? kin[idx] : KeyT(0);
        v[i] = kFirst ? idx : (ok ? vin[idx] : 0u);
    }
    // Rank in input order: step i handles 32 consecutive keys; lanes holding
    // the same digit find each other with match.any and the lowest lane
    // advances the warp's counter for that digit.
    const unsigned int lt = lanemask_lt();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const uint32_t idx = wbase + i * 32 + lane;
        const bool ok = idx < n;
        const unsigned int dig = ok ? (unsigned int)((k[i] >> shift) & kDigitMask) : 0xFFFFFFFFu;
        // lanes holding the same digit: one ballot per digit bit (and one for
        // validity), AND-combined -- the ballot form of match.any
        unsigned int peers = __ballot_sync(0xFFFFFFFFu, ok);
        if (!ok) peers = ~peers;
#pragma unroll
        for (int b = 0; b < kBits; ++b) {
            const bool bit = (dig >> b) & 1u;
            const unsigned int bal = __ballot_sync(0xFFFFFFFFu, bit);
            peers &= bit ? bal : ~bal;
        }
        const int leader = __ffs(peers) - 1;
        unsigned int old = 0;
        if (ok && lane == leader) {
            old = s_whist[warp][dig];
            s_whist[warp][dig] = old + __popc(peers);
        }
        old = __shfl_sync(0xFFFFFFFFu, old, leader);
        rank[i] = old + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();

    // Per digit d (= tid < kR): warp prefix, tile total, early publication of
    // the tile's aggregate, then the look-back over earlier tiles.
    const int d = tid;
    const bool dv = (unsigned int)d < kR;
    unsigned int total = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const unsigned int c = s_whist[w][d];
        s_whist[w][d] = total;
        total += c;
    }
    unsigned int* my_status = status + (size_t)tile * kRadix + d;
    if (dv) {
        if (tile == 0) st_relaxed_gpu(my_status, kFlagInclusive | total);
        else st_relaxed_gpu(my_status, kFlagAggregate | total);
    }

    const unsigned int tile_off = block_excl_scan256(total, s_scan);
    const unsigned int gcount = dv ? __ldg(hist + d) : 0u;
    const unsigned int gexcl = block_excl_scan256(gcount, s_scan);

    unsigned int excl = 0;
    if (tile > 0 && dv) {
        int j = (int)tile - 1;
        unsigned int spins = 0;
        while (j >= 0) {
            const unsigned int s = ld_relaxed_gpu(status + (size_t)j * kRadix + d);
            const unsigned int flag = s & kFlagMask;
            if (flag == 0u) {
                if (++spins > spin_limit) {
                    clr_raise(CLR_DEVERR_SORT_TIMEOUT);
                    break;
                }
                if (spins > 64) __nanosleep(32);
                continue;
            }
            excl += s & kValueMask;
            if (flag == kFlagInclusive) break;
            --j;
        }
        st_relaxed_gpu(my_status, kFlagInclusive | (excl + total));
    }
    s_tile_off[d] = tile_off;
    s_gbase[d] = gexcl + excl - tile_off;
    __syncthreads();

    // Scatter into shared memory in digit order.
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const uint32_t idx = wbase + i * 32 + lane;
        if (idx < n) {
            const unsigned int dig = (unsigned int)((k[i] >> shift) & kDigitMask);
            const uint32_t pos = s_tile_off[dig] + s_whist[warp][dig] + rank[i];
            s_keys[pos] = k[i];
            s_vals[pos] = v[i];
        }
    }
    __syncthreads();
    // Write out: consecutive threads take consecutive sorted slots, so every
    // digit's run is written contiguously.
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const uint32_t p = i * kSortThreads + tid;
        if (p < tile_n) {
            const KeyT key = s_keys[p];
            const unsigned int dig = (unsigned int)((key >> shift) & kDigitMask);
            const uint32_t g = s_gbase[dig] + p;
            kout[g] = key;
            vout[g] = s_vals[p];
        }
    }
}

// ------------------------------------------------------------ Karras tree

template <typename KeyT>
__device__ __forceinline__ int clz_key(KeyT x);
template <>
__device__ __forceinline__ int clz_key<uint32_t>(uint32_t x) { return __clz(x); }
template <>
__device__ __forceinline__ int clz_key<uint64_t>(uint64_t x) { return __clzll(x); }

// _numCommonBits (lbvh_construction.cl:322-332) on packed keys: the leading
// common bits of the 3b-bit keys, extended by the common bits of the sorted
// positions when the keys are equal (delta_adj below, for adjacent pairs).

struct TriVerts {
    float p[3][3];
};

// Triangle t's vertices: from its 48-byte staging record (the nine floats
// packed in three float4, two DRAM sectors) when the build staged them, else
// from the SoA arrays.
__device__ __forceinline__ TriVerts load_tri_staged(const float* vx, const float* vy, const float* vz,
                                                    const uint32_t* tri, const float4* stage, uint32_t t);

__device__ __forceinline__ TriVerts load_tri(const float* vx, const float* vy, const float* vz,
                                             const uint32_t* tri, uint32_t t) {
    TriVerts tv;
    for (int k = 0; k < 3; ++k) {
        const uint32_t v = tri_vertex(tri, t, k);
        tv.p[k][0] = __ldg(vx + v);
        tv.p[k][1] = __ldg(vy + v);
        tv.p[k][2] = __ldg(vz + v);
    }
    return tv;
}

__device__ __forceinline__ TriVerts load_tri_staged(const float* vx, const float* vy, const float* vz,
                                                    const uint32_t* tri, const float4* stage, uint32_t t) {
    if (stage == nullptr) return load_tri(vx, vy, vz, tri, t);
    const float4 a = __ldg(stage + 3ull * t), b = __ldg(stage + 3ull * t + 1), c = __ldg(stage + 3ull * t + 2);
    TriVerts tv;
    tv.p[0][0] = a.x; tv.p[0][1] = a.y; tv.p[0][2] = a.z;
    tv.p[1][0] = a.w; tv.p[1][1] = b.x; tv.p[1][2] = b.y;
    tv.p[2][0] = b.z; tv.p[2][1] = b.w; tv.p[2][2] = c.x;
    return tv;
}


// Writes leaf `leaf`'s triangle record from its vertices and returns its box
// (calcAABBs).
__device__ __forceinline__ void emit_leaf_verts(const TriVerts& tv, uint32_t rec_id, uint32_t leaf,
                                                float4* __restrict__ tris, float box[6]) {
    for (int k = 0; k < 3; ++k) {
        box[k] = fminf(tv.p[0][k], fminf(tv.p[1][k], tv.p[2][k]));
        box[3 + k] = fmaxf(tv.p[0][k], fmaxf(tv.p[1][k], tv.p[2][k]));
    }
    float4* r = tris + 3u * leaf;
    r[0] = make_float4(tv.p[0][0], tv.p[0][1], tv.p[0][2], __uint_as_float(rec_id));
    r[1] = make_float4(fsub(tv.p[1][0], tv.p[0][0]), fsub(tv.p[1][1], tv.p[0][1]), fsub(tv.p[1][2], tv.p[0][2]), 0.f);
    r[2] = make_float4(fsub(tv.p[2][0], tv.p[0][0]), fsub(tv.p[2][1], tv.p[0][1]), fsub(tv.p[2][2], tv.p[0][2]), 0.f);
}

// The same from triangle `tid` of the (global) vertex arrays or its staging
// record; `rec_id` is the id recorded.
__device__ __forceinline__ void emit_leaf(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                                          const float4* stage, uint32_t tid, uint32_t rec_id, uint32_t leaf,
                                          float4* __restrict__ tris, float box[6]) {
    emit_leaf_verts(load_tri_staged(vx, vy, vz, tri, stage, tid), rec_id, leaf, tris, box);
}

// ---------------------------------------------------- staging-record gather
//
// The tree pass reads its leaves' staging records in key order: scattered
// 48-byte rows of the staging array.  With the array described as a 2-D
// tensor (n rows of 12 floats), one TMA tile::gather4 copy brings four such
// rows into shared memory; eight lanes of a warp issue the warp's 32 rows,
// and the warp waits on its own mbarrier (bounded) -- instead of 96 scattered
// 16-byte loads through L1 per warp.
constexpr int kStageFloats = 12;
// one gather4 copy (4 rows, 192 bytes) per 256-byte slot: tensor copies into
// shared memory start on 128-byte boundaries
constexpr int kGatherSlotFloats = 64;
constexpr unsigned int kGatherWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// The copies have not completed within the limit: report it, then keep
// waiting (again bounded) so that no copy lands after the block is gone.
static __device__ __noinline__ bool gather_wait_overdue(uint32_t bar) {
    clr_raise(CLR_DEVERR_QUEUE);
    uint32_t done = 0;
    for (unsigned int spins = 0; !done && spins < kGatherWaitLimit; ++spins)
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar)
            : "memory");
    return false;
}

// Stages the staging records of leaves B + 32 w .. + 31 (w = this warp) into
// `rows`: lane l's record at rows[(l / 4) * kGatherSlotFloats + (l % 4) * 12]
// (triangle ids tj per lane, id 0 for lanes past the array: a valid row whose
// copy is not used).  Returns false if the wait gave up.
__device__ __forceinline__ bool gather_warp_records(const CUtensorMap* tmap, uint64_t* bar, float* rows, uint32_t tj) {
    const int lane = threadIdx.x & 31;
    const uint32_t b = smem_u32(bar);
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
                     "r"(32u * kStageFloats * 4u)
                     : "memory");
    }
    const uint32_t r0 = __shfl_sync(0xFFFFFFFFu, tj, (4 * lane) & 31);
    const uint32_t r1 = __shfl_sync(0xFFFFFFFFu, tj, (4 * lane + 1) & 31);
    const uint32_t r2 = __shfl_sync(0xFFFFFFFFu, tj, (4 * lane + 2) & 31);
    const uint32_t r3 = __shfl_sync(0xFFFFFFFFu, tj, (4 * lane + 3) & 31);
    if (lane < 8)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
            "%4, %5, %6}], [%7];" ::"r"(smem_u32(rows + lane * kGatherSlotFloats)),
            "l"(tmap), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(b)
            : "memory");
    uint32_t done = 0;
    for (unsigned int spins = 0; !done; ++spins) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(b)
            : "memory");
        if (!done && spins > kGatherWaitLimit) return gather_wait_overdue(b);
    }
    return true;
}

// Adjacent common prefix delta(i, i+1), i in [0, n-2].
template <typename KeyT>
__device__ __forceinline__ int delta_adj(const KeyT* __restrict__ keys, int kbits, uint32_t i) {
    const KeyT x = __ldcg(keys + i) ^ __ldcg(keys + i + 1);
    if (x != 0) return clz_key<KeyT>(x) - ((int)(8 * sizeof(KeyT)) - kbits);
    return kbits + __clz(i ^ (i + 1));
}

// Tree emission and refit in one bottom-up pass (one thread per leaf).
//
// The binary radix tree of constructBinaryRadixTree (lbvh_construction.cl:
// 342-410) is the unique tree in which a node covering sorted positions
// [lo, hi] has as parent the node that extends it towards the neighbour with
// the longer common prefix: to the right (split = hi, this node is child 0)
// when delta(hi, hi+1) > delta(lo-1, lo), else to the left (split = lo-1,
// child 1).  The two deltas never tie for distinct extended keys.  So each
// leaf thread climbs: it writes its box, reference and far range end into the
// parent's child slot, and the second of the two children to arrive (an
// arrival word per node, acquire / release ordered) merges both boxes and
// continues upwards, exactly as calcNodeAABBs (:415-492) climbs.  Internal
// nodes are stored at index = split position; the reference's index of a node
// (its hi if it is child 0, its lo if child 1, 0 for the root) is recorded for
// the reference-layout export, and children and visiting order are the
// reference's.

__device__ __forceinline__ void tri_box(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                                        const float4* stage, uint32_t t, float box[6]) {
    const TriVerts tv = load_tri_staged(vx, vy, vz, tri, stage, t);
    for (int k = 0; k < 3; ++k) {
        box[k] = fminf(tv.p[0][k], fminf(tv.p[1][k], tv.p[2][k]));
        box[3 + k] = fmaxf(tv.p[0][k], fmaxf(tv.p[1][k], tv.p[2][k]));
    }
}

// Arrival word of a node whose children finish in different blocks (the
// tree pass's `counters`, zeroed by the Morton pass): bits 0-1 count the
// children delivered, kArrReady says the first child's slot is written, and
// bits 16-23 hold delta + 1 at the first child's far range end.  The first
// arrival writes its slot and then publishes it with a release-ordered OR;
// the second arrival's acquiring add usually finds the slot published
// already, so a level of the climb costs one atomic and one slot load.
constexpr unsigned int kArrReady = 0x100u;

__device__ __forceinline__ unsigned int atom_add_acquire_gpu(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.add.acquire.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void red_or_release_gpu(unsigned int* p, unsigned int v) {
    asm volatile("red.release.gpu.global.or.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Child slot `slot` of node `nd`: box, reference, the child's far range end.
__device__ __forceinline__ void write_slot(float* nd, int slot, const float box[6], uint32_t ref, uint32_t far_in) {
    float2* b2 = reinterpret_cast<float2*>(nd + 6 * slot);
    __stcg(b2 + 0, make_float2(box[0], box[1]));
    __stcg(b2 + 1, make_float2(box[2], box[3]));
    __stcg(b2 + 2, make_float2(box[4], box[5]));
    unsigned int* w = reinterpret_cast<unsigned int*>(nd);
    __stcg(w + 12 + slot, ref);
    __stcg(w + 14 + slot, far_in);
}

// The device-scope climb from a finished node [lo, hi] (reference `ref`, box
// `box`, d_lo = delta(lo-1, lo) and d_hi = delta(hi, hi+1), -1 past the
// array's ends): deliver into the parent's child slot; the second arrival
// merges the sibling's box and continues with the parent.
template <typename KeyT>
__device__ __forceinline__ void climb_global(const KeyT* __restrict__ keys, uint32_t n, int kbits,
                                             float* __restrict__ nodes, unsigned int* __restrict__ counters,
                                             uint32_t* __restrict__ karras_idx, float* __restrict__ root_box,
                                             uint32_t lo, uint32_t hi, int d_lo, int d_hi, uint32_t ref,
                                             float box[6]) {
    // every level up adds at least one common bit of the (3b + 32)-bit key
    for (int step = 0; step <= kMaxDepth; ++step) {
        if (lo == 0 && hi == n - 1) {
            root_box[0] = box[0]; root_box[1] = box[1]; root_box[2] = box[2];
            root_box[3] = __uint_as_float(ref);
            root_box[4] = box[3]; root_box[5] = box[4]; root_box[6] = box[5];
            root_box[7] = 0.f;
            return;
        }
        // the parent extends towards the larger adjacent delta (lo == 0 and
        // hi == n - 1 give -1 on their side)
        const bool left = d_hi > d_lo;
        const uint32_t split = left ? hi : lo - 1;
        const int slot = left ? 0 : 1;
        float* nd = nodes + 16u * split;
        unsigned int* ctr = counters + split;
        const unsigned int old = atom_add_acquire_gpu(ctr, 1u);
        write_slot(nd, slot, box, ref, left ? lo : hi);
        if ((old & 3u) == 0u) {
            red_or_release_gpu(ctr, kArrReady | ((unsigned int)((left ? d_lo : d_hi) + 1) << 16));
            return;
        }
        unsigned int word = old;
        for (unsigned int spins = 0; !(word & kArrReady); ++spins) {
            if (spins > kSpinLimit) {  // the sibling never published: report, never read its slot
                clr_raise(CLR_DEVERR_REFIT);
                return;
            }
            if (spins > 64) __nanosleep(32);
            word = ld_acquire_gpu(ctr);
        }
        const int d_sib = (int)((word >> 16) & 0xFFu) - 1;
        const float* sb = nd + 6 * (1 - slot);
        float b[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) b[k] = __ldcg(sb + k);
        const uint32_t far_end = __ldcg(reinterpret_cast<const unsigned int*>(nd) + 14 + (1 - slot));
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            box[k] = fminf(box[k], b[k]);
            box[3 + k] = fmaxf(box[3 + k], b[3 + k]);
        }
        if (left) {
            hi = far_end;
            d_hi = d_sib;
        } else {
            lo = far_end;
            d_lo = d_sib;
        }
        if (lo > hi || hi >= n) break;  // corrupt slot: report, never index out of range
        ref = split;
    }
    clr_raise(CLR_DEVERR_REFIT);
}

// The same, from a node whose outer deltas are read from the keys.
template <typename KeyT>
__device__ __forceinline__ void climb_global_from(const KeyT* __restrict__ keys, uint32_t n, int kbits,
                                                  float* __restrict__ nodes, unsigned int* __restrict__ counters,
                                                  uint32_t* __restrict__ karras_idx, float* __restrict__ root_box,
                                                  uint32_t lo, uint32_t hi, uint32_t ref, float box[6]) {
    const int d_lo = lo == 0 ? -1 : delta_adj(keys, kbits, lo - 1);
    const int d_hi = hi + 1 >= n ? -1 : delta_adj(keys, kbits, hi);
    climb_global<KeyT>(keys, n, kbits, nodes, counters, karras_idx, root_box, lo, hi, d_lo, d_hi, ref, box);
}

// Leaf j's climb over one tree of n leaves.  All arrays are the tree's own
// (offset to its first leaf); sidx holds vertex-array triangle ids, recorded
// minus id_base.
template <typename KeyT>
__device__ __forceinline__ void tree_climb(const KeyT* __restrict__ keys, const uint32_t* __restrict__ sidx,
                                           uint32_t n, int kbits, const float* __restrict__ vx,
                                           const float* __restrict__ vy, const float* __restrict__ vz,
                                           const uint32_t* __restrict__ tri, const float4* __restrict__ stage,
                                           float* __restrict__ nodes,
                                           float4* __restrict__ tris, unsigned int* __restrict__ counters,
                                           uint32_t* __restrict__ karras_idx, float* __restrict__ root_box,
                                           uint32_t j, uint32_t id_base) {
    float box[6];
    const uint32_t tj = __ldg(sidx + j);
    emit_leaf(vx, vy, vz, tri, stage, tj, tj - id_base, j, tris, box);
    // adjacent deltas around leaf j (-1 outside the array)
    const int dl = j > 0 ? delta_adj(keys, kbits, j - 1) : -1;
    const int dj = j + 1 < n ? delta_adj(keys, kbits, j) : -1;
    const bool j_left = (j == 0) || (j != n - 1 && dj > dl);
    uint32_t lo = j, hi = j, ref = j | kLeafBit;
    // A node whose two children are the leaves j and j+1 is finished by leaf
    // j's thread alone (no arrival counter); leaf j+1's thread stops here.
    if (j > 0 && !j_left) {
        const int dll = j > 1 ? delta_adj(keys, kbits, j - 2) : -1;
        const bool prev_left = (j - 1 == 0) || (dl > dll);
        if (prev_left) return;  // leaf j-1 builds our common parent
    }
    if (j_left && j + 1 < n) {
        const int dr = j + 2 < n ? delta_adj(keys, kbits, j + 1) : -1;
        const bool next_right = (j + 1 == n - 1) || (dr < dj);
        if (next_right) {
            float b1[6];
            tri_box(vx, vy, vz, tri, stage, __ldg(sidx + j + 1), b1);
            float* nd = nodes + 16u * j;
            float4* n4 = reinterpret_cast<float4*>(nd);
            n4[0] = make_float4(box[0], box[1], box[2], box[3]);
            n4[1] = make_float4(box[4], box[5], b1[0], b1[1]);
            n4[2] = make_float4(b1[2], b1[3], b1[4], b1[5]);
            n4[3] = make_float4(__uint_as_float(j | kLeafBit), __uint_as_float((j + 1) | kLeafBit),
                                __uint_as_float(j), __uint_as_float(j + 1));
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                box[k] = fminf(box[k], b1[k]);
                box[3 + k] = fmaxf(box[3 + k], b1[3 + k]);
            }
            hi = j + 1;
            ref = j;
        }
    }
    climb_global_from<KeyT>(keys, n, kbits, nodes, counters, karras_idx, root_box, lo, hi, ref, box);
}

// The same climb with block-local merging.  Block b owns leaves [B, E]
// (kTreeBlock consecutive positions).  The node split at s covers the maximal
// range around s whose other adjacent deltas all exceed delta(s, s+1), so it
// lies inside [B, E] exactly when some delta(k, k+1) < delta(s, s+1) exists
// for k in [B-1, s-1] and for k in [s+1, E] (out-of-array deltas count as
// -1).  The block finds these nodes with prefix / suffix minima of its deltas;
// both children of such a node are finished by threads of the block, which
// meet in shared memory (CTA-scope acq_rel counter, no device fence), and the
// second writes the whole 64-byte node.  A node that crosses a block edge is
// reached by threads of two blocks and uses the device-scope protocol of
// tree_climb; so are all its ancestors.
constexpr int kTreeBlock = 128;
// largest tree whose block-crossing climbs run inside the tree pass
constexpr uint32_t kClimbHereMaxTris = 2u << 20;

__device__ __forceinline__ unsigned int atomic_add_acq_rel_cta(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.add.acq_rel.cta.shared::cta.u32 %0, [%1], %2;"
                 : "=r"(old)
                 : "r"((unsigned int)__cvta_generic_to_shared(p)), "r"(v)
                 : "memory");
    return old;
}

template <typename KeyT, bool kWide, bool kTma>
__global__ void __launch_bounds__(kTreeBlock, 16) k_build_tree(const __grid_constant__ CUtensorMap stage_map,
                                                           const KeyT* __restrict__ keys,
                                                           const uint32_t* __restrict__ sidx, uint32_t n, int kbits,
                                                           const float* __restrict__ vx, const float* __restrict__ vy,
                                                           const float* __restrict__ vz, const uint32_t* __restrict__ tri,
                                                           const float4* __restrict__ stage,
                                                           float* __restrict__ nodes, float4* __restrict__ tris,
                                                           unsigned int* __restrict__ counters,
                                                           uint32_t* __restrict__ karras_idx,
                                                           float* __restrict__ root_box,
                                                           uint32_t* __restrict__ worklist,
                                                           unsigned int* __restrict__ wl_count,
                                                           int climb_here) {
    __shared__ int s_d[kTreeBlock + 1];           // delta(k, k+1), k = B-1 .. E
    __shared__ int s_wmin[3][kTreeBlock / 32];     // per warp: prefix min, suffix min from lanes 0 and 1
    __shared__ unsigned char s_local[kTreeBlock];  // node split at B + i lies inside the block
    // child slots of the block's nodes: {box min xyz, box max x}, {box max yz, ref, far end}
    __shared__ __align__(16) float4 s_slot[kTreeBlock][2][2];
    __shared__ unsigned int s_cnt[kTreeBlock];
    // staging records gathered by TMA (kTma) and each warp's mbarrier
    __shared__ __align__(128) float s_rec[kTma ? (kTreeBlock / 4) * kGatherSlotFloats : 1];
    __shared__ __align__(8) uint64_t s_bar[kTreeBlock / 32];
    const uint32_t B = blockIdx.x * kTreeBlock;
    const uint32_t E = min(B + kTreeBlock - 1, n - 1);
    const int nd = (int)(E - B) + 2;  // entries of s_d (<= kTreeBlock + 1)
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t j = B + t;
    constexpr int kBig = 0x7FFFFFFF;
    for (int i = t; i < nd; i += kTreeBlock) {
        const int64_t k = (int64_t)B - 1 + i;
        s_d[i] = (k < 0 || k + 1 >= (int64_t)n) ? -1 : delta_adj(keys, kbits, (uint32_t)k);
    }
    s_cnt[t] = 0u;
    __syncthreads();
    // prefix minimum pm = min(s_d[0..t]) and the suffix minimum from t+2,
    // by warp shuffles and per-warp minima; s_d[256] (if present) is last
    const int v = t < nd ? s_d[t] : kBig;
    int pm = v, sm = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(0xFFFFFFFFu, pm, o), b = __shfl_down_sync(0xFFFFFFFFu, sm, o);
        if (lane >= o) pm = min(pm, a);
        if (lane + o < 32) sm = min(sm, b);
    }
    const int sm2 = __shfl_down_sync(0xFFFFFFFFu, sm, 2);
    if (lane == 31) s_wmin[0][warp] = pm;
    if (lane == 0) s_wmin[1][warp] = sm;
    if (lane == 1) s_wmin[2][warp] = sm;
    __syncthreads();
    for (int w = 0; w < warp; ++w) pm = min(pm, s_wmin[0][w]);
    const int tail = nd == kTreeBlock + 1 ? s_d[kTreeBlock] : kBig;
    int after = tail;  // min of s_d over the warps after this one
    for (int w = warp + 1; w < kTreeBlock / 32; ++w) after = min(after, s_wmin[1][w]);
    int s2;  // min(s_d[t+2 ..])
    if (lane < 30) {
        s2 = min(sm2, after);
    } else if (lane == 30) {
        s2 = after;
    } else if (warp + 1 < kTreeBlock / 32) {
        int after2 = tail;
        for (int w = warp + 2; w < kTreeBlock / 32; ++w) after2 = min(after2, s_wmin[1][w]);
        s2 = min(s_wmin[2][warp + 1], after2);
    } else {
        s2 = kBig;
    }
    // the node split at B + t (s_d index t + 1) lies inside the block when a
    // smaller delta bounds it on both sides within the block's window
    if (t + 1 < nd - 1) {
        const int ds = s_d[t + 1];
        s_local[t] = (pm < ds && s2 < ds) ? 1 : 0;
    }
    __syncthreads();
    auto block_local = [&](uint32_t split) -> bool {
        return split >= B && split < E && s_local[split - B] != 0;
    };
    // leaves: record and box; the box goes to the left neighbour lane, which
    // merges two adjacent leaves whose parent is their own node (no block
    // barrier after this: a warp climbs while the block's other warps gather)
    float box[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (kTma) {
        if (B + 32u * warp < n) {  // the warp has leaves
            const uint32_t tj = j < n ? __ldg(sidx + j) : 0u;
            float* rows = s_rec + 8 * warp * kGatherSlotFloats;
            if (gather_warp_records(&stage_map, &s_bar[warp], rows, tj) && j < n) {
                const float* r = rows + (lane >> 2) * kGatherSlotFloats + (lane & 3) * kStageFloats;
                TriVerts tv;
#pragma unroll
                for (int k = 0; k < 9; ++k) tv.p[k / 3][k % 3] = r[k];
                emit_leaf_verts(tv, tj, j, tris, box);
            }
        }
    } else if (j < n) {
        const uint32_t tj = __ldg(sidx + j);
        emit_leaf(vx, vy, vz, tri, stage, tj, tj, j, tris, box);
    }
    float nbox[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) nbox[k] = __shfl_down_sync(0xFFFFFFFFu, box[k], 1);
    if (j >= n) return;
    const int dl = s_d[t];      // delta(j-1, j)
    const int dj = s_d[t + 1];  // delta(j, j+1)
    const bool j_left = (j == 0) || (j != n - 1 && dj > dl);
    uint32_t lo = j, hi = j, ref = j | kLeafBit;
    if (j > 0 && !j_left) {
        const int dll = j < 2 ? -1 : (t >= 1 ? s_d[t - 1] : delta_adj(keys, kbits, j - 2));
        const bool prev_left = (j - 1 == 0) || (dl > dll);
        if (prev_left) return;  // leaf j-1 builds our common parent
    }
    if (j_left && j + 1 < n) {
        const int dr = j + 2 >= n ? -1 : (t + 2 < nd ? s_d[t + 2] : delta_adj(keys, kbits, j + 1));
        const bool next_right = (j + 1 == n - 1) || (dr < dj);
        if (next_right) {
            float b1[6];
            if (lane < 31) {
#pragma unroll
                for (int k = 0; k < 6; ++k) b1[k] = nbox[k];
            } else {
                tri_box(vx, vy, vz, tri, stage, __ldg(sidx + j + 1), b1);
            }
            st_node(nodes + 16u * j, kWide, make_float4(box[0], box[1], box[2], box[3]),
                    make_float4(box[4], box[5], b1[0], b1[1]), make_float4(b1[2], b1[3], b1[4], b1[5]),
                    make_float4(__uint_as_float(j | kLeafBit), __uint_as_float((j + 1) | kLeafBit),
                                __uint_as_float(j), __uint_as_float(j + 1)));
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                box[k] = fminf(box[k], b1[k]);
                box[3 + k] = fmaxf(box[3 + k], b1[3 + k]);
            }
            hi = j + 1;
            ref = j;
        }
    }
    bool local = true;  // false once the climb has left the block
    for (int step = 0; step <= kMaxDepth; ++step) {
        if (lo == 0 && hi == n - 1) {
            root_box[0] = box[0]; root_box[1] = box[1]; root_box[2] = box[2];
            root_box[3] = __uint_as_float(ref);
            root_box[4] = box[3]; root_box[5] = box[4]; root_box[6] = box[5];
            root_box[7] = 0.f;
            return;
        }
        // delta(hi, hi+1) and delta(lo-1, lo): from shared memory inside the
        // block's window, -1 past the array's ends
        const int d_hi = hi + 1 >= n ? -1 : (hi >= B && hi <= E) ? s_d[hi - B + 1] : delta_adj(keys, kbits, hi);
        const int d_lo = lo == 0 ? -1 : (lo >= B && lo <= E + 1) ? s_d[lo - B] : delta_adj(keys, kbits, lo - 1);
        const bool left = (lo == 0) || (hi != n - 1 && d_hi > d_lo);
        const uint32_t split = left ? hi : lo - 1;
        const int slot = left ? 0 : 1;
        const uint32_t far_in = left ? lo : hi;
        local = local && block_local(split);
        uint32_t far_end;
        if (local) {
            const int ls = (int)(split - B);
            s_slot[ls][slot][0] = make_float4(box[0], box[1], box[2], box[3]);
            s_slot[ls][slot][1] = make_float4(box[4], box[5], __uint_as_float(ref), __uint_as_float(far_in));
            if (atomic_add_acq_rel_cta(&s_cnt[ls], 1u) == 0u) return;
            const float4 a0 = s_slot[ls][0][0], a1 = s_slot[ls][0][1];
            const float4 c0 = s_slot[ls][1][0], c1 = s_slot[ls][1][1];
            far_end = __float_as_uint(slot == 0 ? c1.w : a1.w);
            st_node(nodes + 16u * split, kWide, a0, make_float4(a1.x, a1.y, c0.x, c0.y),
                    make_float4(c0.z, c0.w, c1.x, c1.y), make_float4(a1.z, c1.z, a1.w, c1.w));
            box[0] = fminf(a0.x, c0.x);
            box[1] = fminf(a0.y, c0.y);
            box[2] = fminf(a0.z, c0.z);
            box[3] = fmaxf(a0.w, c0.w);
            box[4] = fmaxf(a1.x, c1.x);
            box[5] = fmaxf(a1.y, c1.y);
        } else {
            if (climb_here) {
                // small trees: continue with the device-scope climb right here
                // (its waits are for first arrivals, which are running)
                climb_global<KeyT>(keys, n, kbits, nodes, counters, karras_idx, root_box, lo, hi, d_lo, d_hi, ref,
                                   box);
                return;
            }
            // first node across a block edge: deliver this child; the second
            // arrival hands the finished node to k_build_tree_top, so that this
            // block retires instead of waiting on device-scope climbs.  Both
            // slots are read only after this kernel, so no ordering is needed
            // here; the first arrival's word still carries kArrReady and its
            // far-end delta for a second arrival in k_build_tree_top.
            const unsigned int old = atomicAdd(counters + split, 1u);
            write_slot(nodes + 16u * split, slot, box, ref, far_in);
            if ((old & 3u) == 0u) {
                atomicOr(counters + split, kArrReady | ((unsigned int)((left ? d_lo : d_hi) + 1) << 16));
                return;
            }
            worklist[atomicAdd(wl_count, 1u)] = split;
            return;
        }
        if (left) hi = far_end;
        else lo = far_end;
        if (lo > hi || hi >= n) break;  // corrupt slot: report, never index out of range
        ref = split;
    }
    clr_raise(CLR_DEVERR_REFIT);
}

// The nodes across block edges finished by k_build_tree: each continues the
// device-scope climb from its merged box and range.
template <typename KeyT>
__global__ void __launch_bounds__(256) k_build_tree_top(const KeyT* __restrict__ keys, uint32_t n, int kbits,
                                                        float* __restrict__ nodes, unsigned int* __restrict__ counters,
                                                        uint32_t* __restrict__ karras_idx, float* __restrict__ root_box,
                                                        const uint32_t* __restrict__ worklist,
                                                        const unsigned int* __restrict__ wl_count) {
    const uint32_t cnt = *wl_count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const uint32_t split = worklist[i];
        if (split + 1 >= n) {  // corrupt entry: report, never index out of range
            clr_raise(CLR_DEVERR_REFIT);
            continue;
        }
        const float* nd = nodes + 16u * split;
        const unsigned int* w = reinterpret_cast<const unsigned int*>(nd);
        float b[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) b[k] = __ldcg(nd + k);
        float box[6];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            box[k] = fminf(b[k], b[6 + k]);
            box[3 + k] = fmaxf(b[3 + k], b[9 + k]);
        }
        const uint32_t lo = __ldcg(w + 14), hi = __ldcg(w + 15);
        if (lo > hi || hi >= n) {
            clr_raise(CLR_DEVERR_REFIT);
            continue;
        }
        climb_global_from<KeyT>(keys, n, kbits, nodes, counters, karras_idx, root_box, lo, hi, split, box);
    }
}

// Single-triangle scene: one leaf, no internal node (the reference requires
// at least two triangles; here traversal treats the leaf as the root).
__global__ void k_single(const float* vx, const float* vy, const float* vz, const uint32_t* tri, float4* tris,
                         float* root_box) {
    float box[6];
    emit_leaf(vx, vy, vz, tri, nullptr, 0u, 0u, 0u, tris, box);
    for (int k = 0; k < 3; ++k) { root_box[k] = box[k]; root_box[4 + k] = box[3 + k]; }
    root_box[3] = __uint_as_float(kLeafBit);
    root_box[7] = 0.f;
}

// --------------------------------------------------------- reference export

// The reference's index of every internal node, from its parent's slots: a
// child 0 covers [lo, p] and is indexed by its hi (= the parent's split p), a
// child 1 covers [p+1, hi] and is indexed by its lo (= p + 1); the root is 0.
__global__ void k_karras_index(const float4* __restrict__ nodes, const float* __restrict__ root_box, uint32_t n,
                               uint32_t* __restrict__ karras_idx) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        const uint32_t root = __float_as_uint(root_box[3]);
        if (!(root & kLeafBit) && root + 1 < n) karras_idx[root] = 0;
    }
    if (p >= n - 1) return;
    const float4 r = nodes[4u * p + 3];
    const uint32_t c0 = __float_as_uint(r.x), c1 = __float_as_uint(r.y);
    if (!(c0 & kLeafBit) && c0 + 1 < n) karras_idx[c0] = p;
    if (!(c1 & kLeafBit) && c1 + 1 < n) karras_idx[c1] = p + 1;
}

// Node a (stored at its split position) becomes InternalNode[karras_idx[a]]
// with children c = {a, a+1}: in the reference's numbering a child-0 internal
// node is indexed by its hi (= a) and a child-1 internal node by its lo (= a+1).
__global__ void k_export(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                         const uint32_t* __restrict__ karras_idx, uint32_t n, uint8_t* __restrict__ inodes,
                         uint8_t* __restrict__ lnodes, uint32_t* __restrict__ parents) {
    const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n - 1) return;
    const uint32_t k = karras_idx[a];
    const float4 q0 = nodes[4u * a], q1 = nodes[4u * a + 1], q2 = nodes[4u * a + 2], r = nodes[4u * a + 3];
    const float bx[2][6] = {{q0.x, q0.y, q0.z, q0.w, q1.x, q1.y}, {q1.z, q1.w, q2.x, q2.y, q2.z, q2.w}};
    const bool is_leaf[2] = {(__float_as_uint(r.x) & kLeafBit) != 0, (__float_as_uint(r.y) & kLeafBit) != 0};
    if (inodes) {
        float* f = reinterpret_cast<float*>(inodes + 48u * k);
        for (int c = 0; c < 3; ++c) {
            f[c] = fminf(bx[0][c], bx[1][c]);
            f[4 + c] = fmaxf(bx[0][3 + c], bx[1][3 + c]);
        }
        f[3] = 0.f;
        f[7] = 0.f;
        uint8_t* ch = inodes + 48u * k + 32u;
        ch[0] = is_leaf[0];
        ch[1] = is_leaf[1];
        ch[2] = ch[3] = 0;
        uint32_t* cc = reinterpret_cast<uint32_t*>(inodes + 48u * k + 36u);
        cc[0] = a;
        cc[1] = a + 1;
        cc[2] = 0;
    }
    for (int s = 0; s < 2; ++s) {
        const uint32_t child = a + s;
        if (parents) parents[is_leaf[s] ? child : n + child] = k;
        if (is_leaf[s] && lnodes) {
            float* f = reinterpret_cast<float*>(lnodes + 48u * child);
            for (int c = 0; c < 3; ++c) { f[c] = bx[s][c]; f[4 + c] = bx[s][3 + c]; }
            f[3] = 0.f;
            f[7] = 0.f;
            uint32_t* u = reinterpret_cast<uint32_t*>(lnodes + 48u * child + 32u);
            u[0] = __float_as_uint(tris[3u * child].w);
            u[1] = u[2] = u[3] = 0;
        }
    }
    if (k == 0 && parents) parents[n] = 0xFFFFFFFFu;
}

__global__ void k_export_single(const float* __restrict__ root_box, const float4* __restrict__ tris,
                                uint8_t* __restrict__ lnodes, uint32_t* __restrict__ parents) {
    if (lnodes) {
        float* f = reinterpret_cast<float*>(lnodes);
        for (int k = 0; k < 8; ++k) f[k] = root_box[k];
        f[3] = 0.f;
        uint32_t* u = reinterpret_cast<uint32_t*>(lnodes + 32);
        u[0] = __float_as_uint(tris[0].w);
        u[1] = u[2] = u[3] = 0;
    }
    if (parents) parents[0] = 0xFFFFFFFFu;
}

template <typename KeyT>
__global__ void k_keys_to_u64(const KeyT* __restrict__ in, uint64_t* __restrict__ out, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint64_t)in[i];
}

// ------------------------------------------------- segmented (batched) build
//
// Many scenes in one build: scene s owns triangles [off[s], off[s+1]) of the
// concatenated arrays.  Each scene is quantised in its own box, its keys carry
// the scene id above the 3b Morton bits (so one stable sort keeps scenes
// apart and each scene's order is its standalone order), and each scene's
// tree is climbed with scene-local positions and ids.  The deltas of two keys
// of one scene are the standalone deltas (the id bits are equal), so every
// scene's nodes, triangle records and root are bit-identical to a build of
// that scene alone.

constexpr uint32_t kSegBoxChunk = 4096;  // triangles per block of k_seg_box

// The scene owning position i: the largest s < nseg with off[s] <= i.
__device__ __forceinline__ uint32_t seg_of(const uint32_t* __restrict__ off, uint32_t nseg, uint32_t i) {
    uint32_t lo = 0, hi = nseg;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void seg_box_flush(unsigned int* __restrict__ boxw, uint32_t s, const float mn[3],
                                              const float mx[3]) {
    for (int k = 0; k < 3; ++k) {
        if (mn[k] == mn[k]) atomicMax(boxw + 6u * s + k, ~float_to_ordered(mn[k]));
        if (mx[k] == mx[k]) atomicMax(boxw + 6u * s + 3 + k, float_to_ordered(mx[k]));
    }
}

// Per-scene bounds of the triangles' vertices (k_scene_box per scene).
__global__ void __launch_bounds__(256) k_seg_box(const float* __restrict__ vx, const float* __restrict__ vy,
                                                 const float* __restrict__ vz, const uint32_t* __restrict__ tri,
                                                 const uint32_t* __restrict__ off, uint32_t nseg, uint32_t n,
                                                 unsigned int* __restrict__ boxw) {
    const uint32_t t0 = blockIdx.x * kSegBoxChunk, t1 = min(t0 + kSegBoxChunk, n);
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t cur = 0xFFFFFFFFu;
    for (uint32_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        const uint32_t s = seg_of(off, nseg, t);
        if (s != cur) {
            if (cur != 0xFFFFFFFFu) seg_box_flush(boxw, cur, mn, mx);
            cur = s;
            for (int k = 0; k < 3; ++k) {
                mn[k] = INFINITY;
                mx[k] = -INFINITY;
            }
        }
        const TriVerts tv = load_tri(vx, vy, vz, tri, t);
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k) {
                mn[k] = fminf(mn[k], tv.p[v][k]);
                mx[k] = fmaxf(mx[k], tv.p[v][k]);
            }
    }
    // a warp whose lanes all end in one scene combines before the atomics
    const unsigned int act = __activemask();
    const uint32_t s0 = __shfl_sync(act, cur, __ffs(act) - 1);
    if (__all_sync(act, cur == s0) && act == 0xFFFFFFFFu) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = warp_min(mn[k]);
            mx[k] = warp_max(mx[k]);
        }
        if ((threadIdx.x & 31) == 0 && cur != 0xFFFFFFFFu) seg_box_flush(boxw, cur, mn, mx);
    } else if (cur != 0xFFFFFFFFu) {
        seg_box_flush(boxw, cur, mn, mx);
    }
}

// Keys (scene id << 3b | Morton code of the centroid in the scene's box) and
// the digit histograms of every sort pass.
template <int kBits>
__global__ void __launch_bounds__(256) k_morton_seg(const float* __restrict__ vx, const float* __restrict__ vy,
                                                    const float* __restrict__ vz, const uint32_t* __restrict__ tri,
                                                    const uint32_t* __restrict__ off, uint32_t nseg, uint32_t n,
                                                    uint32_t bits, const unsigned int* __restrict__ boxw,
                                                    uint64_t* __restrict__ keys, unsigned int* __restrict__ hist,
                                                    int npasses, unsigned int* __restrict__ counters,
                                                    float4* __restrict__ stage) {
    constexpr uint32_t kMask = (1u << kBits) - 1u;
    __shared__ unsigned int sh[kMaxPasses * kRadix];
    for (int i = threadIdx.x; i < npasses * kRadix; i += blockDim.x) sh[i] = 0;
    const uint32_t numDivs = 1u << bits;
    const float fDivs = (float)numDivs;
    __syncthreads();
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t s = seg_of(off, nseg, t);
        float smin[3], ssize[3];
        load_scene_box(boxw + 6u * s, smin, ssize);
        const TriVerts tv = load_tri(vx, vy, vz, tri, t);
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            const float mn = fminf(tv.p[0][k], fminf(tv.p[1][k], tv.p[2][k]));
            const float mx = fmaxf(tv.p[0][k], fmaxf(tv.p[1][k], tv.p[2][k]));
            const float center = fmul(fadd(mn, mx), 0.5f);
            const float normPos = fdiv(fsub(center, smin[k]), ssize[k]);
            const uint32_t v = __float2uint_rz(fmul(normPos, fDivs));
            q[k] = min(v, numDivs - 1u);
        }
        const uint64_t key = ((uint64_t)s << (3 * bits)) | make_key<uint64_t>(q[0], q[1], q[2]);
        keys[t] = key;
        if (stage) stage_tri(stage, t, tv.p);
        counters[t] = 0u;
        for (int p = 0; p < npasses; ++p) atomicAdd(&sh[p * kRadix + (uint32_t)((key >> (kBits * p)) & kMask)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npasses * kRadix; i += blockDim.x)
        if (sh[i]) atomicAdd(hist + i, sh[i]);
}

// One thread per leaf; each climbs its own scene's tree.
template <typename KeyT>
__global__ void __launch_bounds__(256) k_build_tree_seg(const KeyT* __restrict__ keys,
                                                        const uint32_t* __restrict__ sidx,
                                                        const uint32_t* __restrict__ off, uint32_t nseg, uint32_t n,
                                                        int kbits, const float* __restrict__ vx,
                                                        const float* __restrict__ vy, const float* __restrict__ vz,
                                                        const uint32_t* __restrict__ tri,
                                                        const float4* __restrict__ stage, float* __restrict__ nodes,
                                                        float4* __restrict__ tris, unsigned int* __restrict__ counters,
                                                        uint32_t* __restrict__ karras_idx,
                                                        float* __restrict__ root_boxes) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t s = seg_of(off, nseg, j);
    const uint32_t s0 = __ldg(off + s), ns = __ldg(off + s + 1) - s0;
    tree_climb<KeyT>(keys + s0, sidx + s0, ns, kbits, vx, vy, vz, tri, stage, nodes + 16ull * s0, tris + 3ull * s0,
                     counters + s0, karras_idx + s0, root_boxes + 8ull * s, j - s0, s0);
}

}  // namespace clr

// =============================================================== host side

using namespace clr;

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Lays the scratch pool out for `cap` triangles.  Returns its size; assigns
// the handle's pointers when `base` is non-NULL.
// Digit histogram (added to a zeroed `hist`, one 256-thread block each) of the
// low 8 bits of n keys, the stall test's input, and the
// tile counter set so that the next block to start takes tile 1.
__global__ void k_debug_hist(const uint32_t* __restrict__ keys, uint32_t n, unsigned int* __restrict__ hist,
                             unsigned int* __restrict__ tile_ctr) {
    __shared__ unsigned int h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[keys[i] & 0xFFu], 1u);
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) *tile_ctr = 1u;
    if (h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

// Polls of a look-back before a sort pass gives up (CLR_DEVERR_SORT_TIMEOUT);
// lowered only by clr_debug_set_wait_limits.
static unsigned int g_sort_spin_limit = kSpinLimit;

static size_t pool_layout(clr_lbvh* h, uint32_t cap, char* base, bool stage = true) {
    const size_t tiles = div_up(cap ? cap : 1, kMinSortTile) + 1;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const size_t o_keys0 = take(8ull * cap), o_keys1 = take(8ull * cap);
    const size_t o_vals0 = take(4ull * cap), o_vals1 = take(4ull * cap);
    const size_t o_kidx = take(4ull * cap), o_cnt = take(4ull * cap);
    const size_t o_stage = stage ? take(48ull * cap) : 0;
    // the region cleared per build: histograms, tile counters and scene box
    // first, then the look-back words, of which a build clears only the
    // passes and tiles it uses (zero_prefix_bytes)
    const size_t o_zero = off;
    const size_t o_hist = take(4ull * kMaxPasses * kRadix);
    const size_t o_tiles = take(4ull * (kMaxPasses + 1));  // + the tree pass's worklist count
    const size_t o_box = take(4ull * 8);
    const size_t o_status = take(4ull * kMaxPasses * tiles * kRadix);
    if (base) {
        h->keys[0] = base + o_keys0;
        h->keys[1] = base + o_keys1;
        h->vals[0] = reinterpret_cast<uint32_t*>(base + o_vals0);
        h->vals[1] = reinterpret_cast<uint32_t*>(base + o_vals1);
        h->karras_idx = reinterpret_cast<uint32_t*>(base + o_kidx);
        h->stage = stage ? reinterpret_cast<float4*>(base + o_stage) : nullptr;
        h->counters = reinterpret_cast<unsigned int*>(base + o_cnt);
        h->zero_region = base + o_zero;
        h->zero_bytes = off - o_zero;
        h->hist = reinterpret_cast<unsigned int*>(base + o_hist);
        h->status = reinterpret_cast<unsigned int*>(base + o_status);
        h->status_stride = tiles * kRadix;
        h->zero_prefix_bytes = o_status - o_zero;
        h->tile_ctr = reinterpret_cast<unsigned int*>(base + o_tiles);
        h->boxw = reinterpret_cast<unsigned int*>(base + o_box);
        h->pool_bytes = off;
    }
    return off;
}

static int pool_grow(clr_lbvh* h, uint32_t cap) {
    if (h->pool && cap <= h->capacity) return CLR_OK;
    if (h->pool) {
        cudaFree(h->pool);
        h->pool = nullptr;
    }
    const size_t bytes = pool_layout(h, cap, nullptr);
    if (cudaMalloc(&h->pool, bytes) != cudaSuccess) {
        cudaGetLastError();
        h->pool = nullptr;
        h->capacity = 0;
        return clr_set_error(CLR_ENOMEM, "cudaMalloc(%zu) for the LBVH scratch pool failed", bytes);
    }
    h->capacity = cap;
    pool_layout(h, cap, static_cast<char*>(h->pool));
    return CLR_OK;
}

extern "C" int clr_lbvh_create(uint32_t capacity, clr_lbvh** out) {
    if (!out) return clr_set_error(CLR_EINVAL, "clr_lbvh_create: out is NULL");
    clr_lbvh* h = new (std::nothrow) clr_lbvh{};
    if (!h) return clr_set_error(CLR_ENOMEM, "clr_lbvh_create: host allocation failed");
    int rc = pool_grow(h, capacity > 0 ? capacity : 1);
    if (rc != CLR_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return CLR_OK;
}

extern "C" int clr_lbvh_destroy(clr_lbvh* h) {
    if (!h) return CLR_OK;
    if (h->pool) cudaFree(h->pool);
    if (h->seg_pool) cudaFree(h->seg_pool);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    for (int s = 0; s < 2; ++s) {
        if (h->in_buf[s]) cudaFree(h->in_buf[s]);
        if (h->in_copied[s]) cudaEventDestroy(h->in_copied[s]);
        if (h->in_consumed[s]) cudaEventDestroy(h->in_consumed[s]);
    }
    if (h->copy_gate) cudaEventDestroy(h->copy_gate);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    delete h;
    return CLR_OK;
}

// Event bookkeeping for clr_lbvh_set_profiling: mark(h, st, name) closes the
// previous pass and opens the next.
struct PassTimer {
    clr_lbvh* h;
    cudaStream_t st;
    PassTimer(clr_lbvh* hh, cudaStream_t s) : h(hh), st(s) {
        h->num_timed = 0;
        if (h->profiling) cudaEventRecord(h->ev[0], st);
    }
    void done(const char* name) {
        if (!h->profiling || h->num_timed >= clr_lbvh::kMaxTimed) return;
        h->ev_name[h->num_timed] = name;
        cudaEventRecord(h->ev[++h->num_timed], st);
    }
};

// Clears what a build of n keys reads before writing: the digit histograms,
// tile counters and scene box, and the look-back words of the passes and
// tiles it uses, laid out with a stride of its own tile count.
static cudaError_t clear_for_build(clr_lbvh* h, uint32_t n, int items, int npasses, cudaStream_t st) {
    const size_t tiles = div_up(n ? n : 1, (unsigned int)(kSortThreads * items));
    h->status_stride = tiles * kRadix;
    return cudaMemsetAsync(h->zero_region, 0, h->zero_prefix_bytes + 4ull * npasses * h->status_stride, st);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (null when
// the driver does not offer it: the tree pass then gathers with plain loads).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        cudaGetLastError();
    });
    return fn;
}

// Cleared only by clr_debug_set_tma_gather.
static bool g_tma_gather = true;

// The staging array (n rows of 12 floats, 48-byte rows) as a tensor map whose
// box is one row: the tile::gather4 form.
static bool stage_map_for(clr_lbvh* h, uint32_t n) {
    if (!g_tma_gather) return false;
    if (h->map_base == h->stage && h->map_rows == n) return h->map_ok;
    h->map_base = h->stage;
    h->map_rows = n;
    h->map_ok = false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || (reinterpret_cast<uintptr_t>(h->stage) & 15u)) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)kStageFloats, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)kStageFloats * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)kStageFloats, 1u};
    const cuuint32_t estride[2] = {1u, 1u};
    h->map_ok = enc(&h->stage_map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float4*>(h->stage), dims, strides,
                    box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    return h->map_ok;
}

template <typename KeyT>
static int run_build(clr_lbvh* h, const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                     uint32_t n, uint32_t bits, clr_bvh* out, cudaStream_t st) {
    const int kbits = 3 * (int)bits;
    const int npasses = (kbits + 7) / 8;
    const int grid_stream = clr_sm_count() * 8;
    PassTimer timer(h, st);
    CLR_CUDA_TRY(clear_for_build(h, n, SortCfg<KeyT>::kItems, npasses, st));
    k_scene_box<<<grid_stream, 256, 0, st>>>(vx, vy, vz, tri, n, h->boxw);
    CLR_LAUNCH_CHECK("k_scene_box");
    timer.done("scene_box");
    KeyT* keys[2] = {static_cast<KeyT*>(h->keys[0]), static_cast<KeyT*>(h->keys[1])};
    k_morton<KeyT><<<grid_stream, 256, 0, st>>>(vx, vy, vz, tri, n, bits, h->boxw, keys[0], h->hist, npasses,
                                                h->counters, h->stage);
    CLR_LAUNCH_CHECK("k_morton");
    timer.done("morton");
    constexpr int kTile = kSortThreads * SortCfg<KeyT>::kItems;
    const unsigned int tiles = div_up(n, kTile);
    for (int p = 0; p < npasses; ++p) {
        const int src = p & 1, dst = src ^ 1;
        if (p == 0)
            k_onesweep<KeyT, true><<<tiles, kSortThreads, 0, st>>>(
                keys[src], nullptr, keys[dst], h->vals[dst], n, 8 * p, h->hist + p * kRadix,
                h->status + p * h->status_stride, h->tile_ctr + p, g_sort_spin_limit);
        else
            k_onesweep<KeyT, false><<<tiles, kSortThreads, 0, st>>>(
                keys[src], h->vals[src], keys[dst], h->vals[dst], n, 8 * p, h->hist + p * kRadix,
                h->status + p * h->status_stride, h->tile_ctr + p, g_sort_spin_limit);
        CLR_LAUNCH_CHECK("k_onesweep");
        timer.done("sort_pass");
    }
    const int fin = npasses & 1;
    h->final_buf = fin;
    float4* tris = static_cast<float4*>(out->tris);
    if (n == 1) {
        k_single<<<1, 1, 0, st>>>(vx, vy, vz, tri, tris, out->root_box);
        CLR_LAUNCH_CHECK("k_single");
        timer.done("single");
    } else {
        // worklist of the block-crossing nodes: the sort's free ping-pong side
        uint32_t* worklist = h->vals[fin ^ 1];
        unsigned int* wl_count = h->tile_ctr + kMaxPasses;
        const bool wide = (reinterpret_cast<uintptr_t>(out->nodes) & 31u) == 0u;  // 32-byte node stores
        const bool tma = h->stage != nullptr && stage_map_for(h, n);               // TMA record gathers
        // block-crossing climbs: inside the tree pass for small trees (no
        // second launch, the climbs overlap the other blocks), handed to
        // k_build_tree_top for large ones (blocks held by long climbs would
        // delay the rest of the pass)
        const bool climb_here = n <= kClimbHereMaxTris;
        const unsigned int grid = div_up(n, kTreeBlock);
        float* nodes = reinterpret_cast<float*>(out->nodes);
#define CLR_TREE_ARGS                                                                                               \
    keys[fin], h->vals[fin], n, kbits, vx, vy, vz, tri, h->stage, nodes, tris, h->counters, h->karras_idx, out->root_box, \
        worklist, wl_count, climb_here ? 1 : 0
        if (wide && tma) k_build_tree<KeyT, true, true><<<grid, kTreeBlock, 0, st>>>(h->stage_map, CLR_TREE_ARGS);
        else if (wide) k_build_tree<KeyT, true, false><<<grid, kTreeBlock, 0, st>>>(h->stage_map, CLR_TREE_ARGS);
        else if (tma) k_build_tree<KeyT, false, true><<<grid, kTreeBlock, 0, st>>>(h->stage_map, CLR_TREE_ARGS);
        else k_build_tree<KeyT, false, false><<<grid, kTreeBlock, 0, st>>>(h->stage_map, CLR_TREE_ARGS);
#undef CLR_TREE_ARGS
        CLR_LAUNCH_CHECK("k_build_tree");
        if (!climb_here) {
            k_build_tree_top<KeyT><<<clr_sm_count() * 4, 256, 0, st>>>(
                keys[fin], n, kbits, reinterpret_cast<float*>(out->nodes), h->counters, h->karras_idx, out->root_box,
                worklist, wl_count);
            CLR_LAUNCH_CHECK("k_build_tree_top");
        }
        timer.done("build_tree");
    }
    return CLR_OK;
}

extern "C" int clr_lbvh_build(clr_lbvh* h, const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                              uint32_t num_tris, uint32_t bits_per_dim, clr_bvh* out, void* stream) {
    if (!h || !out) return clr_set_error(CLR_EINVAL, "clr_lbvh_build: NULL handle or output");
    if (bits_per_dim < 1 || bits_per_dim > 21)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build: bits_per_dim %u outside [1, 21]", bits_per_dim);
    if (num_tris >= (1u << 30))
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build: %u triangles exceed the 2^30 limit", num_tris);
    if (num_tris > 0 && (!vx || !vy || !vz || !out->tris || !out->root_box || (num_tris > 1 && !out->nodes)))
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build: NULL input or output buffer");
    out->num_tris = num_tris;
    out->bits_per_dim = bits_per_dim;
    h->last_n = num_tris;
    h->last_bits = bits_per_dim;
    if (num_tris == 0) return CLR_OK;
    int rc = pool_grow(h, num_tris);
    if (rc != CLR_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (bits_per_dim <= 10) return run_build<uint32_t>(h, vx, vy, vz, tri, num_tris, bits_per_dim, out, st);
    return run_build<uint64_t>(h, vx, vy, vz, tri, num_tris, bits_per_dim, out, st);
}

// ------------------------------------------------- builds from host inputs

// The copy stream and the four buffer events, made on first use.
static int host_path_init(clr_lbvh* h) {
    if (h->copy_stream) return CLR_OK;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[5] = {};
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {  // nothing half-made stays behind
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (st) cudaStreamDestroy(st);
        return clr_set_error(CLR_ECUDA, "clr_lbvh_build_host: copy stream or events: %s", cudaGetErrorString(e));
    }
    h->in_copied[0] = ev[0];
    h->in_copied[1] = ev[1];
    h->in_consumed[0] = ev[2];
    h->in_consumed[1] = ev[3];
    h->copy_gate = ev[4];
    h->copy_stream = st;
    return CLR_OK;
}

// Input buffer s holds at least `bytes`.  Growing frees the old buffer, which
// waits for the work that may still read it.
static int in_buf_grow(clr_lbvh* h, int s, size_t bytes) {
    if (h->in_buf[s] && bytes <= h->in_bytes[s]) return CLR_OK;
    if (h->in_buf[s]) {
        CLR_CUDA_TRY(cudaEventSynchronize(h->in_consumed[s]));
        CLR_CUDA_TRY(cudaStreamSynchronize(h->copy_stream));
        cudaFree(h->in_buf[s]);
        h->in_buf[s] = nullptr;
        h->in_bytes[s] = 0;
    }
    if (cudaMalloc(&h->in_buf[s], bytes) != cudaSuccess) {
        cudaGetLastError();
        h->in_buf[s] = nullptr;
        return clr_set_error(CLR_ENOMEM, "cudaMalloc of a %zu-byte input buffer failed", bytes);
    }
    h->in_bytes[s] = bytes;
    return CLR_OK;
}

extern "C" int clr_lbvh_build_host(clr_lbvh* h, const float* host_vx, const float* host_vy, const float* host_vz,
                                   const uint32_t* host_tri, uint32_t num_verts, uint32_t num_tris,
                                   uint32_t bits_per_dim, clr_bvh* out, float* host_root_box, void* stream) {
    if (!h || !out) return clr_set_error(CLR_EINVAL, "clr_lbvh_build_host: NULL handle or output");
    if (bits_per_dim < 1 || bits_per_dim > 21)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_host: bits_per_dim %u outside [1, 21]", bits_per_dim);
    if (num_tris >= (1u << 30))
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_host: %u triangles exceed the 2^30 limit", num_tris);
    if (!host_tri && num_verts != 3ull * num_tris)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_host: a soup of %u triangles has %llu vertices, not %u",
                             num_tris, 3ull * num_tris, num_verts);
    if (num_tris > 0 && (!host_vx || !host_vy || !host_vz || num_verts == 0 || !out->tris || !out->root_box ||
                         (num_tris > 1 && !out->nodes)))
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_host: NULL input or output buffer");
    if (num_tris == 0) return clr_lbvh_build(h, nullptr, nullptr, nullptr, nullptr, 0, bits_per_dim, out, stream);
    int rc = host_path_init(h);
    if (rc != CLR_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int s = (int)(h->host_calls & 1u);
    const size_t vbytes = 4ull * num_verts, vstride = align_up(vbytes, 256);
    rc = in_buf_grow(h, s, 3 * vstride + (host_tri ? 12ull * num_tris : 0));
    if (rc != CLR_OK) return rc;
    char* base = static_cast<char*>(h->in_buf[s]);
    float* d[3] = {reinterpret_cast<float*>(base), reinterpret_cast<float*>(base + vstride),
                   reinterpret_cast<float*>(base + 2 * vstride)};
    uint32_t* dtri = host_tri ? reinterpret_cast<uint32_t*>(base + 3 * vstride) : nullptr;
    // the copy waits for the build that last read this buffer (two calls
    // back), not for the previous call's build: the two overlap
    if (h->in_used[s]) CLR_CUDA_TRY(cudaStreamWaitEvent(h->copy_stream, h->in_consumed[s], 0));
    const float* src[3] = {host_vx, host_vy, host_vz};
    for (int k = 0; k < 3; ++k)
        CLR_CUDA_TRY(cudaMemcpyAsync(d[k], src[k], vbytes, cudaMemcpyHostToDevice, h->copy_stream));
    if (dtri)
        CLR_CUDA_TRY(cudaMemcpyAsync(dtri, host_tri, 12ull * num_tris, cudaMemcpyHostToDevice, h->copy_stream));
    CLR_CUDA_TRY(cudaEventRecord(h->in_copied[s], h->copy_stream));
    CLR_CUDA_TRY(cudaStreamWaitEvent(st, h->in_copied[s], 0));
    rc = clr_lbvh_build(h, d[0], d[1], d[2], dtri, num_tris, bits_per_dim, out, stream);
    if (rc != CLR_OK) return rc;
    CLR_CUDA_TRY(cudaEventRecord(h->in_consumed[s], st));
    h->in_used[s] = true;
    ++h->host_calls;
    if (host_root_box)
        CLR_CUDA_TRY(cudaMemcpyAsync(host_root_box, out->root_box, 32, cudaMemcpyDeviceToHost, st));
    return CLR_OK;
}

extern "C" int clr_lbvh_host_copy_after(clr_lbvh* h, void* stream) {
    if (!h) return clr_set_error(CLR_EINVAL, "clr_lbvh_host_copy_after: NULL handle");
    int rc = host_path_init(h);
    if (rc != CLR_OK) return rc;
    CLR_CUDA_TRY(cudaEventRecord(h->copy_gate, static_cast<cudaStream_t>(stream)));
    CLR_CUDA_TRY(cudaStreamWaitEvent(h->copy_stream, h->copy_gate, 0));
    return CLR_OK;
}

extern "C" int clr_lbvh_host_copy_wait(clr_lbvh* h) {
    if (!h) return clr_set_error(CLR_EINVAL, "clr_lbvh_host_copy_wait: NULL handle");
    if (!h->copy_stream) return CLR_OK;
    CLR_CUDA_TRY(cudaStreamSynchronize(h->copy_stream));
    return CLR_OK;
}

static int seg_grow(clr_lbvh* h, uint32_t nseg) {
    if (h->seg_pool && nseg <= h->seg_cap) return CLR_OK;
    if (h->seg_pool) cudaFree(h->seg_pool);
    h->seg_pool = nullptr;
    h->seg_cap = 0;
    const size_t off_bytes = align_up(4ull * (nseg + 1), 256);
    if (cudaMalloc(&h->seg_pool, off_bytes + 24ull * nseg) != cudaSuccess) {
        cudaGetLastError();
        h->seg_pool = nullptr;
        return clr_set_error(CLR_ENOMEM, "cudaMalloc for %u scene descriptors failed", nseg);
    }
    h->seg_off = static_cast<uint32_t*>(h->seg_pool);
    h->seg_box = reinterpret_cast<unsigned int*>(static_cast<char*>(h->seg_pool) + off_bytes);
    h->seg_cap = nseg;
    return CLR_OK;
}

template <int kBits>
static void launch_sort_pass(uint64_t* kin, uint32_t* vin, uint64_t* kout, uint32_t* vout, uint32_t n, int p,
                             clr_lbvh* h, unsigned int tiles, cudaStream_t st) {
    if (p == 0)
        k_onesweep<uint64_t, true, kBits><<<tiles, kSortThreads, 0, st>>>(
            kin, nullptr, kout, vout, n, kBits * p, h->hist + p * kRadix, h->status + p * h->status_stride,
            h->tile_ctr + p, g_sort_spin_limit);
    else
        k_onesweep<uint64_t, false, kBits><<<tiles, kSortThreads, 0, st>>>(
            kin, vin, kout, vout, n, kBits * p, h->hist + p * kRadix, h->status + p * h->status_stride,
            h->tile_ctr + p, g_sort_spin_limit);
}

extern "C" int clr_lbvh_build_batched(clr_lbvh* h, const float* vx, const float* vy, const float* vz,
                                      const uint32_t* tri, const uint32_t* scene_offsets, uint32_t num_scenes,
                                      uint32_t bits_per_dim, uint32_t radix_bits, void* nodes, void* tris,
                                      float* root_boxes, void* stream) {
    if (!h || !scene_offsets || num_scenes == 0)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_batched: NULL handle / offsets or no scene");
    if (radix_bits == 0) radix_bits = 8;
    if (radix_bits < 6 || radix_bits > 8)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_batched: radix_bits %u outside [6, 8]", radix_bits);
    if (scene_offsets[0] != 0) return clr_set_error(CLR_EINVAL, "clr_lbvh_build_batched: offsets[0] must be 0");
    for (uint32_t s = 0; s < num_scenes; ++s)
        if (scene_offsets[s + 1] <= scene_offsets[s])
            return clr_set_error(CLR_EINVAL, "clr_lbvh_build_batched: scene %u has no triangle", s);
    const uint32_t n = scene_offsets[num_scenes];
    if (n >= (1u << 30))
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_batched: %u triangles exceed the 2^30 limit", n);
    uint32_t sbits = 0;
    while ((1ull << sbits) < num_scenes) ++sbits;
    const int kbits = 3 * (int)bits_per_dim;
    const int total_bits = kbits + (int)sbits;
    const int npasses = (total_bits + (int)radix_bits - 1) / (int)radix_bits;
    if (bits_per_dim < 1 || total_bits > 64 || npasses > kMaxPasses)
        return clr_set_error(CLR_EINVAL,
                             "clr_lbvh_build_batched: %u bits per axis and %u scenes need %d key bits / %d passes",
                             bits_per_dim, num_scenes, total_bits, npasses);
    if (!vx || !vy || !vz || !nodes || !tris || !root_boxes)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_batched: NULL input or output buffer");
    int rc = pool_grow(h, n);
    if (rc != CLR_OK) return rc;
    rc = seg_grow(h, num_scenes);
    if (rc != CLR_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    h->last_n = 0;  // the reference-layout export covers single-scene builds only
    PassTimer timer(h, st);
    CLR_CUDA_TRY(cudaMemcpyAsync(h->seg_off, scene_offsets, 4ull * (num_scenes + 1), cudaMemcpyHostToDevice, st));
    CLR_CUDA_TRY(clear_for_build(h, n, SortCfg<uint64_t>::kItems, npasses, st));
    CLR_CUDA_TRY(cudaMemsetAsync(h->seg_box, 0, 24ull * num_scenes, st));
    k_seg_box<<<div_up(n, kSegBoxChunk), 256, 0, st>>>(vx, vy, vz, tri, h->seg_off, num_scenes, n, h->seg_box);
    CLR_LAUNCH_CHECK("k_seg_box");
    timer.done("scene_box");
    uint64_t* keys[2] = {static_cast<uint64_t*>(h->keys[0]), static_cast<uint64_t*>(h->keys[1])};
    const int grid_stream = clr_sm_count() * 8;
    if (radix_bits == 8)
        k_morton_seg<8><<<grid_stream, 256, 0, st>>>(vx, vy, vz, tri, h->seg_off, num_scenes, n, bits_per_dim,
                                                     h->seg_box, keys[0], h->hist, npasses, h->counters, h->stage);
    else if (radix_bits == 7)
        k_morton_seg<7><<<grid_stream, 256, 0, st>>>(vx, vy, vz, tri, h->seg_off, num_scenes, n, bits_per_dim,
                                                     h->seg_box, keys[0], h->hist, npasses, h->counters, h->stage);
    else
        k_morton_seg<6><<<grid_stream, 256, 0, st>>>(vx, vy, vz, tri, h->seg_off, num_scenes, n, bits_per_dim,
                                                     h->seg_box, keys[0], h->hist, npasses, h->counters, h->stage);
    CLR_LAUNCH_CHECK("k_morton_seg");
    timer.done("morton");
    constexpr int kTile = kSortThreads * SortCfg<uint64_t>::kItems;
    const unsigned int tiles = div_up(n, kTile);
    for (int p = 0; p < npasses; ++p) {
        const int src = p & 1, dst = src ^ 1;
        if (radix_bits == 8) launch_sort_pass<8>(keys[src], h->vals[src], keys[dst], h->vals[dst], n, p, h, tiles, st);
        else if (radix_bits == 7) launch_sort_pass<7>(keys[src], h->vals[src], keys[dst], h->vals[dst], n, p, h, tiles, st);
        else launch_sort_pass<6>(keys[src], h->vals[src], keys[dst], h->vals[dst], n, p, h, tiles, st);
        CLR_LAUNCH_CHECK("k_onesweep");
        timer.done("sort_pass");
    }
    const int fin = npasses & 1;
    h->final_buf = fin;
    k_build_tree_seg<uint64_t><<<div_up(n, 256), 256, 0, st>>>(
        keys[fin], h->vals[fin], h->seg_off, num_scenes, n, kbits, vx, vy, vz, tri, h->stage, static_cast<float*>(nodes),
        static_cast<float4*>(tris), h->counters, h->karras_idx, root_boxes);
    CLR_LAUNCH_CHECK("k_build_tree_seg");
    timer.done("build_tree");
    return CLR_OK;
}

// ---------------------------------------------------------------- ray order
//
// Rays sorted by the Morton code of their origin before the searches: the
// rays a warp searches together then start in the same region of the scene
// and share the tree's nodes in L1 / L2.  The order changes no ray's answer
// (each is written to its own index).  Keys: the origin quantised to 8 bits
// per axis in the tree's root box (clamped outside it), 24 bits, sorted by
// three one-sweep passes of the build's radix sort.
constexpr int kRayKeyBits = 8;
constexpr int kRayPasses = 3;

__global__ void __launch_bounds__(256) k_ray_keys(const float4* __restrict__ rays, uint32_t n,
                                                  const float* __restrict__ root_box, uint32_t* __restrict__ keys,
                                                  unsigned int* __restrict__ hist) {
    __shared__ unsigned int sh[kRayPasses * kRadix];
    for (int i = threadIdx.x; i < kRayPasses * kRadix; i += blockDim.x) sh[i] = 0;
    float mn[3], sc[3];
    for (int k = 0; k < 3; ++k) {
        mn[k] = __ldg(root_box + k);
        const float ext = __ldg(root_box + 4 + k) - mn[k];
        sc[k] = ext > 0.f ? (float)(1 << kRayKeyBits) / ext : 0.f;
    }
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 o = __ldg(rays + 2ull * i);
        const float c[3] = {o.x, o.y, o.z};
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            const float f = (c[k] - mn[k]) * sc[k];  // NaN and out-of-box origins clamp below
            q[k] = f > 0.f ? (uint32_t)fminf(f, (float)((1 << kRayKeyBits) - 1)) : 0u;
        }
        const uint32_t key = spread3_10(q[0]) | (spread3_10(q[1]) << 1) | (spread3_10(q[2]) << 2);
        keys[i] = key;
        for (int p = 0; p < kRayPasses; ++p) atomicAdd(&sh[p * kRadix + ((key >> (8 * p)) & 0xFFu)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kRayPasses * kRadix; i += blockDim.x)
        if (sh[i]) atomicAdd(hist + i, sh[i]);
}

namespace {
struct RaySortLayout {
    uint32_t* keys[2];
    uint32_t* vals[2];
    unsigned int* hist;     // [pass][256]
    unsigned int* tiles;    // [pass] tile counters
    unsigned int* status;   // [pass][tile][256]
    size_t status_stride;
    char* zero;             // hist, tile counters, status: cleared per call
    size_t zero_bytes;
};
}  // namespace

static size_t ray_sort_layout(uint32_t n, char* base, RaySortLayout* L) {
    constexpr unsigned int kTile = kSortThreads * SortCfg<uint32_t>::kItems;
    const size_t tiles = div_up(n ? n : 1, kTile);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const size_t o_k0 = take(4ull * n), o_k1 = take(4ull * n), o_v0 = take(4ull * n), o_v1 = take(4ull * n);
    const size_t o_zero = off;
    const size_t o_hist = take(4ull * kRayPasses * kRadix), o_tiles = take(4ull * kRayPasses),
                 o_status = take(4ull * kRayPasses * tiles * kRadix);
    if (base && L) {
        L->keys[0] = reinterpret_cast<uint32_t*>(base + o_k0);
        L->keys[1] = reinterpret_cast<uint32_t*>(base + o_k1);
        L->vals[0] = reinterpret_cast<uint32_t*>(base + o_v0);
        L->vals[1] = reinterpret_cast<uint32_t*>(base + o_v1);
        L->hist = reinterpret_cast<unsigned int*>(base + o_hist);
        L->tiles = reinterpret_cast<unsigned int*>(base + o_tiles);
        L->status = reinterpret_cast<unsigned int*>(base + o_status);
        L->status_stride = tiles * kRadix;
        L->zero = base + o_zero;
        L->zero_bytes = off - o_zero;
    }
    return off;
}

// Sorts the ray indices by origin key; returns the order (in the workspace).
static int ray_order(const clr_bvh* bvh, const float* rays, uint32_t n, void* workspace, uint64_t workspace_bytes,
                     cudaStream_t st, const uint32_t** order) {
    if (!bvh || !rays) return clr_set_error(CLR_EINVAL, "trace (sorted): NULL bvh or rays");
    if (!bvh->root_box) return clr_set_error(CLR_EINVAL, "trace (sorted): bvh has no root box");
    if (!workspace || workspace_bytes < ray_sort_layout(n, nullptr, nullptr))
        return clr_set_error(CLR_ECAPACITY, "trace (sorted): workspace of %llu bytes is smaller than %zu",
                             (unsigned long long)workspace_bytes, ray_sort_layout(n, nullptr, nullptr));
    if (reinterpret_cast<uintptr_t>(workspace) & 255u)
        return clr_set_error(CLR_EINVAL, "trace (sorted): workspace must be 256-byte aligned");
    if (reinterpret_cast<uintptr_t>(rays) & 15u) return clr_set_error(CLR_EINVAL, "trace: rays must be 16-byte aligned");
    RaySortLayout L;
    ray_sort_layout(n, static_cast<char*>(workspace), &L);
    CLR_CUDA_TRY(cudaMemsetAsync(L.zero, 0, L.zero_bytes, st));
    const unsigned int grid = std::min(div_up(n, 256u), (unsigned int)clr_sm_count() * 8u);
    k_ray_keys<<<grid, 256, 0, st>>>(reinterpret_cast<const float4*>(rays), n, bvh->root_box, L.keys[0], L.hist);
    CLR_LAUNCH_CHECK("k_ray_keys");
    constexpr int kTile = kSortThreads * SortCfg<uint32_t>::kItems;
    const unsigned int tiles = div_up(n, kTile);
    for (int p = 0; p < kRayPasses; ++p) {
        const int src = p & 1, dst = src ^ 1;
        if (p == 0)
            k_onesweep<uint32_t, true><<<tiles, kSortThreads, 0, st>>>(
                L.keys[src], nullptr, L.keys[dst], L.vals[dst], n, 8 * p, L.hist + p * kRadix,
                L.status + p * L.status_stride, L.tiles + p, g_sort_spin_limit);
        else
            k_onesweep<uint32_t, false><<<tiles, kSortThreads, 0, st>>>(
                L.keys[src], L.vals[src], L.keys[dst], L.vals[dst], n, 8 * p, L.hist + p * kRadix,
                L.status + p * L.status_stride, L.tiles + p, g_sort_spin_limit);
        CLR_LAUNCH_CHECK("k_onesweep (rays)");
    }
    *order = L.vals[kRayPasses & 1];
    return CLR_OK;
}

int clr_trace_closest_in_order(const clr_bvh* bvh, const float* rays, uint32_t num_rays, const uint32_t* order,
                               uint32_t* hit_id, float* hit_t, void* stream);
int clr_trace_shadow_in_order(const clr_bvh* bvh, const float* rays, uint32_t num_rays, const uint32_t* order,
                              uint8_t* occluded, void* stream);

extern "C" int clr_trace_sort_workspace_bytes(uint32_t num_rays, uint64_t* bytes) {
    if (!bytes) return clr_set_error(CLR_EINVAL, "clr_trace_sort_workspace_bytes: bytes is NULL");
    *bytes = ray_sort_layout(num_rays, nullptr, nullptr);
    return CLR_OK;
}

extern "C" int clr_trace_closest_sorted(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                        float* hit_t, void* workspace, uint64_t workspace_bytes, void* stream) {
    if (num_rays == 0) return clr_trace_closest_in_order(bvh, rays, 0, nullptr, hit_id, hit_t, stream);
    if (!bvh || bvh->num_tris == 0) return clr_trace_closest_in_order(bvh, rays, num_rays, nullptr, hit_id, hit_t, stream);
    const uint32_t* order = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = ray_order(bvh, rays, num_rays, workspace, workspace_bytes, st, &order);
    if (rc != CLR_OK) return rc;
    return clr_trace_closest_in_order(bvh, rays, num_rays, order, hit_id, hit_t, stream);
}

extern "C" int clr_trace_shadow_sorted(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint8_t* occluded,
                                       void* workspace, uint64_t workspace_bytes, void* stream) {
    if (num_rays == 0) return clr_trace_shadow_in_order(bvh, rays, 0, nullptr, occluded, stream);
    if (!bvh || bvh->num_tris == 0) return clr_trace_shadow_in_order(bvh, rays, num_rays, nullptr, occluded, stream);
    const uint32_t* order = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = ray_order(bvh, rays, num_rays, workspace, workspace_bytes, st, &order);
    if (rc != CLR_OK) return rc;
    return clr_trace_shadow_in_order(bvh, rays, num_rays, order, occluded, stream);
}

extern "C" int clr_lbvh_export_reference(clr_lbvh* h, const clr_bvh* bvh, void* inodes, void* lnodes,
                                         uint32_t* parents, uint32_t* sorted_idx, uint64_t* keys, void* stream) {
    if (!h || !bvh) return clr_set_error(CLR_EINVAL, "clr_lbvh_export_reference: NULL argument");
    const uint32_t n = bvh->num_tris;
    if (n != h->last_n) return clr_set_error(CLR_EINVAL, "clr_lbvh_export_reference: bvh is not the last build");
    if (n == 0) return CLR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n == 1) {
        k_export_single<<<1, 1, 0, st>>>(bvh->root_box, static_cast<const float4*>(bvh->tris),
                                         static_cast<uint8_t*>(lnodes), parents);
        CLR_LAUNCH_CHECK("k_export_single");
    } else {
        k_karras_index<<<div_up(n - 1, 256), 256, 0, st>>>(static_cast<const float4*>(bvh->nodes), bvh->root_box, n,
                                                           h->karras_idx);
        CLR_LAUNCH_CHECK("k_karras_index");
        k_export<<<div_up(n - 1, 256), 256, 0, st>>>(static_cast<const float4*>(bvh->nodes),
                                                     static_cast<const float4*>(bvh->tris), h->karras_idx, n,
                                                     static_cast<uint8_t*>(inodes), static_cast<uint8_t*>(lnodes),
                                                     parents);
        CLR_LAUNCH_CHECK("k_export");
    }
    const int fin = h->final_buf;
    if (sorted_idx) CLR_CUDA_TRY(cudaMemcpyAsync(sorted_idx, h->vals[fin], 4ull * n, cudaMemcpyDeviceToDevice, st));
    if (keys) {
        if (h->last_bits <= 10)
            k_keys_to_u64<uint32_t><<<div_up(n, 256), 256, 0, st>>>(static_cast<const uint32_t*>(h->keys[fin]), keys, n);
        else
            k_keys_to_u64<uint64_t><<<div_up(n, 256), 256, 0, st>>>(static_cast<const uint64_t*>(h->keys[fin]), keys, n);
        CLR_LAUNCH_CHECK("k_keys_to_u64");
    }
    return CLR_OK;
}

extern "C" int clr_lbvh_set_profiling(clr_lbvh* h, int enable) {
    if (!h) return clr_set_error(CLR_EINVAL, "clr_lbvh_set_profiling: NULL handle");
    if (enable && !h->ev[0])
        for (auto& e : h->ev) CLR_CUDA_TRY(cudaEventCreate(&e));
    h->profiling = enable != 0;
    h->num_timed = 0;
    return CLR_OK;
}

extern "C" int clr_lbvh_pass_times(clr_lbvh* h, float* ms, const char** names, int max_passes, int* num_passes) {
    if (!h || !num_passes) return clr_set_error(CLR_EINVAL, "clr_lbvh_pass_times: NULL argument");
    if (!h->profiling) return clr_set_error(CLR_EINVAL, "clr_lbvh_pass_times: profiling is off");
    const int n = h->num_timed < max_passes ? h->num_timed : max_passes;
    if (h->num_timed > 0) CLR_CUDA_TRY(cudaEventSynchronize(h->ev[h->num_timed]));
    for (int i = 0; i < n; ++i) {
        if (ms) CLR_CUDA_TRY(cudaEventElapsedTime(ms + i, h->ev[i], h->ev[i + 1]));
        if (names) names[i] = h->ev_name[i];
    }
    *num_passes = n;
    return CLR_OK;
}

// ====================================================== allocation-free build
//
// clr_lbvh_build_noalloc serves callers that must not allocate device memory
// themselves: hosts that hand this library a fixed device-memory budget
// through their own allocator and forbid any other allocation, and per-frame
// loops where the implicit device synchronisation of cudaMalloc/cudaFree
// would stall the pipeline.  Its scratch lives in the file-scope array below,
// sized for kNoAllocMaxTris triangles; every GPU that loads this library holds
// that array until the process exits.  The build is the same pipeline as
// clr_lbvh_build, run on a scratch layout carved out of the array.

namespace {
constexpr uint32_t kNoAllocMaxTris = 1u << 18;               // 262,144 triangles
constexpr size_t kNoAllocScratchBytes = 12ull << 20;         // 12 MiB
constexpr int kNoAllocMaxDevices = 64;
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch per device, resolved by the first call
// made while that device is current, together with the CUDA context it was
// resolved in.  The address is only valid in that context: after a device
// reset (or with another context made current on the device) the next call
// resolves it again, so the first call after such a change is again a set-up
// call and belongs outside any stream capture.
struct NoAllocAddr {
    void* ctx = nullptr;
    void* addr = nullptr;
};
static NoAllocAddr g_noalloc_addr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mutex;

// The current context of the calling thread (cuCtxGetCurrent, reached through
// the runtime so that the library links no driver stub); null if unavailable.
static void* current_context() {
    using CtxGet = int (*)(void**);
    static CtxGet fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGet>(f);
    }();
    void* ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

static int noalloc_scratch(void** out) {
    int dev = -1;
    CLR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_noalloc: device %d out of range", dev);
    // cudaGetDevice does not create the context; the symbol lookup below
    // does, so a null context only ever means "not resolved yet"
    void* ctx = current_context();
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoAllocAddr& a = g_noalloc_addr[dev];
    if (!a.addr || !ctx || a.ctx != ctx) {
        void* p = nullptr;
        CLR_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        a.addr = p;
        a.ctx = current_context();
    }
    *out = a.addr;
    return CLR_OK;
}

extern "C" int clr_lbvh_build_noalloc(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                                      uint32_t num_tris, uint32_t bits_per_dim, clr_bvh* out, void* stream) {
    if (!out) return clr_set_error(CLR_EINVAL, "clr_lbvh_build_noalloc: NULL output");
    if (bits_per_dim < 1 || bits_per_dim > 21)
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_noalloc: bits_per_dim %u outside [1, 21]", bits_per_dim);
    if (num_tris > kNoAllocMaxTris)
        return clr_set_error(CLR_ECAPACITY,
                             "clr_lbvh_build_noalloc: %u triangles exceed its fixed scratch limit of %u; "
                             "use clr_lbvh_build",
                             num_tris, kNoAllocMaxTris);
    if (num_tris > 0 && (!vx || !vy || !vz || !out->tris || !out->root_box || (num_tris > 1 && !out->nodes)))
        return clr_set_error(CLR_EINVAL, "clr_lbvh_build_noalloc: NULL input or output buffer");
    out->num_tris = num_tris;
    out->bits_per_dim = bits_per_dim;
    if (num_tris == 0) return CLR_OK;
    void* base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc != CLR_OK) return rc;
    // laid out for this call's triangle count, so that the part cleared per
    // build (digit histograms and look-back words) covers only the tiles this
    // build uses; the layout grows with the count and, at the maximum count,
    // still fits the array
    clr_lbvh h{};
    if (pool_layout(&h, kNoAllocMaxTris, nullptr, false) > kNoAllocScratchBytes)
        return clr_set_error(CLR_ECAPACITY, "clr_lbvh_build_noalloc: scratch layout exceeds the static array");
    pool_layout(&h, num_tris, static_cast<char*>(base), false);
    h.capacity = num_tris;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (bits_per_dim <= 10) return run_build<uint32_t>(&h, vx, vy, vz, tri, num_tris, bits_per_dim, out, st);
    return run_build<uint64_t>(&h, vx, vy, vz, tri, num_tris, bits_per_dim, out, st);
}

// ============================================================ bounded waits
//
// The sort's look-back is the one place where a block of the build waits on
// another block.  Its wait is bounded: after g_sort_spin_limit polls the block
// raises CLR_DEVERR_SORT_TIMEOUT, finishes its tile with the prefix it has
// (its writes stay inside the output, only their order is wrong) and returns.

int clr_batch_set_iteration_cap(uint32_t cap);  // render_batch.cu

extern "C" int clr_debug_set_wait_limits(uint32_t sort_spin_limit, uint32_t batch_iteration_cap) {
    g_sort_spin_limit = sort_spin_limit ? sort_spin_limit : kSpinLimit;
    return clr_batch_set_iteration_cap(batch_iteration_cap);
}

extern "C" int clr_debug_set_tma_gather(int enable) {
    g_tma_gather = enable != 0;
    return CLR_OK;
}

extern "C" int clr_debug_lookback_stall(uint32_t* keys, uint32_t* scratch, uint32_t tile_keys, void* stream) {
    // One sort pass over two tiles of 32-bit keys in which only the second
    // tile's block runs: the first tile never publishes its digit counts, so
    // the second tile's look-back finds no flag and must give up.
    constexpr int kTile = kSortThreads * SortCfg<uint32_t>::kItems;
    if (!keys || !scratch) return clr_set_error(CLR_EINVAL, "clr_debug_lookback_stall: NULL argument");
    if (tile_keys != (uint32_t)kTile)
        return clr_set_error(CLR_EINVAL, "clr_debug_lookback_stall: tile_keys must be %d", kTile);
    const uint32_t n = 2u * kTile;
    // scratch: keys out [n], values out [n], histogram [256], look-back words
    // [2][256] (zero: nothing published), tile counter [1] = 1
    uint32_t* kout = scratch;
    uint32_t* vout = kout + n;
    unsigned int* hist = vout + n;
    unsigned int* status = hist + kRadix;
    unsigned int* tile_ctr = status + 2 * kRadix;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CLR_CUDA_TRY(cudaMemsetAsync(hist, 0, 4ull * 3 * kRadix, st));  // histogram and look-back words
    k_debug_hist<<<div_up(n, 256), 256, 0, st>>>(keys, n, hist, tile_ctr);
    CLR_LAUNCH_CHECK("k_debug_hist");
    k_onesweep<uint32_t, true><<<1, kSortThreads, 0, st>>>(keys, nullptr, kout, vout, n, 0, hist, status, tile_ctr,
                                                          g_sort_spin_limit);
    CLR_LAUNCH_CHECK("k_onesweep");
    return CLR_OK;
}
