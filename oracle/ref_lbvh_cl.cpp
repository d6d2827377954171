/*
 * The reference's own LBVH construction kernels run on the CPU
 * (OpenCL_PathTracer/OpenCL/lbvh_construction.cl with extra_atomics.cl, and
 * the global scan of CommonSources/OpenCL/generic_kernels.cl), compiled as
 * C++ through the OpenCL C subset of oracle/ref_stubs/opencl_c.hpp, and
 * launched in the order and with the sizes of LBVHBuilder::perform
 * (OpenCL_PathTracer/LBVHBuilder.cpp:160-375; work-group sizes
 * LBVHBuilder.cpp:21-23, 30) and GlobalScan::perform
 * (CommonSources/CLGenericKernels.cpp:107-151).
 *
 * TEST INFRASTRUCTURE ONLY: it pins the oracle's C restatement of the build
 * (oracle/lbvh_oracle.c) against the reference's kernels themselves.  Built
 * only where the reference sources are present (oracle/build_oracle.py, which
 * compiles the kernels from the reference checkout through a pipe: nothing
 * of them is copied), into oracle/_ref/libref_lbvh_cl.so.
 *
 * Execution: oracle/ref_cl_exec.cpp.
 */
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "opencl_c.hpp"

typedef float3 point3;

// the kernels (C linkage through the `kernel` qualifier)
extern "C" {
void calcAABBs(const point3* vertices, const uchar* faces, uint numFaces, uchar* AABBs);
void unifyAABBs(const uchar* AABBs, uint numAABBs, uchar* unifiedAABBs);
void calcMortonCodes(const uchar* AABBs, uint numPrimitives, point3 minEntireAABB, point3 sizeEntireAABB,
                     uint numDivs, uint3* mortonCodes, uint* indices);
void blockwiseSort(const uint3* mortonCodes, uint numPrimitives, uchar bitID, uint* indices, uchar* radixDigits);
void calcBlockwiseHistograms(const uchar* radixDigits, uint numPrimitives, uint numBlocks, uint* histograms,
                             ushort* localOffsets);
void globalScatter(const uchar* radixDigits, uint numPrimitives, const uint* globalBucketOffsets,
                   const ushort* localOffsets, const uint* indicesSrc, uint* indicesDst);
void constructBinaryRadixTree(const uint3* mortonCodes, uint bitsPerDim, const uchar* AABBs, const uint* indices,
                              uint numPrimitives, uchar* iNodes, uchar* lNodes, uint* parentIdxs, uint* counters);
void calcNodeAABBs(uchar* _iNodes, uint* counters, const uchar* _lNodes, uint numPrimitives,
                   const uint* parentIdxs);
void localScan(uint* elements, uint numElements, uint* blockSums);
void addOffset(const uint* blockOffsets, uint* elements, uint numElements);
}

namespace {

template <typename F>
void run(size_t global_size, size_t local_size, bool barriers, F f) {
    clshim::launch(global_size, local_size, barriers, [](void* p) { (*static_cast<F*>(p))(); }, &f);
}

size_t round_up(size_t n, size_t m) { return (n + m - 1) / m * m; }

// GlobalScan::perform (CLGenericKernels.cpp:107-151): exclusive scan in place
void global_scan(uint* elements, uint num) {
    const uint block = 128;
    std::vector<std::vector<uint>> sums;
    std::vector<uint*> bufs{elements};
    std::vector<uint> counts{num};
    while (num > 1) {
        const uint blocks = (num + block - 1) / block;
        sums.emplace_back(blocks, 0u);
        uint* src = bufs.back();
        uint* dst = sums.back().data();
        const uint n = num;
        run(size_t(blocks) * block, block, true, [=] { localScan(src, n, dst); });
        num = blocks;
        bufs.push_back(dst);
        counts.push_back(num);
    }
    for (size_t depth = bufs.size() - 1; depth > 1; --depth) {
        const uint n = counts[depth - 2];
        const uint blocks = (n + block - 1) / block;
        const uint* off = bufs[depth - 1];
        uint* el = bufs[depth - 2];
        run(size_t(blocks) * block, block, false, [=] { addOffset(off, el, n); });
    }
}

}  // namespace

extern "C" {

/* LBVHBuilder::perform on the CPU.  Vertex k of triangle t is
 * (vx,vy,vz)[tri[3t+k]] (or [3t+k] when tri is NULL).  Outputs (caller
 * allocated): inodes (n-1) x 48 B, lnodes n x 48 B, parents 2n-1 uint32,
 * sorted_idx n, morton n x uint3 (16 B each), box 6 floats (scene min,
 * max).  Returns 0, or -1 for n < 2 (the reference does not build one
 * triangle). */
int ref_cl_lbvh_build(const float* vx, const float* vy, const float* vz, const uint32_t* tri, uint32_t n,
                      uint32_t bits, void* inodes, void* lnodes, uint32_t* parents, uint32_t* sorted_idx,
                      void* morton, float* box) {
    if (n < 2) return -1;
    const uint32_t nv = tri ? 0u : 3u * n;
    uint32_t num_verts = nv;
    if (tri)
        for (uint64_t i = 0; i < 3ull * n; ++i) num_verts = std::max(num_verts, tri[i] + 1u);
    std::vector<point3> verts(num_verts);
    for (uint32_t i = 0; i < num_verts; ++i) verts[i] = point3(vx[i], vy[i], vz[i]);
    struct FaceRec {  // Face.hpp / lbvh_construction.cl:16-23, 56 bytes
        uint32_t p[3], vn[3], vt[3], uv[3], alpha;
        uint16_t mat, light;
    };
    static_assert(sizeof(FaceRec) == 56, "Face is 56 bytes");
    std::vector<FaceRec> faces(n);
    for (uint32_t t = 0; t < n; ++t) {
        FaceRec& f = faces[t];
        std::memset(&f, 0xFF, sizeof(f));
        for (int k = 0; k < 3; ++k) f.p[k] = tri ? tri[3u * t + k] : 3u * t + k;
    }
    const uint32_t kAABB = 48;  // AABB: min, max, center (16 B each)
    std::vector<uchar> aabbs(size_t(kAABB) * n);
    const point3* vp = verts.data();
    const uchar* fp = reinterpret_cast<const uchar*>(faces.data());
    uchar* ap = aabbs.data();

    // calcAABBs
    run(round_up(n, 128), 128, false, [=] { calcAABBs(vp, fp, n, ap); });
    // unifyAABBs until one box is left (ping-pong buffers)
    std::vector<uchar> uni[2];
    const uchar* src = ap;
    uint32_t num = n, merged = (n + 127) / 128, swap = 0;
    uchar* out = nullptr;
    while (true) {
        std::vector<uchar>& dst = uni[swap++ % 2];
        dst.assign(size_t(kAABB) * merged, 0);
        out = dst.data();
        const uint32_t cnt = num;
        const uchar* s = src;
        uchar* d = out;
        run(size_t(merged) * 128, 128, true, [=] { unifyAABBs(s, cnt, d); });
        if (merged == 1) break;
        src = out;
        num = merged;
        merged = (num + 127) / 128;
    }
    point3 mn, mx;
    std::memcpy(&mn, out, 16);
    std::memcpy(&mx, out + 16, 16);
    const point3 size(mx.x - mn.x, mx.y - mn.y, mx.z - mn.z);  // on the host, LBVHBuilder.cpp:236-240
    box[0] = mn.x; box[1] = mn.y; box[2] = mn.z; box[3] = mx.x; box[4] = mx.y; box[5] = mx.z;

    // calcMortonCodes
    std::vector<uint3> codes(n);
    std::vector<uint> idx(n), shadow(n);
    uint3* cp = codes.data();
    uint* ip = idx.data();
    const uint divs = 1u << bits;
    run(round_up(n, 128), 128, false, [=] { calcMortonCodes(ap, n, mn, size, divs, cp, ip); });

    // b rounds of the blockwise 3-bit radix sort
    const uint32_t groups = (n + 63) / 64;
    std::vector<uchar> digits(size_t(groups) * 64);
    std::vector<uint> hist(size_t(groups) * 8);
    std::vector<ushort> loffs(size_t(groups) * 8);
    uint* cur = idx.data();
    uint* other = shadow.data();
    for (uint32_t i = 0; i < bits; ++i) {
        uchar* dp = digits.data();
        uint* hp = hist.data();
        ushort* lp = loffs.data();
        const uint3* ccp = codes.data();
        const uchar bit = (uchar)i;
        uint* c = cur;
        run(size_t(groups) * 64, 64, true, [=] { blockwiseSort(ccp, n, bit, c, dp); });
        run(round_up(groups, 128), 128, false, [=] { calcBlockwiseHistograms(dp, n, groups, hp, lp); });
        global_scan(hp, groups * 8);
        uint* o = other;
        run(size_t(groups) * 64, 64, false, [=] { globalScatter(dp, n, hp, lp, c, o); });
        std::swap(cur, other);
    }

    // constructBinaryRadixTree, calcNodeAABBs
    std::vector<uint> counters(n);
    uchar* inp = static_cast<uchar*>(inodes);
    uchar* lnp = static_cast<uchar*>(lnodes);
    uint* pp = parents;
    uint* cntp = counters.data();
    const uint* sorted = cur;
    const uint3* ccp = codes.data();
    std::memset(parents, 0xFF, sizeof(uint32_t) * (2ull * n - 1));
    run(round_up(n, 64), 64, false, [=] { constructBinaryRadixTree(ccp, bits, ap, sorted, n, inp, lnp, pp, cntp); });
    run(round_up(n, 64), 64, false, [=] { calcNodeAABBs(inp, cntp, lnp, n, pp); });

    std::memcpy(sorted_idx, cur, sizeof(uint32_t) * n);
    std::memcpy(morton, codes.data(), sizeof(uint3) * n);
    return 0;
}

}  // extern "C"
