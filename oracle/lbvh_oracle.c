/*
 * CPU oracle for the LBVH build and BVH traversal hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against; nothing in the shipped library links or calls it.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * It restates, in plain C, the algorithms of the reference (shocker-0x15/CLeaR,
 * an OpenCL 1.2 path tracer) with the reference's own floating-point
 * expressions, evaluated in the same order, so that the integer outputs
 * (sorted order, tree topology, hit triangle ids) are bit-identical:
 *
 *   orc_lbvh_build      OpenCL_PathTracer/OpenCL/lbvh_construction.cl:81-492
 *                       driven as OpenCL_PathTracer/LBVHBuilder.cpp:160-375
 *   orc_trace_closest   OpenCL_PathTracer/OpenCL/bvh_traversal.cl:54-108,160-215
 *                       (face ids are uint32 here; the reference truncates to
 *                        ushort at bvh_traversal.cl:43,56)
 *   orc_trace_shadow    the any-hit form of the same traversal (the reference
 *                       has none; it shoots a closest-hit ray, pathtracer.cl:121)
 *   orc_midbvh_build    OpenCL_PathTracer/BVH.hpp:86-175 (the reference's CPU
 *                       midpoint-split builder, used as the CPU baseline)
 *
 * Build with -ffp-contract=off and without fast-math: the reference's float
 * results are defined without fused multiply-add.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ENOMEM 2
#define ORC_ESTACK 3

/* 48-byte node records, byte-compatible with LBVH::InternalNode/LeafNode
 * (OpenCL_PathTracer/LBVHBuilder.h:17-29). */
typedef struct {
    float min[4];
    float max[4];
    uint8_t isChild[2];
    uint8_t pad0[2];
    uint32_t c[2];
    uint8_t pad1[4];
} orc_inode;

typedef struct {
    float min[4];
    float max[4];
    uint32_t objIdx;
    uint8_t pad[12];
} orc_lnode;

/* BVHNode of the reference's CPU builder (OpenCL_PathTracer/BVH.hpp:61-68). */
typedef struct {
    float min[4];
    float max[4];
    uint32_t children[2];
    uint32_t pad[2];
} orc_bvhnode;

static inline uint32_t vidx(const uint32_t* tri, uint32_t t, uint32_t k) {
    return tri ? tri[3u * t + k] : 3u * t + k;
}

static inline int clz32(uint32_t v) { return v ? __builtin_clz(v) : 32; }

/* convert_uint_rtz for the in-range values the reference produces; NaN (a
 * zero-extent scene axis gives 0/0) maps to 0 and values past the range
 * saturate, which is what the CUDA conversion __float2uint_rz does. */
static inline uint32_t cvt_rtz_u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}

/* 3b-bit Morton key whose order equals the reference's LSD sort order: the
 * per-bit digit is x | y<<1 | z<<2 (lbvh_construction.cl:245-246), sorted from
 * bit 0 upwards (LBVHBuilder.cpp:263). */
uint64_t orc_morton_key(uint32_t qx, uint32_t qy, uint32_t qz, uint32_t bits) {
    uint64_t k = 0;
    for (uint32_t b = 0; b < bits; ++b) {
        uint64_t d = ((qx >> b) & 1u) | (((qy >> b) & 1u) << 1) | (((qz >> b) & 1u) << 2);
        k |= d << (3u * b);
    }
    return k;
}

/* _numCommonBits, lbvh_construction.cl:322-332.  Returns the reference's
 * signed 8-bit value; out-of-range j gives -1. */
static int8_t num_common_bits(const uint32_t* q, const uint32_t* indices, int64_t n, uint32_t bits,
                              const uint32_t* qi, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t* qj = q + 3u * indices[j];
    int dx = clz32(qi[0] ^ qj[0]) - (32 - (int)bits);
    int dy = clz32(qi[1] ^ qj[1]) - (32 - (int)bits);
    int dz = clz32(qi[2] ^ qj[2]) - (32 - (int)bits);
    int r = dz * 3 + 0;
    if (dy * 3 + 1 < r) r = dy * 3 + 1;
    if (dx * 3 + 2 < r) r = dx * 3 + 2;
    int8_t ret = (int8_t)r;
    if ((uint32_t)(int32_t)ret != bits * 3u) return ret;
    return (int8_t)(ret + clz32((uint32_t)(int32_t)i ^ (uint32_t)(int32_t)j));
}

static inline int8_t sign8(int v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

/*
 * Full LBVH build.  Vertex k of triangle t is (vx,vy,vz)[tri[3t+k]] (or
 * [3t+k] when tri is NULL).  Outputs (caller-allocated):
 *   inodes[n-1], lnodes[n]     reference-layout nodes (root = inodes[0])
 *   parents[2n-1]              leaves at [0,n), internal nodes at [n,2n-1)
 *   sorted_idx[n]              triangle ids in sorted (leaf) order
 *   q[3n] (optional)           per-triangle quantised coordinates, input order
 *   scene_box[6] (optional)    min xyz, max xyz of the whole scene
 * n == 1 gives one leaf and no internal node (the reference does not support
 * it; traversal treats the single leaf as the root).
 */
int orc_lbvh_build(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                   uint32_t n, uint32_t bits,
                   orc_inode* inodes, orc_lnode* lnodes, uint32_t* parents,
                   uint32_t* sorted_idx, uint32_t* q_out, float* scene_box) {
    if (bits < 1 || bits > 21) return ORC_EINVAL;
    if (n == 0) return ORC_OK;
    float* box = (float*)malloc(sizeof(float) * 9u * n); /* min3 max3 center3 */
    uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * 3u * n);
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * n);
    if (!box || !q || !idx || !tmp) { free(box); free(q); free(idx); free(tmp); return ORC_ENOMEM; }

    /* calcAABBs, lbvh_construction.cl:81-96 */
    for (uint32_t t = 0; t < n; ++t) {
        uint32_t a = vidx(tri, t, 0), b = vidx(tri, t, 1), c = vidx(tri, t, 2);
        const float p0[3] = {vx[a], vy[a], vz[a]};
        const float p1[3] = {vx[b], vy[b], vz[b]};
        const float p2[3] = {vx[c], vy[c], vz[c]};
        for (int k = 0; k < 3; ++k) {
            float mn = fminf(p0[k], fminf(p1[k], p2[k]));
            float mx = fmaxf(p0[k], fmaxf(p1[k], p2[k]));
            box[9u * t + k] = mn;
            box[9u * t + 3 + k] = mx;
            box[9u * t + 6 + k] = (mn + mx) * 0.5f;
        }
    }
    /* unifyAABBs (lbvh_construction.cl:105-162): min/max over all boxes. */
    float smin[3] = {INFINITY, INFINITY, INFINITY}, smax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t t = 0; t < n; ++t)
        for (int k = 0; k < 3; ++k) {
            smin[k] = fminf(smin[k], box[9u * t + k]);
            smax[k] = fmaxf(smax[k], box[9u * t + 3 + k]);
        }
    /* scene size on the host, LBVHBuilder.cpp:236-240 */
    float ssize[3] = {smax[0] - smin[0], smax[1] - smin[1], smax[2] - smin[2]};
    if (scene_box) for (int k = 0; k < 3; ++k) { scene_box[k] = smin[k]; scene_box[3 + k] = smax[k]; }

    /* calcMortonCodes, lbvh_construction.cl:169-181 with numDivs = 1<<bits
     * (LBVHBuilder.cpp:244). */
    const uint32_t numDivs = 1u << bits;
    for (uint32_t t = 0; t < n; ++t) {
        for (int k = 0; k < 3; ++k) {
            float normPos = (box[9u * t + 6 + k] - smin[k]) / ssize[k];
            uint32_t v = cvt_rtz_u32(normPos * (float)numDivs);
            q[3u * t + k] = v < numDivs - 1u ? v : numDivs - 1u;
        }
        idx[t] = t;
    }
    if (q_out) memcpy(q_out, q, sizeof(uint32_t) * 3u * n);

    /* Radix sort, LBVHBuilder.cpp:263-287.  Each round is blockwiseSort
     * (a stable in-block split on the 3-bit digit, :231-272), block
     * histograms stored digit-major (:279-298), a global exclusive scan and a
     * scatter at scanned offset + in-block rank (:304-316): together a stable
     * partition of the whole index array by the round's digit.  It is
     * restated here as a stable counting sort per round. */
    for (uint32_t bit = 0; bit < bits; ++bit) {
        uint32_t count[8] = {0}, off[8];
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t* qq = q + 3u * idx[i];
            uint32_t d = ((qq[0] >> bit) & 1u) | (((qq[1] >> bit) & 1u) << 1) | (((qq[2] >> bit) & 1u) << 2);
            count[d]++;
        }
        uint32_t s = 0;
        for (int d = 0; d < 8; ++d) { off[d] = s; s += count[d]; }
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t* qq = q + 3u * idx[i];
            uint32_t d = ((qq[0] >> bit) & 1u) | (((qq[1] >> bit) & 1u) << 1) | (((qq[2] >> bit) & 1u) << 2);
            tmp[off[d]++] = idx[i];
        }
        uint32_t* sw = idx; idx = tmp; tmp = sw;
    }
    memcpy(sorted_idx, idx, sizeof(uint32_t) * n);

    /* constructBinaryRadixTree, lbvh_construction.cl:342-410 */
    for (uint32_t g = 0; g < n; ++g) {
        uint32_t objIdx = idx[g];
        orc_lnode* ln = lnodes + g;
        memset(ln, 0, sizeof(*ln));
        for (int k = 0; k < 3; ++k) { ln->min[k] = box[9u * objIdx + k]; ln->max[k] = box[9u * objIdx + 3 + k]; }
        ln->objIdx = objIdx;
        if (g >= n - 1) continue;
        const uint32_t* qi = q + 3u * objIdx;
        const int64_t gi = (int64_t)g, nn = (int64_t)n;
        int8_t commonR = num_common_bits(q, idx, nn, bits, qi, gi, gi + 1);
        int8_t commonL = num_common_bits(q, idx, nn, bits, qi, gi, gi - 1);
        int8_t d = sign8((int)commonR - (int)commonL);
        int8_t minNum = d > 0 ? commonL : commonR;
        int64_t lMax = 2;
        while (num_common_bits(q, idx, nn, bits, qi, gi, gi + lMax * d) > minNum) lMax <<= 1;
        int64_t l = 0;
        for (int64_t t = lMax >> 1; t >= 1; t >>= 1)
            if (num_common_bits(q, idx, nn, bits, qi, gi, gi + (l + t) * d) > minNum) l += t;
        int64_t otherEnd = gi + l * d;
        int8_t numNode = num_common_bits(q, idx, nn, bits, qi, gi, otherEnd);
        int64_t split = 0;
        float scale = 0.5f;
        for (;;) {
            uint32_t t = (uint32_t)ceilf((float)(uint32_t)l * scale);
            if (num_common_bits(q, idx, nn, bits, qi, gi, gi + (split + (int64_t)t) * d) > numNode) split += t;
            if (t <= 1) break;
            scale *= 0.5f;
        }
        int64_t splitPos = gi + split * d + (d < 0 ? d : 0);
        orc_inode* in = inodes + g;
        memset(in, 0, sizeof(*in));
        int64_t lo = gi < otherEnd ? gi : otherEnd, hi = gi < otherEnd ? otherEnd : gi;
        int leftIsLeaf = lo == splitPos, rightIsLeaf = hi == splitPos + 1;
        in->isChild[0] = (uint8_t)leftIsLeaf;
        in->c[0] = (uint32_t)splitPos;
        parents[leftIsLeaf ? (uint32_t)splitPos : n + (uint32_t)splitPos] = g;
        in->isChild[1] = (uint8_t)rightIsLeaf;
        in->c[1] = (uint32_t)(splitPos + 1);
        parents[rightIsLeaf ? (uint32_t)(splitPos + 1) : n + (uint32_t)(splitPos + 1)] = g;
    }

    /* calcNodeAABBs (lbvh_construction.cl:415-492): every internal node's box
     * is the union of its children's boxes.  The reference climbs with atomic
     * counters; min/max are exact, so a post-order walk gives the same values. */
    if (n >= 2) {
        uint32_t* stack = tmp; /* reuse: post-order walk with visit marks */
        uint8_t* seen = (uint8_t*)calloc(n - 1, 1);
        if (!seen) { free(box); free(q); free(idx); free(tmp); return ORC_ENOMEM; }
        uint32_t sp = 0;
        stack[sp++] = 0;
        while (sp) {
            uint32_t v = stack[sp - 1];
            orc_inode* in = inodes + v;
            if (!seen[v]) {
                seen[v] = 1;
                for (int c = 0; c < 2; ++c) if (!in->isChild[c]) stack[sp++] = in->c[c];
                continue;
            }
            --sp;
            const float *amin, *amax, *bmin, *bmax;
            if (in->isChild[0]) { amin = lnodes[in->c[0]].min; amax = lnodes[in->c[0]].max; }
            else { amin = inodes[in->c[0]].min; amax = inodes[in->c[0]].max; }
            if (in->isChild[1]) { bmin = lnodes[in->c[1]].min; bmax = lnodes[in->c[1]].max; }
            else { bmin = inodes[in->c[1]].min; bmax = inodes[in->c[1]].max; }
            for (int k = 0; k < 3; ++k) { in->min[k] = fminf(amin[k], bmin[k]); in->max[k] = fmaxf(amax[k], bmax[k]); }
        }
        free(seen);
    }
    free(box); free(q); free(idx); free(tmp);
    return ORC_OK;
}

/* ------------------------------------------ the same build on all host cores
 *
 * orc_lbvh_build_mt is orc_lbvh_build run data-parallel, stage by stage, the
 * way the reference's kernels run on an OpenCL device: calcAABBs and
 * calcMortonCodes per triangle, unifyAABBs as a reduction, each of the b
 * sort rounds as a stable split on its 3-bit digit (per-thread digit counts
 * over contiguous chunks, a scan over digit-major (digit, chunk) pairs, a
 * scatter: the blockwiseSort / calcBlockwiseHistograms / GlobalScan /
 * globalScatter round of LBVHBuilder.cpp:263-287), constructBinaryRadixTree
 * per internal node, and calcNodeAABBs as the reference's bottom-up climb with
 * an atomic arrival counter per node (lbvh_construction.cl:415-492).  Every
 * stage computes the serial build's values, so the outputs are identical.
 * It is the CPU baseline of the build (the reference's OpenCL kernels cannot
 * run on a host without an OpenCL driver); `threads` <= 0 uses all cores. */
#ifdef _OPENMP
#include <omp.h>
#endif

static void karras_node(const uint32_t* q, const uint32_t* idx, uint32_t n, uint32_t bits, uint32_t g,
                        orc_inode* inodes, uint32_t* parents) {
    const uint32_t* qi = q + 3u * idx[g];
    const int64_t gi = (int64_t)g, nn = (int64_t)n;
    int8_t commonR = num_common_bits(q, idx, nn, bits, qi, gi, gi + 1);
    int8_t commonL = num_common_bits(q, idx, nn, bits, qi, gi, gi - 1);
    int8_t d = sign8((int)commonR - (int)commonL);
    int8_t minNum = d > 0 ? commonL : commonR;
    int64_t lMax = 2;
    while (num_common_bits(q, idx, nn, bits, qi, gi, gi + lMax * d) > minNum) lMax <<= 1;
    int64_t l = 0;
    for (int64_t t = lMax >> 1; t >= 1; t >>= 1)
        if (num_common_bits(q, idx, nn, bits, qi, gi, gi + (l + t) * d) > minNum) l += t;
    int64_t otherEnd = gi + l * d;
    int8_t numNode = num_common_bits(q, idx, nn, bits, qi, gi, otherEnd);
    int64_t split = 0;
    float scale = 0.5f;
    for (;;) {
        uint32_t t = (uint32_t)ceilf((float)(uint32_t)l * scale);
        if (num_common_bits(q, idx, nn, bits, qi, gi, gi + (split + (int64_t)t) * d) > numNode) split += t;
        if (t <= 1) break;
        scale *= 0.5f;
    }
    int64_t splitPos = gi + split * d + (d < 0 ? d : 0);
    orc_inode* in = inodes + g;
    memset(in, 0, sizeof(*in));
    int64_t lo = gi < otherEnd ? gi : otherEnd, hi = gi < otherEnd ? otherEnd : gi;
    int leftIsLeaf = lo == splitPos, rightIsLeaf = hi == splitPos + 1;
    in->isChild[0] = (uint8_t)leftIsLeaf;
    in->c[0] = (uint32_t)splitPos;
    parents[leftIsLeaf ? (uint32_t)splitPos : n + (uint32_t)splitPos] = g;
    in->isChild[1] = (uint8_t)rightIsLeaf;
    in->c[1] = (uint32_t)(splitPos + 1);
    parents[rightIsLeaf ? (uint32_t)(splitPos + 1) : n + (uint32_t)(splitPos + 1)] = g;
}

int orc_lbvh_build_mt(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                      uint32_t n, uint32_t bits,
                      orc_inode* inodes, orc_lnode* lnodes, uint32_t* parents,
                      uint32_t* sorted_idx, float* scene_box, int threads) {
    if (bits < 1 || bits > 21) return ORC_EINVAL;
    if (n == 0) return ORC_OK;
    int nt = 1;
#ifdef _OPENMP
    nt = threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
#endif
    float* box = (float*)malloc(sizeof(float) * 9u * n);
    uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * 3u * n);
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* cnt = (uint32_t*)malloc(sizeof(uint32_t) * 8u * (uint32_t)nt);
    uint32_t* arrivals = (uint32_t*)calloc(n > 1 ? n - 1 : 1, sizeof(uint32_t));
    float* red = (float*)malloc(sizeof(float) * 6u * (uint32_t)nt);
    if (!box || !q || !idx || !tmp || !cnt || !arrivals || !red) {
        free(box); free(q); free(idx); free(tmp); free(cnt); free(arrivals); free(red);
        return ORC_ENOMEM;
    }
    const int64_t N = (int64_t)n;
    const uint32_t numDivs = 1u << bits;
    float smin[3], smax[3], ssize[3];
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
        int tid = 0, T = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        T = omp_get_num_threads();
#endif
        const int64_t c0 = N * tid / T, c1 = N * (tid + 1) / T;  /* this thread's chunk */
        /* calcAABBs, lbvh_construction.cl:81-96; unifyAABBs per chunk */
        float mn3[3] = {INFINITY, INFINITY, INFINITY}, mx3[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t t = c0; t < c1; ++t) {
            uint32_t a = vidx(tri, (uint32_t)t, 0), b = vidx(tri, (uint32_t)t, 1), c = vidx(tri, (uint32_t)t, 2);
            const float p0[3] = {vx[a], vy[a], vz[a]}, p1[3] = {vx[b], vy[b], vz[b]}, p2[3] = {vx[c], vy[c], vz[c]};
            for (int k = 0; k < 3; ++k) {
                float mn = fminf(p0[k], fminf(p1[k], p2[k]));
                float mx = fmaxf(p0[k], fmaxf(p1[k], p2[k]));
                box[9u * t + k] = mn;
                box[9u * t + 3 + k] = mx;
                box[9u * t + 6 + k] = (mn + mx) * 0.5f;
                mn3[k] = fminf(mn3[k], mn);
                mx3[k] = fmaxf(mx3[k], mx);
            }
        }
        for (int k = 0; k < 3; ++k) { red[6 * tid + k] = mn3[k]; red[6 * tid + 3 + k] = mx3[k]; }
#ifdef _OPENMP
#pragma omp barrier
#pragma omp single
#endif
        {
            for (int k = 0; k < 3; ++k) { smin[k] = INFINITY; smax[k] = -INFINITY; }
            for (int u = 0; u < T; ++u)
                for (int k = 0; k < 3; ++k) {
                    smin[k] = fminf(smin[k], red[6 * u + k]);
                    smax[k] = fmaxf(smax[k], red[6 * u + 3 + k]);
                }
            for (int k = 0; k < 3; ++k) ssize[k] = smax[k] - smin[k];
        }
        /* calcMortonCodes, lbvh_construction.cl:169-181 */
        for (int64_t t = c0; t < c1; ++t) {
            for (int k = 0; k < 3; ++k) {
                float normPos = (box[9u * t + 6 + k] - smin[k]) / ssize[k];
                uint32_t v = cvt_rtz_u32(normPos * (float)numDivs);
                q[3u * t + k] = v < numDivs - 1u ? v : numDivs - 1u;
            }
            idx[t] = (uint32_t)t;
        }
        /* b rounds of a stable split on the round's 3-bit digit */
        uint32_t *src = idx, *dst = tmp;
        for (uint32_t bit = 0; bit < bits; ++bit) {
#ifdef _OPENMP
#pragma omp barrier
#endif
            uint32_t c8[8] = {0};
            for (int64_t i = c0; i < c1; ++i) {
                const uint32_t* qq = q + 3u * src[i];
                c8[((qq[0] >> bit) & 1u) | (((qq[1] >> bit) & 1u) << 1) | (((qq[2] >> bit) & 1u) << 2)]++;
            }
            for (int d = 0; d < 8; ++d) cnt[8 * tid + d] = c8[d];
#ifdef _OPENMP
#pragma omp barrier
#endif
            /* offset of (digit d, chunk tid) = all smaller digits + digit d of earlier chunks */
            uint32_t off[8];
            uint32_t base = 0;
            for (int d = 0; d < 8; ++d) {
                uint32_t before = 0, total = 0;
                for (int u = 0; u < T; ++u) {
                    if (u < tid) before += cnt[8 * u + d];
                    total += cnt[8 * u + d];
                }
                off[d] = base + before;
                base += total;
            }
            for (int64_t i = c0; i < c1; ++i) {
                const uint32_t* qq = q + 3u * src[i];
                uint32_t d = ((qq[0] >> bit) & 1u) | (((qq[1] >> bit) & 1u) << 1) | (((qq[2] >> bit) & 1u) << 2);
                dst[off[d]++] = src[i];
            }
            uint32_t* sw = src; src = dst; dst = sw;
        }
#ifdef _OPENMP
#pragma omp barrier
#endif
        /* leaves, then constructBinaryRadixTree (lbvh_construction.cl:342-410) */
        for (int64_t g = c0; g < c1; ++g) {
            uint32_t objIdx = src[g];
            orc_lnode* ln = lnodes + g;
            memset(ln, 0, sizeof(*ln));
            for (int k = 0; k < 3; ++k) { ln->min[k] = box[9u * objIdx + k]; ln->max[k] = box[9u * objIdx + 3 + k]; }
            ln->objIdx = objIdx;
            sorted_idx[g] = objIdx;
        }
        for (int64_t g = c0; g < c1; ++g)
            if (g < N - 1) karras_node(q, src, n, bits, (uint32_t)g, inodes, parents);
#ifdef _OPENMP
#pragma omp barrier
#endif
        /* calcNodeAABBs: from each leaf, climb; the second child to arrive at
         * a node (acquire-release counter) merges both boxes and goes on */
        if (n >= 2)
            for (int64_t g = c0; g < c1; ++g) {
                uint32_t node = parents[g];
                for (;;) {
                    if (__atomic_fetch_add(&arrivals[node], 1u, __ATOMIC_ACQ_REL) == 0) break;
                    orc_inode* in = inodes + node;
                    const float *amin, *amax, *bmin, *bmax;
                    if (in->isChild[0]) { amin = lnodes[in->c[0]].min; amax = lnodes[in->c[0]].max; }
                    else { amin = inodes[in->c[0]].min; amax = inodes[in->c[0]].max; }
                    if (in->isChild[1]) { bmin = lnodes[in->c[1]].min; bmax = lnodes[in->c[1]].max; }
                    else { bmin = inodes[in->c[1]].min; bmax = inodes[in->c[1]].max; }
                    for (int k = 0; k < 3; ++k) {
                        in->min[k] = fminf(amin[k], bmin[k]);
                        in->max[k] = fmaxf(amax[k], bmax[k]);
                    }
                    if (node == 0) break;
                    node = parents[n + node];
                }
            }
    }
    if (scene_box) for (int k = 0; k < 3; ++k) { scene_box[k] = smin[k]; scene_box[3 + k] = smax[k]; }
    free(box); free(q); free(idx); free(tmp); free(cnt); free(arrivals); free(red);
    return ORC_OK;
}

/* ---------------------------------------------------------------- traversal */

typedef struct { float x, y, z; } v3;
static inline v3 v3sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 v3cross(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static inline float v3dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* rayTriangleIntersection, bvh_traversal.cl:54-108 (no alpha texture on this
 * path).  Updates *t and returns 1 when the hit is accepted. */
static int ray_tri(const float* vx, const float* vy, const float* vz, const uint32_t* tri, uint32_t f,
                   v3 org, v3 dir, float* t) {
    uint32_t a = vidx(tri, f, 0), b = vidx(tri, f, 1), c = vidx(tri, f, 2);
    v3 p0 = {vx[a], vy[a], vz[a]}, p1 = {vx[b], vy[b], vz[b]}, p2 = {vx[c], vy[c], vz[c]};
    v3 e1 = v3sub(p1, p0), e2 = v3sub(p2, p0);
    v3 p = v3cross(dir, e2);
    float det = v3dot(e1, p);
    if (det > -0.000001f && det < 0.000001f) return 0;
    float invDet = 1.0f / det;
    v3 d = v3sub(org, p0);
    float b1 = v3dot(d, p) * invDet;
    if (b1 < 0.0f || b1 > 1.0f) return 0;
    v3 qv = v3cross(d, e1);
    float b2 = v3dot(dir, qv) * invDet;
    if (b2 < 0.0f || b1 + b2 > 1.0f) return 0;
    float tt = v3dot(e2, qv) * invDet;
    if (tt < 0.0f || tt > *t) return 0;
    *t = tt;
    return 1;
}

/* rayAABBIntersection, bvh_traversal.cl:160-179 (Woo's outside-plane test). */
static int ray_box(const float* bmin, const float* bmax, v3 org, v3 dir, float tBound) {
    const float o[3] = {org.x, org.y, org.z}, dd[3] = {dir.x, dir.y, dir.z};
    int lmu[3];
    for (int k = 0; k < 3; ++k) lmu[k] = o[k] < bmin[k] ? -1 : (o[k] > bmax[k] ? 1 : 0);
    if (lmu[0] | lmu[1] | lmu[2]) {
        float tk[3];
        for (int k = 0; k < 3; ++k) {
            float cand = o[k] < bmin[k] ? bmin[k] : (o[k] > bmax[k] ? bmax[k] : 0.0f);
            tk[k] = (lmu[k] != 0 && dd[k] != 0.0f) ? (cand - o[k]) / dd[k] : -1.0f;
        }
        float maxt = fmaxf(tk[0], fmaxf(tk[1], tk[2]));
        if (maxt < 0.0f || maxt > tBound) return 0;
        for (int k = 0; k < 3; ++k) {
            float coord = o[k] + maxt * dd[k];
            int hit = (coord >= bmin[k] && coord <= bmax[k]) || tk[k] == maxt;
            if (!hit) return 0;
        }
    }
    return 1;
}

#define ORC_STACK 256

/* rays: 8 floats per ray {ox,oy,oz,tmax, dx,dy,dz,unused}.
 * Closest hit, rayIntersection (bvh_traversal.cl:182-215) with t starting at
 * tmax (the reference starts at INFINITY).  Miss: id 0xFFFFFFFF, t = tmax.
 * stats (optional, 4 per ray): internal nodes popped, internal boxes
 * accepted, leaf box tests, leaf boxes accepted (= triangle tests); the
 * second plus the fourth is numAABBHit of rayIntersectionVis
 * (bvh_traversal.cl:217-254). */
int orc_trace_closest(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                      const orc_inode* inodes, const orc_lnode* lnodes, uint32_t n,
                      const float* rays, uint32_t nrays, uint32_t* hit_id, float* hit_t,
                      uint32_t* stats) {
    int status = ORC_OK;
    for (uint32_t r = 0; r < nrays; ++r) {
        const float* R = rays + 8u * r;
        v3 org = {R[0], R[1], R[2]}, dir = {R[4], R[5], R[6]};
        float t = R[3];
        uint32_t best = 0xFFFFFFFFu;
        uint32_t s_in = 0, s_acc = 0, s_leaf = 0, s_tri = 0;
        if (n == 1) {
            ++s_leaf;
            if (ray_box(lnodes[0].min, lnodes[0].max, org, dir, t)) {
                ++s_tri;
                if (ray_tri(vx, vy, vz, tri, lnodes[0].objIdx, org, dir, &t)) best = lnodes[0].objIdx;
            }
        } else if (n >= 2) {
            uint32_t stack[ORC_STACK];
            uint32_t depth = 0;
            stack[depth++] = 0;
            while (depth > 0) {
                const orc_inode* in = inodes + stack[--depth];
                ++s_in;
                if (!ray_box(in->min, in->max, org, dir, t)) continue;
                ++s_acc;
                for (int i = 0; i < 2; ++i) {
                    if (!in->isChild[i]) {
                        if (depth >= ORC_STACK) { status = ORC_ESTACK; continue; }
                        stack[depth++] = in->c[i];
                        continue;
                    }
                    const orc_lnode* ln = lnodes + in->c[i];
                    ++s_leaf;
                    if (!ray_box(ln->min, ln->max, org, dir, t)) continue;
                    ++s_tri;
                    if (ray_tri(vx, vy, vz, tri, ln->objIdx, org, dir, &t)) best = ln->objIdx;
                }
            }
        }
        hit_id[r] = best;
        hit_t[r] = t;
        if (stats) {
            stats[4u * r] = s_in;
            stats[4u * r + 1] = s_acc;
            stats[4u * r + 2] = s_leaf;
            stats[4u * r + 3] = s_tri;
        }
    }
    return status;
}

/* Shadow (any-hit) query: occluded[r] = 1 when some triangle reachable with the
 * box bound held at tmax is hit with 0 <= t <= tmax.  The bound never shrinks,
 * so the answer does not depend on the visiting order. */
int orc_trace_shadow(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                     const orc_inode* inodes, const orc_lnode* lnodes, uint32_t n,
                     const float* rays, uint32_t nrays, uint8_t* occluded) {
    int status = ORC_OK;
    for (uint32_t r = 0; r < nrays; ++r) {
        const float* R = rays + 8u * r;
        v3 org = {R[0], R[1], R[2]}, dir = {R[4], R[5], R[6]};
        const float tmax = R[3];
        int occ = 0;
        if (n == 1) {
            float t = tmax;
            occ = ray_box(lnodes[0].min, lnodes[0].max, org, dir, tmax) &&
                  ray_tri(vx, vy, vz, tri, lnodes[0].objIdx, org, dir, &t);
        } else if (n >= 2) {
            uint32_t stack[ORC_STACK];
            uint32_t depth = 0;
            stack[depth++] = 0;
            while (depth > 0 && !occ) {
                const orc_inode* in = inodes + stack[--depth];
                if (!ray_box(in->min, in->max, org, dir, tmax)) continue;
                for (int i = 0; i < 2 && !occ; ++i) {
                    if (!in->isChild[i]) {
                        if (depth >= ORC_STACK) { status = ORC_ESTACK; continue; }
                        stack[depth++] = in->c[i];
                        continue;
                    }
                    const orc_lnode* ln = lnodes + in->c[i];
                    if (!ray_box(ln->min, ln->max, org, dir, tmax)) continue;
                    float t = tmax;
                    if (ray_tri(vx, vy, vz, tri, ln->objIdx, org, dir, &t)) occ = 1;
                }
            }
        }
        occluded[r] = (uint8_t)occ;
    }
    return status;
}

/* ------------------------------------------------- CPU midpoint BVH builder */

typedef struct {
    float mn[3], mx[3];
} obox;

static inline float ctr(const obox* b, int axis) { return (b->mn[axis] + b->mx[axis]) * 0.5f; }
/* std::min / std::max as CLUtil::minCLfloat3 uses them (CommonSources/clUtility.cpp:544-552) */
static inline float smin_(float a, float b) { return (b < a) ? b : a; }
static inline float smax_(float a, float b) { return (a < b) ? b : a; }

typedef struct {
    const obox* leaves;
    uint32_t* lIdx;
    orc_bvhnode* nodes;
    uint32_t count;
} midctx;

/* BVH::divide(start, end, axis, pivot, &split), BVH.hpp:119-138 */
static uint32_t mid_divide(midctx* c, uint32_t start, uint32_t end, int axis, float pivot) {
    if (end - start <= 2) return (start + end) / 2;
    uint32_t left = start - 1, right = end;
    for (;;) {
        while (ctr(&c->leaves[c->lIdx[++left]], axis) < pivot) {}
        while (ctr(&c->leaves[c->lIdx[--right]], axis) > pivot) {}
        if (left < right) { uint32_t s = c->lIdx[left]; c->lIdx[left] = c->lIdx[right]; c->lIdx[right] = s; }
        else return left > start + 1 ? left : start + 1;
    }
}

/* BVH::buildRecursive, BVH.hpp:140-170, with the recursion kept on an
 * explicit stack in the same pre-order, so node numbering is identical. */
static void mid_build(midctx* c, uint32_t n) {
    typedef struct { uint32_t node, start, end, phase, split; } frame;
    uint32_t cap = 256, sp = 0;
    frame* st = (frame*)malloc(sizeof(frame) * cap);
    st[sp++] = (frame){0, 0, n, 0, 0};
    while (sp) {
        frame* f = &st[sp - 1];
        if (f->phase == 0) {
            obox bb = {{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
            for (uint32_t i = f->start; i < f->end; ++i)
                for (int k = 0; k < 3; ++k) {
                    bb.mn[k] = smin_(bb.mn[k], c->leaves[c->lIdx[i]].mn[k]);
                    bb.mx[k] = smax_(bb.mx[k], c->leaves[c->lIdx[i]].mx[k]);
                }
            orc_bvhnode* nd = &c->nodes[f->node];
            for (int k = 0; k < 3; ++k) { nd->min[k] = bb.mn[k]; nd->max[k] = bb.mx[k]; }
            if (f->end - f->start < 2) { nd->children[0] = c->lIdx[f->start]; --sp; continue; }
            float dx = bb.mx[0] - bb.mn[0], dy = bb.mx[1] - bb.mn[1], dz = bb.mx[2] - bb.mn[2];
            int axis = (dx > dy && dx > dz) ? 0 : (dy > dz ? 1 : 2);
            f->split = mid_divide(c, f->start, f->end, axis, ctr(&bb, axis));
            uint32_t child = c->count++;
            c->nodes[f->node].children[0] = child;
            f->phase = 1;
            if (sp == cap) { cap *= 2; st = (frame*)realloc(st, sizeof(frame) * cap); f = &st[sp - 1]; }
            st[sp++] = (frame){child, f->start, f->split, 0, 0};
        } else if (f->phase == 1) {
            uint32_t child = c->count++;
            c->nodes[f->node].children[1] = child;
            f->phase = 2;
            uint32_t s = f->split, e = f->end;
            if (sp == cap) { cap *= 2; st = (frame*)realloc(st, sizeof(frame) * cap); f = &st[sp - 1]; }
            st[sp++] = (frame){child, s, e, 0, 0};
        } else {
            --sp;
        }
    }
    free(st);
}

/* Reference CPU build (Scene.cpp:328-334 + BVH.hpp:172-175).  nodes must hold
 * 2n-1 entries; returns the node count. */
int64_t orc_midbvh_build(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                         uint32_t n, orc_bvhnode* nodes) {
    if (n == 0) return 0;
    obox* leaves = (obox*)malloc(sizeof(obox) * n);
    uint32_t* lIdx = (uint32_t*)malloc(sizeof(uint32_t) * n);
    if (!leaves || !lIdx) { free(leaves); free(lIdx); return -1; }
    for (uint32_t t = 0; t < n; ++t) {
        uint32_t a = vidx(tri, t, 0), b = vidx(tri, t, 1), cc = vidx(tri, t, 2);
        obox bb = {{vx[a], vy[a], vz[a]}, {vx[a], vy[a], vz[a]}};
        const float pb[3] = {vx[b], vy[b], vz[b]}, pc[3] = {vx[cc], vy[cc], vz[cc]};
        for (int k = 0; k < 3; ++k) {
            bb.mn[k] = smin_(bb.mn[k], pb[k]); bb.mx[k] = smax_(bb.mx[k], pb[k]);
            bb.mn[k] = smin_(bb.mn[k], pc[k]); bb.mx[k] = smax_(bb.mx[k], pc[k]);
        }
        leaves[t] = bb;
        lIdx[t] = t;
    }
    memset(nodes, 0, sizeof(orc_bvhnode) * (2u * (uint64_t)n - 1u));
    for (uint64_t i = 0; i < 2u * (uint64_t)n - 1u; ++i) nodes[i].children[0] = nodes[i].children[1] = 0xFFFFFFFFu;
    midctx c = {leaves, lIdx, nodes, 1};
    mid_build(&c, n);
    free(leaves); free(lIdx);
    return (int64_t)c.count;
}

/* Closest hit over the midpoint BVH, bvh_traversal.cl:256-285. */
int orc_trace_closest_mid(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                          const orc_bvhnode* nodes, uint32_t n, const float* rays, uint32_t nrays,
                          uint32_t* hit_id, float* hit_t) {
    int status = ORC_OK;
    for (uint32_t r = 0; r < nrays; ++r) {
        const float* R = rays + 8u * r;
        v3 org = {R[0], R[1], R[2]}, dir = {R[4], R[5], R[6]};
        float t = R[3];
        uint32_t best = 0xFFFFFFFFu;
        if (n) {
            uint32_t stack[ORC_STACK];
            uint32_t depth = 0;
            stack[depth++] = 0;
            while (depth > 0) {
                const orc_bvhnode* nd = nodes + stack[--depth];
                if (!ray_box(nd->min, nd->max, org, dir, t)) continue;
                if (nd->children[1] != 0xFFFFFFFFu) {
                    if (depth + 2 > ORC_STACK) { status = ORC_ESTACK; continue; }
                    stack[depth++] = nd->children[1];
                    stack[depth++] = nd->children[0];
                } else if (ray_tri(vx, vy, vz, tri, nd->children[0], org, dir, &t)) {
                    best = nd->children[0];
                }
            }
        }
        hit_id[r] = best;
        hit_t[r] = t;
    }
    return status;
}
