// BVH traversal on sm_103a: closest-hit and shadow (any-hit) queries.
//
// The root node index is root_box[3] (bit pattern).  clr_trace_closest
// visits nodes in the reference's order (OpenCL/bvh_traversal.cl:182-215):
// pop a node, handle child 0 then child 1, a leaf child is box-tested and its
// triangle tested at once, an internal child is pushed (so child 1's subtree
// is explored before child 0's).  The reference tests a popped node's box
// against the current t; here both child boxes are tested when their parent
// is loaded (one 64-byte node fetch) and the entry distance rides on the
// stack, compared with t at pop time.  The bound-independent half of the test
// does not depend on t, so the set of boxes accepted, and with it the hit, is
// the reference's.
// clr_trace_closest_ordered visits the nearer child first and replays, in the
// reference's order, every ray whose answer could depend on the order
// (traverse.cuh): the same ids and distances, with far fewer nodes visited.
#include "common.cuh"
#include "traverse.cuh"

CLR_DEFINE_STATUS_READER(traverse)

namespace clr {

constexpr int kTraceThreads = 128;

// Ray-per-lane loops.  Each thread walks the rays r, r + P, r + 2P, ... (P =
// threads in the grid) one after the other, so a lane whose ray finishes
// early starts its next ray instead of idling while the warp's longest ray
// completes.  The grid is sized to fill the GPU once.  Rays are independent
// and each is traversed exactly as alone, so results do not depend on P.

struct ClosestState {
    Ray ray;
    float ix, iy, iz;
    float t;
    uint32_t best;
    float tr;         // fast search: the relaxed bound of t,
    float gbest, t2;  // the winner's leaf-box entry and the other candidates' smallest tt
    int sp;
    bool exact;  // searching in the reference's order
};

__device__ __forceinline__ void closest_begin(ClosestState& s, const float4* __restrict__ rays, uint32_t r,
                                              const float* __restrict__ root_box, uint32_t n,
                                              const float4* __restrict__ tris, uint2* stack, bool exact) {
    s.ray = load_ray(rays, r);
    s.ix = 1.0f / s.ray.dx;
    s.iy = 1.0f / s.ray.dy;
    s.iz = 1.0f / s.ray.dz;
    s.t = s.ray.tmax;
    s.tr = relaxed_bound(s.t, replay_scale(root_box));
    s.best = 0xFFFFFFFFu;
    s.gbest = -INFINITY;
    s.t2 = INFINITY;
    s.sp = 0;
    s.exact = exact || n < 2;  // one triangle: no order to depend on
    float entry;
    if (!box_test_fast(__ldg(root_box + 0), __ldg(root_box + 1), __ldg(root_box + 2), __ldg(root_box + 4),
                       __ldg(root_box + 5), __ldg(root_box + 6), s.ray, s.ix, s.iy, s.iz, entry))
        return;
    if (n == 1) {
        if (!(entry > s.t)) tri_hit(tris, 0, s.ray, s.t, s.best);
    } else if (n >= 2) {
        // the pop-time bound test applies the root's entry (both modes)
        stack[s.sp++] = make_uint2(__float_as_uint(__ldg(root_box + 3)), __float_as_uint(entry));
    }
}

// One pop of rayIntersection's loop (bvh_traversal.cl:191-208).
// Reference order (s.exact): children in the fixed order, internal ones
// pushed with their own entry distance, compared with t when popped.
// Fast search: nearer child first, boxes culled against the relaxed bound,
// every reached leaf tested with the bookkeeping of the replay decision
// (traverse.cuh).
__device__ __forceinline__ void closest_step(ClosestState& s, const float4* __restrict__ nodes,
                                             const float4* __restrict__ tris, uint2* stack, float S) {
    --s.sp;
    const uint32_t node = stack[s.sp].x;
    const float key = __uint_as_float(stack[s.sp].y);
    if (key > (s.exact ? s.t : s.tr)) return;  // the reference's bound test at pop
    const NodeBoxes nb = load_node(nodes, node);
    float e0, e1;
    const bool p0 = box_test_fast(nb.b0[0], nb.b0[1], nb.b0[2], nb.b0[3], nb.b0[4], nb.b0[5], s.ray, s.ix, s.iy, s.iz, e0);
    const bool p1 = box_test_fast(nb.b1[0], nb.b1[1], nb.b1[2], nb.b1[3], nb.b1[4], nb.b1[5], s.ray, s.ix, s.iy, s.iz, e1);
    // reference order: child 0 then child 1 (internal children pushed, so
    // child 1's subtree pops first).  Fast: far child handled first so the
    // near internal child is popped first; near leaf tested first.
    const bool swap = !s.exact && (e1 < e0);
    const bool both_internal = !(nb.ref0 & kLeafBit) && !(nb.ref1 & kLeafBit);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int c = s.exact ? k : (both_internal ? (swap ? k : 1 - k) : (swap ? 1 - k : k));
        const uint32_t ref = c ? nb.ref1 : nb.ref0;
        if (!(c ? p1 : p0)) continue;
        const float e = c ? e1 : e0;
        if (ref & kLeafBit) {
            if (s.exact) {
                if (!(e > s.t)) tri_hit(tris, ref & ~kLeafBit, s.ray, s.t, s.best);
                continue;
            }
            if (e > s.tr) continue;
            const uint32_t leaf = ref & ~kLeafBit;
            const float4 a = __ldg(tris + 3u * leaf), b = __ldg(tris + 3u * leaf + 1u), cc = __ldg(tris + 3u * leaf + 2u);
            float tt, b1, b2;
            if (!tri_eval(a, b, cc, s.ray, tt, b1, b2)) continue;
            if (tt < s.t || (tt == s.t && s.best == 0xFFFFFFFFu)) {
                if (s.best != 0xFFFFFFFFu) s.t2 = fminf(s.t2, s.t);
                s.t = tt;
                s.tr = relaxed_bound(tt, S);
                s.best = __float_as_uint(a.w);
                s.gbest = e;
            } else {
                s.t2 = fminf(s.t2, tt);
            }
        } else {
            if (s.sp < kStackSize) stack[s.sp++] = make_uint2(ref, __float_as_uint(e));
            else clr_raise(CLR_DEVERR_STACK);
        }
    }
}

// Rays searched again in the reference's order, summed over launches
// (clr_trace_replays).
static __device__ unsigned long long g_replays = 0;

// kFast: the nearer-first search with replay; otherwise the reference's order.
// Both give the reference's ids and distances.  With `order`, the r-th ray
// searched is rays[order[r]] (results go to its own index): rays sorted by
// origin share the tree's nodes within a warp.
template <bool kFast>
__global__ void __launch_bounds__(kTraceThreads) k_trace_closest(const float4* __restrict__ nodes,
                                                                 const float4* __restrict__ tris,
                                                                 const float* __restrict__ root_box, uint32_t n,
                                                                 const float4* __restrict__ rays, uint32_t nr,
                                                                 const uint32_t* __restrict__ order,
                                                                 uint32_t* __restrict__ hit_id,
                                                                 float* __restrict__ hit_t) {
    const uint32_t P = gridDim.x * blockDim.x;
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    const float S = replay_scale(root_box);
    uint2 stack[kStackSize];
    ClosestState s;
    uint32_t q = order ? __ldg(order + r) : r;
    closest_begin(s, rays, q, root_box, n, tris, stack, !kFast);
    unsigned int replays = 0;
    // a valid tree pops each internal node at most once per ray and search
    uint32_t guard = 0;
    for (;;) {
        if (s.sp > 0 && guard < n) {
            closest_step(s, nodes, tris, stack, S);
            ++guard;
            continue;
        }
        if (kFast && !s.exact && needs_replay(s.t, s.gbest, s.t2, S)) {
            ++replays;
            guard = 0;
            closest_begin(s, rays, q, root_box, n, tris, stack, true);
            continue;
        }
        hit_id[q] = s.best;
        hit_t[q] = s.t;
        r += P;
        if (r >= nr) break;
        guard = 0;
        q = order ? __ldg(order + r) : r;
        closest_begin(s, rays, q, root_box, n, tris, stack, !kFast);
    }
    if (kFast && replays) atomicAdd(&g_replays, (unsigned long long)replays);
}

// Any-hit: the bound stays at tmax, so the accepted set of boxes does not
// depend on the visiting order; the first accepted triangle ends the query.
// kNearFirst searches the nearer child of a node first: a blocker is met
// sooner when the rays of a warp are close together (origin order, 11 %
// faster), while for scattered rays the extra divergence costs about 2 %.
template <bool kNearFirst>
__global__ void __launch_bounds__(kTraceThreads) k_trace_shadow(const float4* __restrict__ nodes,
                                                                const float4* __restrict__ tris,
                                                                const float* __restrict__ root_box, uint32_t n,
                                                                const float4* __restrict__ rays, uint32_t nr,
                                                                const uint32_t* __restrict__ order,
                                                                uint8_t* __restrict__ occluded) {
    const uint32_t P = gridDim.x * blockDim.x;
    uint32_t stack[kStackSize];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nr; i += P) {
        const uint32_t r = order ? __ldg(order + i) : i;
        const Ray ray = load_ray(rays, r);
        const float ix = 1.0f / ray.dx, iy = 1.0f / ray.dy, iz = 1.0f / ray.dz;
        const float tmax = ray.tmax;
        bool occ = false;
        float entry;
        const bool root_ok = box_test_fast(__ldg(root_box + 0), __ldg(root_box + 1), __ldg(root_box + 2),
                                           __ldg(root_box + 4), __ldg(root_box + 5), __ldg(root_box + 6), ray, ix,
                                           iy, iz, entry) &&
                             !(entry > tmax);
        if (n == 1) {
            float t = tmax;
            uint32_t id;
            if (root_ok) occ = tri_hit(tris, 0, ray, t, id);
        } else if (n >= 2 && root_ok) {
            int sp = 0;
            stack[sp++] = __float_as_uint(__ldg(root_box + 3));
            for (uint32_t guard = 0; sp > 0 && !occ && guard < n; ++guard) {
                const uint32_t node = stack[--sp];
                const NodeBoxes nb = load_node(nodes, node);
                float e0, e1;
                const bool p0 = box_test_fast(nb.b0[0], nb.b0[1], nb.b0[2], nb.b0[3], nb.b0[4], nb.b0[5], ray, ix, iy,
                                              iz, e0) && !(e0 > tmax);
                const bool p1 = box_test_fast(nb.b1[0], nb.b1[1], nb.b1[2], nb.b1[3], nb.b1[4], nb.b1[5], ray, ix, iy,
                                              iz, e1) && !(e1 > tmax);
                const bool near1 = kNearFirst && e1 < e0;  // the nearer child is pushed last
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int c = near1 ? k : 1 - k;
                    const uint32_t ref = c ? nb.ref1 : nb.ref0;
                    const bool pass = c ? p1 : p0;
                    if (!pass || occ) continue;
                    if (ref & kLeafBit) {
                        float t = tmax;
                        uint32_t id;
                        if (tri_hit(tris, ref & ~kLeafBit, ray, t, id)) occ = true;
                    } else if (sp < kStackSize) {
                        stack[sp++] = ref;
                    } else {
                        clr_raise(CLR_DEVERR_STACK);
                    }
                }
            }
        }
        occluded[r] = occ ? 1 : 0;
    }
}

// Grid that fills every SM once for a ray-per-lane kernel.
template <typename K>
static unsigned int persistent_grid(K kernel, uint32_t nr) {
    const int sms = clr_sm_count();
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceThreads, 0) != cudaSuccess || per_sm <= 0)
        per_sm = 1;
    const unsigned int full = (unsigned int)(sms * per_sm);
    const unsigned int need = div_up(nr, kTraceThreads);
    return need < full ? need : full;
}

}  // namespace clr

using namespace clr;

static int check_trace_args(const clr_bvh* bvh, const float* rays, uint32_t num_rays, const void* out0) {
    if (!bvh) return clr_set_error(CLR_EINVAL, "trace: bvh is NULL");
    if (num_rays == 0) return CLR_OK;
    if (!rays || !out0) return clr_set_error(CLR_EINVAL, "trace: NULL rays or output");
    if (reinterpret_cast<uintptr_t>(rays) & 15u) return clr_set_error(CLR_EINVAL, "trace: rays must be 16-byte aligned");
    if (bvh->num_tris > 0 && (!bvh->tris || !bvh->root_box || (bvh->num_tris > 1 && !bvh->nodes)))
        return clr_set_error(CLR_EINVAL, "trace: bvh buffers are NULL");
    return CLR_OK;
}

template <bool kFast>
static int trace_closest(const clr_bvh* bvh, const float* rays, uint32_t num_rays, const uint32_t* order,
                         uint32_t* hit_id, float* hit_t, void* stream) {
    int rc = check_trace_args(bvh, rays, num_rays, hit_id);
    if (rc != CLR_OK || num_rays == 0) return rc;
    if (!hit_t) return clr_set_error(CLR_EINVAL, "clr_trace_closest: hit_t is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_trace_closest<kFast><<<persistent_grid(k_trace_closest<kFast>, num_rays), kTraceThreads, 0, st>>>(
        static_cast<const float4*>(bvh->nodes), static_cast<const float4*>(bvh->tris), bvh->root_box, bvh->num_tris,
        reinterpret_cast<const float4*>(rays), num_rays, order, hit_id, hit_t);
    CLR_LAUNCH_CHECK("k_trace_closest");
    return CLR_OK;
}

static int trace_shadow(const clr_bvh* bvh, const float* rays, uint32_t num_rays, const uint32_t* order,
                        uint8_t* occluded, void* stream) {
    int rc = check_trace_args(bvh, rays, num_rays, occluded);
    if (rc != CLR_OK || num_rays == 0) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // shadow segments are short (most end at the first accepted triangle):
    // one ray per thread with hardware block scheduling balances them best
    const unsigned int grid = div_up(num_rays, kTraceThreads);
    if (order)
        k_trace_shadow<true><<<grid, kTraceThreads, 0, st>>>(
            static_cast<const float4*>(bvh->nodes), static_cast<const float4*>(bvh->tris), bvh->root_box,
            bvh->num_tris, reinterpret_cast<const float4*>(rays), num_rays, order, occluded);
    else
        k_trace_shadow<false><<<grid, kTraceThreads, 0, st>>>(
            static_cast<const float4*>(bvh->nodes), static_cast<const float4*>(bvh->tris), bvh->root_box,
            bvh->num_tris, reinterpret_cast<const float4*>(rays), num_rays, nullptr, occluded);
    CLR_LAUNCH_CHECK("k_trace_shadow");
    return CLR_OK;
}

// The searches over a ray order (lbvh_build.cu sorts the rays).
int clr_trace_closest_in_order(const clr_bvh* bvh, const float* rays, uint32_t num_rays, const uint32_t* order,
                               uint32_t* hit_id, float* hit_t, void* stream) {
    return trace_closest<true>(bvh, rays, num_rays, order, hit_id, hit_t, stream);
}
int clr_trace_shadow_in_order(const clr_bvh* bvh, const float* rays, uint32_t num_rays, const uint32_t* order,
                              uint8_t* occluded, void* stream) {
    return trace_shadow(bvh, rays, num_rays, order, occluded, stream);
}

extern "C" int clr_trace_closest(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                 float* hit_t, void* stream) {
    return trace_closest<false>(bvh, rays, num_rays, nullptr, hit_id, hit_t, stream);
}

extern "C" int clr_trace_closest_ordered(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                         float* hit_t, void* stream) {
    return trace_closest<true>(bvh, rays, num_rays, nullptr, hit_id, hit_t, stream);
}

extern "C" int clr_trace_replays(uint64_t* count, int clear) {
    if (!count) return clr_set_error(CLR_EINVAL, "clr_trace_replays: NULL count");
    unsigned long long v = 0;
    CLR_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_replays, sizeof(v)));
    if (clear) {
        const unsigned long long z = 0;
        CLR_CUDA_TRY(cudaMemcpyToSymbol(g_replays, &z, sizeof(z)));
    }
    *count = v;
    return CLR_OK;
}

extern "C" int clr_trace_shadow(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint8_t* occluded,
                                void* stream) {
    return trace_shadow(bvh, rays, num_rays, nullptr, occluded, stream);
}
