// BVH traversal on sm_103a: closest-hit and shadow (any-hit) queries.
//
// The closest-hit kernel visits nodes in the reference's order
// (OpenCL/bvh_traversal.cl:182-215): pop a node, handle child 0 then child 1,
// a leaf child is box-tested and its triangle tested at once, an internal
// child is pushed (so child 1's subtree is explored before child 0's).
// The reference tests a popped node's box against the current t; here both
// child boxes are tested when their parent is loaded (one 64-byte node fetch)
// and the entry distance rides on the stack, compared with t at pop time.
// The bound-independent half of the test does not depend on t, so the set of
// boxes accepted, and with it the hit, is the reference's.
#include "common.cuh"
#include "traverse.cuh"

CLR_DEFINE_STATUS_READER(traverse)

namespace clr {

constexpr int kTraceThreads = 128;

__global__ void __launch_bounds__(kTraceThreads) k_trace_closest(const float4* __restrict__ nodes,
                                                                 const float4* __restrict__ tris,
                                                                 const float* __restrict__ root_box, uint32_t n,
                                                                 const float4* __restrict__ rays, uint32_t nr,
                                                                 uint32_t* __restrict__ hit_id,
                                                                 float* __restrict__ hit_t) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    const Ray ray = load_ray(rays, r);
    float t = ray.tmax;
    uint32_t best = 0xFFFFFFFFu;
    float entry;
    const bool root_ok = box_test(__ldg(root_box + 0), __ldg(root_box + 1), __ldg(root_box + 2), __ldg(root_box + 4),
                                  __ldg(root_box + 5), __ldg(root_box + 6), ray, entry) &&
                         !(entry > t);
    if (n == 1) {
        if (root_ok) tri_hit(tris, 0, ray, t, best);
    } else if (n >= 2 && root_ok) {
        uint2 stack[kStackSize];
        int sp = 0;
        stack[sp++] = make_uint2(0u, __float_as_uint(entry));
        // a valid tree visits each internal node at most once per ray
        for (uint32_t guard = 0; sp > 0 && guard < n; ++guard) {
            --sp;
            const uint32_t node = stack[sp].x;
            if (__uint_as_float(stack[sp].y) > t) continue;  // the reference's bound test at pop
            const NodeBoxes nb = load_node(nodes, node);
            float e0, e1;
            const bool p0 = box_test(nb.b0[0], nb.b0[1], nb.b0[2], nb.b0[3], nb.b0[4], nb.b0[5], ray, e0);
            const bool p1 = box_test(nb.b1[0], nb.b1[1], nb.b1[2], nb.b1[3], nb.b1[4], nb.b1[5], ray, e1);
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const uint32_t ref = s ? nb.ref1 : nb.ref0;
                const bool pass = s ? p1 : p0;
                const float e = s ? e1 : e0;
                if (ref & kLeafBit) {
                    if (pass && !(e > t)) tri_hit(tris, ref & ~kLeafBit, ray, t, best);
                } else if (pass) {
                    if (sp < kStackSize) stack[sp++] = make_uint2(ref, __float_as_uint(e));
                    else clr_raise(CLR_DEVERR_STACK);
                }
            }
        }
    }
    hit_id[r] = best;
    hit_t[r] = t;
}

// Any-hit: the bound stays at tmax, so the accepted set of boxes does not
// depend on the visiting order; the first accepted triangle ends the query.
__global__ void __launch_bounds__(kTraceThreads) k_trace_shadow(const float4* __restrict__ nodes,
                                                                const float4* __restrict__ tris,
                                                                const float* __restrict__ root_box, uint32_t n,
                                                                const float4* __restrict__ rays, uint32_t nr,
                                                                uint8_t* __restrict__ occluded) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    const Ray ray = load_ray(rays, r);
    const float tmax = ray.tmax;
    bool occ = false;
    float entry;
    const bool root_ok = box_test(__ldg(root_box + 0), __ldg(root_box + 1), __ldg(root_box + 2), __ldg(root_box + 4),
                                  __ldg(root_box + 5), __ldg(root_box + 6), ray, entry) &&
                         !(entry > tmax);
    if (n == 1) {
        float t = tmax;
        uint32_t id;
        if (root_ok) occ = tri_hit(tris, 0, ray, t, id);
    } else if (n >= 2 && root_ok) {
        uint32_t stack[kStackSize];
        int sp = 0;
        stack[sp++] = 0u;
        for (uint32_t guard = 0; sp > 0 && !occ && guard < n; ++guard) {
            const uint32_t node = stack[--sp];
            const NodeBoxes nb = load_node(nodes, node);
            float e0, e1;
            const bool p0 = box_test(nb.b0[0], nb.b0[1], nb.b0[2], nb.b0[3], nb.b0[4], nb.b0[5], ray, e0) && !(e0 > tmax);
            const bool p1 = box_test(nb.b1[0], nb.b1[1], nb.b1[2], nb.b1[3], nb.b1[4], nb.b1[5], ray, e1) && !(e1 > tmax);
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const uint32_t ref = s ? nb.ref1 : nb.ref0;
                const bool pass = s ? p1 : p0;
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

extern "C" int clr_trace_closest(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                 float* hit_t, void* stream) {
    int rc = check_trace_args(bvh, rays, num_rays, hit_id);
    if (rc != CLR_OK || num_rays == 0) return rc;
    if (!hit_t) return clr_set_error(CLR_EINVAL, "clr_trace_closest: hit_t is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_trace_closest<<<div_up(num_rays, kTraceThreads), kTraceThreads, 0, st>>>(
        static_cast<const float4*>(bvh->nodes), static_cast<const float4*>(bvh->tris), bvh->root_box, bvh->num_tris,
        reinterpret_cast<const float4*>(rays), num_rays, hit_id, hit_t);
    CLR_LAUNCH_CHECK("k_trace_closest");
    return CLR_OK;
}

extern "C" int clr_trace_shadow(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint8_t* occluded,
                                void* stream) {
    int rc = check_trace_args(bvh, rays, num_rays, occluded);
    if (rc != CLR_OK || num_rays == 0) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_trace_shadow<<<div_up(num_rays, kTraceThreads), kTraceThreads, 0, st>>>(
        static_cast<const float4*>(bvh->nodes), static_cast<const float4*>(bvh->tris), bvh->root_box, bvh->num_tris,
        reinterpret_cast<const float4*>(rays), num_rays, occluded);
    CLR_LAUNCH_CHECK("k_trace_shadow");
    return CLR_OK;
}
