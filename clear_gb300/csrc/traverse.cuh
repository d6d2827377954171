// Device-side ray/box and ray/triangle tests and node access, shared by the
// traversal kernels and the path tracer.  Every float operation is rounded
// separately (common.cuh), matching the reference's expressions.
#pragma once

#include "common.cuh"

namespace clr {

// Depth bound of the radix tree plus one (3b + 32 levels for b <= 21).
constexpr int kStackSize = 96;

struct Ray {
    float ox, oy, oz, tmax;
    float dx, dy, dz;
};

__device__ __forceinline__ Ray load_ray(const float4* rays, uint32_t r) {
    const float4 a = __ldg(rays + 2u * r), b = __ldg(rays + 2u * r + 1u);
    return Ray{a.x, a.y, a.z, a.w, b.x, b.y, b.z};
}

// rayAABBIntersection (OpenCL/bvh_traversal.cl:160-179), Woo's outside-plane
// test.  Returns the part of the test that does not depend on the bound;
// `entry` receives the entry distance maxt (-inf when the origin is inside),
// and the full test is  result && !(entry > tBound).
__device__ __forceinline__ bool box_test(float mnx, float mny, float mnz, float mxx, float mxy, float mxz,
                                         const Ray& r, float& entry) {
    const bool lx = r.ox < mnx, ux = r.ox > mxx;
    const bool ly = r.oy < mny, uy = r.oy > mxy;
    const bool lz = r.oz < mnz, uz = r.oz > mxz;
    if (!(lx | ux | ly | uy | lz | uz)) {
        entry = -INFINITY;
        return true;
    }
    const float cx = lx ? mnx : (ux ? mxx : 0.0f);
    const float cy = ly ? mny : (uy ? mxy : 0.0f);
    const float cz = lz ? mnz : (uz ? mxz : 0.0f);
    const float tx = ((lx | ux) && r.dx != 0.0f) ? fdiv(fsub(cx, r.ox), r.dx) : -1.0f;
    const float ty = ((ly | uy) && r.dy != 0.0f) ? fdiv(fsub(cy, r.oy), r.dy) : -1.0f;
    const float tz = ((lz | uz) && r.dz != 0.0f) ? fdiv(fsub(cz, r.oz), r.dz) : -1.0f;
    const float maxt = fmaxf(tx, fmaxf(ty, tz));
    entry = maxt;
    if (maxt < 0.0f) return false;
    const float qx = fadd(r.ox, fmul(maxt, r.dx));
    const float qy = fadd(r.oy, fmul(maxt, r.dy));
    const float qz = fadd(r.oz, fmul(maxt, r.dz));
    const bool hx = (qx >= mnx && qx <= mxx) || tx == maxt;
    const bool hy = (qy >= mny && qy <= mxy) || ty == maxt;
    const bool hz = (qz >= mnz && qz <= mxz) || tz == maxt;
    return hx && hy && hz;
}

// Same result as box_test, with fewer IEEE divisions: t = (plane - o) / d is
// first estimated with the ray's reciprocal direction; only axes whose
// estimate lies within 2^-20 (relative) of the largest estimate can hold the
// maximum, and only those are divided exactly.  An estimate is within a few
// ulp of the exact quotient, so every other axis is strictly below the exact
// maximum: its exact value would neither win the max nor satisfy t == maxt.
__device__ __forceinline__ bool box_test_fast(float mnx, float mny, float mnz, float mxx, float mxy, float mxz,
                                              const Ray& r, float ix, float iy, float iz, float& entry) {
    const bool lx = r.ox < mnx, ux = r.ox > mxx;
    const bool ly = r.oy < mny, uy = r.oy > mxy;
    const bool lz = r.oz < mnz, uz = r.oz > mxz;
    if (!(lx | ux | ly | uy | lz | uz)) {
        entry = -INFINITY;
        return true;
    }
    const float cx = lx ? mnx : (ux ? mxx : 0.0f);
    const float cy = ly ? mny : (uy ? mxy : 0.0f);
    const float cz = lz ? mnz : (uz ? mxz : 0.0f);
    const bool ax = (lx | ux) && r.dx != 0.0f;
    const bool ay = (ly | uy) && r.dy != 0.0f;
    const bool az = (lz | uz) && r.dz != 0.0f;
    float tx = ax ? (cx - r.ox) * ix : -1.0f;
    float ty = ay ? (cy - r.oy) * iy : -1.0f;
    float tz = az ? (cz - r.oz) * iz : -1.0f;
    const float m = fmaxf(tx, fmaxf(ty, tz));
    if (m < 0.0f) {  // every quotient is negative (signs are exact)
        entry = m;
        return false;
    }
    const float thr = (m < 3.0e38f) ? m - fabsf(m) * 0x1p-20f - 1e-30f : -INFINITY;
    if (ax && tx >= thr) tx = fdiv(fsub(cx, r.ox), r.dx);
    if (ay && ty >= thr) ty = fdiv(fsub(cy, r.oy), r.dy);
    if (az && tz >= thr) tz = fdiv(fsub(cz, r.oz), r.dz);
    const float maxt = fmaxf(tx, fmaxf(ty, tz));
    entry = maxt;
    if (maxt < 0.0f) return false;
    const float qx = fadd(r.ox, fmul(maxt, r.dx));
    const float qy = fadd(r.oy, fmul(maxt, r.dy));
    const float qz = fadd(r.oz, fmul(maxt, r.dz));
    const bool hx = (qx >= mnx && qx <= mxx) || tx == maxt;
    const bool hy = (qy >= mny && qy <= mxy) || ty == maxt;
    const bool hz = (qz >= mnz && qz <= mxz) || tz == maxt;
    return hx && hy && hz;
}

// rayTriangleIntersection (OpenCL/bvh_traversal.cl:54-108), Moller-Trumbore
// with |det| < 1e-6 rejected: whether the ray meets the triangle at some
// tt >= 0, and tt with its barycentrics, before any comparison with the
// current bound.  Record = {p0, id}, {p1-p0}, {p2-p0}.
__device__ __forceinline__ bool tri_eval(const float4 a, const float4 e1, const float4 e2, const Ray& r, float& tt,
                                         float& b1, float& b2) {
    const float px = fsub(fmul(r.dy, e2.z), fmul(r.dz, e2.y));
    const float py = fsub(fmul(r.dz, e2.x), fmul(r.dx, e2.z));
    const float pz = fsub(fmul(r.dx, e2.y), fmul(r.dy, e2.x));
    const float det = dot3(e1.x, e1.y, e1.z, px, py, pz);
    if (det > -0.000001f && det < 0.000001f) return false;
    const float invDet = fdiv(1.0f, det);
    const float dx = fsub(r.ox, a.x), dy = fsub(r.oy, a.y), dz = fsub(r.oz, a.z);
    b1 = fmul(dot3(dx, dy, dz, px, py, pz), invDet);
    if (b1 < 0.0f || b1 > 1.0f) return false;
    const float qx = fsub(fmul(dy, e1.z), fmul(dz, e1.y));
    const float qy = fsub(fmul(dz, e1.x), fmul(dx, e1.z));
    const float qz = fsub(fmul(dx, e1.y), fmul(dy, e1.x));
    b2 = fmul(dot3(r.dx, r.dy, r.dz, qx, qy, qz), invDet);
    if (b2 < 0.0f || fadd(b1, b2) > 1.0f) return false;
    tt = fmul(dot3(e2.x, e2.y, e2.z, qx, qy, qz), invDet);
    return !(tt < 0.0f);
}

// The reference's test against the current bound t: a hit at tt > t is
// rejected (so an equal-t hit tested later wins), an accepted one moves t.
__device__ __forceinline__ bool tri_test(const float4 a, const float4 e1, const float4 e2, const Ray& r, float& t,
                                         float* b1_out = nullptr, float* b2_out = nullptr) {
    float tt, b1, b2;
    if (!tri_eval(a, e1, e2, r, tt, b1, b2) || tt > t) return false;
    t = tt;
    if (b1_out) *b1_out = b1;
    if (b2_out) *b2_out = b2;
    return true;
}

__device__ __forceinline__ bool tri_hit(const float4* __restrict__ tris, uint32_t leaf, const Ray& r, float& t,
                                        uint32_t& id) {
    const float4 a = __ldg(tris + 3u * leaf), b = __ldg(tris + 3u * leaf + 1u), c = __ldg(tris + 3u * leaf + 2u);
    if (tri_test(a, b, c, r, t)) {
        id = __float_as_uint(a.w);
        return true;
    }
    return false;
}

struct NodeBoxes {
    float b0[6], b1[6];
    uint32_t ref0, ref1;
};

__device__ __forceinline__ NodeBoxes load_node(const float4* __restrict__ nodes, uint32_t i) {
    const float4 a = __ldg(nodes + 4u * i), b = __ldg(nodes + 4u * i + 1u), c = __ldg(nodes + 4u * i + 2u),
                 d = __ldg(nodes + 4u * i + 3u);
    NodeBoxes nb;
    nb.b0[0] = a.x; nb.b0[1] = a.y; nb.b0[2] = a.z; nb.b0[3] = a.w; nb.b0[4] = b.x; nb.b0[5] = b.y;
    nb.b1[0] = b.z; nb.b1[1] = b.w; nb.b1[2] = c.x; nb.b1[3] = c.y; nb.b1[4] = c.z; nb.b1[5] = c.w;
    nb.ref0 = __float_as_uint(d.x);
    nb.ref1 = __float_as_uint(d.y);
    return nb;
}

// ---------------------------------------------- nearer-first with replay
//
// The reference's closest-hit search (bvh_traversal.cl:182-215) visits the
// children of a node in a fixed order and keeps the LAST triangle accepted at
// the smallest t; which triangle that is, on ties and near-ties, depends on the
// visiting order.  The fast search visits the nearer child first and decides,
// per ray, whether its answer is necessarily the reference's; if not, the ray
// is searched again in the reference's order (a "replay").
//
// Notation for one ray: a candidate is a triangle whose Moller-Trumbore test
// passes with tt >= 0 and whose boxes, leaf box and ancestors, pass the part
// of Woo's test that does not depend on the bound; G(j) is the largest entry
// distance over candidate j's boxes.  Exact arithmetic gives G(j) <= tt(j);
// with rounding G(j) can exceed tt(j) by a few ulp ("inversion").
//
// The fast search culls a box when its entry distance exceeds the relaxed
// bound t + kReplayDelta (|t| + S) (S: the scene box's largest extent / 16),
// tests every leaf it reaches, and records
//   T, B      the smallest tt and the triangle that first reached it,
//   G(B)      the largest entry distance over B's boxes, which is its leaf
//             box's: an ancestor's entry that is >= 0 comes from an axis on
//             which the origin lies outside the ancestor's slab, hence outside
//             the leaf's slab on the same side with the leaf's plane no nearer,
//             and (plane - o) / d is monotone in the plane under rounding,
//   t2        the smallest tt of every other candidate it tested.
// With V = max(T, G(B)), the answer (T, B) is final unless
//   t2 <= V                                   (a tie or near-tie), or
//   G(B) > T + kReplayDelta / 4 (|T| + S)     (B's own boxes lie well past it).
// Proof sketch, assuming no inversion exceeds kReplayDelta / 4 (|tt| + S):
// every other candidate then has tt > V.  Tested ones by t2 > V.  A culled
// one lies under a box whose entry exceeded the relaxed bound of a t >= T, so
// its G > T + kReplayDelta (|T| + S) >= V + kReplayDelta / 4 (|V| + S) (as
// G(B) is within kReplayDelta / 4 (|T| + S) of T), and its tt > V by the
// inversion bound.  In the reference's search, before B is tested t holds
// only tt values > V >= every entry on B's path, so B is reached and
// accepted, and no later candidate (tt > V >= T) is; the reference returns
// (T, B) with the same barycentrics.  Inversions measured on the
// random-triangle, terrain and Cornell scenes stay below 2^-21 relative; the
// bound assumed is 2^-14.
constexpr float kReplayDelta = 0x1p-12f;

__device__ __forceinline__ float replay_scale(const float* root_box) {
    const float ex = __ldg(root_box + 4) - __ldg(root_box + 0), ey = __ldg(root_box + 5) - __ldg(root_box + 1),
                ez = __ldg(root_box + 6) - __ldg(root_box + 2);
    const float m = fmaxf(ex, fmaxf(ey, ez));
    return (m < INFINITY) ? m * 0.0625f : 0.0f;
}

__device__ __forceinline__ float relaxed_bound(float t, float S) { return t + kReplayDelta * (fabsf(t) + S); }

__device__ __forceinline__ bool needs_replay(float t, float gbest, float t2, float S) {
    const float V = fmaxf(t, gbest);
    return (t2 < INFINITY && t2 <= V) || (gbest > t + 0.25f * kReplayDelta * (fabsf(t) + S));
}

}  // namespace clr
