// Scene access, hit records, BSDF/EDF construction, light sampling and the
// camera of the path tracer, shared by the megakernel (render.cu) and the
// wavefront form (render_wf.cu).  Reads the reference's scene blobs.
#pragma once

#include "common.cuh"
#include "shading.cuh"
#include "traverse.cuh"

namespace clr {

constexpr float kEpsilon = 0.00001f;  // global.cl:28
constexpr uint16_t kNone16 = 0xFFFF;
constexpr uint32_t kNone32 = 0xFFFFFFFFu;

struct DScene {
    const float4* vertices;
    const float4* normals;
    const float4* tangents;
    const float2* uvs;
    const uint8_t* faces;
    const uint8_t* lights;
    const uint8_t* materials;
    const uint8_t* textures;
    const uint8_t* others;
    const float4* nodes;
    const float4* tris;
    const float* root_box;
    uint32_t num_tris;
    bool alpha;  // CLR_SCENE_ALPHA: cutout test on closest hits
};

struct Face {
    uint32_t p[3], vn[3], vt[3], uv[3];
    uint32_t alphaTex;
    uint16_t mat, light;
};

__device__ __forceinline__ Face load_face(const DScene& sc, uint32_t id) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(sc.faces + 56u * id);
    Face f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f.p[k] = w[k];
        f.vn[k] = w[3 + k];
        f.vt[k] = w[6 + k];
        f.uv[k] = w[9 + k];
    }
    f.alphaTex = w[12];
    f.mat = (uint16_t)(w[13] & 0xFFFFu);
    f.light = (uint16_t)(w[13] >> 16);
    return f;
}

__device__ __forceinline__ f3 vtx(const float4* a, uint32_t i) {
    const float4 v = __ldg(a + i);
    return mk(v.x, v.y, v.z);
}

// ------------------------------------------------------------- traversal

struct Hit {
    uint32_t id;
    float t, b1, b2;
};

// evaluateAlphaTexture (texture.cl:124-148): the alpha byte of an RGBA8
// image, a Gray8 image's value, a procedural float texture; 1 otherwise.
// Only "reads 0" matters, and k / 255 is 0 only for k = 0.
static __device__ __noinline__ bool alpha_is_zero(const uint8_t* t, float2 uv) {
    uint32_t x, y;
    const uint8_t* d;
    switch (t[0]) {
        case kTexRGBA8:
            image_xy(t, uv, x, y, d);
            return d[4u * (y * ldb<uint32_t>(t + 4) + x) + 3u] == 0;
        case kTexGray8:
            image_xy(t, uv, x, y, d);
            return d[y * ldb<uint32_t>(t + 4) + x] == 0;
        case kTexFloatProc:
            return eval_float_texture(t, uv) == 0.0f;
        default:
            return false;
    }
}

// rayTriangleIntersection's cutout test (bvh_traversal.cl:94-105) for an
// accepted hit on face `id` at barycentrics (b1, b2): the face has uvs
// (uv0 set) and an alpha texture that reads 0 at the interpolated uv.
static __device__ __noinline__ bool alpha_cutout(const DScene& sc, uint32_t id, float b1, float b2) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(sc.faces + 56u * id);
    const uint32_t tex = __ldg(w + 12), t0 = __ldg(w + 9);
    if (tex == kNone32 || t0 == kNone32) return false;
    const float b0 = 1.0f - b1 - b2;
    const float2 uv0 = __ldg(sc.uvs + t0), uv1 = __ldg(sc.uvs + __ldg(w + 10)), uv2 = __ldg(sc.uvs + __ldg(w + 11));
    const float2 uv = make_float2(b0 * uv0.x + b1 * uv1.x + b2 * uv2.x, b0 * uv0.y + b1 * uv1.y + b2 * uv2.y);
    return alpha_is_zero(sc.textures + tex, uv);
}

// rayIntersection for the renderer: returns the closest hit with its
// barycentrics.  kOrdered visits the nearer child first.
// Closest hit.  With kCount, boxes[0] counts the internal boxes and boxes[1]
// the leaf boxes the search accepts (their sum is the reference's numAABBHit
// of rayIntersectionVis, bvh_traversal.cl:217-254, in its visiting order when
// !kOrdered): the nodes loaded and the triangles tested.
// Kernels that trace from several call sites may define
// CLR_TRAVERSAL_OUTLINED before including this header to keep one copy of
// each search instead of one inlined copy per site.
#ifdef CLR_TRAVERSAL_OUTLINED
#define CLR_TRAVERSAL_ATTR __noinline__
#else
#define CLR_TRAVERSAL_ATTR
#endif

// The record returned is the last hit recorded, at its own distance; with
// kAlpha (scenes with CLR_SCENE_ALPHA) a cutout moves the bound without being
// recorded (see alpha_cutout).  Whether the bound ended finite is the
// reference's "hit" for shadow rays.
// kOrdered runs the nearer-first search and replays the ray in the
// reference's order when its answer could depend on the order (traverse.cuh),
// so both forms return the reference's record.  Scenes with cutouts are always
// searched in the reference's order: a cutout moves the bound without a
// record, which makes the record depend on the order in ways the replay test
// does not cover.
// What a search leaves: its final bound and the leaf (sorted position) of the
// triangle it recorded.  The record's distance and barycentrics are computed
// again from that leaf afterwards (the same arithmetic gives the same values),
// which keeps them out of the registers the search loop holds.
struct SearchResult {
    float t;
    uint32_t leaf;
};

// The reference's order (bvh_traversal.cl:191-208).
template <bool kCount, bool kAlpha>
static __device__ __forceinline__ SearchResult search_reference_order(const DScene& sc, const Ray& ray, float ix,
                                                                     float iy, float iz, float root_entry,
                                                                     uint2* stack, uint32_t* boxes) {
    float t = INFINITY;
    uint32_t best = kNone32;
    int sp = 0;
    stack[sp++] = make_uint2(__float_as_uint(sc.root_box[3]), __float_as_uint(root_entry));
    for (uint32_t guard = 0; sp > 0 && guard < sc.num_tris; ++guard) {
        --sp;
        if (__uint_as_float(stack[sp].y) > t) continue;
        if (kCount) ++boxes[0];
        const NodeBoxes nb = load_node(sc.nodes, stack[sp].x);
        float e0, e1;
        const bool p0 = box_test_fast(nb.b0[0], nb.b0[1], nb.b0[2], nb.b0[3], nb.b0[4], nb.b0[5], ray, ix, iy, iz, e0);
        const bool p1 = box_test_fast(nb.b1[0], nb.b1[1], nb.b1[2], nb.b1[3], nb.b1[4], nb.b1[5], ray, ix, iy, iz, e1);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const uint32_t ref = c ? nb.ref1 : nb.ref0;
            if (!(c ? p1 : p0)) continue;
            const float e = c ? e1 : e0;
            if (ref & kLeafBit) {
                if (e > t) continue;
                if (kCount) ++boxes[1];
                const uint32_t leaf = ref & ~kLeafBit;
                const float4 a = __ldg(sc.tris + 3u * leaf);
                float b1, b2;
                if (tri_test(a, __ldg(sc.tris + 3u * leaf + 1u), __ldg(sc.tris + 3u * leaf + 2u), ray, t, &b1, &b2)) {
                    if (kAlpha && alpha_cutout(sc, __float_as_uint(a.w), b1, b2)) continue;
                    best = leaf;
                }
            } else if (sp < kStackSize) {
                stack[sp++] = make_uint2(ref, __float_as_uint(e));
            } else {
                clr_raise(CLR_DEVERR_STACK);
            }
        }
    }
    return SearchResult{t, best};
}

// The nearer-first search with the bookkeeping of the replay decision
// (traverse.cuh); sets `replay` when the ray must be searched again in the
// reference's order.  Not for scenes with cutouts.
template <bool kCount>
static __device__ __forceinline__ SearchResult search_nearer_first(const DScene& sc, const Ray& ray, float ix,
                                                                   float iy, float iz, float root_entry,
                                                                   uint2* stack, uint32_t* boxes, bool& replay) {
    float t = INFINITY, tr = INFINITY;  // the bound and its relaxed form
    uint32_t best = kNone32;
    float gbest = -INFINITY, t2 = INFINITY;
    int sp = 0;
    stack[sp++] = make_uint2(__float_as_uint(sc.root_box[3]), __float_as_uint(root_entry));
    for (uint32_t guard = 0; sp > 0 && guard < sc.num_tris; ++guard) {
        --sp;
        if (__uint_as_float(stack[sp].y) > tr) continue;
        if (kCount) ++boxes[0];
        const NodeBoxes nb = load_node(sc.nodes, stack[sp].x);
        float e0, e1;
        const bool p0 = box_test_fast(nb.b0[0], nb.b0[1], nb.b0[2], nb.b0[3], nb.b0[4], nb.b0[5], ray, ix, iy, iz, e0);
        const bool p1 = box_test_fast(nb.b1[0], nb.b1[1], nb.b1[2], nb.b1[3], nb.b1[4], nb.b1[5], ray, ix, iy, iz, e1);
        const bool both_internal = !(nb.ref0 & kLeafBit) && !(nb.ref1 & kLeafBit);
        const bool swap = e1 < e0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            // leaves: near first; internal: far pushed first
            const int c = both_internal ? (swap ? k : 1 - k) : (swap ? 1 - k : k);
            const uint32_t ref = c ? nb.ref1 : nb.ref0;
            if (!(c ? p1 : p0)) continue;
            const float e = c ? e1 : e0;
            if (ref & kLeafBit) {
                if (e > tr) continue;
                if (kCount) ++boxes[1];
                const uint32_t leaf = ref & ~kLeafBit;
                float tt, b1, b2;
                if (!tri_eval(__ldg(sc.tris + 3u * leaf), __ldg(sc.tris + 3u * leaf + 1u),
                              __ldg(sc.tris + 3u * leaf + 2u), ray, tt, b1, b2))
                    continue;
                if (tt < t || (tt == t && best == kNone32)) {
                    if (best != kNone32) t2 = fminf(t2, t);
                    t = tt;
                    tr = relaxed_bound(tt, replay_scale(sc.root_box));
                    best = leaf;
                    gbest = e;
                } else {
                    t2 = fminf(t2, tt);
                }
            } else if (sp < kStackSize) {
                stack[sp++] = make_uint2(ref, __float_as_uint(e));
            } else {
                clr_raise(CLR_DEVERR_STACK);
            }
        }
    }
    replay = needs_replay(t, gbest, t2, replay_scale(sc.root_box));
    return SearchResult{t, best};
}

// The record returned is the last hit recorded, at its own distance; with
// kAlpha (scenes with CLR_SCENE_ALPHA) a cutout moves the bound without being
// recorded (see alpha_cutout).  Whether the bound ended finite is the
// reference's "hit" for shadow rays.
// kOrdered runs the nearer-first search and replays the ray in the
// reference's order when its answer could depend on the order (traverse.cuh),
// so both forms return the reference's record.  Scenes with cutouts are always
// searched in the reference's order: a cutout moves the bound without a
// record, which makes the record depend on the order in ways the replay test
// does not cover.
template <bool kOrdered, bool kCount, bool kAlpha>
static __device__ CLR_TRAVERSAL_ATTR uint32_t intersect_search(const DScene& sc, f3 org, f3 dir, Hit& h, uint2* stack,
                                                               uint32_t* boxes) {
    const Ray ray{org.x, org.y, org.z, INFINITY, dir.x, dir.y, dir.z};
    const float ix = 1.0f / dir.x, iy = 1.0f / dir.y, iz = 1.0f / dir.z;
    float entry;
    const float* rb = sc.root_box;
    if (!box_test_fast(rb[0], rb[1], rb[2], rb[4], rb[5], rb[6], ray, ix, iy, iz, entry)) return 0u;
    SearchResult r{INFINITY, kNone32};
    if (sc.num_tris == 1) {  // the root box is the leaf's box
        if (kCount) ++boxes[1];
        float b1, b2;
        const float4 a = __ldg(sc.tris);
        if (tri_test(a, __ldg(sc.tris + 1u), __ldg(sc.tris + 2u), ray, r.t, &b1, &b2) &&
            !(kAlpha && alpha_cutout(sc, __float_as_uint(a.w), b1, b2)))
            r.leaf = 0;
    } else if (sc.num_tris >= 2) {
        bool replay = true;
        if (kOrdered && !kAlpha) r = search_nearer_first<kCount>(sc, ray, ix, iy, iz, entry, stack, boxes, replay);
        if (replay) r = search_reference_order<kCount, kAlpha>(sc, ray, ix, iy, iz, entry, stack, boxes);
    }
    const uint32_t bound = r.t < INFINITY ? 2u : 0u;
    h.id = kNone32;
    if (r.leaf == kNone32) return bound;
    const float4 a = __ldg(sc.tris + 3u * r.leaf);
    tri_eval(a, __ldg(sc.tris + 3u * r.leaf + 1u), __ldg(sc.tris + 3u * r.leaf + 2u), ray, h.t, h.b1, h.b2);
    h.id = __float_as_uint(a.w);
    return bound | 1u;
}

// The search with the cutout test compiled in only for scenes that need it:
// bit 0 set when a hit is recorded, bit 1 when the bound ended finite.
// kAlpha 0 or 1 fixes the choice at compile time (a kernel instantiated per
// scene kind); -1 reads the scene's flag at the call.
template <bool kOrdered, bool kCount = false, int kAlpha = -1>
static __device__ __forceinline__ uint32_t intersect_status(const DScene& sc, f3 org, f3 dir, Hit& h, uint2* stack,
                                                            uint32_t* boxes) {
    if (kAlpha >= 0) return intersect_search<kOrdered, kCount, (kAlpha > 0)>(sc, org, dir, h, stack, boxes);
    return sc.alpha ? intersect_search<kOrdered, kCount, true>(sc, org, dir, h, stack, boxes)
                    : intersect_search<kOrdered, kCount, false>(sc, org, dir, h, stack, boxes);
}

template <bool kOrdered, bool kCount = false, int kAlpha = -1>
static __device__ __forceinline__ bool intersect_impl(const DScene& sc, f3 org, f3 dir, Hit& h, uint2* stack,
                                                      uint32_t* boxes) {
    return (intersect_status<kOrdered, kCount, kAlpha>(sc, org, dir, h, stack, boxes) & 1u) != 0;
}

template <bool kOrdered>
static __device__ __forceinline__ bool intersect(const DScene& sc, f3 org, f3 dir, Hit& h, uint2* stack) {
    return intersect_impl<kOrdered, false>(sc, org, dir, h, stack, nullptr);
}

// Whether the ray hits any triangle at all (environment shadow rays of paths
// that have no light face yet: the reference's test "closest hit exists"
// has the same answer, since any triangle the closest-hit search would
// accept is also reachable with the bound held at infinity, and vice versa).
// With kCount, boxes[0] counts the nodes loaded and boxes[1] the triangles
// tested, as in intersect_impl.
template <bool kOrdered, bool kCount = false>
__device__ CLR_TRAVERSAL_ATTR bool occluded_any(const DScene& sc, f3 org, f3 dir, uint2* stack, uint32_t* boxes = nullptr) {
    Ray ray{org.x, org.y, org.z, INFINITY, dir.x, dir.y, dir.z};
    const float ix = 1.0f / dir.x, iy = 1.0f / dir.y, iz = 1.0f / dir.z;
    float entry;
    const float* rb = sc.root_box;
    if (!box_test_fast(rb[0], rb[1], rb[2], rb[4], rb[5], rb[6], ray, ix, iy, iz, entry)) return false;
    auto hit_leaf = [&](uint32_t leaf) {
        if (kCount) ++boxes[1];
        float t = INFINITY;
        return tri_test(__ldg(sc.tris + 3u * leaf), __ldg(sc.tris + 3u * leaf + 1u), __ldg(sc.tris + 3u * leaf + 2u),
                        ray, t);
    };
    if (sc.num_tris == 1) return hit_leaf(0);
    if (sc.num_tris < 2) return false;
    int sp = 0;
    stack[sp++] = make_uint2(__float_as_uint(rb[3]), 0u);
    for (uint32_t guard = 0; sp > 0 && guard < sc.num_tris; ++guard) {
        if (kCount) ++boxes[0];
        const NodeBoxes nb = load_node(sc.nodes, stack[--sp].x);
        float e0, e1;
        const bool p0 = box_test_fast(nb.b0[0], nb.b0[1], nb.b0[2], nb.b0[3], nb.b0[4], nb.b0[5], ray, ix, iy, iz, e0);
        const bool p1 = box_test_fast(nb.b1[0], nb.b1[1], nb.b1[2], nb.b1[3], nb.b1[4], nb.b1[5], ray, ix, iy, iz, e1);
        // nearer child last on the stack so it is explored first
        const bool near1 = kOrdered && (e1 < e0);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int c = near1 ? k : 1 - k;
            const uint32_t ref = c ? nb.ref1 : nb.ref0;
            if (!(c ? p1 : p0)) continue;
            if (ref & kLeafBit) {
                if (hit_leaf(ref & ~kLeafBit)) return true;
            } else if (sp < kStackSize) {
                stack[sp++] = make_uint2(ref, 0u);
            } else {
                clr_raise(CLR_DEVERR_STACK);
            }
        }
    }
    return false;
}

// rayTriangleIntersection's hit record + calcHitpointParameters
// (bvh_traversal.cl:87-100, 110-158).
__device__ __forceinline__ void surface_point(const DScene& sc, f3 org, f3 dir, const Hit& h, SurfPt& sp) {
    const Face f = load_face(sc, h.id);
    const f3 p0 = vtx(sc.vertices, f.p[0]), p1 = vtx(sc.vertices, f.p[1]), p2 = vtx(sc.vertices, f.p[2]);
    const f3 e1 = p1 - p0, e2 = p2 - p0;
    const float b1 = h.b1, b2 = h.b2;
    const float b0 = 1.0f - b1 - b2;
    sp.p = org + dir * h.t;
    sp.gNormal = normalize(cross(e1, e2));
    sp.faceID = h.id;
    const bool hasUV = f.uv[0] != kNone32;
    float2 uv0 = make_float2(0.f, 0.f), uv1 = uv0, uv2 = uv0;
    sp.uv = make_float2(0.f, 0.f);
    if (hasUV) {
        uv0 = __ldg(sc.uvs + f.uv[0]);
        uv1 = __ldg(sc.uvs + f.uv[1]);
        uv2 = __ldg(sc.uvs + f.uv[2]);
        sp.uv = make_float2(b0 * uv0.x + b1 * uv1.x + b2 * uv2.x, b0 * uv0.y + b1 * uv1.y + b2 * uv2.y);
    }
    // calcHitpointParameters recomputes b2 from (b0, b1)
    const float c0 = b0, c1 = b1, c2 = 1.0f - c0 - c1;
    const bool hasVN = f.vn[0] != kNone32;
    if (hasVN)
        sp.sNormal = normalize(c0 * vtx(sc.normals, f.vn[0]) + c1 * vtx(sc.normals, f.vn[1]) + c2 * vtx(sc.normals, f.vn[2]));
    else
        sp.sNormal = sp.gNormal;
    sp.hasTangent = f.vt[0] != kNone32;
    if (sp.hasTangent)
        sp.sTangent = normalize(c0 * vtx(sc.tangents, f.vt[0]) + c1 * vtx(sc.tangents, f.vt[1]) +
                                c2 * vtx(sc.tangents, f.vt[2]));
    else
        sp.sTangent = mk(0, 0, 0);
    sp.uDir = mk(0, 0, 0);
    if (hasUV) {
        const float du0 = uv0.x - uv2.x, dv0 = uv0.y - uv2.y, du1 = uv1.x - uv2.x, dv1 = uv1.y - uv2.y;
        const f3 dP0 = p0 - p2, dP1 = p1 - p2;
        const float invDetUV = 1.0f / (du0 * dv1 - dv0 * du1);
        const f3 uDir = invDetUV * mk(dv1 * dP0.x - dv0 * dP1.x, dv1 * dP0.y - dv0 * dP1.y, dv1 * dP0.z - dv0 * dP1.z);
        sp.uDir = hasVN ? normalize(cross(cross(sp.sNormal, uDir), sp.sNormal)) : normalize(uDir);
    }
}

// ------------------------------------------------------------------ BSDF

// BSDFAlloc, reflection.cl:185-342
__device__ __forceinline__ void bsdf_alloc(const DScene& sc, uint32_t offset, const SurfPt& sp, BSDF& f) {
    const uint8_t* m = sc.materials + offset;
    const bool hasBump = m[1] != 0;
    const uint32_t idx_bump = ldb<uint32_t>(m + 4);
    f.n = sp.sNormal;
    if (sp.hasTangent) f.s = sp.sTangent;
    else make_tangent(sp.sNormal, f.s);
    if (hasBump) {
        const f3 c = eval_color_texture(sc.textures + idx_bump, sp.uv);
        const f3 nBump = normalize(mk(2.0f * c.x - 1.0f, 2.0f * c.y - 1.0f, 2.0f * c.z - 1.0f));
        const f3 vDir = cross(sp.uDir, sp.sNormal);
        f.n = mk(dot(mk(sp.uDir.x, vDir.x, sp.sNormal.x), nBump), dot(mk(sp.uDir.y, vDir.y, sp.sNormal.y), nBump),
                 dot(mk(sp.uDir.z, vDir.z, sp.sNormal.z), nBump));
        f3 ax = cross(sp.sNormal, f.n);
        const float sinTH = fminf(length(ax), 1.0f);
        if (sinTH > 0.0001f) {
            ax = normalize(ax);
            const float cosTH = cosf(asinf(sinTH));
            const float om = 1 - cosTH;
            const f3 s = f.s;
            f.s = mk(dot(mk(ax.x * ax.x * om + cosTH, ax.x * ax.y * om - ax.z * sinTH, ax.z * ax.x * om + ax.y * sinTH), s),
                     dot(mk(ax.x * ax.y * om + ax.z * sinTH, ax.y * ax.y * om + cosTH, ax.y * ax.z * om - ax.x * sinTH), s),
                     dot(mk(ax.z * ax.x * om - ax.y * sinTH, ax.y * ax.z * om + ax.x * sinTH, ax.z * ax.z * om + cosTH), s));
        }
    }
    f.t = cross(f.n, f.s);
    f.ng = sp.gNormal;
    f.mat = m;
    f.tex = sc.textures;
    f.others = sc.others;
    f.uv = sp.uv;
    // component offsets (AlignPtrG(&matsData_p, 4) per element, reflection.cl:230-341)
    const int num = min((int)m[0], kMaxBxDFs);
    uint32_t off = 8;  // sizeof(MaterialInfo)
#pragma unroll
    for (int i = 0; i < kMaxBxDFs; ++i) {
        if (i < num) {
            off = (off + 3u) & ~3u;
            f.off[i] = (uint16_t)off;
            f.type[i] = elem_type(m[off]);
            off += elem_size(m[off]);
        } else {
            f.off[i] = 0;
            f.type[i] = 0;
        }
    }
    f.num = num;
    if (num == 0) {  // a material without components renders black
        f.num = 1;
        f.off[0] = 0xFFFF;
        f.type[0] = kTyReflection | kTyDiffuse;
    }
}

// ---------------------------------------------------------------- lights

struct LightPt {
    f3 p, gNormal, sNormal, sTangent, uDir;
    float2 uv;
    uint32_t faceID;
    bool hasTangent, atInfinity;
};

__device__ __forceinline__ const uint8_t* env_light_property(const DScene& sc) {
    const uint32_t env_off = ldb<uint32_t>(sc.others + 4);
    return sc.materials + ldb<uint32_t>(sc.others + env_off);
}

__device__ __forceinline__ const uint8_t* light_distribution(const DScene& sc) {
    return sc.others + ldb<uint32_t>(sc.others + 8);
}

// EDFAlloc, light.cl:295-379
__device__ __forceinline__ void edf_alloc(const DScene& sc, uint32_t offset, const LightPt& lp, EDF& e) {
    e.env = lp.atInfinity;
    e.tex = sc.textures;
    e.uv = lp.uv;
    e.prop = lp.atInfinity ? env_light_property(sc) : sc.materials + offset;
    if (!lp.atInfinity) {
        e.n = lp.sNormal;
        if (lp.hasTangent) e.s = lp.sTangent;
        else make_tangent(lp.sNormal, e.s);
        e.t = cross(e.n, e.s);
        e.ng = lp.gNormal;
    }
    // ImageBasedEnvLElem (16 B) / DiffuseLElem (8 B), 4-byte aligned after
    // the 1-byte LightPropertyInfo
    const int num = min((int)e.prop[0], kMaxBxDFs);
    const uint32_t size = lp.atInfinity ? 16u : 8u;
    uint32_t off = 1;
    int k = 0;
#pragma unroll
    for (int i = 0; i < kMaxBxDFs; ++i) {
        off = (off + 3u) & ~3u;
        const bool ok = i < num && e.prop[off] == 0;
        e.off[i] = (uint16_t)off;
        if (ok && k == i) {
            ++k;
            off += size;
        }
    }
    e.num = k;
}

__device__ __forceinline__ void light_from_surface(const SurfPt& s, LightPt& l) {
    l.p = s.p;
    l.gNormal = s.gNormal;
    l.sNormal = s.sNormal;
    l.sTangent = s.sTangent;
    l.uDir = s.uDir;
    l.uv = s.uv;
    l.faceID = s.faceID;
    l.hasTangent = s.hasTangent;
    l.atInfinity = false;
}

// sampleLightPos, light.cl:138-245; returns the light property offset.
__device__ __forceinline__ void sample_light(const DScene& sc, float uL, float u0, float u1, LightPt& lp, EDF& e, float& areaPDF) {
    const uint8_t* dist = light_distribution(sc);
    const uint32_t li = sample_discrete_1d(dist, uL, &areaPDF);
    const uint8_t atInf = sc.lights[8u * li];
    const uint32_t ref = ldb<uint32_t>(sc.lights + 8u * li + 4);
    uint32_t lightProp = kNone16;
    if (atInf) {
        lp.atInfinity = true;
        const uint8_t* l = env_light_property(sc);
        areaPDF *= 1.0f;
        const uint8_t* p = l + 1;
        for (int i = 0; i < (int)l[0]; ++i) {
            p = align_ptr(p, 4);
            if (p[0] != 0) break;
            if (i == 0) {  // whichIBL = 0
                float uvPDF;
                lp.uv = sample_cc_2d(sc.others + ldb<uint32_t>(p + 12), u0, u1, &uvPDF);
                const float theta = lp.uv.y * kPi, phi = lp.uv.x * 2 * kPi;
                const float sinTheta = sinf(theta);
                lp.p = mk(-sinf(phi) * sinTheta, cosf(theta), cosf(phi) * sinTheta);
                areaPDF *= uvPDF / (2 * kPi * kPi * sinTheta);
                continue;
            }
            p += 16;
        }
    } else {
        lp.atInfinity = false;
        lp.faceID = ref;
        const Face f = load_face(sc, ref);
        const f3 p0 = vtx(sc.vertices, f.p[0]), p1 = vtx(sc.vertices, f.p[1]), p2 = vtx(sc.vertices, f.p[2]);
        const float su1 = sqrtf(u0);
        const float b0 = 1.0f - su1, b1 = u1 * su1;
        const float b2 = 1.0f - b0 - b1;
        const f3 ng = cross(p1 - p0, p2 - p0);
        const float area = 0.5f * length(ng);
        areaPDF *= 1.0f / area;
        lp.p = b0 * p0 + b1 * p1 + b2 * p2;
        lp.gNormal = normalize(ng);
        const bool hasVN = f.vn[0] != kNone32 && f.vn[1] != kNone32 && f.vn[2] != kNone32;
        lp.sNormal = hasVN ? normalize(b0 * vtx(sc.normals, f.vn[0]) + b1 * vtx(sc.normals, f.vn[1]) +
                                       b2 * vtx(sc.normals, f.vn[2]))
                           : lp.gNormal;
        lp.hasTangent = f.vt[0] != kNone32 && f.vt[1] != kNone32 && f.vt[2] != kNone32;
        if (lp.hasTangent)
            lp.sTangent = normalize(b0 * vtx(sc.tangents, f.vt[0]) + b1 * vtx(sc.tangents, f.vt[1]) +
                                    b2 * vtx(sc.tangents, f.vt[2]));
        const bool hasUV = f.uv[0] != kNone32 && f.uv[1] != kNone32 && f.uv[2] != kNone32;
        if (hasUV) {
            const float2 uv0 = __ldg(sc.uvs + f.uv[0]), uv1 = __ldg(sc.uvs + f.uv[1]), uv2 = __ldg(sc.uvs + f.uv[2]);
            lp.uv = make_float2(b0 * uv0.x + b1 * uv1.x + b2 * uv2.x, b0 * uv0.y + b1 * uv1.y + b2 * uv2.y);
            const float du0 = uv0.x - uv2.x, dv0 = uv0.y - uv2.y, du1 = uv1.x - uv2.x, dv1 = uv1.y - uv2.y;
            const f3 dP0 = p0 - p2, dP1 = p1 - p2;
            const float invDetUV = 1.0f / (du0 * dv1 - dv0 * du1);
            const f3 uDir = invDetUV * mk(dv1 * dP0.x - dv0 * dP1.x, dv1 * dP0.y - dv0 * dP1.y, dv1 * dP0.z - dv0 * dP1.z);
            lp.uDir = hasVN ? normalize(cross(cross(lp.sNormal, uDir), lp.sNormal)) : normalize(uDir);
        }
        lightProp = f.light;
    }
    edf_alloc(sc, lightProp, lp, e);
}

// The shadow test of next-event estimation (pathtracer.cl:119-122):
// "closest hit face == lpos.faceID, or the light is at infinity and nothing
// is hit".  lpos is one variable for the whole path: sampling the
// environment leaves its faceID as the last area light the path sampled or
// hit (sampleLightPos and LightPointFromSurfacePoint are its only writers),
// so an environment shadow ray whose closest hit is that face also counts
// as unoccluded.  Paths start with faceID = kNone32, a value no face has
// (the reference leaves it unset).  After a miss the reference compares an
// unset hit record; a miss never matches here.
//
// Shadow entries carry the test as one word: an area light's face, or for
// the environment kEnvLightBit | the path's light face (kNone32 when there is
// none; face ids are below 2^30).
constexpr uint32_t kEnvLightBit = 0x80000000u;

__device__ __forceinline__ uint32_t shadow_light_word(const LightPt& lp) {
    return lp.atInfinity ? (kEnvLightBit | lp.faceID) : lp.faceID;
}

template <bool kOrdered, bool kCount = false, int kAlpha = -1>
__device__ __forceinline__ bool shadow_visible(const DScene& sc, f3 org, f3 dir, uint32_t light, uint2* stack,
                                               uint32_t* boxes = nullptr) {
    if (light == kNone32) return !occluded_any<kOrdered, kCount>(sc, org, dir, stack, boxes);
    Hit h;
    const uint32_t st = intersect_status<kOrdered, kCount, kAlpha>(sc, org, dir, h, stack, boxes);
    const bool rec = (st & 1u) != 0, bounded = (st & 2u) != 0;
    if (light & kEnvLightBit) return !bounded || (rec && h.id == (light & ~kEnvLightBit));
    return rec && h.id == light;
}

// getAreaPDF, light.cl:247-292
__device__ __forceinline__ float area_pdf(const DScene& sc, const LightPt& lp) {
    const uint8_t* dist = light_distribution(sc);
    const uint32_t numItems = ldb<uint32_t>(dist + 4);
    if (lp.atInfinity) {
        const uint8_t* l = env_light_property(sc);
        float a = 0.0f;
        const uint8_t* p = l + 1;
        for (int i = 0; i < (int)l[0]; ++i) {
            p = align_ptr(p, 4);
            if (p[0] != 0) break;
            const float uvPDF = pdf_cc_2d(sc.others + ldb<uint32_t>(p + 12), lp.uv);
            a += uvPDF / (2 * kPi * kPi * sinf(lp.uv.y * kPi)) * 1.0f;
            p += 16;
        }
        for (uint32_t i = 0; i < numItems; ++i)
            if (sc.lights[8u * i]) return a * prob_discrete_1d(dist, i);
    } else {
        const Face f = load_face(sc, lp.faceID);
        const f3 p0 = vtx(sc.vertices, f.p[0]), p1 = vtx(sc.vertices, f.p[1]), p2 = vtx(sc.vertices, f.p[2]);
        const f3 ng = cross(p1 - p0, p2 - p0);
        const float a = 1.0f / (0.5f * length(ng));
        for (uint32_t i = 0; i < numItems; ++i)
            if (!sc.lights[8u * i] && ldb<uint32_t>(sc.lights + 8u * i + 4) == lp.faceID)
                return a * prob_discrete_1d(dist, i);
    }
    return 0.0f;
}

// ---------------------------------------------------------------- camera

// mulMat4x4G_V3 / _P3 / _P4 (matrix.cl): column-major 4x4, row r = m[r], m[4+r], m[8+r], m[12+r]
__device__ __forceinline__ f3 mat_v3(const float* m, f3 v) {
    return mk(m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z,
              m[2] * v.x + m[6] * v.y + m[10] * v.z);
}
__device__ __forceinline__ f3 mat_p3(const float* m, f3 p) {
    f3 r = mk(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12] * 1.0f, m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13] * 1.0f,
              m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14] * 1.0f);
    const float w = m[3] * p.x + m[7] * p.y + m[11] * p.z + m[15] * 1.0f;
    if (w != 1.0f) r = r / w;
    return r;
}

struct Camera {
    const uint8_t* blob;
    const float* l2w;
    float lensRadius, objPDistance, virtualPlaneArea;
};

__device__ __forceinline__ Camera load_camera(const DScene& sc) {
    Camera c;
    c.blob = sc.others + ldb<uint32_t>(sc.others + 0);
    c.l2w = reinterpret_cast<const float*>(c.blob + 64);
    c.virtualPlaneArea = ldb<float>(c.blob + 132);
    c.lensRadius = ldb<float>(c.blob + 136);
    c.objPDistance = ldb<float>(c.blob + 140);
    return c;
}


// sampleLensPos + IDFAlloc + sample_We (camera.cl:60-115): the primary ray of
// pixel (gx, gy), its throughput alpha and direction pdf; consumes 4 randoms.
// The same ray for given samples: lens (cu0, cu1) and pixel position
// (gx + pu0, gy + pu1).
__device__ __forceinline__ void camera_ray_at(const Camera& cam, uint32_t gx, uint32_t gy, float cu0, float cu1,
                                              float pu0, float pu1, f3& org, f3& dir, f3& alpha, float& dirPDF) {
    float ux, uy;
    concentric_disk(cu0, cu1, ux, uy);
    const f3 idfDir = mat_v3(cam.l2w, mk(0.0f, 0.0f, 1.0f));
    const f3 lensLocal = mk(ux * cam.lensRadius, uy * cam.lensRadius, 0.0f);
    org = mat_p3(cam.l2w, lensLocal);
    const float pxs = gx + pu0;
    const float pys = gy + pu1;
    const float* r2c = reinterpret_cast<const float*>(cam.blob + 192);
    float4 pc = make_float4(r2c[0] * pxs + r2c[4] * pys + r2c[8] * 0.0f + r2c[12] * 1.0f,
                            r2c[1] * pxs + r2c[5] * pys + r2c[9] * 0.0f + r2c[13] * 1.0f,
                            r2c[2] * pxs + r2c[6] * pys + r2c[10] * 0.0f + r2c[14] * 1.0f,
                            r2c[3] * pxs + r2c[7] * pys + r2c[11] * 0.0f + r2c[15] * 1.0f);
    if (pc.w != 1.0f) {
        const float rw = 1.0f / pc.w;
        pc.x *= rw;
        pc.y *= rw;
        pc.z *= rw;
        pc.w *= rw;
    }
    f3 d = normalize(mk(pc.x, pc.y, pc.z));
    if (cam.lensRadius > 0.0f) {
        const float ft = -cam.objPDistance / d.z;
        const f3 pFocus = mk(0, 0, 0) + ft * d;
        d = normalize(pFocus - mk(lensLocal.x, lensLocal.y, 0.0f));
    }
    dir = mat_v3(cam.l2w, d);
    dirPDF = 1.0f / (powf(-d.z, 3) * cam.virtualPlaneArea);
    alpha = mk(1, 1, 1);
    alpha *= fabsf(dot(idfDir, dir)) / dirPDF;
}

__device__ __forceinline__ void camera_ray(const Camera& cam, uint32_t gx, uint32_t gy, Rng& rng, f3& org, f3& dir,
                                           f3& alpha, float& dirPDF) {
    const float cu0 = rng.uniform(), cu1 = rng.uniform();
    const float pu0 = rng.uniform(), pu1 = rng.uniform();
    camera_ray_at(cam, gx, gy, cu0, cu1, pu0, pu1, org, dir, alpha, dirPDF);
}

// dirToPolarYTop (global.cl:438-441) -> equirectangular uv
__device__ __forceinline__ float2 env_uv(f3 dir) {
    const float theta = acosf(clampf(dir.y, -1.0f, 1.0f));
    const float phi = fmodf(atan2f(-dir.x, dir.z) + 2.0f * kPi, 2 * kPi);
    return make_float2(phi / (2.0f * kPi), theta / kPi);
}

static inline DScene make_dscene(const clr_scene* scene) {
    DScene sc;
    sc.vertices = reinterpret_cast<const float4*>(scene->vertices);
    sc.normals = reinterpret_cast<const float4*>(scene->normals);
    sc.tangents = reinterpret_cast<const float4*>(scene->tangents);
    sc.uvs = reinterpret_cast<const float2*>(scene->uvs);
    sc.faces = static_cast<const uint8_t*>(scene->faces);
    sc.lights = static_cast<const uint8_t*>(scene->lights);
    sc.materials = scene->materials;
    sc.textures = scene->textures;
    sc.others = scene->others;
    sc.nodes = static_cast<const float4*>(scene->bvh->nodes);
    sc.tris = static_cast<const float4*>(scene->bvh->tris);
    sc.root_box = scene->bvh->root_box;
    sc.num_tris = scene->bvh->num_tris;
    sc.alpha = (scene->flags & CLR_SCENE_ALPHA) != 0;
    return sc;
}

// Blocks for a ray kernel: no more than fit on the GPU at once.  Its loop
// hands each thread a fixed run of rays; blocks beyond the resident ones would
// start only as the first finish, and the last of them would end the launch.
template <typename K>
static inline unsigned int resident_grid(K kernel, int block, size_t smem, unsigned int work_blocks) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm <= 0) {
        cudaGetLastError();
        per_sm = 1;
    }
    const unsigned int full = (unsigned int)(clr_sm_count() * per_sm);
    return std::max(1u, std::min(work_blocks, full));
}

static inline bool same_scene(const DScene& a, const DScene& b) {
    return a.vertices == b.vertices && a.normals == b.normals && a.tangents == b.tangents && a.uvs == b.uvs &&
           a.faces == b.faces && a.lights == b.lights && a.materials == b.materials && a.textures == b.textures &&
           a.others == b.others && a.nodes == b.nodes && a.tris == b.tris && a.root_box == b.root_box &&
           a.num_tris == b.num_tris && a.alpha == b.alpha;
}

// A block of a render loop's iterations as a CUDA graph, captured on a
// stream of the calling thread and kept per thread and device for the last
// argument set (`same` compares two sets): the loops launch several kernels
// per iteration, and their launch gaps cost more than the kernels of a small
// image.  Returns null when capture is not possible; the caller then launches
// the kernels itself.  `drop` forgets the graph after a failed launch.  A
// thread's graphs and capture streams are not destroyed when it exits (the
// runtime may be shut down by then): one graph per device per thread remains.
template <typename Args>
struct BlockGraphCache {
    static constexpr int kDevices = 64;
    struct Entry {
        cudaStream_t cap = nullptr;
        cudaGraphExec_t exec = nullptr;
        Args args{};
    };
    Entry e[kDevices];

    template <typename Launch, typename Same>
    cudaGraphExec_t get(const Args& a, Launch launch, Same same) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevices) return nullptr;
        Entry& g = e[dev];
        if (g.exec && same(g.args, a)) return g.exec;
        if (!g.cap && cudaStreamCreateWithFlags(&g.cap, cudaStreamNonBlocking) != cudaSuccess) {
            g.cap = nullptr;
            return nullptr;
        }
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(g.cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return nullptr;
        launch(a, g.cap);
        if (cudaStreamEndCapture(g.cap, &graph) != cudaSuccess || !graph) return nullptr;
        const cudaError_t err = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (err != cudaSuccess) {
            g.exec = nullptr;
            return nullptr;
        }
        g.args = a;
        return g.exec;
    }
    void drop() {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevices) return;
        e[dev].exec = nullptr;
        e[dev].cap = nullptr;
    }
};

static inline int check_render_args(const clr_scene* scene, uint32_t* rand_states, float* pixels) {
    if (!scene || !scene->bvh) return clr_set_error(CLR_EINVAL, "clr_render: NULL scene or bvh");
    if (!rand_states || !pixels || !scene->vertices || !scene->faces || !scene->lights || !scene->materials ||
        !scene->textures || !scene->others)
        return clr_set_error(CLR_EINVAL, "clr_render: NULL buffer");
    if ((reinterpret_cast<uintptr_t>(pixels) | reinterpret_cast<uintptr_t>(rand_states) |
         reinterpret_cast<uintptr_t>(scene->vertices) | reinterpret_cast<uintptr_t>(scene->others)) & 15u)
        return clr_set_error(CLR_EINVAL, "clr_render: pixels, rand_states, vertices and others must be 16-byte aligned");
    return CLR_OK;
}

}  // namespace clr
