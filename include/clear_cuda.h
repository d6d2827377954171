/*
 * clear_cuda.h -- C ABI of the GB300 (sm_103a) LBVH build, BVH traversal and
 * path tracer.
 *
 * Conventions (all entry points):
 *   - return an int status (CLR_OK = 0); no C++ exception crosses the ABI;
 *     clr_last_error_string() describes the last failure of the calling thread;
 *   - every data pointer is a DEVICE pointer owned by the caller, unless the
 *     parameter says "host";
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream); work is enqueued asynchronously on it;
 *   - a handle is not thread-safe, distinct handles are independent.
 *
 * Each declaration cites the reference (shocker-0x15/CLeaR) interface it
 * replaces, as file:line within that project.
 */
#ifndef CLEAR_CUDA_H
#define CLEAR_CUDA_H

#include <stdint.h>

#if defined(__GNUC__)
#define CLR_API __attribute__((visibility("default")))
#else
#define CLR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum {
    CLR_OK = 0,
    CLR_EINVAL = 1,     /* bad argument */
    CLR_ECUDA = 2,      /* a CUDA runtime call failed */
    CLR_ENOMEM = 3,     /* device allocation failed */
    CLR_ETIMEOUT = 4,   /* a bounded device-side wait gave up */
    CLR_ESTACK = 5,     /* a traversal stack would have overflowed */
    CLR_ECAPACITY = 6   /* a fixed-size buffer is too small */
};

/* Device-side error bits, read back with clr_device_status(). */
#define CLR_DEVERR_SORT_TIMEOUT 0x1u  /* radix-sort look-back spin hit its limit */
#define CLR_DEVERR_STACK        0x2u  /* traversal stack full (ray reported as miss) */
#define CLR_DEVERR_REFIT        0x4u  /* refit climb exceeded the tree depth bound */
#define CLR_DEVERR_QUEUE        0x8u  /* a wavefront queue or bounded wait failed */
#define CLR_DEVERR_INPUT        0x10u /* scene data not laid out as the entry point requires */

/* Byte sizes of the records below. */
#define CLR_NODE_BYTES 64u      /* internal node: both child boxes + child refs */
#define CLR_TRI_BYTES 48u       /* triangle record: p0, p1-p0, p2-p0, triangle id */
#define CLR_REF_NODE_BYTES 48u  /* reference LBVH::InternalNode / LeafNode */

/*
 * A built BVH.  The caller allocates the three device buffers, sized
 *   nodes    : max(num_tris - 1, 1) * CLR_NODE_BYTES
 *   tris     : num_tris * CLR_TRI_BYTES                (in leaf = sorted order)
 *   root_box : 8 floats {min x,y,z, root, max x,y,z, 0}; `root` holds the
 *              uint32 bit pattern of the root's child reference
 * Internal node (16 floats), stored at the index of its split position (the
 * last sorted leaf of its left subtree): child-0 box
 * {minx,miny,minz,maxx,maxy,maxz}, child-1 box, two uint32 child references
 * (bit 31 set = leaf index, clear = internal-node index), and the far ends of
 * the two children's leaf ranges.  Leaf i's triangle record is
 * tris[i] = {p0.xyz, id, (p1-p0).xyz, 0, (p2-p0).xyz, 0}.
 * The tree is the reference's Karras radix tree
 * (OpenCL/lbvh_construction.cl:342-410) with the same children in the same
 * order; clr_lbvh_export_reference renumbers it into the reference layout.
 */
typedef struct clr_bvh {
    uint32_t num_tris;
    uint32_t bits_per_dim;
    void* nodes;
    void* tris;
    float* root_box;
} clr_bvh;

/* ------------------------------------------------------------ LBVH build */

typedef struct clr_lbvh clr_lbvh;

/* Replaces LBVHBuilder::LBVHBuilder(context, device, numFaces)
 * (OpenCL_PathTracer/LBVHBuilder.h:70, LBVHBuilder.cpp:19-48): allocates the
 * builder's scratch pool for up to `capacity` triangles on the current
 * device.  The pool grows on demand in clr_lbvh_build, as the reference's
 * does (LBVHBuilder.cpp:167-170). */
CLR_API int clr_lbvh_create(uint32_t capacity, clr_lbvh** out);
CLR_API int clr_lbvh_destroy(clr_lbvh* h);

/* Replaces LBVHBuilder::perform(queue, vertices, faces, numFaces,
 * numBitsPerDim, internalNodes, leafNodes, events, profiling)
 * (OpenCL_PathTracer/LBVHBuilder.h:72-74, LBVHBuilder.cpp:160-375).
 * Vertex k of triangle t is (vx,vy,vz)[tri[3t+k]], or [3t+k] when tri is
 * NULL (unindexed soup).  bits_per_dim in [1, 21] (the reference uses 20 in
 * main.cpp:365; 10 gives 30-bit keys).  Fills out->nodes/tris/root_box and
 * sets out->num_tris and out->bits_per_dim.  No host synchronisation:
 * the scene box stays on the device (the reference reads it back,
 * LBVHBuilder.cpp:229).  The builds of one handle share its scratch pool, as
 * the reference's builder shares its buffers: issue them on one stream, or
 * make a second stream wait for the first's build; separate handles build
 * concurrently. */
CLR_API int clr_lbvh_build(clr_lbvh* h, const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                   uint32_t num_tris, uint32_t bits_per_dim, clr_bvh* out, void* stream);

/* Upload and build from host arrays: what the reference host does by
 * creating the vertex and face buffers from host memory
 * (CL_MEM_COPY_HOST_PTR, OpenCL_PathTracer/main.cpp:342-343) and then calling
 * LBVHBuilder::perform (main.cpp:365).  host_vx/vy/vz hold num_verts
 * vertices (num_verts = 3 * num_tris for a soup, host_tri NULL); host_tri
 * holds 3 vertex indices per triangle.  Same outputs and results as
 * clr_lbvh_build on the same data; if host_root_box is not NULL the 8-float
 * root record (root_box of clr_bvh) is copied back to it on `stream` after
 * the build.
 *
 * For a stream of builds (a scene per frame): the inputs go into one of two
 * device input buffers owned by the builder, used in turn, on a copy stream
 * of the builder's own; the build waits on `stream` for that copy.  A copy
 * waits only for the build that last read its buffer (two calls back), so the
 * copy of call k+1 runs while call k builds.  Copies are not ordered after
 * other work on `stream`: clr_lbvh_host_copy_after(h, stream) orders every
 * later copy after the work queued on `stream` so far.  Page-locked host
 * arrays (cudaHostAlloc, cudaHostRegister) make the copies asynchronous; the
 * caller keeps the host arrays unchanged until the copy is done
 * (clr_lbvh_host_copy_wait, or a synchronisation of `stream`).  The input
 * buffers grow to the largest call (12 bytes per vertex + 12 per indexed
 * triangle, each) and are freed by clr_lbvh_destroy. */
CLR_API int clr_lbvh_build_host(clr_lbvh* h, const float* host_vx, const float* host_vy, const float* host_vz,
                                const uint32_t* host_tri, uint32_t num_verts, uint32_t num_tris,
                                uint32_t bits_per_dim, clr_bvh* out, float* host_root_box, void* stream);

/* Later clr_lbvh_build_host copies start after the work queued on `stream`
 * so far (e.g. after an event that opens a timed region). */
CLR_API int clr_lbvh_host_copy_after(clr_lbvh* h, void* stream);

/* Blocks the host until every clr_lbvh_build_host copy issued so far is done:
 * their host arrays may then be changed. */
CLR_API int clr_lbvh_host_copy_wait(clr_lbvh* h);

/* Allocation-free build, for callers that may not allocate device memory:
 * hosts that give this library a fixed device-memory budget through their own
 * allocator and forbid any other allocation, and per-frame loops where the
 * device synchronisation implied by cudaMalloc/cudaFree would stall the
 * pipeline.  No counterpart in the reference (its builder allocates a scratch
 * pool, LBVHBuilder.cpp:50-158).
 * Same inputs, outputs and results as clr_lbvh_build, but the scratch is a
 * fixed array inside this library: at most 262,144 triangles (larger inputs
 * fail with CLR_ECAPACITY), and every GPU that loads the library keeps that
 * 12 MiB array until the process exits.  The first call on a device resolves
 * the array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  A device reset (or another
 * context made current on the device) gives the array a new address: the
 * next call resolves it again, so it too belongs outside any stream capture.
 * All calls share the one
 * array, so calls that overlap on the GPU (different streams or threads)
 * race: serialise them.  Nothing is allocated or freed. */
CLR_API int clr_lbvh_build_noalloc(const float* vx, const float* vy, const float* vz, const uint32_t* tri,
                                   uint32_t num_tris, uint32_t bits_per_dim, clr_bvh* out, void* stream);

/* Segmented build of many scenes at once (an addition beside
 * LBVHBuilder::perform, which builds one scene per call): scene s owns
 * triangles [scene_offsets[s], scene_offsets[s+1]) of the concatenated inputs
 * (`tri` holds indices into the concatenated vertex arrays, or is NULL for a
 * soup); scene_offsets is a HOST array of num_scenes + 1 entries starting at
 * 0, every scene non-empty.  One scene-box pass, one Morton pass (keys carry
 * the scene id above the 3 x bits_per_dim Morton bits), one radix sort of
 * radix_bits-bit digits (6, 7 or 8; 0 = 8) and one tree pass build every
 * scene.  Scene s's BVH is
 *   {n_s, bits_per_dim, nodes + CLR_NODE_BYTES * off_s,
 *    tris + CLR_TRI_BYTES * off_s, root_boxes + 8 * s}
 * (triangle ids scene-local) and is bit-identical to clr_lbvh_build of that
 * scene alone.  `nodes` holds total_tris nodes, `tris` total_tris records. */
CLR_API int clr_lbvh_build_batched(clr_lbvh* builder, const float* vx, const float* vy, const float* vz,
                                   const uint32_t* tri, const uint32_t* scene_offsets, uint32_t num_scenes,
                                   uint32_t bits_per_dim, uint32_t radix_bits, void* nodes, void* tris,
                                   float* root_boxes, void* stream);

/* Parity/debug export of the last build of `h` into the reference layouts:
 * inodes: (n-1) x 48 B LBVH::InternalNode, lnodes: n x 48 B LBVH::LeafNode
 * (LBVHBuilder.h:17-29), parents: 2n-1 uint32 (leaves at [0,n), internal at
 * [n,2n-1), lbvh_construction.cl:399-409; root entry = 0xFFFFFFFF),
 * sorted_idx: n uint32, keys: n uint64 sorted Morton keys.  Any output may be
 * NULL. */
CLR_API int clr_lbvh_export_reference(clr_lbvh* h, const clr_bvh* bvh, void* inodes, void* lnodes, uint32_t* parents,
                              uint32_t* sorted_idx, uint64_t* keys, void* stream);

/* Per-pass timing of the build, the counterpart of the reference's
 * `profiling` flag (LBVHBuilder.cpp:173-348, one event per pass).  When
 * enabled, clr_lbvh_build records a CUDA event around every kernel it
 * launches; clr_lbvh_pass_times then waits for the last build and returns
 * the per-kernel times in ms, in launch order: scene box, Morton, each sort
 * pass, Karras, refit.  names (optional) receives a static label per pass. */
CLR_API int clr_lbvh_set_profiling(clr_lbvh* h, int enable);
CLR_API int clr_lbvh_pass_times(clr_lbvh* h, float* ms, const char** names, int max_passes, int* num_passes);

/* ------------------------------------------------------------- traversal */

/* rays: 8 floats per ray {ox,oy,oz,tmax, dx,dy,dz,0} (32 B, 16-B aligned).
 *
 * Closest hit.  Replaces rayIntersection (OpenCL/bvh_traversal.cl:182-215):
 * the same depth-first visiting order and the same triangle/box arithmetic,
 * so hit ids and t are those of the reference (with uint32 triangle ids; the
 * reference truncates to ushort, bvh_traversal.cl:56).  t starts at tmax.
 * Miss: hit_id = 0xFFFFFFFF, hit_t = tmax. */
CLR_API int clr_trace_closest(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id, float* hit_t,
                      void* stream);

/* The same query (same ids and distances, bit for bit) visiting the nearer
 * child first, by box entry distance: about a quarter of the node visits.
 * Where the reference's answer depends on its fixed child order -- two
 * triangles hit at the same t, or a box whose rounded entry distance lies a
 * few ulp past a hit inside it -- the ray is detected and searched again in
 * the reference's order; clr_trace_replays counts those rays. */
CLR_API int clr_trace_closest_ordered(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                      float* hit_t, void* stream);

/* Rays that clr_trace_closest_ordered searched again in the reference's order
 * on the current device, summed over its launches (synchronous read; clear
 * resets the count). */
CLR_API int clr_trace_replays(uint64_t* count, int clear);

/* Shadow (any-hit) query; the reference shoots a closest-hit ray for this
 * (OpenCL/pathtracer.cl:119-122).  occluded[r] = 1 when a triangle is hit at
 * 0 <= t <= tmax. */
CLR_API int clr_trace_shadow(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint8_t* occluded, void* stream);

/* clr_trace_closest_ordered and clr_trace_shadow with the rays searched in
 * the order of the Morton code of their origins (8 bits per axis in the
 * tree's root box): the rays a warp searches together start in the same
 * region and share the tree's nodes in the caches.  The same answers, each
 * written at its ray's own index; for rays given in no spatial order (random
 * directions and origins) about 1.7x the closest-hit and 1.2x the shadow
 * throughput (the sorted shadow query searches nearer children first), for rays already
 * ordered (a camera's) a cost of about a millisecond per 16 M rays.  The
 * 256-byte aligned device workspace holds clr_trace_sort_workspace_bytes(n)
 * bytes (16 per ray and the sort's tile words); its contents are scratch. */
CLR_API int clr_trace_sort_workspace_bytes(uint32_t num_rays, uint64_t* bytes);
CLR_API int clr_trace_closest_sorted(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                     float* hit_t, void* workspace, uint64_t workspace_bytes, void* stream);
CLR_API int clr_trace_shadow_sorted(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint8_t* occluded,
                                    void* workspace, uint64_t workspace_bytes, void* stream);

/* ----------------------------------------------------------- path tracer */

/*
 * Scene in the reference's byte-blob format (OpenCL/pathtracer.cl:25-46,
 * OpenCL_PathTracer/Scene.h:165-225), all device pointers:
 *   vertices, normals, tangents : float4 per entry (cl_float3 layout)
 *   uvs       : float2 per entry
 *   faces     : 56-byte Face records (Face.hpp:15-21)
 *   lights    : 8-byte LightInfo {u8 atInfinity, u32 reference}
 *   materials, textures, others : the three scene blobs; others[0..2] are the
 *               u32 offsets of the camera, the environment head and the light
 *               power distribution (Scene.cpp:39-41)
 *   bvh       : an LBVH built over the faces' vertices (clr_lbvh_build)
 */
typedef struct clr_scene {
    const float* vertices;
    const float* normals;
    const float* tangents;
    const float* uvs;
    const void* faces;
    const void* lights;
    const uint8_t* materials;
    const uint8_t* textures;
    const uint8_t* others;
    const clr_bvh* bvh;
    uint32_t flags;  /* CLR_SCENE_*; 0 when none apply */
} clr_scene;

/* Some face has an alpha texture (Face::alphaTexPtr).  The closest-hit
 * searches then apply the reference's cutout test (bvh_traversal.cl:102-105):
 * a face with uvs whose alpha texture reads 0 at the hit is not recorded,
 * though the search bound has already moved to its distance, so it still
 * hides what lies behind it, and a shadow ray counts as blocked by it.  When
 * a ray's only hits are such cutouts the reference reads an intersection
 * record it never wrote; here that ray is a miss.  Without the flag alpha
 * textures are not read. */
#define CLR_SCENE_ALPHA 0x1u

/* Trace with nearer-child-first traversal, replaying in the reference's order
 * the rays whose hit could depend on the order (see clr_trace_closest_ordered):
 * the same image as without the flag, faster.  Scenes with CLR_SCENE_ALPHA are
 * always traced in the reference's order. */
#define CLR_RENDER_ORDERED 0x1u
/* clr_render: run the wavefront form (identical results, several times
 * faster) on a workspace the library keeps per device until the process
 * exits, grown to the largest image rendered; renders that share it take
 * turns on the GPU.  Not for stream capture (it may allocate, and it orders
 * itself after earlier renders through an event).  clr_render_wavefront
 * takes a caller-owned workspace instead. */
#define CLR_RENDER_WAVEFRONT 0x2u

/* Replaces the `pathtracing` kernel (OpenCL/pathtracer.cl:25-271) launched
 * once per tile per sample (main.cpp:477-494): adds `spp` path samples per
 * pixel of a width x height image to `pixels` (float4 per pixel, xyz =
 * accumulated radiance, w untouched), advancing the per-pixel XORShift128
 * states `rand_states` (4 x uint32 per pixel, pixel (x,y) at 4*(y*width+x)).
 * max_depth caps the number of bounces (0 = the reference's 100).  The
 * caller divides by the sample count, as the reference's `scaling` pass does
 * (post_processing.cl:20-26). */
CLR_API int clr_render(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states, float* pixels,
                       uint32_t spp, uint32_t max_depth, uint32_t flags, void* stream);

/* clr_render that also counts what the paths visit, for the path's traffic
 * per sample (the reference's visiting counter, rayIntersectionVis in
 * bvh_traversal.cl:217-254, extended to whole paths).  The same image and
 * random-number updates as clr_render.  Adds to counts (5 device uint64,
 * zeroed by the caller): [0] closest-hit rays traced, [1] shadow rays
 * traced, [2] BVH nodes loaded and [3] triangles tested by both, [4] surface
 * hits shaded. */
CLR_API int clr_render_counted(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                               float* pixels, uint32_t spp, uint32_t max_depth, uint32_t flags,
                               unsigned long long* counts, void* stream);

/* Wavefront form of clr_render: the same paths, random numbers and
 * contributions (identical results), split into extend / shade / shadow
 * kernels over path state in `workspace`, with per-pixel path regeneration;
 * escaped and surface-hit paths are shaded by separate kernels.
 * The caller provides a 256-byte aligned device workspace of at least
 * clr_render_workspace_bytes(width, height) bytes.  Waits on `stream` every
 * eight iterations to stop once every pixel has its spp samples.  Those
 * eight iterations are launched as one CUDA graph, captured on a stream of
 * the calling thread and kept per thread and device for the last argument
 * set (scene, workspace, states, pixels, sizes, flags); a call with other
 * arguments captures anew.  Not for stream capture (it synchronises). */
CLR_API int clr_render_workspace_bytes(uint32_t width, uint32_t height, uint64_t* bytes);
CLR_API int clr_render_wavefront(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                                 float* pixels, uint32_t spp, uint32_t max_depth, uint32_t flags, void* workspace,
                                 uint64_t workspace_bytes, void* stream);

/* clr_render_wavefront for the image rows [row0, row0 + rows) only (the
 * reference renders per 64 x 64 tile, main.cpp:477-494): `rand_states` and
 * `pixels` hold those rows alone (width * rows entries, row-major from row0),
 * the camera sees the whole width x height image.  Each pixel's samples
 * depend only on its own random state, so the rows of a band are
 * bit-identical to the same rows of a whole-image render: one process per
 * GPU renders a band and the bands are gathered (clear_gb300/shard.py).  The
 * workspace holds clr_render_workspace_bytes(width, rows) bytes. */
CLR_API int clr_render_wavefront_rows(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t row0,
                                      uint32_t rows, uint32_t* rand_states, float* pixels, uint32_t spp,
                                      uint32_t max_depth, uint32_t flags, void* workspace, uint64_t workspace_bytes,
                                      void* stream);

/* Replaces the `bvh_visualizer` kernel (OpenCL/bvh_visualizer.cl:25-84): one
 * ray per pixel through the lens centre and pixel centre; adds to `pixels`
 * (float4 per pixel) the hit material's base colour plus 0.025 per BVH box
 * the closest-hit search accepts (internal and leaf,
 * in the reference's visiting order, rayIntersectionVis,
 * bvh_traversal.cl:217-254).  `visits` (optional, uint32 per pixel) receives
 * that box count. */
CLR_API int clr_bvh_visualize(const clr_scene* scene, uint32_t width, uint32_t height, float* pixels,
                              uint32_t* visits, void* stream);

/* The visiting statistics of the closest-hit search, the counter of
 * rayIntersectionVis (bvh_traversal.cl:217-254) per ray: counts[2r] internal
 * boxes accepted (nodes loaded), counts[2r+1] leaf boxes accepted (triangles
 * tested), in the reference's order with t starting unbounded (tmax is not
 * read).  hit_id (optional) receives the closest hit as clr_trace_closest
 * gives it for tmax = infinity.  For measuring traversal traffic. */
CLR_API int clr_trace_closest_counted(const clr_bvh* bvh, const float* rays, uint32_t num_rays, uint32_t* hit_id,
                                      uint32_t* counts, void* stream);

/* ----------------------------------------------------- post-processing */

/* Replaces the `scaling` + `toneMapping` kernel pair that turns the
 * accumulation buffer into the BMP image (OpenCL/post_processing.cl:20-26,
 * 98-117; main.cpp:526-536), fused into one kernel.  `accum` holds float4 per
 * pixel (xyz = radiance summed over `spp` samples); `bgr` receives the
 * reference's BMP pixel array: 8-bit BGR, rows bottom-up, each row
 * 3 * width + width % 4 bytes (padding written as zero), ready for a BMP
 * file header (BMPExporter.cpp:14-55). */
CLR_API int clr_postprocess_ldr(const float* accum, uint32_t width, uint32_t height, uint32_t spp, uint8_t* bgr,
                                void* stream);

/* The luminance and tone-mapping scale clr_postprocess_ldr computes per
 * pixel, written as float4 {Y, expf(-Y), scale, 0} to `scales` (16-byte
 * aligned, width * height entries) instead of the bytes: the check that Y and
 * scale are exactly the double-precision expressions of the reference's
 * double literals (Y = (float)(0.2989 r + 0.5866 g + 0.1144 b),
 * scale = (float)((1 - e) / Y)) although they are computed in float. */
CLR_API int clr_postprocess_scales(const float* accum, uint32_t width, uint32_t height, uint32_t spp, float* scales,
                                   void* stream);

/* Recomputes, on the device and in place, the importance distribution of an
 * image-based environment light after its texels changed: the
 * ContinuousConsts2D_H that createContinuousConsts2D_H_FromImageTexture
 * (OpenCL_PathTracer/CreateFunctions.cpp:246-349) builds on the host, one
 * stratum per texel, at byte `dist_offset` of the `others` blob, from the
 * RGBA16F image texture at byte `tex_offset` of the `textures` blob, of
 * `width` x `height` texels (width at most 25,596).  `row_weight` (height
 * floats, device) weights each row's luminance; NULL uses the reference's
 * zenith correction cos(pi (0.5 - (i + 0.5) / height)) with the device's
 * cosf.  The structure's headers must already be laid out (by the scene
 * encoder); a mismatch with them, or with width / height, sets
 * CLR_DEVERR_INPUT. */
CLR_API int clr_env_distribution_update(uint8_t* others, uint32_t dist_offset, const uint8_t* textures,
                                        uint32_t tex_offset, uint32_t height, uint32_t width,
                                        const float* row_weight, void* stream);

/* ------------------------------------------------------------- batched */

/* Many scenes rendered by one wavefront (an addition; the reference renders
 * one scene per process).  Scene s has its own blobs, BVH (e.g. one scene of
 * clr_lbvh_build_batched), camera and widths[s] x heights[s] image; the
 * batch's pixels are numbered scene after scene, and rand_states / pixels
 * passed to clr_batch_render are the concatenation of the per-scene arrays.
 * Each scene's result is bit-identical to clr_render_wavefront of that scene
 * with the same states.  A fixed pool of pool_slots path slots renders every
 * sample of one pixel, then takes the next unrendered pixel. */
typedef struct clr_batch clr_batch;
typedef struct clr_batch_config {
    uint32_t trace_block;  /* threads per block of the extend and shadow kernels (32 .. 256, multiple of 32; 0 = 128) */
    uint32_t shade_block;  /* threads per block of the shading kernel (32 .. 128, multiple of 32; 0 = 128) */
    uint32_t pool_slots;   /* path slots = queue capacity (0 or more than the pixels = one per pixel) */
    uint32_t reserved;
} clr_batch_config;

#define CLR_BATCH_GRAPH 0x2u /* clr_batch_render: run the whole frame loop as one CUDA graph launch */

/* `scenes`, `widths`, `heights` are host arrays of num_scenes entries; the
 * scene structs' device pointers must stay valid for the batch's life. */
CLR_API int clr_batch_create(const clr_scene* scenes, const uint32_t* widths, const uint32_t* heights,
                             uint32_t num_scenes, const clr_batch_config* cfg, clr_batch** out);
CLR_API int clr_batch_destroy(clr_batch* batch);
CLR_API int clr_batch_set_config(clr_batch* batch, const clr_batch_config* cfg);
CLR_API int clr_batch_get_config(const clr_batch* batch, clr_batch_config* cfg);
CLR_API int clr_batch_pixels(const clr_batch* batch, uint32_t* total_pixels);
/* Adds spp samples to every pixel of every scene.  flags: CLR_RENDER_ORDERED,
 * CLR_BATCH_GRAPH (the graph is captured on first use and reused while the
 * buffers, spp, max_depth, flags and configuration stay the same; without it
 * the host checks every 8 iterations whether paths remain). */
CLR_API int clr_batch_render(clr_batch* batch, uint32_t* rand_states, float* pixels, uint32_t spp, uint32_t max_depth,
                             uint32_t flags, void* stream);

/* ------------------------------------------------------------- adjoint */

/* Parameters of clr_render_adjoint (all pointers are device pointers).
 * A differentiated parameter is a constant texture of the textures blob
 * (TEX_COLOR_CONSTANT: 3 channels, kind 0; TEX_FLOAT_CONSTANT: 1 channel,
 * kind 1), named by its byte offset; every material component that reads it
 * contributes.  The environment parameter is the image texture the scene's
 * image-based environment light reads (its texels, as decoded colours). */
typedef struct clr_adjoint_params {
    const uint32_t* param_tex;   /* K textures-blob offsets */
    const uint8_t* param_kind;   /* K kinds: 0 colour, 1 float */
    uint32_t num_params;         /* K */
    float* grad_params;          /* K x 4 floats, accumulated: xyz (colour) or x (float) */
    uint32_t env_tex;            /* textures-blob offset of the environment texture, 0xFFFFFFFF = none */
    float* grad_env;             /* texels x 4 floats (row-major), accumulated: xyz */
    uint32_t* tape;              /* optional: tape_capacity records of CLR_TAPE_WORDS words */
    uint32_t tape_capacity;
    uint32_t* tape_count;        /* records written (may exceed the capacity: the rest were dropped) */
} clr_adjoint_params;

/* Tape records (32 uint32 words) of every replayed path, for checking the
 * gradient against a re-evaluation of the same paths.  Words 0-3: pixel,
 * sample, depth, kind (bits 0-7) | CLR_TAPE_VISIBLE.  Floats follow:
 *   CAM    (0): 4-6 camera weight alpha0;
 *   EMIT   (1): 4 MIS weight, 5-7 emitted radiance, 8 environment texel (or
 *               0xFFFFFFFF), 9 environment multiplier;
 *   RR     (2): 4 1 / continuation probability;
 *   NEE    (3): 4 scalar weight, 5-7 light radiance, 8 texel, 9 multiplier,
 *               10 material offset, 11-12 uv, 13-15 vout and 16-18 vin in
 *               the shading frame, 19 component mask; counts if VISIBLE;
 *   SAMPLE (4): 4 |cos| / pdf, 10-19 as NEE; word 19 = 0x80000000 | index
 *               for a sampled specular component. */
#define CLR_TAPE_WORDS 32u
#define CLR_TAPE_VISIBLE 0x100u

/* Path-replay backpropagation through the wavefront path tracer (an addition
 * beside the reference, which has no derivatives).  Given dLoss/dAccum
 * (float4 per pixel, xyz used) for the image that clr_render_wavefront would
 * accumulate from the same rand_states, spp and max_depth, adds
 * sum_pixels dLoss/dAccum . dAccum/dtheta to grad_params and grad_env, with
 * sampling decisions, pdfs, MIS weights and roulette probabilities held
 * constant.  rand_states advance exactly as in the forward render.  The
 * workspace (256-byte aligned) holds at least
 * clr_render_adjoint_workspace_bytes(width, height, num_params) bytes
 * (including 132 bytes per pixel in which the primal pass keeps the hit
 * records and next-event visibilities of each path's first 8 vertices for the
 * replay pass).  width * height must stay below 2^27 (CLR_EINVAL). */
CLR_API int clr_render_adjoint_workspace_bytes(uint32_t width, uint32_t height, uint32_t num_params,
                                               uint64_t* bytes);
/* clr_render_adjoint flag: the replay pass traces every ray again instead of
 * taking the primal pass's hit records and next-event visibilities for the
 * first 8 vertices: the same paths and gradients, with the replay's
 * intersections all recomputed from the RNG seeds (more traversal work). */
#define CLR_ADJOINT_RETRACE 0x4u
CLR_API int clr_render_adjoint(const clr_scene* scene, uint32_t width, uint32_t height, uint32_t* rand_states,
                               const float* dloss_daccum, uint32_t spp, uint32_t max_depth, uint32_t flags,
                               const clr_adjoint_params* params, void* workspace, uint64_t workspace_bytes,
                               void* stream);

/* ------------------------------------------------------ Wavefront .obj */

/* Parsing half of loadModel / OBJ::load (ModelLoader.cpp:155-495): the
 * .obj's vertex positions, uvs (stored as 1 - v) and normals, its faces
 * grouped by runs of `f` lines, and the materials of its .mtl library, with
 * the reference's line rules (host code; no device work).  Turning this into
 * scene records -- the `%05u_` material names, matte or glass materials,
 * textures, faces -- is the caller's part (clear_gb300/model_loader.py). */
enum { CLR_OBJ_VTN = 0, CLR_OBJ_VN = 1, CLR_OBJ_VT = 2, CLR_OBJ_V = 3, CLR_OBJ_NONE = 4 };

typedef struct clr_obj_group {
    uint32_t first_face, num_faces; /* range in the face array */
    uint32_t format;                /* CLR_OBJ_*, fixed by the run's first face */
    uint32_t smooth;                /* `s` value in effect (0 = off) */
    uint32_t name;                  /* `g` name, offset in the string table */
    uint32_t material;              /* `usemtl` name, offset in the string table */
} clr_obj_group;

typedef struct clr_obj_material { /* OBJ::Material (ModelLoader.cpp:34-51) */
    float Kd[3], Ks[3], Ka[3];
    float Ns, Ni;                   /* defaults 100 and 1 */
    uint32_t name, map_Kd, map_Ks, map_Ka; /* string offsets (0 = none); maps include the .mtl's directory */
} clr_obj_material;

typedef struct clr_obj_counts {
    uint32_t num_positions, num_uvs, num_normals, num_faces;
    uint32_t num_groups, num_materials;
    uint32_t num_skipped;           /* face lines dropped: no format, or an index outside the lists */
    uint32_t string_bytes;
} clr_obj_counts;

typedef struct clr_obj_model clr_obj_model;

/* Parses `path` and the first .mtl of each `mtllib` line.  CLR_EINVAL if the
 * .obj cannot be opened. */
CLR_API int clr_obj_parse(const char* path, clr_obj_model** model);
CLR_API int clr_obj_counts_of(const clr_obj_model* model, clr_obj_counts* counts);
/* Pointers into the model (valid until clr_obj_free): positions 3 floats and
 * uvs 2 floats per entry, normals 3 floats, faces 9 uint32 per triangle
 * (p0 p1 p2, uv0 uv1 uv2, n0 n1 n2; 0-based, UINT32_MAX where the group's
 * format has no such index), groups, materials, the string table.  Any
 * output pointer may be NULL. */
CLR_API int clr_obj_data(const clr_obj_model* model, const float** positions, const float** uvs,
                         const float** normals, const uint32_t** faces, const clr_obj_group** groups,
                         const clr_obj_material** materials, const char** strings);
CLR_API void clr_obj_free(clr_obj_model* model);

/* ----------------------------------------------------------------- misc */

/* Reads (and optionally clears) the device error bits CLR_DEVERR_* of the
 * current device.  Synchronises the device. */
CLR_API int clr_device_status(uint32_t* bits, int clear);

/* Thread-local description of the last failure. */
CLR_API const char* clr_last_error_string(void);

/* ------------------------------------------------------- bounded waits
 * The reference has no bounded waits (its host catches cl::Error only,
 * main.cpp:546-551); these two entry points exist to test the ones here. */

/* Lowers the bounds of the two waits that can run out: the polls of a radix
 * sort pass's look-back (CLR_DEVERR_SORT_TIMEOUT when exceeded) and the
 * iterations of the batched frame loop (CLR_DEVERR_QUEUE when paths remain).
 * 0 restores the built-in bound.  Process-wide; for tests. */
CLR_API int clr_debug_set_wait_limits(uint32_t sort_spin_limit, uint32_t batch_iteration_cap);

/* One sort pass over 2 * tile_keys 32-bit keys (tile_keys = 4096) in which
 * only the second tile's block runs, so its look-back waits for a tile that
 * never publishes, runs out of polls, raises CLR_DEVERR_SORT_TIMEOUT and
 * returns.  scratch holds 4 * (4 * tile_keys + 769) bytes. */
CLR_API int clr_debug_lookback_stall(uint32_t* keys, uint32_t* scratch, uint32_t tile_keys, void* stream);

/* Whether the LBVH tree pass gathers its staging records with TMA copies
 * (1, the default where the driver offers the tensor-map encoder) or with
 * plain loads (0); both give the same tree.  Process-wide; for tests. */
CLR_API int clr_debug_set_tma_gather(int enable);

#ifdef __cplusplus
}
#endif
#endif /* CLEAR_CUDA_H */
