/*
 * xr.h -- C ABI of the GB300-native ReSTIR GI frame pipeline (libxr.so).
 *
 * This is the drop-in boundary for the reference's ReSTIR GI render pass
 * (0Setsuna0/XVK_Ray).  Every entry point names the reference interface it
 * replaces.  Plain C types only: pointers, sizes, POD structs.  No exception
 * crosses the ABI; every call returns an xr_status and the message of the last
 * failure is available from xr_last_error().
 *
 * Threading: one context per host thread.  All work of a context is ordered on
 * its own CUDA stream; xr_render_frame() and xr_read_output_async() are
 * asynchronous, xr_read_output(), xr_wait_output(), xr_read_buffer() and
 * xr_sync() synchronise.
 */
#ifndef XR_H
#define XR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XR_API_VERSION 1

typedef int32_t xr_status;
enum {
    XR_OK = 0,
    XR_ERR_INVALID_ARGUMENT = 1,
    XR_ERR_CUDA = 2,
    XR_ERR_OUT_OF_MEMORY = 3,
    XR_ERR_STATE = 4,          /* call out of order (e.g. render before the BVH is built) */
    XR_ERR_OVERFLOW = 5,       /* a device-side bound (traversal stack, queue) was exceeded */
    XR_ERR_TIMEOUT = 6,        /* a bounded device-side wait gave up */
    XR_ERR_UNSUPPORTED = 7
};

typedef struct XrContext XrContext;

/* src/Asset/Vertex.h:11-16 (AVertex, 36 B) == shader/HLSL/ReSTIRGI/Vertex.hlsl:2-8 */
typedef struct XrVertex {
    float pos[3];
    float normal[3];
    float tex_coord[2];
    int32_t material_index;
} XrVertex;

/* src/Asset/Material.h:8-58 (AMaterial, 32 B) == Material.hlsl:7-14.
   material_model: 0 Lambertian, 1 Metallic (GGX conductor, roughness = fuzziness),
   4 DiffuseLight (emits base_color * 4, BSDF.hlsl:27-32), 5 Plastic (GGX coat
   over Lambert, roughness = fuzziness).  Models 1 and 5 are extensions of this
   library (the reference renders only 0 and 4). */
typedef struct XrMaterial {
    float base_color[4];
    int32_t base_color_texture_index;
    float fuzziness;
    float refraction_index;
    uint32_t material_model;
} XrMaterial;
enum { XR_MAT_LAMBERTIAN = 0, XR_MAT_METALLIC = 1, XR_MAT_DIELECTRIC = 2, XR_MAT_ISOTROPIC = 3,
       XR_MAT_DIFFUSE_LIGHT = 4, XR_MAT_PLASTIC = 5 };

/* src/Asset/Scene.cpp:37 -- per-model uvec2{indexOffset, vertexOffset}; indices
   of a model are relative to its vertexOffset (Ray.rchit.hlsl:29-40). */
typedef struct XrMeshRange {
    uint32_t index_offset;
    uint32_t vertex_offset;
} XrMeshRange;

/* src/Asset/UniformBuffer.h:16-32 (UniformBufferObject, 412 B), glm column-major
   matrices.  number_of_bounces is the path depth; has_sky_box and reuse are
   0/1; current_frame drives the RNG and the reservoir ping-pong. */
typedef struct XrUniformBufferObject {
    float view[16];
    float view_prev[16];
    float projection[16];
    float projection_prev[16];
    float view_inverse[16];
    float projection_inverse[16];
    uint32_t spp;
    uint32_t total_number_of_samples;
    uint32_t number_of_bounces;
    uint32_t random_seed;
    uint32_t has_sky_box;
    uint32_t reuse;
    uint32_t current_frame;
} XrUniformBufferObject;

/* Render-pass parameters.  In the reference these are shader #defines and UI
   toggles (ReSTIRGITemporalReuse.rgen.hlsl:3, ReSTIRGISpatialReuse.rgen.hlsl:4-6,
   src/Editor/UI.cpp:178-204). */
typedef struct XrParams {
    uint32_t width, height;
    uint32_t compat_reference;   /* 1: reproduce the reference bit for bit, quirks included
                                    (aliased previous G-buffer, no-op visibility, M caps 30/300,
                                    6 neighbours in 5 px, RNG reuse across passes) */
    uint32_t temporal_on;        /* merge the previous frame's reservoir */
    uint32_t spatial_on;         /* run spatial reuse (corrected mode; compat always runs it) */
    uint32_t m_cap_temporal;     /* corrected mode, <= 255 */
    uint32_t m_cap_spatial;      /* corrected mode, <= 255 */
    uint32_t n_neighbours;       /* corrected mode, <= 32 */
    float radius_px;             /* corrected mode */
    uint32_t visibility;         /* corrected mode: trace a shadow ray per reused neighbour */
    uint32_t seed;               /* corrected mode: mixed into every pass's RNG stream */
    uint32_t write_pt;           /* also write the plain 1-spp path-traced radiance */
    uint32_t write_hdr;          /* also write the linear radiance before tone mapping */
} XrParams;

/* Defaults of the corrected pipeline (the benchmark's settings): temporal + spatial on, M cap
   20 / 120, 5 neighbours, 30 px, visibility on, seed 1. */
void xr_params_default(XrParams* p, uint32_t width, uint32_t height);
/* The reference's own constants (compat_reference = 1). */
void xr_params_reference(XrParams* p, uint32_t width, uint32_t height);

typedef struct XrDeviceDesc {
    int32_t device;              /* CUDA ordinal */
    uint32_t width, height;      /* swap-chain extent (src/main.cpp:52) */
} XrDeviceDesc;

typedef struct XrStats {
    uint32_t frames;
    uint32_t error_flags;        /* device-side flags seen so far (XR_DEVFLAG_*) */
    float ms_initial, ms_temporal, ms_spatial, ms_frame;   /* last frame, CUDA events */
    uint64_t rays_traced;        /* closest-hit rays of the last frame */
    uint64_t shadow_rays;        /* any-hit rays of the last frame */
    uint32_t bvh_nodes, bvh_triangles, bvh_depth;   /* bvh_triangles: leaf slots (>= triangles: split
                                                       large triangles are referenced by several pieces) */
    float ms_bvh_build;
    uint64_t query_rays;         /* rays of the last xr_trace_rays call */
    uint64_t query_node_visits;  /* BVH nodes visited by those rays */
    uint64_t query_tri_tests;    /* triangle tests of those rays */
    uint64_t nonfinite_rays;     /* rays of the last frame ended as misses for a non-finite origin/direction */
    uint32_t instances;          /* instances of xr_set_instances (0: none) */
    uint32_t tlas_nodes;         /* nodes of the top-level BVH */
    float ms_tlas_build;         /* last top-level BVH build */
    float ms_refit;              /* last xr_update_vertices refit */
} XrStats;
enum { XR_DEVFLAG_STACK_OVERFLOW = 1u, XR_DEVFLAG_QUEUE_OVERFLOW = 2u, XR_DEVFLAG_BAD_INDEX = 4u,
       XR_DEVFLAG_MMA_TIMEOUT = 8u /* a tensor-core completion wait of the radiance cache gave up (1 s) */ };

/* ---- lifetime: replaces Application/ApplicationRT/ApplicationReSTIRGI construction
        (src/Vulkan/RayTracing/ApplicationReSTIRGI.cpp:25-29) ---- */
xr_status xr_create(const XrDeviceDesc* desc, XrContext** out);
void xr_destroy(XrContext* ctx);

/* ---- scene: replaces AScene's concatenation + GPU upload (src/Asset/Scene.cpp:16-87).
        Host arrays are copied; the caller keeps ownership. ---- */
xr_status xr_upload_scene(XrContext* ctx,
                          const XrVertex* vertices, uint32_t vertex_count,
                          const uint32_t* indices, uint32_t index_count,
                          const XrMaterial* materials, uint32_t material_count,
                          const XrMeshRange* ranges, uint32_t range_count);

/* ---- replaces ApplicationRT::CreateAccelerationStructures (ApplicationRT.cpp:55-66):
        LBVH from 63-bit Morton codes, collapsed to an 8-wide compressed BVH. ---- */
xr_status xr_build_bvh(XrContext* ctx);

/* ---- replaces InitReSTIRGITracer (ApplicationReSTIRGI.cpp:304-374) + UI toggles ---- */
xr_status xr_set_params(XrContext* ctx, const XrParams* params);
xr_status xr_get_params(XrContext* ctx, XrParams* params);

/* ---- replaces ApplicationReSTIRGI::Render (ApplicationReSTIRGI.cpp:150-275):
        initial sample -> temporal reuse -> spatial reuse + shading, stream ordered.
        The UBO is the one PathTracer::GetUniformBufferObject builds
        (src/pathTracer.cpp:169-201).  Enqueues the frame and returns; the UBO is
        staged in one of two page-locked slots (by frame parity), so a call waits
        only until the frame two before it has started on the device. ---- */
xr_status xr_render_frame(XrContext* ctx, const XrUniformBufferObject* ubo);

/* Converged reference: the plain path tracer with the initial-sample pass's path
   semantics (shader/HLSL/ReSTIRGI/ReSTIRGIInitialSample.rgen.hlsl:41-181; the
   reference's own multi-spp mode is shader/HLSL/rgen.hlsl:31-151) averaged over
   `spp` samples with FP64 accumulation; sample k uses current_frame = frame0 + k
   for its random numbers.  host_rgb receives width*height*3 doubles.  Needs
   params.write_pt; overwrites the frame's G-buffer and candidates, so the next
   xr_render_frame starts without temporal history. */
xr_status xr_render_reference(XrContext* ctx, const XrUniformBufferObject* ubo, uint32_t frame0, uint32_t spp,
                              double* host_rgb);

/* Output images (the reference's OutputImage, ApplicationReSTIRGI.cpp:248-271). */
enum {
    XR_OUT_LDR8 = 0,   /* width*height RGBA8: ACES + gamma 1/2.2 */
    XR_OUT_HDR = 1,    /* width*height float4: linear radiance before tone mapping */
    XR_OUT_PT = 2      /* width*height float4: plain 1-spp path-traced radiance (write_pt) */
};
xr_status xr_read_output(XrContext* ctx, uint32_t which, void* host, size_t bytes);
/* Frames in flight (the reference's per-frame fences and asynchronous present,
   src/Vulkan/ApplicationRZ.cpp:125-195): enqueues the copy of the last rendered
   frame's RGBA8 image (width*height*4 bytes) into `host` on the context's copy
   stream and returns at once; the next frames render while it runs.  The RGBA8
   image alternates between two device buffers by frame parity, and a frame that
   would overwrite a buffer still being read waits for that read on the device.
   At most two reads are in flight (XR_ERR_STATE for a third).  `host` must stay
   valid, and should be page-locked for the copy to overlap, until the
   xr_wait_output() that covers it returns.  Device error flags are reported by
   xr_sync(). */
xr_status xr_read_output_async(XrContext* ctx, void* host, size_t bytes);
/* Blocks until the oldest xr_read_output_async() copy not yet waited for has
   landed in host memory (returns at once when none is in flight). */
xr_status xr_wait_output(XrContext* ctx);
/* Device pointer of an output image as the last frame wrote it (valid until the
   next xr_set_params/xr_destroy; the RGBA8 image's buffer alternates with the
   frame parity). */
xr_status xr_output_device_ptr(XrContext* ctx, uint32_t which, void** device_ptr);
xr_status xr_sync(XrContext* ctx);
xr_status xr_get_stats(XrContext* ctx, XrStats* stats);
/* CUDA events on the context stream (slots 0..7) for callers that time work
   without access to the stream; xr_event_elapsed synchronises on slot b. */
xr_status xr_event_record(XrContext* ctx, uint32_t slot);
xr_status xr_event_elapsed(XrContext* ctx, uint32_t slot_a, uint32_t slot_b, float* ms);

/* ---- parity/debug access in the reference's own layouts ---- */
enum {
    XR_BUF_SAMPLES = 0,     /* N x ReSTIRGISample (96 B, ReSTIRGICommon.hlsl:6-20) */
    XR_BUF_TEMPORAL = 1,    /* 2N x ReSTIRGIReservoir (112 B, ReSTIRGICommon.hlsl:22-30) */
    XR_BUF_SPATIAL = 2      /* 2N (compat) or N (corrected) x ReSTIRGIReservoir */
};
/* Reads (or, for fixed-candidate checks, writes) a pipeline buffer converted
   to/from the reference layout.  Fields the corrected layout does not store read
   back as 0.  *bytes_out receives the full size when host is NULL. */
xr_status xr_read_buffer(XrContext* ctx, uint32_t which, void* host, size_t bytes, size_t* bytes_out);
xr_status xr_write_buffer(XrContext* ctx, uint32_t which, const void* host, size_t bytes);
/* Runs one pass on the buffers as they are: 1 = temporal, 2 = spatial. */
xr_status xr_run_pass(XrContext* ctx, const XrUniformBufferObject* ubo, uint32_t pass);

/* ---- closest-hit / any-hit queries on the built BVH (TraceRay semantics of
        ReSTIRGIInitialSample.rgen.hlsl:90-98 and ReSTIRGISpatialReuse.rgen.hlsl:44-62).
        rays: n x 8 floats {o.xyz, tmin, d.xyz, tmax} in host memory.  prim = -1 on
        miss; t and bary (b1, b2) are written on a hit.  Ties: lowest primitive id. */
xr_status xr_trace_rays(XrContext* ctx, const float* rays, uint32_t n, int32_t any_hit,
                        int32_t* prim, float* t, float* bary);
/* Same on device pointers, asynchronous on the context stream. */
xr_status xr_trace_rays_device(XrContext* ctx, const float* d_rays, uint32_t n, int32_t any_hit,
                               int32_t* d_prim, float* d_t, float* d_bary);
/* No counterpart in the reference.  xr_trace_rays for callers that cannot
   allocate device memory where they query rays (an engine that owns all device
   memory through its own allocator, a real-time loop where allocation's implicit
   synchronisation is not allowed): the staging lives in one fixed device array
   of this library (65536 rays, about 3 MiB, held on each GPU until exit), so at
   most 65536 rays per call; larger batches fail with XR_ERR_INVALID_ARGUMENT.
   Allocates nothing.  The first call on a device looks the array's address up
   and should come before any stream capture; a device reset (cudaDeviceReset)
   after it is not supported.  Calls share the array: calls that overlap on the
   GPU race, so serialise them.  An instanced world whose top-level BVH is stale
   after xr_update_vertices is refused with XR_ERR_STATE, because rebuilding it
   allocates: render a frame or call xr_trace_rays / xr_get_stats once first.
   Same results as xr_trace_rays. */
xr_status xr_trace_rays_noalloc(XrContext* ctx, const float* rays, uint32_t n, int32_t any_hit,
                                int32_t* prim, float* t, float* bary);

/* ---- host helpers (no GPU work) ---- */
/* Camera for one frame: replaces PathTracer::GetUniformBufferObject
   (src/pathTracer.cpp:169-201) with glm::perspective(fov, aspect, 0.001, 1000),
   projection[1][1] *= -1, depth zero-to-one.  prev may be NULL (first frame). */
typedef struct XrCamera {
    float position[3];
    float yaw_deg, pitch_deg;    /* view = R(pitch, yaw) * T(-position) (src/Editor/Camera.cpp:21-27) */
    float fov_deg;
} XrCamera;
xr_status xr_camera_ubo(const XrCamera* cam, uint32_t width, uint32_t height,
                        const XrUniformBufferObject* prev, uint32_t current_frame,
                        uint32_t number_of_bounces, uint32_t has_sky_box, uint32_t reuse,
                        XrUniformBufferObject* out);

/* Procedural scenes (deterministic).  Call once with NULL arrays to get the
   counts, then with arrays of at least those sizes. */
typedef struct XrSceneData {
    XrVertex* vertices; uint32_t vertex_count;
    uint32_t* indices; uint32_t index_count;
    XrMaterial* materials; uint32_t material_count;
    XrCamera camera;             /* the scene's default camera */
} XrSceneData;
/* Cornell box: 5 walls + 2 rotated boxes (15 / -18 deg) + a 0.5 x 0.5 light of
   radiance (17, 12, 4); Lambertian (0.73)/(0.65,0.05,0.05)/(0.12,0.45,0.15). */
xr_status xr_scene_cornell(XrSceneData* out);
/* Ground plane + n_objects icospheres (subdivision 2) and boxes, scale U[0.2,2],
   random rotation, GGX roughness U[0.05,1], albedo U[0.1,0.9], metallic
   Bernoulli(0.3), n_lights emissive quads of radiance U[5,50]. */
typedef struct XrProceduralDesc {
    uint32_t seed;
    uint32_t n_objects;          /* 4096 -> ~1M triangles */
    uint32_t n_lights;           /* 16 */
    float extent;                /* objects are placed in [-extent, extent]^2 */
    uint32_t sphere_subdiv;      /* 2 -> 320 triangles per sphere */
} XrProceduralDesc;
xr_status xr_scene_procedural(const XrProceduralDesc* desc, XrSceneData* out);

/* Page-locked host memory for the read-back images (cudaMallocHost). */
xr_status xr_alloc_host(size_t bytes, void** ptr);
void xr_free_host(void* ptr);

/* ---- base-colour textures: replaces the reference's per-model image upload
        (src/Asset/Scene.cpp:56-72, src/Asset/TextureImage.cpp:25 -- R8G8B8A8_UNORM)
        and its sampler (src/Vulkan/XVKSampler.h:11-27: linear, clamp to edge).
   RGBA8 texels, row 0 = texture coordinate v = 0; a material whose
   base_color_texture_index >= 0 takes the bilinearly filtered texture RGB instead of
   its base colour (BSDF.hlsl:22-23).  Upload the textures before the scene(s) that
   use them; the texture list is shared by all scenes of the context. */
typedef struct XrTexture {
    uint32_t width, height;
    const uint8_t* rgba8;        /* width * height * 4 bytes */
} XrTexture;
xr_status xr_upload_textures(XrContext* ctx, const XrTexture* textures, uint32_t n);
/* PNG scanline reconstruction for the scene loader (filters None/Sub/Up/Average/Paeth):
   filtered = rows x (1 filter byte + row_bytes), bpp = bytes per pixel (1..8); no GPU. */
xr_status xr_png_unfilter(const uint8_t* filtered, uint32_t rows, uint32_t row_bytes, uint32_t bpp, uint8_t* out);

/* ---- several scenes and views in one context ----
   No single counterpart in the reference, which renders one view of one scene per
   Render call (ApplicationReSTIRGI.cpp:150-275): here one frame renders every view
   of the context in the same kernel launches (one path queue, one traversal
   launch per bounce, one launch per reservoir pass for all views).  Scenes are
   concatenated on the device -- each keeps its own BVH, reached through its root
   node -- so rays of a view only ever see their own scene.  Results of a view are
   bit-identical to rendering it alone.  All views of a frame share the frame
   index parity (the reservoir ping-pong); the learned cache needs a single scene. */
typedef struct XrView {
    uint32_t scene;              /* index into the xr_upload_scenes list */
    uint32_t width, height;
} XrView;

/* Uploads n scenes and builds their BVHs (replaces xr_upload_scene + xr_build_bvh). */
xr_status xr_upload_scenes(XrContext* ctx, const XrSceneData* scenes, uint32_t n);
/* Views and the common parameters (params->width/height are ignored). */
xr_status xr_set_views(XrContext* ctx, const XrView* views, uint32_t n, const XrParams* params);
/* One frame of every view; ubos[v] is view v's camera, all with the same current_frame parity.
   With graphs enabled the frame's launches are captured once per parity and replayed. */
xr_status xr_render_views(XrContext* ctx, const XrUniformBufferObject* ubos);
xr_status xr_read_view_output(XrContext* ctx, uint32_t view, uint32_t which, void* host, size_t bytes);
/* xr_render_reference for every view: host_rgb holds 3 doubles per pixel of all views, view by view. */
xr_status xr_render_reference_views(XrContext* ctx, const XrUniformBufferObject* ubos, uint32_t frame0, uint32_t spp,
                                    double* host_rgb);
xr_status xr_set_graphs(XrContext* ctx, int enabled);   /* CUDA-graph replay of frames */

/* Launch configuration chosen by xr_autotune.  0 in any field = its default.
   Launch shapes never change results: every configuration renders bit-identically. */
typedef struct XrTuning {
    uint32_t trace_ctas_per_sm;  /* persistent traversal CTAs per SM (default: occupancy maximum) */
    uint32_t shade_ctas_per_sm;  /* persistent shading CTAs per SM (default: occupancy maximum) */
    float ms_per_frame;          /* xr_autotune: best measured configuration */
    float ms_default;            /* xr_autotune: the all-defaults configuration */
    uint32_t configs_tried;
    /* ray queues of the persistent traversal: a warp refills from its queue once this many
       lanes are idle (default 8), and postpones triangle tests that fewer lanes than this
       have (default 8) */
    uint32_t refill_min, postpone_below;
    uint32_t ray_bundle;         /* camera rays of a 16 x 8 tile per warp: 0 8x4 blocks (default), 1 16x2 rows, 2 4x8 */
    uint32_t temporal_block;     /* threads per block of the temporal pass: 32, 64 (default), 128, 256 */
    uint32_t spatial_block;      /* threads per block of the spatial passes: 64, 128 (default), 256 */
} XrTuning;
/* Coordinate descent over the fields above (in the order listed): for each, the
   value whose `frames` frames run shortest (ubos: frames x views, in frame order)
   with the others at the best so far.  The choice stays for the context's later
   frames and is written to *out. */
xr_status xr_autotune(XrContext* ctx, const XrUniformBufferObject* ubos, uint32_t frames, XrTuning* out);
/* Applies a launch configuration (e.g. one xr_autotune chose earlier); 0 = occupancy maximum. */
xr_status xr_set_tuning(XrContext* ctx, const XrTuning* tuning);

/* ---- instances, dynamic top-level BVH and refit ----
   Replaces the reference's top-level acceleration structure over one identity
   instance per model (ApplicationRT.cpp:226-258, XVKTLAccelerationStructure.cpp:88)
   and the ObjectToWorld / WorldToObject mapping of its closest-hit shader
   (Ray.rchit.hlsl:46-55).  The scenes of xr_upload_scenes (or the one of
   xr_upload_scene + xr_build_bvh) are the bottom-level BVHs; instances place
   transformed copies of them.  A top-level 8-wide BVH over the instances' world
   boxes is built on the device; a ray enters an instance's BVH in its object
   space (origin and direction mapped by world-to-object, t stays the world
   ray's) and its hit is mapped back: position by object-to-world, shading and
   geometric normals by the inverse transpose.  Closest hit: smallest t, then the
   lowest instance, then the lowest primitive.  With instances set, every view
   renders the instanced world; the learned cache is not available. */
typedef struct XrInstance {
    uint32_t scene;                  /* bottom-level BVH: index into the uploaded scenes */
    uint32_t reserved;               /* 0 */
    float object_to_world[12];       /* row-major 3 x 4: world = M (x, y, z, 1) */
} XrInstance;                        /* 56 bytes */
/* Replaces the instance list (n = 0: back to the scenes without instances) and
   rebuilds the top-level BVH; call again whenever transforms change (e.g. each frame).
   The instance arrays keep their device addresses while n stays within the largest
   list set so far, so captured frame graphs stay valid across such calls. */
xr_status xr_set_instances(XrContext* ctx, const XrInstance* instances, uint32_t n);
/* 24 floats per instance: object-to-world, then world-to-object (its inverse, computed
   in double precision and rounded to float), row-major 3 x 4, as traversal uses them. */
xr_status xr_get_instance_transforms(XrContext* ctx, float* out, uint32_t n);
/* No counterpart in the reference (its geometry is static).  New vertices of scene
   `scene` (same count, indices and materials as uploaded), then a refit of its BVH
   on the device: triangle slots take the new positions, node boxes are recomputed
   level by level from the deepest and requantised, the topology is kept; with
   instances set, the top-level BVH is rebuilt over the new bounds by the next
   trace, frame or xr_get_stats (once for any number of updates before it). */
xr_status xr_update_vertices(XrContext* ctx, uint32_t scene, const XrVertex* vertices, uint32_t count);
/* xr_trace_rays that also reports each hit's instance (-1 on a miss or without instances). */
xr_status xr_trace_rays_instanced(XrContext* ctx, const float* rays, uint32_t n, int32_t any_hit, int32_t* prim,
                                  int32_t* instance, float* t, float* bary);

/* ---- learned radiance cache ----
   No counterpart in the reference renderer (it has no learned component): the
   cache of Mueller et al., "Real-time Neural Radiance Caching for Path Tracing"
   (SIGGRAPH 2021) over the multiresolution hash encoding of "Instant Neural
   Graphics Primitives" (SIGGRAPH 2022).  16 levels x 2 features x 2^19 binary16
   entries (resolutions 16 ... 2048 over the scene cube), inputs position,
   normal, direction, roughness, albedo, material kind -> 4 x 64 ReLU layers ->
   RGB; bfloat16 weights, FP32 accumulation on the tensor cores; Adam.
   With `enabled`, corrected-mode paths end at their first secondary vertex x_s
   and the ReSTIR GI candidate takes L_out = Le(x_s) + cache(x_s); about
   `train_samples` training paths a frame continue to full depth and their
   suffix radiance at x_s is the training target (relative L2 loss); one Adam
   step per frame when `train` is set.  A training path needs a surface at its
   first bounce, so the number of pixels selected for training adapts frame by
   frame (the previous frame's selected pixels x train_samples / its training
   records, at least train_samples) to yield about train_samples records.
   xr_render_reference never uses the cache. */
typedef struct XrCacheParams {
    uint32_t enabled;            /* paths terminate into the cache (corrected mode only) */
    uint32_t train;              /* one Adam step per rendered frame */
    uint32_t train_samples;      /* training paths wanted per frame, <= 1,048,576 (default 65,536) */
    float learning_rate;         /* Adam step size (default 1e-2) */
    float beta1, beta2, epsilon; /* Adam (defaults 0.9, 0.99, 1e-15) */
    uint32_t seed;               /* parameter initialisation used by xr_cache_reset */
} XrCacheParams;

/* One cache sample (queries and training through the API).  kind = material
   model (XR_MAT_*): 1 and 5 set the metal and plastic inputs.  72 bytes. */
typedef struct XrCacheSample {
    float pos[3];
    float normal[3];
    float wo[3];                 /* unit direction from pos towards the previous path vertex */
    float albedo[3];
    float roughness;
    uint32_t kind;
    float target[3];             /* outgoing radiance (training only) */
    uint32_t pixel;              /* carried through, unused by the API calls */
} XrCacheSample;

typedef struct XrCacheStats {
    uint32_t steps;              /* Adam steps taken since the last reset */
    uint32_t queries;            /* cache queries of the last frame */
    uint32_t train_samples;      /* training samples of the last frame (before rounding to 128) */
    float loss;                  /* mean relative L2 loss of the last training step */
    float ms_infer, ms_train;    /* last frame (CUDA events): inference and training + Adam, each on its own
                                    side stream beside the rest of the frame, from its start to its end */
    float bounds_lo[3];          /* scene cube: unit position = (x - lo) * inv_extent */
    float inv_extent;
} XrCacheStats;

enum { XR_CACHE_MLP = 0, XR_CACHE_GRID = 1, XR_CACHE_MLP_GRAD = 2, XR_CACHE_GRID_GRAD = 3,
       XR_CACHE_MLP_M = 4, XR_CACHE_MLP_V = 5, XR_CACHE_GRID_M = 6, XR_CACHE_GRID_V = 7,
       XR_CACHE_QUERIES = 8,        /* last frame's query records, 8 words each */
       XR_CACHE_TRAIN_RECORDS = 9,  /* last frame's training records, 12 words each */
       XR_CACHE_ADAM_STEP = 10      /* one uint32: Adam steps taken; writing it also sets the
                                       bias-correction state (beta1^t, beta2^t of the current
                                       parameters).  With arrays 0..7 the whole trained state,
                                       for checkpoint and resume */ };
/* MLP arrays: 17,408 floats, layer l < 4 at l * 4096 as [64 out][64 in], layer 4 at
   16384 as [16 out][64 in] (outputs 3..15 unused).  Table arrays: 16 x 2^19 x 2
   floats, level-major, 2 features per entry (the binary16 table is derived). */

void xr_cache_params_default(XrCacheParams* out);
xr_status xr_cache_set_params(XrContext* ctx, const XrCacheParams* p);   /* allocates ~0.3 GB on first use */
xr_status xr_cache_get_params(XrContext* ctx, XrCacheParams* out);
xr_status xr_cache_reset(XrContext* ctx, uint32_t seed);               /* re-initialise weights, table, Adam state */
xr_status xr_cache_set_bounds(XrContext* ctx, const float lo[3], float inv_extent);
/* Predicted outgoing radiance of n samples (host arrays). */
xr_status xr_cache_query(XrContext* ctx, const XrCacheSample* s, uint32_t n, float* out_rgb);
/* Gradients of the mean relative L2 loss over n samples (n a multiple of 128,
   <= 1,048,576); with apply != 0 followed by one Adam step.  *loss may be NULL. */
xr_status xr_cache_train(XrContext* ctx, const XrCacheSample* s, uint32_t n, int apply, float* loss);
/* One Adam step on the current gradients (e.g. written with xr_cache_write), which it then zeroes. */
xr_status xr_cache_step(XrContext* ctx);
/* Self-test of the failure path of the cache's bounded tensor-core waits (no counterpart
   in the reference): one CTA takes tensor memory and an mbarrier as the cache kernels do
   and waits on a phase that nothing completes, with a limit of limit_us microseconds
   (1 .. 1e6).  The wait gives up, the kernel raises XR_DEVFLAG_MMA_TIMEOUT, frees its
   tensor memory and returns, and the call returns XR_ERR_TIMEOUT the first time the
   context sees the flag.  The context stays usable. */
xr_status xr_cache_selftest_wait(XrContext* ctx, uint32_t limit_us);
xr_status xr_cache_read(XrContext* ctx, int which, void* host, size_t bytes, size_t* bytes_needed);
xr_status xr_cache_write(XrContext* ctx, int which, const void* host, size_t bytes);   /* arrays 0..7, step 10 */
xr_status xr_cache_get_stats(XrContext* ctx, XrCacheStats* out);

const char* xr_last_error(const XrContext* ctx);   /* ctx may be NULL: last global error */
uint32_t xr_api_version(void);

#ifdef __cplusplus
}
#endif
#endif /* XR_H */
