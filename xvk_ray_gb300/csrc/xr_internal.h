// xr_internal.h -- context, device data layout and launch wrappers of libxr.so.
//
// Device layout (structure of arrays, every per-pixel access one 128-bit or
// 64-bit load/store):
//   corrected mode ("packed"):
//     gb_pos[2]  float4 {x_view.xyz, oct16(n_view)}      ping-pong by frame parity
//     gb_mat[2]  u32 material id of the visible point (0xFFFFFFFF = invalid)
//     cand_a     float4 {x_sample.xyz, p_q}
//     cand_b     float4 {L_out.rgb, oct12(n_sample) | has_sample << 31}
//                (for invalid pixels .rgb holds the directly seen emission)
//     res_t[2]   2 planes float4: {x_s.xyz, W}, {L.rgb, oct12(n_s) | M << 24}  (32 B/pixel)
//     res_s      same, single buffer
//   compat mode ("wide", the reference's fields at full precision):
//     s_xv {x_view, matID} s_nv {n_view, randSeed} s_xs {x_sample, p_q}
//     s_ns {n_sample, 0}   s_L {L_out, 0}
//     res_t / res_s: 4 planes {x_s, W} {L, w_sum} {n_s, m} {f, 0}, 2N entries each
//   path queues (wavefront): 3 float4 per path {o, pixel} {d, rng} {throughput, p_q}
#pragma once

#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/xr.h"

#ifdef __CUDACC__
#include <cuda_fp16.h>
#else
struct __half2;
#endif

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <cuda_runtime_api.h>
#endif
#include <nvtx3/nvToolsExt.h>

namespace xr {

// An NVTX range over a host-side scope (frame, BVH build, top-level rebuild, refit, cache
// step): visible to a profiler's timeline, a no-op call otherwise (NVTX v3 is header-only).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int kStackSize = 40;

// Per-context device counter words (zeroed per frame except the error word).
constexpr uint32_t kCntShadow = 32;        // shadow rays queued by the spatial pass
constexpr uint32_t kCntFetchPath = 64;     // + bounce: ray-fetch counter of that bounce's trace
constexpr uint32_t kCntFetchShadow = 96;   // ray-fetch counter of the shadow trace
constexpr uint32_t kCntFetchQuery = 97;    // ray-fetch counter of xr_trace_rays
constexpr uint32_t kCntNonFinite = 98;     // rays ended early for a non-finite origin or direction
constexpr uint32_t kCntCacheQuery = 99;    // radiance-cache query records of the frame
constexpr uint32_t kCntCacheTrain = 100;   // radiance-cache training records of the frame
constexpr uint32_t kCntCacheNee = 101;     // next-event rays of the current bounce's training paths
constexpr uint32_t kCntFetchNee = 102;     // ray-fetch counter of the next-event trace
constexpr uint32_t kCntError = 127;        // sticky XR_DEVFLAG_* bits
constexpr uint32_t kCounterWords = 128;
constexpr uint32_t kMaxBounces = 31;

// 8-wide compressed BVH node, 80 B (five 16-byte words).
//  w0: origin p.xyz, byte-packed {e.x, e.y, e.z (biased by 127), internal mask}
//  w1: child_base, tri_base, meta[0..3], meta[4..7]
//  w2..w4: q_lo.x[8], q_lo.y[8], q_lo.z[8], q_hi.x[8], q_hi.y[8], q_hi.z[8]
// meta byte = (bits << 5) | position: a hit child contributes bits << position
// to one 32-bit mask.  Empty: 0.  Leaf of 1..3 triangles at tri_base + offset:
// bits = 1, 3 or 7 (unary count), position = offset (0..23).  Internal child in
// slot s: bits = 1, position = 24 + s; it is node child_base + popc(imask & ((1 << s) - 1)).
struct alignas(16) WideNode {
    float px, py, pz;
    uint32_t exyz_imask;
    uint32_t child_base, tri_base;
    uint32_t meta[2];
    uint32_t q[12];
};
static_assert(sizeof(WideNode) == 80, "wide node is 80 B");

struct DeviceScene {
    const float4* tri;        // 3 float4 per BVH triangle slot: v0 {xyz, prim id}, v1, v2
    const WideNode* nodes;
    uint32_t n_nodes;
    const uint4* tri_idx;     // per primitive {i0, i1, i2, material of v0}
    const float4* vpos;       // per vertex {pos, 0}
    const float4* vnrm;       // per vertex {normal, 0}
    const XrMaterial* mats;
    uint32_t n_mats;
    uint32_t ntri;
    uint32_t n_tri_slots;     // BVH triangle slots (>= ntri: split triangles have several)
    // emissive triangles (next-event estimation of the cache's training paths)
    const uint32_t* light_prim;      // primitive of light k
    const float* light_cdf;          // inclusive CDF of the power pmf (last entry 1)
    const float* light_pmf;          // probability of light k (power / total power)
    const float* prim_light_pdf;     // per primitive: pmf / area (0: not a sampled light)
    uint32_t n_lights;
    // base-colour textures (texture.cuh)
    const float2* vuv;               // per vertex texture coordinate
    const uint4* tex_info;           // per texture {first texel, width, height, 0}
    const uint32_t* texels;          // RGBA8 texels of all textures, row 0 = v 0
    uint32_t n_tex;
    // instances (xr_set_instances): a top-level BVH over the instances' world boxes
    // whose leaves are instance records; `nodes` then holds the bottom-level BVHs
    const WideNode* tlas_nodes;
    uint32_t n_tlas_nodes;
    const float4* inst_slots;        // 4 float4 per top-level leaf slot: world-to-object rows, {instance, root}
    uint32_t n_inst_slots;
    const float4* inst_xform;        // 6 float4 per instance: object-to-world rows, world-to-object rows
    uint32_t n_inst;                 // 0: no instances
    // traversal queue tuning (xr_set_tuning / xr_autotune): idle lanes before a warp refills
    // from the ray queue, and lanes with triangles below which a warp postpones its tests
    uint32_t refill_min, postpone_below;
};

// One view of a multi-view context: its pixels are [pix_off, pix_off + W H) of the
// per-pixel buffers, its camera rays start at BVH node `root` (the first node of
// its scene in the concatenated node array), its 16x8 raygen tiles follow tile_off.
struct ViewInfo {
    uint32_t pix_off;
    uint32_t W, H;
    uint32_t root;
    uint32_t tile_off;
    uint32_t pad[3];
};

struct FrameArgs {
    DeviceScene sc;
    const XrUniformBufferObject* ubo;   // device copies of this frame's UBOs, one per view
    uint32_t W, H, N;                   // single view: its extent; several: W = H = 0, N = all pixels
    const ViewInfo* views;              // n_views entries (device)
    uint32_t n_views, n_tiles;
    uint32_t multi_root;                // views over more than one scene
    uint32_t compat, temporal_on, spatial_on, visibility, write_pt, seed;
    uint32_t m_cap_t, m_cap_s, n_nb;
    float radius;
    uint32_t parity;                    // current_frame % 2 (host copy for pointer selection)
    // corrected layout
    float4* gb_pos_cur; const float4* gb_pos_prev;
    uint32_t* gb_mat_cur; const uint32_t* gb_mat_prev;
    float4* cand_a; float4* cand_b;
    float4* rt_cur0; float4* rt_cur1; const float4* rt_prev0; const float4* rt_prev1;
    float4* rs0; float4* rs1;
    // compat layout
    float4* s_xv; float4* s_nv; float4* s_xs; float4* s_ns; float4* s_L;
    float4* rw[4];            // temporal reservoirs, 2N entries per plane
    float4* rsw[4];           // spatial reservoirs, 2N entries per plane
    // shared
    float4* thr0;             // bounce-0 throughput (write_pt)
    float2* gb_uv;            // texture coordinate of the visible point (read only when the scene has textures)
    float4* le0;              // directly seen emission (write_pt, compat)
    uchar4* out_ldr; float4* out_hdr; float4* out_pt;
    // wavefront
    float4* q_in[3]; float4* q_out[3];
    uint4* hits;              // closest-hit record per queue slot {prim, t, b1, b2}
    int32_t* hit_inst;        // its instance (scenes with instances)
    uint2* shadow_q;          // corrected spatial pass: {pixel << 5 | slot, neighbour pixel}
    uint32_t* occ;            // per pixel: occluded neighbour slots
    uint32_t* reproj;         // corrected mode, per pixel: its visible point's pixel in the previous frame (kInvalid: none)
    uint2* nb_slot;           // corrected spatial pass, plane per slot: {neighbour pixel, merge weight
                              // target * Jacobian * W * M} of a similar neighbour, {kInvalid, 0} otherwise
    uint8_t* nb_m;            // and plane per slot: that neighbour's M
    uint32_t* counters;       // [b] paths entering bounce b, then the kCnt* words above
    uint32_t grid_persistent, grid_trace;
    uint32_t ray_bundle;      // camera-ray slot order in a 16 x 8 tile: 0 8x4 blocks, 1 16x2 rows, 2 4x8 blocks
    uint32_t blk_temporal, blk_spatial;   // threads per block of the temporal and spatial kernels
    // learned radiance cache (corrected mode): paths end at x_s unless selected for training
    uint32_t cache_on;
    uint4* cache_q;           // query records, 2 uint4 each (capacity N)
    uint4* cache_t;           // training records, 3 uint4 each (capacity cache_t_cap)
    uint32_t cache_t_cap;
    const uint32_t* cache_sel; // device word: pixels selected for training this frame (nullptr: none;
                               // restir.cu: cache_training_pixel), set per frame by k_cache_select_next
    float4* cache_nee;        // next-event rays: 3 float4 each {o, record}, {d, tmax}, {contribution, 0}
};

// Learned radiance cache state (nrc.cu, cache_api.cu).
struct CacheState {
    bool allocated = false;
    bool grads_dirty = false;        // gradients left by a gradient-only xr_cache_train
    XrCacheParams params{};
    float lo[3] = {0.0f, 0.0f, 0.0f};
    float inv_ext = 1.0f;
    uint32_t step = 0;               // Adam steps taken
    float* mlp = nullptr;            // FP32 master weights (17,408)
    float* mlp_grad = nullptr;
    float* mlp_m = nullptr;
    float* mlp_v = nullptr;
    uint8_t* w_fwd = nullptr;        // bfloat16 weight images (shared-memory layout)
    uint8_t* w_bwd = nullptr;
    float* grid = nullptr;           // FP32 master table (16 x 2^19 x 2)
    __half2* table = nullptr;        // binary16 table used by the kernels
    float* grid_grad = nullptr;
    float* grid_m = nullptr;
    float* grid_v = nullptr;
    float* loss = nullptr;           // mean loss of the last training launch
    float* adam = nullptr;           // device Adam state {beta1^t, beta2^t, 1 - beta1^t, 1 - beta2^t}
    uint4* queries = nullptr;        // query records (capacity query_cap)
    uint4* train = nullptr;          // training records (capacity train_cap)
    uint8_t* tiles = nullptr;        // training tiles: inputs, then input gradients (128 B a record)
    uint32_t* order = nullptr;       // spatial order of the records (8 x train_cap words): keys, values, twice;
                                     // then the unit positions in that order (float4)
    uint32_t* order_hist = nullptr;  // radix-sort digit counts (128 x 256 words)
    float4* nee = nullptr;           // next-event rays of one bounce (capacity train_cap)
    uint32_t query_cap = 0, train_cap = 0;
    uint32_t* sel = nullptr;         // device word: training pixels of the next frame (adaptive)
    uint32_t sel_target = 0, sel_pixels = 0;   // the target and extent it was last set for (0: to be set)
    bool frame_used = false;         // the last frame ran with the cache
    bool frame_trained = false;
};

// One scene of a context: its ranges in the concatenated vertex, primitive,
// material, node and triangle-slot arrays, the node ranges of its BVH levels
// (relative to node_off), the finest grid exponent of its quantisation and the
// bounds of its vertices.
struct ScenePart {
    uint32_t vert_off = 0, nv = 0, prim_off = 0, ntri = 0, mat_off = 0, nm = 0;
    uint32_t node_off = 0, n_nodes = 0, slot_off = 0, n_slots = 0;
    std::vector<uint32_t> levels;
    int emin = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    // the root node's child boxes as stored (lo xyz, hi xyz per child), read back on first
    // use after each build or refit: the instance world boxes are taken over them
    std::vector<double> root_boxes;
};

// Input and output of a wide-BVH build (bvh_build.cu): triangles (tri_idx, vpos),
// or boxes whose leaves copy a 4-float4 record per primitive (instances).
struct WideBuild {
    uint32_t n = 0;
    const uint4* tri_idx = nullptr;
    const float4* vpos = nullptr;
    const float4* box_lo = nullptr;
    const float4* box_hi = nullptr;
    const float4* records = nullptr;
    const uint32_t* ref_prim = nullptr;   // box input of triangle pieces: the triangle of each box
    int emin_floor = -1000;             // lower bound of the finest grid exponent
    int builder = 0;                    // 0: XR_BVH_BUILDER (PLOC unless "lbvh"), 1: PLOC, 2: LBVH
    // Caller's arrays to build into (capacity max(n - 1, 1) nodes and 4 n slot words); the build allocates its
    // own when they are null.
    WideNode* nodes_into = nullptr;
    float4* slots_into = nullptr;
    WideNode* nodes = nullptr;          // device arrays owned by the caller afterwards
    float4* slots = nullptr;
    uint32_t n_nodes = 0, n_slots = 0, depth = 0;
    int emin = 0;
    std::vector<uint32_t> level_off;    // first node of each level, then the node count
    float ms = 0.0f;
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;   // stream-ordered scratch of builds and refits, kept cached between frames
    int sm_count = 0;
    XrParams params{};
    bool params_set = false;
    std::string last_error;

    // scene
    uint32_t nv = 0, ntri = 0, nm = 0;
    uint4* d_tri_idx = nullptr;
    float4* d_vpos = nullptr;
    float4* d_vnrm = nullptr;
    float2* d_vuv = nullptr;
    uint4* d_tex_info = nullptr;
    uint32_t* d_texels = nullptr;
    uint32_t n_tex = 0;
    XrMaterial* d_mats = nullptr;
    bool scene_ready = false;
    bool scene_has_non_lambert = false;

    // BVH
    // emissive triangles (light sampling tables)
    uint32_t* d_light_prim = nullptr;
    float* d_light_cdf = nullptr;
    float* d_light_pmf = nullptr;
    float* d_prim_light_pdf = nullptr;
    uint32_t n_lights = 0;

    WideNode* d_nodes = nullptr;
    float4* d_tris = nullptr;
    uint32_t n_nodes = 0, n_tri_slots = 0, bvh_depth = 0;
    bool bvh_ready = false;
    float ms_bvh = 0.0f;
    std::vector<uint32_t> bvh_levels;   // build of a single scene: first node of each level, then the node count
    int bvh_emin = 0;                   // its finest grid exponent
    float scene_lo[3] = {0, 0, 0}, scene_hi[3] = {0, 0, 0};   // bounds of the uploaded scene's vertices
    // the scenes of the context (one after xr_upload_scene, n after xr_upload_scenes):
    // ranges in the concatenated arrays, BVH levels for refit, vertex bounds
    std::vector<ScenePart> parts;
    // instances (xr_set_instances)
    std::vector<XrInstance> instances;
    std::vector<float> inst_xform_host;   // 24 floats per instance: object-to-world, world-to-object
    float4* d_inst_xform = nullptr;
    WideNode* d_tlas_nodes = nullptr;
    float4* d_inst_slots = nullptr;
    uint32_t n_tlas_nodes = 0, n_inst_slots = 0;   // of the last top-level build
    uint32_t inst_cap = 0;   // instances the transform, top-level node and slot arrays have room for
    bool tlas_stale = false;   // a bottom-level refit moved instanced geometry: rebuild before the next use
    float ms_tlas = 0.0f, ms_refit = 0.0f;
    cudaEvent_t refit_ev[2] = {};   // around the last refit; read by xr_get_stats once the stream is idle
    bool refit_timed = false;

    // per-pixel buffers
    uint32_t W = 0, H = 0, N = 0;
    void* pix_mem = nullptr;       // one allocation for all per-pixel buffers
    size_t pix_bytes = 0;
    FrameArgs fa{};                // pointers of the current allocation
    float4* gb_pos[2] = {nullptr, nullptr};
    uint32_t* gb_mat[2] = {nullptr, nullptr};
    float4* rt0[2] = {nullptr, nullptr};
    float4* rt1[2] = {nullptr, nullptr};
    float4* q[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    uint32_t* d_counters = nullptr;
    XrUniformBufferObject* d_ubo = nullptr;
    // Pinned staging of the UBOs, one slot per frame parity (2 x ubo_cap): the host fills
    // frame k's slot once frame k-2's upload has read it (ubo_ev), so it can enqueue a
    // frame while the two before it are still in flight.
    XrUniformBufferObject* h_ubo = nullptr;
    cudaEvent_t ubo_ev[2] = {};
    uint32_t ubo_slot = 0;                    // slot of the UBOs staged last

    // statistics
    uint32_t frames = 0;
    uint32_t last_bounces = 0;
    unsigned long long* d_work = nullptr;   // node visits, triangle tests of the last ray query
    uint64_t query_rays = 0;
    uint32_t error_flags = 0;
    cudaEvent_t ev[8] = {};          // 0..3 frame passes, 4 end of cache training, 5 unused, 6/7 cache inference
    // The cache's inference runs on infer_stream beside the training paths' bounces 2..
    // (forked at infer_fork_ev once bounce 1's queries exist, joined by the temporal pass
    // at infer_ev); its training on side_stream (first stage forked with the inference,
    // second stage after the paths at fork_ev, Adam after infer_ev, joined after the
    // temporal pass at join_ev).  ev_train0 times the training's start.
    cudaStream_t side_stream = nullptr, infer_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, infer_fork_ev = nullptr, infer_ev = nullptr, join_ev = nullptr;
    cudaEvent_t ev_train0 = nullptr;
    bool side_pending = false, infer_pending = false;
    cudaEvent_t user_ev[8] = {};
    // asynchronous image reads (xr_read_output_async): the LDR image is double-buffered by
    // frame parity; a read copies the last frame's buffer on copy_stream once the frame is done
    cudaStream_t copy_stream = nullptr;
    uchar4* ldr[2] = {nullptr, nullptr};
    cudaEvent_t ldr_ready[2] = {};   // recorded on the frame stream: the buffer's frame is complete
    cudaEvent_t ldr_copied[2] = {};  // recorded on copy_stream: the buffer has been read
    bool ldr_copy_pending[2] = {false, false};   // a frame that writes the buffer waits for the read first
    uint32_t ldr_reads[2] = {0u, 0u};    // buffers of the reads xr_wait_output has not waited for, oldest first
    uint32_t ldr_nreads = 0;
    XrStats stats{};
    CacheState cache;

    // views (xr_set_views; empty: one view of scene 0 with the parameters' extent)
    std::vector<XrView> views;
    std::vector<ViewInfo> view_info;      // host copy of the device view table
    ViewInfo* d_views = nullptr;
    uint32_t ubo_cap = 1;                 // UBOs d_ubo (and each slot of h_ubo) hold
    std::vector<uint32_t> scene_roots;    // first node of each scene (kNoRoot: empty scene)
    // CUDA graphs of one frame per parity of the frame index (xr_render_views)
    bool graphs_on = false;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    uint32_t graph_bounces[2] = {0, 0};
    // launch configuration (xr_autotune): persistent CTAs per SM, 0 = occupancy maximum
    uint32_t tune_trace_ctas = 0, tune_shade_ctas = 0;
    uint32_t tune_refill = 0, tune_postpone = 0, tune_bundle = 0, tune_temporal_block = 0, tune_spatial_block = 0;
};

constexpr uint32_t kNoRoot = 0xFFFFFFFFu;
void invalidate_graphs(Context* c);
// Records `e` on the context's stream (an external event node when the stream is being captured).
cudaError_t record_event(Context* c, cudaEvent_t e);
cudaError_t record_event_on(cudaStream_t st, cudaEvent_t e);
xr_status realloc_pixels(Context* c);   // per-pixel buffers and view table for the current views / params

xr_status fail(const Context* ctx, xr_status code, const std::string& msg);
xr_status cuda_check(Context* ctx, cudaError_t e, const char* what);
// Stream-ordered allocations from the context's pool, ordered on its stream.
xr_status pool_alloc_bytes(Context* ctx, void** p, size_t bytes, const char* what);
template <typename T>
inline xr_status pool_alloc(Context* ctx, T** p, size_t count, const char* what) {
    return pool_alloc_bytes(ctx, (void**)p, (count ? count : 1) * sizeof(T), what);
}
void pool_free(Context* ctx, void* p);
xr_status check_flags(Context* c);   // reads the sticky device error word; new bits -> error status

// Makes `dev` current for the scope of a C ABI call and restores the caller's device.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// ---- launch wrappers (bvh_build.cu) ----
xr_status build_bvh(Context* ctx);
xr_status build_wide(Context* ctx, WideBuild& wb);
void launch_refit_slots(float4* tris, uint32_t first, uint32_t n, const uint4* tri_idx, const float4* vpos,
                        cudaStream_t st);
void launch_refit_level(WideNode* nodes, uint32_t first, uint32_t n, const float4* tris, float4* box_lo,
                        float4* box_hi, int emin, cudaStream_t st);
xr_status refit_part(Context* c, uint32_t part, int emin);   // instances.cu
void free_lights(Context* c);
xr_status upload_lights(Context* c, const std::vector<uint4>& tri, const std::vector<float4>& pos,
                        const XrMaterial* m, uint32_t nm);
xr_status rebuild_tlas(Context* c);                           // instances.cu
xr_status sync_tlas(Context* c);
void apply_tuning(Context* c);     // xr_api.cu: the context's tuning into fa (and fa.sc) before launches   // instances.cu: rebuild a stale top level (no-op otherwise)
void free_instances(Context* c);                              // instances.cu

// ---- launch wrappers (trace.cu) ----
// `fetch` must be zero when the launch starts (the kernel's ray-fetch counter).
void launch_trace(const DeviceScene& sc, const float* rays, uint32_t n, int any_hit, int32_t* prim, int32_t* inst,
                  float* t, float* bary, uint32_t* fetch, uint32_t* flags, unsigned long long* work, int sm_count,
                  cudaStream_t st);

// ---- launch wrappers (restir.cu) ----
// after_bounce1(arg), when given, is called once bounce 1's shading is enqueued (or after the
// loop for a single bounce): the enqueue point of work that needs only bounce 1's records.
void launch_initial(const FrameArgs& fa, uint32_t number_of_bounces, cudaStream_t st,
                    void (*after_bounce1)(void*) = nullptr, void* arg = nullptr);
void launch_temporal(const FrameArgs& fa, bool write_image, cudaStream_t st);
void launch_spatial(const FrameArgs& fa, cudaStream_t st);
void launch_accumulate_sample(const FrameArgs& fa, double* acc, cudaStream_t st);
void launch_export_samples(const FrameArgs& fa, uint32_t* out, cudaStream_t st);
void launch_import_samples(const FrameArgs& fa, const uint32_t* in, cudaStream_t st);
void launch_reproject(const FrameArgs& fa, cudaStream_t st);   // reprojection of the stored G-buffer (temporal pass on its own)
void launch_export_res_wide(float4* const planes[4], uint32_t n, uint32_t* out, cudaStream_t st);
void launch_export_res_packed(const float4* p0, const float4* p1, uint32_t n, uint32_t* out, cudaStream_t st);
void launch_import_res_wide(float4* const planes[4], uint32_t n, const uint32_t* in, cudaStream_t st);
void launch_import_res_packed(float4* p0, float4* p1, uint32_t n, const uint32_t* in, cudaStream_t st);

// ---- launch wrappers (nrc.cu) ----
cudaError_t cache_configure_kernels();
void launch_cache_init(CacheState& cs, uint32_t seed, cudaStream_t st);
void launch_cache_refresh(CacheState& cs, cudaStream_t st);   // binary16 table + bfloat16 images from the masters
void launch_cache_pack(const XrCacheSample* s, uint32_t n, uint4* rec, uint32_t stride, cudaStream_t st);
// count from *count_ptr (device) when non-null, else count_host; cand_b non-null: add to candidates
void launch_cache_infer(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host, float* out3,
                        float4* cand_b, uint32_t* err, int sm_count, cudaStream_t st);
void launch_cache_train(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host,
                        uint32_t cap, bool apply, uint32_t* err, int sm_count, cudaStream_t st);
void launch_cache_encode_stage(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host,
                               uint32_t cap, int sm_count, cudaStream_t st);
void launch_cache_grad_stage(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host,
                             uint32_t cap, uint32_t* err, int sm_count, cudaStream_t st);
void launch_cache_adam(CacheState& cs, cudaStream_t st);   // one Adam step on the gradients (bias correction on the device)
void launch_cache_adam_reset(CacheState& cs, cudaStream_t st);
void launch_cache_wait_selftest(uint64_t limit_ns, uint32_t* err, cudaStream_t st);   // a wait that runs out
// Training pixels of the next frame from this frame's training records: sel * target / got,
// clamped to [target, n] (set_to != 0: set the word to set_to instead)
void launch_cache_select_next(uint32_t* sel, const uint32_t* got, uint32_t target, uint32_t n, uint32_t set_to,
                              cudaStream_t st);
// ---- cache_api.cu ----
xr_status cache_prepare_frame(Context* c, uint32_t frame);   // capacities; sets the FrameArgs cache fields
void cache_after_bounce1(void* ctx);          // the cache's inference, forked once bounce 1's queries exist
void cache_after_paths(Context* c);           // its training after the bounce loop; the frame waits for the inference
void cache_free(Context* c);
void cache_scene_bounds(Context* c, const float* vertices, uint32_t nv);

}  // namespace xr

struct XrContext : public xr::Context {};
