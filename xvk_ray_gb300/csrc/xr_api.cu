// xr_api.cu -- the C ABI of libxr.so (include/xr.h).
//
// Host orchestration of the reference's render pass (ApplicationReSTIRGI.cpp:150-275):
// upload the frame's UBO, then initial sample -> temporal reuse -> spatial reuse
// in stream order on the context's own stream.  No exception leaves this file;
// every failure returns a status and records a message for xr_last_error().
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "xr_internal.h"

namespace xr {

namespace {
std::mutex g_err_mu;
std::string g_last_error;
thread_local std::string t_err_copy;

size_t align256(size_t v) { return (v + 255u) & ~size_t(255u); }
}  // namespace

xr_status fail(const Context* ctx, xr_status code, const std::string& msg) {
    {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_last_error = msg;
    }
    if (ctx) const_cast<Context*>(ctx)->last_error = msg;
    return code;
}

xr_status cuda_check(Context* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return XR_OK;
    (void)cudaGetLastError();
    xr_status code = (e == cudaErrorMemoryAllocation) ? XR_ERR_OUT_OF_MEMORY : XR_ERR_CUDA;
    return fail(ctx, code, std::string(what) + ": " + cudaGetErrorString(e));
}

xr_status pool_alloc_bytes(Context* ctx, void** p, size_t bytes, const char* what) {
    *p = nullptr;
    return cuda_check(ctx, cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream), what);
}

void pool_free(Context* ctx, void* p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

void invalidate_graphs(Context* c) {
    for (int i = 0; i < 2; i++) {
        if (c->graph[i]) cudaGraphExecDestroy(c->graph[i]);
        c->graph[i] = nullptr;
        c->graph_bounces[i] = 0u;
    }
}

uint32_t persistent_grid(int sm_count, bool compat);
uint32_t trace_grid(int sm_count, bool instances);

namespace {

void free_pixels(Context* c) {
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);   // reads still in flight from the images
    c->ldr[0] = c->ldr[1] = nullptr;
    c->ldr_copy_pending[0] = c->ldr_copy_pending[1] = false;
    c->ldr_nreads = 0;
    if (c->pix_mem) cudaFree(c->pix_mem);
    c->pix_mem = nullptr;
    c->pix_bytes = 0;
    FrameArgs z{};
    z.sc = c->fa.sc;
    c->fa = z;
    for (int i = 0; i < 2; i++) { c->gb_pos[i] = nullptr; c->gb_mat[i] = nullptr; c->rt0[i] = nullptr; c->rt1[i] = nullptr; }
}

// One allocation holds every per-pixel buffer of the selected layout.
xr_status alloc_pixels(Context* c) {
    free_pixels(c);
    invalidate_graphs(c);
    const XrParams& P = c->params;
    // views: the xr_set_views list, else one view of scene 0 with the parameters' extent
    std::vector<XrView> views = c->views;
    if (views.empty()) views.push_back(XrView{0u, P.width, P.height});
    std::vector<ViewInfo> vinfo(views.size());
    size_t Ntot = 0;
    uint32_t tiles = 0;
    bool multi_root = false;
    for (size_t v = 0; v < views.size(); v++) {
        ViewInfo& vi = vinfo[v];
        vi = ViewInfo{};
        vi.pix_off = (uint32_t)Ntot;
        vi.W = views[v].width;
        vi.H = views[v].height;
        vi.root = views[v].scene < c->scene_roots.size() ? c->scene_roots[views[v].scene] : 0u;
        vi.tile_off = tiles;
        if (vi.root != 0u) multi_root = true;
        Ntot += (size_t)vi.W * vi.H;
        tiles += ((vi.W + 15u) / 16u) * ((vi.H + 7u) / 8u);
    }
    if (Ntot >= (1ull << 31)) return fail(c, XR_ERR_INVALID_ARGUMENT, "views: more than 2^31 pixels in total");
    const size_t N = Ntot;
    const bool compat = P.compat_reference != 0;
    struct Item { void** dst; size_t bytes; };
    std::vector<Item> items;
    FrameArgs& fa = c->fa;
    auto add = [&](void** dst, size_t bytes) { items.push_back({dst, bytes}); };
    if (compat) {
        add((void**)&fa.s_xv, N * 16); add((void**)&fa.s_nv, N * 16); add((void**)&fa.s_xs, N * 16);
        add((void**)&fa.s_ns, N * 16); add((void**)&fa.s_L, N * 16);
        for (int k = 0; k < 4; k++) add((void**)&fa.rw[k], 2 * N * 16);
        for (int k = 0; k < 4; k++) add((void**)&fa.rsw[k], 2 * N * 16);
        if (P.write_pt) add((void**)&fa.le0, N * 16);
    } else {
        for (int i = 0; i < 2; i++) { add((void**)&c->gb_pos[i], N * 16); add((void**)&c->gb_mat[i], N * 4); }
        add((void**)&fa.cand_a, N * 16); add((void**)&fa.cand_b, N * 16);
        for (int i = 0; i < 2; i++) { add((void**)&c->rt0[i], N * 16); add((void**)&c->rt1[i], N * 16); }
        add((void**)&fa.rs0, N * 16); add((void**)&fa.rs1, N * 16);
    }
    if (P.write_pt) { add((void**)&fa.thr0, N * 16); add((void**)&fa.out_pt, N * 16); }
    add((void**)&fa.gb_uv, N * 8);   // written and read only when the scene has textures
    if (!compat) {
        add((void**)&fa.occ, N * 4);
        add((void**)&fa.shadow_q, N * std::max<uint32_t>(P.n_neighbours, 1u) * 8);
        add((void**)&fa.nb_slot, N * std::max<uint32_t>(P.n_neighbours, 1u) * 8);
        add((void**)&fa.nb_m, N * std::max<uint32_t>(P.n_neighbours, 1u));
        add((void**)&fa.reproj, N * 4);
    }
    add((void**)&fa.hits, N * 16);
    add((void**)&fa.hit_inst, N * 4);
    add((void**)&c->ldr[0], N * 4);   // LDR image of even / odd frames
    add((void**)&c->ldr[1], N * 4);
    if (P.write_hdr) add((void**)&fa.out_hdr, N * 16);
    for (int i = 0; i < 2; i++)
        for (int k = 0; k < 3; k++) add((void**)&c->q[i][k], N * 16);
    size_t total = 0;
    for (auto& it : items) total += align256(it.bytes);
    void* mem = nullptr;
    xr_status s = cuda_check(c, cudaMalloc(&mem, total), "cudaMalloc (per-pixel buffers)");
    if (s) return s;
    s = cuda_check(c, cudaMemsetAsync(mem, 0, total, c->stream), "memset (per-pixel buffers)");
    if (s) { cudaFree(mem); return s; }
    size_t off = 0;
    for (auto& it : items) { *it.dst = (char*)mem + off; off += align256(it.bytes); }
    fa.out_ldr = c->ldr[0];
    c->pix_mem = mem;
    c->pix_bytes = total;
    if (!compat)
        for (int i = 0; i < 2; i++) cudaMemsetAsync(c->gb_mat[i], 0xFF, N * 4, c->stream);
    c->W = views[0].width; c->H = views[0].height; c->N = (uint32_t)N;
    fa.W = c->W; fa.H = c->H; fa.N = c->N;
    fa.n_views = (uint32_t)views.size();
    fa.n_tiles = tiles;
    fa.multi_root = multi_root ? 1u : 0u;
    cudaFree(c->d_views);
    c->d_views = nullptr;
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_views, vinfo.size() * sizeof(ViewInfo)), "view table"))) return s;
    cudaMemcpy(c->d_views, vinfo.data(), vinfo.size() * sizeof(ViewInfo), cudaMemcpyHostToDevice);
    c->view_info = vinfo;
    fa.views = c->d_views;
    if (views.size() > c->ubo_cap) {
        cudaStreamSynchronize(c->stream);
        cudaFree(c->d_ubo);
        cudaFreeHost(c->h_ubo);
        c->d_ubo = nullptr;
        c->h_ubo = nullptr;
        c->ubo_cap = 0;
        if ((s = cuda_check(c, cudaMalloc((void**)&c->d_ubo, views.size() * sizeof(XrUniformBufferObject)), "ubo")) ||
            (s = cuda_check(c, cudaMallocHost((void**)&c->h_ubo, 2 * views.size() * sizeof(XrUniformBufferObject)), "ubo staging")))
            return s;
        c->ubo_cap = (uint32_t)views.size();
    }
    fa.counters = c->d_counters;
    fa.ubo = c->d_ubo;
    for (int k = 0; k < 3; k++) { fa.q_out[k] = c->q[0][k]; fa.q_in[k] = c->q[1][k]; }
    return cuda_check(c, cudaStreamSynchronize(c->stream), "per-pixel buffer init");
}

void set_frame_pointers(Context* c, uint32_t parity) {
    FrameArgs& fa = c->fa;
    const XrParams& P = c->params;
    fa.parity = parity;
    if (c->ldr[parity]) {
        fa.out_ldr = c->ldr[parity];
        // work that writes this image waits until an asynchronous read of it has finished
        if (c->ldr_copy_pending[parity]) {
            cudaStreamWaitEvent(c->stream, c->ldr_copied[parity], 0);
            c->ldr_copy_pending[parity] = false;
        }
    }
    fa.compat = P.compat_reference; fa.temporal_on = P.temporal_on; fa.spatial_on = P.spatial_on;
    fa.visibility = P.visibility; fa.write_pt = P.write_pt; fa.seed = P.seed;
    fa.m_cap_t = P.m_cap_temporal; fa.m_cap_s = P.m_cap_spatial; fa.n_nb = P.n_neighbours; fa.radius = P.radius_px;
    if (!P.compat_reference) {
        fa.gb_pos_cur = c->gb_pos[parity]; fa.gb_pos_prev = c->gb_pos[1 - parity];
        fa.gb_mat_cur = c->gb_mat[parity]; fa.gb_mat_prev = c->gb_mat[1 - parity];
        fa.rt_cur0 = c->rt0[parity]; fa.rt_cur1 = c->rt1[parity];
        fa.rt_prev0 = c->rt0[1 - parity]; fa.rt_prev1 = c->rt1[1 - parity];
    }
    fa.grid_persistent = c->tune_shade_ctas ? c->tune_shade_ctas * (uint32_t)c->sm_count
                                            : persistent_grid(c->sm_count, P.compat_reference != 0);
    fa.grid_trace = c->tune_trace_ctas ? c->tune_trace_ctas * (uint32_t)c->sm_count : trace_grid(c->sm_count, !c->instances.empty());
    apply_tuning(c);
}

// Host side of a frame's UBO upload: wait until the last transfer from the frame
// parity's pinned staging slot has read it (the frame two before), then overwrite the
// slot with the n views' UBOs.
xr_status stage_ubos(Context* c, const XrUniformBufferObject* ubos, uint32_t n) {
    const uint32_t slot = ubos[0].current_frame & 1u;
    xr_status s = cuda_check(c, cudaEventSynchronize(c->ubo_ev[slot]), "ubo staging");
    if (s) return s;
    XrUniformBufferObject* h = c->h_ubo + (size_t)slot * c->ubo_cap;
    for (uint32_t i = 0; i < n; i++) h[i] = ubos[i];
    c->ubo_slot = slot;
    return XR_OK;
}
// Records `e` on the context's stream; inside a stream capture it becomes an
// event-record node of the graph (an external event), so the host can still
// wait on it and time with it when the graph is replayed.
}  // namespace

cudaError_t record_event_on(cudaStream_t st, cudaEvent_t e) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t q = cudaStreamIsCapturing(st, &cs);
    if (q != cudaSuccess) return q;
    if (cs == cudaStreamCaptureStatusActive) return cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    return cudaEventRecord(e, st);
}

cudaError_t record_event(Context* c, cudaEvent_t e) { return record_event_on(c->stream, e); }

namespace {

// Stream side: the transfer from the slot staged last (also what a captured frame
// graph replays; the graph of a frame parity reads that parity's slot).
xr_status enqueue_ubos(Context* c, uint32_t n) {
    const uint32_t slot = c->ubo_slot;
    xr_status s = cuda_check(c, cudaMemcpyAsync(c->d_ubo, c->h_ubo + (size_t)slot * c->ubo_cap,
                                                n * sizeof(XrUniformBufferObject), cudaMemcpyHostToDevice, c->stream),
                             "ubo upload");
    if (s) return s;
    return cuda_check(c, record_event(c, c->ubo_ev[slot]), "ubo event");
}

}  // namespace

// Launch-shape tuning of the context into the kernel arguments (0 = the default of each).
void apply_tuning(Context* c) {
    FrameArgs& fa = c->fa;
    fa.sc.refill_min = c->tune_refill;
    fa.sc.postpone_below = c->tune_postpone;
    fa.ray_bundle = c->tune_bundle;
    fa.blk_temporal = c->tune_temporal_block;
    fa.blk_spatial = c->tune_spatial_block;
}

namespace {

xr_status upload_ubo(Context* c, const XrUniformBufferObject* ubo) {
    xr_status s = stage_ubos(c, ubo, 1u);
    if (s) return s;
    return enqueue_ubos(c, 1u);
}

}  // namespace

xr_status check_flags(Context* c) {
    uint32_t flags = 0;
    xr_status s = cuda_check(c, cudaMemcpy(&flags, c->d_counters + kCntError, 4, cudaMemcpyDeviceToHost), "read device flags");
    if (s) return s;
    const uint32_t fresh = flags & ~c->error_flags;
    if (fresh) {
        c->error_flags |= flags;
        std::string m = "device-side check failed:";
        if (flags & XR_DEVFLAG_STACK_OVERFLOW) m += " traversal stack overflow;";
        if (flags & XR_DEVFLAG_QUEUE_OVERFLOW) m += " path queue overflow;";
        if (flags & XR_DEVFLAG_BAD_INDEX) m += " material index out of range;";
        if (flags & XR_DEVFLAG_MMA_TIMEOUT) m += " radiance-cache tensor-core wait timed out;";
        return fail(c, fresh == XR_DEVFLAG_MMA_TIMEOUT ? XR_ERR_TIMEOUT : XR_ERR_OVERFLOW, m);
    }
    return XR_OK;
}

namespace {

xr_status validate_params(const Context* c, const XrParams* p) {
    if (!p) return fail(c, XR_ERR_INVALID_ARGUMENT, "params: null");
    if (p->width == 0 || p->height == 0 || p->width > 16384 || p->height > 16384)
        return fail(c, XR_ERR_INVALID_ARGUMENT, "params: width/height must be in [1, 16384]");
    if (!p->compat_reference) {
        if (p->m_cap_temporal == 0 || p->m_cap_temporal > 255 || p->m_cap_spatial == 0 || p->m_cap_spatial > 255)
            return fail(c, XR_ERR_INVALID_ARGUMENT, "params: M caps must be in [1, 255] (8-bit M in the 32 B reservoir)");
        if (p->n_neighbours > 32) return fail(c, XR_ERR_INVALID_ARGUMENT, "params: n_neighbours must be <= 32");
        if (!(p->radius_px >= 0.0f) || !(p->radius_px <= 4096.0f))
            return fail(c, XR_ERR_INVALID_ARGUMENT, "params: radius_px must be in [0, 4096]");
    }
    return XR_OK;
}

}  // namespace
xr_status realloc_pixels(Context* c) { return alloc_pixels(c); }

}  // namespace xr

using namespace xr;

extern "C" {

uint32_t xr_api_version(void) { return XR_API_VERSION; }

const char* xr_last_error(const XrContext* ctx) {
    if (ctx) return ctx->last_error.c_str();
    std::lock_guard<std::mutex> lk(g_err_mu);
    t_err_copy = g_last_error;
    return t_err_copy.c_str();
}

xr_status xr_create(const XrDeviceDesc* desc, XrContext** out) {
    if (!desc || !out) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "create: null argument");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, XR_ERR_CUDA, std::string("create: no CUDA device (") + cudaGetErrorString(e) + ")");
    if (desc->device < 0 || desc->device >= ndev) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "create: bad device ordinal");
    XrContext* c = new XrContext();
    xr_cache_params_default(&c->cache.params);
    c->device = desc->device;
    DeviceGuard g(c->device);
    xr_status s = XR_OK;
    cudaDeviceProp prop;
    if ((s = cuda_check(c, cudaGetDeviceProperties(&prop, c->device), "device properties"))) goto bad;
    if (prop.major < 10) { s = fail(c, XR_ERR_UNSUPPORTED, "create: this library is built for sm_103a (GB300)"); goto bad; }
    c->sm_count = prop.multiProcessorCount;
    if ((s = cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream"))) goto bad;
    if ((s = cuda_check(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking), "copy stream"))) goto bad;
    if ((s = cuda_check(c, cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking), "side stream"))) goto bad;
    if ((s = cuda_check(c, cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming), "event"))) goto bad;
    if ((s = cuda_check(c, cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming), "event"))) goto bad;
    if ((s = cuda_check(c, cudaEventCreateWithFlags(&c->infer_ev, cudaEventDisableTiming), "event"))) goto bad;
    if ((s = cuda_check(c, cudaEventCreateWithFlags(&c->infer_fork_ev, cudaEventDisableTiming), "event"))) goto bad;
    if ((s = cuda_check(c, cudaEventCreate(&c->ev_train0), "event"))) goto bad;
    if ((s = cuda_check(c, cudaStreamCreateWithFlags(&c->infer_stream, cudaStreamNonBlocking), "inference stream")))
        goto bad;
    for (int i = 0; i < 2; i++) {
        if ((s = cuda_check(c, cudaEventCreateWithFlags(&c->ldr_ready[i], cudaEventDisableTiming), "event"))) goto bad;
        if ((s = cuda_check(c, cudaEventCreateWithFlags(&c->ldr_copied[i], cudaEventDisableTiming), "event"))) goto bad;
    }
    {   // the context's own pool: freed scratch stays cached for the next build instead of going back to the driver
        cudaMemPoolProps pp{};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.handleTypes = cudaMemHandleTypeNone;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = c->device;
        if ((s = cuda_check(c, cudaMemPoolCreate(&c->pool, &pp), "memory pool"))) goto bad;
        uint64_t keep = UINT64_MAX;
        if ((s = cuda_check(c, cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep), "memory pool")))
            goto bad;
    }
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_counters, kCounterWords * 4), "counters"))) goto bad;
    if ((s = cuda_check(c, cudaMemset(c->d_counters, 0, kCounterWords * 4), "counters"))) goto bad;
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_work, 2 * sizeof(unsigned long long)), "work counters"))) goto bad;
    if ((s = cuda_check(c, cudaMemset(c->d_work, 0, 2 * sizeof(unsigned long long)), "work counters"))) goto bad;
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_ubo, sizeof(XrUniformBufferObject)), "ubo"))) goto bad;
    if ((s = cuda_check(c, cudaMallocHost((void**)&c->h_ubo, 2 * sizeof(XrUniformBufferObject)), "ubo staging"))) goto bad;
    for (int i = 0; i < 8; i++)
        if ((s = cuda_check(c, cudaEventCreate(&c->ev[i]), "event"))) goto bad;
    for (int i = 0; i < 8; i++)
        if ((s = cuda_check(c, cudaEventCreate(&c->user_ev[i]), "event"))) goto bad;
    for (int i = 0; i < 2; i++)
        if ((s = cuda_check(c, cudaEventCreate(&c->refit_ev[i]), "event"))) goto bad;
    for (int i = 0; i < 2; i++)
        if ((s = cuda_check(c, cudaEventCreateWithFlags(&c->ubo_ev[i], cudaEventDisableTiming), "event"))) goto bad;
    {
        XrParams p;
        xr_params_default(&p, desc->width ? desc->width : 1, desc->height ? desc->height : 1);
        c->params = p;
        if ((s = alloc_pixels(c))) goto bad;
        c->params_set = desc->width != 0 && desc->height != 0;
    }
    *out = c;
    return XR_OK;
bad:
    xr_destroy(c);
    return s;
}

void xr_destroy(XrContext* c) {
    if (!c) return;
    DeviceGuard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_pixels(c);
    invalidate_graphs(c);
    cudaFree(c->d_views);
    cache_free(c);
    cudaFree(c->d_tri_idx); cudaFree(c->d_vpos); cudaFree(c->d_vnrm); cudaFree(c->d_mats);
    cudaFree(c->d_nodes); cudaFree(c->d_tris); cudaFree(c->d_counters); cudaFree(c->d_ubo); cudaFree(c->d_work);
    cudaFree(c->d_vuv); cudaFree(c->d_tex_info); cudaFree(c->d_texels);
    free_lights(c);
    free_instances(c);
    if (c->h_ubo) cudaFreeHost(c->h_ubo);
    for (int i = 0; i < 8; i++) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i < 8; i++) if (c->user_ev[i]) cudaEventDestroy(c->user_ev[i]);
    for (int i = 0; i < 2; i++) if (c->refit_ev[i]) cudaEventDestroy(c->refit_ev[i]);
    for (int i = 0; i < 2; i++) if (c->ubo_ev[i]) cudaEventDestroy(c->ubo_ev[i]);
    for (int i = 0; i < 2; i++) {
        if (c->ldr_ready[i]) cudaEventDestroy(c->ldr_ready[i]);
        if (c->ldr_copied[i]) cudaEventDestroy(c->ldr_copied[i]);
    }
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->join_ev) cudaEventDestroy(c->join_ev);
    if (c->infer_ev) cudaEventDestroy(c->infer_ev);
    if (c->infer_fork_ev) cudaEventDestroy(c->infer_fork_ev);
    if (c->ev_train0) cudaEventDestroy(c->ev_train0);
    if (c->infer_stream) { cudaStreamSynchronize(c->infer_stream); cudaStreamDestroy(c->infer_stream); }
    if (c->side_stream) { cudaStreamSynchronize(c->side_stream); cudaStreamDestroy(c->side_stream); }
    if (c->stream) cudaStreamSynchronize(c->stream);   // pool frees queued by free_instances
    if (c->pool) cudaMemPoolDestroy(c->pool);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

}  // extern "C"

void xr::free_lights(Context* c) {
    cudaFree(c->d_light_prim); cudaFree(c->d_light_cdf); cudaFree(c->d_light_pmf); cudaFree(c->d_prim_light_pdf);
    c->d_light_prim = nullptr; c->d_light_cdf = nullptr; c->d_light_pmf = nullptr; c->d_prim_light_pdf = nullptr;
    c->n_lights = 0;
}

// Light-sampling tables of the emissive (DiffuseLight) triangles: power =
// area * luminance(4 * base colour) (the emission of shade_step), pmf = power /
// total, inclusive CDF in primitive order with the last entry 1, and per
// primitive pmf / area (the area-measure density of picking a point on it).
xr_status xr::upload_lights(Context* c, const std::vector<uint4>& tri, const std::vector<float4>& pos,
                            const XrMaterial* m, uint32_t nm) {
    std::vector<uint32_t> prim;
    std::vector<float> area, power;
    for (uint32_t i = 0; i < (uint32_t)tri.size(); i++) {
        const uint32_t mi = tri[i].w;
        if (mi >= nm || m[mi].material_model != XR_MAT_DIFFUSE_LIGHT) continue;
        const float4 p0 = pos[tri[i].x], p1 = pos[tri[i].y], p2 = pos[tri[i].z];
        const float e0x = p2.x - p0.x, e0y = p2.y - p0.y, e0z = p2.z - p0.z;
        const float e1x = p1.x - p0.x, e1y = p1.y - p0.y, e1z = p1.z - p0.z;
        const float cx = e0y * e1z - e0z * e1y, cy = e0z * e1x - e0x * e1z, cz = e0x * e1y - e0y * e1x;
        const float a = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
        const float lr = m[mi].base_color[0] * 4.0f, lg = m[mi].base_color[1] * 4.0f, lb = m[mi].base_color[2] * 4.0f;
        const float lum = 0.2126f * lr + 0.7152f * lg + 0.0722f * lb;
        const float pw = a * lum;
        if (!(pw > 0.0f) || !std::isfinite(pw)) continue;
        prim.push_back(i);
        area.push_back(a);
        power.push_back(pw);
    }
    const uint32_t n = (uint32_t)prim.size();
    c->n_lights = n;
    if (n == 0) return XR_OK;
    float total = 0.0f;
    for (float pw : power) total = total + pw;
    std::vector<float> pmf(n), cdf(n), prim_pdf(tri.size(), 0.0f);
    float run = 0.0f;
    for (uint32_t k = 0; k < n; k++) {
        pmf[k] = power[k] / total;
        run = run + pmf[k];
        cdf[k] = run;
        prim_pdf[prim[k]] = pmf[k] / area[k];
    }
    cdf[n - 1] = 1.0f;
    xr_status s;
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_light_prim, (size_t)n * 4), "light tables")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_light_cdf, (size_t)n * 4), "light tables")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_light_pmf, (size_t)n * 4), "light tables")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_prim_light_pdf, tri.size() * 4), "light tables")))
        return s;
    cudaMemcpy(c->d_light_prim, prim.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_light_cdf, cdf.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_light_pmf, pmf.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_prim_light_pdf, prim_pdf.data(), tri.size() * 4, cudaMemcpyHostToDevice);
    return XR_OK;
}

extern "C" {

xr_status xr_upload_textures(XrContext* c, const XrTexture* t, uint32_t n) {
    if (!c || (n && !t)) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload_textures: null argument");
    size_t total = 0;
    std::vector<uint4> info(n);
    for (uint32_t i = 0; i < n; i++) {
        if (!t[i].rgba8 || t[i].width == 0 || t[i].height == 0 || t[i].width > 16384 || t[i].height > 16384)
            return fail(c, XR_ERR_INVALID_ARGUMENT, "upload_textures: each texture needs texels and a size in [1, 16384]");
        info[i] = make_uint4((uint32_t)total, t[i].width, t[i].height, 0u);
        total += (size_t)t[i].width * t[i].height;
        if (total >= (1ull << 32)) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload_textures: more than 2^32 texels");
    }
    DeviceGuard g(c->device);
    cudaStreamSynchronize(c->stream);
    invalidate_graphs(c);
    cudaFree(c->d_tex_info); cudaFree(c->d_texels);
    c->d_tex_info = nullptr; c->d_texels = nullptr; c->n_tex = 0;
    xr_status s;
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_tex_info, std::max<size_t>(n, 1) * 16), "texture alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_texels, std::max<size_t>(total, 1) * 4), "texture alloc")))
        return s;
    if (n) cudaMemcpy(c->d_tex_info, info.data(), (size_t)n * 16, cudaMemcpyHostToDevice);
    for (uint32_t i = 0; i < n; i++)
        cudaMemcpy(c->d_texels + info[i].x, t[i].rgba8, (size_t)t[i].width * t[i].height * 4, cudaMemcpyHostToDevice);
    if ((s = cuda_check(c, cudaGetLastError(), "texture upload"))) return s;
    c->n_tex = n;
    DeviceScene& sc = c->fa.sc;
    sc.tex_info = c->d_tex_info; sc.texels = c->d_texels; sc.n_tex = c->n_tex;
    return XR_OK;
}

xr_status xr_upload_scene(XrContext* c, const XrVertex* v, uint32_t nv, const uint32_t* idx, uint32_t ni,
                          const XrMaterial* m, uint32_t nm, const XrMeshRange* ranges, uint32_t nranges) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "upload: null context");
    if ((nv && !v) || (ni && !idx) || (nm && !m) || (nranges && !ranges))
        return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: null array with non-zero count");
    if (ni % 3 != 0) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: index count must be a multiple of 3");
    DeviceGuard g(c->device);
    std::vector<XrMeshRange> rg;
    if (nranges == 0) rg.push_back({0u, 0u});
    else rg.assign(ranges, ranges + nranges);
    const uint32_t ntri = ni / 3;
    std::vector<uint4> tri(ntri);
    for (size_t r = 0; r < rg.size(); r++) {
        uint32_t b = rg[r].index_offset, e = (r + 1 < rg.size()) ? rg[r + 1].index_offset : ni;
        if (b % 3 || e % 3 || b > e || e > ni) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: bad mesh range index offsets");
        for (uint32_t i = b; i < e; i += 3) {
            uint32_t g0 = rg[r].vertex_offset + idx[i], g1 = rg[r].vertex_offset + idx[i + 1], g2 = rg[r].vertex_offset + idx[i + 2];
            if (g0 >= nv || g1 >= nv || g2 >= nv) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: vertex index out of range");
            int32_t mi = v[g0].material_index;
            if (mi < -1 || mi >= (int32_t)nm) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: material index out of range");
            tri[i / 3] = make_uint4(g0, g1, g2, (uint32_t)mi);
        }
    }
    bool non_lambert = false;
    for (uint32_t i = 0; i < nm; i++) {
        if (m[i].base_color_texture_index >= (int32_t)c->n_tex)
            return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: base-colour texture index out of range (upload the textures first)");
        uint32_t mm = m[i].material_model;
        if (mm != XR_MAT_LAMBERTIAN && mm != XR_MAT_DIFFUSE_LIGHT) non_lambert = true;
        if (mm > XR_MAT_PLASTIC) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: unknown material model");
    }
    std::vector<float4> pos(nv), nrm(nv);
    std::vector<float2> uv(nv);
    for (uint32_t i = 0; i < nv; i++) {
        pos[i] = make_float4(v[i].pos[0], v[i].pos[1], v[i].pos[2], 0.0f);
        nrm[i] = make_float4(v[i].normal[0], v[i].normal[1], v[i].normal[2], 0.0f);
        uv[i] = make_float2(v[i].tex_coord[0], v[i].tex_coord[1]);
        if (!std::isfinite(v[i].pos[0]) || !std::isfinite(v[i].pos[1]) || !std::isfinite(v[i].pos[2]))
            return fail(c, XR_ERR_INVALID_ARGUMENT, "upload: non-finite vertex position");
    }
    cudaStreamSynchronize(c->stream);
    free_instances(c);
    c->parts.clear();
    cudaFree(c->d_tri_idx); cudaFree(c->d_vpos); cudaFree(c->d_vnrm); cudaFree(c->d_mats); cudaFree(c->d_vuv);
    c->d_tri_idx = nullptr; c->d_vpos = nullptr; c->d_vnrm = nullptr; c->d_mats = nullptr; c->d_vuv = nullptr;
    free_lights(c);
    c->scene_ready = false; c->bvh_ready = false;
    for (int k = 0; k < 3; k++) { c->scene_lo[k] = nv ? INFINITY : 0.0f; c->scene_hi[k] = nv ? -INFINITY : 0.0f; }
    for (uint32_t i = 0; i < nv; i++)
        for (int k = 0; k < 3; k++) {
            c->scene_lo[k] = std::min(c->scene_lo[k], v[i].pos[k]);
            c->scene_hi[k] = std::max(c->scene_hi[k], v[i].pos[k]);
        }
    xr_status s;
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_tri_idx, std::max<size_t>(ntri, 1) * 16), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_vpos, std::max<size_t>(nv, 1) * 16), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_vnrm, std::max<size_t>(nv, 1) * 16), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_mats, std::max<size_t>(nm, 1) * sizeof(XrMaterial)), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_vuv, std::max<size_t>(nv, 1) * 8), "scene alloc")))
        return s;
    if (ntri) cudaMemcpy(c->d_tri_idx, tri.data(), (size_t)ntri * 16, cudaMemcpyHostToDevice);
    if (nv) { cudaMemcpy(c->d_vpos, pos.data(), (size_t)nv * 16, cudaMemcpyHostToDevice);
              cudaMemcpy(c->d_vnrm, nrm.data(), (size_t)nv * 16, cudaMemcpyHostToDevice);
              cudaMemcpy(c->d_vuv, uv.data(), (size_t)nv * 8, cudaMemcpyHostToDevice); }
    if (nm) cudaMemcpy(c->d_mats, m, (size_t)nm * sizeof(XrMaterial), cudaMemcpyHostToDevice);
    if ((s = upload_lights(c, tri, pos, m, nm))) return s;
    if ((s = cuda_check(c, cudaGetLastError(), "scene upload"))) return s;
    c->nv = nv; c->ntri = ntri; c->nm = nm;
    c->scene_has_non_lambert = non_lambert;
    cache_scene_bounds(c, reinterpret_cast<const float*>(v), nv);
    invalidate_graphs(c);
    c->scene_roots.clear();   // a single scene, root node 0
    if (c->views.size() > 1) {   // views of a former scene list: back to one view
        c->views.clear();
        if (c->pix_mem && (s = alloc_pixels(c))) return s;
    }
    c->scene_ready = true;
    return XR_OK;
}

xr_status xr_build_bvh(XrContext* c) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "build_bvh: null context");
    if (!c->scene_ready) return fail(c, XR_ERR_STATE, "build_bvh: upload a scene first");
    DeviceGuard g(c->device);
    invalidate_graphs(c);
    xr_status s = build_bvh(c);
    if (s) return s;
    ScenePart part;
    part.nv = c->nv; part.ntri = c->ntri; part.nm = c->nm;
    part.n_nodes = c->n_nodes; part.n_slots = c->n_tri_slots;
    part.levels = c->bvh_levels;
    part.emin = c->bvh_emin;
    for (int k = 0; k < 3; k++) { part.lo[k] = c->scene_lo[k]; part.hi[k] = c->scene_hi[k]; }
    c->parts.assign(1, part);
    DeviceScene& sc = c->fa.sc;
    sc.tri = c->d_tris; sc.nodes = c->d_nodes; sc.n_nodes = c->n_nodes;
    sc.tri_idx = c->d_tri_idx; sc.vpos = c->d_vpos; sc.vnrm = c->d_vnrm;
    sc.mats = c->d_mats; sc.n_mats = c->nm; sc.ntri = c->ntri; sc.n_tri_slots = c->n_tri_slots;
    sc.light_prim = c->d_light_prim; sc.light_cdf = c->d_light_cdf; sc.light_pmf = c->d_light_pmf;
    sc.prim_light_pdf = c->d_prim_light_pdf; sc.n_lights = c->n_lights;
    sc.vuv = c->d_vuv; sc.tex_info = c->d_tex_info; sc.texels = c->d_texels; sc.n_tex = c->n_tex;
    if (!c->instances.empty()) return rebuild_tlas(c);   // the instances now refer to the new BVH
    return XR_OK;
}

xr_status xr_set_params(XrContext* c, const XrParams* p) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "set_params: null context");
    xr_status s = validate_params(c, p);
    if (s) return s;
    DeviceGuard g(c->device);
    const XrParams& o = c->params;
    bool realloc = !c->pix_mem || o.width != p->width || o.height != p->height || o.compat_reference != p->compat_reference ||
                   o.write_pt != p->write_pt || o.write_hdr != p->write_hdr ||
                   (!p->compat_reference && o.n_neighbours != p->n_neighbours);
    if (!c->views.empty()) {   // back to a single view of scene 0
        c->views.clear();
        realloc = true;
    }
    c->params = *p;
    c->params_set = true;
    invalidate_graphs(c);
    if (realloc) {
        cudaStreamSynchronize(c->stream);
        if ((s = alloc_pixels(c))) return s;
    }
    return XR_OK;
}

xr_status xr_get_params(XrContext* c, XrParams* p) {
    if (!c || !p) return fail(c, XR_ERR_INVALID_ARGUMENT, "get_params: null argument");
    *p = c->params;
    return XR_OK;
}

static void* output_ptr(XrContext* c, uint32_t which, size_t* bytes);


// Every stream operation of one frame once its UBOs are staged: the UBO transfer,
// the per-frame counters, the three passes and the timing events.  This is the
// sequence a frame graph captures.
static xr_status enqueue_frame(Context* c, uint32_t n_ubo, uint32_t nb, bool reuse0) {
    xr_status s = enqueue_ubos(c, n_ubo);
    if (s) return s;
    cudaMemsetAsync(c->d_counters, 0, kCntError * 4, c->stream);   // keep the sticky error word
    const bool compat = c->params.compat_reference != 0;
    record_event(c, c->ev[0]);
    launch_initial(c->fa, nb, c->stream, c->fa.cache_on ? cache_after_bounce1 : nullptr, c);
    cache_after_paths(c);   // radiance-cache training; the temporal pass waits for the inference (when enabled)
    record_event(c, c->ev[1]);
    bool temporal_writes_image = compat ? !reuse0 : (c->params.spatial_on == 0u);
    launch_temporal(c->fa, temporal_writes_image, c->stream);
    // The cache's training joins the frame stream here: it runs beside the temporal pass
    // (HBM-bound, while the training waits on latency) but not beside the spatial pass,
    // whose shadow-ray traversal it slows by more than it saves (4 x 4K: 51.5 ms joined
    // before the shadow rays, 49.9 ms joined here).
    if (c->side_pending) {
        cudaEventRecord(c->join_ev, c->side_stream);
        cudaStreamWaitEvent(c->stream, c->join_ev, 0);
        c->side_pending = false;
    }
    record_event(c, c->ev[2]);
    if (compat || c->params.spatial_on) launch_spatial(c->fa, c->stream);
    record_event(c, c->ev[3]);
    return cuda_check(c, cudaGetLastError(), "render launch");
}

// One frame of the context's n views (n = 1 for xr_render_frame).
static xr_status render_impl(Context* c, const XrUniformBufferObject* ubos, uint32_t n, const char* who) {
    NvtxRange nvtx_range("xr frame");
    if (!c->params_set) return fail(c, XR_ERR_STATE, std::string(who) + ": set the parameters (extent) first");
    if (!c->bvh_ready) return fail(c, XR_ERR_STATE, std::string(who) + ": build the BVH first");
    const uint32_t nb = ubos[0].number_of_bounces;
    if (nb > kMaxBounces) return fail(c, XR_ERR_INVALID_ARGUMENT, std::string(who) + ": number_of_bounces must be <= 31");
    for (uint32_t i = 1; i < n; i++)
        if (ubos[i].number_of_bounces != nb || ubos[i].current_frame % 2u != ubos[0].current_frame % 2u ||
            ubos[i].reuse != ubos[0].reuse)
            return fail(c, XR_ERR_INVALID_ARGUMENT,
                        std::string(who) + ": all views of a frame share number_of_bounces, reuse and the frame parity");
    if (c->params.compat_reference && c->scene_has_non_lambert)
        return fail(c, XR_ERR_UNSUPPORTED, std::string(who) + ": reference mode renders only Lambertian and DiffuseLight materials");
    DeviceGuard g(c->device);
    xr_status s = sync_tlas(c);
    if (s) return s;
    if ((s = stage_ubos(c, ubos, n))) return s;
    const uint32_t parity = ubos[0].current_frame % 2u;
    set_frame_pointers(c, parity);
    if ((s = cache_prepare_frame(c, ubos[0].current_frame))) return s;
    const bool reuse0 = ubos[0].reuse != 0u;
    if (c->graphs_on) {
        if (!c->graph[parity] || c->graph_bounces[parity] != (nb | (reuse0 ? 0x100u : 0u))) {
            if (c->graph[parity]) cudaGraphExecDestroy(c->graph[parity]);
            c->graph[parity] = nullptr;
            cudaGraph_t gr = nullptr;
            if ((s = cuda_check(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "frame capture")))
                return s;
            const xr_status e = enqueue_frame(c, n, nb, reuse0);
            const cudaError_t ce = cudaStreamEndCapture(c->stream, &gr);
            if (e) { if (gr) cudaGraphDestroy(gr); return e; }
            if ((s = cuda_check(c, ce, "frame capture end"))) return s;
            s = cuda_check(c, cudaGraphInstantiate(&c->graph[parity], gr, 0), "frame graph instantiate");
            cudaGraphDestroy(gr);
            if (s) return s;
            c->graph_bounces[parity] = nb | (reuse0 ? 0x100u : 0u);
        }
        if ((s = cuda_check(c, cudaGraphLaunch(c->graph[parity], c->stream), "frame graph launch"))) return s;
    } else if ((s = enqueue_frame(c, n, nb, reuse0))) {
        return s;
    }
    if (c->cache.frame_trained) c->cache.step++;   // one Adam step per trained frame (the bias correction advances on the device)
    c->frames++;
    c->last_bounces = nb;
    return XR_OK;
}

xr_status xr_render_frame(XrContext* c, const XrUniformBufferObject* ubo) {
    if (!c || !ubo) return fail(c, XR_ERR_INVALID_ARGUMENT, "render_frame: null argument");
    if (c->fa.n_views > 1u) return fail(c, XR_ERR_STATE, "render_frame: the context has several views (xr_render_views)");
    return render_impl(c, ubo, 1u, "render_frame");
}

xr_status xr_render_views(XrContext* c, const XrUniformBufferObject* ubos) {
    if (!c || !ubos) return fail(c, XR_ERR_INVALID_ARGUMENT, "render_views: null argument");
    return render_impl(c, ubos, c->fa.n_views, "render_views");
}

xr_status xr_set_views(XrContext* c, const XrView* views, uint32_t n, const XrParams* p) {
    if (!c || !views || n == 0 || !p) return fail(c, XR_ERR_INVALID_ARGUMENT, "set_views: bad argument");
    const uint32_t n_scenes = c->scene_roots.empty() ? 1u : (uint32_t)c->scene_roots.size();
    for (uint32_t v = 0; v < n; v++) {
        if (views[v].scene >= n_scenes) return fail(c, XR_ERR_INVALID_ARGUMENT, "set_views: scene index out of range");
        if (views[v].width == 0 || views[v].height == 0 || views[v].width > 16384 || views[v].height > 16384)
            return fail(c, XR_ERR_INVALID_ARGUMENT, "set_views: width/height must be in [1, 16384]");
    }
    XrParams q = *p;
    q.width = views[0].width;
    q.height = views[0].height;
    xr_status s = validate_params(c, &q);
    if (s) return s;
    if (n > 1 && c->cache.params.enabled && n_scenes > 1)
        return fail(c, XR_ERR_UNSUPPORTED, "set_views: the learned cache covers one scene");
    DeviceGuard g(c->device);
    cudaStreamSynchronize(c->stream);
    c->views.assign(views, views + n);
    c->params = q;
    c->params_set = true;
    return alloc_pixels(c);
}

xr_status xr_read_view_output(XrContext* c, uint32_t view, uint32_t which, void* host, size_t bytes) {
    if (!c || !host) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_view_output: null argument");
    if (view >= c->view_info.size()) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_view_output: view out of range");
    size_t all;
    char* src = (char*)output_ptr(c, which, &all);
    if (!src) return fail(c, XR_ERR_STATE, "read_view_output: that image is not enabled (write_hdr / write_pt)");
    const size_t bpp = all / c->N;
    const ViewInfo& vi = c->view_info[view];
    const size_t need = (size_t)vi.W * vi.H * bpp;
    if (bytes < need) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_view_output: host buffer too small");
    DeviceGuard g(c->device);
    xr_status s = cuda_check(c, cudaMemcpyAsync(host, src + (size_t)vi.pix_off * bpp, need, cudaMemcpyDeviceToHost,
                                                c->stream), "read_view_output copy");
    if (s) return s;
    return xr_sync(c);
}

xr_status xr_set_graphs(XrContext* c, int enabled) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "set_graphs: null context");
    DeviceGuard g(c->device);
    c->graphs_on = enabled != 0;
    invalidate_graphs(c);
    return XR_OK;
}

static bool valid_block(uint32_t b) { return b == 0 || b == 32 || b == 64 || b == 128 || b == 256; }

xr_status xr_set_tuning(XrContext* c, const XrTuning* t) {
    if (!c || !t) return fail(c, XR_ERR_INVALID_ARGUMENT, "set_tuning: null argument");
    if (t->trace_ctas_per_sm > 64 || t->shade_ctas_per_sm > 64)
        return fail(c, XR_ERR_INVALID_ARGUMENT, "set_tuning: at most 64 CTAs per SM");
    if (t->refill_min > 32 || t->postpone_below > 32 || t->ray_bundle > 2 || !valid_block(t->temporal_block) ||
        !valid_block(t->spatial_block))
        return fail(c, XR_ERR_INVALID_ARGUMENT,
                    "set_tuning: refill_min / postpone_below <= 32, ray_bundle <= 2, blocks of 32 .. 256 threads");
    DeviceGuard g(c->device);
    c->tune_trace_ctas = t->trace_ctas_per_sm;
    c->tune_shade_ctas = t->shade_ctas_per_sm;
    c->tune_refill = t->refill_min;
    c->tune_postpone = t->postpone_below;
    c->tune_bundle = t->ray_bundle;
    c->tune_temporal_block = t->temporal_block;
    c->tune_spatial_block = t->spatial_block;
    invalidate_graphs(c);
    return XR_OK;
}

// The tuning knobs, one field of XrTuning each, in the order the tuner visits them.
namespace {
struct Knob {
    uint32_t* field;
    std::vector<uint32_t> values;   // the first is the current default
};
}  // namespace

xr_status xr_autotune(XrContext* c, const XrUniformBufferObject* ubos, uint32_t frames, XrTuning* out) {
    if (!c || !ubos || frames == 0) return fail(c, XR_ERR_INVALID_ARGUMENT, "autotune: bad argument");
    DeviceGuard g(c->device);
    const uint32_t n = c->fa.n_views;
    int occ_t = 0, occ_s = 0;
    {
        // the occupancy maxima are what 0 (the default) resolves to
        const uint32_t t0 = trace_grid(c->sm_count, !c->instances.empty()), s0 = persistent_grid(c->sm_count, c->params.compat_reference != 0);
        occ_t = (int)(t0 / (uint32_t)c->sm_count);
        occ_s = (int)(s0 / (uint32_t)c->sm_count);
    }
    auto fractions = [](int occ) {
        std::vector<uint32_t> v{0u};
        for (int x : {occ * 3 / 4, occ / 2})
            if (x >= 1 && x != occ && std::find(v.begin(), v.end(), (uint32_t)x) == v.end()) v.push_back((uint32_t)x);
        return v;
    };
    // coordinate descent: each knob in turn takes the value with the shortest frames, the
    // others held at the best so far (0 = the built-in default of every knob)
    std::vector<Knob> knobs = {
        {&c->tune_trace_ctas, fractions(occ_t)},                       // persistent traversal CTAs per SM
        {&c->tune_shade_ctas, fractions(occ_s)},                       // persistent shading CTAs per SM
        {&c->tune_refill, {0u, 4u, 6u, 12u, 16u}},                     // ray-queue refill: idle lanes per fetch
        {&c->tune_postpone, {0u, 4u, 12u, 16u}},                       // triangle tests postponed below this many lanes
        {&c->tune_bundle, {0u, 1u, 2u}},                               // camera-ray bundle: 8x4, 16x2, 4x8 pixels
        {&c->tune_temporal_block, {0u, 32u, 128u, 256u}},              // temporal pass block (default 64)
        {&c->tune_spatial_block, {0u, 64u, 256u}},                     // spatial passes' block (default 128)
    };
    for (Knob& k : knobs) *k.field = 0u;
    xr_status s = XR_OK;
    uint32_t tried = 0;
    float best = 1e30f, dflt = 0.0f;
    auto time_frames = [&](float* ms) -> xr_status {
        invalidate_graphs(c);
        // one untimed frame (graph capture, caches), then the timed frames
        xr_status e = render_impl(c, ubos, n, "autotune");
        if (e) return e;
        cudaEventRecord(c->user_ev[6], c->stream);
        for (uint32_t f = 0; f < frames && !e; f++) e = render_impl(c, ubos + (size_t)f * n, n, "autotune");
        if (e) return e;
        cudaEventRecord(c->user_ev[7], c->stream);
        if ((e = xr_sync(c))) return e;
        cudaEventElapsedTime(ms, c->user_ev[6], c->user_ev[7]);
        *ms /= (float)frames;
        tried++;
        return XR_OK;
    };
    if ((s = time_frames(&dflt))) return s;
    best = dflt;
    for (Knob& k : knobs) {
        const uint32_t keep = *k.field;
        uint32_t pick = keep;
        for (uint32_t v : k.values) {
            if (v == keep) continue;
            *k.field = v;
            float ms = 0.0f;
            if ((s = time_frames(&ms))) break;
            if (ms < best) { best = ms; pick = v; }
        }
        *k.field = pick;
        if (s) break;
    }
    invalidate_graphs(c);
    if (s) return s;
    if (out) {
        out->trace_ctas_per_sm = c->tune_trace_ctas ? c->tune_trace_ctas : (uint32_t)occ_t;
        out->shade_ctas_per_sm = c->tune_shade_ctas ? c->tune_shade_ctas : (uint32_t)occ_s;
        out->ms_per_frame = best;
        out->ms_default = dflt;
        out->configs_tried = tried;
        out->refill_min = c->tune_refill;
        out->postpone_below = c->tune_postpone;
        out->ray_bundle = c->tune_bundle;
        out->temporal_block = c->tune_temporal_block;
        out->spatial_block = c->tune_spatial_block;
    }
    return XR_OK;
}

// FP64 accumulation of spp samples of the plain path tracer for the n views.
static xr_status render_reference_impl(XrContext* c, const XrUniformBufferObject* ubos, uint32_t n, uint32_t frame0,
                                       uint32_t spp, double* host_rgb, const char* who) {
    if (!c->params_set || !c->bvh_ready) return fail(c, XR_ERR_STATE, std::string(who) + ": parameters and BVH required");
    if (!c->params.write_pt) return fail(c, XR_ERR_STATE, std::string(who) + ": set write_pt in the parameters");
    for (uint32_t i = 0; i < n; i++)
        if (ubos[i].number_of_bounces != ubos[0].number_of_bounces || ubos[i].number_of_bounces > kMaxBounces)
            return fail(c, XR_ERR_INVALID_ARGUMENT, std::string(who) + ": number_of_bounces must be equal and <= 31");
    if (c->params.compat_reference && c->scene_has_non_lambert)
        return fail(c, XR_ERR_UNSUPPORTED, std::string(who) + ": reference mode renders only Lambertian and DiffuseLight materials");
    DeviceGuard g(c->device);
    xr_status s = sync_tlas(c);
    if (s) return s;
    const size_t n3 = (size_t)c->N * 3;
    double* acc = nullptr;
    if ((s = cuda_check(c, cudaMalloc((void**)&acc, n3 * sizeof(double)), "render_reference alloc"))) return s;
    cudaMemsetAsync(acc, 0, n3 * sizeof(double), c->stream);
    std::vector<XrUniformBufferObject> u(ubos, ubos + n);
    for (uint32_t k = 0; k < spp && !s; k++) {
        for (auto& x : u) x.current_frame = frame0 + k;
        if ((s = stage_ubos(c, u.data(), n)) || (s = enqueue_ubos(c, n))) break;
        set_frame_pointers(c, u[0].current_frame % 2u);
        c->fa.cache_on = 0;   // the converged reference is the plain path tracer
        c->fa.cache_sel = nullptr;
        c->cache.frame_used = false;
        cudaMemsetAsync(c->d_counters, 0, kCntError * 4, c->stream);
        launch_initial(c->fa, u[0].number_of_bounces, c->stream);
        launch_accumulate_sample(c->fa, acc, c->stream);
        s = cuda_check(c, cudaGetLastError(), "render_reference launch");
    }
    if (!s) s = cuda_check(c, cudaMemcpyAsync(host_rgb, acc, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                           "render_reference copy");
    if (!s) s = xr_sync(c);
    cudaFree(acc);
    if (s) return s;
    for (size_t i = 0; i < n3; i++) host_rgb[i] /= (double)spp;
    return XR_OK;
}

xr_status xr_render_reference(XrContext* c, const XrUniformBufferObject* ubo, uint32_t frame0, uint32_t spp,
                              double* host_rgb) {
    if (!c || !ubo || !host_rgb || spp == 0) return fail(c, XR_ERR_INVALID_ARGUMENT, "render_reference: bad argument");
    if (c->fa.n_views > 1u) return fail(c, XR_ERR_STATE, "render_reference: the context has several views");
    return render_reference_impl(c, ubo, 1u, frame0, spp, host_rgb, "render_reference");
}

xr_status xr_render_reference_views(XrContext* c, const XrUniformBufferObject* ubos, uint32_t frame0, uint32_t spp,
                                    double* host_rgb) {
    if (!c || !ubos || !host_rgb || spp == 0) return fail(c, XR_ERR_INVALID_ARGUMENT, "render_reference_views: bad argument");
    return render_reference_impl(c, ubos, c->fa.n_views, frame0, spp, host_rgb, "render_reference_views");
}

xr_status xr_sync(XrContext* c) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "sync: null context");
    DeviceGuard g(c->device);
    xr_status s = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
    if (s) return s;
    if (c->copy_stream && (s = cuda_check(c, cudaStreamSynchronize(c->copy_stream), "sync (image reads)"))) return s;
    return check_flags(c);
}

static void* output_ptr(XrContext* c, uint32_t which, size_t* bytes) {
    const size_t N = c->N;
    switch (which) {
        case XR_OUT_LDR8: *bytes = N * 4; return c->fa.out_ldr;
        case XR_OUT_HDR: *bytes = N * 16; return c->fa.out_hdr;
        case XR_OUT_PT: *bytes = N * 16; return c->fa.out_pt;
        default: *bytes = 0; return nullptr;
    }
}

xr_status xr_read_output(XrContext* c, uint32_t which, void* host, size_t bytes) {
    if (!c || !host) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_output: null argument");
    size_t need;
    void* src = output_ptr(c, which, &need);
    if (!src) return fail(c, XR_ERR_STATE, "read_output: that image is not enabled (write_hdr / write_pt)");
    if (bytes < need) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_output: host buffer too small");
    DeviceGuard g(c->device);
    xr_status s = cuda_check(c, cudaMemcpyAsync(host, src, need, cudaMemcpyDeviceToHost, c->stream), "read_output copy");
    if (s) return s;
    return xr_sync(c);
}

xr_status xr_read_output_async(XrContext* c, void* host, size_t bytes) {
    if (!c || !host) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_output_async: null argument");
    const size_t need = (size_t)c->N * 4;
    if (bytes < need) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_output_async: host buffer too small");
    if (!c->frames) return fail(c, XR_ERR_STATE, "read_output_async: no frame rendered yet");
    if (c->ldr_nreads == 2u)
        return fail(c, XR_ERR_STATE, "read_output_async: two reads in flight already (call xr_wait_output)");
    DeviceGuard g(c->device);
    const uint32_t p = c->fa.parity;   // the buffer the last frame wrote
    xr_status s = cuda_check(c, cudaEventRecord(c->ldr_ready[p], c->stream), "read_output_async event");
    if (!s) s = cuda_check(c, cudaStreamWaitEvent(c->copy_stream, c->ldr_ready[p], 0), "read_output_async wait");
    if (!s) s = cuda_check(c, cudaMemcpyAsync(host, c->ldr[p], need, cudaMemcpyDeviceToHost, c->copy_stream),
                           "read_output_async copy");
    if (!s) s = cuda_check(c, cudaEventRecord(c->ldr_copied[p], c->copy_stream), "read_output_async event");
    if (s) return s;
    c->ldr_copy_pending[p] = true;
    c->ldr_reads[c->ldr_nreads++] = p;
    return XR_OK;
}

xr_status xr_wait_output(XrContext* c) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "wait_output: null context");
    if (c->ldr_nreads == 0u) return XR_OK;
    DeviceGuard g(c->device);
    const xr_status s = cuda_check(c, cudaEventSynchronize(c->ldr_copied[c->ldr_reads[0]]), "wait_output");
    c->ldr_reads[0] = c->ldr_reads[1];
    c->ldr_nreads--;
    return s;
}

xr_status xr_output_device_ptr(XrContext* c, uint32_t which, void** dptr) {
    if (!c || !dptr) return fail(c, XR_ERR_INVALID_ARGUMENT, "output_device_ptr: null argument");
    size_t need;
    *dptr = output_ptr(c, which, &need);
    if (!*dptr) return fail(c, XR_ERR_STATE, "output_device_ptr: that image is not enabled");
    return XR_OK;
}

xr_status xr_get_stats(XrContext* c, XrStats* st) {
    if (!c || !st) return fail(c, XR_ERR_INVALID_ARGUMENT, "get_stats: null argument");
    DeviceGuard g(c->device);
    xr_status s = sync_tlas(c);
    if (!s) s = xr_sync(c);
    if (!s && c->refit_timed) {
        cudaEventElapsedTime(&c->ms_refit, c->refit_ev[0], c->refit_ev[1]);
        c->refit_timed = false;
    }
    XrStats o;
    memset(&o, 0, sizeof(o));
    o.frames = c->frames;
    o.error_flags = c->error_flags;
    if (c->frames) {
        cudaEventElapsedTime(&o.ms_initial, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&o.ms_temporal, c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&o.ms_spatial, c->ev[2], c->ev[3]);
        cudaEventElapsedTime(&o.ms_frame, c->ev[0], c->ev[3]);
        uint32_t cnt[kCounterWords];
        cudaMemcpy(cnt, c->d_counters, sizeof(cnt), cudaMemcpyDeviceToHost);
        o.rays_traced = 0;
        for (uint32_t b = 0; b < c->last_bounces && b <= kMaxBounces; b++) o.rays_traced += cnt[b];
        o.shadow_rays = cnt[kCntShadow];
        o.nonfinite_rays = cnt[kCntNonFinite];
    }
    o.bvh_nodes = c->n_nodes; o.bvh_triangles = c->n_tri_slots; o.bvh_depth = c->bvh_depth;
    o.ms_bvh_build = c->ms_bvh;
    o.instances = (uint32_t)c->instances.size();
    o.tlas_nodes = c->n_tlas_nodes;
    o.ms_tlas_build = c->ms_tlas;
    o.ms_refit = c->ms_refit;
    if (c->query_rays) {
        unsigned long long w[2] = {0, 0};
        cudaMemcpy(w, c->d_work, sizeof(w), cudaMemcpyDeviceToHost);
        o.query_rays = c->query_rays;
        o.query_node_visits = w[0];
        o.query_tri_tests = w[1];
    }
    *st = o;
    return s;
}

xr_status xr_read_buffer(XrContext* c, uint32_t which, void* host, size_t bytes, size_t* bytes_out) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "read_buffer: null context");
    const size_t N = c->N;
    const bool compat = c->params.compat_reference != 0;
    size_t need;
    switch (which) {
        case XR_BUF_SAMPLES: need = N * 96; break;
        case XR_BUF_TEMPORAL: need = 2 * N * 112; break;
        case XR_BUF_SPATIAL: need = (compat ? 2 * N : N) * 112; break;
        default: return fail(c, XR_ERR_INVALID_ARGUMENT, "read_buffer: unknown buffer");
    }
    if (bytes_out) *bytes_out = need;
    if (!host) return XR_OK;
    if (bytes < need) return fail(c, XR_ERR_INVALID_ARGUMENT, "read_buffer: host buffer too small");
    DeviceGuard g(c->device);
    uint32_t* tmp = nullptr;
    xr_status s = cuda_check(c, cudaMalloc((void**)&tmp, need), "read_buffer alloc");
    if (s) return s;
    set_frame_pointers(c, c->fa.parity);
    if (which == XR_BUF_SAMPLES) {
        launch_export_samples(c->fa, tmp, c->stream);
    } else if (compat) {
        launch_export_res_wide(which == XR_BUF_TEMPORAL ? c->fa.rw : c->fa.rsw, (uint32_t)(2 * N), tmp, c->stream);
    } else if (which == XR_BUF_TEMPORAL) {
        launch_export_res_packed(c->rt0[0], c->rt1[0], (uint32_t)N, tmp, c->stream);
        launch_export_res_packed(c->rt0[1], c->rt1[1], (uint32_t)N, tmp + 28 * N, c->stream);
    } else {
        launch_export_res_packed(c->fa.rs0, c->fa.rs1, (uint32_t)N, tmp, c->stream);
    }
    s = cuda_check(c, cudaMemcpyAsync(host, tmp, need, cudaMemcpyDeviceToHost, c->stream), "read_buffer copy");
    if (!s) s = cuda_check(c, cudaStreamSynchronize(c->stream), "read_buffer sync");
    cudaFree(tmp);
    return s;
}

xr_status xr_write_buffer(XrContext* c, uint32_t which, const void* host, size_t bytes) {
    if (!c || !host) return fail(c, XR_ERR_INVALID_ARGUMENT, "write_buffer: null argument");
    const size_t N = c->N;
    const bool compat = c->params.compat_reference != 0;
    size_t need;
    switch (which) {
        case XR_BUF_SAMPLES: need = N * 96; break;
        case XR_BUF_TEMPORAL: need = 2 * N * 112; break;
        default: return fail(c, XR_ERR_INVALID_ARGUMENT, "write_buffer: only samples and temporal reservoirs can be written");
    }
    if (bytes != need) return fail(c, XR_ERR_INVALID_ARGUMENT, "write_buffer: size mismatch");
    DeviceGuard g(c->device);
    uint32_t* tmp = nullptr;
    xr_status s = cuda_check(c, cudaMalloc((void**)&tmp, need), "write_buffer alloc");
    if (s) return s;
    s = cuda_check(c, cudaMemcpyAsync(tmp, host, need, cudaMemcpyHostToDevice, c->stream), "write_buffer copy");
    if (!s) {
        set_frame_pointers(c, c->fa.parity);
        if (which == XR_BUF_SAMPLES) {
            launch_import_samples(c->fa, tmp, c->stream);
        } else if (compat) {
            launch_import_res_wide(c->fa.rw, (uint32_t)(2 * N), tmp, c->stream);
        } else {
            launch_import_res_packed(c->rt0[0], c->rt1[0], (uint32_t)N, tmp, c->stream);
            launch_import_res_packed(c->rt0[1], c->rt1[1], (uint32_t)N, tmp + 28 * N, c->stream);
        }
        s = cuda_check(c, cudaStreamSynchronize(c->stream), "write_buffer sync");
    }
    cudaFree(tmp);
    return s;
}

xr_status xr_run_pass(XrContext* c, const XrUniformBufferObject* ubo, uint32_t pass) {
    if (!c || !ubo) return fail(c, XR_ERR_INVALID_ARGUMENT, "run_pass: null argument");
    if (pass != 1 && pass != 2) return fail(c, XR_ERR_INVALID_ARGUMENT, "run_pass: pass must be 1 (temporal) or 2 (spatial)");
    if (!c->params_set || !c->bvh_ready) return fail(c, XR_ERR_STATE, "run_pass: parameters and BVH required");
    DeviceGuard g(c->device);
    xr_status s = sync_tlas(c);
    if (s) return s;
    if ((s = upload_ubo(c, ubo))) return s;
    set_frame_pointers(c, ubo->current_frame % 2u);
    const bool compat = c->params.compat_reference != 0;
    if (pass == 1 && !compat && c->params.temporal_on) launch_reproject(c->fa, c->stream);
    if (pass == 1) launch_temporal(c->fa, compat ? (ubo->reuse == 0u) : (c->params.spatial_on == 0u), c->stream);
    else launch_spatial(c->fa, c->stream);
    s = cuda_check(c, cudaGetLastError(), "run_pass launch");
    if (s) return s;
    return xr_sync(c);
}

static xr_status trace_device(XrContext* c, const float* d_rays, uint32_t n, int32_t any_hit, int32_t* d_prim,
                              int32_t* d_inst, float* d_t, float* d_bary) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "trace: null context");
    if (!c->bvh_ready) return fail(c, XR_ERR_STATE, "trace: build the BVH first");
    if (n && (!d_rays || !d_prim || !d_t || !d_bary)) return fail(c, XR_ERR_INVALID_ARGUMENT, "trace: null array");
    DeviceGuard g(c->device);
    if (xr_status s0 = sync_tlas(c)) return s0;
    apply_tuning(c);
    cudaMemsetAsync(c->d_counters + kCntFetchQuery, 0, 4, c->stream);
    cudaMemsetAsync(c->d_work, 0, 2 * sizeof(unsigned long long), c->stream);
    c->query_rays = n;
    launch_trace(c->fa.sc, d_rays, n, any_hit, d_prim, d_inst, d_t, d_bary, c->d_counters + kCntFetchQuery,
                 c->d_counters + kCntError, c->d_work, c->sm_count, c->stream);
    return cuda_check(c, cudaGetLastError(), "trace launch");
}

xr_status xr_trace_rays_device(XrContext* c, const float* d_rays, uint32_t n, int32_t any_hit, int32_t* d_prim,
                               float* d_t, float* d_bary) {
    return trace_device(c, d_rays, n, any_hit, d_prim, nullptr, d_t, d_bary);
}

static xr_status trace_host(XrContext* c, const float* rays, uint32_t n, int32_t any_hit, int32_t* prim,
                            int32_t* inst, float* t, float* bary) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "trace: null context");
    if (n == 0) return XR_OK;
    if (!rays || !prim || !t || !bary) return fail(c, XR_ERR_INVALID_ARGUMENT, "trace: null array");
    DeviceGuard g(c->device);
    float* dr = nullptr; int32_t* dp = nullptr; int32_t* di = nullptr; float* dt = nullptr; float* db = nullptr;
    xr_status s = XR_OK;
    if ((s = cuda_check(c, cudaMalloc((void**)&dr, (size_t)n * 32), "trace alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&dp, (size_t)n * 4), "trace alloc")) ||
        (inst && (s = cuda_check(c, cudaMalloc((void**)&di, (size_t)n * 4), "trace alloc"))) ||
        (s = cuda_check(c, cudaMalloc((void**)&dt, (size_t)n * 4), "trace alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&db, (size_t)n * 8), "trace alloc")))
        goto out;
    cudaMemcpyAsync(dr, rays, (size_t)n * 32, cudaMemcpyHostToDevice, c->stream);
    if ((s = trace_device(c, dr, n, any_hit, dp, di, dt, db))) goto out;
    cudaMemcpyAsync(prim, dp, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (inst) cudaMemcpyAsync(inst, di, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(t, dt, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(bary, db, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream);
    s = xr_sync(c);
out:
    cudaFree(dr); cudaFree(dp); cudaFree(di); cudaFree(dt); cudaFree(db);
    return s;
}

xr_status xr_trace_rays(XrContext* c, const float* rays, uint32_t n, int32_t any_hit, int32_t* prim, float* t,
                        float* bary) {
    return trace_host(c, rays, n, any_hit, prim, nullptr, t, bary);
}

xr_status xr_trace_rays_instanced(XrContext* c, const float* rays, uint32_t n, int32_t any_hit, int32_t* prim,
                                  int32_t* instance, float* t, float* bary) {
    if (c && n && !instance) return fail(c, XR_ERR_INVALID_ARGUMENT, "trace: null instance array");
    return trace_host(c, rays, n, any_hit, prim, instance, t, bary);
}

xr_status xr_event_record(XrContext* c, uint32_t slot) {
    if (!c || slot >= 8) return fail(c, XR_ERR_INVALID_ARGUMENT, "event_record: bad argument");
    DeviceGuard g(c->device);
    return cuda_check(c, cudaEventRecord(c->user_ev[slot], c->stream), "event_record");
}

xr_status xr_event_elapsed(XrContext* c, uint32_t a, uint32_t b, float* ms) {
    if (!c || a >= 8 || b >= 8 || !ms) return fail(c, XR_ERR_INVALID_ARGUMENT, "event_elapsed: bad argument");
    DeviceGuard g(c->device);
    xr_status s = cuda_check(c, cudaEventSynchronize(c->user_ev[b]), "event_elapsed sync");
    if (s) return s;
    return cuda_check(c, cudaEventElapsedTime(ms, c->user_ev[a], c->user_ev[b]), "event_elapsed");
}

xr_status xr_alloc_host(size_t bytes, void** ptr) {
    if (!ptr) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "alloc_host: null argument");
    return cuda_check(nullptr, cudaMallocHost(ptr, bytes), "cudaMallocHost");
}

void xr_free_host(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
}

}  // extern "C"
