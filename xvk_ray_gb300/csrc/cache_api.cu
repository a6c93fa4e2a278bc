// cache_api.cu -- C ABI of the learned radiance cache (include/xr.h) and its
// place in the frame: after the wavefront bounce loop, one inference launch adds
// the cache's radiance to every query's candidate, then one training launch and
// one Adam step consume the frame's training records, all stream-ordered before
// the temporal pass.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "nrc.cuh"
#include "xr_internal.h"

namespace xr {

namespace {

constexpr uint32_t kMaxApiSamples = 1u << 20;
constexpr uint32_t kMaxTrainSamples = 1u << 20;

size_t array_floats(int which) {
    switch (which) {
        case XR_CACHE_MLP: case XR_CACHE_MLP_GRAD: case XR_CACHE_MLP_M: case XR_CACHE_MLP_V:
            return (size_t)nrc::kMlpParams;
        case XR_CACHE_GRID: case XR_CACHE_GRID_GRAD: case XR_CACHE_GRID_M: case XR_CACHE_GRID_V:
            return nrc::kGridParams;
        default:
            return 0;
    }
}

float* array_ptr(CacheState& cs, int which) {
    switch (which) {
        case XR_CACHE_MLP: return cs.mlp;
        case XR_CACHE_GRID: return cs.grid;
        case XR_CACHE_MLP_GRAD: return cs.mlp_grad;
        case XR_CACHE_GRID_GRAD: return cs.grid_grad;
        case XR_CACHE_MLP_M: return cs.mlp_m;
        case XR_CACHE_MLP_V: return cs.mlp_v;
        case XR_CACHE_GRID_M: return cs.grid_m;
        case XR_CACHE_GRID_V: return cs.grid_v;
        default: return nullptr;
    }
}

// Host-side initial MLP weights: U(-a, a) with a = sqrt(6 / (fan_in + fan_out))
// (Glorot and Bengio 2010) from a counter-based hash; unused outputs 3..15 zero.
void init_mlp(std::vector<float>& w, uint32_t seed) {
    w.assign(nrc::kMlpParams, 0.0f);
    for (int l = 0; l <= nrc::kHidden; ++l) {
        const int rows = l < nrc::kHidden ? nrc::kWidth : nrc::kOut;
        const float a = sqrtf(6.0f / (float)(nrc::kIn + rows));
        for (int o = 0; o < rows; ++o)
            for (int i = 0; i < nrc::kIn; ++i) {
                const uint32_t idx = (uint32_t)(l * nrc::kWidth * nrc::kIn + o * nrc::kIn + i);
                w[idx] = (l == nrc::kHidden && o >= 3) ? 0.0f : (nrc::init_u01(idx, seed, 2u) * 2.0f - 1.0f) * a;
            }
    }
}

xr_status cache_init(Context* c, uint32_t seed) {
    CacheState& cs = c->cache;
    std::vector<float> w;
    init_mlp(w, seed);
    xr_status s = cuda_check(c, cudaMemcpyAsync(cs.mlp, w.data(), w.size() * 4, cudaMemcpyHostToDevice, c->stream),
                             "cache init");
    if (s) return s;
    cudaMemsetAsync(cs.mlp_grad, 0, (size_t)nrc::kMlpParams * 4, c->stream);
    cudaMemsetAsync(cs.mlp_m, 0, (size_t)nrc::kMlpParams * 4, c->stream);
    cudaMemsetAsync(cs.mlp_v, 0, (size_t)nrc::kMlpParams * 4, c->stream);
    cudaMemsetAsync(cs.grid_grad, 0, nrc::kGridParams * 4, c->stream);
    cudaMemsetAsync(cs.grid_m, 0, nrc::kGridParams * 4, c->stream);
    cudaMemsetAsync(cs.grid_v, 0, nrc::kGridParams * 4, c->stream);
    cs.step = 0;
    cs.grads_dirty = false;
    cs.sel_target = 0;   // the next frame selects `target` training pixels again
    launch_cache_init(cs, seed, c->stream);
    launch_cache_adam_reset(cs, c->stream);
    s = cuda_check(c, cudaGetLastError(), "cache init launch");
    if (s) return s;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "cache init");
}

xr_status cache_alloc(Context* c) {
    CacheState& cs = c->cache;
    if (cs.allocated) return XR_OK;
    xr_status s = cuda_check(c, cache_configure_kernels(), "cache kernel attributes");
    if (s) return s;
    const size_t mb = (size_t)nrc::kMlpParams * 4, gb = nrc::kGridParams * 4;
    float** mlp_arrays[] = {&cs.mlp, &cs.mlp_grad, &cs.mlp_m, &cs.mlp_v};
    for (float** p : mlp_arrays)
        if ((s = cuda_check(c, cudaMalloc((void**)p, mb), "cache alloc"))) return s;
    float** grid_arrays[] = {&cs.grid, &cs.grid_grad, &cs.grid_m, &cs.grid_v};
    for (float** p : grid_arrays)
        if ((s = cuda_check(c, cudaMalloc((void**)p, gb), "cache alloc"))) return s;
    if ((s = cuda_check(c, cudaMalloc((void**)&cs.table, nrc::kGridParams * 2), "cache alloc"))) return s;
    if ((s = cuda_check(c, cudaMalloc((void**)&cs.w_fwd, nrc::kImageBytes), "cache alloc"))) return s;
    if ((s = cuda_check(c, cudaMalloc((void**)&cs.w_bwd, nrc::kImageBytes), "cache alloc"))) return s;
    if ((s = cuda_check(c, cudaMalloc((void**)&cs.loss, sizeof(float)), "cache alloc"))) return s;
    if ((s = cuda_check(c, cudaMalloc((void**)&cs.adam, 4 * sizeof(float)), "cache alloc"))) return s;
    if ((s = cuda_check(c, cudaMalloc((void**)&cs.sel, sizeof(uint32_t)), "cache alloc"))) return s;
    if ((s = cuda_check(c, cudaMalloc((void**)&cs.order_hist, 256 * 128 * sizeof(uint32_t)), "cache alloc"))) return s;
    cs.sel_target = 0;
    cs.allocated = true;
    return cache_init(c, cs.params.seed);
}

xr_status ensure_records(Context* c, uint32_t queries, uint32_t train) {
    CacheState& cs = c->cache;
    xr_status s;
    if (queries > cs.query_cap) {
        cudaFree(cs.queries);
        cs.queries = nullptr;
        cs.query_cap = 0;
        if ((s = cuda_check(c, cudaMalloc((void**)&cs.queries, (size_t)queries * 32), "cache query records"))) return s;
        cs.query_cap = queries;
    }
    if (train > cs.train_cap) {
        cudaFree(cs.train);
        cudaFree(cs.tiles);
        cudaFree(cs.order);
        cudaFree(cs.nee);
        cs.train = nullptr;
        cs.tiles = nullptr;
        cs.order = nullptr;
        cs.nee = nullptr;
        cs.train_cap = 0;
        if ((s = cuda_check(c, cudaMalloc((void**)&cs.train, (size_t)train * 48), "cache training records"))) return s;
        if ((s = cuda_check(c, cudaMalloc((void**)&cs.tiles, (size_t)train * 128), "cache training tiles"))) return s;
        if ((s = cuda_check(c, cudaMalloc((void**)&cs.order, (size_t)train * 32), "cache training order"))) return s;
        if ((s = cuda_check(c, cudaMalloc((void**)&cs.nee, (size_t)train * 48), "cache next-event rays"))) return s;
        cs.train_cap = train;
    }
    return XR_OK;
}

xr_status validate(const Context* c, const XrCacheParams* p) {
    if (!p) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache params: null");
    if (p->train_samples > kMaxTrainSamples)
        return fail(c, XR_ERR_INVALID_ARGUMENT, "cache params: train_samples must be <= 1048576");
    // epsilon > 0: a weight whose gradient and moments are zero would otherwise step by 0 / 0
    if (!(p->learning_rate > 0.0f) || !(p->beta1 >= 0.0f && p->beta1 < 1.0f) || !(p->beta2 >= 0.0f && p->beta2 < 1.0f) ||
        !(p->epsilon > 0.0f))
        return fail(c, XR_ERR_INVALID_ARGUMENT, "cache params: learning_rate > 0, 0 <= beta < 1, epsilon > 0");
    return XR_OK;
}

// Uploads API samples and packs them into records (stride 2: query, 3: training).
xr_status upload_samples(Context* c, const XrCacheSample* s, uint32_t n, uint32_t stride, uint4* rec) {
    XrCacheSample* d = nullptr;
    xr_status st = cuda_check(c, cudaMalloc((void**)&d, (size_t)n * sizeof(XrCacheSample)), "cache samples");
    if (st) return st;
    st = cuda_check(c, cudaMemcpyAsync(d, s, (size_t)n * sizeof(XrCacheSample), cudaMemcpyHostToDevice, c->stream),
                    "cache samples upload");
    if (!st) launch_cache_pack(d, n, rec, stride, c->stream);
    if (!st) st = cuda_check(c, cudaStreamSynchronize(c->stream), "cache pack");
    cudaFree(d);
    return st;
}

}  // namespace

void cache_free(Context* c) {
    CacheState& cs = c->cache;
    void* ptrs[] = {cs.mlp, cs.mlp_grad, cs.mlp_m, cs.mlp_v, cs.grid, cs.grid_grad, cs.grid_m, cs.grid_v,
                    cs.table, cs.w_fwd, cs.w_bwd, cs.loss, cs.adam, cs.queries, cs.train, cs.tiles, cs.order,
                    cs.order_hist, cs.nee, cs.sel};
    for (void* p : ptrs) cudaFree(p);
    cs = CacheState{};
}

// Scene cube of the hash encoding: the vertices' bounding box, grown by 1% of
// its largest side on every face; unit position = (x - lo) * inv_extent.
void cache_scene_bounds(Context* c, const float* xyz9, uint32_t nv) {
    CacheState& cs = c->cache;
    if (nv == 0) return;
    float lo[3] = {xyz9[0], xyz9[1], xyz9[2]}, hi[3] = {xyz9[0], xyz9[1], xyz9[2]};
    for (uint32_t i = 1; i < nv; ++i)
        for (int a = 0; a < 3; ++a) {
            const float v = xyz9[(size_t)i * 9 + a];
            lo[a] = std::fmin(lo[a], v);
            hi[a] = std::fmax(hi[a], v);
        }
    float ext = std::fmax(hi[0] - lo[0], std::fmax(hi[1] - lo[1], hi[2] - lo[2]));
    if (!(ext > 0.0f)) ext = 1.0f;
    const float pad = 0.01f * ext;
    for (int a = 0; a < 3; ++a) cs.lo[a] = lo[a] - pad;
    cs.inv_ext = 1.0f / (ext + 2.0f * pad);
}

xr_status cache_prepare_frame(Context* c, uint32_t frame) {
    CacheState& cs = c->cache;
    FrameArgs& fa = c->fa;
    fa.cache_on = 0;
    fa.cache_sel = nullptr;
    cs.frame_used = false;
    cs.frame_trained = false;
    if (!cs.params.enabled) return XR_OK;
    if (c->params.compat_reference)
        return fail(c, XR_ERR_UNSUPPORTED, "render_frame: the radiance cache runs in corrected mode only");
    xr_status s = cache_alloc(c);
    if (s) return s;
    // the training records of a frame: about `target` (adaptive selection), at most one per pixel
    const uint32_t target = cs.params.train ? (cs.params.train_samples < c->N ? cs.params.train_samples : c->N) : 0u;
    const uint32_t tcap = target ? c->N : 0u;
    if ((s = ensure_records(c, c->N, tcap > 0 ? tcap : 1u))) return s;
    if (target && (cs.sel_target != target || cs.sel_pixels != c->N)) {   // new target or extent: select `target`
        launch_cache_select_next(cs.sel, nullptr, target, c->N, target, c->stream);
        cs.sel_target = target;
        cs.sel_pixels = c->N;
    }
    if (cs.grads_dirty) {
        cudaMemsetAsync(cs.mlp_grad, 0, (size_t)nrc::kMlpParams * 4, c->stream);
        cudaMemsetAsync(cs.grid_grad, 0, nrc::kGridParams * 4, c->stream);
        cs.grads_dirty = false;
    }
    fa.cache_on = 1;
    fa.cache_q = cs.queries;
    fa.cache_t = cs.train;
    fa.cache_nee = cs.nee;
    fa.cache_t_cap = tcap;
    fa.cache_sel = target ? cs.sel : nullptr;
    (void)frame;
    cs.frame_used = true;
    cs.frame_trained = tcap > 0;
    return XR_OK;
}

// Once bounce 1's shading is enqueued the frame's query records are complete: the
// inference runs on the inference stream beside the rest of the bounce loop, which
// from bounce 2 on traces only the training paths and writes only their records
// (no candidate, no query).
void cache_after_bounce1(void* ctx) {
    Context* c = static_cast<Context*>(ctx);
    CacheState& cs = c->cache;
    if (!c->fa.cache_on) return;
    cudaEventRecord(c->infer_fork_ev, c->stream);
    cudaStreamWaitEvent(c->infer_stream, c->infer_fork_ev, 0);
    if (cs.frame_trained) {
        // the training's first stage needs only bounce 1's record words (not the targets
        // the later bounces accumulate): it runs beside them on the side stream too
        cudaStreamWaitEvent(c->side_stream, c->infer_fork_ev, 0);
        record_event_on(c->side_stream, c->ev_train0);
        launch_cache_encode_stage(cs, cs.train, c->d_counters + kCntCacheTrain, 0u, c->fa.cache_t_cap, c->sm_count,
                                  c->side_stream);
        c->side_pending = true;
    }
    record_event_on(c->infer_stream, c->ev[6]);
    launch_cache_infer(cs, cs.queries, c->d_counters + kCntCacheQuery, 0u, nullptr, c->fa.cand_b,
                       c->d_counters + kCntError, c->sm_count, c->infer_stream);
    record_event_on(c->infer_stream, c->ev[7]);
    cudaEventRecord(c->infer_ev, c->infer_stream);
    c->infer_pending = true;
}

// After the bounce loop: the training's second stage (gradients, then Adam once
// the inference, which reads the table and weights Adam overwrites, is done) on
// the side stream, which the frame stream joins after the temporal pass
// (enqueue_frame); the frame stream waits for the inference before that pass.
void cache_after_paths(Context* c) {
    CacheState& cs = c->cache;
    if (!c->fa.cache_on) return;
    uint32_t* err = c->d_counters + kCntError;
    if (cs.frame_trained) {
        if (!c->side_pending) {   // no bounce 1 (a single-bounce frame): the first stage runs here
            cudaEventRecord(c->fork_ev, c->stream);
            cudaStreamWaitEvent(c->side_stream, c->fork_ev, 0);
            record_event_on(c->side_stream, c->ev_train0);
            launch_cache_encode_stage(cs, cs.train, c->d_counters + kCntCacheTrain, 0u, c->fa.cache_t_cap,
                                      c->sm_count, c->side_stream);
        }
        // the second stage reads the records' targets: after the whole bounce loop
        cudaEventRecord(c->fork_ev, c->stream);
        cudaStreamWaitEvent(c->side_stream, c->fork_ev, 0);
        launch_cache_grad_stage(cs, cs.train, c->d_counters + kCntCacheTrain, 0u, c->fa.cache_t_cap, err, c->sm_count,
                                c->side_stream);
        launch_cache_select_next(cs.sel, c->d_counters + kCntCacheTrain, cs.sel_target, c->N, 0u, c->side_stream);
        if (c->infer_pending) cudaStreamWaitEvent(c->side_stream, c->infer_ev, 0);
        launch_cache_adam(cs, c->side_stream);
        record_event_on(c->side_stream, c->ev[4]);
        c->side_pending = true;
    } else {
        record_event(c, c->ev_train0);
        record_event(c, c->ev[4]);
    }
    if (c->infer_pending) {
        cudaStreamWaitEvent(c->stream, c->infer_ev, 0);
        c->infer_pending = false;
    }
}

}  // namespace xr

using namespace xr;

extern "C" {

void xr_cache_params_default(XrCacheParams* p) {
    if (!p) return;
    p->enabled = 0;
    p->train = 1;
    p->train_samples = 65536;
    p->learning_rate = 1e-2f;
    p->beta1 = 0.9f;
    p->beta2 = 0.99f;
    p->epsilon = 1e-15f;
    p->seed = 1;
}

xr_status xr_cache_set_params(XrContext* c, const XrCacheParams* p) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "cache_set_params: null context");
    xr_status s = validate(c, p);
    if (s) return s;
    if (p->enabled && !c->instances.empty())
        return fail(c, XR_ERR_UNSUPPORTED, "cache_set_params: the learned cache covers one scene without instances");
    DeviceGuard g(c->device);
    invalidate_graphs(c);
    c->cache.params = *p;
    if (p->enabled) return cache_alloc(c);
    return XR_OK;
}

xr_status xr_cache_get_params(XrContext* c, XrCacheParams* out) {
    if (!c || !out) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_get_params: null argument");
    *out = c->cache.params;
    return XR_OK;
}

xr_status xr_cache_reset(XrContext* c, uint32_t seed) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "cache_reset: null context");
    DeviceGuard g(c->device);
    c->cache.params.seed = seed;
    if (!c->cache.allocated) return cache_alloc(c);
    return cache_init(c, seed);
}

xr_status xr_cache_set_bounds(XrContext* c, const float lo[3], float inv_extent) {
    if (!c || !lo || !(inv_extent > 0.0f)) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_set_bounds: bad argument");
    for (int a = 0; a < 3; ++a) c->cache.lo[a] = lo[a];
    c->cache.inv_ext = inv_extent;
    return XR_OK;
}

xr_status xr_cache_query(XrContext* c, const XrCacheSample* smp, uint32_t n, float* out_rgb) {
    if (!c || (n && (!smp || !out_rgb))) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_query: null argument");
    if (n > kMaxApiSamples) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_query: at most 1048576 samples per call");
    if (n == 0) return XR_OK;
    DeviceGuard g(c->device);
    xr_status s = cache_alloc(c);
    if (!s) s = ensure_records(c, n, 1u);
    if (s) return s;
    CacheState& cs = c->cache;
    if ((s = upload_samples(c, smp, n, 2u, cs.queries))) return s;
    float* d_out = nullptr;
    if ((s = cuda_check(c, cudaMalloc((void**)&d_out, (size_t)n * 12), "cache query output"))) return s;
    launch_cache_infer(cs, cs.queries, nullptr, n, d_out, nullptr, c->d_counters + kCntError, c->sm_count, c->stream);
    s = cuda_check(c, cudaGetLastError(), "cache query launch");
    if (!s) s = cuda_check(c, cudaMemcpyAsync(out_rgb, d_out, (size_t)n * 12, cudaMemcpyDeviceToHost, c->stream),
                           "cache query copy");
    if (!s) s = xr_sync(c);
    cudaFree(d_out);
    cs.frame_used = false;
    return s;
}

xr_status xr_cache_train(XrContext* c, const XrCacheSample* smp, uint32_t n, int apply, float* loss) {
    if (!c || !smp) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_train: null argument");
    if (n == 0 || n % nrc::kTile || n > kMaxApiSamples)
        return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_train: n must be a positive multiple of 128, <= 1048576");
    DeviceGuard g(c->device);
    xr_status s = cache_alloc(c);
    if (!s) s = ensure_records(c, 1u, n);
    if (s) return s;
    CacheState& cs = c->cache;
    if ((s = upload_samples(c, smp, n, 3u, cs.train))) return s;
    cudaMemsetAsync(cs.mlp_grad, 0, (size_t)nrc::kMlpParams * 4, c->stream);
    cudaMemsetAsync(cs.grid_grad, 0, nrc::kGridParams * 4, c->stream);
    launch_cache_train(cs, cs.train, nullptr, n, n, apply != 0, c->d_counters + kCntError, c->sm_count, c->stream);
    if (apply) cs.step++;
    s = cuda_check(c, cudaGetLastError(), "cache train launch");
    float l = 0.0f;
    if (!s) s = cuda_check(c, cudaMemcpyAsync(&l, cs.loss, 4, cudaMemcpyDeviceToHost, c->stream), "cache loss");
    if (!s) s = xr_sync(c);
    cs.grads_dirty = apply == 0;
    cs.frame_used = false;
    if (loss) *loss = l;
    return s;
}

xr_status xr_cache_step(XrContext* c) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "cache_step: null context");
    DeviceGuard g(c->device);
    xr_status s = cache_alloc(c);
    if (s) return s;
    launch_cache_adam(c->cache, c->stream);
    c->cache.step++;
    c->cache.grads_dirty = false;
    if ((s = cuda_check(c, cudaGetLastError(), "cache step launch"))) return s;
    return xr_sync(c);
}

xr_status xr_cache_selftest_wait(XrContext* c, uint32_t limit_us) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "cache_selftest_wait: null context");
    if (limit_us == 0 || limit_us > 1000000u)
        return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_selftest_wait: limit_us must be in [1, 1000000]");
    DeviceGuard g(c->device);
    launch_cache_wait_selftest((uint64_t)limit_us * 1000ull, c->d_counters + kCntError, c->stream);
    xr_status s = cuda_check(c, cudaGetLastError(), "cache_selftest_wait launch");
    if (s) return s;
    return xr_sync(c);   // the raised flag comes back as XR_ERR_TIMEOUT
}

xr_status xr_cache_read(XrContext* c, int which, void* host, size_t bytes, size_t* needed) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "cache_read: null context");
    CacheState& cs = c->cache;
    if (!cs.allocated) return fail(c, XR_ERR_STATE, "cache_read: the cache is not allocated");
    DeviceGuard g(c->device);
    xr_status s = xr_sync(c);
    if (s) return s;
    size_t need;
    const void* src;
    if (which == XR_CACHE_QUERIES || which == XR_CACHE_TRAIN_RECORDS) {
        uint32_t cnt = 0;
        if (cs.frame_used) {
            s = cuda_check(c, cudaMemcpy(&cnt, c->d_counters + (which == XR_CACHE_QUERIES ? kCntCacheQuery : kCntCacheTrain),
                                         4, cudaMemcpyDeviceToHost), "cache record count");
            if (s) return s;
        }
        if (which == XR_CACHE_QUERIES) {
            cnt = cnt < cs.query_cap ? cnt : cs.query_cap;
            need = (size_t)cnt * 32;
            src = cs.queries;
        } else {
            const uint32_t cap = c->fa.cache_t_cap;
            cnt = cnt < cap ? cnt : cap;
            need = (size_t)cnt * 48;
            src = cs.train;
        }
    } else if (which == XR_CACHE_ADAM_STEP) {
        if (needed) *needed = 4;
        if (!host) return XR_OK;
        if (bytes < 4) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_read: host buffer too small");
        std::memcpy(host, &cs.step, 4);
        return XR_OK;
    } else {
        need = array_floats(which) * 4;
        src = array_ptr(cs, which);
        if (!src) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_read: unknown array");
    }
    if (needed) *needed = need;
    if (!host) return XR_OK;
    if (bytes < need) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_read: host buffer too small");
    if (need == 0) return XR_OK;
    return cuda_check(c, cudaMemcpy(host, src, need, cudaMemcpyDeviceToHost), "cache_read copy");
}

xr_status xr_cache_write(XrContext* c, int which, const void* host, size_t bytes) {
    if (!c || !host) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_write: null argument");
    DeviceGuard g(c->device);
    xr_status s = cache_alloc(c);
    if (s) return s;
    CacheState& cs = c->cache;
    if (which == XR_CACHE_ADAM_STEP) {
        if (bytes != 4) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_write: the step count is one uint32");
        std::memcpy(&cs.step, host, 4);
        // the device's bias-correction state after that many steps: the products
        // k_cache_adam_advance forms, one float multiplication per step
        float st[4] = {1.0f, 1.0f, 0.0f, 0.0f};
        for (uint32_t i = 0; i < cs.step; i++) {
            const float p1 = st[0] * cs.params.beta1, p2 = st[1] * cs.params.beta2;
            st[0] = p1;
            st[1] = p2;
            st[2] = 1.0f - p1;
            st[3] = 1.0f - p2;
        }
        if ((s = xr_sync(c))) return s;
        return cuda_check(c, cudaMemcpy(cs.adam, st, sizeof(st), cudaMemcpyHostToDevice), "cache_write adam state");
    }
    float* dst = array_ptr(cs, which);
    if (!dst) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_write: arrays 0..7 and the step count (10) only");
    if (bytes != array_floats(which) * 4) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_write: size mismatch");
    if ((s = xr_sync(c))) return s;
    if ((s = cuda_check(c, cudaMemcpy(dst, host, bytes, cudaMemcpyHostToDevice), "cache_write copy"))) return s;
    if (which == XR_CACHE_MLP || which == XR_CACHE_GRID) {
        launch_cache_refresh(cs, c->stream);
        if ((s = cuda_check(c, cudaGetLastError(), "cache refresh"))) return s;
    }
    if (which == XR_CACHE_MLP_GRAD || which == XR_CACHE_GRID_GRAD) cs.grads_dirty = false;
    return xr_sync(c);
}

xr_status xr_cache_get_stats(XrContext* c, XrCacheStats* out) {
    if (!c || !out) return fail(c, XR_ERR_INVALID_ARGUMENT, "cache_get_stats: null argument");
    DeviceGuard g(c->device);
    xr_status s = xr_sync(c);
    CacheState& cs = c->cache;
    XrCacheStats o;
    std::memset(&o, 0, sizeof(o));
    o.steps = cs.step;
    for (int a = 0; a < 3; ++a) o.bounds_lo[a] = cs.lo[a];
    o.inv_extent = cs.inv_ext;
    if (cs.allocated) cudaMemcpy(&o.loss, cs.loss, 4, cudaMemcpyDeviceToHost);
    if (cs.frame_used) {
        uint32_t cnt[2] = {0, 0};
        cudaMemcpy(cnt, c->d_counters + kCntCacheQuery, 8, cudaMemcpyDeviceToHost);
        o.queries = cnt[0];
        o.train_samples = cnt[1];
        cudaEventElapsedTime(&o.ms_infer, c->ev[6], c->ev[7]);
        cudaEventElapsedTime(&o.ms_train, c->ev_train0, c->ev[4]);
    }
    *out = o;
    return s;
}

}  // extern "C"
