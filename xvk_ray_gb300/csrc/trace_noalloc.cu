// trace_noalloc.cu -- batch ray queries that allocate no memory.
//
// xr_trace_rays stages the caller's host rays and results through device
// buffers it allocates on every call.  Some callers cannot allocate device
// memory at the point where they query rays: an engine whose device memory is
// owned by its own allocator, or a real-time loop in which allocation (an
// implicit device synchronisation) is forbidden.  xr_trace_rays_noalloc gives
// them the same queries with the staging held in one file-scope __device__
// array of fixed size (kMaxRays rays, about 3 MiB, resident on every GPU that
// loads this library until the process exits).
//
// The array's host-side name is only a stand-in for the symbol, so its device
// address is looked up once per device with that device current
// (cudaGetSymbolAddress) and cached; the first call on a device does this
// set-up, so make that first call before any stream capture.  The cached
// address belongs to the device's context of that moment: a host that resets
// the device (cudaDeviceReset) and goes on using the library is not supported.
// Every call shares the array and it keeps the last call's contents.  Calls
// that overlap on the GPU (several host threads, or contexts on different
// streams of one device) race on the array: serialise them.  The error word and
// the kernel's ray-fetch counter must start at zero and are cleared at the
// start of every call.
//
// An instanced world whose top-level BVH went stale (xr_update_vertices moved
// instanced geometry) is refused with XR_ERR_STATE: rebuilding it allocates
// build scratch, so this entry point leaves the rebuild to the next frame,
// xr_trace_rays or xr_get_stats call.
#include <mutex>
#include <string>

#include "xr_internal.h"

namespace xr {
namespace {

constexpr uint32_t kMaxRays = 65536;
constexpr int kMaxDevices = 64;

struct TraceScratch {
    float4 rays[2 * kMaxRays];   // {o.xyz, tmin}, {d.xyz, tmax}
    float2 bary[kMaxRays];
    int32_t prim[kMaxRays];
    float t[kMaxRays];
    uint32_t flags;               // device-side error word, cleared per call
    uint32_t fetch;               // the kernel's ray-fetch counter, cleared per call
};

}  // namespace
}  // namespace xr

static __device__ __align__(256) xr::TraceScratch g_trace_scratch;

namespace xr {
namespace {

std::mutex g_scratch_mu;
TraceScratch* g_scratch_addr[kMaxDevices] = {};

// Device address of g_trace_scratch on `device`, which must be current.
xr_status scratch_for(Context* c, TraceScratch** out) {
    if (c->device < 0 || c->device >= kMaxDevices)
        return fail(c, XR_ERR_UNSUPPORTED, "trace_rays_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[c->device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_trace_scratch);
        if (e != cudaSuccess || !p) return cuda_check(c, e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                                                      "trace_rays_noalloc: cudaGetSymbolAddress");
        g_scratch_addr[c->device] = static_cast<TraceScratch*>(p);
    }
    *out = g_scratch_addr[c->device];
    return XR_OK;
}

}  // namespace
}  // namespace xr

using namespace xr;

extern "C" xr_status xr_trace_rays_noalloc(XrContext* c, const float* rays, uint32_t n, int32_t any_hit,
                                           int32_t* prim, float* t, float* bary) {
    if (!c) return fail(nullptr, XR_ERR_INVALID_ARGUMENT, "trace_rays_noalloc: null context");
    if (n > kMaxRays)
        return fail(c, XR_ERR_INVALID_ARGUMENT,
                    "trace_rays_noalloc: at most " + std::to_string(kMaxRays) + " rays per call, got " +
                        std::to_string(n) + " (split the batch)");
    if (n == 0) return XR_OK;
    if (!rays || !prim || !t || !bary) return fail(c, XR_ERR_INVALID_ARGUMENT, "trace_rays_noalloc: null array");
    if (!c->bvh_ready) return fail(c, XR_ERR_STATE, "trace_rays_noalloc: build the BVH first");
    if (c->tlas_stale)
        return fail(c, XR_ERR_STATE,
                    "trace_rays_noalloc: the top-level BVH is stale after xr_update_vertices; rebuilding it "
                    "allocates, so render a frame or call xr_trace_rays / xr_get_stats once first");
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != c->device) cudaSetDevice(c->device);
    TraceScratch* s = nullptr;
    uint32_t flags = 0;
    xr_status st = scratch_for(c, &s);
    cudaStream_t sm = c->stream;
    if (!st) st = cuda_check(c, cudaMemsetAsync(&s->flags, 0, 2 * sizeof(uint32_t), sm), "trace_rays_noalloc: clear");
    if (!st)
        st = cuda_check(c, cudaMemcpyAsync(s->rays, rays, (size_t)n * 32, cudaMemcpyHostToDevice, sm),
                        "trace_rays_noalloc: ray upload");
    if (!st) {
        launch_trace(c->fa.sc, reinterpret_cast<const float*>(s->rays), n, any_hit, s->prim, nullptr, s->t,
                     reinterpret_cast<float*>(s->bary), &s->fetch, &s->flags, nullptr, c->sm_count, sm);
        st = cuda_check(c, cudaGetLastError(), "trace_rays_noalloc: launch");
    }
    if (!st) st = cuda_check(c, cudaMemcpyAsync(prim, s->prim, (size_t)n * 4, cudaMemcpyDeviceToHost, sm),
                             "trace_rays_noalloc: read back");
    if (!st) st = cuda_check(c, cudaMemcpyAsync(t, s->t, (size_t)n * 4, cudaMemcpyDeviceToHost, sm),
                             "trace_rays_noalloc: read back");
    if (!st) st = cuda_check(c, cudaMemcpyAsync(bary, s->bary, (size_t)n * 8, cudaMemcpyDeviceToHost, sm),
                             "trace_rays_noalloc: read back");
    if (!st) st = cuda_check(c, cudaMemcpyAsync(&flags, &s->flags, 4, cudaMemcpyDeviceToHost, sm),
                             "trace_rays_noalloc: read back");
    if (s) {   // whatever was queued completes before the outputs are handed back
        const xr_status ss = cuda_check(c, cudaStreamSynchronize(sm), "trace_rays_noalloc");
        if (!st) st = ss;
    }
    if (!st && flags) st = fail(c, XR_ERR_OVERFLOW, "trace_rays_noalloc: traversal stack overflow or malformed BVH");
    if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
    return st;
}
