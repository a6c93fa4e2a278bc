// trace.cu -- batch closest-hit / any-hit queries (xr_trace_rays).
//
// The TraceRay calls of the reference (ReSTIRGIInitialSample.rgen.hlsl:90-98,
// ReSTIRGISpatialReuse.rgen.hlsl:58-59) as a standalone persistent kernel on the
// same traversal engine as the frame, used by the hit-id parity tests and by
// callers that want the BVH without the frame.
#include <algorithm>

#include "wavefront_trace.cuh"

namespace xr {
namespace {

constexpr int kTraceBlock = 128;

template <bool ANY>
__global__ void __launch_bounds__(kTraceBlock) k_trace(DeviceScene sc, const float4* __restrict__ rays, uint32_t n,
                                                       int32_t* __restrict__ prim, float* __restrict__ t,
                                                       float2* __restrict__ bary, uint32_t* fetch, uint32_t* flags,
                                                       unsigned long long* work) {
    trace_persistent<ANY>(
        sc, n, fetch,
        [&](uint32_t i) {
            float4 a = rays[2 * i], b = rays[2 * i + 1];
            RayIn r;
            r.root = 0u;
            r.o = xyz(a); r.tmin = a.w; r.d = xyz(b); r.tmax = b.w;
            return r;
        },
        [&](uint32_t i, const HitRec& h) {
            prim[i] = h.prim;
            t[i] = h.prim >= 0 ? h.t : -1.0f;
            bary[i] = make_float2(h.b1, h.b2);
        },
        flags, work);
}

}  // namespace

void launch_trace(const DeviceScene& sc, const float* rays, uint32_t n, int any_hit, int32_t* prim, float* t,
                  float* bary, uint32_t* fetch, uint32_t* flags, unsigned long long* work, int sm_count,
                  cudaStream_t st) {
    if (n == 0) return;
    static int occ[2] = {0, 0};
    int& o = occ[any_hit ? 1 : 0];
    if (o == 0) {
        int v = 0;
        if (any_hit) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_trace<true>, kTraceBlock, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_trace<false>, kTraceBlock, 0);
        o = v > 0 ? v : 4;
    }
    uint32_t blocks = std::min<uint32_t>((n + kTraceBlock - 1) / kTraceBlock, (uint32_t)(sm_count * o));
    const float4* r = reinterpret_cast<const float4*>(rays);
    float2* b = reinterpret_cast<float2*>(bary);
    if (any_hit) k_trace<true><<<blocks, kTraceBlock, 0, st>>>(sc, r, n, prim, t, b, fetch, flags, work);
    else k_trace<false><<<blocks, kTraceBlock, 0, st>>>(sc, r, n, prim, t, b, fetch, flags, work);
}

}  // namespace xr
