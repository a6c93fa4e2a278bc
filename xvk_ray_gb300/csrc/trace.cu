// trace.cu -- batch closest-hit / any-hit queries (xr_trace_rays).
//
// The TraceRay calls of the reference (ReSTIRGIInitialSample.rgen.hlsl:90-98,
// ReSTIRGISpatialReuse.rgen.hlsl:58-59) as a standalone kernel, used by the
// hit-id parity tests and by callers that want the BVH without the frame.
#include <algorithm>

#include "traverse.cuh"

namespace xr {
namespace {

template <bool ANY>
__global__ void __launch_bounds__(128) k_trace(DeviceScene sc, const float4* __restrict__ rays, uint32_t n,
                                               int32_t* __restrict__ prim, float* __restrict__ t,
                                               float2* __restrict__ bary, uint32_t* flags) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 a = rays[2 * i], b = rays[2 * i + 1];
        HitRec h;
        if (!traverse<ANY>(sc, xyz(a), xyz(b), a.w, b.w, h)) atomicOr(flags, (uint32_t)XR_DEVFLAG_STACK_OVERFLOW);
        prim[i] = h.prim;
        t[i] = h.prim >= 0 ? h.t : -1.0f;
        bary[i] = make_float2(h.b1, h.b2);
    }
}

}  // namespace

void launch_trace(const DeviceScene& sc, const float* rays, uint32_t n, int any_hit, int32_t* prim, float* t,
                  float* bary, uint32_t* flags, int sm_count, cudaStream_t st) {
    if (n == 0) return;
    uint32_t blocks = std::min<uint32_t>((n + 127) / 128, (uint32_t)sm_count * 16u);
    const float4* r = reinterpret_cast<const float4*>(rays);
    float2* b = reinterpret_cast<float2*>(bary);
    if (any_hit) k_trace<true><<<blocks, 128, 0, st>>>(sc, r, n, prim, t, b, flags);
    else k_trace<false><<<blocks, 128, 0, st>>>(sc, r, n, prim, t, b, flags);
}

}  // namespace xr
