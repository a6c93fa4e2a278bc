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

template <bool ANY, bool INST>
__global__ void __launch_bounds__(kTraceBlock) k_trace(DeviceScene sc, const float4* __restrict__ rays, uint32_t n,
                                                       int32_t* __restrict__ prim, int32_t* __restrict__ inst,
                                                       float* __restrict__ t, float2* __restrict__ bary, uint32_t* fetch,
                                                       uint32_t* flags, unsigned long long* work) {
    trace_persistent<ANY, INST>(
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
            if (inst) inst[i] = h.prim >= 0 ? h.inst : -1;
            t[i] = h.prim >= 0 ? h.t : -1.0f;
            bary[i] = make_float2(h.b1, h.b2);
        },
        flags, work);
}

template <bool ANY, bool INST>
int trace_occupancy() {
    static int occ = 0;
    if (occ == 0) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_trace<ANY, INST>, kTraceBlock, 0);
        occ = v > 0 ? v : 4;
    }
    return occ;
}

template <bool ANY, bool INST>
void launch_k_trace(const DeviceScene& sc, const float4* r, uint32_t n, int32_t* prim, int32_t* inst, float* t,
                    float2* b, uint32_t* fetch, uint32_t* flags, unsigned long long* work, int sm_count,
                    cudaStream_t st) {
    const uint32_t blocks = std::min<uint32_t>((n + kTraceBlock - 1) / kTraceBlock,
                                               (uint32_t)(sm_count * trace_occupancy<ANY, INST>()));
    k_trace<ANY, INST><<<blocks, kTraceBlock, 0, st>>>(sc, r, n, prim, inst, t, b, fetch, flags, work);
}

}  // namespace

void launch_trace(const DeviceScene& sc, const float* rays, uint32_t n, int any_hit, int32_t* prim, int32_t* inst,
                  float* t, float* bary, uint32_t* fetch, uint32_t* flags, unsigned long long* work, int sm_count,
                  cudaStream_t st) {
    if (n == 0) return;
    const float4* r = reinterpret_cast<const float4*>(rays);
    float2* b = reinterpret_cast<float2*>(bary);
    if (sc.n_inst) {
        if (any_hit) launch_k_trace<true, true>(sc, r, n, prim, inst, t, b, fetch, flags, work, sm_count, st);
        else launch_k_trace<false, true>(sc, r, n, prim, inst, t, b, fetch, flags, work, sm_count, st);
    } else {
        if (inst) cudaMemsetAsync(inst, 0xFF, (size_t)n * 4, st);   // -1: no instances
        if (any_hit) launch_k_trace<true, false>(sc, r, n, prim, nullptr, t, b, fetch, flags, work, sm_count, st);
        else launch_k_trace<false, false>(sc, r, n, prim, nullptr, t, b, fetch, flags, work, sm_count, st);
    }
}

}  // namespace xr
