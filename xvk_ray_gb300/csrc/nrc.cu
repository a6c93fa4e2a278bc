// nrc.cu -- learned radiance cache kernels: inference and training on the
// 5th-generation tensor cores (tcgen05, BF16 operands, FP32 accumulators in
// tensor memory), Adam, initialisation.
//
// Tiles of 128 samples (one per thread of a 4-warp CTA; thread t of warp w owns
// row 32 w + t and reads accumulator lane 32 w + t).  Per layer the CTA stages
// the tile's activations in shared memory (K-major canonical layout, bfloat16),
// one thread issues the MMAs of the layer (K = 64 in four K = 16 steps) against
// the layer's weights kept in shared memory, tcgen05.commit arrives on an
// mbarrier, and every thread reads its accumulator row back with tcgen05.ld,
// applies ReLU and writes the next layer's activations.
//
// Training runs as three launches over the same 128-sample tiles:
//  * k_cache_encode (many warps per SM): the hash-grid gathers; writes each
//    tile's bfloat16 inputs in the shared-memory image layout (16 KB a tile);
//  * k_cache_train (one CTA per SM): copies a tile's inputs, forward + backward
//    fused, every layer's activations kept in shared memory, the weight
//    gradients of all its tiles accumulated in tensor memory (dW_l = dZ_l^T H_l,
//    M = 128 with the rows beyond the layer's outputs zero); writes the input
//    gradient of the 32 encoding features over the tile's inputs;
//  * k_cache_scatter (many warps per SM): the hash-table gradients through the
//    trilinear weights, with vector atomics.
// The latency of the gathers and the atomics is hidden by occupancy in the two
// outer launches instead of stalling the four warps that drive the tensor core.
// Every wait on the tensor core is bounded (1 s of wall time);
// on expiry the kernel sets XR_DEVFLAG_MMA_TIMEOUT, stops and frees its tensor
// memory.
#include <cmath>
#include <utility>

#include "nrc.cuh"
#include "umma.cuh"
#include "xr_internal.h"

namespace xr {
namespace nrc {
namespace {

constexpr uint64_t kWaitNs = 1000000000ull;
constexpr uint32_t kActBytes = kTile * kIn * 2;   // one [128][64] bf16 operand (16 KB)

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    return (uint32_t)umma::bf16_bits(a) | ((uint32_t)umma::bf16_bits(b) << 16);
}

// Row r of a K-major [*][K] bf16 operand <- K float values (rounded to bfloat16).
template <int K>
__device__ __forceinline__ void store_row(uint8_t* base, uint32_t r, const float* v) {
#pragma unroll
    for (int c = 0; c < K; c += 8) {
        uint4 w = make_uint4(pack2(v[c], v[c + 1]), pack2(v[c + 2], v[c + 3]), pack2(v[c + 4], v[c + 5]),
                             pack2(v[c + 6], v[c + 7]));
        *reinterpret_cast<uint4*>(base + umma::kmajor_offset(r, c, K)) = w;
    }
}

// Row r of a K-major [*][64] bf16 operand -> 64 float values.
__device__ __forceinline__ void load_row64(const uint8_t* base, uint32_t r, float* v) {
#pragma unroll
    for (int c = 0; c < 64; c += 8) {
        const uint4 w = *reinterpret_cast<const uint4*>(base + umma::kmajor_offset(r, c, 64));
        const uint32_t u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            v[c + 2 * j] = umma::bf16_value((uint16_t)(u[j] & 0xFFFFu));
            v[c + 2 * j + 1] = umma::bf16_value((uint16_t)(u[j] >> 16));
        }
    }
}

// The transposed operands of the weight-gradient MMAs (dZ^T, H^T: K = 128 samples)
// use the K-major canonical layout with the core matrices adjacent in K 144 bytes
// apart instead of 128 (LBO = 144, 8-row groups 16 x 144 = 2304 bytes apart).  A
// warp writes one column per lane: 32 consecutive samples, four core matrices'
// 16-byte rows, which then start on banks 0, 4, 8 and 12 instead of all on bank 0
// (no 4-way conflict on the 64 two-byte stores of each column).
constexpr uint32_t kTLbo = 144, kTSbo = 16u * kTLbo;
__host__ __device__ __forceinline__ uint32_t t_offset(uint32_t r, uint32_t k) {
    return (r >> 3) * kTSbo + (k >> 3) * kTLbo + (r & 7u) * 16u + (k & 7u) * 2u;
}
template <int ROWS>
__device__ __forceinline__ void store_col_t(uint8_t* base, uint32_t col, const float* v) {
#pragma unroll
    for (int r = 0; r < ROWS; ++r)
        *reinterpret_cast<uint16_t*>(base + t_offset((uint32_t)r, col)) = umma::bf16_bits(v[r]);
}

__device__ __forceinline__ void copy_image(uint8_t* dst, const uint8_t* __restrict__ src, uint32_t bytes) {
    for (uint32_t i = threadIdx.x * 16u; i < bytes; i += blockDim.x * 16u)
        *reinterpret_cast<uint4*>(dst + i) = __ldg(reinterpret_cast<const uint4*>(src + i));
}

// Shared-memory writes of every thread become visible to the tensor core, and
// every earlier tcgen05.ld of every thread is ordered before what follows.
__device__ __forceinline__ void publish() {
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
}

// D (+)= A[128][K] * B[N][K]^T, `steps` K = 16 steps; issued by one thread.
__device__ __forceinline__ void gemm(uint32_t d_tmem, const uint8_t* A, const uint8_t* B, uint32_t K, uint32_t N,
                                     uint32_t steps, bool accumulate) {
    const uint32_t id = umma::idesc_bf16_f32(128, N);
    const uint32_t a0 = umma::smem_u32(A), b0 = umma::smem_u32(B);
    for (uint32_t s = 0; s < steps; ++s) {
        const uint64_t ad = umma::smem_desc(a0 + 256u * s, 128u, K * 16u);
        const uint64_t bd = umma::smem_desc(b0 + 256u * s, 128u, K * 16u);
        umma::mma_bf16(d_tmem, ad, bd, id, (accumulate || s > 0) ? 1u : 0u);
    }
}

// D (+)= A[128][128] * B[N][128]^T over the transposed (padded) layout; one thread.
__device__ __forceinline__ void gemm_t(uint32_t d_tmem, const uint8_t* A, const uint8_t* B, uint32_t N,
                                       bool accumulate) {
    const uint32_t id = umma::idesc_bf16_f32(128, N);
    const uint32_t a0 = umma::smem_u32(A), b0 = umma::smem_u32(B);
    for (uint32_t s = 0; s < 8u; ++s) {   // K = 16 per step: two core matrices
        const uint64_t ad = umma::smem_desc(a0 + 2u * kTLbo * s, kTLbo, kTSbo);
        const uint64_t bd = umma::smem_desc(b0 + 2u * kTLbo * s, kTLbo, kTSbo);
        umma::mma_bf16(d_tmem, ad, bd, id, (accumulate || s > 0) ? 1u : 0u);
    }
}

// Every thread waits for the last commit; the outcome is the same in all threads.
__device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t& phase) {
    bool ok = umma::mbar_wait(bar, phase & 1u, kWaitNs);
    phase++;
    ok = __syncthreads_and(ok) != 0;
    umma::fence_after_sync();
    return ok;
}

// 64 accumulator columns [c0, c0 + 64) of this thread's lane.
__device__ __forceinline__ void tmem_row64(uint32_t taddr, float* v) {
    umma::tmem_ld16(taddr, v);
    umma::tmem_ld16(taddr + 16u, v + 16);
    umma::tmem_ld16(taddr + 32u, v + 32);
    umma::tmem_ld16(taddr + 48u, v + 48);
    umma::tmem_wait_ld();
}

__device__ __forceinline__ void inputs_of(const Bounds& bnd, const __half2* table, const uint4* rec, uint32_t stride,
                                          uint32_t i, float4& ra, uint4& rb, float* v) {
    const uint4 a = rec[(size_t)i * stride], b = rec[(size_t)i * stride + 1];
    ra = make_float4(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z), __uint_as_float(a.w));
    rb = b;
    network_inputs(bnd, table, ra, rb, v);
}

}  // namespace

// ---------------------------------------------------------------------------
// inference: MODE 0 writes out3[i] (test/API path), MODE 1 adds the prediction
// (clamped at 0) to the candidate radiance cand_b[pixel].rgb of the frame.
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(128) k_cache_infer(const uint4* __restrict__ rec, const uint32_t* count_ptr,
                                                     uint32_t count_host, Bounds bnd, const __half2* __restrict__ table,
                                                     const uint8_t* __restrict__ w_fwd, float* __restrict__ out3,
                                                     float4* __restrict__ cand_b, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sW = smem;                  // forward weight image
    uint8_t* sX = smem + kImageBytes;    // activations of the current layer
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t count = count_ptr ? *(volatile const uint32_t*)count_ptr : count_host;
    const uint32_t ntiles = (count + kTile - 1u) / kTile;
    if (blockIdx.x >= ntiles) return;

    if (warp == 0) umma::tmem_alloc(&tslot, 64);
    if (tid == 0) { umma::mbar_init(&bar, 1); umma::mbar_fence_init(); }
    copy_image(sW, w_fwd, kImageBytes);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t lane_addr = tmem + ((warp * 32u) << 16);
    uint32_t phase = 0;
    bool ok = true;

    for (uint32_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const uint32_t i = tile * kTile + tid;
        const bool valid = i < count;
        float v[kIn];
        float4 ra = make_float4(0, 0, 0, 0);
        uint4 rb = make_uint4(0, 0, 0, 0);
        if (valid) inputs_of(bnd, table, rec, 2u, i, ra, rb, v);
        else {
#pragma unroll
            for (int j = 0; j < kIn; ++j) v[j] = 0.0f;
        }
        store_row<kIn>(sX, tid, v);
        for (int l = 0; l <= kHidden && ok; ++l) {
            publish();
            if (tid == 0) {
                gemm(tmem, sX, sW + l * kLayerBytes, 64u, l < kHidden ? 64u : 16u, 4u, false);
                umma::commit(&bar);
            }
            ok = wait_mma(&bar, phase);
            if (!ok) break;
            if (l < kHidden) {
                tmem_row64(lane_addr, v);
#pragma unroll
                for (int j = 0; j < kWidth; ++j) v[j] = fmaxf(v[j], 0.0f);
                store_row<kIn>(sX, tid, v);
            } else {
                umma::tmem_ld16(lane_addr, v);
                umma::tmem_wait_ld();
                if (valid) {
                    if (MODE == 0) {
                        out3[(size_t)i * 3 + 0] = v[0];
                        out3[(size_t)i * 3 + 1] = v[1];
                        out3[(size_t)i * 3 + 2] = v[2];
                    } else {
                        const uint32_t pixel = __float_as_uint(ra.w);
                        float3 L = f3(fmaxf(v[0], 0.0f), fmaxf(v[1], 0.0f), fmaxf(v[2], 0.0f));
                        if (!isfinite(L.x + L.y + L.z)) L = f3(0.0f, 0.0f, 0.0f);
                        float4 c = cand_b[pixel];
                        c.x = c.x + L.x; c.y = c.y + L.y; c.z = c.z + L.z;
                        cand_b[pixel] = c;
                    }
                }
            }
        }
    }
    if (!ok && tid == 0) atomicOr(err, (uint32_t)XR_DEVFLAG_MMA_TIMEOUT);
    if (!ok) umma::mbar_wait(&bar, phase & 1u, kWaitNs);   // let an MMA still in flight finish
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 64);
}

// ---------------------------------------------------------------------------
// training: gradients of the mean relative L2 loss over n = min(count, cap)
// rounded down to a multiple of 128 samples.  `tiles` holds 16 KB per tile:
// the inputs [128][64] bf16 in the K-major image layout (k_cache_encode), then
// the input gradients [32][128] fp32 of the encoding features, feature-major
// (k_cache_train), read by k_cache_scatter.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t train_samples(const uint32_t* count_ptr, uint32_t count_host, uint32_t cap) {
    uint32_t count = count_ptr ? *(volatile const uint32_t*)count_ptr : count_host;
    if (count > cap) count = cap;
    return count & ~(kTile - 1u);
}

// Sample j of the tiles is record perm[j] (the spatial order below); its unit
// position goes to upos[j] for k_cache_scatter.
__global__ void __launch_bounds__(256) k_cache_encode(const uint4* __restrict__ rec, const uint32_t* __restrict__ perm,
                                                      const uint32_t* count_ptr, uint32_t count_host, uint32_t cap,
                                                      Bounds bnd, const __half2* __restrict__ table,
                                                      uint8_t* __restrict__ tiles, float4* __restrict__ upos) {
    const uint32_t n = train_samples(count_ptr, count_host, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float v[kIn];
        float4 ra;
        uint4 rb;
        inputs_of(bnd, table, rec, 3u, perm[i], ra, rb, v);
        const float3 p = unit_pos(bnd, xyz(ra));
        upos[i] = make_float4(p.x, p.y, p.z, 0.0f);
        store_row<kIn>(tiles + (size_t)(i / kTile) * kActBytes, i % kTile, v);
    }
}

// ---- spatial order of the training samples ----
// The samples lie on the scene's surfaces, so at the coarse levels a few table
// entries take most of the gradient updates (1080p, 65,536 samples: 36K updates
// of one entry at level 0, 4K at level 8, 180 at level 15), and atomics on one
// address serialise in L2.  The samples are therefore taken in the order of the
// 24-bit Morton code of their unit position (stable LSD radix sort, 3 passes of
// 8 bits, kOrderBlocks blocks sharing the device-side sample count): the 32
// samples of a warp are then neighbours, and k_cache_scatter sums runs of equal
// table entries across the warp before one atomic per run (the hottest entry
// takes ~30x fewer atomics).  The training loss and gradients are sums over the
// samples, so the order changes their rounding only.
constexpr uint32_t kOrderBlocks = 128, kOrderThreads = 256;

__device__ __forceinline__ void order_span(uint32_t n, uint32_t b, uint32_t& beg, uint32_t& end) {
    uint32_t chunk = (n + kOrderBlocks - 1u) / kOrderBlocks;
    chunk = (chunk + kOrderThreads - 1u) / kOrderThreads * kOrderThreads;
    beg = b * chunk < n ? b * chunk : n;
    end = beg + chunk < n ? beg + chunk : n;
}

__device__ __forceinline__ uint32_t spread8(uint32_t x) {   // bit j of x -> bit 3 j
    x &= 0xFFu;
    x = (x | (x << 8)) & 0x0000F00Fu;
    x = (x | (x << 4)) & 0x000C30C3u;
    x = (x | (x << 2)) & 0x00249249u;
    return x;
}

// Adds the digits of one row of 256 samples (d >= 256: past the end) to the
// block's counts, one shared-memory atomic per distinct digit of a warp.
__device__ __forceinline__ void count_digit(uint32_t* h, uint32_t d) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    if (d < 256u && (peers & ((1u << lane) - 1u)) == 0u) atomicAdd(&h[d], (uint32_t)__popc(peers));
}

// Keys (24-bit Morton code of the unit position) and the counts of their low digit.
__global__ void __launch_bounds__(kOrderThreads) k_cache_order_keys(const uint4* __restrict__ rec,
                                                                    const uint32_t* count_ptr, uint32_t count_host,
                                                                    uint32_t cap, Bounds bnd,
                                                                    uint32_t* __restrict__ keys,
                                                                    uint32_t* __restrict__ vals,
                                                                    uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint32_t beg, end;
    order_span(train_samples(count_ptr, count_host, cap), blockIdx.x, beg, end);
    for (uint32_t t = beg; t < end; t += kOrderThreads) {   // spans are whole multiples of the block
        const uint32_t i = t + threadIdx.x;
        uint32_t d = 256u + (threadIdx.x & 31u);
        if (i < end) {
            const uint4 a = rec[(size_t)i * 3];
            const float3 p = unit_pos(bnd, f3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z)));
            const uint32_t qx = min((uint32_t)(p.x * 256.0f), 255u), qy = min((uint32_t)(p.y * 256.0f), 255u);
            const uint32_t qz = min((uint32_t)(p.z * 256.0f), 255u);
            const uint32_t key = spread8(qx) | (spread8(qy) << 1) | (spread8(qz) << 2);
            keys[i] = key;
            vals[i] = i;
            d = key & 0xFFu;
        }
        count_digit(h, d);
    }
    __syncthreads();
    hist[blockIdx.x * 256u + threadIdx.x] = h[threadIdx.x];
}

// per-block digit counts, block-major: hist[b * 256 + d]
__global__ void __launch_bounds__(kOrderThreads) k_cache_order_hist(const uint32_t* __restrict__ keys,
                                                                    const uint32_t* count_ptr, uint32_t count_host,
                                                                    uint32_t cap, uint32_t shift,
                                                                    uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint32_t beg, end;
    order_span(train_samples(count_ptr, count_host, cap), blockIdx.x, beg, end);
    for (uint32_t t = beg; t < end; t += kOrderThreads) {
        const uint32_t i = t + threadIdx.x;
        count_digit(h, i < end ? (keys[i] >> shift) & 0xFFu : 256u + (threadIdx.x & 31u));
    }
    __syncthreads();
    hist[blockIdx.x * 256u + threadIdx.x] = h[threadIdx.x];
}

// Stable scatter.  Block b places digit d after every sample of a smaller digit
// and after the samples of digit d in blocks before b: thread d sums the counts
// of all blocks (read coalesced, from L2), the digit totals are scanned across
// the block, and a sample's rank among the block's earlier samples of its digit
// comes from the warps' match masks.
__global__ void __launch_bounds__(kOrderThreads) k_cache_order_scatter(const uint32_t* __restrict__ kin,
                                                                       const uint32_t* __restrict__ vin,
                                                                       uint32_t* __restrict__ kout,
                                                                       uint32_t* __restrict__ vout,
                                                                       const uint32_t* count_ptr, uint32_t count_host,
                                                                       uint32_t cap, uint32_t shift,
                                                                       const uint32_t* __restrict__ hist) {
    constexpr uint32_t kWarps = kOrderThreads / 32u;
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kWarps][256];
    __shared__ uint32_t wtot[kWarps];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    {
        uint32_t total = 0, before = 0;
#pragma unroll 16
        for (uint32_t b = 0; b < kOrderBlocks; ++b) {
            const uint32_t c = hist[b * 256u + threadIdx.x];
            total += c;
            before += b < blockIdx.x ? c : 0u;
        }
        uint32_t incl = total;   // exclusive scan of the digit totals: warps, then across the 8 warps
#pragma unroll
        for (uint32_t d = 1; d < 32u; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d) incl += t;
        }
        if (lane == 31u) wtot[warp] = incl;
        __syncthreads();
        uint32_t off = 0;
        for (uint32_t w = 0; w < warp; ++w) off += wtot[w];
        base[threadIdx.x] = off + incl - total + before;
    }
    uint32_t beg, end;
    order_span(train_samples(count_ptr, count_host, cap), blockIdx.x, beg, end);
    for (uint32_t t = beg; t < end; t += kOrderThreads) {
#pragma unroll
        for (uint32_t w = 0; w < kWarps; ++w) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const uint32_t i = t + threadIdx.x;
        const bool valid = i < end;
        const uint32_t key = valid ? kin[i] : 0u, val = valid ? vin[i] : 0u;
        const uint32_t d = valid ? (key >> shift) & 0xFFu : 256u + lane;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0u) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t before = 0;
            for (uint32_t w = 0; w < warp; ++w) before += wcnt[w][d];
            const uint32_t pos = base[d] + before + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        uint32_t tot = 0;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; ++w) tot += wcnt[w][threadIdx.x];
        base[threadIdx.x] += tot;
        __syncthreads();
    }
}

// *p += (x, y) as one reduction without a return value (red): unlike atomicAdd
// on a float2, whose result the thread has to wait for, the thread goes on at once.
__device__ __forceinline__ void red_add2(float2* p, float x, float y) {
    asm volatile("red.relaxed.gpu.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(x), "f"(y) : "memory");
}

// p[0] += (x0, y0), p[1] += (x1, y1): one 16-byte reduction; p 16-byte aligned.
__device__ __forceinline__ void red_add4(float2* p, float x0, float y0, float x1, float y1) {
    asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(x0), "f"(y0), "f"(x1),
                 "f"(y1)
                 : "memory");
}

// Table gradients, one thread per (sample, level): the 32 threads of a warp take
// 32 neighbouring samples (spatial order) of one tile at one level, so the
// gradient loads are coalesced and samples in the same cell come in runs.  The
// samples of a run share all 8 table entries; each entry's updates are summed
// across the run (segmented scan, steps up to the warp's longest run) and added
// by the run's last thread.  A warp without runs (most warps of the fine levels)
// adds directly.
__global__ void __launch_bounds__(256) k_cache_scatter(const float4* __restrict__ upos, const uint32_t* count_ptr,
                                                       uint32_t count_host, uint32_t cap,
                                                       const float* __restrict__ tiles, float2* grid_grad,
                                                       const uint32_t* err) {
    if (*(volatile const uint32_t*)err & (uint32_t)XR_DEVFLAG_MMA_TIMEOUT) return;   // gradients incomplete
    const uint32_t n = train_samples(count_ptr, count_host, cap);
    const uint32_t units = n * (uint32_t)kLevels, lane = threadIdx.x & 31u;
    // units is a multiple of 32 and so is the stride: every warp runs the loop whole
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < units; u += gridDim.x * blockDim.x) {
        const uint32_t lv = (u / kTile) % kLevels, s = u % kTile;
        const uint32_t i = u / (kTile * kLevels) * kTile + s;
        const float4 q = upos[i];
        const float* g = tiles + (size_t)(i / kTile) * (kActBytes / 4) + 2u * lv * kTile + s;
        const float g0 = g[0], g1 = g[kTile];
        const LevelCell cell = level_cell((int)lv, f3(q.x, q.y, q.z));
        const uint64_t key = (uint64_t)cell.i0[0] | ((uint64_t)cell.i0[1] << 21) | ((uint64_t)cell.i0[2] << 42);
        const uint64_t prev = __shfl_up_sync(0xFFFFFFFFu, key, 1);
        const uint32_t heads = __ballot_sync(0xFFFFFFFFu, lane == 0u || prev != key);
        const uint32_t start = 31u - (uint32_t)__clz(heads & (0xFFFFFFFFu >> (31u - lane)));
        const uint32_t longest = __reduce_max_sync(0xFFFFFFFFu, lane - start + 1u);
        const bool last = lane == 31u || ((heads >> (lane + 1u)) & 1u);
        LevelCorners c;
        cell_corners((int)lv, cell, c);
        float2* glv = grid_grad + (size_t)lv * kT;
        float v[16];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            v[2 * k] = c.w[k] * g0;
            v[2 * k + 1] = c.w[k] * g1;
        }
        if (longest > 1u) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                for (uint32_t d = 1; d < longest; d <<= 1) {
                    const float t = __shfl_up_sync(0xFFFFFFFFu, v[j], d);
                    if (lane >= start + d) v[j] += t;
                }
            }
        }
        if (last) {
            // corners k and k + 1 differ in x only; where their entries are the two halves of one
            // 16-byte pair (always for an even x in a hashed level), one reduction adds both
#pragma unroll
            for (int k = 0; k < 8; k += 2) {
                const uint32_t a = c.idx[k], b = c.idx[k + 1];
                if (b == (a ^ 1u)) {
                    if (a & 1u) red_add4(glv + b, v[2 * k + 2], v[2 * k + 3], v[2 * k], v[2 * k + 1]);
                    else red_add4(glv + a, v[2 * k], v[2 * k + 1], v[2 * k + 2], v[2 * k + 3]);
                } else {
                    red_add2(glv + a, v[2 * k], v[2 * k + 1]);
                    red_add2(glv + b, v[2 * k + 2], v[2 * k + 3]);
                }
            }
        }
    }
}

// Forward + backward of every tile.
// Shared memory (223,232 B): forward image, backward image, H_0..H_4, dZ,
// dZ^T [128][128] (rows beyond the layer's outputs zero) and H^T [64][128] in
// the padded transposed layout.
// Tensor memory (512 columns): 0..63 forward / dX accumulator, 64 + 64 l: dW_l.
constexpr uint32_t kOffWf = 0, kOffWb = kImageBytes, kOffX = 2 * kImageBytes;
constexpr uint32_t kOffDZ = kOffX + 5 * kActBytes, kOffDZT = kOffDZ + kActBytes, kOffHT = kOffDZT + 16u * kTSbo;
constexpr uint32_t kTrainSmem = kOffHT + 8u * kTSbo;
static_assert(kTrainSmem == 223232 && kTrainSmem <= 232448, "training shared memory layout");

__global__ void __launch_bounds__(128, 1) k_cache_train(const uint4* __restrict__ rec, const uint32_t* __restrict__ perm,
                                                        const uint32_t* count_ptr,
                                                        uint32_t count_host, uint32_t cap, uint8_t* tiles,
                                                        const uint8_t* __restrict__ w_fwd,
                                                        const uint8_t* __restrict__ w_bwd, float* mlp_grad,
                                                        float* loss_acc, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sWf = smem + kOffWf;
    uint8_t* sWb = smem + kOffWb;
    uint8_t* sX = smem + kOffX;
    uint8_t* sDZ = smem + kOffDZ;
    uint8_t* sDZT = smem + kOffDZT;
    uint8_t* sHT = smem + kOffHT;
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t n = train_samples(count_ptr, count_host, cap);
    const uint32_t ntiles = n / kTile;
    if (blockIdx.x >= ntiles) return;
    const float inv_count = 1.0f / (float)(3u * n);

    if (warp == 0) umma::tmem_alloc(&tslot, 512);
    if (tid == 0) { umma::mbar_init(&bar, 1); umma::mbar_fence_init(); }
    copy_image(sWf, w_fwd, kImageBytes);
    copy_image(sWb, w_bwd, kImageBytes);
    // rows 64..127 of dZ^T (row groups 8..15) stay zero -- the padding of the
    // M = 128 weight-gradient MMAs
    for (uint32_t off = 8u * kTSbo + tid * 16u; off < 16u * kTSbo; off += 128u * 16u)
        *reinterpret_cast<uint4*>(sDZT + off) = make_uint4(0, 0, 0, 0);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t lane_addr = tmem + ((warp * 32u) << 16);
    uint32_t phase = 0;
    bool ok = true, first = true;
    float loss = 0.0f;

    for (uint32_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const uint32_t i = tile * kTile + tid;
        uint8_t* tile_mem = tiles + (size_t)tile * kActBytes;
        {
            // the tile's inputs, 8 x 16 B per thread; plain loads: this launch rewrites the tile below
            uint4 q[kActBytes / 16 / kTile];
#pragma unroll
            for (uint32_t k = 0; k < kActBytes / 16 / kTile; ++k)
                q[k] = reinterpret_cast<const uint4*>(tile_mem)[k * kTile + tid];
#pragma unroll
            for (uint32_t k = 0; k < kActBytes / 16 / kTile; ++k)
                reinterpret_cast<uint4*>(sX)[k * kTile + tid] = q[k];
        }
        const uint4 rt = rec[(size_t)perm[i] * 3 + 2];
        float v[kIn];
        // ---- forward, keeping H_0..H_4 ----
        float y[16];
        for (int l = 0; l <= kHidden && ok; ++l) {
            publish();
            if (tid == 0) {
                gemm(tmem, sX + l * kActBytes, sWf + l * kLayerBytes, 64u, l < kHidden ? 64u : 16u, 4u, false);
                umma::commit(&bar);
            }
            ok = wait_mma(&bar, phase);
            if (!ok) break;
            if (l < kHidden) {
                tmem_row64(lane_addr, v);
#pragma unroll
                for (int j = 0; j < kWidth; ++j) v[j] = fmaxf(v[j], 0.0f);
                store_row<kIn>(sX + (l + 1) * kActBytes, tid, v);
            } else {
                umma::tmem_ld16(lane_addr, y);
                umma::tmem_wait_ld();
            }
        }
        if (!ok) break;
        // ---- loss and output gradient ----
        float dz[kWidth];
        {
            const float t[3] = {__uint_as_float(rt.x), __uint_as_float(rt.y), __uint_as_float(rt.z)};
#pragma unroll
            for (int c = 0; c < 16; ++c) dz[c] = 0.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float d = y[c] - t[c];
                const float den = y[c] * y[c] + 0.01f;
                loss += d * d / den * inv_count;
                dz[c] = 2.0f * d / den * inv_count;
            }
        }
        store_row<16>(sDZ, tid, dz);
        store_col_t<16>(sDZT, tid, dz);
        // rows 16..63 of dZ^T (row groups 2..7): zero -- the previous tile's hidden
        // layers left values there
        for (uint32_t off = 2u * kTSbo + tid * 16u; off < 8u * kTSbo; off += 128u * 16u)
            *reinterpret_cast<uint4*>(sDZT + off) = make_uint4(0, 0, 0, 0);
        // ---- backward: layer 4 .. 0 ----
        for (int l = kHidden; l >= 0 && ok; --l) {
            // H_l^T from this thread's own row of H_l
            load_row64(sX + l * kActBytes, tid, v);
            store_col_t<64>(sHT, tid, v);
            publish();
            if (tid == 0) {
                const uint32_t K = l == kHidden ? 16u : 64u;
                gemm(tmem, sDZ, sWb + l * kLayerBytes, K, 64u, K / 16u, false);                  // dX = dZ W_l
                gemm_t(tmem + 64u + 64u * (uint32_t)l, sDZT, sHT, 64u, !first);                // dW_l += dZ^T H_l
                umma::commit(&bar);
            }
            ok = wait_mma(&bar, phase);
            if (!ok) break;
            float dx[kWidth];
            tmem_row64(lane_addr, dx);
            if (l > 0) {
                // dZ_l = dH_l * relu'(Z_l), with Z_l > 0 exactly where this thread's row of H_l (in v) is
#pragma unroll
                for (int j = 0; j < kWidth; ++j) dz[j] = v[j] > 0.0f ? dx[j] : 0.0f;
                store_row<kIn>(sDZ, tid, dz);
                // the bf16-rounded values of dz, as the MMA will see them
#pragma unroll
                for (int j = 0; j < kWidth; ++j) dz[j] = umma::bf16_value(umma::bf16_bits(dz[j]));
                store_col_t<64>(sDZT, tid, dz);
            } else {
                // gradients of the 32 encoding features, feature-major over the tile's inputs (every
                // thread's loads of the tile completed before the first barrier of this tile)
                float* g = reinterpret_cast<float*>(tile_mem) + tid;
#pragma unroll
                for (int j = 0; j < 2 * kLevels; ++j) g[j * kTile] = dx[j];
            }
        }
        first = false;
    }
    // loss (mean over the batch)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, o);
    if (lane == 0 && ok) atomicAdd(loss_acc, loss);
    // weight gradients: rows 0..63 live in warps 0 and 1
    if (ok && !first && warp < 2) {
        for (int l = 0; l <= kHidden; ++l) {
            const uint32_t rows = l < kHidden ? 64u : 16u;
            for (uint32_t c = 0; c < 64u; c += 16u) {
                float g[16];
                umma::tmem_ld16(lane_addr + 64u + 64u * (uint32_t)l + c, g);
                umma::tmem_wait_ld();
                if (tid < rows) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) atomicAdd(mlp_grad + l * 4096 + tid * 64u + c + j, g[j]);
                }
            }
        }
    }
    if (!ok && tid == 0) atomicOr(err, (uint32_t)XR_DEVFLAG_MMA_TIMEOUT);
    if (!ok) umma::mbar_wait(&bar, phase & 1u, kWaitNs);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// Adam (Kingma and Ba 2015) and weight images
// ---------------------------------------------------------------------------
struct AdamArgs {
    float lr, b1, b2, eps;
    const float* state;   // {beta1^t, beta2^t, bc1 = 1 - beta1^t, bc2 = 1 - beta2^t} of the current step
};

__device__ __forceinline__ void adam_step(float& w, float& m, float& v, float g, const AdamArgs& a, float bc1,
                                          float bc2) {
    m = a.b1 * m + (1.0f - a.b1) * g;
    v = a.b2 * v + (1.0f - a.b2) * (g * g);
    const float mh = m / bc1, vh = v / bc2;
    w = w - a.lr * mh / (sqrtf(vh) + a.eps);
}

// One step of the bias-correction powers: beta^t = beta^(t-1) * beta in FP32, kept
// on the device so that a replayed frame graph advances them.
__global__ void k_cache_adam_advance(float* state, float b1, float b2) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const float p1 = state[0] * b1, p2 = state[1] * b2;
        state[0] = p1;
        state[1] = p2;
        state[2] = 1.0f - p1;
        state[3] = 1.0f - p2;
    }
}
__global__ void k_cache_adam_state_reset(float* state) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        state[0] = 1.0f; state[1] = 1.0f; state[2] = 0.0f; state[3] = 0.0f;
    }
}

__device__ __forceinline__ void write_images(uint32_t i, float w, uint8_t* w_fwd, uint8_t* w_bwd) {
    const uint32_t l = i < 16384u ? i >> 12 : 4u;
    const uint32_t rem = i - l * 4096u, o = rem >> 6, in = rem & 63u;
    const uint16_t b = umma::bf16_bits(w);
    *reinterpret_cast<uint16_t*>(w_fwd + l * kLayerBytes + umma::kmajor_offset(o, in, 64)) = b;
    *reinterpret_cast<uint16_t*>(w_bwd + l * kLayerBytes + umma::kmajor_offset(in, o, l < 4 ? 64u : 16u)) = b;
}

__global__ void k_cache_adam_mlp(float* w, float* g, float* m, float* v, uint8_t* w_fwd, uint8_t* w_bwd, AdamArgs a,
                                 int apply) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)kMlpParams) return;
    float wi = w[i];
    if (apply) {
        float mi = m[i], vi = v[i];
        adam_step(wi, mi, vi, g[i], a, a.state[2], a.state[3]);
        w[i] = wi; m[i] = mi; v[i] = vi;
        g[i] = 0.0f;
    }
    write_images(i, wi, w_fwd, w_bwd);
}

// Sparse update: a table value changes only where its gradient is non-zero.
// A thread takes 4 entries (two 16-byte gradient loads: the pass over the whole
// gradient is a stream; a few percent of the entries are non-zero).
constexpr uint32_t kAdamGridPer = 4;

__global__ void k_cache_adam_grid(float2* w, float2* g, float2* m, float2* v, __half2* table, AdamArgs a) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kGridParams / 2 / kAdamGridPer) return;
    const float4 q0 = reinterpret_cast<const float4*>(g)[2 * t], q1 = reinterpret_cast<const float4*>(g)[2 * t + 1];
    const float2 grs[kAdamGridPer] = {make_float2(q0.x, q0.y), make_float2(q0.z, q0.w), make_float2(q1.x, q1.y),
                                      make_float2(q1.z, q1.w)};
#pragma unroll
    for (uint32_t j = 0; j < kAdamGridPer; ++j) {
        const float2 gr = grs[j];
        if (gr.x == 0.0f && gr.y == 0.0f) continue;
        const size_t e = t * kAdamGridPer + j;
        float2 wi = w[e], mi = m[e], vi = v[e];
        const float bc1 = a.state[2], bc2 = a.state[3];
        if (gr.x != 0.0f) adam_step(wi.x, mi.x, vi.x, gr.x, a, bc1, bc2);
        if (gr.y != 0.0f) adam_step(wi.y, mi.y, vi.y, gr.y, a, bc1, bc2);
        w[e] = wi; m[e] = mi; v[e] = vi;
        g[e] = make_float2(0.0f, 0.0f);
        table[e] = __floats2half2_rn(wi.x, wi.y);
    }
}

__global__ void k_cache_init_grid(float2* w, __half2* table, uint32_t seed) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kGridParams / 2) return;
    const float a = (init_u01((uint32_t)(2 * e), seed, 1u) * 2.0f - 1.0f) * 1e-4f;
    const float b = (init_u01((uint32_t)(2 * e + 1), seed, 1u) * 2.0f - 1.0f) * 1e-4f;
    w[e] = make_float2(a, b);
    table[e] = __floats2half2_rn(a, b);
}

__global__ void k_cache_table_from_master(const float2* w, __half2* table) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kGridParams / 2) return;
    const float2 x = w[e];
    table[e] = __floats2half2_rn(x.x, x.y);
}

// XrCacheSample (18 words) -> record (stride 2 or 3 uint4)
__global__ void k_cache_pack(const XrCacheSample* s, uint32_t n, uint4* rec, uint32_t stride) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const XrCacheSample q = s[i];
    rec[(size_t)i * stride] = make_uint4(__float_as_uint(q.pos[0]), __float_as_uint(q.pos[1]),
                                         __float_as_uint(q.pos[2]), q.pixel);
    rec[(size_t)i * stride + 1] = pack_b(f3(q.normal[0], q.normal[1], q.normal[2]), f3(q.wo[0], q.wo[1], q.wo[2]),
                                         f3(q.albedo[0], q.albedo[1], q.albedo[2]), q.kind, q.roughness);
    if (stride == 3)
        rec[(size_t)i * stride + 2] = make_uint4(__float_as_uint(q.target[0]), __float_as_uint(q.target[1]),
                                                 __float_as_uint(q.target[2]), 0u);
}

// The training-path selection of the next frame.  A frame selects `sel` pixels
// (cache_training_pixel); those whose first bounce reaches a surface take a
// training record, `got` of them.  The next frame selects sel * target / got
// pixels (at least target, at most n; all of them when got is 0), so that about
// `target` records come out of a frame whatever share of the paths escapes the
// scene.  Integer arithmetic, replayed exactly by the oracle.
__global__ void k_cache_select_next(uint32_t* sel, const uint32_t* got_ptr, uint32_t target, uint32_t n,
                                    uint32_t set_to) {
    if (set_to) { *sel = set_to; return; }
    const uint64_t got = *got_ptr, cur = *sel;
    uint64_t next = got ? cur * target / got : (uint64_t)n;
    if (next < target) next = target;
    if (next > n) next = n;
    *sel = (uint32_t)next;
}

// The failure path of the bounded tensor-core waits, on its own: the CTA takes
// tensor memory and an mbarrier exactly as the cache kernels do, then waits on a
// phase that nothing completes (no MMA is issued and nothing arrives), so the
// wait gives up after limit_ns, the flag is raised and the tensor memory is
// freed -- the steps wait_mma's callers take on expiry.
__global__ void __launch_bounds__(128) k_cache_wait_selftest(uint64_t limit_ns, uint32_t* err) {
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) umma::tmem_alloc(&tslot, 32);
    if (tid == 0) { umma::mbar_init(&bar, 1); umma::mbar_fence_init(); }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot;
    bool ok = umma::mbar_wait(&bar, 0u, limit_ns);
    ok = __syncthreads_and(ok) != 0;
    if (!ok && tid == 0) atomicOr(err, (uint32_t)XR_DEVFLAG_MMA_TIMEOUT);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 32);
}

}  // namespace nrc

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
using namespace nrc;

static nrc::AdamArgs adam_args(const CacheState& cs) {
    nrc::AdamArgs a;
    a.lr = cs.params.learning_rate;
    a.b1 = cs.params.beta1;
    a.b2 = cs.params.beta2;
    a.eps = cs.params.epsilon;
    a.state = cs.adam;
    return a;
}

static nrc::Bounds bounds_of(const CacheState& cs) {
    nrc::Bounds b;
    b.lo[0] = cs.lo[0]; b.lo[1] = cs.lo[1]; b.lo[2] = cs.lo[2];
    b.inv_ext = cs.inv_ext;
    return b;
}

cudaError_t cache_configure_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k_cache_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_cache_infer<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kImageBytes + kActBytes));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_cache_infer<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(kImageBytes + kActBytes));
}

void launch_cache_init(CacheState& cs, uint32_t seed, cudaStream_t st) {
    const uint32_t n2 = (uint32_t)(kGridParams / 2);
    k_cache_init_grid<<<(n2 + 255) / 256, 256, 0, st>>>(reinterpret_cast<float2*>(cs.grid), cs.table, seed);
    k_cache_adam_mlp<<<(kMlpParams + 255) / 256, 256, 0, st>>>(cs.mlp, cs.mlp_grad, cs.mlp_m, cs.mlp_v, cs.w_fwd,
                                                                cs.w_bwd, adam_args(cs), 0);
}

void launch_cache_refresh(CacheState& cs, cudaStream_t st) {
    const uint32_t n2 = (uint32_t)(kGridParams / 2);
    k_cache_table_from_master<<<(n2 + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float2*>(cs.grid), cs.table);
    k_cache_adam_mlp<<<(kMlpParams + 255) / 256, 256, 0, st>>>(cs.mlp, cs.mlp_grad, cs.mlp_m, cs.mlp_v, cs.w_fwd,
                                                                cs.w_bwd, adam_args(cs), 0);
}

void launch_cache_pack(const XrCacheSample* s, uint32_t n, uint4* rec, uint32_t stride, cudaStream_t st) {
    if (n) k_cache_pack<<<(n + 127) / 128, 128, 0, st>>>(s, n, rec, stride);
}

void launch_cache_infer(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host,
                        float* out3, float4* cand_b, uint32_t* err, int sm_count, cudaStream_t st) {
    const uint32_t smem = kImageBytes + kActBytes;
    uint32_t grid = (uint32_t)sm_count * 4u;
    if (!count_ptr) {
        const uint32_t tiles = (count_host + kTile - 1u) / kTile;
        if (tiles == 0) return;
        if (tiles < grid) grid = tiles;
    }
    if (cand_b)
        k_cache_infer<1><<<grid, 128, smem, st>>>(rec, count_ptr, count_host, bounds_of(cs), cs.table, cs.w_fwd,
                                                  nullptr, cand_b, err);
    else
        k_cache_infer<0><<<grid, 128, smem, st>>>(rec, count_ptr, count_host, bounds_of(cs), cs.table, cs.w_fwd,
                                                  out3, nullptr, err);
}

void launch_cache_train(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host,
                        uint32_t cap, bool apply, uint32_t* err, int sm_count, cudaStream_t st) {
    launch_cache_encode_stage(cs, rec, count_ptr, count_host, cap, sm_count, st);
    launch_cache_grad_stage(cs, rec, count_ptr, count_host, cap, err, sm_count, st);
    if (apply) launch_cache_adam(cs, st);
}

static uint32_t train_grid(int sm_count, const uint32_t* count_ptr, uint32_t count_host, uint32_t cap) {
    uint32_t grid = (uint32_t)sm_count;
    if (!count_ptr) {
        const uint32_t tiles = (count_host < cap ? count_host : cap) / kTile;
        if (tiles < grid) grid = tiles;
    }
    return grid;
}

// Stage 1 of a training batch: spatial order and the encoded inputs.  It reads the
// records' position, normal, direction and material words (not the targets), the
// table, and writes its own scratch and the zeroed loss.
void launch_cache_encode_stage(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host,
                               uint32_t cap, int sm_count, cudaStream_t st) {
    cudaMemsetAsync(cs.loss, 0, sizeof(float), st);
    if (!train_grid(sm_count, count_ptr, count_host, cap)) return;
    const nrc::Bounds bnd = bounds_of(cs);
    const uint32_t wide = (uint32_t)sm_count * 8u;   // 8 x 256 threads per SM, grid-stride
    uint32_t* k0 = cs.order;
    uint32_t* v0 = cs.order + cs.train_cap;
    uint32_t* k1 = cs.order + 2 * (size_t)cs.train_cap;
    uint32_t* v1 = cs.order + 3 * (size_t)cs.train_cap;
    k_cache_order_keys<<<kOrderBlocks, kOrderThreads, 0, st>>>(rec, count_ptr, count_host, cap, bnd, k0, v0,
                                                               cs.order_hist);
    for (uint32_t shift = 0; shift < 24u; shift += 8u) {
        if (shift)
            k_cache_order_hist<<<kOrderBlocks, kOrderThreads, 0, st>>>(k0, count_ptr, count_host, cap, shift,
                                                                       cs.order_hist);
        k_cache_order_scatter<<<kOrderBlocks, kOrderThreads, 0, st>>>(k0, v0, k1, v1, count_ptr, count_host, cap,
                                                                      shift, cs.order_hist);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    // three passes: the order ends in the second key / value pair
    float4* upos = reinterpret_cast<float4*>(cs.order + 4 * (size_t)cs.train_cap);
    k_cache_encode<<<wide, 256, 0, st>>>(rec, v0, count_ptr, count_host, cap, bnd, cs.table, cs.tiles, upos);
}

// Stage 2: forward + backward (which read the records' targets) and the
// table-gradient scatter; they read the weights and write only the gradients,
// the loss and the tiles.
void launch_cache_grad_stage(CacheState& cs, const uint4* rec, const uint32_t* count_ptr, uint32_t count_host,
                             uint32_t cap, uint32_t* err, int sm_count, cudaStream_t st) {
    const uint32_t grid = train_grid(sm_count, count_ptr, count_host, cap);
    if (!grid) return;
    const uint32_t wide = (uint32_t)sm_count * 8u;
    const uint32_t* perm = cs.order + 3 * (size_t)cs.train_cap;   // the sort's result (second value array)
    const float4* upos = reinterpret_cast<const float4*>(cs.order + 4 * (size_t)cs.train_cap);
    k_cache_train<<<grid, 128, kTrainSmem, st>>>(rec, perm, count_ptr, count_host, cap, cs.tiles, cs.w_fwd, cs.w_bwd,
                                                 cs.mlp_grad, cs.loss, err);
    k_cache_scatter<<<wide, 256, 0, st>>>(upos, count_ptr, count_host, cap, reinterpret_cast<const float*>(cs.tiles),
                                          reinterpret_cast<float2*>(cs.grid_grad), err);
}

void launch_cache_select_next(uint32_t* sel, const uint32_t* got, uint32_t target, uint32_t n, uint32_t set_to,
                              cudaStream_t st) {
    k_cache_select_next<<<1, 1, 0, st>>>(sel, got, target, n, set_to);
}

void launch_cache_wait_selftest(uint64_t limit_ns, uint32_t* err, cudaStream_t st) {
    k_cache_wait_selftest<<<1, 128, 0, st>>>(limit_ns, err);
}

void launch_cache_adam_reset(CacheState& cs, cudaStream_t st) {
    k_cache_adam_state_reset<<<1, 32, 0, st>>>(cs.adam);
}

void launch_cache_adam(CacheState& cs, cudaStream_t st) {
    const nrc::AdamArgs a = adam_args(cs);
    k_cache_adam_advance<<<1, 32, 0, st>>>(cs.adam, cs.params.beta1, cs.params.beta2);
    k_cache_adam_mlp<<<(kMlpParams + 255) / 256, 256, 0, st>>>(cs.mlp, cs.mlp_grad, cs.mlp_m, cs.mlp_v, cs.w_fwd,
                                                                cs.w_bwd, a, 1);
    const uint32_t n2 = (uint32_t)(kGridParams / 2 / kAdamGridPer);
    k_cache_adam_grid<<<(n2 + 255) / 256, 256, 0, st>>>(
        reinterpret_cast<float2*>(cs.grid), reinterpret_cast<float2*>(cs.grid_grad),
        reinterpret_cast<float2*>(cs.grid_m), reinterpret_cast<float2*>(cs.grid_v), cs.table, a);
}

}  // namespace xr
