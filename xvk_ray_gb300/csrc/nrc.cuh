// nrc.cuh -- learned radiance cache: constants, record format, hash-grid
// encoding and network inputs (device side).
//
// The cache follows Mueller, Rousselle, Novak and Keller, "Real-time Neural
// Radiance Caching for Path Tracing" (SIGGRAPH 2021) with the multiresolution
// hash encoding of Mueller, Evans, Schied and Keller, "Instant Neural Graphics
// Primitives" (SIGGRAPH 2022):
//   * 16 levels, 2 features per level, 2^19 binary16 entries per level, level
//     resolutions N_l = floor(16 * 2^(7 l / 15)) (16 ... 2048 cells over the
//     scene cube); corners indexed densely where (N_l + 1)^3 <= 2^19, else by
//     the spatial hash (x * 1 ^ y * 2654435761 ^ z * 805459861) mod 2^19;
//   * network input (64 values, bfloat16): 32 interpolated features, normal,
//     direction towards the previous vertex, its mirror direction about the
//     normal, albedo, roughness, metal flag, plastic flag, 1, then 16 zeros;
//   * 4 hidden layers of width 64 with ReLU and a 64 -> 16 output layer (3
//     outputs used, no biases), bfloat16 weights, FP32 accumulation.
// The arithmetic of the encoding is the CPU oracle's operation for operation
// (-fmad=false), so the bfloat16 network inputs are identical on both sides.
//
// Record (32 bytes, 2 x uint4): {pos.xyz (f32 bits), pixel}, {oct16(normal),
// oct16(direction), albedo rgb unorm8 | material model << 24, roughness bits}.
// Training record (48 bytes): record + {target.rgb, 0}.
#pragma once
#include "device_math.cuh"

namespace xr {
namespace nrc {

constexpr int kLevels = 16;
constexpr uint32_t kLog2T = 19, kT = 1u << kLog2T;
constexpr int kIn = 64, kWidth = 64, kOut = 16, kHidden = 4;
constexpr int kMlpParams = kHidden * kWidth * kIn + kOut * kWidth;   // 17,408
constexpr size_t kGridParams = (size_t)kLevels * kT * 2;            // 16,777,216
constexpr uint32_t kTile = 128;                                     // samples per MMA tile (M)
// bfloat16 weight images in the K-major canonical shared-memory layout:
// forward  : layer l < 4 at l * 8192 as [64 out][64 in], layer 4 at 32768 as [16 out][64 in]
// backward : layer l < 4 at l * 8192 as [64 in][64 out], layer 4 at 32768 as [64 in][16 out]
constexpr uint32_t kLayerBytes = 64 * 64 * 2;
constexpr uint32_t kImageBytes = 4 * kLayerBytes + 16 * 64 * 2;      // 34,816

static __constant__ const uint32_t kRes[kLevels] = {16, 22, 30, 42, 58, 80, 111, 153,
                                                          212, 294, 406, 561, 776, 1072, 1482, 2048};

struct Bounds {
    float lo[3];
    float inv_ext;
};

__device__ __forceinline__ uint32_t unorm8(float x) {
    return (uint32_t)(fminf(fmaxf(x, 0.0f), 1.0f) * 255.0f + 0.5f);
}

__device__ __forceinline__ uint4 pack_b(float3 n, float3 wo, float3 albedo, uint32_t kind, float roughness) {
    return make_uint4(oct_encode(n, 16), oct_encode(wo, 16),
                      unorm8(albedo.x) | (unorm8(albedo.y) << 8) | (unorm8(albedo.z) << 16) | ((kind & 255u) << 24),
                      __float_as_uint(roughness));
}

// counter-based uniform in [0, 1) for parameter initialisation
__device__ __host__ __forceinline__ uint32_t init_mix(uint32_t s) {
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}
__device__ __host__ __forceinline__ float init_u01(uint32_t i, uint32_t seed, uint32_t salt) {
    const uint32_t h = init_mix(i ^ init_mix(seed * 0x85EBCA6Bu + salt));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

struct LevelCorners {
    uint32_t idx[8];
    float w[8];
};

// The cell of level l that holds the unit position p: its lowest corner and the
// position's fractions inside it.
struct LevelCell {
    uint32_t i0[3];
    float f[3];
};

__device__ __forceinline__ LevelCell level_cell(int l, float3 p) {
    const uint32_t res = kRes[l];
    const float fr = (float)res;
    const float s[3] = {p.x * fr, p.y * fr, p.z * fr};
    LevelCell c;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int ii = (int)floorf(s[a]);
        if (ii > (int)res - 1) ii = (int)res - 1;
        if (ii < 0) ii = 0;
        c.i0[a] = (uint32_t)ii;
        c.f[a] = s[a] - (float)ii;
    }
    return c;
}

// The 8 table entries of a cell and their trilinear weights.
__device__ __forceinline__ void cell_corners(int l, const LevelCell& cell, LevelCorners& c) {
    const uint32_t res = kRes[l];
    const bool dense = (uint64_t)(res + 1u) * (res + 1u) * (res + 1u) <= (uint64_t)kT;
    const uint32_t st = res + 1u;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t cx = cell.i0[0] + (k & 1), cy = cell.i0[1] + ((k >> 1) & 1), cz = cell.i0[2] + ((k >> 2) & 1);
        const float wx = (k & 1) ? cell.f[0] : 1.0f - cell.f[0];
        const float wy = (k & 2) ? cell.f[1] : 1.0f - cell.f[1];
        const float wz = (k & 4) ? cell.f[2] : 1.0f - cell.f[2];
        c.w[k] = (wx * wy) * wz;
        c.idx[k] = dense ? cx + st * (cy + st * cz) : ((cx * 1u) ^ (cy * 2654435761u) ^ (cz * 805459861u)) & (kT - 1u);
    }
}

__device__ __forceinline__ void level_corners(int l, float3 p, LevelCorners& c) {
    cell_corners(l, level_cell(l, p), c);
}

__device__ __forceinline__ float3 unit_pos(const Bounds& b, float3 x) {
    float3 p = f3((x.x - b.lo[0]) * b.inv_ext, (x.y - b.lo[1]) * b.inv_ext, (x.z - b.lo[2]) * b.inv_ext);
    p.x = fminf(fmaxf(p.x, 0.0f), 1.0f);
    p.y = fminf(fmaxf(p.y, 0.0f), 1.0f);
    p.z = fminf(fmaxf(p.z, 0.0f), 1.0f);
    return p;
}

// The 64 network inputs of one record, as float values (rounded to bfloat16 by
// the caller when staged for the tensor core).
__device__ __forceinline__ void network_inputs(const Bounds& bnd, const __half2* __restrict__ table, float4 ra,
                                               uint4 rb, float* v) {
    const float3 p = unit_pos(bnd, xyz(ra));
#pragma unroll
    for (int l = 0; l < kLevels; ++l) {
        LevelCorners c;
        level_corners(l, p, c);
        __half2 t[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) t[k] = __ldg(table + (size_t)l * kT + c.idx[k]);
        float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float2 tv = __half22float2(t[k]);
            a0 = a0 + c.w[k] * tv.x;
            a1 = a1 + c.w[k] * tv.y;
        }
        v[2 * l] = a0;
        v[2 * l + 1] = a1;
    }
    const float3 n = oct_decode(rb.x, 16), wo = oct_decode(rb.y, 16);
    const float ndw = dot(n, wo);
    const float3 refl = n * (2.0f * ndw) - wo;
    const uint32_t kind = rb.z >> 24;
    v[32] = n.x; v[33] = n.y; v[34] = n.z;
    v[35] = wo.x; v[36] = wo.y; v[37] = wo.z;
    v[38] = refl.x; v[39] = refl.y; v[40] = refl.z;
    v[41] = (float)(rb.z & 255u) / 255.0f;
    v[42] = (float)((rb.z >> 8) & 255u) / 255.0f;
    v[43] = (float)((rb.z >> 16) & 255u) / 255.0f;
    v[44] = __uint_as_float(rb.w);
    v[45] = kind == 1u ? 1.0f : 0.0f;
    v[46] = kind == 5u ? 1.0f : 0.0f;
    v[47] = 1.0f;
#pragma unroll
    for (int j = 48; j < kIn; ++j) v[j] = 0.0f;
}

}  // namespace nrc
}  // namespace xr
