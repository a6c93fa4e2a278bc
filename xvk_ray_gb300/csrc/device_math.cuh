// device_math.cuh -- float3 helpers, RNG, sin/cos, octahedral codes for the kernels.
//
// Arithmetic contract (shared with the CPU oracle): every translation unit that
// includes this file is compiled with -fmad=false, so each written operation is
// one IEEE binary32 operation; fused multiply-adds appear only where written as
// __fmaf_rn.  Division and sqrt are IEEE (no fast-math).  Hence the kernels
// reproduce the oracle bit for bit on identical inputs.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

namespace xr {

__host__ __device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 div3(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) { float r = 1.0f / sqrtf(dot(a, a)); return a * r; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 f4(float3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ float sel3(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// out = M v with a column-major 4x4 matrix (HLSL mul(M, v) on glm data), summed
// left to right.
__device__ __forceinline__ float4 mat_mul(const float* m, float4 v) {
    float4 o;
    o.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    o.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    o.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    o.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return o;
}

// Float values of the reference's HLSL constants (ReSTIRGICommon.hlsl:1-3).
#define XR_PI_F ((float)3.14159265359)
#define XR_TWO_PI_F ((float)6.28318530718)
#define XR_INV_PI_F ((float)(1.0 / 3.14159265359))

// sin and cos: argument reduced by pi/2 (two-term Cody-Waite split, FMA), then
// Taylor series of sin (to r^11) and cos (to r^12) on [-pi/4, pi/4] by Horner.
__device__ __forceinline__ void sincos_xr(float a, float* s, float* c) {
    float k = rintf(a * 0.636619772367581343f);
    float r = __fmaf_rn(k, -1.57079637050628662109375f, a);
    r = __fmaf_rn(k, 4.37113900018624283e-08f, r);
    float r2 = r * r;
    float p = -2.50521083854417188e-08f;
    p = __fmaf_rn(p, r2, 2.75573192239858907e-06f);
    p = __fmaf_rn(p, r2, -1.98412698412698413e-04f);
    p = __fmaf_rn(p, r2, 8.33333333333333333e-03f);
    p = __fmaf_rn(p, r2, -1.66666666666666667e-01f);
    float sr = __fmaf_rn(p, r2 * r, r);
    float q = 2.08767569878680990e-09f;
    q = __fmaf_rn(q, r2, -2.75573192239858907e-07f);
    q = __fmaf_rn(q, r2, 2.48015873015873016e-05f);
    q = __fmaf_rn(q, r2, -1.38888888888888889e-03f);
    q = __fmaf_rn(q, r2, 4.16666666666666667e-02f);
    q = __fmaf_rn(q, r2, -0.5f);
    float cr = __fmaf_rn(q, r2, 1.0f);
    int quad = ((int)k) & 3;
    float ss = (quad & 1) ? cr : sr;
    float cc = (quad & 1) ? sr : cr;
    *s = (quad & 2) ? -ss : ss;
    *c = (quad == 1 || quad == 2) ? -cc : cc;
}

// ---- random.hlsl:1-20 ----
__device__ __forceinline__ uint32_t wang_mix(uint32_t s) {
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}
__device__ __forceinline__ uint32_t init_random_seed(uint32_t x, uint32_t y, uint32_t w, uint32_t frame) {
    return wang_mix(x + y * w) * (frame + 1u);
}
__device__ __forceinline__ uint32_t next_random(uint32_t& st) {
    st = st * 747796405u + 2891336453u;
    uint32_t word = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ __forceinline__ float random_float(uint32_t& st) {
    return (float)(next_random(st) & 0x00FFFFFFu) / 16777216.0f;
}
enum { kPassInitial = 0, kPassTemporal = 1, kPassSpatial = 2 };
// compat: every pass reseeds identically (the reference's behaviour);
// corrected: passes get decorrelated streams mixed with the user seed.
__device__ __forceinline__ uint32_t pass_rng(bool compat, uint32_t x, uint32_t y, uint32_t w, uint32_t frame,
                                             uint32_t pass, uint32_t seed) {
    uint32_t s = init_random_seed(x, y, w, frame);
    if (compat) return s;
    return s ^ wang_mix(frame * 0x9E3779B9u + pass * 0x85EBCA6Bu + seed * 0xC2B2AE35u);
}

// ---- octahedral unit-vector codes (corrected-mode storage) ----
__device__ __forceinline__ float sgn_nz(float v) { return v >= 0.0f ? 1.0f : -1.0f; }
__device__ __forceinline__ uint32_t oct_encode(float3 n, uint32_t bits) {
    float l1 = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
    float u = n.x / l1, v = n.y / l1;
    if (n.z < 0.0f) {
        float ou = (1.0f - fabsf(v)) * sgn_nz(u);
        float ov = (1.0f - fabsf(u)) * sgn_nz(v);
        u = ou; v = ov;
    }
    float scale = (float)((1u << (bits - 1)) - 1u);
    u = fminf(fmaxf(u, -1.0f), 1.0f);
    v = fminf(fmaxf(v, -1.0f), 1.0f);
    int32_t qu = (int32_t)rintf(u * scale);
    int32_t qv = (int32_t)rintf(v * scale);
    uint32_t mask = (1u << bits) - 1u;
    return ((uint32_t)qu & mask) | (((uint32_t)qv & mask) << bits);
}
__device__ __forceinline__ float3 oct_decode(uint32_t code, uint32_t bits) {
    uint32_t mask = (1u << bits) - 1u;
    int32_t qu = (int32_t)(code & mask), qv = (int32_t)((code >> bits) & mask);
    int32_t half = 1 << (bits - 1);
    if (qu >= half) qu -= (1 << bits);
    if (qv >= half) qv -= (1 << bits);
    float scale = (float)((1u << (bits - 1)) - 1u);
    float u = (float)qu / scale, v = (float)qv / scale;
    float z = 1.0f - fabsf(u) - fabsf(v);
    if (z < 0.0f) {
        float ou = (1.0f - fabsf(v)) * sgn_nz(u);
        float ov = (1.0f - fabsf(u)) * sgn_nz(v);
        u = ou; v = ov;
    }
    return normalize(f3(u, v, z));
}

// RG16F storage of the motion vector: binary16 round-to-nearest-even and back.
__device__ __forceinline__ float half_round(float x) { return __half2float(__float2half_rn(x)); }

// ---- Sampling.hlsl:4-56 ----
__device__ __forceinline__ void branchless_onb(float3 n, float3* b1, float3* b2) {
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *b1 = f3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    *b2 = f3(b, sign + n.y * n.y * a, -n.y);
}
__device__ __forceinline__ float3 to_world(float3 v, float3 T, float3 B, float3 N) {
    return T * v.x + B * v.y + N * v.z;
}
__device__ __forceinline__ float3 to_local(float3 v, float3 T, float3 B, float3 N) {
    return f3(dot(v, T), dot(v, B), dot(v, N));
}
__device__ __forceinline__ float3 sample_hemisphere(float xi_x, float xi_y) {
    float phi = XR_TWO_PI_F * xi_x;
    float cos_theta = sqrtf(1.0f - xi_y);
    float sin_theta = sqrtf(xi_y);
    float s, c;
    sincos_xr(phi, &s, &c);
    return f3(sin_theta * c, sin_theta * s, cos_theta);
}
__device__ __forceinline__ float2 world_to_screen_uv(float3 p, const float* view, const float* proj) {
    float4 vp = mat_mul(view, make_float4(p.x, p.y, p.z, 1.0f));
    float4 cp = mat_mul(proj, vp);
    float nx = cp.x / cp.w, ny = cp.y / cp.w;
    return make_float2(nx * 0.5f + 0.5f, ny * 0.5f + 0.5f);
}

// ---- ReSTIRGICommon.hlsl:123-131 + gamma 1/2.2 + UNORM8 ----
__device__ __forceinline__ float aces1(float x) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
    float v = (x * (a * x + b)) / (x * (c * x + d) + e);
    return fminf(fmaxf(v, 0.0f), 1.0f);
}
__device__ __forceinline__ unsigned char unorm8(float v) {
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    return (unsigned char)(int)(v * 255.0f + 0.5f);
}
__device__ __forceinline__ uchar4 tonemap_ldr(float3 c) {
    const float g = (float)(1.0 / 2.2);
    float r = powf(aces1(c.x), g), gg = powf(aces1(c.y), g), b = powf(aces1(c.z), g);
    return make_uchar4(unorm8(r), unorm8(gg), unorm8(b), 255);
}

}  // namespace xr
