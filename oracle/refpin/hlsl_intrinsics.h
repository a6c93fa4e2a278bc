// hlsl_intrinsics.h -- HLSL intrinsics for one shader namespace (TEST
// INFRASTRUCTURE: the reference pin of the CPU oracle).
//
// Included inside each `namespace ref_<shader> { ... }` right before the
// shader's rewritten source, with no include guard, so that unqualified calls
// in the shader resolve to these definitions first and no C library overload
// (sqrt(double), floor(double), ...) can take part.
//
// Conventions for what HLSL leaves to the compiler and driver -- the ones the
// oracle and the CUDA kernels share, so the pin tests the shader source:
//   dot / mul / length: products summed left to right, one rounding each;
//   normalize(v) = v * (1 / sqrt(dot(v, v))); rsqrt(x) = 1 / sqrt(x);
//   sin / cos / sincos: two-term Cody-Waite reduction by pi/2 and Taylor
//     polynomials to degree 11 / 12 in fused multiply-adds (this project's);
//   pow: the C library's powf; max / min: fmaxf / fminf;
//   Texture2D.SampleLevel: bilinear, clamp to edge, RGBA8 UNORM texels.

using hlsl::uint;
using hlsl::uint2;
using hlsl::uint3;
using hlsl::int2;
using hlsl::float2;
using hlsl::float3;
using hlsl::float4;
using hlsl::float4x4;
using hlsl::float3x4;
using hlsl::float4x3;
using hlsl::StructuredBuffer;
using hlsl::RWStructuredBuffer;
using hlsl::ByteAddressBuffer;
using hlsl::RWTexture2D;
using hlsl::Texture2D;
using hlsl::SamplerState;
using hlsl::RaytracingAccelerationStructure;
using hlsl::RayDesc;
using hlsl::RAY_FLAG_NONE;
using hlsl::RAY_FLAG_FORCE_OPAQUE;
using hlsl::RAY_FLAG_FORCE_NON_OPAQUE;
using hlsl::RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH;
using hlsl::RAY_FLAG_SKIP_CLOSEST_HIT_SHADER;

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline uint dot(uint2 a, uint2 b) { return a.x * b.x + a.y * b.y; }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float rsqrt(float x) { return 1.0f / __builtin_sqrtf(x); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float length(float3 v) { return __builtin_sqrtf(dot(v, v)); }
inline float3 normalize(float3 v) { const float r = 1.0f / __builtin_sqrtf(dot(v, v)); return v * r; }
inline float4 normalize(float4 v) { const float r = 1.0f / __builtin_sqrtf(dot(v, v)); return v * r; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float max(float a, float b) { return __builtin_fmaxf(a, b); }
inline float min(float a, float b) { return __builtin_fminf(a, b); }
inline uint min(uint a, int b) { return a < (uint)b ? a : (uint)b; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float3 clamp(float3 v, float lo, float hi) { return float3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)); }
inline int2 clamp(int2 v, int2 lo, int2 hi) {
    const int x = v.x < lo.x ? lo.x : (v.x > hi.x ? hi.x : v.x);
    const int y = v.y < lo.y ? lo.y : (v.y > hi.y ? hi.y : v.y);
    return int2(x, y);
}
inline float3 pow(float3 v, float e) {
    return float3(__builtin_powf(v.x, e), __builtin_powf(v.y, e), __builtin_powf(v.z, e));
}
inline float asfloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline int asint(uint u) { return (int)u; }

inline void sincos(float a, float& s, float& c) {
    const float k = __builtin_rintf(a * 0.636619772367581343f);
    float r = __builtin_fmaf(k, -1.57079637050628662109375f, a);
    r = __builtin_fmaf(k, 4.37113900018624283e-08f, r);
    const float r2 = r * r;
    float p = -2.50521083854417188e-08f;
    p = __builtin_fmaf(p, r2, 2.75573192239858907e-06f);
    p = __builtin_fmaf(p, r2, -1.98412698412698413e-04f);
    p = __builtin_fmaf(p, r2, 8.33333333333333333e-03f);
    p = __builtin_fmaf(p, r2, -1.66666666666666667e-01f);
    const float sr = __builtin_fmaf(p, r2 * r, r);
    float q = 2.08767569878680990e-09f;
    q = __builtin_fmaf(q, r2, -2.75573192239858907e-07f);
    q = __builtin_fmaf(q, r2, 2.48015873015873016e-05f);
    q = __builtin_fmaf(q, r2, -1.38888888888888889e-03f);
    q = __builtin_fmaf(q, r2, 4.16666666666666667e-02f);
    q = __builtin_fmaf(q, r2, -0.5f);
    const float cr = __builtin_fmaf(q, r2, 1.0f);
    switch (((int)k) & 3) {
        case 0: s = sr; c = cr; break;
        case 1: s = cr; c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}
inline float cos(float a) { float s, c; sincos(a, s, c); return c; }
inline float sin(float a) { float s, c; sincos(a, s, c); return s; }

// mul: glm column-major float4x4 times a column vector; row-major 3x4 / 4x3
// (instance transforms) with a column or a row vector
inline float4 mul(const float4x4& M, float4 v) {
    const float* m = M.m;
    return float4(m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w,
                  m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w,
                  m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w,
                  m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w);
}
inline float3 mul(const float3x4& M, float4 v) {
    float o[3];
    for (int r = 0; r < 3; ++r) o[r] = M.m[r][0] * v.x + M.m[r][1] * v.y + M.m[r][2] * v.z + M.m[r][3] * v.w;
    return float3(o[0], o[1], o[2]);
}
inline float3 mul(float4 v, const float4x3& M) {
    float o[3];
    for (int c = 0; c < 3; ++c) o[c] = v.x * M.m[0][c] + v.y * M.m[1][c] + v.z * M.m[2][c] + v.w * M.m[3][c];
    return float3(o[0], o[1], o[2]);
}
inline float4 mul(float3 v, const float3x4& M) {
    float o[4];
    for (int c = 0; c < 4; ++c) o[c] = v.x * M.m[0][c] + v.y * M.m[1][c] + v.z * M.m[2][c];
    return float4(o[0], o[1], o[2], o[3]);
}

// ---- ray-tracing pipeline system values (identity instances, as the reference builds them) ----
inline uint3 DispatchRaysIndex() { return hlsl::g_launch_id; }
inline uint3 DispatchRaysDimensions() { return hlsl::g_launch_size; }
inline uint PrimitiveIndex() { return hlsl::g_hit.primitive; }
inline uint InstanceIndex() { return hlsl::g_hit.instance; }
inline float RayTCurrent() { return hlsl::g_hit.t; }
inline float3x4 ObjectToWorld3x4() { return float3x4{{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}}}; }
inline float3x4 WorldToObject3x4() { return float3x4{{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}}}; }
inline float4x3 WorldToObject4x3() { return float4x3{{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}}}; }

template <class P>
inline void TraceRay(RaytracingAccelerationStructure, uint flags, uint, uint, uint, uint, RayDesc ray, P& payload) {
    hlsl::ShimPayload s;
    s.Position = payload.Position;
    s.Normal = payload.Normal;
    s.GeometryNormal = payload.GeometryNormal;
    s.UV = payload.UV;
    s.MaterialIndex = payload.MaterialIndex;
    s.HitT = payload.HitT;
    hlsl::g_trace_hook(flags, ray, s);
    payload.Position = s.Position;
    payload.Normal = s.Normal;
    payload.GeometryNormal = s.GeometryNormal;
    payload.UV = s.UV;
    payload.MaterialIndex = s.MaterialIndex;
    payload.HitT = s.HitT;
}
