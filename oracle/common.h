// common.h -- arithmetic shared by the oracle's translation units (TEST INFRASTRUCTURE).
//
// Every helper performs each written float operation as one IEEE binary32
// operation (the oracle is built with -ffp-contract=off), which is what the
// bit-exact comparisons with the CUDA path rely on.
#ifndef XR_ORACLE_COMMON_H
#define XR_ORACLE_COMMON_H
#include <cmath>
#include <cstdint>
#include <cstring>

namespace xro {

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

inline f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
inline f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(f3 a) { return sqrtf(dot(a, a)); }
inline f3 normalize(f3 a) { float r = 1.0f / sqrtf(dot(a, a)); return a * r; }
inline f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float comp(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
inline f3 xyz(f4 v) { return {v.x, v.y, v.z}; }

// Integer mix (the Wang hash steps of random.hlsl:3-9).
inline uint32_t wang(uint32_t s) {
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}

// ----------------------------------------------------------------------------
// Octahedral unit-vector codes used by the corrected-mode storage layout.
// bits = 16: 16+16 bits; bits = 12: 12+12 bits in the low 24 bits.
// ----------------------------------------------------------------------------
inline float sgn_nz(float v) { return v >= 0.0f ? 1.0f : -1.0f; }
inline uint32_t oct_encode(f3 n, uint32_t bits) {
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
inline f3 oct_decode(uint32_t code, uint32_t bits) {
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
    return normalize(f3{u, v, z});
}

// ----------------------------------------------------------------------------
// 16-bit float formats
// ----------------------------------------------------------------------------
inline uint32_t f32_bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float f32_from(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
// bfloat16 round-to-nearest-even (finite inputs), returned as its float value.
inline float bf16_round(float f) {
    uint32_t u = f32_bits(f);
    if ((u & 0x7F800000u) == 0x7F800000u) return f;   // inf / nan unchanged
    u += 0x7FFFu + ((u >> 16) & 1u);
    return f32_from(u & 0xFFFF0000u);
}
inline float half_value(uint16_t h) { _Float16 v; std::memcpy(&v, &h, 2); return (float)v; }
inline uint16_t half_bits(float f) { _Float16 v = (_Float16)f; uint16_t h; std::memcpy(&h, &v, 2); return h; }

}  // namespace xro

#endif
