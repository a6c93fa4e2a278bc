// hlsl_shim.h -- the HLSL types, literal semantics and resource objects that let
// the reference's ReSTIR GI shader sources compile, unmodified in their logic,
// as C++17 (TEST INFRASTRUCTURE: the reference pin of the CPU oracle).
//
// The shader files are copied by refpin/__init__.py through a purely mechanical
// rewrite (comments, attributes and register bindings dropped, `inout`/`out`
// parameters as references, swizzles as member calls, floating literals wrapped
// in HLSL_LIT) and included inside one C++ namespace per shader, after
// hlsl_intrinsics.h.  Everything an HLSL compiler and the GPU driver would
// supply is defined here, with these semantics:
//
//  * HLSL "literal float": an unsuffixed floating literal keeps double precision
//    while combined with other literals (and with integer literals, as in
//    `25 * PI / 180`), and is converted to float where it meets a float operand,
//    a float parameter or a float variable -- which is how dxc types literals.
//  * vector arithmetic is per component, one IEEE binary32 operation each (the
//    recipe builds with -ffp-contract=off);
//  * float4x4 holds the 16 floats of a constant-buffer matrix as the host
//    uploaded them (glm, column-major): element (row r, column c) at m[4 c + r],
//    so mul(M, v) is the glm product M v.
//
// The intrinsics whose evaluation an HLSL program leaves to the compiler and
// driver (dot and mul summation order, normalize, rsqrt, sin/cos, pow, texture
// filtering, image-format conversion) are given this project's conventions in
// hlsl_intrinsics.h -- the same conventions the oracle and the CUDA kernels use,
// so that what the pin checks is everything the shader source itself fixes:
// control flow, the order of its written operations, its constants, its data
// flow and its quirks.
#ifndef XR_REFPIN_HLSL_SHIM_H
#define XR_REFPIN_HLSL_SHIM_H

#include <cstddef>
#include <cstdint>
#include <cstring>

namespace hlsl {

typedef uint32_t uint;

// ---------------------------------------------------------------------------
// literal float
// ---------------------------------------------------------------------------
struct lit {
    double v;
    constexpr explicit lit(double d) : v(d) {}
    constexpr operator float() const { return (float)v; }
};
#define HLSL_LIT(x) (::hlsl::lit(x))

constexpr lit operator-(lit a) { return lit(-a.v); }
#define HLSL_LIT_OPS(OP)                                                                     \
    constexpr lit operator OP(lit a, lit b) { return lit(a.v OP b.v); }                     \
    constexpr lit operator OP(lit a, int b) { return lit(a.v OP (double)b); }               \
    constexpr lit operator OP(int a, lit b) { return lit((double)a OP b.v); }               \
    inline float operator OP(float a, lit b) { return a OP (float)b.v; }                    \
    inline float operator OP(lit a, float b) { return (float)a.v OP b; }
HLSL_LIT_OPS(+)
HLSL_LIT_OPS(-)
HLSL_LIT_OPS(*)
HLSL_LIT_OPS(/)
#undef HLSL_LIT_OPS
#define HLSL_LIT_CMP(OP)                                                                     \
    constexpr bool operator OP(lit a, lit b) { return a.v OP b.v; }                         \
    inline bool operator OP(float a, lit b) { return a OP (float)b.v; }                     \
    inline bool operator OP(lit a, float b) { return (float)a.v OP b; }
HLSL_LIT_CMP(<)
HLSL_LIT_CMP(<=)
HLSL_LIT_CMP(>)
HLSL_LIT_CMP(>=)
HLSL_LIT_CMP(==)
HLSL_LIT_CMP(!=)
#undef HLSL_LIT_CMP

// ---------------------------------------------------------------------------
// vectors
// ---------------------------------------------------------------------------
struct float3;
struct uint2 {
    uint x, y;
    uint2() : x(0), y(0) {}
    uint2(uint a, uint b) : x(a), y(b) {}
    uint2 xy() const { return *this; }
};
struct uint3 {
    uint x, y, z;
    uint3() : x(0), y(0), z(0) {}
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    uint2 xy() const { return uint2(x, y); }
};
struct float2 {
    float x, y;
    float2() : x(0), y(0) {}
    float2(float v) : x(v), y(v) {}
    float2(lit v) : x((float)v), y((float)v) {}
    float2(float a, float b) : x(a), y(b) {}
    explicit float2(uint2 v) : x((float)v.x), y((float)v.y) {}
    float2 xy() const { return *this; }
};
// float -> int conversions truncate toward zero (HLSL float-to-int)
struct int2 {
    int x, y;
    int2() : x(0), y(0) {}
    int2(int a, int b) : x(a), y(b) {}
    explicit int2(uint2 v) : x((int)v.x), y((int)v.y) {}
    explicit int2(float2 v) : x((int)v.x), y((int)v.y) {}
};

struct float3 {
    union { float x; float r; };
    union { float y; float g; };
    union { float z; float b; };
    float3() : x(0), y(0), z(0) {}
    float3(float v) : x(v), y(v), z(v) {}
    float3(lit v) : x((float)v), y((float)v), z((float)v) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    float3 xyz() const { return *this; }
    float2 xy() const { return float2(x, y); }
};
// an assignable three-component swizzle of an lvalue (v.xyz = ..., v.rgb)
struct Swz3 {
    float& a; float& b; float& c;
    operator float3() const { return float3(a, b, c); }
    Swz3& operator=(const float3& v) { a = v.x; b = v.y; c = v.z; return *this; }
};
struct float4 {
    union { float x; float r; };
    union { float y; float g; };
    union { float z; float b; };
    union { float w; float a; };
    float4() : x(0), y(0), z(0), w(0) {}
    float4(float v) : x(v), y(v), z(v), w(v) {}
    float4(float a_, float b_, float c_, float d_) : x(a_), y(b_), z(c_), w(d_) {}
    float4(float3 v, float d_) : x(v.x), y(v.y), z(v.z), w(d_) {}
    Swz3 xyz() & { return Swz3{x, y, z}; }
    float3 xyz() const& { return float3(x, y, z); }
    float3 xyz() && { return float3(x, y, z); }
    Swz3 rgb() & { return Swz3{x, y, z}; }
    float3 rgb() const& { return float3(x, y, z); }
    float3 rgb() && { return float3(x, y, z); }
    float2 xy() const { return float2(x, y); }
};
static_assert(sizeof(float3) == 12 && sizeof(float4) == 16 && sizeof(float2) == 8, "HLSL vector sizes");

// float3 / float2 / float4 arithmetic: per component, one rounding each
#define HLSL_VEC3_OPS(OP)                                                                    \
    inline float3 operator OP(float3 a, float3 b) { return float3(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
    inline float3 operator OP(float3 a, float s) { return float3(a.x OP s, a.y OP s, a.z OP s); }       \
    inline float3 operator OP(float s, float3 a) { return float3(s OP a.x, s OP a.y, s OP a.z); }       \
    inline float3 operator OP(float3 a, lit s) { return a OP (float)s; }                                \
    inline float3 operator OP(lit s, float3 a) { return (float)s OP a; }                                \
    inline float3& operator OP##=(float3& a, float3 b) { a = a OP b; return a; }                      \
    inline float3& operator OP##=(float3& a, float s) { a = a OP s; return a; }                       \
    inline float3& operator OP##=(float3& a, lit s) { a = a OP (float)s; return a; }
HLSL_VEC3_OPS(+)
HLSL_VEC3_OPS(-)
HLSL_VEC3_OPS(*)
HLSL_VEC3_OPS(/)
#undef HLSL_VEC3_OPS
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }

#define HLSL_VEC2_OPS(OP)                                                                    \
    inline float2 operator OP(float2 a, float2 b) { return float2(a.x OP b.x, a.y OP b.y); }           \
    inline float2 operator OP(float2 a, float s) { return float2(a.x OP s, a.y OP s); }                \
    inline float2 operator OP(float s, float2 a) { return float2(s OP a.x, s OP a.y); }                \
    inline float2 operator OP(float2 a, lit s) { return a OP (float)s; }                                \
    inline float2 operator OP(lit s, float2 a) { return (float)s OP a; }
HLSL_VEC2_OPS(+)
HLSL_VEC2_OPS(-)
HLSL_VEC2_OPS(*)
HLSL_VEC2_OPS(/)
#undef HLSL_VEC2_OPS

inline float4 operator*(float4 a, float s) { return float4(a.x * s, a.y * s, a.z * s, a.w * s); }

inline int2 operator+(int2 a, int2 b) { return int2(a.x + b.x, a.y + b.y); }
inline int2 operator-(int2 a, int b) { return int2(a.x - b, a.y - b); }

// ---------------------------------------------------------------------------
// matrices (constant-buffer float4x4 as uploaded; instance transforms)
// ---------------------------------------------------------------------------
struct float4x4 { float m[16]; };            // (row r, column c) at m[4 c + r]
struct float3x4 { float m[3][4]; };          // rows
struct float4x3 { float m[4][3]; };          // rows

// ---------------------------------------------------------------------------
// resources
// ---------------------------------------------------------------------------
template <class T>
struct StructuredBuffer {
    T* data = nullptr;
    size_t n = 0;
    template <class I>
    T& operator[](I i) const {
        static thread_local T dummy;
        const size_t k = (size_t)(uint)i;
        if (!data || k >= n) { dummy = T(); return dummy; }   // a null or too-short binding reads zeros
        return data[k];
    }
};
template <class T>
using RWStructuredBuffer = StructuredBuffer<T>;

struct ByteAddressBuffer {
    const uint32_t* words = nullptr;
    size_t n = 0;
    uint Load(uint byte_offset) const {
        const size_t k = byte_offset / 4u;
        return (words && k < n) ? words[k] : 0u;
    }
};

// Storage images: `half` is set for the RG16F image (binary16 round to nearest
// even on store, ApplicationReSTIRGI.cpp:363); the others are RGBA32F.
inline float round_half(float x) { return (float)(_Float16)x; }
inline float2 store_format(float2 v, bool half) { return half ? float2(round_half(v.x), round_half(v.y)) : v; }
inline float4 store_format(float4 v, bool) { return v; }

template <class T>
struct TexRef {
    T* p;
    bool half;
    operator T() const { return *p; }
    TexRef& operator=(const T& v) { *p = store_format(v, half); return *this; }
    TexRef& operator=(const TexRef& o) { *p = store_format((T)o, half); return *this; }
    float2 xy() const { return ((T)*this).xy(); }
    float3 xyz() const { return T(*this).xyz(); }
};

template <class T>
struct RWTexture2D {
    T* data = nullptr;
    uint w = 0, h = 0;
    bool half = false;
    TexRef<T> operator[](uint2 c) const { return at((long)c.x, (long)c.y); }
    TexRef<T> operator[](int2 c) const { return at((long)c.x, (long)c.y); }
    TexRef<T> at(long x, long y) const {
        static thread_local T dummy;
        if (!data || x < 0 || y < 0 || x >= (long)w || y >= (long)h) return TexRef<T>{&dummy, half};
        return TexRef<T>{data + (size_t)y * w + (size_t)x, half};
    }
};

struct SamplerState {};
struct Texture2D {
    const uint32_t* texels = nullptr;   // RGBA8, row-major
    int w = 0, h = 0;
    float4 SampleLevel(SamplerState, float2 uv, int) const;   // hlsl_intrinsics.h
};
constexpr int kMaxTextures = 256;   // capacity of the shaders' unsized texture arrays

struct RaytracingAccelerationStructure {};
struct RayDesc {
    float3 Origin;
    float TMin;
    float3 Direction;
    float TMax;
};
enum : uint {
    RAY_FLAG_NONE = 0x00u,
    RAY_FLAG_FORCE_OPAQUE = 0x01u,
    RAY_FLAG_FORCE_NON_OPAQUE = 0x02u,
    RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH = 0x04u,
    RAY_FLAG_SKIP_CLOSEST_HIT_SHADER = 0x08u,
};

// The ray-tracing pipeline around a TraceRay call: the payload travels as this
// neutral record between the calling shader's namespace and the hit / miss
// shaders' namespaces; the harness installs the traversal hook.
struct ShimPayload {
    float3 Position, Normal, GeometryNormal;
    float2 UV;
    int MaterialIndex;
    float HitT;
};
inline void (*g_trace_hook)(uint flags, const RayDesc& ray, ShimPayload& payload) = nullptr;

// State of the shader invocation running on this host thread.
struct HitState {
    uint primitive = 0, instance = 0;
    float t = 0.0f;
};
inline thread_local uint3 g_launch_id, g_launch_size;
inline thread_local HitState g_hit;

}  // namespace hlsl

#endif
