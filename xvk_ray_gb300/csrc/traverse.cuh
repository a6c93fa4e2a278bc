// traverse.cuh -- ray/triangle and node primitives of the 8-wide compressed BVH traversal.
//
// Replaces TraceRay against the driver-built BLAS/TLAS (ReSTIRGIInitialSample.rgen.hlsl:90-98,
// ReSTIRGISpatialReuse.rgen.hlsl:58-59): opaque triangles, no culling, hits accepted
// for tmin <= t <= tmax, closest hit wins and ties go to the lowest primitive id
// (the reference's hardware traversal leaves ties unspecified).
//
// Triangle test: Woop, Benthin and Wald, "Watertight Ray/Triangle Intersection"
// (JCGT 2013) in the same operation order as the CPU oracle, including the
// double-precision recomputation when an edge function is exactly zero.
//
// Node test: child boxes are stored quantised to 8 bits against a power-of-two
// grid, rounded outwards with a slack of max(1/32 cell, 2^-17 of the scene's
// largest coordinate) on every side, and the slab test runs on
// t = q * (2^e / d) + (p - o) / d with one fused multiply-add per plane and a
// relative widening of 2e-6 of the far planes.  Together they exceed every
// rounding error of that arithmetic and of the watertight triangle test, so a box
// is never rejected while it can contain a hit at t <= the current closest t;
// traversal order only changes speed.
#pragma once
#include "device_math.cuh"
#include "xr_internal.h"

namespace xr {

struct RayTri {
    float3 o;          // origin
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__device__ __forceinline__ RayTri prep_ray(float3 o, float3 d) {
    RayTri r;
    r.o = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    float dz = sel3(d, kz);
    if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = sel3(d, kx) / dz;
    r.Sy = sel3(d, ky) / dz;
    r.Sz = 1.0f / dz;
    return r;
}

// Returns true on a hit with tmin <= t <= tmax; writes t and (b1, b2).
__device__ __forceinline__ bool hit_triangle(const RayTri& r, float3 v0, float3 v1, float3 v2, float tmin,
                                             float tmax, float* t_out, float* b1, float* b2) {
    float3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Akz = sel3(A, r.kz), Bkz = sel3(B, r.kz), Ckz = sel3(C, r.kz);
    float Ax = sel3(A, r.kx) - r.Sx * Akz;
    float Ay = sel3(A, r.ky) - r.Sy * Akz;
    float Bx = sel3(B, r.kx) - r.Sx * Bkz;
    float By = sel3(B, r.ky) - r.Sy * Bkz;
    float Cx = sel3(C, r.kx) - r.Sx * Ckz;
    float Cy = sel3(C, r.ky) - r.Sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double Ud = (double)Cx * (double)By - (double)Cy * (double)Bx;
        double Vd = (double)Ax * (double)Cy - (double)Ay * (double)Cx;
        double Wd = (double)Bx * (double)Ay - (double)By * (double)Ax;
        if ((Ud < 0.0 || Vd < 0.0 || Wd < 0.0) && (Ud > 0.0 || Vd > 0.0 || Wd > 0.0)) return false;
        double det = Ud + Vd + Wd;
        if (det == 0.0) return false;
        double T = Ud * (double)Az + Vd * (double)Bz + Wd * (double)Cz;
        float t = (float)(T / det);
        if (!(t >= tmin && t <= tmax)) return false;
        *t_out = t;
        *b1 = (float)(Vd / det);
        *b2 = (float)(Wd / det);
        return true;
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float T = U * Az + V * Bz + W * Cz;
    float t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    *t_out = t;
    *b1 = V / det;
    *b2 = W / det;
    return true;
}

struct HitRec {
    int32_t prim;   // -1: miss
    float t, b1, b2;
    int32_t inst;   // instance of the hit (scenes with instances; -1 otherwise)
};

// 3 x 4 row-major transforms (rows r0, r1, r2; column 3 = translation), each
// component one product at a time in the order written (no contraction), as in
// the oracle.
__device__ __forceinline__ float3 xform_point(float4 r0, float4 r1, float4 r2, float3 p) {
    return make_float3(((r0.x * p.x + r0.y * p.y) + r0.z * p.z) + r0.w, ((r1.x * p.x + r1.y * p.y) + r1.z * p.z) + r1.w,
                       ((r2.x * p.x + r2.y * p.y) + r2.z * p.z) + r2.w);
}
__device__ __forceinline__ float3 xform_dir(float4 r0, float4 r1, float4 r2, float3 d) {
    return make_float3((r0.x * d.x + r0.y * d.y) + r0.z * d.z, (r1.x * d.x + r1.y * d.y) + r1.z * d.z,
                       (r2.x * d.x + r2.y * d.y) + r2.z * d.z);
}
// Transpose of the linear part applied to v: the inverse transpose of the
// object-to-world map when the rows are those of world-to-object (normals).
__device__ __forceinline__ float3 xform_normal(float4 r0, float4 r1, float4 r2, float3 v) {
    return make_float3((r0.x * v.x + r1.x * v.y) + r2.x * v.z, (r0.y * v.x + r1.y * v.y) + r2.y * v.z,
                       (r0.z * v.x + r1.z * v.y) + r2.z * v.z);
}

__device__ __forceinline__ uint32_t byte_of(uint32_t w0, uint32_t w1, uint32_t i) {
    uint32_t w = i < 4 ? w0 : w1;
    return (w >> ((i & 3u) * 8u)) & 0xFFu;
}

}  // namespace xr
