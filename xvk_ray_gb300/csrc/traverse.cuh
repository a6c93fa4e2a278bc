// traverse.cuh -- closest-hit / any-hit traversal of the 8-wide compressed BVH.
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
// grid with one cell of slack on every side, and the slab test runs on
// t = q * (2^e / d) + (p - o) / d with one fused multiply-add per plane.  The
// slack (>= 2^-18 of the scene's largest coordinate) exceeds every rounding
// error of that arithmetic, so a box is never rejected while it can contain a
// hit at t <= the current closest t; traversal order only changes speed.
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
};

__device__ __forceinline__ uint32_t byte_of(uint32_t w0, uint32_t w1, uint32_t i) {
    uint32_t w = i < 4 ? w0 : w1;
    return (w >> ((i & 3u) * 8u)) & 0xFFu;
}

// One ray through the wide BVH.  ANY: stop at the first accepted hit.
// Returns false when the traversal stack would overflow or the tree is malformed
// (the caller flags it).
template <bool ANY>
__device__ __forceinline__ bool traverse(const DeviceScene& sc, float3 o, float3 d, float tmin, float tmax,
                                         HitRec& h) {
    h.prim = -1; h.t = tmax; h.b1 = 0.0f; h.b2 = 0.0f;
    if (sc.n_nodes == 0) return true;
    const RayTri rt = prep_ray(o, d);
    const float idx = 1.0f / d.x, idy = 1.0f / d.y, idz = 1.0f / d.z;
    // visit near children first: slot bit k set means the child lies on the +k side
    const uint32_t flip = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    const float tmin_box = tmin * (1.0f - 1e-6f) - 1e-30f;

    uint2 stack[kStackSize];
    int sp = 0;
    uint32_t node = 0;
    bool ok = true;
    // a well-formed tree visits each node at most once; the limit only stops a
    // corrupted one from looping
    uint32_t visits_left = sc.n_nodes;
    // group = children of the last visited node still to visit
    uint32_t g_base = 0, g_hits = 0, g_imask = 0;
    while (true) {
        // ---- visit `node`: test its 8 child boxes, then its leaf triangles ----
        if (node >= sc.n_nodes || visits_left == 0u) { ok = false; break; }
        visits_left--;
        {
            const uint4* np = reinterpret_cast<const uint4*>(sc.nodes + node);
            uint4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
            float px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
            uint32_t ex = w0.w & 0xFFu, ey = (w0.w >> 8) & 0xFFu, ez = (w0.w >> 16) & 0xFFu;
            uint32_t imask = w0.w >> 24;
            float sx = __uint_as_float(ex << 23) * idx;   // 2^(e-127) / d
            float sy = __uint_as_float(ey << 23) * idy;
            float sz = __uint_as_float(ez << 23) * idz;
            float ax = (px - o.x) * idx, ay = (py - o.y) * idy, az = (pz - o.z) * idz;
            const float tlimit = h.t * (1.0f + 1e-6f) + 1e-30f;
            uint32_t hits = 0, trimask = 0;
#pragma unroll
            for (uint32_t i = 0; i < 8; i++) {
                uint32_t meta = byte_of(w1.z, w1.w, i);
                float qlx = (float)byte_of(w2.x, w2.y, i), qly = (float)byte_of(w2.z, w2.w, i);
                float qlz = (float)byte_of(w3.x, w3.y, i), qhx = (float)byte_of(w3.z, w3.w, i);
                float qhy = (float)byte_of(w4.x, w4.y, i), qhz = (float)byte_of(w4.z, w4.w, i);
                float tx0 = __fmaf_rn(qlx, sx, ax), tx1 = __fmaf_rn(qhx, sx, ax);
                float ty0 = __fmaf_rn(qly, sy, ay), ty1 = __fmaf_rn(qhy, sy, ay);
                float tz0 = __fmaf_rn(qlz, sz, az), tz1 = __fmaf_rn(qhz, sz, az);
                float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin_box));
                float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tlimit));
                bool hit = meta != 0u && tn <= tf * (1.0f + 2e-6f) + 1e-30f;
                if (hit) {
                    if (meta == 0x80u) {
                        hits |= 1u << (i ^ flip);
                    } else {
                        uint32_t cnt = meta >> 5, off = meta & 31u;
                        trimask |= ((1u << cnt) - 1u) << off;
                    }
                }
            }
            uint32_t tri_base = w1.y;
            while (trimask) {
                uint32_t bit = __ffs(trimask) - 1u;
                trimask &= trimask - 1u;
                if (tri_base + bit >= sc.ntri) { ok = false; continue; }
                const float4* tp = sc.tri + 3u * (tri_base + bit);
                float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                int32_t prim = (int32_t)__float_as_uint(a.w);
                float tt, b1, b2;
                if (hit_triangle(rt, xyz(a), xyz(b), xyz(c), tmin, h.t, &tt, &b1, &b2)) {
                    if (h.prim < 0 || tt < h.t || (tt == h.t && prim < h.prim)) {
                        h.prim = prim; h.t = tt; h.b1 = b1; h.b2 = b2;
                        if (ANY) return ok;
                    }
                }
            }
            if (hits) {
                if (g_hits) {
                    if (sp == kStackSize) { ok = false; }
                    else stack[sp++] = make_uint2(g_base, g_hits | (g_imask << 8));
                }
                g_base = w1.x; g_hits = hits; g_imask = imask;
            }
        }
        // ---- pick the next node ----
        if (!g_hits) {
            if (sp == 0) break;
            uint2 e = stack[--sp];
            g_base = e.x; g_hits = e.y & 0xFFu; g_imask = (e.y >> 8) & 0xFFu;
        }
        uint32_t k = __ffs(g_hits) - 1u;
        g_hits &= g_hits - 1u;
        uint32_t slot = k ^ flip;
        node = g_base + __popc(g_imask & ((1u << slot) - 1u));
    }
    return ok;
}

}  // namespace xr
