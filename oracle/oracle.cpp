// oracle.cpp -- CPU oracle for the ReSTIR GI frame pipeline (TEST INFRASTRUCTURE).
//
// Only the tests, the smoke check and the benchmark's CPU-baseline leg use this
// file, always as the checker.  See xr_oracle.h for the list of reference
// shader files restated here and for the arithmetic contract.
//
// Build: g++ -O3 -std=c++17 -fopenmp -ffp-contract=off -fno-fast-math -fPIC -shared
// (recipe in oracle/Makefile).  -ffp-contract=off is load-bearing: every
// expression below is evaluated as written, one rounding per operation.
#include "xr_oracle.h"
#include "common.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

namespace {

// vector types, IEEE-exact helpers, Wang hash, octahedral codes: common.h
using namespace xro;

// HLSL mul(M, v) with a glm column-major matrix: out_r = sum_c M[c][r] v_c,
// summed left to right.
inline f4 mul(const float* m, f4 v) {
    f4 o;
    o.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    o.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    o.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    o.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return o;
}

// ReSTIRGICommon.hlsl:1-4 (float values of the HLSL literals)
const float PI_F = (float)3.14159265359;
const float TWO_PI_F = (float)6.28318530718;
const float INV_PI_F = (float)(1.0 / 3.14159265359);

// sin/cos used by every path on both sides: reduce by pi/2 with a two-term
// Cody-Waite split of pi/2 (hi = nearest float, lo = remainder) using fused
// multiply-adds, then Taylor polynomials (coefficients +-1/n!) on [-pi/4, pi/4]
// to degree 11 (sin) and 12 (cos), evaluated by Horner with fused multiply-adds.
inline void sincos_xr(float a, float* s, float* c) {
    float k = rintf(a * 0.636619772367581343f);
    float r = fmaf(k, -1.57079637050628662109375f, a);
    r = fmaf(k, 4.37113900018624283e-08f, r);
    float r2 = r * r;
    float p = -2.50521083854417188e-08f;
    p = fmaf(p, r2, 2.75573192239858907e-06f);
    p = fmaf(p, r2, -1.98412698412698413e-04f);
    p = fmaf(p, r2, 8.33333333333333333e-03f);
    p = fmaf(p, r2, -1.66666666666666667e-01f);
    float sr = fmaf(p, r2 * r, r);
    float q = 2.08767569878680990e-09f;
    q = fmaf(q, r2, -2.75573192239858907e-07f);
    q = fmaf(q, r2, 2.48015873015873016e-05f);
    q = fmaf(q, r2, -1.38888888888888889e-03f);
    q = fmaf(q, r2, 4.16666666666666667e-02f);
    q = fmaf(q, r2, -0.5f);
    float cr = fmaf(q, r2, 1.0f);
    int quad = ((int)k) & 3;
    switch (quad) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}
inline float cos_xr(float a) { float s, c; sincos_xr(a, &s, &c); return c; }
inline float sin_xr(float a) { float s, c; sincos_xr(a, &s, &c); return s; }

// RG16F storage of the motion vector (ApplicationReSTIRGI.cpp:363): IEEE
// binary16 round-to-nearest-even and back.
inline float half_round(float x) { return (float)(_Float16)x; }

// ----------------------------------------------------------------------------
// random.hlsl:1-20
// ----------------------------------------------------------------------------
inline uint32_t init_random_seed(uint32_t x, uint32_t y, uint32_t width, uint32_t frame) {
    uint32_t seed = x * 1u + y * width;
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed * (frame + 1u);
}
inline uint32_t next_random(uint32_t& state) {
    state = state * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
inline float random_float(uint32_t& state) {
    return (float)(next_random(state) & 0x00FFFFFFu) / 16777216.0f;
}
enum { PASS_INITIAL = 0, PASS_TEMPORAL = 1, PASS_SPATIAL = 2 };
// Reference: every pass reseeds with InitRandomSeed(pixel, frame) (quirk kept in
// compatibility mode).  Corrected mode decorrelates passes and mixes the seed.
inline uint32_t pass_rng(bool compat, uint32_t x, uint32_t y, uint32_t w, uint32_t frame,
                         uint32_t pass, uint32_t seed) {
    uint32_t s = init_random_seed(x, y, w, frame);
    if (compat) return s;
    return s ^ wang(frame * 0x9E3779B9u + pass * 0x85EBCA6Bu + seed * 0xC2B2AE35u);
}

// ----------------------------------------------------------------------------
// Scene, watertight triangle test, traversal
// ----------------------------------------------------------------------------
enum { MAT_LAMBERTIAN = 0, MAT_METALLIC = 1, MAT_DIELECTRIC = 2, MAT_ISOTROPIC = 3,
       MAT_DIFFUSE_LIGHT = 4, MAT_PLASTIC = 5 };

struct Material {   // Material.hlsl:7-14 / src/Asset/Material.h:44-57, 32 B
    float base[4];
    int32_t tex;
    float fuzz;
    float ior;
    uint32_t model;
};
static_assert(sizeof(Material) == 32, "material layout");

struct BNode { float lo[3], hi[3]; int32_t left; int32_t count; };

struct Scene {
    std::vector<float> vert;       // nv x 9 words (Vertex.hlsl:12-33)
    std::vector<uint32_t> idx;     // 3 x ntri
    std::vector<Material> mat;
    uint32_t nv = 0, ntri = 0, nm = 0;
    std::vector<f3> p0, p1, p2;    // triangle positions
    std::vector<BNode> nodes;
    std::vector<uint32_t> order;
    bool brute = true;
    // base-colour textures: per texture {first texel, width, height}, RGBA8 texels
    std::vector<uint32_t> tex_info;
    std::vector<uint32_t> texels;
    // emissive triangles (next-event estimation of the radiance cache's training paths)
    std::vector<uint32_t> light_prim;
    std::vector<float> light_cdf, light_pmf, prim_light_pdf;
    // A world of instanced scenes (or_world_*): the arrays above hold the scenes
    // concatenated (indices and material indices relocated, as xr_upload_scenes
    // does); parts are the scenes themselves (local primitive ids, own BVHs),
    // part_prim0 the first primitive of each in the concatenation.
    struct Inst { uint32_t part; float o2w[12], w2o[12]; };
    std::vector<Scene> parts;
    std::vector<uint32_t> part_prim0;
    std::vector<Inst> inst;
};

// Light-sampling tables: power = area * luminance(4 * base colour) per
// DiffuseLight triangle, pmf = power / total, inclusive CDF in primitive order
// (last entry 1), per primitive pmf / area.
void build_lights(Scene& s);

struct RayPre { f3 o, d; int kx, ky, kz; float Sx, Sy, Sz; };
inline RayPre prep_ray(f3 o, f3 d) {
    RayPre r; r.o = o; r.d = d;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    float dz = comp(d, kz);
    if (dz < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = comp(d, kx) / dz; r.Sy = comp(d, ky) / dz; r.Sz = 1.0f / dz;
    return r;
}
// Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013,
// with the double-precision recomputation when an edge function is exactly 0.
// Accepts tmin <= t <= tmax; returns t and (b1, b2) = weights of v1, v2.
inline bool hit_triangle(const RayPre& r, f3 v0, f3 v1, f3 v2, float tmin, float tmax,
                         float* t_out, float* b1, float* b2) {
    f3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float Ax = comp(A, r.kx) - r.Sx * Akz;
    float Ay = comp(A, r.ky) - r.Sy * Akz;
    float Bx = comp(B, r.kx) - r.Sx * Bkz;
    float By = comp(B, r.ky) - r.Sy * Bkz;
    float Cx = comp(C, r.kx) - r.Sx * Ckz;
    float Cy = comp(C, r.ky) - r.Sy * Ckz;
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
        *t_out = t; *b1 = (float)(Vd / det); *b2 = (float)(Wd / det);
        return true;
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float T = U * Az + V * Bz + W * Cz;
    float t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    *t_out = t; *b1 = V / det; *b2 = W / det;
    return true;
}

void build_bvh(Scene& s) {
    s.order.resize(s.ntri);
    for (uint32_t i = 0; i < s.ntri; i++) s.order[i] = i;
    std::vector<f3> cen(s.ntri);
    for (uint32_t i = 0; i < s.ntri; i++) {
        cen[i] = f3{(s.p0[i].x + s.p1[i].x + s.p2[i].x) / 3.0f, (s.p0[i].y + s.p1[i].y + s.p2[i].y) / 3.0f,
                    (s.p0[i].z + s.p1[i].z + s.p2[i].z) / 3.0f};
    }
    s.nodes.clear();
    s.nodes.reserve(2 * s.ntri / 2 + 8);
    struct Task { int node; uint32_t b, e; };
    std::vector<Task> st;
    s.nodes.push_back(BNode{});
    st.push_back({0, 0, s.ntri});
    while (!st.empty()) {
        Task tk = st.back(); st.pop_back();
        BNode n;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
        for (uint32_t i = tk.b; i < tk.e; i++) {
            uint32_t t = s.order[i];
            f3 ps[3] = {s.p0[t], s.p1[t], s.p2[t]};
            for (auto& p : ps)
                for (int k = 0; k < 3; k++) {
                    lo[k] = std::min(lo[k], (double)comp(p, k));
                    hi[k] = std::max(hi[k], (double)comp(p, k));
                }
            for (int k = 0; k < 3; k++) {
                clo[k] = std::min(clo[k], (double)comp(cen[t], k));
                chi[k] = std::max(chi[k], (double)comp(cen[t], k));
            }
        }
        for (int k = 0; k < 3; k++) {
            // enlarge so that float rounding of the triangle test never falls outside
            double pad = 1e-5 * (std::max(fabs(lo[k]), fabs(hi[k])) + (hi[k] - lo[k])) + 1e-7;
            n.lo[k] = (float)(lo[k] - pad);
            n.hi[k] = (float)(hi[k] + pad);
        }
        uint32_t cnt = tk.e - tk.b;
        if (cnt <= 4) {
            n.left = (int32_t)tk.b; n.count = (int32_t)cnt;
            s.nodes[tk.node] = n;
            continue;
        }
        int ax = 0;
        for (int k = 1; k < 3; k++) if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
        uint32_t mid = tk.b + cnt / 2;
        std::nth_element(s.order.begin() + tk.b, s.order.begin() + mid, s.order.begin() + tk.e,
                         [&](uint32_t a, uint32_t b) {
                             float ca = comp(cen[a], ax), cb = comp(cen[b], ax);
                             return ca < cb || (ca == cb && a < b);
                         });
        int l = (int)s.nodes.size();
        s.nodes.push_back(BNode{});
        s.nodes.push_back(BNode{});
        n.left = l; n.count = 0;
        s.nodes[tk.node] = n;
        st.push_back({l, tk.b, mid});
        st.push_back({l + 1, mid, tk.e});
    }
}

inline bool box_test(const BNode& n, const double o[3], const double d[3], double tmin, double tmax,
                     double* tnear) {
    double t0 = tmin, t1 = tmax;
    for (int k = 0; k < 3; k++) {
        if (d[k] == 0.0) {
            if (o[k] < n.lo[k] || o[k] > n.hi[k]) return false;
            continue;
        }
        double a = (n.lo[k] - o[k]) / d[k], b = (n.hi[k] - o[k]) / d[k];
        if (a > b) std::swap(a, b);
        t0 = std::max(t0, a); t1 = std::min(t1, b);
    }
    *tnear = t0;
    return t0 <= t1 * (1.0 + 1e-7) + 1e-12;
}

struct Hit { int32_t prim; float t, b1, b2; int32_t inst = -1; };

// 3 x 4 row-major transforms, one product at a time in the order written
// (instances.cu / traverse.cuh evaluate the same expressions).
inline f3 xform_point(const float* m, f3 p) {
    return f3{((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
              ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]};
}
inline f3 xform_dir(const float* m, f3 d) {
    return f3{(m[0] * d.x + m[1] * d.y) + m[2] * d.z, (m[4] * d.x + m[5] * d.y) + m[6] * d.z,
              (m[8] * d.x + m[9] * d.y) + m[10] * d.z};
}
// transpose of the linear part of m (the rows of world-to-object): normals
inline f3 xform_normal(const float* m, f3 v) {
    return f3{(m[0] * v.x + m[4] * v.y) + m[8] * v.z, (m[1] * v.x + m[5] * v.y) + m[9] * v.z,
              (m[2] * v.x + m[6] * v.y) + m[10] * v.z};
}

Hit trace(const Scene& s, f3 o, f3 d, float tmin, float tmax, bool any_hit);

// Closest hit over instances: each instance's scene is traced with the ray in
// its object space (t is the world ray's); smallest t wins, then the lowest
// instance (visited first here), then the lowest primitive (within the scene).
Hit trace_instanced(const Scene& s, f3 o, f3 d, float tmin, float tmax, bool any_hit) {
    Hit best{-1, tmax, 0.0f, 0.0f};
    for (uint32_t i = 0; i < (uint32_t)s.inst.size(); i++) {
        const Scene::Inst& I = s.inst[i];
        const Scene& P = s.parts[I.part];
        if (P.ntri == 0) continue;
        const f3 oo = xform_point(I.w2o, o), od = xform_dir(I.w2o, d);
        const float chk = oo.x + oo.y + oo.z + od.x + od.y + od.z;
        if (!std::isfinite(chk) || (od.x == 0.0f && od.y == 0.0f && od.z == 0.0f)) continue;
        Hit h = trace(P, oo, od, tmin, best.t, any_hit);
        if (h.prim < 0) continue;
        if (best.prim < 0 || h.t < best.t) {
            best = h;
            best.prim = (int32_t)(s.part_prim0[I.part] + (uint32_t)h.prim);
            best.inst = (int32_t)i;
            if (any_hit) return best;
        }
    }
    return best;
}

// Closest hit (ties: lowest primitive id) or, with any_hit, the first hit found.
Hit trace(const Scene& s, f3 o, f3 d, float tmin, float tmax, bool any_hit) {
    if (!s.inst.empty()) return trace_instanced(s, o, d, tmin, tmax, any_hit);
    Hit h{-1, tmax, 0.0f, 0.0f};
    RayPre r = prep_ray(o, d);
    auto test = [&](uint32_t t) -> bool {
        float tt, b1, b2;
        if (!hit_triangle(r, s.p0[t], s.p1[t], s.p2[t], tmin, h.t, &tt, &b1, &b2)) return false;
        if (h.prim >= 0 && !(tt < h.t || (tt == h.t && (int32_t)t < h.prim))) return false;
        h.prim = (int32_t)t; h.t = tt; h.b1 = b1; h.b2 = b2;
        return true;
    };
    if (s.brute) {
        for (uint32_t t = 0; t < s.ntri; t++)
            if (test(t) && any_hit) return h;
        return h;
    }
    double od[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BNode& n = s.nodes[stack[--sp]];
        double tn;
        double limit = (double)h.t * (1.0 + 1e-6) + 1e-9;
        if (!box_test(n, od, dd, (double)tmin * (1.0 - 1e-6) - 1e-9, limit, &tn)) continue;
        if (n.count > 0) {
            for (int i = 0; i < n.count; i++)
                if (test(s.order[n.left + i]) && any_hit) return h;
        } else {
            stack[sp++] = n.left;
            stack[sp++] = n.left + 1;
        }
    }
    return h;
}

// Ray.rchit.hlsl:26-60 (identity instance transforms, as the reference's TLAS
// uses, XVKTLAccelerationStructure.cpp:88) and Ray.rmiss.hlsl:3-8.
struct Payload { f3 pos, normal, geo_normal; f2 uv; int32_t mat; float hit_t; };

inline f3 vert_pos(const Scene& s, uint32_t v) { const float* p = &s.vert[(size_t)v * 9]; return {p[0], p[1], p[2]}; }
inline f3 vert_nrm(const Scene& s, uint32_t v) { const float* p = &s.vert[(size_t)v * 9 + 3]; return {p[0], p[1], p[2]}; }
inline f2 vert_uv(const Scene& s, uint32_t v) { const float* p = &s.vert[(size_t)v * 9 + 6]; return {p[0], p[1]}; }
inline int32_t vert_mat(const Scene& s, uint32_t v) { int32_t m; memcpy(&m, &s.vert[(size_t)v * 9 + 8], 4); return m; }

Payload closest_hit(const Scene& s, const Hit& h) {
    Payload pl;
    uint32_t i0 = s.idx[(size_t)h.prim * 3 + 0], i1 = s.idx[(size_t)h.prim * 3 + 1], i2 = s.idx[(size_t)h.prim * 3 + 2];
    float bx = 1.0f - h.b1 - h.b2, by = h.b1, bz = h.b2;
    f3 n0 = vert_nrm(s, i0), n1 = vert_nrm(s, i1), n2 = vert_nrm(s, i2);
    f3 nm = n0 * bx + n1 * by + n2 * bz;
    f3 normal = normalize(nm);
    f2 u0 = vert_uv(s, i0), u1 = vert_uv(s, i1), u2 = vert_uv(s, i2);
    f2 uv{u0.x * bx + u1.x * by + u2.x * bz, u0.y * bx + u1.y * by + u2.y * bz};
    f3 v0 = vert_pos(s, i0), v1 = vert_pos(s, i1), v2 = vert_pos(s, i2);
    f3 pos = v0 * bx + v1 * by + v2 * bz;
    f3 e0 = v2 - v0, e1 = v1 - v0;
    f3 geo = cross(e0, e1);
    if (h.inst >= 0 && !s.inst.empty()) {
        // Ray.rchit.hlsl:46-55: position by object-to-world, normals by its inverse transpose
        const Scene::Inst& I = s.inst[h.inst];
        pos = xform_point(I.o2w, pos);
        normal = xform_normal(I.w2o, normal);
        geo = xform_normal(I.w2o, geo);
    }
    pl.geo_normal = normalize(geo);
    pl.pos = pos;
    pl.normal = normalize(normal);
    pl.uv = uv;
    pl.mat = vert_mat(s, i0);
    pl.hit_t = h.t;
    return pl;
}

// ----------------------------------------------------------------------------
// Sampling.hlsl:4-56, BSDF.hlsl:7-57; GGX lobes for the corrected mode
// ----------------------------------------------------------------------------
inline void branchless_onb(f3 n, f3* b1, f3* b2) {
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *b1 = f3{1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x};
    *b2 = f3{b, sign + n.y * n.y * a, -n.y};
}
inline f3 to_world(f3 v, f3 T, f3 B, f3 N) { return T * v.x + B * v.y + N * v.z; }
inline f3 to_local(f3 v, f3 T, f3 B, f3 N) { return f3{dot(v, T), dot(v, B), dot(v, N)}; }
inline f3 sample_hemisphere(f2 xi) {
    float phi = TWO_PI_F * xi.x;
    float cos_theta = sqrtf(1.0f - xi.y);
    float sin_theta = sqrtf(xi.y);
    float s, c;
    sincos_xr(phi, &s, &c);
    return f3{sin_theta * c, sin_theta * s, cos_theta};
}
inline f2 world_to_screen_uv(f3 p, const float* view, const float* proj) {
    f4 vp = mul(view, f4{p.x, p.y, p.z, 1.0f});
    f4 cp = mul(proj, vp);
    f3 ndc{cp.x / cp.w, cp.y / cp.w, cp.z / cp.w};
    return f2{ndc.x * 0.5f + 0.5f, ndc.y * 0.5f + 0.5f};
}

// GGX (Trowbridge-Reitz) with height-correlated Smith masking, Schlick Fresnel;
// sampling of visible normals after Heitz, "Sampling the GGX Distribution of
// Visible Normals", JCGT 7(4), 2018.  All vectors in the local frame (z = n).
inline float ggx_lambda(f3 w, float a2) {
    float c2 = w.z * w.z;
    float s2 = fmaxf(0.0f, 1.0f - c2);
    return (sqrtf(1.0f + a2 * s2 / c2) - 1.0f) * 0.5f;
}
inline float ggx_d(float nh, float a2) {
    float k = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (PI_F * k * k);
}
inline f3 schlick(f3 f0, float c) {
    float m = 1.0f - c; m = fminf(fmaxf(m, 0.0f), 1.0f);
    float m5 = m * m * m * m * m;
    return f0 + (f3{1.0f, 1.0f, 1.0f} - f0) * m5;
}
struct Lobe { f3 f; float pdf; };
// Evaluates f and the sampling pdf of the corrected-mode material for (wo, wi).
inline Lobe eval_material(const Material& m, f3 wo, f3 wi) {
    Lobe r{f3{0, 0, 0}, 0.0f};
    f3 albedo{m.base[0], m.base[1], m.base[2]};
    if (wi.z <= 0.0f) return r;
    if (m.model == MAT_LAMBERTIAN) {
        r.f = albedo * INV_PI_F;
        r.pdf = wi.z * INV_PI_F;
        return r;
    }
    if (wo.z <= 0.0f) return r;
    float rough = fminf(fmaxf(m.fuzz, 0.02f), 1.0f);
    float alpha = rough * rough;
    float a2 = alpha * alpha;
    f3 h = normalize(wo + wi);
    float nh = h.z, oh = dot(wo, h);
    float d = ggx_d(nh, a2);
    float g2 = 1.0f / (1.0f + ggx_lambda(wo, a2) + ggx_lambda(wi, a2));
    float g1 = 1.0f / (1.0f + ggx_lambda(wo, a2));
    float pdf_spec = g1 * d / (4.0f * wo.z);
    if (m.model == MAT_METALLIC) {
        f3 F = schlick(albedo, oh);
        r.f = F * (d * g2 / (4.0f * wo.z * wi.z));
        r.pdf = pdf_spec;
        return r;
    }
    // MAT_PLASTIC: dielectric GGX coat (F0 = 0.04) over a Lambertian base.
    f3 F = schlick(f3{0.04f, 0.04f, 0.04f}, oh);
    r.f = F * (d * g2 / (4.0f * wo.z * wi.z)) + albedo * (0.96f * INV_PI_F);
    r.pdf = 0.25f * pdf_spec + 0.75f * (wi.z * INV_PI_F);
    return r;
}
inline f3 sample_vndf(f3 wo, float alpha, float u1, float u2) {
    f3 vh = normalize(f3{alpha * wo.x, alpha * wo.y, wo.z});
    float lensq = vh.x * vh.x + vh.y * vh.y;
    f3 t1 = lensq > 0.0f ? f3{-vh.y, vh.x, 0.0f} * (1.0f / sqrtf(lensq)) : f3{1.0f, 0.0f, 0.0f};
    f3 t2 = cross(vh, t1);
    float r = sqrtf(u1);
    float s, c;
    sincos_xr(TWO_PI_F * u2, &s, &c);
    float p1 = r * c, p2 = r * s;
    float sh = 0.5f * (1.0f + vh.z);
    p2 = (1.0f - sh) * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1)) + sh * p2;
    f3 nh = t1 * p1 + t2 * p2 + vh * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2));
    return normalize(f3{alpha * nh.x, alpha * nh.y, fmaxf(0.0f, nh.z)});
}

// BSDF.hlsl:34-57 (SampleBSDF), :7-25 (SampleLambertian); corrected mode adds the
// GGX conductor (MAT_METALLIC) and GGX-over-Lambert (MAT_PLASTIC) lobes.
f3 sample_bsdf(bool compat, f3 n, const Material& mat, f3 wo_world, f3* wi_world, float* pdf_w,
               float* cos_theta, uint32_t& seed) {
    f3 f{0, 0, 0};
    *pdf_w = 0.0f; *cos_theta = 0.0f; *wi_world = f3{0, 0, 0};
    f3 T, B;
    branchless_onb(n, &T, &B);
    f3 wo_local = to_local(wo_world, T, B, n);
    f3 wi_local{0, 0, 0};
    if (mat.model == MAT_LAMBERTIAN) {
        f2 xi;
        xi.x = random_float(seed);
        xi.y = random_float(seed);
        wi_local = sample_hemisphere(xi);
        *cos_theta = wi_local.z;
        *pdf_w = *cos_theta * INV_PI_F;
        if (*cos_theta <= 0.0f) {
            *pdf_w = 0.0f;
            f = f3{0, 0, 0};
        } else {
            f = f3{mat.base[0], mat.base[1], mat.base[2]} * INV_PI_F;
        }
    } else if (!compat && (mat.model == MAT_METALLIC || mat.model == MAT_PLASTIC)) {
        float rough = fminf(fmaxf(mat.fuzz, 0.02f), 1.0f);
        float alpha = rough * rough;
        float us = mat.model == MAT_PLASTIC ? random_float(seed) : 0.0f;
        float u1 = random_float(seed), u2 = random_float(seed);
        if (mat.model == MAT_METALLIC || us < 0.25f) {
            if (wo_local.z > 0.0f) {
                f3 h = sample_vndf(wo_local, alpha, u1, u2);
                float oh = dot(wo_local, h);
                wi_local = h * (2.0f * oh) - wo_local;
            }
        } else {
            wi_local = sample_hemisphere(f2{u1, u2});
        }
        Lobe l = eval_material(mat, wo_local, wi_local);
        *cos_theta = wi_local.z;
        *pdf_w = l.pdf;
        f = l.f;
        if (!(l.pdf > 0.0f)) { *pdf_w = 0.0f; f = f3{0, 0, 0}; }
    }
    *wi_world = to_world(wi_local, T, B, n);
    return f;
}

// ----------------------------------------------------------------------------
// ReSTIRGICommon.hlsl:6-131
// ----------------------------------------------------------------------------
struct Sample {
    f3 x_view; uint32_t materialID;
    f3 n_view; uint32_t randSeed;
    f3 x_sample; float p_q;
    f3 n_sample; uint32_t pad1;   // corrected mode: bit 31 = has sample, bits 0..23 = oct12 code of n_sample
    f3 L_out; uint32_t pad2;
    f3 f; uint32_t pad3;
};
struct Reservoir { float w_sum; float W; uint32_t m; uint32_t pad; Sample s; };
static_assert(sizeof(Sample) == 96, "ReSTIRGISample is 96 B (ApplicationReSTIRGI.cpp:311)");
static_assert(sizeof(Reservoir) == 112, "ReSTIRGIReservoir is 112 B (ApplicationReSTIRGI.cpp:326)");

inline Sample init_sample() {
    Sample s;
    memset(&s, 0, sizeof(s));
    s.materialID = 0xFFFFFFFFu;
    return s;
}
inline Reservoir init_reservoir() {
    Reservoir r;
    r.w_sum = 0.0f; r.W = 0.0f; r.m = 0; r.pad = 0;
    r.s = init_sample();
    return r;
}
inline void update_reservoir(Reservoir& r, const Sample& s, float w_new, uint32_t& seed) {
    r.w_sum += w_new;
    r.m++;
    if (random_float(seed) < w_new / fmaxf(1e-10f, r.w_sum)) r.s = s;
}
inline void merge_reservoir(Reservoir& t, const Reservoir& src, float p_hat, uint32_t& seed) {
    uint32_t M0 = t.m;
    float w_new = p_hat * src.W * (float)src.m;
    update_reservoir(t, src.s, w_new, seed);
    t.m = M0 + src.m;
}
inline float p_hat_of(f3 L) { return length(L); }
inline bool is_similar(const Sample& cur, const Sample& his) {
    f3 d = cur.x_view - his.x_view;
    float dist2 = dot(d, d);
    if (dist2 > 0.1f) return false;
    if (dot(cur.n_view, his.n_view) < 0.8f) return false;
    if (cur.materialID != his.materialID) return false;
    return true;
}
inline bool is_similar_geo(f3 cp, f3 cn, f3 pp, f3 pn) {
    if (dot(cn, pn) < 0.8f) return false;
    f3 d = cp - pp;
    if (dot(d, d) > 0.1f) return false;
    return true;
}
inline float aces1(float x) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
    float v = (x * (a * x + b)) / (x * (c * x + d) + e);
    return fminf(fmaxf(v, 0.0f), 1.0f);
}
// ReSTIRGITemporalReuse.rgen.hlsl:33-40
inline float eval_target(const Sample& s, f3 x_curr, f3 n_curr) {
    f3 wi = normalize(s.x_sample - x_curr);
    float c = dot(n_curr, wi);
    if (c <= 0.0f) return 0.0f;
    return length(s.L_out);
}

inline uint8_t to_unorm8(float v) {
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    return (uint8_t)(int)(v * 255.0f + 0.5f);
}

// Bilinear sampling with clamp to edge of an RGBA8 UNORM texture (the reference's
// sampler, src/Vulkan/XVKSampler.h:11-27, on R8G8B8A8_UNORM images), the same
// operations in the same order as the kernels' tex_bilinear.
inline f3 tex_bilinear(const Scene& s, uint32_t t, f2 uv) {
    const uint32_t off = s.tex_info[3 * (size_t)t], wu = s.tex_info[3 * (size_t)t + 1], hu = s.tex_info[3 * (size_t)t + 2];
    const int w = (int)wu, h = (int)hu;
    float x = uv.x * (float)w - 0.5f, y = uv.y * (float)h - 0.5f;
    if (!std::isfinite(x)) x = 0.0f;
    if (!std::isfinite(y)) y = 0.0f;
    x = fminf(fmaxf(x, -1.0f), (float)w);
    y = fminf(fmaxf(y, -1.0f), (float)h);
    const float x0f = floorf(x), y0f = floorf(y);
    const float fx = x - x0f, fy = y - y0f;
    const int x0 = (int)x0f, y0 = (int)y0f;
    const int xa = std::min(std::max(x0, 0), w - 1), xb = std::min(std::max(x0 + 1, 0), w - 1);
    const int ya = std::min(std::max(y0, 0), h - 1), yb = std::min(std::max(y0 + 1, 0), h - 1);
    auto texel = [&](int xx, int yy, int ch) {
        const uint32_t v = s.texels[off + (size_t)yy * w + xx];
        return (float)((v >> (8 * ch)) & 255u) / 255.0f;
    };
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    float c[3];
    for (int ch = 0; ch < 3; ch++)
        c[ch] = (texel(xa, ya, ch) * gx + texel(xb, ya, ch) * fx) * gy + (texel(xa, yb, ch) * gx + texel(xb, yb, ch) * fx) * fy;
    return f3{c[0], c[1], c[2]};
}

// Material m at texture coordinate uv: a base-colour texture replaces the base
// colour's RGB (BSDF.hlsl:22-23).
inline Material resolve_material(const Scene& s, uint32_t m, f2 uv) {
    Material r = s.mat[m];
    const uint32_t n_tex = (uint32_t)(s.tex_info.size() / 3);
    if (r.tex >= 0 && (uint32_t)r.tex < n_tex) {
        const f3 c = tex_bilinear(s, (uint32_t)r.tex, uv);
        r.base[0] = c.x; r.base[1] = c.y; r.base[2] = c.z;
    }
    return r;
}

void build_lights(Scene& s) {
    std::vector<float> area, power;
    for (uint32_t t = 0; t < s.ntri; t++) {
        const int32_t mi = vert_mat(s, s.idx[(size_t)t * 3]);
        if (mi < 0 || (uint32_t)mi >= s.nm || s.mat[mi].model != MAT_DIFFUSE_LIGHT) continue;
        const f3 cr = cross(s.p2[t] - s.p0[t], s.p1[t] - s.p0[t]);
        const float a = 0.5f * sqrtf(dot(cr, cr));
        const float lr = s.mat[mi].base[0] * 4.0f, lg = s.mat[mi].base[1] * 4.0f, lb = s.mat[mi].base[2] * 4.0f;
        const float lum = 0.2126f * lr + 0.7152f * lg + 0.0722f * lb;
        const float pw = a * lum;
        if (!(pw > 0.0f) || !std::isfinite(pw)) continue;
        s.light_prim.push_back(t);
        area.push_back(a);
        power.push_back(pw);
    }
    const size_t n = s.light_prim.size();
    s.prim_light_pdf.assign(s.ntri, 0.0f);
    if (n == 0) return;
    float total = 0.0f;
    for (float pw : power) total = total + pw;
    s.light_pmf.resize(n);
    s.light_cdf.resize(n);
    float run = 0.0f;
    for (size_t k = 0; k < n; k++) {
        s.light_pmf[k] = power[k] / total;
        run = run + s.light_pmf[k];
        s.light_cdf[k] = run;
        s.prim_light_pdf[s.light_prim[k]] = s.light_pmf[k] / area[k];
    }
    s.light_cdf[n - 1] = 1.0f;
}

// Next-event estimation of a training path's vertex x (shading normal n,
// geometric normal g facing wo): light by power (binary search of the CDF),
// uniform point (square-root parameterisation), balance heuristic against the
// BSDF sampling pdf; the contribution is added when the shadow ray is clear.
// Consumes three random numbers in every case.
f3 next_event(const Scene& sc, const Material& mat, f3 x, f3 n, f3 g, f3 wo, f3 thr, uint32_t& rng) {
    const f3 zero{0.0f, 0.0f, 0.0f};
    const float u0 = random_float(rng), u1 = random_float(rng), u2 = random_float(rng);
    const uint32_t nl_count = (uint32_t)sc.light_prim.size();
    if (nl_count == 0) return zero;
    uint32_t lo = 0, hi = nl_count - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (u0 < sc.light_cdf[mid]) hi = mid;
        else lo = mid + 1;
    }
    const uint32_t prim = sc.light_prim[lo];
    const f3 p0 = sc.p0[prim], p1 = sc.p1[prim], p2 = sc.p2[prim];
    const float su = sqrtf(u1);
    const float b0 = 1.0f - su, b1 = u2 * su, b2 = 1.0f - b0 - b1;
    const f3 y = p0 * b0 + p1 * b1 + p2 * b2;
    const f3 nl = normalize(cross(p2 - p0, p1 - p0));
    const f3 dv = y - x;
    const float dist2 = dot(dv, dv);
    const float dist = sqrtf(dist2);
    if (!(dist > 0.05f)) return zero;
    const f3 wi = dv * (1.0f / dist);
    const float cos_l = fabsf(dot(nl, wi));
    if (!(cos_l > 1e-6f)) return zero;
    f3 T, B;
    branchless_onb(n, &T, &B);
    const f3 wil = to_local(wi, T, B, n);
    if (!(wil.z > 0.0f)) return zero;
    const Lobe lb = eval_material(mat, to_local(wo, T, B, n), wil);
    const float pdf_l = sc.prim_light_pdf[prim] * dist2 / cos_l;
    const uint32_t li0 = sc.idx[(size_t)prim * 3], li1 = sc.idx[(size_t)prim * 3 + 1], li2 = sc.idx[(size_t)prim * 3 + 2];
    f2 luv{0.0f, 0.0f};
    if (!sc.tex_info.empty()) {
        const f2 t0 = vert_uv(sc, li0), t1 = vert_uv(sc, li1), t2 = vert_uv(sc, li2);
        luv = f2{t0.x * b0 + t1.x * b1 + t2.x * b2, t0.y * b0 + t1.y * b1 + t2.y * b2};
    }
    const Material lm = resolve_material(sc, (uint32_t)vert_mat(sc, li0), luv);
    const f3 Le = f3{lm.base[0], lm.base[1], lm.base[2]} * 4.0f;
    const f3 contrib = thr * Le * lb.f * (wil.z / (pdf_l + lb.pdf));
    if (!(contrib.x + contrib.y + contrib.z > 0.0f)) return zero;
    const f3 off = dot(wi, g) > 0.0f ? g : -g;
    const Hit h = trace(sc, x + off * 0.01f, wi, 0.0f, dist - 0.02f, true);
    return h.prim >= 0 ? zero : contrib;
}

// ----------------------------------------------------------------------------
// The renderer: initial sample, temporal, spatial (ApplicationReSTIRGI.cpp:150-275)
// ----------------------------------------------------------------------------
struct Renderer {
    const Scene* sc;
    OrParams P;
    uint32_t W, H, N;
    bool compat;
    std::vector<Sample> samples;
    std::vector<Reservoir> temporal, spatial;
    std::vector<f4> gpos;                 // GBufferPos (x_view, valid)
    std::vector<f2> motion;               // GMotionVector after RG16F rounding
    std::vector<uint32_t> gnrm_code;      // corrected mode: oct16 code of n_view
    std::vector<f4> prev_gpos;            // corrected mode: previous frame
    std::vector<uint32_t> prev_code, prev_mat;
    std::vector<f3> le0, thr0;
    std::vector<f4> hdr, pt;
    std::vector<f2> gb_uv;                // texture coordinate of the visible point (textured scenes)
    std::vector<uint8_t> ldr;
    std::vector<uint32_t> written;
    // learned radiance cache (corrected mode, or_renderer_set_cache): per pixel the
    // query record (8 words) and training record (12 words) of the last frame
    bool cache_on = false;
    uint32_t cache_sel_n = 0;      // training pixels of this frame (adapted after every frame)
    uint32_t cache_target = 0;     // training records wanted per frame
    void* nrc = nullptr;
    std::vector<uint32_t> cache_q, cache_t;
    std::vector<uint8_t> cache_q_valid, cache_t_valid;
};

inline uint32_t unorm8_of(float v) { return (uint32_t)(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f + 0.5f); }

// Training pixels of a frame: (pixel * (2^31 - 1) + off) mod N < sel_n, with
// off = frame * 2654435761 mod N -- a permutation of the pixels per frame.
inline bool cache_training_pixel(const Renderer& R, uint32_t p, uint32_t frame) {
    if (R.cache_sel_n == 0) return false;
    const uint64_t off = ((uint64_t)frame * 2654435761ull) % (uint64_t)R.N;
    return ((uint64_t)p * 2147483647ull + off) % (uint64_t)R.N < R.cache_sel_n;
}

void write_output(Renderer& R, uint32_t p, f3 hdr_c, bool tonemap) {
    f3 c = hdr_c;
    if (tonemap) {
        c = f3{aces1(c.x), aces1(c.y), aces1(c.z)};
        const float g = (float)(1.0 / 2.2);
        c = f3{powf(c.x, g), powf(c.y, g), powf(c.z, g)};
    }
    R.hdr[p] = f4{hdr_c.x, hdr_c.y, hdr_c.z, 1.0f};
    R.ldr[4 * p + 0] = to_unorm8(c.x);
    R.ldr[4 * p + 1] = to_unorm8(c.y);
    R.ldr[4 * p + 2] = to_unorm8(c.z);
    R.ldr[4 * p + 3] = 255;
    R.written[p] = 1;
}

// ReSTIRGIInitialSample.rgen.hlsl:35-214 for one pixel.
void initial_pixel(Renderer& R, uint32_t x, uint32_t y, const OrUBO& u) {
    const Scene& sc = *R.sc;
    const bool compat = R.compat;
    const uint32_t p = y * R.W + x;
    uint32_t rng = pass_rng(compat, x, y, R.W, u.current_frame, PASS_INITIAL, R.P.seed);
    float ox = random_float(rng);
    float oy = random_float(rng);
    f2 pixel{(float)x + ox, (float)y + oy};
    f2 uv{(pixel.x / (float)R.W) * 2.0f - 1.0f, (pixel.y / (float)R.H) * 2.0f - 1.0f};
    f4 origin = mul(u.view_inverse, f4{0, 0, 0, 1});
    f4 target = mul(u.projection_inverse, f4{uv.x, uv.y, 1, 1});
    f3 tn = normalize(xyz(target));
    f3 direction = normalize(xyz(mul(u.view_inverse, f4{tn.x, tn.y, tn.z, 0.0f})));
    f3 o = xyz(origin);

    f3 throughput{1, 1, 1}, throughput0{1, 1, 1};
    f3 x_view{0, 0, 0}, n_view{0, 0, 0}, x_sample{0, 0, 0}, n_sample{0, 0, 0}, L_out{0, 0, 0}, f_{0, 0, 0};
    f3 le0{0, 0, 0};
    float p_q = 0.0f;
    uint32_t mat_idx = 0xFFFFFFFFu, rand_seed = 0;
    f2 test_uv{0, 0};
    bool valid = false, has_sample = false;
    bool cache_query = false, cache_train = false;
    uint32_t rec[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const bool cache = !compat && R.cache_on;
    float prev_pdf = 0.0f;   // cache training paths: sampling pdf of the previous vertex (MIS)
    const f3 sky{1, 1, 1};
    for (uint32_t bounce = 0;; bounce++) {
        if (bounce == u.number_of_bounces) break;
        Hit h = trace(sc, o, direction, 0.0001f, 10000.0f, false);
        Payload pl;
        pl.mat = -1;
        if (h.prim >= 0) pl = closest_hit(sc, h);
        if (pl.mat == -1) {
            if (u.has_sky_box) L_out = L_out + throughput * sky;
            if (bounce == 0 && u.has_sky_box) le0 = sky;
            if (bounce == 1) {
                x_sample = o + direction * 1000.0f;
                n_sample = -direction;
                has_sample = true;
            }
            break;
        }
        const Material mat = resolve_material(sc, (uint32_t)pl.mat, pl.uv);
        if (bounce == 0 && !sc.tex_info.empty()) R.gb_uv[p] = pl.uv;
        if (!compat) {
            f3 wo = -direction;
            if (dot(pl.geo_normal, wo) < 0.0f) pl.geo_normal = -pl.geo_normal;
            if (dot(pl.normal, pl.geo_normal) < 0.0f) pl.normal = -pl.normal;
        }
        if (mat.model == MAT_DIFFUSE_LIGHT) {
            // reference mode emits the light's untextured base colour (:117-121: mat.baseColor,
            // not SampleDiffuseLight); corrected mode takes its base-colour texture
            const Material& em = compat ? sc.mat[(uint32_t)pl.mat] : mat;
            f3 Le = f3{em.base[0], em.base[1], em.base[2]} * 4.0f;
            f3 term = throughput * f3{em.base[0], em.base[1], em.base[2]} * 4.0f;
            if (cache && bounce >= 2) {
                // balance heuristic against the previous vertex's next-event estimate
                const float lp = sc.light_prim.empty() ? 0.0f : sc.prim_light_pdf[h.prim];
                const float cos_l = fabsf(dot(pl.geo_normal, direction));
                const float pdf_l = (lp > 0.0f && cos_l > 1e-6f && pl.hit_t > 0.05f)
                                        ? lp * (pl.hit_t * pl.hit_t) / cos_l : 0.0f;
                term = term * (prev_pdf / (prev_pdf + pdf_l));
            }
            L_out = L_out + term;
            if (bounce == 1) { x_sample = pl.pos; n_sample = pl.normal; has_sample = true; }
            if (bounce == 0) { x_view = pl.pos; n_view = pl.normal; le0 = Le; }
            break;
        }
        float pdf = 0.0f, cos_theta = 0.0f;
        f3 wi{0, 0, 0};
        f3 wo = -direction;
        if (bounce == 1) { x_sample = pl.pos; n_sample = pl.normal; has_sample = true; }
        uint32_t seed_this = rng;
        if (cache && bounce >= 1 && bounce + 1 < u.number_of_bounces &&
            (bounce >= 2 || cache_training_pixel(R, p, u.current_frame)))
            L_out = L_out + next_event(sc, mat, pl.pos, pl.normal, pl.geo_normal, wo, throughput, rng);
        f3 f = sample_bsdf(compat, pl.normal, mat, wo, &wi, &pdf, &cos_theta, rng);
        f3 factor = f * cos_theta / f3{pdf, pdf, pdf};
        if (!compat && !(pdf > 0.0f)) factor = f3{0, 0, 0};
        if (bounce == 0) {
            valid = true;
            x_view = pl.pos; n_view = pl.normal;
            rand_seed = seed_this;
            mat_idx = (uint32_t)pl.mat;
            throughput0 = throughput0 * factor;
            test_uv = pl.uv;
            p_q = pdf;
            f_ = f;
        } else {
            throughput = throughput * factor;
        }
        if (cache && bounce == 1) {
            // the path ends here into the cache unless the pixel trains it
            cache_query = true;
            cache_train = cache_training_pixel(R, p, u.current_frame);
            rec[0] = f32_bits(pl.pos.x); rec[1] = f32_bits(pl.pos.y); rec[2] = f32_bits(pl.pos.z); rec[3] = p;
            rec[4] = oct_encode(pl.normal, 16);
            rec[5] = oct_encode(wo, 16);
            rec[6] = unorm8_of(mat.base[0]) | (unorm8_of(mat.base[1]) << 8) | (unorm8_of(mat.base[2]) << 16) |
                     ((mat.model & 255u) << 24);
            rec[7] = f32_bits(mat.fuzz);
        }
        if (!compat && !(pdf > 0.0f)) break;   // corrected mode: an absorbed path ends here
        if (cache && bounce == 1 && !cache_train) break;
        if (bounce > 3) {
            float pr = fmaxf(throughput.x, fmaxf(throughput.y, throughput.z));
            if (random_float(rng) > pr) break;
            throughput = throughput * (1.0f / pr);
        }
        f3 hit_position = o + direction * pl.hit_t;
        f3 gn = pl.geo_normal;
        f3 off = dot(wi, gn) > 0.0f ? gn : -gn;
        o = hit_position + off * 0.01f;
        direction = wi;
        prev_pdf = pdf;
    }
    if (cache) {
        R.cache_q_valid[p] = cache_query;
        R.cache_t_valid[p] = cache_train;
        if (cache_query) {
            std::memcpy(&R.cache_q[(size_t)p * 8], rec, sizeof(rec));
            if (cache_train) {
                // the suffix radiance (bounces >= 2) is the training target
                std::memcpy(&R.cache_t[(size_t)p * 12], rec, sizeof(rec));
                R.cache_t[(size_t)p * 12 + 8] = f32_bits(L_out.x);
                R.cache_t[(size_t)p * 12 + 9] = f32_bits(L_out.y);
                R.cache_t[(size_t)p * 12 + 10] = f32_bits(L_out.z);
                R.cache_t[(size_t)p * 12 + 11] = 0u;
            }
            // the candidate takes the cache's radiance (clamped at zero; non-finite -> 0)
            f3 Lc{0.0f, 0.0f, 0.0f};
            if (R.nrc) {
                float pred[3];
                or_nrc_infer(R.nrc, rec, 1, pred, 0);
                Lc = f3{fmaxf(pred[0], 0.0f), fmaxf(pred[1], 0.0f), fmaxf(pred[2], 0.0f)};
                if (!std::isfinite(Lc.x + Lc.y + Lc.z)) Lc = f3{0.0f, 0.0f, 0.0f};
            }
            L_out = f3{0.0f, 0.0f, 0.0f} + Lc;
        }
    }
    Sample s;
    s.x_view = x_view; s.n_view = n_view; s.x_sample = x_sample; s.n_sample = n_sample;
    s.L_out = L_out; s.materialID = mat_idx; s.randSeed = rand_seed; s.p_q = p_q; s.f = f_;
    s.pad1 = 0; s.pad2 = 0; s.pad3 = 0;
    R.le0[p] = le0;
    R.thr0[p] = throughput0;
    if (valid) {
        R.gpos[p] = f4{x_view.x, x_view.y, x_view.z, 1.0f};
        f2 cur_uv{((float)x + 0.5f) / (float)R.W, ((float)y + 0.5f) / (float)R.H};
        f2 prev_uv = world_to_screen_uv(x_view, u.view_prev, u.projection_prev);
        f2 mv{cur_uv.x - prev_uv.x, cur_uv.y - prev_uv.y};
        R.motion[p] = compat ? f2{half_round(mv.x), half_round(mv.y)} : mv;
    } else {
        R.gpos[p] = f4{0, 0, 0, 0};
        R.motion[p] = f2{0, 0};
        s.L_out = f3{0, 0, 0};
        s.n_sample = f3{0, 0, 0};
    }
    if (!compat) {
        // storage quantisation of the corrected-mode layout
        if (valid) {
            uint32_t c16 = oct_encode(s.n_view, 16);
            R.gnrm_code[p] = c16;
            s.n_view = oct_decode(c16, 16);
            if (has_sample) {
                uint32_t c12 = oct_encode(s.n_sample, 12);
                s.pad1 = c12 | 0x80000000u;
                s.n_sample = oct_decode(c12, 12);
            } else {
                s.pad1 = 0; s.n_sample = f3{0, 0, 0}; s.x_sample = f3{0, 0, 0}; s.L_out = f3{0, 0, 0};
            }
        } else {
            R.gnrm_code[p] = 0;
            s.pad1 = 0;
            s.x_view = f3{0, 0, 0};   // the corrected layout keeps no position for invalid pixels
            s.n_view = f3{0, 0, 0};
        }
        s.f = f3{0, 0, 0};
        s.randSeed = R.gnrm_code[p];   // corrected layout keeps the oct16 code of n_view here
    }
    R.samples[p] = s;
}

// Corrected-mode target function: |L f(wo, wi) cos| with the BSDF of the
// pixel's visible point (position, normal, material, wo towards the camera) --
// the factor the reservoir's estimate is shaded with, so W absorbs it and a
// glossy lobe cannot turn the resampled estimate into fireflies.  Reference mode
// keeps the reference's |L| (ReSTIRGITemporalReuse.rgen.hlsl:33-40,
// ReSTIRGISpatialReuse.rgen.hlsl:91-133), which is exact for its Lambertian-only
// scenes up to the cosine.
// Near-specular visible points (GGX conductor or plastic coat with roughness
// below 0.25) take no temporal or spatial reuse in corrected mode: their
// reservoir is the initial candidate alone (the path-traced estimate), since a
// reconnection sample from another pixel lands in their sharp lobe with a
// target far above the one it was resampled for.
constexpr float kReuseMinRoughness = 0.25f;

struct PixelShading {
    Material m;
    f3 x, n, wo, T, B;
    bool reuse;
};
inline PixelShading pixel_shading(const Renderer& R, const Sample& s, const OrUBO& u, uint32_t p) {
    PixelShading P;
    P.m = resolve_material(*R.sc, s.materialID, R.sc->tex_info.empty() ? f2{0.0f, 0.0f} : R.gb_uv[p]);
    P.x = s.x_view;
    P.n = s.n_view;
    f3 cam{u.view_inverse[12], u.view_inverse[13], u.view_inverse[14]};   // translation column (column-major)
    P.wo = normalize(cam - P.x);
    branchless_onb(P.n, &P.T, &P.B);
    const bool glossy = (P.m.model == MAT_METALLIC || P.m.model == MAT_PLASTIC) && P.m.fuzz < kReuseMinRoughness;
    P.reuse = !glossy;
    return P;
}
inline float target_corrected(const PixelShading& P, f3 xs, f3 L) {
    f3 wi = normalize(xs - P.x);
    float c = dot(P.n, wi);
    if (c <= 0.0f) return 0.0f;
    f3 f = eval_material(P.m, to_local(P.wo, P.T, P.B, P.n), to_local(wi, P.T, P.B, P.n)).f;
    return length(L * f * c);
}

void shade_output(Renderer& R, uint32_t p, const Reservoir& r, const Sample& s_new, const OrUBO& u) {
    f3 color{0, 0, 0};
    if (r.W > 0.0f) {
        f3 x_curr = s_new.x_view;
        f3 n_curr = s_new.n_view;
        f3 wi = normalize(r.s.x_sample - x_curr);
        float cos_theta = fmaxf(0.0f, dot(n_curr, wi));
        f3 f = r.s.f;
        if (!R.compat) {
            // corrected mode: the pixel's BSDF along the reconnection direction; a
            // near-specular pixel (no reuse) takes the path tracer's ratio f cos / pdf
            // at that one direction (the sampled direction left from a point offset
            // along the normal, and in a sharp lobe f alone varies by orders of
            // magnitude over that angle)
            const PixelShading P = pixel_shading(R, s_new, u, p);
            const Lobe lb = eval_material(P.m, to_local(P.wo, P.T, P.B, P.n), to_local(wi, P.T, P.B, P.n));
            if (P.reuse) color = r.s.L_out * r.W * lb.f * cos_theta;
            else if (lb.pdf > 0.0f) color = r.s.L_out * lb.f * (cos_theta / lb.pdf);
            write_output(R, p, color, true);
            return;
        }
        color = r.s.L_out * r.W * f * cos_theta;
    }
    write_output(R, p, color, true);
}

// ReSTIRGITemporalReuse.rgen.hlsl:41-151
void temporal_pixel(Renderer& R, uint32_t x, uint32_t y, const OrUBO& u, bool out_here) {
    const bool compat = R.compat;
    const uint32_t p = y * R.W + x, N = R.N;
    uint32_t rng = pass_rng(compat, x, y, R.W, u.current_frame, PASS_TEMPORAL, R.P.seed);
    uint32_t pingpong = u.current_frame % 2u;
    uint32_t cur = pingpong * N, prev = (1u - pingpong) * N;
    const Sample s_new = R.samples[p];
    Reservoir r_prev = init_reservoir();
    if (compat) {
        if (length(s_new.n_sample) == 0.0f) {
            Reservoir e = init_reservoir();
            R.temporal[cur + p] = e;
            R.spatial[cur + p] = e;
            return;
        }
    } else {
        bool valid = s_new.materialID != 0xFFFFFFFFu;
        bool hs = (s_new.pad1 & 0x80000000u) != 0;
        if (!valid || !hs) {
            R.temporal[cur + p] = init_reservoir();
            if (out_here) write_output(R, p, valid ? f3{0, 0, 0} : R.le0[p], true);
            return;
        }
    }
    bool found = false;
    if (compat) {
        f2 mv = R.motion[p];
        f2 uvc{((float)x + 0.5f) / (float)R.W, ((float)y + 0.5f) / (float)R.H};
        f2 puv{uvc.x - mv.x, uvc.y - mv.y};
        // int2(prevUV * size) truncates toward zero: in range iff -1 < v < size
        float fx = puv.x * (float)R.W, fy = puv.y * (float)R.H;
        if (fx > -1.0f && fx < (float)R.W && fy > -1.0f && fy < (float)R.H) {
            uint32_t q = (uint32_t)(int32_t)fy * R.W + (uint32_t)(int32_t)fx;
            // the "previous" G-buffer aliases the current one (ApplicationReSTIRGI.cpp:367-372)
            if (R.gpos[q].w != 0.0f) {
                r_prev = R.temporal[prev + q];
                found = true;
            } else {
                R.spatial[cur + p] = init_reservoir();
            }
        }
        if (!R.P.temporal_on) found = false;
    } else if (R.P.temporal_on && pixel_shading(R, s_new, u, p).reuse) {
        f2 puv = world_to_screen_uv(s_new.x_view, u.view_prev, u.projection_prev);
        float fx = floorf(puv.x * (float)R.W), fy = floorf(puv.y * (float)R.H);
        if (fx >= 0.0f && fx < (float)R.W && fy >= 0.0f && fy < (float)R.H) {
            uint32_t q = (uint32_t)fy * R.W + (uint32_t)fx;
            if (R.prev_mat[q] == s_new.materialID &&
                is_similar_geo(s_new.x_view, s_new.n_view, xyz(R.prev_gpos[q]), oct_decode(R.prev_code[q], 16))) {
                r_prev = R.temporal[prev + q];
                found = true;
            }
        }
    }
    f3 x_curr = s_new.x_view;
    f3 n_curr = normalize(s_new.n_view);
    PixelShading P{};
    if (!compat) P = pixel_shading(R, s_new, u, p);
    auto target = [&](const Sample& smp) {
        return compat ? eval_target(smp, x_curr, n_curr) : target_corrected(P, smp.x_sample, smp.L_out);
    };
    Reservoir r_final = init_reservoir();
    float tp_new = target(s_new);
    float w_new = (s_new.p_q > 1e-6f) ? (tp_new / s_new.p_q) : 0.0f;
    update_reservoir(r_final, s_new, w_new, rng);
    if (found) {
        float tp_prev = target(r_prev.s);
        merge_reservoir(r_final, r_prev, tp_prev, rng);
    } else {
        r_final.m = 1;
    }
    uint32_t cap = compat ? 30u : R.P.m_cap_temporal;
    if (r_final.m > cap) {
        r_final.w_sum *= (float)cap / (float)r_final.m;
        r_final.m = cap;
    }
    float tp_final = target(r_final.s);
    if (tp_final > 1e-6f && r_final.m > 0) r_final.W = r_final.w_sum / ((float)r_final.m * tp_final);
    else r_final.W = 0.0f;
    R.temporal[cur + p] = r_final;
    if (out_here) shade_output(R, p, r_final, s_new, u);
}

// ReSTIRGISpatialReuse.rgen.hlsl:35-42
inline uint32_t neighbor_index(uint32_t x, uint32_t y, uint32_t W, uint32_t H, float max_r, uint32_t& seed) {
    float randa = random_float(seed) * 2.0f * PI_F;
    float randr = sqrtf(random_float(seed)) * max_r;
    float s, c;
    sincos_xr(randa, &s, &c);
    int32_t ox = (int32_t)floorf(c * randr), oy = (int32_t)floorf(s * randr);
    int32_t cx = std::min(std::max((int32_t)x + ox, 0), (int32_t)W - 1);
    int32_t cy = std::min(std::max((int32_t)y + oy, 0), (int32_t)H - 1);
    return (uint32_t)cy * W + (uint32_t)cx;
}

// ReSTIRGISpatialReuse.rgen.hlsl:64-183
void spatial_pixel(Renderer& R, uint32_t x, uint32_t y, const OrUBO& u) {
    const bool compat = R.compat;
    const uint32_t p = y * R.W + x, N = R.N;
    uint32_t rng = pass_rng(compat, x, y, R.W, u.current_frame, PASS_SPATIAL, R.P.seed);
    uint32_t pingpong = u.current_frame % 2u;
    uint32_t read_off = pingpong * N;
    uint32_t write_off = compat ? (1u - pingpong) * N : 0u;
    const Sample s_new = R.samples[p];
    if (compat) {
        // background black, lights white, whatever `reuse` says (:80-89); only the
        // shaded colour at the end is gated by it (:179-182)
        if (length(s_new.n_view) == 0.0f) {
            write_output(R, p, f3{0, 0, 0}, false);
            return;
        }
        if (length(s_new.n_sample) == 0.0f) {
            write_output(R, p, f3{1, 1, 1}, false);
            return;
        }
    } else {
        bool valid = s_new.materialID != 0xFFFFFFFFu;
        bool hs = (s_new.pad1 & 0x80000000u) != 0;
        if (!valid || !hs) {
            R.spatial[p] = init_reservoir();
            write_output(R, p, valid ? f3{0, 0, 0} : R.le0[p], true);
            return;
        }
    }
    Reservoir center = R.temporal[read_off + p];
    Reservoir r_s = init_reservoir();
    PixelShading P{};
    if (!compat) P = pixel_shading(R, s_new, u, p);
    auto target = [&](const Sample& smp) {
        return compat ? p_hat_of(smp.L_out) : target_corrected(P, smp.x_sample, smp.L_out);
    };
    const uint32_t nn = compat ? 6u : (P.reuse ? R.P.n_neighbours : 0u);
    const float radius = compat ? 5.0f : R.P.radius_px;
    // reference: one stream, each pick followed by its merge's draw; corrected:
    // the first 2 nn draws pick the neighbours and the merges draw after them
    uint32_t rng_pick = rng;
    if (!compat)
        for (uint32_t k = 0; k < 2u * nn; k++) next_random(rng);
    uint32_t& pick = compat ? rng : rng_pick;
    merge_reservoir(r_s, center, target(center.s), rng);
    for (uint32_t i = 0; i < nn; i++) {
        uint32_t nb = neighbor_index(x, y, R.W, R.H, radius, pick);
        const Sample& s_nb = R.samples[nb];
        if (compat) {
            if (length(s_nb.n_view) == 0.0f || !is_similar(s_new, s_nb)) continue;
        } else {
            if (s_nb.materialID == 0xFFFFFFFFu || !is_similar(s_new, s_nb)) continue;
        }
        const Reservoir& r_nb = R.temporal[read_off + nb];
        f3 x_s = r_nb.s.x_sample, n_s = r_nb.s.n_sample;
        f3 v_orig = s_nb.x_view - x_s;
        float d2o = dot(v_orig, v_orig);
        f3 v_curr = s_new.x_view - x_s;
        float d2c = dot(v_curr, v_curr);
        float jac = 1.0f;
        if (d2o > 1e-6f && d2c > 1e-6f) {
            f3 dir_o = v_orig * (1.0f / sqrtf(d2o));
            f3 dir_c = v_curr * (1.0f / sqrtf(d2c));
            float cpo = fmaxf(0.0f, dot(n_s, dir_o));
            float cpc = fmaxf(0.0f, dot(n_s, dir_c));
            if (cpo > 1e-6f) jac = (cpc * d2o) / (cpo * d2c);
        }
        jac = fminf(fmaxf(jac, 0.1f), 10.0f);
        float ph = target(r_nb.s) * jac;
        bool occluded = false;
        if (!compat && R.P.visibility && ph > 0.0f) {
            // corrected CheckVisibility (ReSTIRGISpatialReuse.rgen.hlsl:44-62): from
            // the centre pixel's visible point, not the selected sample's
            f3 from = s_new.x_view, to = x_s;
            f3 dir = to - from;
            float dist = length(dir);
            f3 ro = from + s_new.n_view * 0.01f;
            Hit hh = trace(*R.sc, ro, normalize(dir), 0.0f, dist - 0.01f, true);
            occluded = hh.prim >= 0;
            if (occluded) ph = 0.0f;
        }
        if (occluded) {
            // corrected: an occluded neighbour merges with weight 0 (its M below)
            const uint32_t M0 = r_s.m;
            update_reservoir(r_s, r_nb.s, 0.0f, rng);
            r_s.m = M0 + r_nb.m;
        } else {
            merge_reservoir(r_s, r_nb, ph, rng);
        }
        // reference: a neighbour whose weight is zero does not count towards M
        // (ReSTIRGISpatialReuse.rgen.hlsl:140-143); corrected: every similar
        // neighbour counts (1/M normalisation) except one whose sample is occluded
        if (compat ? ph == 0.0f : occluded) r_s.m -= r_nb.m;
    }
    if (compat) {
        r_s.m = std::min(r_s.m, 300u);
    } else if (r_s.m > R.P.m_cap_spatial) {
        r_s.w_sum *= (float)R.P.m_cap_spatial / (float)r_s.m;
        r_s.m = R.P.m_cap_spatial;
    }
    float phf = target(r_s.s);
    if (phf > 1e-6f && r_s.m > 0) r_s.W = r_s.w_sum / ((float)r_s.m * phf);
    else r_s.W = 0.0f;
    R.spatial[write_off + p] = r_s;
    if (compat) {
        if (u.reuse) shade_output(R, p, r_s, s_new, u);
    } else {
        shade_output(R, p, r_s, s_new, u);
    }
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

uint32_t or_init_random_seed(uint32_t x, uint32_t y, uint32_t width, uint32_t frame) {
    return init_random_seed(x, y, width, frame);
}
void or_random_sequence(uint32_t state, uint32_t n, uint32_t* out_u32, float* out_f) {
    uint32_t s1 = state, s2 = state;
    for (uint32_t i = 0; i < n; i++) {
        if (out_u32) out_u32[i] = next_random(s1);
        if (out_f) out_f[i] = random_float(s2);
    }
}
void or_sincos(const float* a, uint32_t n, float* s, float* c) {
    for (uint32_t i = 0; i < n; i++) sincos_xr(a[i], &s[i], &c[i]);
}
// ---- the restated helpers one by one (checked against the reference's own
//      source, compiled by oracle/refpin, on the same inputs) ----
void or_units_onb(const float* n3, uint32_t n, float* out6) {
    for (uint32_t i = 0; i < n; i++) {
        f3 b1, b2;
        branchless_onb(f3{n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]}, &b1, &b2);
        float* o = out6 + 6 * (size_t)i;
        o[0] = b1.x; o[1] = b1.y; o[2] = b1.z; o[3] = b2.x; o[4] = b2.y; o[5] = b2.z;
    }
}
void or_units_sample_hemisphere(const float* xi2, uint32_t n, float* out3) {
    for (uint32_t i = 0; i < n; i++) {
        f3 v = sample_hemisphere(f2{xi2[2 * i], xi2[2 * i + 1]});
        out3[3 * i] = v.x; out3[3 * i + 1] = v.y; out3[3 * i + 2] = v.z;
    }
}
// reference-mode SampleBSDF: out 9 words {f.rgb, wi.xyz, pdf, cos, seed after}
void or_units_sample_bsdf(const float* n3, const float* wo3, const uint32_t* materials8, const uint32_t* seeds,
                          uint32_t n, float* out9) {
    for (uint32_t i = 0; i < n; i++) {
        Material m;
        memcpy(&m, materials8 + 8 * (size_t)i, 32);
        f3 wi;
        float pdf, ct;
        uint32_t seed = seeds[i];
        f3 f = sample_bsdf(true, f3{n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]}, m,
                           f3{wo3[3 * i], wo3[3 * i + 1], wo3[3 * i + 2]}, &wi, &pdf, &ct, seed);
        float* o = out9 + 9 * (size_t)i;
        o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = wi.x; o[4] = wi.y; o[5] = wi.z; o[6] = pdf; o[7] = ct;
        memcpy(&o[8], &seed, 4);
    }
}
void or_units_update_list(const uint32_t* samples24, const float* weights, uint32_t n, uint32_t k,
                          const uint32_t* seeds, uint32_t* out28, uint32_t* seeds_out) {
    for (uint32_t i = 0; i < n; i++) {
        Reservoir r = init_reservoir();
        uint32_t seed = seeds[i];
        for (uint32_t j = 0; j < k; j++) {
            Sample smp;
            memcpy(&smp, samples24 + ((size_t)i * k + j) * 24, 96);
            update_reservoir(r, smp, weights[(size_t)i * k + j], seed);
        }
        memcpy(out28 + (size_t)i * 28, &r, 112);
        seeds_out[i] = seed;
    }
}
void or_units_merge_list(const uint32_t* res28, const float* p_hats, uint32_t n, uint32_t k, const uint32_t* seeds,
                         uint32_t* out28, uint32_t* seeds_out) {
    for (uint32_t i = 0; i < n; i++) {
        Reservoir t = init_reservoir();
        uint32_t seed = seeds[i];
        for (uint32_t j = 0; j < k; j++) {
            Reservoir src;
            memcpy(&src, res28 + ((size_t)i * k + j) * 28, 112);
            merge_reservoir(t, src, p_hats[(size_t)i * k + j], seed);
        }
        memcpy(out28 + (size_t)i * 28, &t, 112);
        seeds_out[i] = seed;
    }
}
void or_units_similar(const uint32_t* a24, const uint32_t* b24, uint32_t n, uint32_t* out2) {
    for (uint32_t i = 0; i < n; i++) {
        Sample a, b;
        memcpy(&a, a24 + 24 * (size_t)i, 96);
        memcpy(&b, b24 + 24 * (size_t)i, 96);
        out2[2 * i] = is_similar(a, b) ? 1u : 0u;
        out2[2 * i + 1] = is_similar_geo(a.x_view, a.n_view, b.x_view, b.n_view) ? 1u : 0u;
    }
}
void or_units_aces(const float* in3, uint32_t n, float* out3) {
    for (uint32_t i = 0; i < 3 * n; i++) out3[i] = aces1(in3[i]);
}
// EvaluateTargetFunction of the temporal pass and p_hat of the spatial pass
void or_units_targets(const uint32_t* samples24, const float* x3, const float* n3, uint32_t n, float* out2) {
    for (uint32_t i = 0; i < n; i++) {
        Sample smp;
        memcpy(&smp, samples24 + 24 * (size_t)i, 96);
        out2[2 * i] = eval_target(smp, f3{x3[3 * i], x3[3 * i + 1], x3[3 * i + 2]}, f3{n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]});
        out2[2 * i + 1] = p_hat_of(smp.L_out);
    }
}
void or_units_world_to_screen_uv(const float* p3, uint32_t n, const float* view16, const float* proj16, float* out2) {
    for (uint32_t i = 0; i < n; i++) {
        f2 uv = world_to_screen_uv(f3{p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]}, view16, proj16);
        out2[2 * i] = uv.x; out2[2 * i + 1] = uv.y;
    }
}
void or_units_neighbor_index(uint32_t x, uint32_t y, uint32_t w, uint32_t h, float max_r, uint32_t seed, uint32_t k,
                             uint32_t* out) {
    for (uint32_t j = 0; j < k; j++) out[j] = neighbor_index(x, y, w, h, max_r, seed);
}
void or_oct_roundtrip(const float* n3, uint32_t count, uint32_t bits, float* out3, uint32_t* codes) {
    for (uint32_t i = 0; i < count; i++) {
        f3 n{n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]};
        uint32_t c = oct_encode(n, bits);
        f3 d = oct_decode(c, bits);
        codes[i] = c;
        out3[3 * i] = d.x; out3[3 * i + 1] = d.y; out3[3 * i + 2] = d.z;
    }
}

void* or_scene_create(const float* vertices, uint32_t nv, const uint32_t* indices, uint32_t ntri,
                      const float* materials, uint32_t nm) {
    Scene* s = new Scene();
    s->nv = nv; s->ntri = ntri; s->nm = nm;
    s->vert.assign(vertices, vertices + (size_t)nv * 9);
    s->idx.assign(indices, indices + (size_t)ntri * 3);
    s->mat.resize(nm);
    if (nm) memcpy(s->mat.data(), materials, (size_t)nm * 32);
    s->p0.resize(ntri); s->p1.resize(ntri); s->p2.resize(ntri);
    for (uint32_t t = 0; t < ntri; t++) {
        s->p0[t] = vert_pos(*s, s->idx[3 * (size_t)t]);
        s->p1[t] = vert_pos(*s, s->idx[3 * (size_t)t + 1]);
        s->p2[t] = vert_pos(*s, s->idx[3 * (size_t)t + 2]);
    }
    s->brute = ntri <= 256;
    if (!s->brute) build_bvh(*s);
    build_lights(*s);
    return s;
}
void or_scene_destroy(void* scene) { delete (Scene*)scene; }

// Inverse of a 3 x 4 affine map: adjugate over determinant in double precision,
// rounded to float (the expressions and order of instances.cu).
static bool invert_affine(const float m[12], float out[12]) {
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    const double A = e * i - f * h, B = f * g - d * i, C = d * h - e * g;
    const double det = a * A + b * B + c * C;
    if (!std::isfinite(det) || det == 0.0) return false;
    const double r = 1.0 / det;
    const double inv[9] = {A * r, (c * h - b * i) * r, (b * f - c * e) * r,
                           B * r, (a * i - c * g) * r, (c * d - a * f) * r,
                           C * r, (b * g - a * h) * r, (a * e - b * d) * r};
    const double tx = m[3], ty = m[7], tz = m[11];
    for (int k = 0; k < 3; k++) {
        out[4 * k + 0] = (float)inv[3 * k + 0];
        out[4 * k + 1] = (float)inv[3 * k + 1];
        out[4 * k + 2] = (float)inv[3 * k + 2];
        out[4 * k + 3] = (float)(-((inv[3 * k + 0] * tx + inv[3 * k + 1] * ty) + inv[3 * k + 2] * tz));
    }
    for (int k = 0; k < 12; k++)
        if (!std::isfinite(out[k])) return false;
    return true;
}

static void world_concat(Scene& w) {
    w.vert.clear(); w.idx.clear(); w.mat.clear(); w.part_prim0.clear();
    uint32_t vo = 0, mo = 0, po = 0;
    for (const Scene& p : w.parts) {
        w.part_prim0.push_back(po);
        for (uint32_t v = 0; v < p.nv; v++) {
            const float* src = &p.vert[(size_t)v * 9];
            float q[9];
            memcpy(q, src, sizeof(q));
            int32_t mi;
            memcpy(&mi, &q[8], 4);
            if (mi >= 0) mi += (int32_t)mo;
            memcpy(&q[8], &mi, 4);
            w.vert.insert(w.vert.end(), q, q + 9);
        }
        for (uint32_t k = 0; k < p.ntri * 3; k++) w.idx.push_back(p.idx[k] + vo);
        w.mat.insert(w.mat.end(), p.mat.begin(), p.mat.end());
        vo += p.nv; mo += p.nm; po += p.ntri;
    }
    w.nv = vo; w.nm = mo; w.ntri = po;
    // without instances the world is traced as one scene (brute force)
    w.p0.resize(po); w.p1.resize(po); w.p2.resize(po);
    for (uint32_t t = 0; t < po; t++) {
        w.p0[t] = vert_pos(w, w.idx[3 * (size_t)t]);
        w.p1[t] = vert_pos(w, w.idx[3 * (size_t)t + 1]);
        w.p2[t] = vert_pos(w, w.idx[3 * (size_t)t + 2]);
    }
}

// A world of n scenes (copied), concatenated as xr_upload_scenes does; trace and
// render it after or_world_set_instances.
void* or_world_create(void* const* scenes, uint32_t n) {
    Scene* w = new Scene();
    for (uint32_t k = 0; k < n; k++) {
        w->parts.push_back(*(const Scene*)scenes[k]);
        w->parts.back().tex_info.clear();
        w->parts.back().texels.clear();
    }
    world_concat(*w);
    w->brute = true;
    return w;
}

// Instances: n x {part, 3 x 4 object-to-world}.  Returns 0, or -1 for a bad part
// or a singular transform.
int or_world_set_instances(void* world, const uint32_t* part, const float* o2w12, uint32_t n) {
    Scene& w = *(Scene*)world;
    std::vector<Scene::Inst> v(n);
    for (uint32_t i = 0; i < n; i++) {
        if (part[i] >= w.parts.size()) return -1;
        v[i].part = part[i];
        memcpy(v[i].o2w, o2w12 + 12 * (size_t)i, 48);
        if (!invert_affine(v[i].o2w, v[i].w2o)) return -1;
    }
    w.inst = v;
    return 0;
}

// 24 floats per instance: object-to-world, world-to-object.
void or_world_transforms(void* world, float* out24) {
    const Scene& w = *(const Scene*)world;
    for (size_t i = 0; i < w.inst.size(); i++) {
        memcpy(out24 + 24 * i, w.inst[i].o2w, 48);
        memcpy(out24 + 24 * i + 12, w.inst[i].w2o, 48);
    }
}

// New vertices of one part (same count); its BVH is rebuilt from scratch.
int or_world_update_vertices(void* world, uint32_t part, const float* vertices9, uint32_t nv) {
    Scene& w = *(Scene*)world;
    if (part >= w.parts.size() || w.parts[part].nv != nv) return -1;
    Scene& p = w.parts[part];
    p.vert.assign(vertices9, vertices9 + (size_t)nv * 9);
    for (uint32_t t = 0; t < p.ntri; t++) {
        p.p0[t] = vert_pos(p, p.idx[3 * (size_t)t]);
        p.p1[t] = vert_pos(p, p.idx[3 * (size_t)t + 1]);
        p.p2[t] = vert_pos(p, p.idx[3 * (size_t)t + 2]);
    }
    if (!p.brute) build_bvh(p);
    world_concat(w);
    return 0;
}

// Base-colour textures (n; sizes as width, height pairs; texels RGBA8 concatenated,
// row 0 = v 0) -- the layout of xr_upload_textures.
void or_scene_set_textures(void* scene, const uint32_t* sizes2, uint32_t n, const uint8_t* rgba8) {
    Scene& s = *(Scene*)scene;
    s.tex_info.clear();
    s.texels.clear();
    size_t off = 0;
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t w = sizes2[2 * i], h = sizes2[2 * i + 1];
        s.tex_info.push_back((uint32_t)off);
        s.tex_info.push_back(w);
        s.tex_info.push_back(h);
        off += (size_t)w * h;
    }
    s.texels.resize(off);
    if (off) std::memcpy(s.texels.data(), rgba8, off * 4);
}

void or_trace(void* scene, const float* rays, uint32_t n, int any_hit, int32_t* prim, float* t,
              float* bary) {
    const Scene& s = *(const Scene*)scene;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        const float* r = rays + 8 * i;
        Hit h = trace(s, f3{r[0], r[1], r[2]}, f3{r[4], r[5], r[6]}, r[3], r[7], any_hit != 0);
        prim[i] = h.prim;
        t[i] = h.prim >= 0 ? h.t : -1.0f;
        bary[2 * i] = h.b1;
        bary[2 * i + 1] = h.b2;
    }
}

void or_trace_inst(void* scene, const float* rays, uint32_t n, int any_hit, int32_t* prim, int32_t* inst, float* t,
                   float* bary) {
    const Scene& s = *(const Scene*)scene;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        const float* r = rays + 8 * i;
        Hit h = trace(s, f3{r[0], r[1], r[2]}, f3{r[4], r[5], r[6]}, r[3], r[7], any_hit != 0);
        prim[i] = h.prim;
        inst[i] = h.prim >= 0 ? h.inst : -1;
        t[i] = h.prim >= 0 ? h.t : -1.0f;
        bary[2 * i] = h.b1;
        bary[2 * i + 1] = h.b2;
    }
}

void* or_renderer_create(void* scene, const OrParams* params) {
    Renderer* R = new Renderer();
    R->sc = (const Scene*)scene;
    R->P = *params;
    R->W = params->width; R->H = params->height; R->N = R->W * R->H;
    R->compat = params->compat_reference != 0;
    uint32_t N = R->N;
    R->samples.assign(N, init_sample());
    Reservoir z;
    memset(&z, 0, sizeof(z));
    R->temporal.assign(2 * (size_t)N, z);
    R->spatial.assign(2 * (size_t)N, z);
    R->gpos.assign(N, f4{0, 0, 0, 0});
    R->motion.assign(N, f2{0, 0});
    R->gnrm_code.assign(N, 0);
    R->prev_gpos.assign(N, f4{0, 0, 0, 0});
    R->prev_code.assign(N, 0);
    R->prev_mat.assign(N, 0xFFFFFFFFu);
    R->le0.assign(N, f3{0, 0, 0});
    R->thr0.assign(N, f3{0, 0, 0});
    R->hdr.assign(N, f4{0, 0, 0, 0});
    R->pt.assign(N, f4{0, 0, 0, 0});
    R->ldr.assign(4 * (size_t)N, 0);
    R->written.assign(N, 0);
    R->gb_uv.assign(N, f2{0.0f, 0.0f});
    return R;
}
void or_renderer_destroy(void* r) { delete (Renderer*)r; }

static void end_frame(Renderer& R) {
    if (!R.compat) {
        for (uint32_t p = 0; p < R.N; p++) {
            R.prev_gpos[p] = R.gpos[p];
            R.prev_code[p] = R.gnrm_code[p];
            R.prev_mat[p] = R.samples[p].materialID;
        }
    }
}

static void run_temporal(Renderer& R, const OrUBO& u) {
    bool out_here = R.compat ? (u.reuse == 0) : (R.P.spatial_on == 0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t y = 0; y < (int64_t)R.H; y++)
        for (uint32_t x = 0; x < R.W; x++) temporal_pixel(R, x, (uint32_t)y, u, out_here);
}
static void run_spatial(Renderer& R, const OrUBO& u) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t y = 0; y < (int64_t)R.H; y++)
        for (uint32_t x = 0; x < R.W; x++) spatial_pixel(R, x, (uint32_t)y, u);
}

int or_render_frame(void* rp, const OrUBO* u) {
    Renderer& R = *(Renderer*)rp;
    std::fill(R.written.begin(), R.written.end(), 0u);
#pragma omp parallel for schedule(dynamic, 2)
    for (int64_t y = 0; y < (int64_t)R.H; y++)
        for (uint32_t x = 0; x < R.W; x++) initial_pixel(R, x, (uint32_t)y, *u);
    if (R.cache_on && R.cache_target) {
        // the next frame's training pixels: sel * target / got clamped to [target, N]
        // (all pixels when no record came out), as the kernels' k_cache_select_next
        uint64_t got = 0;
        for (uint32_t p = 0; p < R.N; p++) got += R.cache_t_valid[p] ? 1u : 0u;
        uint64_t next = got ? (uint64_t)R.cache_sel_n * R.cache_target / got : (uint64_t)R.N;
        next = std::min<uint64_t>(std::max<uint64_t>(next, R.cache_target), R.N);
        R.cache_sel_n = (uint32_t)next;
    }
    if (R.P.write_pt) {
        for (uint32_t p = 0; p < R.N; p++) {
            const Sample& s = R.samples[p];
            f3 v = s.materialID != 0xFFFFFFFFu ? R.thr0[p] * s.L_out : R.le0[p];
            R.pt[p] = f4{v.x, v.y, v.z, 1.0f};
        }
    }
    run_temporal(R, *u);
    if (R.compat || R.P.spatial_on) run_spatial(R, *u);
    end_frame(R);
    return 0;
}

int or_set_samples(void* rp, const float* words, const OrUBO* u) {
    Renderer& R = *(Renderer*)rp;
    memcpy(R.samples.data(), words, (size_t)R.N * sizeof(Sample));
    // the G-buffer and motion vectors the reuse passes read are functions of the samples
    for (uint32_t p = 0; p < R.N; p++) {
        const Sample& s = R.samples[p];
        bool valid = s.materialID != 0xFFFFFFFFu;
        uint32_t x = p % R.W, y = p / R.W;
        R.gpos[p] = valid ? f4{s.x_view.x, s.x_view.y, s.x_view.z, 1.0f} : f4{0, 0, 0, 0};
        R.motion[p] = f2{0, 0};
        if (valid) {
            f2 cur_uv{((float)x + 0.5f) / (float)R.W, ((float)y + 0.5f) / (float)R.H};
            f2 prev_uv = world_to_screen_uv(s.x_view, u->view_prev, u->projection_prev);
            f2 mv{cur_uv.x - prev_uv.x, cur_uv.y - prev_uv.y};
            R.motion[p] = R.compat ? f2{half_round(mv.x), half_round(mv.y)} : mv;
        }
        R.gnrm_code[p] = R.compat ? 0u : s.randSeed;
    }
    return 0;
}

int or_end_frame(void* rp) {
    end_frame(*(Renderer*)rp);
    return 0;
}

int or_run_pass(void* rp, const OrUBO* u, int pass) {
    Renderer& R = *(Renderer*)rp;
    if (pass == 1) run_temporal(R, *u);
    else if (pass == 2) run_spatial(R, *u);
    else return 1;
    return 0;
}

int or_write_temporal(void* rp, const float* words, size_t bytes) {
    Renderer& R = *(Renderer*)rp;
    if (bytes != R.temporal.size() * sizeof(Reservoir)) return 1;
    memcpy(R.temporal.data(), words, bytes);
    return 0;
}

int or_renderer_set_cache(void* rp, int enabled, uint32_t train_samples, void* nrc) {
    Renderer& R = *(Renderer*)rp;
    if (enabled && R.compat) return 1;
    R.cache_on = enabled != 0;
    R.cache_target = enabled ? std::min(train_samples, R.N) : 0u;
    R.cache_sel_n = R.cache_target;
    R.nrc = nrc;
    if (R.cache_on && R.cache_q.empty()) {
        R.cache_q.assign((size_t)R.N * 8, 0u);
        R.cache_t.assign((size_t)R.N * 12, 0u);
        R.cache_q_valid.assign(R.N, 0);
        R.cache_t_valid.assign(R.N, 0);
    }
    return 0;
}

size_t or_read(void* rp, int which, void* dst, size_t bytes) {
    Renderer& R = *(Renderer*)rp;
    const void* src = nullptr;
    size_t n = 0;
    std::vector<float> tmp;
    switch (which) {
        case OR_BUF_SAMPLES: src = R.samples.data(); n = R.samples.size() * sizeof(Sample); break;
        case OR_BUF_TEMPORAL: src = R.temporal.data(); n = R.temporal.size() * sizeof(Reservoir); break;
        case OR_BUF_SPATIAL: src = R.spatial.data(); n = R.spatial.size() * sizeof(Reservoir); break;
        case OR_BUF_HDR: src = R.hdr.data(); n = R.hdr.size() * sizeof(f4); break;
        case OR_BUF_LDR: src = R.ldr.data(); n = R.ldr.size(); break;
        case OR_BUF_PT: src = R.pt.data(); n = R.pt.size() * sizeof(f4); break;
        case OR_BUF_GBUF_POS: src = R.gpos.data(); n = R.gpos.size() * sizeof(f4); break;
        case OR_BUF_MOTION: src = R.motion.data(); n = R.motion.size() * sizeof(f2); break;
        case OR_BUF_WRITTEN: src = R.written.data(); n = R.written.size() * 4; break;
        case OR_BUF_CACHE_QUERIES:
        case OR_BUF_CACHE_TRAIN: {
            // valid records only, in pixel order
            const bool q = which == OR_BUF_CACHE_QUERIES;
            const size_t words = q ? 8 : 12;
            std::vector<uint32_t> out;
            if (R.cache_on)
                for (uint32_t p = 0; p < R.N; ++p)
                    if (q ? R.cache_q_valid[p] : R.cache_t_valid[p]) {
                        const uint32_t* r = q ? &R.cache_q[(size_t)p * 8] : &R.cache_t[(size_t)p * 12];
                        out.insert(out.end(), r, r + words);
                    }
            n = out.size() * 4;
            if (dst && bytes >= n && n) memcpy(dst, out.data(), n);
            return n;
        }
        default: return 0;
    }
    if (dst && bytes >= n) memcpy(dst, src, n);
    return n;
}

int or_pt_reference(void* scene, const OrParams* params, const OrUBO* ubo, uint32_t frame0, uint32_t spp,
                    double* out_rgb) {
    Renderer* R = (Renderer*)or_renderer_create(scene, params);
    uint32_t N = R->N;
    std::fill(out_rgb, out_rgb + 3 * (size_t)N, 0.0);
    OrUBO u = *ubo;
    for (uint32_t s = 0; s < spp; s++) {
        u.current_frame = frame0 + s;
#pragma omp parallel for schedule(dynamic, 2)
        for (int64_t y = 0; y < (int64_t)R->H; y++) {
            for (uint32_t x = 0; x < R->W; x++) {
                initial_pixel(*R, x, (uint32_t)y, u);
                uint32_t p = (uint32_t)y * R->W + x;
                const Sample& sm = R->samples[p];
                f3 v = sm.materialID != 0xFFFFFFFFu ? R->thr0[p] * sm.L_out : R->le0[p];
                out_rgb[3 * (size_t)p + 0] += (double)v.x;
                out_rgb[3 * (size_t)p + 1] += (double)v.y;
                out_rgb[3 * (size_t)p + 2] += (double)v.z;
            }
        }
    }
    for (size_t i = 0; i < 3 * (size_t)N; i++) out_rgb[i] /= (double)spp;
    or_renderer_destroy(R);
    return 0;
}

}  // extern "C"
