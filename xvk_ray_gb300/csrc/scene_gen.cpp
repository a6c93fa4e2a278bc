// scene_gen.cpp -- host-side scene builders and the per-frame camera UBO.
//
// xr_camera_ubo() replaces PathTracer::GetUniformBufferObject
// (src/pathTracer.cpp:169-201): glm::perspective(fov, aspect, 0.001, 1000) with
// GLM_FORCE_DEPTH_ZERO_TO_ONE and projection[1][1] *= -1, view = R * T(-position)
// (src/Editor/Camera.cpp:21-27), previous matrices carried from the last frame.
// The scenes are the synthetic inputs of the benchmark configurations: the
// reference renders glTF files, which are not part of this workload.
//
// Host C++ only, on the public header alone: the CPU oracle's build compiles
// this same file into its own workload library, so that the CPU baseline renders
// the identical scene and camera path without loading libxr.so.  Errors go
// through xr::fail (the library's last-error string; a plain status there).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "xr.h"

namespace xr {
struct Context;
xr_status fail(const Context* ctx, xr_status code, const std::string& msg);
}  // namespace xr

namespace {

struct Mat4 { double m[16]; };   // column-major, m[c*4 + r]

Mat4 identity() { Mat4 a{}; a.m[0] = a.m[5] = a.m[10] = a.m[15] = 1.0; return a; }
Mat4 mul(const Mat4& a, const Mat4& b) {
    Mat4 o{};
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) {
            double s = 0.0;
            for (int k = 0; k < 4; k++) s += a.m[k * 4 + r] * b.m[c * 4 + k];
            o.m[c * 4 + r] = s;
        }
    return o;
}
Mat4 rot_x(double a) { Mat4 r = identity(); double c = cos(a), s = sin(a); r.m[5] = c; r.m[6] = s; r.m[9] = -s; r.m[10] = c; return r; }
Mat4 rot_y(double a) { Mat4 r = identity(); double c = cos(a), s = sin(a); r.m[0] = c; r.m[2] = -s; r.m[8] = s; r.m[10] = c; return r; }
Mat4 translate(double x, double y, double z) { Mat4 t = identity(); t.m[12] = x; t.m[13] = y; t.m[14] = z; return t; }
bool invert(const Mat4& a, Mat4* out) {
    // Gauss-Jordan elimination with partial pivoting, in double.
    double w[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) { w[r][c] = a.m[c * 4 + r]; w[r][c + 4] = (r == c) ? 1.0 : 0.0; }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++) if (fabs(w[r][col]) > fabs(w[piv][col])) piv = r;
        if (w[piv][col] == 0.0) return false;
        if (piv != col) for (int c = 0; c < 8; c++) std::swap(w[piv][c], w[col][c]);
        double inv = 1.0 / w[col][col];
        for (int c = 0; c < 8; c++) w[col][c] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            double f = w[r][col];
            if (f != 0.0) for (int c = 0; c < 8; c++) w[r][c] -= f * w[col][c];
        }
    }
    for (int r = 0; r < 4; r++) for (int c = 0; c < 4; c++) out->m[c * 4 + r] = w[r][c + 4];
    return true;
}
void store(const Mat4& a, float* dst) { for (int i = 0; i < 16; i++) dst[i] = (float)a.m[i]; }
Mat4 load(const float* src) { Mat4 a; for (int i = 0; i < 16; i++) a.m[i] = src[i]; return a; }

// splitmix64 stream -> uniform floats in [0, 1)
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * uniform(); }
};

struct V3 { double x, y, z; };
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
V3 cross3(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 norm3(V3 a) { double l = sqrt(dot3(a, a)); return a * (1.0 / l); }

struct Builder {
    std::vector<XrVertex> v;
    std::vector<uint32_t> idx;
    std::vector<XrMaterial> mats;
    uint32_t add_material(float r, float g, float b, uint32_t model, float rough) {
        XrMaterial m{};
        m.base_color[0] = r; m.base_color[1] = g; m.base_color[2] = b; m.base_color[3] = 1.0f;
        m.base_color_texture_index = -1;
        m.fuzziness = rough;
        m.refraction_index = 0.0f;
        m.material_model = model;
        mats.push_back(m);
        return (uint32_t)mats.size() - 1;
    }
    uint32_t vertex(V3 p, V3 n, double u, double w, uint32_t mat) {
        XrVertex x{};
        x.pos[0] = (float)p.x; x.pos[1] = (float)p.y; x.pos[2] = (float)p.z;
        x.normal[0] = (float)n.x; x.normal[1] = (float)n.y; x.normal[2] = (float)n.z;
        x.tex_coord[0] = (float)u; x.tex_coord[1] = (float)w;
        x.material_index = (int32_t)mat;
        v.push_back(x);
        return (uint32_t)v.size() - 1;
    }
    // quad a-b-c-d (counter-clockwise seen from the side the normal points to)
    void quad(V3 a, V3 b, V3 c, V3 d, uint32_t mat) {
        V3 n = norm3(cross3(b - a, c - a));
        uint32_t i0 = vertex(a, n, 0, 0, mat), i1 = vertex(b, n, 1, 0, mat);
        uint32_t i2 = vertex(c, n, 1, 1, mat), i3 = vertex(d, n, 0, 1, mat);
        uint32_t t[6] = {i0, i1, i2, i0, i2, i3};
        idx.insert(idx.end(), t, t + 6);
    }
    // box of half extents h centred at c, rotated by yaw ry (radians) and an
    // optional full rotation matrix rot (row-major 3x3); outward normals
    void box(V3 c, V3 h, const double* rot, uint32_t mat) {
        auto X = [&](double x, double y, double z) {
            V3 l{x * h.x, y * h.y, z * h.z};
            V3 r{rot[0] * l.x + rot[1] * l.y + rot[2] * l.z, rot[3] * l.x + rot[4] * l.y + rot[5] * l.z,
                 rot[6] * l.x + rot[7] * l.y + rot[8] * l.z};
            return c + r;
        };
        quad(X(-1, -1, 1), X(1, -1, 1), X(1, 1, 1), X(-1, 1, 1), mat);     // +z
        quad(X(1, -1, -1), X(-1, -1, -1), X(-1, 1, -1), X(1, 1, -1), mat); // -z
        quad(X(1, -1, 1), X(1, -1, -1), X(1, 1, -1), X(1, 1, 1), mat);     // +x
        quad(X(-1, -1, -1), X(-1, -1, 1), X(-1, 1, 1), X(-1, 1, -1), mat); // -x
        quad(X(-1, 1, 1), X(1, 1, 1), X(1, 1, -1), X(-1, 1, -1), mat);     // +y
        quad(X(-1, -1, -1), X(1, -1, -1), X(1, -1, 1), X(-1, -1, 1), mat); // -y
    }
};

void yaw_matrix(double a, double* r) {
    double c = cos(a), s = sin(a);
    double m[9] = {c, 0, s, 0, 1, 0, -s, 0, c};
    memcpy(r, m, sizeof(m));
}

// Icosahedron subdivided `subdiv` times, projected to the unit sphere; shared
// vertices per sphere, smooth normals.
struct Ico {
    std::vector<V3> p;
    std::vector<uint32_t> t;
};
Ico make_ico(uint32_t subdiv) {
    Ico s;
    const double g = (1.0 + sqrt(5.0)) / 2.0;
    V3 base[12] = {{-1, g, 0}, {1, g, 0}, {-1, -g, 0}, {1, -g, 0}, {0, -1, g}, {0, 1, g},
                   {0, -1, -g}, {0, 1, -g}, {g, 0, -1}, {g, 0, 1}, {-g, 0, -1}, {-g, 0, 1}};
    for (auto& b : base) s.p.push_back(norm3(b));
    uint32_t f[60] = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6,
                      7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7,
                      9, 8, 1};
    s.t.assign(f, f + 60);
    for (uint32_t it = 0; it < subdiv; it++) {
        std::vector<uint32_t> nt;
        std::vector<std::pair<uint64_t, uint32_t>> cache;
        auto mid = [&](uint32_t a, uint32_t b) {
            uint64_t key = a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
            for (auto& kv : cache) if (kv.first == key) return kv.second;
            s.p.push_back(norm3((s.p[a] + s.p[b]) * 0.5));
            uint32_t id = (uint32_t)s.p.size() - 1;
            cache.push_back({key, id});
            return id;
        };
        for (size_t i = 0; i < s.t.size(); i += 3) {
            uint32_t a = s.t[i], b = s.t[i + 1], c = s.t[i + 2];
            uint32_t ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
            uint32_t q[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nt.insert(nt.end(), q, q + 12);
        }
        s.t.swap(nt);
    }
    return s;
}

void random_rotation(Rng& r, double* m) {
    // uniform quaternion (Shoemake)
    double u1 = r.uniform(), u2 = r.uniform(), u3 = r.uniform();
    double a = sqrt(1 - u1), b = sqrt(u1);
    double qx = a * sin(2 * M_PI * u2), qy = a * cos(2 * M_PI * u2), qz = b * sin(2 * M_PI * u3), qw = b * cos(2 * M_PI * u3);
    double mm[9] = {1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw),
                    2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw),
                    2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)};
    memcpy(m, mm, sizeof(mm));
}

xr_status emit(Builder& b, XrSceneData* out) {
    bool fill = out->vertices != nullptr;
    if (fill) {
        if (out->vertex_count < b.v.size() || out->index_count < b.idx.size() || out->material_count < b.mats.size())
            return xr::fail(nullptr, XR_ERR_INVALID_ARGUMENT, "scene arrays too small");
        memcpy(out->vertices, b.v.data(), b.v.size() * sizeof(XrVertex));
        memcpy(out->indices, b.idx.data(), b.idx.size() * 4);
        memcpy(out->materials, b.mats.data(), b.mats.size() * sizeof(XrMaterial));
    }
    out->vertex_count = (uint32_t)b.v.size();
    out->index_count = (uint32_t)b.idx.size();
    out->material_count = (uint32_t)b.mats.size();
    return XR_OK;
}

}  // namespace

extern "C" {

// The two parameter presets (the benchmark's corrected pipeline; the reference's constants).
void xr_params_default(XrParams* p, uint32_t width, uint32_t height) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->width = width; p->height = height;
    p->compat_reference = 0;
    p->temporal_on = 1; p->spatial_on = 1;
    p->m_cap_temporal = 20; p->m_cap_spatial = 120;
    p->n_neighbours = 5; p->radius_px = 30.0f;
    p->visibility = 1; p->seed = 1;
}

void xr_params_reference(XrParams* p, uint32_t width, uint32_t height) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->width = width; p->height = height;
    p->compat_reference = 1;
    p->temporal_on = 1; p->spatial_on = 1;
    p->m_cap_temporal = 30; p->m_cap_spatial = 300;   // ReSTIRGITemporalReuse.rgen.hlsl:3, ReSTIRGISpatialReuse.rgen.hlsl:6
    p->n_neighbours = 6; p->radius_px = 5.0f;         // ReSTIRGISpatialReuse.rgen.hlsl:4-5
    p->visibility = 0; p->seed = 0;
}


xr_status xr_camera_ubo(const XrCamera* cam, uint32_t width, uint32_t height, const XrUniformBufferObject* prev,
                        uint32_t current_frame, uint32_t number_of_bounces, uint32_t has_sky_box, uint32_t reuse,
                        XrUniformBufferObject* out) {
    if (!cam || !out || width == 0 || height == 0) return xr::fail(nullptr, XR_ERR_INVALID_ARGUMENT, "camera: bad args");
    const double deg = M_PI / 180.0;
    Mat4 rot = mul(rot_x(cam->pitch_deg * deg), rot_y(cam->yaw_deg * deg));
    Mat4 view = mul(rot, translate(-cam->position[0], -cam->position[1], -cam->position[2]));
    double fovy = cam->fov_deg * deg, aspect = (double)width / (double)height, zn = 0.001, zf = 1000.0;
    double th = tan(fovy / 2.0);
    Mat4 proj{};
    proj.m[0] = 1.0 / (aspect * th);
    proj.m[5] = 1.0 / th;
    proj.m[10] = zf / (zn - zf);
    proj.m[11] = -1.0;
    proj.m[14] = -(zf * zn) / (zf - zn);
    proj.m[5] *= -1.0;
    XrUniformBufferObject u;
    memset(&u, 0, sizeof(u));
    store(view, u.view);
    store(proj, u.projection);
    Mat4 vi, pi;
    if (!invert(load(u.view), &vi) || !invert(load(u.projection), &pi))
        return xr::fail(nullptr, XR_ERR_INVALID_ARGUMENT, "camera: singular matrix");
    store(vi, u.view_inverse);
    store(pi, u.projection_inverse);
    if (prev && current_frame != 0) {
        memcpy(u.view_prev, prev->view, sizeof(u.view_prev));
        memcpy(u.projection_prev, prev->projection, sizeof(u.projection_prev));
    } else {
        memcpy(u.view_prev, u.view, sizeof(u.view_prev));
        memcpy(u.projection_prev, u.projection, sizeof(u.projection_prev));
    }
    u.spp = 1;
    u.total_number_of_samples = 1;
    u.number_of_bounces = number_of_bounces;
    u.random_seed = 1;
    u.has_sky_box = has_sky_box ? 1u : 0u;
    u.reuse = reuse ? 1u : 0u;
    u.current_frame = current_frame;
    *out = u;
    return XR_OK;
}

xr_status xr_scene_cornell(XrSceneData* out) {
    if (!out) return xr::fail(nullptr, XR_ERR_INVALID_ARGUMENT, "cornell: null output");
    Builder b;
    uint32_t white = b.add_material(0.73f, 0.73f, 0.73f, XR_MAT_LAMBERTIAN, 1.0f);
    uint32_t red = b.add_material(0.65f, 0.05f, 0.05f, XR_MAT_LAMBERTIAN, 1.0f);
    uint32_t green = b.add_material(0.12f, 0.45f, 0.15f, XR_MAT_LAMBERTIAN, 1.0f);
    // DiffuseLight emits base_color * 4 (BSDF.hlsl:27-32): radiance (17,12,4)
    uint32_t light = b.add_material(17.0f / 4.0f, 12.0f / 4.0f, 4.0f / 4.0f, XR_MAT_DIFFUSE_LIGHT, 1.0f);
    // room [-1,1] x [0,2] x [-1,1], open towards +z; inward normals
    b.quad({-1, 0, 1}, {1, 0, 1}, {1, 0, -1}, {-1, 0, -1}, white);     // floor  (+y)
    b.quad({-1, 2, -1}, {1, 2, -1}, {1, 2, 1}, {-1, 2, 1}, white);     // ceiling (-y)
    b.quad({-1, 0, -1}, {1, 0, -1}, {1, 2, -1}, {-1, 2, -1}, white);   // back   (+z)
    b.quad({-1, 0, 1}, {-1, 0, -1}, {-1, 2, -1}, {-1, 2, 1}, red);     // left   (+x)
    b.quad({1, 0, -1}, {1, 0, 1}, {1, 2, 1}, {1, 2, -1}, green);       // right  (-x)
    double r1[9], r2[9];
    yaw_matrix(15.0 * M_PI / 180.0, r1);
    yaw_matrix(-18.0 * M_PI / 180.0, r2);
    b.box({-0.33, 0.6, -0.28}, {0.3, 0.6, 0.3}, r1, white);            // tall box
    b.box({0.35, 0.3, 0.32}, {0.3, 0.3, 0.3}, r2, white);              // short box
    // 0.5 x 0.5 = 0.25 unit^2 light just below the ceiling, facing down
    b.quad({-0.25, 1.98, -0.25}, {0.25, 1.98, -0.25}, {0.25, 1.98, 0.25}, {-0.25, 1.98, 0.25}, light);
    out->camera.position[0] = 0.0f; out->camera.position[1] = 1.0f; out->camera.position[2] = 3.4f;
    out->camera.yaw_deg = 0.0f; out->camera.pitch_deg = 0.0f; out->camera.fov_deg = 45.0f;
    return emit(b, out);
}

xr_status xr_scene_procedural(const XrProceduralDesc* d, XrSceneData* out) {
    if (!d || !out) return xr::fail(nullptr, XR_ERR_INVALID_ARGUMENT, "procedural: null args");
    Builder b;
    Rng rng(d->seed);
    const double E = d->extent;
    uint32_t ground = b.add_material(0.5f, 0.5f, 0.5f, XR_MAT_LAMBERTIAN, 1.0f);
    double G = E * 1.5;
    b.quad({-G, 0, G}, {G, 0, G}, {G, 0, -G}, {-G, 0, -G}, ground);
    Ico ico = make_ico(d->sphere_subdiv);
    for (uint32_t i = 0; i < d->n_objects; i++) {
        double rough = rng.range(0.05, 1.0);
        double ar = rng.range(0.1, 0.9), ag = rng.range(0.1, 0.9), ab = rng.range(0.1, 0.9);
        bool metallic = rng.uniform() < 0.3;
        uint32_t m = b.add_material((float)ar, (float)ag, (float)ab, metallic ? XR_MAT_METALLIC : XR_MAT_PLASTIC,
                                    (float)rough);
        double scale = rng.range(0.2, 2.0);
        double x = rng.range(-E, E), z = rng.range(-E, E);
        double rot[9];
        random_rotation(rng, rot);
        bool sphere = rng.uniform() < 0.75;
        if (sphere) {
            double rad = 0.5 * scale;
            V3 c{x, rad, z};
            uint32_t base = (uint32_t)b.v.size();
            for (const V3& p : ico.p) {
                V3 rp{rot[0] * p.x + rot[1] * p.y + rot[2] * p.z, rot[3] * p.x + rot[4] * p.y + rot[5] * p.z,
                      rot[6] * p.x + rot[7] * p.y + rot[8] * p.z};
                b.vertex(c + rp * rad, rp, 0.5 + atan2(rp.z, rp.x) / (2 * M_PI), acos(std::max(-1.0, std::min(1.0, rp.y))) / M_PI, m);
            }
            for (uint32_t t : ico.t) b.idx.push_back(base + t);
        } else {
            double h = 0.5 * scale;
            b.box({x, h * 0.9, z}, {h, h, h}, rot, m);
        }
    }
    for (uint32_t i = 0; i < d->n_lights; i++) {
        double le = rng.range(5.0, 50.0);
        uint32_t m = b.add_material((float)(le / 4.0), (float)(le / 4.0), (float)(le / 4.0), XR_MAT_DIFFUSE_LIGHT, 1.0f);
        double x = rng.range(-E, E), z = rng.range(-E, E), y = rng.range(6.0, 10.0), s = rng.range(0.75, 1.5);
        b.quad({x - s, y, z - s}, {x + s, y, z - s}, {x + s, y, z + s}, {x - s, y, z + s}, m);   // faces down
    }
    out->camera.position[0] = 0.0f; out->camera.position[1] = 3.0f; out->camera.position[2] = (float)(E * 0.9);
    out->camera.yaw_deg = 0.0f; out->camera.pitch_deg = 12.0f; out->camera.fov_deg = 60.0f;
    return emit(b, out);
}

}  // extern "C"
