// instances.cu -- instances of the uploaded scenes, the top-level BVH over them,
// and the refit of a scene's BVH after new vertex positions.
//
// The reference builds one bottom-level acceleration structure per model and a
// top-level one over identity instances (ApplicationRT.cpp:186-258,
// XVKTLAccelerationStructure.cpp:88); its closest-hit shader maps hits with
// ObjectToWorld / WorldToObject (Ray.rchit.hlsl:46-55).  Here:
//   * each scene's BVH (xr_build_bvh, xr_upload_scenes) is a bottom-level BVH;
//   * xr_set_instances takes object-to-world transforms, inverts them in double
//     precision, bounds every instance in world space (the corners of its scene's
//     root-node child boxes through the exact inverse of the float world-to-object
//     map, rounded outwards) and builds an 8-wide top-level BVH over those boxes
//     with the same device builder as the scenes; its leaves are 64-byte instance
//     records {world-to-object rows, instance, bottom-level root}.  The instance
//     arrays keep their addresses while the count stays within their capacity, so
//     the frame graphs captured over them stay valid;
//   * xr_update_vertices writes new vertices and refits the scene's BVH on the
//     device, one launch per level from the deepest (bvh_build.cu), in stream
//     order without a host wait; with instances it marks the top-level BVH stale
//     and the next trace, frame or statistics call rebuilds it (sync_tlas).
// Scratch of builds and refits comes from the context's stream-ordered pool.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "xr_internal.h"

namespace xr {
namespace {

// Inverse of a 3 x 4 affine map in double precision: the adjugate of the linear
// part over its determinant, translation -A^-1 t; rounded to float.  The oracle
// evaluates the same expressions in the same order.
bool invert_affine(const float m[12], float out[12]) {
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

// Exact (double) inverse of the float world-to-object map: the world-space image
// of an object-space box is bounded through it, so that a ray mapped into object
// space by the float rows meets the object box only if the world ray meets the
// world box (up to the rounding of the ray map, inside the box slack).
void inverse_double(const float w[12], double o[12]) {
    const double a = w[0], b = w[1], c = w[2], d = w[4], e = w[5], f = w[6], g = w[8], h = w[9], i = w[10];
    const double A = e * i - f * h, B = f * g - d * i, C = d * h - e * g;
    const double det = a * A + b * B + c * C;
    const double r = 1.0 / det;
    const double inv[9] = {A * r, (c * h - b * i) * r, (b * f - c * e) * r,
                           B * r, (a * i - c * g) * r, (c * d - a * f) * r,
                           C * r, (b * g - a * h) * r, (a * e - b * d) * r};
    for (int k = 0; k < 3; k++) {
        o[4 * k + 0] = inv[3 * k + 0];
        o[4 * k + 1] = inv[3 * k + 1];
        o[4 * k + 2] = inv[3 * k + 2];
        o[4 * k + 3] = -(inv[3 * k + 0] * w[3] + inv[3 * k + 1] * w[7] + inv[3 * k + 2] * w[11]);
    }
}

// World box of an instance: the corners of the root node's child boxes (or, before
// they are known, of the part's vertex bounds) mapped by the object-to-world
// transform in double precision, rounded outwards.  The child boxes contain the
// geometry with the quantisation slack, and for a rotated instance their union
// maps to a much smaller box than the part's axis-aligned bounds.
void world_box(const ScenePart& p, const float w2o[12], float lo[3], float hi[3]) {
    double m[12];
    inverse_double(w2o, m);
    double l[3] = {INFINITY, INFINITY, INFINITY}, u[3] = {-INFINITY, -INFINITY, -INFINITY};
    const double whole[6] = {p.lo[0], p.lo[1], p.lo[2], p.hi[0], p.hi[1], p.hi[2]};
    const size_t nb = p.root_boxes.empty() ? 1 : p.root_boxes.size() / 6;
    for (size_t b = 0; b < nb; b++) {
        const double* bx = p.root_boxes.empty() ? whole : &p.root_boxes[6 * b];
        for (int corner = 0; corner < 8; corner++) {
            const double x = bx[(corner & 1) ? 3 : 0];
            const double y = bx[(corner & 2) ? 4 : 1];
            const double z = bx[(corner & 4) ? 5 : 2];
            for (int k = 0; k < 3; k++) {
                const double v = m[4 * k] * x + m[4 * k + 1] * y + m[4 * k + 2] * z + m[4 * k + 3];
                l[k] = std::min(l[k], v);
                u[k] = std::max(u[k], v);
            }
        }
    }
    for (int k = 0; k < 3; k++) {
        lo[k] = std::nextafter((float)l[k], -INFINITY);
        hi[k] = std::nextafter((float)u[k], INFINITY);
    }
}

// Reads part p's root node back and decodes its child boxes: plane = origin + q 2^e
// per axis (the quantised grid of the node), children with a zero meta byte absent.
xr_status read_root_boxes(Context* c, ScenePart& p) {
    if (!p.root_boxes.empty() || p.n_nodes == 0) return XR_OK;
    WideNode nd;
    cudaMemcpyAsync(&nd, c->d_nodes + p.node_off, sizeof(nd), cudaMemcpyDeviceToHost, c->stream);
    if (xr_status s = cuda_check(c, cudaStreamSynchronize(c->stream), "root boxes")) return s;
    const double org[3] = {nd.px, nd.py, nd.pz};
    double cell[3];
    for (int k = 0; k < 3; k++) cell[k] = std::ldexp(1.0, (int)((nd.exyz_imask >> (8 * k)) & 0xFFu) - 127);
    for (uint32_t slot = 0; slot < 8; slot++) {
        const uint32_t word = slot < 4 ? 0u : 1u, shift = 8u * (slot & 3u);
        if (((nd.meta[word] >> shift) & 0xFFu) == 0u) continue;
        for (int k = 0; k < 3; k++)
            p.root_boxes.push_back(org[k] + (double)((nd.q[2 * k + word] >> shift) & 0xFFu) * cell[k]);
        for (int k = 0; k < 3; k++)
            p.root_boxes.push_back(org[k] + (double)((nd.q[6 + 2 * k + word] >> shift) & 0xFFu) * cell[k]);
    }
    return XR_OK;
}

int exponent_of(double v) {   // e with 2^(e-1) <= v < 2^e (v > 0)
    int e = 0;
    std::frexp(std::max(v, 1e-20), &e);
    return e;
}

// Finest grid exponent a scene's BVH needs: 2^-17 of its largest coordinate, and
// -- with instances -- of the largest object-space coordinate any point of the
// instanced world maps to (a ray origin), so that the box slack keeps covering
// the watertight triangle test's error, which grows with |v - o|.
int part_emin(const Context* c, uint32_t k, const float* world_lo, const float* world_hi) {
    const ScenePart& p = c->parts[k];
    double amax = 0.0;
    for (int a = 0; a < 3; a++) amax = std::max({amax, (double)std::fabs(p.lo[a]), (double)std::fabs(p.hi[a])});
    if (world_lo) {
        for (size_t i = 0; i < c->instances.size(); i++) {
            if (c->instances[i].scene != k) continue;
            const float* w = &c->inst_xform_host[24 * i + 12];
            for (int corner = 0; corner < 8; corner++) {
                const double x = (corner & 1) ? world_hi[0] : world_lo[0];
                const double y = (corner & 2) ? world_hi[1] : world_lo[1];
                const double z = (corner & 4) ? world_hi[2] : world_lo[2];
                for (int a = 0; a < 3; a++)
                    amax = std::max(amax, std::fabs(w[4 * a] * x + w[4 * a + 1] * y + w[4 * a + 2] * z + w[4 * a + 3]));
            }
        }
    }
    return exponent_of(amax) - 17;
}

// Points the frame's scene at the instance arrays. The bounds the traversal
// checks against are the arrays' capacities, so a rebuild with the same
// instance count leaves the scene -- and the captured frame graphs -- as they
// were. Returns whether anything changed.
bool bind_instances(Context* c) {
    DeviceScene& sc = c->fa.sc;
    const DeviceScene old = sc;
    const uint32_t cap = c->d_tlas_nodes ? c->inst_cap : 0u;
    sc.tlas_nodes = c->d_tlas_nodes;
    sc.n_tlas_nodes = cap ? std::max(cap, 2u) - 1u : 0u;
    sc.inst_slots = c->d_inst_slots;
    sc.n_inst_slots = cap;
    sc.inst_xform = c->d_inst_xform;
    sc.n_inst = (uint32_t)c->instances.size();
    return std::memcmp(&old, &sc, sizeof(sc)) != 0;
}

}  // namespace

void free_instances(Context* c) {
    // pool memory, released in stream order after the launches that read it
    pool_free(c, c->d_tlas_nodes); pool_free(c, c->d_inst_slots); pool_free(c, c->d_inst_xform);
    c->d_tlas_nodes = nullptr; c->d_inst_slots = nullptr; c->d_inst_xform = nullptr;
    c->n_tlas_nodes = 0; c->n_inst_slots = 0; c->inst_cap = 0;
    c->tlas_stale = false;
    c->instances.clear();
    c->inst_xform_host.clear();
    bind_instances(c);
}

xr_status refit_part(Context* c, uint32_t k, int emin) {
    NvtxRange nvtx_range("xr refit");
    ScenePart& p = c->parts[k];
    p.root_boxes.clear();   // new boxes below: read again on next use
    if (p.n_nodes == 0 || p.levels.size() < 2) { p.emin = emin; return XR_OK; }
    cudaStream_t st = c->stream;
    float4 *blo = nullptr, *bhi = nullptr;
    xr_status s;
    if ((s = pool_alloc(c, &blo, c->n_nodes, "refit scratch")) || (s = pool_alloc(c, &bhi, c->n_nodes, "refit scratch"))) {
        pool_free(c, blo);
        return s;
    }
    // stream-ordered behind the frames in flight and ahead of the next; no host wait
    cudaEventRecord(c->refit_ev[0], st);
    launch_refit_slots(c->d_tris, p.slot_off, p.n_slots, c->d_tri_idx, c->d_vpos, st);
    for (size_t L = p.levels.size() - 1; L-- > 0;)
        launch_refit_level(c->d_nodes, p.node_off + p.levels[L], p.levels[L + 1] - p.levels[L], c->d_tris, blo, bhi,
                           emin, st);
    cudaEventRecord(c->refit_ev[1], st);
    c->refit_timed = true;
    s = cuda_check(c, cudaGetLastError(), "refit");
    pool_free(c, blo); pool_free(c, bhi);
    if (!s) p.emin = emin;
    return s;
}

xr_status sync_tlas(Context* c) {
    if (!c->tlas_stale) return XR_OK;
    const xr_status s = rebuild_tlas(c);
    if (s) { free_instances(c); invalidate_graphs(c); }
    return s;
}

xr_status rebuild_tlas(Context* c) {
    NvtxRange nvtx_range("xr top-level build");
    const uint32_t n = (uint32_t)c->instances.size();
    c->tlas_stale = false;
    c->n_tlas_nodes = 0; c->n_inst_slots = 0;
    if (n == 0) return XR_OK;
    for (const XrInstance& in : c->instances)
        if (xr_status s0 = read_root_boxes(c, c->parts[in.scene])) return s0;
    // world boxes, records, and the world's bounds
    std::vector<float4> blo(n), bhi(n), rec(4 * (size_t)n);
    float wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < n; i++) {
        const ScenePart& p = c->parts[c->instances[i].scene];
        const float* w = &c->inst_xform_host[24 * (size_t)i + 12];
        float lo[3], hi[3];
        if (p.ntri) {
            world_box(p, w, lo, hi);
        } else {   // an empty scene: a point box at the instance's origin, never entered
            const float* o = &c->inst_xform_host[24 * (size_t)i];
            for (int a = 0; a < 3; a++) lo[a] = hi[a] = o[4 * a + 3];
        }
        blo[i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        bhi[i] = make_float4(hi[0], hi[1], hi[2], 0.0f);
        for (int a = 0; a < 3; a++) { wlo[a] = std::min(wlo[a], lo[a]); whi[a] = std::max(whi[a], hi[a]); }
        const uint32_t root = p.n_nodes ? p.node_off : kNoRoot;
        for (int r = 0; r < 3; r++) rec[4 * i + r] = make_float4(w[4 * r], w[4 * r + 1], w[4 * r + 2], w[4 * r + 3]);
        float idf, rootf;
        std::memcpy(&idf, &i, 4);
        std::memcpy(&rootf, &root, 4);
        rec[4 * i + 3] = make_float4(idf, rootf, 0.0f, 0.0f);
    }
    // bottom-level grids fine enough for the object-space distances of the world
    xr_status s = XR_OK;
    for (uint32_t k = 0; k < (uint32_t)c->parts.size() && !s; k++) {
        bool used = false;
        for (const XrInstance& in : c->instances) used = used || in.scene == k;
        if (!used) continue;
        const int need = part_emin(c, k, wlo, whi);
        if (need > c->parts[k].emin) s = refit_part(c, k, need);
    }
    if (s) return s;
    float4 *d_lo = nullptr, *d_hi = nullptr, *d_rec = nullptr;
    if ((s = pool_alloc(c, &d_lo, n, "tlas alloc")) || (s = pool_alloc(c, &d_hi, n, "tlas alloc")) ||
        (s = pool_alloc(c, &d_rec, 4 * (size_t)n, "tlas alloc"))) {
        pool_free(c, d_lo); pool_free(c, d_hi);
        return s;
    }
    // pageable sources: each copy returns once its bytes are staged, so the vectors may go out of scope
    cudaMemcpyAsync(d_lo, blo.data(), (size_t)n * 16, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d_hi, bhi.data(), (size_t)n * 16, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d_rec, rec.data(), (size_t)n * 64, cudaMemcpyHostToDevice, c->stream);
    WideBuild wb;
    wb.nodes_into = c->d_tlas_nodes;   // in place: stream order puts the build after the last frame's reads
    wb.slots_into = c->d_inst_slots;
    wb.n = n;
    wb.box_lo = d_lo;
    wb.box_hi = d_hi;
    wb.records = d_rec;
    // The Karras radix tree: no clustering rounds, so fewer host round trips
    // (257 instances: 0.43 ms against 1.19 ms with PLOC, same frame time).
    wb.builder = 2;
    if (const char* e = getenv("XR_TLAS_BUILDER")) wb.builder = strcmp(e, "ploc") == 0 ? 1 : 2;
    s = build_wide(c, wb);
    pool_free(c, d_lo); pool_free(c, d_hi); pool_free(c, d_rec);
    if (s) return s;
    c->n_tlas_nodes = wb.n_nodes;
    c->n_inst_slots = wb.n_slots;
    c->ms_tlas = wb.ms;
    if (bind_instances(c)) invalidate_graphs(c);
    return XR_OK;
}

}  // namespace xr

using namespace xr;

extern "C" {

xr_status xr_set_instances(XrContext* c, const XrInstance* inst, uint32_t n) {
    if (!c || (n && !inst)) return fail(c, XR_ERR_INVALID_ARGUMENT, "set_instances: null argument");
    if (n && !c->bvh_ready) return fail(c, XR_ERR_STATE, "set_instances: build the scene BVH(s) first");
    if (n && c->cache.params.enabled)
        return fail(c, XR_ERR_UNSUPPORTED, "set_instances: the learned cache covers one scene without instances");
    std::vector<float> xf(24 * (size_t)n);
    for (uint32_t i = 0; i < n; i++) {
        if (inst[i].scene >= c->parts.size())
            return fail(c, XR_ERR_INVALID_ARGUMENT, "set_instances: instance " + std::to_string(i) + " names no uploaded scene");
        for (int k = 0; k < 12; k++) {
            if (!std::isfinite(inst[i].object_to_world[k]))
                return fail(c, XR_ERR_INVALID_ARGUMENT, "set_instances: non-finite transform");
            xf[24 * (size_t)i + k] = inst[i].object_to_world[k];
        }
        if (!invert_affine(inst[i].object_to_world, &xf[24 * (size_t)i + 12]))
            return fail(c, XR_ERR_INVALID_ARGUMENT, "set_instances: singular transform of instance " + std::to_string(i));
    }
    DeviceGuard g(c->device);
    if (n == 0) { free_instances(c); invalidate_graphs(c); return XR_OK; }
    xr_status s = XR_OK;
    if (n > c->inst_cap) {   // new arrays; the old ones go back to the pool behind the frames that read them
        free_instances(c);
        if ((s = pool_alloc(c, &c->d_inst_xform, 6 * (size_t)n, "instance alloc")) ||
            (s = pool_alloc(c, &c->d_tlas_nodes, std::max(n, 2u) - 1u, "instance alloc")) ||
            (s = pool_alloc(c, &c->d_inst_slots, 4 * (size_t)n, "instance alloc"))) {
            free_instances(c);
            invalidate_graphs(c);
            return s;
        }
        c->inst_cap = n;
    }
    std::vector<float4> x6(6 * (size_t)n);
    for (uint32_t i = 0; i < n; i++)
        for (int r = 0; r < 6; r++) {
            const float* q = &xf[24 * (size_t)i + 4 * r];
            x6[6 * i + r] = make_float4(q[0], q[1], q[2], q[3]);
        }
    cudaMemcpyAsync(c->d_inst_xform, x6.data(), (size_t)n * 96, cudaMemcpyHostToDevice, c->stream);
    c->instances.assign(inst, inst + n);
    c->inst_xform_host = xf;
    s = rebuild_tlas(c);
    if (s) { free_instances(c); invalidate_graphs(c); }
    return s;
}

xr_status xr_get_instance_transforms(XrContext* c, float* out, uint32_t n) {
    if (!c || (n && !out)) return fail(c, XR_ERR_INVALID_ARGUMENT, "get_instance_transforms: null argument");
    if (n > c->instances.size()) return fail(c, XR_ERR_INVALID_ARGUMENT, "get_instance_transforms: more than the instances set");
    std::memcpy(out, c->inst_xform_host.data(), (size_t)n * 24 * sizeof(float));
    return XR_OK;
}

xr_status xr_update_vertices(XrContext* c, uint32_t scene, const XrVertex* v, uint32_t count) {
    if (!c || (count && !v)) return fail(c, XR_ERR_INVALID_ARGUMENT, "update_vertices: null argument");
    if (!c->bvh_ready || scene >= c->parts.size()) return fail(c, XR_ERR_INVALID_ARGUMENT, "update_vertices: no such scene with a BVH");
    ScenePart& p = c->parts[scene];
    if (count != p.nv) return fail(c, XR_ERR_INVALID_ARGUMENT, "update_vertices: the vertex count must stay as uploaded");
    std::vector<float4> pos(count), nrm(count);
    std::vector<float2> uv(count);
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < count; i++) {
        for (int k = 0; k < 3; k++) {
            if (!std::isfinite(v[i].pos[k])) return fail(c, XR_ERR_INVALID_ARGUMENT, "update_vertices: non-finite vertex position");
            lo[k] = std::min(lo[k], v[i].pos[k]);
            hi[k] = std::max(hi[k], v[i].pos[k]);
        }
        pos[i] = make_float4(v[i].pos[0], v[i].pos[1], v[i].pos[2], 0.0f);
        nrm[i] = make_float4(v[i].normal[0], v[i].normal[1], v[i].normal[2], 0.0f);
        uv[i] = make_float2(v[i].tex_coord[0], v[i].tex_coord[1]);
    }
    DeviceGuard g(c->device);
    xr_status s = XR_OK;
    if (count) {   // in stream order after the frames that still read the old vertices
        cudaMemcpyAsync(c->d_vpos + p.vert_off, pos.data(), (size_t)count * 16, cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(c->d_vnrm + p.vert_off, nrm.data(), (size_t)count * 16, cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(c->d_vuv + p.vert_off, uv.data(), (size_t)count * 8, cudaMemcpyHostToDevice, c->stream);
        if ((s = cuda_check(c, cudaGetLastError(), "update_vertices"))) return s;
        for (int k = 0; k < 3; k++) { p.lo[k] = lo[k]; p.hi[k] = hi[k]; }
    }
    if (c->parts.size() == 1) {
        for (int k = 0; k < 3; k++) { c->scene_lo[k] = p.lo[k]; c->scene_hi[k] = p.hi[k]; }
        cache_scene_bounds(c, reinterpret_cast<const float*>(v), count);
        if (c->n_lights) {   // light areas follow the vertices; the frames in flight still read the old tables
            cudaStreamSynchronize(c->stream);
            std::vector<uint4> tri(c->ntri);
            std::vector<XrMaterial> mats(c->nm);
            cudaMemcpy(tri.data(), c->d_tri_idx, (size_t)c->ntri * 16, cudaMemcpyDeviceToHost);
            cudaMemcpy(mats.data(), c->d_mats, (size_t)c->nm * sizeof(XrMaterial), cudaMemcpyDeviceToHost);
            free_lights(c);
            if ((s = upload_lights(c, tri, pos, mats.data(), c->nm))) return s;
            DeviceScene& sc = c->fa.sc;
            sc.light_prim = c->d_light_prim; sc.light_cdf = c->d_light_cdf; sc.light_pmf = c->d_light_pmf;
            sc.prim_light_pdf = c->d_prim_light_pdf; sc.n_lights = c->n_lights;
            invalidate_graphs(c);
        }
    }
    // the finest grid: the new coordinates, and the instanced world when there is one
    int emin = part_emin(c, scene, nullptr, nullptr);
    if ((s = refit_part(c, scene, emin))) return s;
    // the top level follows at the next render or trace, once for any number of updates
    if (!c->instances.empty()) c->tlas_stale = true;
    return XR_OK;
}

}  // extern "C"
