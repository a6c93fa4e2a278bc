// batch.cu -- several scenes in one context (xr_upload_scenes).
//
// Each scene is uploaded and its BVH built on its own scratch context; the
// context then holds the concatenation of all of them: primitives, vertices,
// materials, 8-wide nodes and triangle slots, with every index relocated by the
// offset of its scene (child and triangle bases of the nodes, the primitive id
// of each triangle slot, the vertex and material indices of each primitive).
// Each scene keeps its own BVH, reached through its root node (the first node of
// its block), so a ray started at its view's root only ever meets its own scene.
#include <algorithm>
#include <string>
#include <vector>

#include "xr_internal.h"

namespace xr {
namespace {

__global__ void k_relocate_nodes(WideNode* __restrict__ dst, const WideNode* __restrict__ src, uint32_t n,
                                 uint32_t node_off, uint32_t slot_off) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    WideNode w = src[i];
    w.child_base += node_off;
    w.tri_base += slot_off;
    dst[i] = w;
}

// 3 float4 per slot; the first carries the primitive id (as bits) in .w
__global__ void k_relocate_slots(float4* __restrict__ dst, const float4* __restrict__ src, uint32_t n4,
                                 uint32_t prim_off) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n4) return;
    float4 v = src[i];
    if (i % 3u == 0u) v.w = __uint_as_float(__float_as_uint(v.w) + prim_off);
    dst[i] = v;
}

__global__ void k_relocate_prims(uint4* __restrict__ dst, const uint4* __restrict__ src, uint32_t n, uint32_t vert_off,
                                 uint32_t mat_off) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint4 v = src[i];
    v.x += vert_off;
    v.y += vert_off;
    v.z += vert_off;
    if (v.w != kInvalid) v.w += mat_off;
    dst[i] = v;
}

uint32_t blocks(size_t n) { return (uint32_t)((n + 255) / 256); }

}  // namespace
}  // namespace xr

using namespace xr;

extern "C" xr_status xr_upload_scenes(XrContext* c, const XrSceneData* scenes, uint32_t n) {
    if (!c || !scenes || n == 0) return fail(c, XR_ERR_INVALID_ARGUMENT, "upload_scenes: bad argument");
    if (n > 1 && c->cache.params.enabled)
        return fail(c, XR_ERR_UNSUPPORTED, "upload_scenes: the learned cache covers one scene");
    DeviceGuard g(c->device);
    // one scratch context per scene: upload + BVH
    std::vector<XrContext*> parts(n, nullptr);
    xr_status s = XR_OK;
    XrDeviceDesc dd{};
    dd.device = c->device;
    dd.width = 1;
    dd.height = 1;
    for (uint32_t k = 0; k < n && !s; k++) {
        const XrSceneData& sd = scenes[k];
        if ((s = xr_create(&dd, &parts[k]))) break;
        parts[k]->n_tex = c->n_tex;   // texture indices are checked against the context's texture list
        if ((s = xr_upload_scene(parts[k], (const XrVertex*)sd.vertices, sd.vertex_count, (const uint32_t*)sd.indices,
                                 sd.index_count, (const XrMaterial*)sd.materials, sd.material_count, nullptr, 0)))
            break;
        s = xr_build_bvh(parts[k]);
    }
    if (s) {
        const std::string msg = xr_last_error(nullptr);
        for (XrContext* p : parts) xr_destroy(p);
        return fail(c, s, "upload_scenes: " + msg);
    }
    for (XrContext* p : parts) cudaStreamSynchronize(p->stream);   // builds ran on the scratch streams
    size_t nv = 0, ntri = 0, nm = 0, nodes = 0, slots = 0;
    uint32_t depth = 0;
    bool non_lambert = false;
    for (XrContext* p : parts) {
        nv += p->nv; ntri += p->ntri; nm += p->nm; nodes += p->n_nodes; slots += p->n_tri_slots;
        depth = std::max(depth, p->bvh_depth);
        non_lambert = non_lambert || p->scene_has_non_lambert;
    }
    if (nodes >= kNoRoot || ntri >= kNoRoot || nv >= kNoRoot) {
        for (XrContext* p : parts) xr_destroy(p);
        return fail(c, XR_ERR_INVALID_ARGUMENT, "upload_scenes: more than 2^32 nodes, primitives or vertices");
    }
    cudaStreamSynchronize(c->stream);
    invalidate_graphs(c);
    free_instances(c);   // instances refer to the former scenes
    c->parts.clear();
    cudaFree(c->d_tri_idx); cudaFree(c->d_vpos); cudaFree(c->d_vnrm); cudaFree(c->d_mats); cudaFree(c->d_vuv);
    cudaFree(c->d_nodes); cudaFree(c->d_tris);
    c->d_tri_idx = nullptr; c->d_vpos = nullptr; c->d_vnrm = nullptr; c->d_mats = nullptr; c->d_vuv = nullptr;
    c->d_nodes = nullptr; c->d_tris = nullptr;
    c->scene_ready = false;
    c->bvh_ready = false;
    if ((s = cuda_check(c, cudaMalloc((void**)&c->d_tri_idx, std::max<size_t>(ntri, 1) * 16), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_vpos, std::max<size_t>(nv, 1) * 16), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_vnrm, std::max<size_t>(nv, 1) * 16), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_vuv, std::max<size_t>(nv, 1) * 8), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_mats, std::max<size_t>(nm, 1) * sizeof(XrMaterial)), "scene alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_nodes, std::max<size_t>(nodes, 1) * sizeof(WideNode)), "bvh alloc")) ||
        (s = cuda_check(c, cudaMalloc((void**)&c->d_tris, std::max<size_t>(slots, 1) * 48), "bvh alloc"))) {
        for (XrContext* p : parts) xr_destroy(p);
        return s;
    }
    std::vector<uint32_t> roots(n);
    std::vector<ScenePart> plist(n);
    size_t ov = 0, ot = 0, om = 0, on = 0, os = 0;
    for (uint32_t k = 0; k < n; k++) {
        Context* p = parts[k];
        roots[k] = p->n_nodes ? (uint32_t)on : kNoRoot;
        ScenePart& sp = plist[k];
        sp.vert_off = (uint32_t)ov; sp.nv = p->nv; sp.prim_off = (uint32_t)ot; sp.ntri = p->ntri;
        sp.mat_off = (uint32_t)om; sp.nm = p->nm; sp.node_off = (uint32_t)on; sp.n_nodes = p->n_nodes;
        sp.slot_off = (uint32_t)os; sp.n_slots = p->n_tri_slots;
        sp.levels = p->bvh_levels;
        sp.emin = p->bvh_emin;
        for (int a = 0; a < 3; a++) { sp.lo[a] = p->scene_lo[a]; sp.hi[a] = p->scene_hi[a]; }
        if (p->ntri)
            k_relocate_prims<<<blocks(p->ntri), 256, 0, c->stream>>>(c->d_tri_idx + ot, p->d_tri_idx, p->ntri,
                                                                     (uint32_t)ov, (uint32_t)om);
        if (p->nv) {
            cudaMemcpyAsync(c->d_vpos + ov, p->d_vpos, (size_t)p->nv * 16, cudaMemcpyDeviceToDevice, c->stream);
            cudaMemcpyAsync(c->d_vnrm + ov, p->d_vnrm, (size_t)p->nv * 16, cudaMemcpyDeviceToDevice, c->stream);
            cudaMemcpyAsync(c->d_vuv + ov, p->d_vuv, (size_t)p->nv * 8, cudaMemcpyDeviceToDevice, c->stream);
        }
        if (p->nm)
            cudaMemcpyAsync(c->d_mats + om, p->d_mats, (size_t)p->nm * sizeof(XrMaterial), cudaMemcpyDeviceToDevice,
                            c->stream);
        if (p->n_nodes)
            k_relocate_nodes<<<blocks(p->n_nodes), 256, 0, c->stream>>>(c->d_nodes + on, p->d_nodes, p->n_nodes,
                                                                        (uint32_t)on, (uint32_t)os);
        if (p->n_tri_slots)
            k_relocate_slots<<<blocks(3 * (size_t)p->n_tri_slots), 256, 0, c->stream>>>(
                c->d_tris + 3 * os, p->d_tris, 3u * p->n_tri_slots, (uint32_t)ot);
        ov += p->nv; ot += p->ntri; om += p->nm; on += p->n_nodes; os += p->n_tri_slots;
    }
    s = cuda_check(c, cudaStreamSynchronize(c->stream), "scene merge");
    // light tables and the cache's scene cube exist for a single scene only
    cudaFree(c->d_light_prim); cudaFree(c->d_light_cdf); cudaFree(c->d_light_pmf); cudaFree(c->d_prim_light_pdf);
    c->d_light_prim = nullptr; c->d_light_cdf = nullptr; c->d_light_pmf = nullptr; c->d_prim_light_pdf = nullptr;
    c->n_lights = 0;
    if (!s && n == 1) {
        c->n_lights = parts[0]->n_lights;
        std::swap(c->d_light_prim, parts[0]->d_light_prim);
        std::swap(c->d_light_cdf, parts[0]->d_light_cdf);
        std::swap(c->d_light_pmf, parts[0]->d_light_pmf);
        std::swap(c->d_prim_light_pdf, parts[0]->d_prim_light_pdf);
        parts[0]->n_lights = 0;
        for (int a = 0; a < 3; a++) c->cache.lo[a] = parts[0]->cache.lo[a];
        c->cache.inv_ext = parts[0]->cache.inv_ext;
    }
    for (XrContext* p : parts) xr_destroy(p);
    if (s) return s;
    c->nv = (uint32_t)nv; c->ntri = (uint32_t)ntri; c->nm = (uint32_t)nm;
    c->n_nodes = (uint32_t)nodes; c->n_tri_slots = (uint32_t)slots; c->bvh_depth = depth;
    c->scene_has_non_lambert = non_lambert;
    c->scene_roots = roots;
    c->parts = plist;
    c->scene_ready = true;
    c->bvh_ready = true;
    DeviceScene& sc = c->fa.sc;
    sc.tri = c->d_tris; sc.nodes = c->d_nodes; sc.n_nodes = c->n_nodes;
    sc.tri_idx = c->d_tri_idx; sc.vpos = c->d_vpos; sc.vnrm = c->d_vnrm;
    sc.mats = c->d_mats; sc.n_mats = c->nm; sc.ntri = c->ntri; sc.n_tri_slots = c->n_tri_slots;
    sc.light_prim = c->d_light_prim; sc.light_cdf = c->d_light_cdf; sc.light_pmf = c->d_light_pmf;
    sc.prim_light_pdf = c->d_prim_light_pdf; sc.n_lights = c->n_lights;
    sc.vuv = c->d_vuv; sc.tex_info = c->d_tex_info; sc.texels = c->d_texels; sc.n_tex = c->n_tex;
    // the views' roots follow the new scene list
    if (c->pix_mem) {
        cudaStreamSynchronize(c->stream);
        return realloc_pixels(c);
    }
    return XR_OK;
}
