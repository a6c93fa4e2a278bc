// ref_pin.cpp -- the reference's own ReSTIR GI shader code, compiled as C++ and
// run on the CPU (TEST INFRASTRUCTURE: it pins the oracle; nothing in the
// product links it).
//
// Each shader of shader/HLSL/ReSTIRGI (random.hlsl, ReSTIRGICommon.hlsl,
// Sampling.hlsl, BSDF.hlsl, Material.hlsl, Vertex.hlsl, UBO.hlsl,
// RayPayload.hlsl, ReSTIRGIInitialSample.rgen.hlsl, ReSTIRGITemporalReuse.rgen.hlsl,
// ReSTIRGISpatialReuse.rgen.hlsl, Ray.rchit.hlsl, Ray.rmiss.hlsl) is included,
// after the mechanical rewrite of refpin/__init__.py, inside a namespace of its
// own; the harness below plays the parts of the Vulkan pipeline around them:
//
//  * one descriptor set for the three ray-generation passes, bound as
//    ReSTIRGIPipeline.cpp:99-196 binds it: binding 9 is the old-samples buffer
//    (initialSampleBufferInfo overwritten, :137-143), binding 18 is left null,
//    bindings 12/16 and 13/17 are the same two images (the position and normal
//    infos overwritten with the "previous" views, :165-177);
//  * ApplicationReSTIRGI::Render (ApplicationReSTIRGI.cpp:150-275): initial
//    sample over W x H, temporal reuse, spatial reuse, then the copy of the
//    never-written samples buffer over the old-samples buffer (zeros here);
//  * TraceRay: the closest / first hit from the oracle's traversal (the driver
//    and RT cores do this in the reference: no source), then the reference's own
//    closest-hit (Ray.rchit.hlsl) or miss (Ray.rmiss.hlsl) shader on the payload,
//    honouring RAY_FLAG_SKIP_CLOSEST_HIT_SHADER; identity instances, one per
//    model, as ApplicationRT.cpp:226-258 builds them.
//
// Pixels of a pass run in parallel (OpenMP): a pass writes only its own pixel's
// entries, as in the reference.
#include "hlsl_shim.h"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "xr_oracle.h"

// The Texture2D sampler of the shim: bilinear, clamp to edge, RGBA8 UNORM
// texels, the operations of the oracle's tex_bilinear (convention; the
// reference's filtering is done by the texture unit).
hlsl::float4 hlsl::Texture2D::SampleLevel(SamplerState, float2 uv, int) const {
    if (!texels || w <= 0 || h <= 0) return float4(0.0f);
    float x = uv.x * (float)w - 0.5f, y = uv.y * (float)h - 0.5f;
    if (!__builtin_isfinite(x)) x = 0.0f;
    if (!__builtin_isfinite(y)) y = 0.0f;
    x = __builtin_fminf(__builtin_fmaxf(x, -1.0f), (float)w);
    y = __builtin_fminf(__builtin_fmaxf(y, -1.0f), (float)h);
    const float x0f = __builtin_floorf(x), y0f = __builtin_floorf(y);
    const float fx = x - x0f, fy = y - y0f;
    const int x0 = (int)x0f, y0 = (int)y0f;
    const int xa = std::min(std::max(x0, 0), w - 1), xb = std::min(std::max(x0 + 1, 0), w - 1);
    const int ya = std::min(std::max(y0, 0), h - 1), yb = std::min(std::max(y0 + 1, 0), h - 1);
    auto texel = [&](int xx, int yy, int ch) {
        const uint32_t v = texels[(size_t)yy * w + xx];
        return (float)((v >> (8 * ch)) & 255u) / 255.0f;
    };
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    float c[3];
    for (int ch = 0; ch < 3; ch++)
        c[ch] = (texel(xa, ya, ch) * gx + texel(xb, ya, ch) * fx) * gy + (texel(xa, yb, ch) * gx + texel(xb, yb, ch) * fx) * fy;
    return float4(c[0], c[1], c[2], 1.0f);
}

// ---------------------------------------------------------------------------
// the shaders, one namespace each
// ---------------------------------------------------------------------------
namespace ref_units {
#include "hlsl_intrinsics.h"
#include "ReSTIRGI/BSDF.hlsl"
}
#undef RAY_PAYLOAD_H
namespace ref_initial {
#include "hlsl_intrinsics.h"
#include "ReSTIRGI/ReSTIRGIInitialSample.rgen.hlsl"
}
#undef RAY_PAYLOAD_H
#undef M_MAX
namespace ref_temporal {
#include "hlsl_intrinsics.h"
#include "ReSTIRGI/ReSTIRGITemporalReuse.rgen.hlsl"
}
#undef RAY_PAYLOAD_H
#undef M_MAX
namespace ref_spatial {
#include "hlsl_intrinsics.h"
#include "ReSTIRGI/ReSTIRGISpatialReuse.rgen.hlsl"
}
#undef RAY_PAYLOAD_H
namespace ref_chit {
#include "hlsl_intrinsics.h"
#include "ReSTIRGI/Ray.rchit.hlsl"
}
#undef RAY_PAYLOAD_H
namespace ref_miss {
#include "hlsl_intrinsics.h"
#include "ReSTIRGI/Ray.rmiss.hlsl"
}

static_assert(sizeof(ref_units::ReSTIRGISample) == 96, "ReSTIRGISample is 96 B (ApplicationReSTIRGI.cpp:311)");
static_assert(sizeof(ref_units::ReSTIRGIReservoir) == 112, "ReSTIRGIReservoir is 112 B (ApplicationReSTIRGI.cpp:326)");
static_assert(sizeof(ref_units::BSDFMaterial) == 32, "BSDFMaterial is 32 B");

namespace {

using hlsl::float2;
using hlsl::float3;
using hlsl::float4;
using hlsl::uint;

// ---------------------------------------------------------------------------
// scene and pipeline state
// ---------------------------------------------------------------------------
struct RefScene {
    std::vector<uint32_t> vertex_words;     // 9 words per vertex (AVertex, Vertex.hlsl:12-33)
    std::vector<uint32_t> indices;          // per model, relative to the model's vertexOffset
    std::vector<uint32_t> materials;        // 8 words per material
    std::vector<hlsl::uint2> offsets;       // per model {indexOffset, vertexOffset} (Scene.cpp:37)
    std::vector<uint32_t> first_prim;       // per model: global index of its first triangle
    std::vector<uint32_t> tex_sizes;        // per texture {w, h}
    std::vector<uint32_t> texels;           // RGBA8, concatenated
    std::vector<size_t> tex_offset;
    void* oracle = nullptr;                 // traversal (global indices)
};

struct RefRenderer {
    RefScene* sc = nullptr;
    uint32_t W = 0, H = 0, N = 0;
    std::vector<uint32_t> samples;          // binding 9: N x 24 words
    std::vector<uint32_t> temporal;         // binding 10: 2N x 28 words
    std::vector<uint32_t> spatial;          // binding 11: 2N x 28 words
    std::vector<float4> accumulation, output, gpos, gnrm, gmatuv;   // bindings 1, 2, 12(=16), 13(=17), 14
    std::vector<float2> motion;             // binding 15 (RG16F)
    uint8_t ubo[412] = {};
};

thread_local RefScene* t_scene = nullptr;

// ---- closest-hit and miss shaders on a neutral payload ----
template <class P>
void to_payload(const hlsl::ShimPayload& s, P& p) {
    p.Position = s.Position; p.Normal = s.Normal; p.GeometryNormal = s.GeometryNormal;
    p.UV = s.UV; p.MaterialIndex = s.MaterialIndex; p.HitT = s.HitT;
}
template <class P>
void from_payload(const P& p, hlsl::ShimPayload& s) {
    s.Position = p.Position; s.Normal = p.Normal; s.GeometryNormal = p.GeometryNormal;
    s.UV = p.UV; s.MaterialIndex = p.MaterialIndex; s.HitT = p.HitT;
}

void bind_hit_shader(RefScene& sc) {
    ref_chit::VertexArray.words = sc.vertex_words.data();
    ref_chit::VertexArray.n = sc.vertex_words.size();
    ref_chit::IndexArray.data = sc.indices.data();
    ref_chit::IndexArray.n = sc.indices.size();
    ref_chit::Materials.data = reinterpret_cast<ref_chit::BSDFMaterial*>(sc.materials.data());
    ref_chit::Materials.n = sc.materials.size() / 8;
    ref_chit::Offsets.data = sc.offsets.data();
    ref_chit::Offsets.n = sc.offsets.size();
}

// TraceRay: traversal by the oracle (closest hit, ties to the lowest primitive;
// or the first hit found for ACCEPT_FIRST_HIT_AND_END_SEARCH), then the
// reference's hit or miss shader.
void trace_hook(uint flags, const hlsl::RayDesc& ray, hlsl::ShimPayload& payload) {
    RefScene& sc = *t_scene;
    const float r8[8] = {ray.Origin.x, ray.Origin.y, ray.Origin.z, ray.TMin,
                         ray.Direction.x, ray.Direction.y, ray.Direction.z, ray.TMax};
    int32_t prim = -1;
    float t = 0.0f, bary[2] = {0.0f, 0.0f};
    const int any = (flags & hlsl::RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH) ? 1 : 0;
    or_trace(sc.oracle, r8, 1, any, &prim, &t, bary);
    if (prim < 0) {
        ref_miss::RayPayload p;
        to_payload(payload, p);
        ref_miss::main(p);
        from_payload(p, payload);
        return;
    }
    if (flags & hlsl::RAY_FLAG_SKIP_CLOSEST_HIT_SHADER) return;
    // the model (instance) holding the primitive and the primitive's index in it
    const auto it = std::upper_bound(sc.first_prim.begin(), sc.first_prim.end(), (uint32_t)prim);
    const uint32_t inst = (uint32_t)(it - sc.first_prim.begin()) - 1u;
    hlsl::g_hit.instance = inst;
    hlsl::g_hit.primitive = (uint32_t)prim - sc.first_prim[inst];
    hlsl::g_hit.t = t;
    ref_chit::RayPayload p;
    to_payload(payload, p);
    ref_chit::HitAttributes attribs;
    attribs.Barycentrics = float2(bary[0], bary[1]);
    ref_chit::main(p, attribs);
    from_payload(p, payload);
}

template <class U>
void fill_ubo(U& u, const uint8_t* raw) {
    const float* f = reinterpret_cast<const float*>(raw);
    std::memcpy(u.modelView.m, f + 0, 64);
    std::memcpy(u.viewPrev.m, f + 16, 64);
    std::memcpy(u.projection.m, f + 32, 64);
    std::memcpy(u.projectionPrev.m, f + 48, 64);
    std::memcpy(u.modelViewInverse.m, f + 64, 64);
    std::memcpy(u.projectionInverse.m, f + 80, 64);
    uint32_t w[7];
    std::memcpy(w, raw + 384, 28);
    u.spp = w[0];
    u.totalNumberOfSamples = w[1];
    u.numberOfBounces = w[2];
    u.randomSeed = w[3];
    u.hasSkyBox = w[4] != 0u;   // host uint32, shader bool (UniformBuffer.h:29-30, UBO.hlsl:13-14)
    u.reuse = w[5] != 0u;
    u.currentFrame = w[6];
}

template <class T>
void bind_image(hlsl::RWTexture2D<T>& img, std::vector<T>& v, uint32_t W, uint32_t H, bool half = false) {
    img.data = v.data(); img.w = W; img.h = H; img.half = half;
}
template <class T, class V>
void bind_buffer(hlsl::StructuredBuffer<T>& b, std::vector<V>& v) {
    b.data = reinterpret_cast<T*>(v.data());
    b.n = v.size() * sizeof(V) / sizeof(T);
}
template <class TexArray>
void bind_textures(TexArray& arr, RefScene& sc) {
    const size_t n = std::min<size_t>(sc.tex_sizes.size() / 2, (size_t)hlsl::kMaxTextures);
    for (size_t t = 0; t < n; ++t) {
        arr[t].texels = sc.texels.data() + sc.tex_offset[t];
        arr[t].w = (int)sc.tex_sizes[2 * t];
        arr[t].h = (int)sc.tex_sizes[2 * t + 1];
    }
}

template <class F>
void for_pixels(RefRenderer& R, F&& body) {
    RefScene* sc = R.sc;
    const uint32_t W = R.W, H = R.H;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t y = 0; y < (int64_t)H; ++y) {
        t_scene = sc;
        hlsl::g_launch_size = hlsl::uint3(W, H, 1);
        for (uint32_t x = 0; x < W; ++x) {
            hlsl::g_launch_id = hlsl::uint3(x, (uint32_t)y, 0);
            body();
        }
    }
}

void run_initial(RefRenderer& R) {
    using namespace ref_initial;
    fill_ubo(uniformBufferObject, R.ubo);
    bind_buffer(samples, R.samples);
    bind_buffer(Materials, R.sc->materials);
    bind_image(AccumulationImage, R.accumulation, R.W, R.H);
    bind_image(OutputImage, R.output, R.W, R.H);
    bind_image(GBufferPos, R.gpos, R.W, R.H);
    bind_image(GNormal, R.gnrm, R.W, R.H);
    bind_image(GMatUV, R.gmatuv, R.W, R.H);
    bind_image(GMotionVector, R.motion, R.W, R.H, true);
    bind_image(GBufferPosPrev, R.gpos, R.W, R.H);   // bindings 12 and 16: one image
    bind_image(GNormalPrev, R.gnrm, R.W, R.H);      // bindings 13 and 17: one image
    bind_textures(TextureSamplers, *R.sc);
    for_pixels(R, [] { ref_initial::main(); });
}

void run_temporal(RefRenderer& R) {
    using namespace ref_temporal;
    fill_ubo(uniformBufferObject, R.ubo);
    bind_buffer(samples, R.samples);
    bind_buffer(temporal_reservoirs, R.temporal);
    bind_buffer(spatial_reservoirs, R.spatial);
    oldsamples.data = nullptr; oldsamples.n = 0;    // binding 18: never written (null)
    bind_buffer(Materials, R.sc->materials);
    bind_image(AccumulationImage, R.accumulation, R.W, R.H);
    bind_image(OutputImage, R.output, R.W, R.H);
    bind_image(GMotionVector, R.motion, R.W, R.H, true);
    bind_image(GPosPrev, R.gpos, R.W, R.H);
    bind_image(GNrmPrev, R.gnrm, R.W, R.H);
    bind_textures(TextureSamplers, *R.sc);
    for_pixels(R, [] { ref_temporal::main(); });
}

void run_spatial(RefRenderer& R) {
    using namespace ref_spatial;
    fill_ubo(uniformBufferObject, R.ubo);
    bind_buffer(samples, R.samples);
    bind_buffer(temporal_reservoirs, R.temporal);
    bind_buffer(spatial_reservoirs, R.spatial);
    bind_buffer(Materials, R.sc->materials);
    bind_image(AccumulationImage, R.accumulation, R.W, R.H);
    bind_image(OutputImage, R.output, R.W, R.H);
    bind_image(GMatUV, R.gmatuv, R.W, R.H);
    bind_image(GMotionVector, R.motion, R.W, R.H, true);
    bind_image(GPosPrev, R.gpos, R.W, R.H);
    bind_image(GNrmPrev, R.gnrm, R.W, R.H);
    bind_textures(TextureSamplers, *R.sc);
    for_pixels(R, [] { ref_spatial::main(); });
}

}  // namespace

// ===========================================================================
// C ABI (ctypes binding in refpin/__init__.py)
// ===========================================================================
extern "C" {

// vertices: nv x 9 words (AVertex); indices: per-model local indices;
// ranges: nmodel x {index_offset, vertex_offset}; materials: nm x 8 words.
void* ref_scene_create(const uint32_t* vertices9, uint32_t nv, const uint32_t* indices, uint32_t ni,
                       const uint32_t* materials8, uint32_t nm, const uint32_t* ranges2, uint32_t nmodel) {
    RefScene* sc = new RefScene();
    sc->vertex_words.assign(vertices9, vertices9 + (size_t)nv * 9);
    sc->indices.assign(indices, indices + ni);
    sc->materials.assign(materials8, materials8 + (size_t)nm * 8);
    std::vector<uint32_t> global(ni);
    for (uint32_t m = 0; m < nmodel; ++m) {
        const uint32_t i0 = ranges2[2 * m], v0 = ranges2[2 * m + 1];
        const uint32_t i1 = m + 1 < nmodel ? ranges2[2 * m + 2] : ni;
        sc->offsets.push_back(hlsl::uint2(i0, v0));
        sc->first_prim.push_back(i0 / 3u);
        for (uint32_t k = i0; k < i1; ++k) global[k] = indices[k] + v0;
    }
    sc->oracle = or_scene_create(reinterpret_cast<const float*>(vertices9), nv, global.data(), ni / 3u,
                                 reinterpret_cast<const float*>(materials8), nm);
    return sc;
}

void ref_scene_set_textures(void* scene, const uint32_t* sizes2, uint32_t n, const uint8_t* rgba8) {
    RefScene* sc = (RefScene*)scene;
    sc->tex_sizes.assign(sizes2, sizes2 + 2 * (size_t)n);
    sc->tex_offset.clear();
    size_t total = 0;
    for (uint32_t t = 0; t < n; ++t) {
        sc->tex_offset.push_back(total);
        total += (size_t)sizes2[2 * t] * sizes2[2 * t + 1];
    }
    sc->texels.resize(total);
    if (total) std::memcpy(sc->texels.data(), rgba8, total * 4);
    or_scene_set_textures(sc->oracle, sizes2, n, rgba8);
}

void ref_scene_destroy(void* scene) {
    RefScene* sc = (RefScene*)scene;
    if (!sc) return;
    or_scene_destroy(sc->oracle);
    delete sc;
}

void* ref_renderer_create(void* scene, uint32_t width, uint32_t height) {
    RefRenderer* R = new RefRenderer();
    R->sc = (RefScene*)scene;
    R->W = width; R->H = height; R->N = width * height;
    const size_t N = R->N;
    R->samples.assign(N * 24, 0u);
    R->temporal.assign(2 * N * 28, 0u);
    R->spatial.assign(2 * N * 28, 0u);
    R->accumulation.assign(N, float4(0.0f));
    R->output.assign(N, float4(0.0f));
    R->gpos.assign(N, float4(0.0f));
    R->gnrm.assign(N, float4(0.0f));
    R->gmatuv.assign(N, float4(0.0f));
    R->motion.assign(N, float2(0.0f));
    return R;
}

void ref_renderer_destroy(void* r) { delete (RefRenderer*)r; }

// One frame of ApplicationReSTIRGI::Render with this frame's 412-byte UBO.
// The previous frame's closing vkCmdCopyBuffer(m_restir_initialSamplesBuffer ->
// m_restir_initialOldSamplesBuffer) copies a buffer no shader writes (zeros
// here); it is applied at the start of the next frame, which is the same for
// every pass and leaves the frame's samples readable afterwards.
void ref_render_frame(void* rp, const uint8_t* ubo412) {
    RefRenderer& R = *(RefRenderer*)rp;
    std::fill(R.samples.begin(), R.samples.end(), 0u);
    std::memcpy(R.ubo, ubo412, 412);
    hlsl::g_trace_hook = &trace_hook;
    bind_hit_shader(*R.sc);
    run_initial(R);
    run_temporal(R);
    run_spatial(R);
}

// Fixed-candidate checks: the G-buffer position and motion images as the initial
// pass writes them for these samples (ReSTIRGIInitialSample.rgen.hlsl:193-213:
// valid where the sample has a material; motion = pixel centre's uv minus
// WorldToScreenUV of x_view with the previous matrices, stored RG16F).
void ref_set_gbuffer_from_samples(void* rp, const uint8_t* ubo412, const uint32_t* samples24) {
    RefRenderer& R = *(RefRenderer*)rp;
    std::memcpy(R.samples.data(), samples24, R.samples.size() * 4);
    ref_initial::UniformBufferObject u;
    fill_ubo(u, ubo412);
    hlsl::RWTexture2D<float2> motion;
    bind_image(motion, R.motion, R.W, R.H, true);
    for (uint32_t p = 0; p < R.N; ++p) {
        ref_units::ReSTIRGISample s;
        std::memcpy(&s, samples24 + 24 * (size_t)p, 96);
        const uint32_t x = p % R.W, y = p / R.W;
        if (s.materialID != 0xFFFFFFFFu) {
            R.gpos[p] = float4(s.x_view, 1.0f);
            const float2 cur = (float2(hlsl::uint2(x, y)) + 0.5f) / float2(hlsl::uint2(R.W, R.H));
            const float2 prev = ref_initial::WorldToScreenUV(s.x_view, u.viewPrev, u.projectionPrev);
            motion.at(x, y) = cur - prev;
        } else {
            R.gpos[p] = float4(0.0f);
            motion.at(x, y) = float2(0.0f);
        }
    }
}

// One reuse pass (1 temporal, 2 spatial) on the buffers as they are, for
// fixed-candidate checks: samples (N x 24 words) and, optionally, the temporal
// reservoirs (2N x 28 words) are written first.
void ref_run_pass(void* rp, const uint8_t* ubo412, int pass, const uint32_t* samples24, const uint32_t* temporal28) {
    RefRenderer& R = *(RefRenderer*)rp;
    std::memcpy(R.ubo, ubo412, 412);
    hlsl::g_trace_hook = &trace_hook;
    bind_hit_shader(*R.sc);
    if (samples24) std::memcpy(R.samples.data(), samples24, R.samples.size() * 4);
    if (temporal28) std::memcpy(R.temporal.data(), temporal28, R.temporal.size() * 4);
    if (pass == 1) run_temporal(R);
    else run_spatial(R);
}

// Buffers: 0 samples (N x 24 words), 1 temporal (2N x 28), 2 spatial (2N x 28),
// 3 output image (N x float4, before the UNORM store), 4 G-buffer position
// (N x float4), 5 motion (N x float2, RG16F values), 6 G-buffer normal, 7 G-buffer
// material/uv.  Also sets the gpos/motion images (for fixed-candidate passes).
size_t ref_read(void* rp, int which, void* dst, size_t bytes) {
    RefRenderer& R = *(RefRenderer*)rp;
    const void* src = nullptr;
    size_t n = 0;
    switch (which) {
        case 0: src = R.samples.data(); n = R.samples.size() * 4; break;
        case 1: src = R.temporal.data(); n = R.temporal.size() * 4; break;
        case 2: src = R.spatial.data(); n = R.spatial.size() * 4; break;
        case 3: src = R.output.data(); n = R.output.size() * 16; break;
        case 4: src = R.gpos.data(); n = R.gpos.size() * 16; break;
        case 5: src = R.motion.data(); n = R.motion.size() * 8; break;
        case 6: src = R.gnrm.data(); n = R.gnrm.size() * 16; break;
        case 7: src = R.gmatuv.data(); n = R.gmatuv.size() * 16; break;
        default: return 0;
    }
    if (dst && bytes >= n) std::memcpy(dst, src, n);
    return n;
}
int ref_write(void* rp, int which, const void* src, size_t bytes) {
    RefRenderer& R = *(RefRenderer*)rp;
    void* dst = nullptr;
    size_t n = 0;
    switch (which) {
        case 4: dst = R.gpos.data(); n = R.gpos.size() * 16; break;
        case 5: dst = R.motion.data(); n = R.motion.size() * 8; break;
        case 6: dst = R.gnrm.data(); n = R.gnrm.size() * 16; break;
        default: return -1;
    }
    if (bytes != n) return -1;
    std::memcpy(dst, src, n);
    return 0;
}

// ---- the helper functions of random.hlsl, ReSTIRGICommon.hlsl, Sampling.hlsl, BSDF.hlsl ----
uint32_t ref_init_random_seed(uint32_t x, uint32_t y, uint32_t w, uint32_t h, uint32_t frame) {
    return ref_units::InitRandomSeed(hlsl::uint2(x, y), hlsl::uint2(w, h), frame);
}
void ref_random_sequence(uint32_t state, uint32_t n, uint32_t* out_u32, float* out_f, float* out_snorm,
                         float* out_disk2) {
    uint32_t s = state;
    for (uint32_t i = 0; i < n; ++i) out_u32[i] = ref_units::NextRandom(s);
    s = state;
    for (uint32_t i = 0; i < n; ++i) out_f[i] = ref_units::RandomFloat(s);
    s = state;
    for (uint32_t i = 0; i < n; ++i) out_snorm[i] = ref_units::RandomFloatSNorm(s);
    s = state;
    for (uint32_t i = 0; i < n; ++i) {
        const float2 d = ref_units::RandomInUnitDisk(s);
        out_disk2[2 * i] = d.x; out_disk2[2 * i + 1] = d.y;
    }
}
// n normals -> BranchlessONB tangents (6 floats each)
void ref_onb(const float* n3, uint32_t n, float* out6) {
    for (uint32_t i = 0; i < n; ++i) {
        float3 b1, b2;
        ref_units::BranchlessONB(float3(n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]), b1, b2);
        out6[6 * i + 0] = b1.x; out6[6 * i + 1] = b1.y; out6[6 * i + 2] = b1.z;
        out6[6 * i + 3] = b2.x; out6[6 * i + 4] = b2.y; out6[6 * i + 5] = b2.z;
    }
}
void ref_sample_hemisphere(const float* xi2, uint32_t n, float* out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const float3 v = ref_units::SampleHemisphere(float2(xi2[2 * i], xi2[2 * i + 1]));
        out3[3 * i] = v.x; out3[3 * i + 1] = v.y; out3[3 * i + 2] = v.z;
    }
}
// SampleBSDF for n (normal, wo, material, seed) cases: out 9 floats {f.rgb, wi.xyz, pdf, cos, seed-after}
void ref_sample_bsdf(const float* n3, const float* wo3, const uint32_t* materials8, const uint32_t* seeds,
                     uint32_t n, float* out9) {
    for (uint32_t i = 0; i < n; ++i) {
        ref_units::BSDFMaterial mat;
        std::memcpy(&mat, materials8 + 8 * (size_t)i, 32);
        float3 wi(0.0f);
        float pdf = 0.0f, cos_theta = 0.0f;
        uint32_t seed = seeds[i];
        const float3 f = ref_units::SampleBSDF(float3(n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]), float2(0.0f), mat,
                                               float3(wo3[3 * i], wo3[3 * i + 1], wo3[3 * i + 2]), true, wi, pdf,
                                               cos_theta, seed);
        float* o = out9 + 9 * (size_t)i;
        o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = wi.x; o[4] = wi.y; o[5] = wi.z; o[6] = pdf; o[7] = cos_theta;
        std::memcpy(&o[8], &seed, 4);
    }
}
// EvaluateBSDF: out 5 floats {f.rgb, pdf, cos}
void ref_evaluate_bsdf(const float* n3, const float* wo3, const float* wi3, const uint32_t* materials8, uint32_t n,
                       float* out5) {
    for (uint32_t i = 0; i < n; ++i) {
        ref_units::BSDFMaterial mat;
        std::memcpy(&mat, materials8 + 8 * (size_t)i, 32);
        float pdf = 0.0f, cos_theta = 0.0f;
        const float3 f = ref_units::EvaluateBSDF(float3(n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]), float2(0.0f), mat,
                                                 cos_theta, float3(wo3[3 * i], wo3[3 * i + 1], wo3[3 * i + 2]),
                                                 float3(wi3[3 * i], wi3[3 * i + 1], wi3[3 * i + 2]), pdf);
        float* o = out5 + 5 * (size_t)i;
        o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = pdf; o[4] = cos_theta;
    }
}
// Reservoir updates on fixed candidates: for each of n lists of k candidates
// (sample words 24 each, weight), starting from InitReservoir with the given seed;
// out: the reservoir (28 words) after the list, and the seed.
void ref_update_list(const uint32_t* samples24, const float* weights, uint32_t n, uint32_t k, const uint32_t* seeds,
                     uint32_t* out28, uint32_t* seeds_out) {
    for (uint32_t i = 0; i < n; ++i) {
        ref_units::ReSTIRGIReservoir r;
        ref_units::InitReservoir(r);
        uint32_t seed = seeds[i];
        for (uint32_t j = 0; j < k; ++j) {
            ref_units::ReSTIRGISample s;
            std::memcpy(&s, samples24 + ((size_t)i * k + j) * 24, 96);
            ref_units::UpdateReservoir(r, s, weights[(size_t)i * k + j], seed);
        }
        std::memcpy(out28 + (size_t)i * 28, &r, 112);
        seeds_out[i] = seed;
    }
}
// MergeReservoir of k source reservoirs into InitReservoir, target p-hats given
void ref_merge_list(const uint32_t* res28, const float* p_hats, uint32_t n, uint32_t k, const uint32_t* seeds,
                    uint32_t* out28, uint32_t* seeds_out) {
    for (uint32_t i = 0; i < n; ++i) {
        ref_units::ReSTIRGIReservoir t;
        ref_units::InitReservoir(t);
        uint32_t seed = seeds[i];
        for (uint32_t j = 0; j < k; ++j) {
            ref_units::ReSTIRGIReservoir s;
            std::memcpy(&s, res28 + ((size_t)i * k + j) * 28, 112);
            ref_units::MergeReservoir(t, s, p_hats[(size_t)i * k + j], seed);
        }
        std::memcpy(out28 + (size_t)i * 28, &t, 112);
        seeds_out[i] = seed;
    }
}
// IsSimilar (both overloads), p_hat, GetTargetPDF, ACESFilm, WorldToScreenUV on
// pairs of samples (24 words each) / points
void ref_similar(const uint32_t* a24, const uint32_t* b24, uint32_t n, uint32_t* out2) {
    for (uint32_t i = 0; i < n; ++i) {
        ref_units::ReSTIRGISample a, b;
        std::memcpy(&a, a24 + 24 * (size_t)i, 96);
        std::memcpy(&b, b24 + 24 * (size_t)i, 96);
        out2[2 * i] = ref_units::IsSimilar(a, b) ? 1u : 0u;
        out2[2 * i + 1] = ref_units::IsSimilar(a.x_view, a.n_view, b.x_view, b.n_view) ? 1u : 0u;
    }
}
void ref_aces(const float* in3, uint32_t n, float* out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const float3 c = ref_units::ACESFilm(float3(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2]));
        out3[3 * i] = c.x; out3[3 * i + 1] = c.y; out3[3 * i + 2] = c.z;
    }
}
void ref_target_pdf(const float* L3, const float* x3, const float* n3, const float* xs3, uint32_t n, float* out2) {
    for (uint32_t i = 0; i < n; ++i) {
        const float3 L(L3[3 * i], L3[3 * i + 1], L3[3 * i + 2]);
        out2[2 * i] = ref_units::p_hat(L);
        out2[2 * i + 1] = ref_units::GetTargetPDF(L, float3(x3[3 * i], x3[3 * i + 1], x3[3 * i + 2]),
                                                  float3(n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]),
                                                  float3(xs3[3 * i], xs3[3 * i + 1], xs3[3 * i + 2]));
    }
}
// EvaluateTargetFunction of the temporal pass (ReSTIRGITemporalReuse.rgen.hlsl:33-40)
// and p_hat (ReSTIRGICommon.hlsl:75-78) for n (sample, x, n) cases
void ref_eval_target(const uint32_t* samples24, const float* x3, const float* n3, uint32_t n, float* out2) {
    for (uint32_t i = 0; i < n; ++i) {
        ref_temporal::ReSTIRGISample smp;
        std::memcpy(&smp, samples24 + 24 * (size_t)i, 96);
        out2[2 * i] = ref_temporal::EvaluateTargetFunction(smp, float3(x3[3 * i], x3[3 * i + 1], x3[3 * i + 2]),
                                                           float3(n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]));
        out2[2 * i + 1] = ref_temporal::p_hat(smp.L_out);
    }
}
void ref_world_to_screen_uv(const float* p3, uint32_t n, const float* view16, const float* proj16, float* out2) {
    hlsl::float4x4 V, P;
    std::memcpy(V.m, view16, 64);
    std::memcpy(P.m, proj16, 64);
    for (uint32_t i = 0; i < n; ++i) {
        const float2 uv = ref_units::WorldToScreenUV(float3(p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]), V, P);
        out2[2 * i] = uv.x; out2[2 * i + 1] = uv.y;
    }
}
// GetNeighborIndex of the spatial pass for pixel (x, y), k picks from the seed
void ref_neighbor_index(uint32_t x, uint32_t y, uint32_t w, uint32_t h, float max_r, uint32_t seed, uint32_t k,
                        uint32_t* out) {
    for (uint32_t j = 0; j < k; ++j) out[j] = ref_spatial::GetNeighborIndex(hlsl::uint2(x, y), hlsl::uint2(w, h), max_r, seed, w);
}

}  // extern "C"
