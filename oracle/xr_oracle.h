/*
 * xr_oracle.h -- C ABI of the CPU oracle for the ReSTIR GI frame pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA path: only
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg (and its
 * reference arm) may load it.  The product library never links or calls it.
 *
 * It restates, in plain C++17 with OpenMP over pixels, the reference's HLSL:
 *   shader/HLSL/random.hlsl:1-20                       (RNG)
 *   shader/HLSL/ReSTIRGI/Sampling.hlsl:4-56            (ONB, hemisphere, reprojection)
 *   shader/HLSL/ReSTIRGI/BSDF.hlsl:7-57                (Lambertian / diffuse light)
 *   shader/HLSL/ReSTIRGI/Ray.rchit.hlsl:26-60          (hit attributes)
 *   shader/HLSL/ReSTIRGI/Ray.rmiss.hlsl:3-8            (miss)
 *   shader/HLSL/ReSTIRGI/ReSTIRGICommon.hlsl:6-131     (reservoirs, similarity, ACES)
 *   shader/HLSL/ReSTIRGI/ReSTIRGIInitialSample.rgen.hlsl:35-214
 *   shader/HLSL/ReSTIRGI/ReSTIRGITemporalReuse.rgen.hlsl:33-151
 *   shader/HLSL/ReSTIRGI/ReSTIRGISpatialReuse.rgen.hlsl:35-183
 * plus the host data flow of src/Vulkan/RayTracing/ApplicationReSTIRGI.cpp:150-275.
 *
 * Parity status: the reference has no tests, fixtures or golden vectors and its
 * Vulkan ray-tracing path cannot run without a graphics stack, so this oracle is
 * pinned only by known-answer tests derived from the formulas themselves
 * (tests/golden/) -- "parity unpinned" by reference outputs.
 *
 * Arithmetic contract shared with the CUDA path: every float operation is a
 * single IEEE-754 binary32 operation in the order written (built with
 * -ffp-contract=off), sqrt and division are correctly rounded, sin/cos come from
 * sincos_xr (Cody-Waite reduction + Taylor polynomials, oracle.cpp), and
 * traversal returns the closest hit with ties broken by the lowest primitive id.
 */
#ifndef XR_ORACLE_H
#define XR_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors XrParams in include/xr.h field for field. */
typedef struct OrParams {
    uint32_t width, height;
    uint32_t compat_reference;   /* 1: reproduce the reference's behaviour bit for bit */
    uint32_t temporal_on, spatial_on;
    uint32_t m_cap_temporal, m_cap_spatial;
    uint32_t n_neighbours;
    float    radius_px;
    uint32_t visibility;         /* 1: trace spatial shadow rays (correct mode only) */
    uint32_t seed;
    uint32_t write_pt;           /* also produce the plain 1-spp path-traced estimate */
    uint32_t write_hdr;          /* (the oracle always keeps the linear image) */
} OrParams;

/* Mirrors the reference UniformBufferObject (src/Asset/UniformBuffer.h:16-32), 412 B. */
typedef struct OrUBO {
    float view[16], view_prev[16], projection[16], projection_prev[16];
    float view_inverse[16], projection_inverse[16];
    uint32_t spp, total_number_of_samples, number_of_bounces, random_seed;
    uint32_t has_sky_box, reuse, current_frame;
} OrUBO;

enum {
    OR_BUF_SAMPLES = 0,     /* N  x 24 words, ReSTIRGISample layout (ReSTIRGICommon.hlsl:6-20) */
    OR_BUF_TEMPORAL = 1,    /* 2N x 28 words, ReSTIRGIReservoir layout (ReSTIRGICommon.hlsl:22-30) */
    OR_BUF_SPATIAL = 2,     /* 2N x 28 words */
    OR_BUF_HDR = 3,         /* N x 4 float: linear colour before ACES */
    OR_BUF_LDR = 4,         /* N x 4 u8: ACES + gamma 1/2.2, rounded */
    OR_BUF_PT = 5,          /* N x 4 float: plain 1-spp path-traced radiance */
    OR_BUF_GBUF_POS = 6,    /* N x 4 float (x_view, valid) */
    OR_BUF_MOTION = 7,      /* N x 2 float (after RG16F rounding in compat mode) */
    OR_BUF_WRITTEN = 8,     /* N x u32: 1 where this frame wrote the output image */
    OR_BUF_CACHE_QUERIES = 9,   /* radiance-cache query records of the frame, 8 words each, pixel order */
    OR_BUF_CACHE_TRAIN = 10     /* radiance-cache training records, 12 words each, pixel order */
};

/* ---- known-answer helpers (random.hlsl, Sampling.hlsl) ---- */
uint32_t or_init_random_seed(uint32_t x, uint32_t y, uint32_t width, uint32_t frame);
void or_random_sequence(uint32_t state, uint32_t n, uint32_t* out_u32, float* out_f);
void or_sincos(const float* a, uint32_t n, float* s, float* c);
void or_oct_roundtrip(const float* n3, uint32_t count, uint32_t bits, float* out3, uint32_t* codes);
/* The restated helpers one by one, for the check against the reference's own
   source compiled by oracle/refpin (reference mode).  Layouts: samples 24 words,
   reservoirs 28 words, materials 8 words; sample_bsdf writes {f.rgb, wi.xyz, pdf,
   cos, seed after}; targets writes {EvaluateTargetFunction, p_hat}. */
void or_units_onb(const float* n3, uint32_t n, float* out6);
void or_units_sample_hemisphere(const float* xi2, uint32_t n, float* out3);
void or_units_sample_bsdf(const float* n3, const float* wo3, const uint32_t* materials8, const uint32_t* seeds,
                          uint32_t n, float* out9);
void or_units_update_list(const uint32_t* samples24, const float* weights, uint32_t n, uint32_t k,
                          const uint32_t* seeds, uint32_t* out28, uint32_t* seeds_out);
void or_units_merge_list(const uint32_t* res28, const float* p_hats, uint32_t n, uint32_t k, const uint32_t* seeds,
                         uint32_t* out28, uint32_t* seeds_out);
void or_units_similar(const uint32_t* a24, const uint32_t* b24, uint32_t n, uint32_t* out2);
void or_units_aces(const float* in3, uint32_t n, float* out3);
void or_units_targets(const uint32_t* samples24, const float* x3, const float* n3, uint32_t n, float* out2);
void or_units_world_to_screen_uv(const float* p3, uint32_t n, const float* view16, const float* proj16, float* out2);
void or_units_neighbor_index(uint32_t x, uint32_t y, uint32_t w, uint32_t h, float max_r, uint32_t seed, uint32_t k,
                             uint32_t* out);

/* ---- scene + traversal ---- */
void* or_scene_create(const float* vertices, uint32_t nv, const uint32_t* indices, uint32_t ntri,
                      const float* materials, uint32_t nm);
void or_scene_destroy(void* scene);
/* Base-colour textures: n sizes (width, height pairs) and the RGBA8 texels concatenated. */
void or_scene_set_textures(void* scene, const uint32_t* sizes2, uint32_t n, const uint8_t* rgba8);
/* rays: n x 8 floats (o.xyz, tmin, d.xyz, tmax). any_hit=1 stops at the first hit.
   prim: -1 on miss.  t, bary (b1, b2) are written on hit. */
void or_trace(void* scene, const float* rays, uint32_t n, int any_hit,
              int32_t* prim, float* t, float* bary);

/* ---- instances (instances.cu; Ray.rchit.hlsl:46-55) ----
   A world of n scenes (copied), concatenated as xr_upload_scenes does, traced and
   rendered through its instances: each scene traced with the ray in the instance's
   object space; closest hit by t, then instance, then primitive.  Returns 0 / -1. */
void* or_world_create(void* const* scenes, uint32_t n);
int or_world_set_instances(void* world, const uint32_t* part, const float* o2w12, uint32_t n);
void or_world_transforms(void* world, float* out24);
int or_world_update_vertices(void* world, uint32_t part, const float* vertices9, uint32_t nv);
void or_trace_inst(void* scene, const float* rays, uint32_t n, int any_hit, int32_t* prim, int32_t* inst,
                   float* t, float* bary);

/* ---- the frame pipeline ---- */
void* or_renderer_create(void* scene, const OrParams* params);
void or_renderer_destroy(void* r);
/* Corrected mode: paths end into the learned radiance cache at their first
   secondary vertex (training pixels continue); nrc (or_nrc_create, may be NULL:
   prediction 0) supplies the candidates' radiance.  Returns non-zero in reference mode. */
int or_renderer_set_cache(void* r, int enabled, uint32_t train_samples, void* nrc);
int or_render_frame(void* r, const OrUBO* ubo);
/* Fixed-candidate checks: load samples (N x 24 words, as read back from the
   CUDA path), optionally the temporal reservoirs, then run one reuse pass. */
int or_set_samples(void* r, const float* samples_words, const OrUBO* ubo);
/* Corrected mode: makes the current G-buffer the previous one (end of a frame). */
int or_end_frame(void* r);
int or_run_pass(void* r, const OrUBO* ubo, int pass);   /* 1 = temporal, 2 = spatial */
size_t or_read(void* r, int which, void* dst, size_t bytes);
int or_write_temporal(void* r, const float* words, size_t bytes);

/* FP64-accumulated plain path tracer (same path semantics as the initial-sample
   pass): frames [frame0, frame0+spp) each contribute one sample per pixel. */
int or_pt_reference(void* scene, const OrParams* params, const OrUBO* ubo,
                    uint32_t frame0, uint32_t spp, double* out_rgb);

/* ---- learned radiance cache (nrc.cpp) ----
   Mirrors XrCacheSample in include/xr.h (72 B). */
typedef struct OrCacheSample {
    float pos[3];
    float normal[3];
    float wo[3];
    float albedo[3];
    float roughness;
    uint32_t kind;
    float target[3];
    uint32_t pixel;
} OrCacheSample;

void* or_nrc_create(uint32_t seed);
void or_nrc_destroy(void* nrc);
void or_nrc_set_bounds(void* nrc, const float* lo3, float inv_extent);
/* 0 MLP weights, 1 hash table, 2 MLP gradient, 3 table gradient, 4/5 MLP Adam m/v, 6/7 table Adam m/v */
float* or_nrc_params(void* nrc, int which, size_t* count);
void or_nrc_pack(const OrCacheSample* s, uint32_t n, uint32_t* records8);
void or_nrc_inputs(void* nrc, const uint32_t* records8, uint32_t n, float* x64, int exact);
void or_nrc_infer(void* nrc, const uint32_t* records8, uint32_t n, float* out3, int exact);
double or_nrc_backward(void* nrc, const uint32_t* records8, const float* target3, uint32_t n, int exact,
                       int loss_kind);
double or_nrc_loss(void* nrc, const uint32_t* records8, const float* target3, uint32_t n, int exact, int loss_kind);
void or_nrc_adam(void* nrc, float lr, float b1, float b2, float eps, float bc1, float bc2);

#ifdef __cplusplus
}
#endif
#endif
