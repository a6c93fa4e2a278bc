// bsdf.cuh -- BSDF sampling and evaluation of the frame kernels.
//
// BSDF.hlsl:7-57 (SampleBSDF -> SampleLambertian, cosine hemisphere, f = albedo/pi)
// is reproduced exactly.  Corrected mode adds two lobes the reference lacks:
//   XR_MAT_METALLIC: GGX conductor, F0 = base colour
//   XR_MAT_PLASTIC : GGX dielectric coat (F0 = 0.04) over Lambert * 0.96,
//                    coat sampled with probability 1/4
// GGX with height-correlated Smith masking and Schlick Fresnel; visible-normal
// sampling after Heitz, "Sampling the GGX Distribution of Visible Normals"
// (JCGT 2018).  Roughness = fuzziness clamped to [0.02, 1], alpha = roughness^2.
#pragma once
#include "device_math.cuh"
#include "xr_internal.h"

namespace xr {

struct Lobe { float3 f; float pdf; };

__device__ __forceinline__ float ggx_lambda(float3 w, float a2) {
    float c2 = w.z * w.z;
    float s2 = fmaxf(0.0f, 1.0f - c2);
    return (sqrtf(1.0f + a2 * s2 / c2) - 1.0f) * 0.5f;
}
__device__ __forceinline__ float ggx_d(float nh, float a2) {
    float k = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (XR_PI_F * k * k);
}
__device__ __forceinline__ float3 schlick(float3 f0, float c) {
    float m = 1.0f - c;
    m = fminf(fmaxf(m, 0.0f), 1.0f);
    float m5 = m * m * m * m * m;
    return f0 + (f3(1.0f, 1.0f, 1.0f) - f0) * m5;
}

__device__ __forceinline__ Lobe eval_material(const XrMaterial& m, float3 wo, float3 wi) {
    Lobe r;
    r.f = f3(0.0f, 0.0f, 0.0f);
    r.pdf = 0.0f;
    float3 albedo = f3(m.base_color[0], m.base_color[1], m.base_color[2]);
    if (wi.z <= 0.0f) return r;
    if (m.material_model == XR_MAT_LAMBERTIAN) {
        r.f = albedo * XR_INV_PI_F;
        r.pdf = wi.z * XR_INV_PI_F;
        return r;
    }
    if (wo.z <= 0.0f) return r;
    float rough = fminf(fmaxf(m.fuzziness, 0.02f), 1.0f);
    float alpha = rough * rough;
    float a2 = alpha * alpha;
    float3 h = normalize(wo + wi);
    float nh = h.z, oh = dot(wo, h);
    float d = ggx_d(nh, a2);
    float g2 = 1.0f / (1.0f + ggx_lambda(wo, a2) + ggx_lambda(wi, a2));
    float g1 = 1.0f / (1.0f + ggx_lambda(wo, a2));
    float pdf_spec = g1 * d / (4.0f * wo.z);
    if (m.material_model == XR_MAT_METALLIC) {
        float3 F = schlick(albedo, oh);
        r.f = F * (d * g2 / (4.0f * wo.z * wi.z));
        r.pdf = pdf_spec;
        return r;
    }
    float3 F = schlick(f3(0.04f, 0.04f, 0.04f), oh);
    r.f = F * (d * g2 / (4.0f * wo.z * wi.z)) + albedo * (0.96f * XR_INV_PI_F);
    r.pdf = 0.25f * pdf_spec + 0.75f * (wi.z * XR_INV_PI_F);
    return r;
}

__device__ __forceinline__ float3 sample_vndf(float3 wo, float alpha, float u1, float u2) {
    float3 vh = normalize(f3(alpha * wo.x, alpha * wo.y, wo.z));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    float3 t1 = lensq > 0.0f ? f3(-vh.y, vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : f3(1.0f, 0.0f, 0.0f);
    float3 t2 = cross(vh, t1);
    float r = sqrtf(u1);
    float s, c;
    sincos_xr(XR_TWO_PI_F * u2, &s, &c);
    float p1 = r * c, p2 = r * s;
    float sh = 0.5f * (1.0f + vh.z);
    p2 = (1.0f - sh) * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1)) + sh * p2;
    float3 nh = t1 * p1 + t2 * p2 + vh * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2));
    return normalize(f3(alpha * nh.x, alpha * nh.y, fmaxf(0.0f, nh.z)));
}

// SampleBSDF (BSDF.hlsl:34-57).  In compat mode only the reference's Lambertian
// case samples; other models return f = 0, pdf = 0 as the reference's switch does.
template <bool COMPAT>
__device__ __forceinline__ float3 sample_bsdf(float3 n, const XrMaterial& mat, float3 wo_world, float3* wi_world,
                                              float* pdf_w, float* cos_theta, uint32_t& seed) {
    float3 f = f3(0.0f, 0.0f, 0.0f);
    *pdf_w = 0.0f;
    *cos_theta = 0.0f;
    float3 T, B;
    branchless_onb(n, &T, &B);
    float3 wo_local = to_local(wo_world, T, B, n);
    float3 wi_local = f3(0.0f, 0.0f, 0.0f);
    const uint32_t model = mat.material_model;
    if (model == XR_MAT_LAMBERTIAN) {
        float xi_x = random_float(seed);
        float xi_y = random_float(seed);
        wi_local = sample_hemisphere(xi_x, xi_y);
        *cos_theta = wi_local.z;
        *pdf_w = *cos_theta * XR_INV_PI_F;
        if (*cos_theta <= 0.0f) {
            *pdf_w = 0.0f;
        } else {
            f = f3(mat.base_color[0], mat.base_color[1], mat.base_color[2]) * XR_INV_PI_F;
        }
    } else if (!COMPAT && (model == XR_MAT_METALLIC || model == XR_MAT_PLASTIC)) {
        float rough = fminf(fmaxf(mat.fuzziness, 0.02f), 1.0f);
        float alpha = rough * rough;
        float us = model == XR_MAT_PLASTIC ? random_float(seed) : 0.0f;
        float u1 = random_float(seed), u2 = random_float(seed);
        if (model == XR_MAT_METALLIC || us < 0.25f) {
            if (wo_local.z > 0.0f) {
                float3 h = sample_vndf(wo_local, alpha, u1, u2);
                float oh = dot(wo_local, h);
                wi_local = h * (2.0f * oh) - wo_local;
            }
        } else {
            wi_local = sample_hemisphere(u1, u2);
        }
        Lobe l = eval_material(mat, wo_local, wi_local);
        *cos_theta = wi_local.z;
        *pdf_w = l.pdf;
        f = l.f;
        if (!(l.pdf > 0.0f)) { *pdf_w = 0.0f; f = f3(0.0f, 0.0f, 0.0f); }
    }
    *wi_world = to_world(wi_local, T, B, n);
    return f;
}

// f of the visible point for the reused direction (corrected-mode shading).
__device__ __forceinline__ float3 eval_world(const XrMaterial& m, float3 n, float3 wo, float3 wi) {
    float3 T, B;
    branchless_onb(n, &T, &B);
    return eval_material(m, to_local(wo, T, B, n), to_local(wi, T, B, n)).f;
}

}  // namespace xr
