// texture.cuh -- base-colour textures: bilinear sampling with clamp to edge.
//
// The reference samples its base-colour textures through one Vulkan sampler
// (src/Vulkan/XVKSampler.h:11-27: linear min/mag filtering, clamp-to-edge
// addressing, a single mip level) from R8G8B8A8_UNORM images
// (src/Asset/TextureImage.cpp:25), and a textured material takes the texture's
// RGB *instead of* its base-colour factor (BSDF.hlsl:22-23 for Lambertian and
// the diffuse light alike).  Here: texel centres at (i + 0.5) / size, the four
// texels around x = u * width - 0.5, y = v * height - 0.5 with indices clamped to
// the edge, UNORM values byte / 255, weights (1 - fx, fx) x (1 - fy, fy), every
// operation one binary32 operation in the order written (the CPU oracle does the
// same; a hardware sampler's fixed-point weights would not be reproducible).
#pragma once
#include "device_math.cuh"
#include "xr_internal.h"

namespace xr {

__device__ __forceinline__ float4 texel_unorm(uint32_t v) {
    return make_float4((float)(v & 255u) / 255.0f, (float)((v >> 8) & 255u) / 255.0f,
                       (float)((v >> 16) & 255u) / 255.0f, (float)(v >> 24) / 255.0f);
}

__device__ __forceinline__ float3 tex_bilinear(const DeviceScene& sc, uint32_t t, float2 uv) {
    const uint4 ti = __ldg(sc.tex_info + t);   // {first texel, width, height, 0}
    const int w = (int)ti.y, h = (int)ti.z;
    float x = uv.x * (float)w - 0.5f, y = uv.y * (float)h - 0.5f;
    if (!isfinite(x)) x = 0.0f;
    if (!isfinite(y)) y = 0.0f;
    x = fminf(fmaxf(x, -1.0f), (float)w);
    y = fminf(fmaxf(y, -1.0f), (float)h);
    const float x0f = floorf(x), y0f = floorf(y);
    const float fx = x - x0f, fy = y - y0f;
    const int x0 = (int)x0f, y0 = (int)y0f;
    const int xa = min(max(x0, 0), w - 1), xb = min(max(x0 + 1, 0), w - 1);
    const int ya = min(max(y0, 0), h - 1), yb = min(max(y0 + 1, 0), h - 1);
    const uint32_t* px = sc.texels + ti.x;
    const float4 t00 = texel_unorm(__ldg(px + ya * w + xa)), t10 = texel_unorm(__ldg(px + ya * w + xb));
    const float4 t01 = texel_unorm(__ldg(px + yb * w + xa)), t11 = texel_unorm(__ldg(px + yb * w + xb));
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    const float r = (t00.x * gx + t10.x * fx) * gy + (t01.x * gx + t11.x * fx) * fy;
    const float g = (t00.y * gx + t10.y * fx) * gy + (t01.y * gx + t11.y * fx) * fy;
    const float b = (t00.z * gx + t10.z * fx) * gy + (t01.z * gx + t11.z * fx) * fy;
    return f3(r, g, b);
}

// Material m as seen at texture coordinate uv: a base-colour texture replaces
// the base-colour factor's RGB.
__device__ __forceinline__ XrMaterial resolve_material(const DeviceScene& sc, uint32_t m, float2 uv) {
    XrMaterial r = sc.mats[m];
    if (r.base_color_texture_index >= 0 && (uint32_t)r.base_color_texture_index < sc.n_tex) {
        const float3 c = tex_bilinear(sc, (uint32_t)r.base_color_texture_index, uv);
        r.base_color[0] = c.x;
        r.base_color[1] = c.y;
        r.base_color[2] = c.z;
    }
    return r;
}

}  // namespace xr
