// restir.cu -- the ReSTIR GI frame: initial sample (wavefront), temporal reuse,
// spatial reuse with fused shading.
//
//   initial sample  ReSTIRGIInitialSample.rgen.hlsl:35-214
//   temporal reuse  ReSTIRGITemporalReuse.rgen.hlsl:33-151
//   spatial reuse   ReSTIRGISpatialReuse.rgen.hlsl:35-183
//   reservoirs      ReSTIRGICommon.hlsl:43-121
//
// The reference runs one ray-generation thread per pixel that loops over the
// bounces.  Here each bounce is one launch over a compacted queue of live
// paths: the first launch generates camera rays per 16x8 pixel tile, every
// launch traces, shades and samples the next direction, and survivors are
// appended to the next queue with one atomic per warp (ballot + popc).  Later
// bounces run on a persistent grid that reads the queue length from device
// memory, so the whole frame is launched without a host round trip.
//
// Per-pixel data is written in the layouts documented in xr_internal.h.
#include <utility>

#include "bsdf.cuh"
#include "nrc.cuh"
#include "texture.cuh"
#include "wavefront_trace.cuh"

namespace xr {
namespace {

constexpr int kBlock = 128;   // raygen (one 16 x 8 tile per block)
// Persistent traversal in one 1024-thread CTA per SM (64 registers: the whole
// register file): swept 128 / 256 / 512 / 1024 threads at the same occupancy,
// 2.597 / 2.577 / 2.552 / 2.525 ms per 1080p frame.  The two-level variants keep
// more state per lane and run one 896-thread CTA per SM (72 registers, no spills).
#ifndef XR_TRACE_BLOCK
#define XR_TRACE_BLOCK 1024
#endif
#ifndef XR_TRACE_BLOCK_INST
#define XR_TRACE_BLOCK_INST 896
#endif
#ifndef XR_SHADE_BLOCK
#define XR_SHADE_BLOCK 128
#endif
constexpr int kTraceBlock = XR_TRACE_BLOCK;   // persistent traversal kernels
constexpr int kTraceBlockInst = XR_TRACE_BLOCK_INST;
template <bool INST> constexpr int trace_block() { return INST ? kTraceBlockInst : kTraceBlock; }
constexpr int kShadeBlock = XR_SHADE_BLOCK;   // persistent shading kernel

struct HitPayload {
    float3 pos, normal, geo;
    float2 uv;
    int32_t mat;
    float t;
};

// Ray.rchit.hlsl:26-60; miss = material -1 (Ray.rmiss.hlsl:3-8).  Without
// instances the object space is the world space (the reference's identity
// instances).  A hit on an instance maps the interpolated position by its
// object-to-world rows (Ray.rchit.hlsl:46-47) and the shading and geometric
// normals by the transpose of its world-to-object rows, the inverse transpose
// (Ray.rchit.hlsl:53 does this for the geometric normal; its shading normal,
// mul(float4(n, 0), WorldToObject4x3()), equals the same thing only for the
// identity transforms it is used with).
__device__ __forceinline__ HitPayload closest_hit(const DeviceScene& sc, const HitRec& h) {
    HitPayload pl;
    uint4 id = __ldg(sc.tri_idx + h.prim);
    float bx = 1.0f - h.b1 - h.b2, by = h.b1, bz = h.b2;
    float3 n0 = xyz(__ldg(sc.vnrm + id.x)), n1 = xyz(__ldg(sc.vnrm + id.y)), n2 = xyz(__ldg(sc.vnrm + id.z));
    float3 nm = n0 * bx + n1 * by + n2 * bz;
    float3 normal = normalize(nm);
    float3 v0 = xyz(__ldg(sc.vpos + id.x)), v1 = xyz(__ldg(sc.vpos + id.y)), v2 = xyz(__ldg(sc.vpos + id.z));
    pl.pos = v0 * bx + v1 * by + v2 * bz;
    pl.uv = make_float2(0.0f, 0.0f);
    if (sc.n_tex) {
        const float2 u0 = __ldg(sc.vuv + id.x), u1 = __ldg(sc.vuv + id.y), u2 = __ldg(sc.vuv + id.z);
        pl.uv = make_float2(u0.x * bx + u1.x * by + u2.x * bz, u0.y * bx + u1.y * by + u2.y * bz);
    }
    float3 e0 = v2 - v0, e1 = v1 - v0;
    float3 geo = cross(e0, e1);
    if (sc.n_inst && h.inst >= 0) {
        const float4* X = sc.inst_xform + 6u * (uint32_t)h.inst;
        const float4 o0 = __ldg(X), o1 = __ldg(X + 1), o2 = __ldg(X + 2);
        const float4 w0 = __ldg(X + 3), w1 = __ldg(X + 4), w2 = __ldg(X + 5);
        pl.pos = xform_point(o0, o1, o2, pl.pos);
        normal = xform_normal(w0, w1, w2, normal);
        geo = xform_normal(w0, w1, w2, geo);
    }
    pl.geo = normalize(geo);
    pl.normal = normalize(normal);
    pl.mat = (int32_t)id.w;
    pl.t = h.t;
    return pl;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// The previous frame's pixel of a visible point (ReSTIRGITemporalReuse.rgen.hlsl:
// motion vector -> previous uv), kInvalid when it falls outside the view.
__device__ __forceinline__ uint32_t reproject(float3 x_view, const XrUniformBufferObject* __restrict__ u, uint32_t W,
                                              uint32_t H, uint32_t base) {
    const float2 puv = world_to_screen_uv(x_view, u->view_prev, u->projection_prev);
    const float fx = floorf(puv.x * (float)W), fy = floorf(puv.y * (float)H);
    if (fx >= 0.0f && fx < (float)W && fy >= 0.0f && fy < (float)H) return base + (uint32_t)fy * W + (uint32_t)fx;
    return kInvalid;
}

// ---- views: a pixel's view, its view-local coordinates and extent ----
__device__ __forceinline__ uint32_t view_index(const FrameArgs& fa, uint32_t p) {
    if (fa.n_views <= 1u) return 0u;
    uint32_t lo = 0, hi = fa.n_views - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (fa.views[mid].pix_off <= p) lo = mid;
        else hi = mid - 1u;
    }
    return lo;
}
struct PixView {
    uint32_t v, x, y, W, H, base;
};
__device__ __forceinline__ PixView pix_view(const FrameArgs& fa, uint32_t p) {
    PixView c;
    if (fa.n_views <= 1u) {
        c.v = 0u; c.base = 0u; c.W = fa.W; c.H = fa.H;
    } else {
        c.v = view_index(fa, p);
        const ViewInfo vi = fa.views[c.v];
        c.base = vi.pix_off; c.W = vi.W; c.H = vi.H;
    }
    const uint32_t l = p - c.base;
    c.x = l % c.W;
    c.y = l / c.W;
    return c;
}
__device__ __forceinline__ uint32_t root_of_pixel(const FrameArgs& fa, uint32_t p) {
    return fa.multi_root ? fa.views[view_index(fa, p)].root : 0u;
}

__device__ __forceinline__ void flag_error(const FrameArgs& fa, uint32_t bits) { atomicOr(&fa.counters[kCntError], bits); }

// ---------------------------------------------------------------------------
// one bounce of one path
// ---------------------------------------------------------------------------
struct PathState {
    float3 o, d, thr;
    uint32_t pixel, rng;
    float pq;
};

template <bool COMPAT>
__device__ __forceinline__ void write_invalid(const FrameArgs& fa, uint32_t p, float3 x_view, float3 n_view, float3 le0) {
    if (COMPAT) {
        fa.s_xv[p] = f4(x_view, __uint_as_float(kInvalid));
        fa.s_nv[p] = f4(n_view, __uint_as_float(0u));
        fa.s_xs[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        fa.s_ns[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        fa.s_L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (fa.write_pt) fa.le0[p] = f4(le0, 0.0f);
    } else {
        fa.gb_pos_cur[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        fa.gb_mat_cur[p] = kInvalid;
        fa.cand_a[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        fa.cand_b[p] = f4(le0, __uint_as_float(0u));
    }
}

template <bool COMPAT>
__device__ __forceinline__ void write_sample(const FrameArgs& fa, uint32_t p, float3 x_s, float3 n_s, float3 L, float pq) {
    if (COMPAT) {
        fa.s_xs[p] = f4(x_s, pq);
        fa.s_ns[p] = f4(n_s, 0.0f);
        fa.s_L[p] = f4(L, 0.0f);
    } else {
        fa.cand_a[p] = f4(x_s, pq);
        fa.cand_b[p] = f4(L, __uint_as_float(oct_encode(n_s, 12) | 0x80000000u));
    }
}

template <bool COMPAT>
__device__ __forceinline__ void add_radiance(const FrameArgs& fa, uint32_t p, float3 add) {
    float4* dst = COMPAT ? fa.s_L : fa.cand_b;
    float4 v = dst[p];
    float3 L = xyz(v) + add;
    dst[p] = f4(L, v.w);
}

// Radiance found at bounce >= 2.  With the radiance cache on, only training
// paths live past bounce 1, and what they find is the training target of their
// record (index carried in the pixel slot, which they no longer need).
template <bool COMPAT>
__device__ __forceinline__ void add_suffix_radiance(const FrameArgs& fa, const PathState& s, float3 add) {
    if (!COMPAT && fa.cache_on) {
        float4* tgt = reinterpret_cast<float4*>(fa.cache_t + (size_t)s.pixel * 3u + 2u);
        float4 v = *tgt;
        *tgt = make_float4(v.x + add.x, v.y + add.y, v.z + add.z, v.w);
    } else {
        add_radiance<COMPAT>(fa, s.pixel, add);
    }
}

// Next-event estimation of the radiance cache's training paths: a light picked
// with probability pmf (its share of the emitted power) by binary search of the
// CDF, a uniform point on it (square-root parameterisation), and the balance
// heuristic against the BSDF sampling of the same vertex, so the contribution is
// thr Le f cos / (pdf_light + pdf_bsdf); an emitter reached by BSDF sampling
// takes the complementary weight.  Same expectation as the plain path tracer's
// emission-only estimate, far lower variance for the small lights.
struct NeeRay {
    bool valid;
    float3 o, d, contrib;
    float tmax;
};

__device__ __forceinline__ uint32_t pick_light(const DeviceScene& sc, float u) {
    uint32_t lo = 0, hi = sc.n_lights - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (u < sc.light_cdf[mid]) hi = mid;
        else lo = mid + 1u;
    }
    return lo;
}

__device__ __forceinline__ NeeRay next_event(const DeviceScene& sc, const XrMaterial& mat, float3 x, float3 n,
                                             float3 g, float3 wo, float3 thr, uint32_t& rng) {
    NeeRay r;
    r.valid = false;
    const float u0 = random_float(rng), u1 = random_float(rng), u2 = random_float(rng);
    if (sc.n_lights == 0u) return r;
    const uint32_t prim = sc.light_prim[pick_light(sc, u0)];
    const uint4 id = __ldg(sc.tri_idx + prim);
    const float3 p0 = xyz(__ldg(sc.vpos + id.x)), p1 = xyz(__ldg(sc.vpos + id.y)), p2 = xyz(__ldg(sc.vpos + id.z));
    const float su = sqrtf(u1);
    const float b0 = 1.0f - su, b1 = u2 * su, b2 = 1.0f - b0 - b1;
    const float3 y = p0 * b0 + p1 * b1 + p2 * b2;
    const float3 nl = normalize(cross(p2 - p0, p1 - p0));
    const float3 dv = y - x;
    const float dist2 = dot(dv, dv);
    const float dist = sqrtf(dist2);
    if (!(dist > 0.05f)) return r;
    const float3 wi = dv * (1.0f / dist);
    const float cos_l = fabsf(dot(nl, wi));
    if (!(cos_l > 1e-6f)) return r;
    float3 T, B;
    branchless_onb(n, &T, &B);
    const float3 wil = to_local(wi, T, B, n);
    if (!(wil.z > 0.0f)) return r;
    const Lobe lb = eval_material(mat, to_local(wo, T, B, n), wil);
    const float pdf_l = sc.prim_light_pdf[prim] * dist2 / cos_l;
    float2 luv = make_float2(0.0f, 0.0f);
    if (sc.n_tex) {
        const float2 t0 = __ldg(sc.vuv + id.x), t1 = __ldg(sc.vuv + id.y), t2 = __ldg(sc.vuv + id.z);
        luv = make_float2(t0.x * b0 + t1.x * b1 + t2.x * b2, t0.y * b0 + t1.y * b1 + t2.y * b2);
    }
    const XrMaterial lm = resolve_material(sc, id.w, luv);
    const float3 Le = f3(lm.base_color[0], lm.base_color[1], lm.base_color[2]) * 4.0f;
    r.contrib = thr * Le * lb.f * (wil.z / (pdf_l + lb.pdf));
    if (!(r.contrib.x + r.contrib.y + r.contrib.z > 0.0f)) return r;
    const float3 off = dot(wi, g) > 0.0f ? g : -g;
    r.o = x + off * 0.01f;
    r.d = wi;
    r.tmax = dist - 0.02f;
    r.valid = true;
    return r;
}

// What the shading of a bounce hands to the radiance cache (corrected mode).
struct CacheEmit {
    bool query;        // bounce 1: x_s is a surface, the candidate takes the cache's radiance
    bool train;        // bounce 1: the pixel is one of the frame's training pixels
    float4 ra;         // record {x_s, pixel}
    uint4 rb;          // record {oct16(n_s), oct16(wo), albedo | kind, roughness}
    NeeRay nee;        // training paths: the next-event ray of this vertex
};

// Training pixels of a frame: (pixel * (2^31 - 1) + off) mod N < sel with
// off = frame * 2654435761 mod N -- a permutation of the pixels that changes every
// frame (the frame index is read on the device, so a replayed graph follows it).
// sel is the device word of k_cache_select_next (adapted every frame).
__device__ __forceinline__ bool cache_training_pixel(const FrameArgs& fa, uint32_t pixel) {
    if (!fa.cache_sel) return false;
    const uint32_t sel = *fa.cache_sel;
    const uint64_t off = ((uint64_t)fa.ubo[0].current_frame * 2654435761ull) % (uint64_t)fa.N;
    const uint64_t k = ((uint64_t)pixel * 2147483647ull + off) % (uint64_t)fa.N;
    return k < sel;
}

// Shades the traced hit `h` of one path: records the bounce's sample fields,
// samples the BSDF and returns true when the path continues to bounce + 1
// (state updated in place).
template <bool COMPAT>
__device__ __forceinline__ bool shade_step(const FrameArgs& fa, const XrUniformBufferObject* __restrict__ u,
                                           uint32_t bounce, uint32_t nb, PathState& s, const HitRec& h,
                                           CacheEmit& ce) {
    const uint32_t p = s.pixel;
    HitPayload pl;
    pl.mat = -1;
    if (h.prim >= 0) pl = closest_hit(fa.sc, h);
    const bool sky = u->has_sky_box != 0u;
    const float3 sky_c = f3(1.0f, 1.0f, 1.0f);
    if (pl.mat == -1) {
        if (bounce == 0) {
            write_invalid<COMPAT>(fa, p, f3(0.0f, 0.0f, 0.0f), f3(0.0f, 0.0f, 0.0f), sky ? sky_c : f3(0.0f, 0.0f, 0.0f));
        } else if (bounce == 1) {
            float3 L = f3(0.0f, 0.0f, 0.0f);
            if (sky) L = L + s.thr * sky_c;
            write_sample<COMPAT>(fa, p, s.o + s.d * 1000.0f, -s.d, L, s.pq);
        } else if (sky) {
            add_suffix_radiance<COMPAT>(fa, s, s.thr * sky_c);
        }
        return false;
    }
    if ((uint32_t)pl.mat >= fa.sc.n_mats) {
        flag_error(fa, XR_DEVFLAG_BAD_INDEX);
        if (bounce == 0) write_invalid<COMPAT>(fa, p, f3(0.0f, 0.0f, 0.0f), f3(0.0f, 0.0f, 0.0f), f3(0.0f, 0.0f, 0.0f));
        else if (bounce == 1) write_sample<COMPAT>(fa, p, f3(0, 0, 0), f3(0, 0, 1), f3(0, 0, 0), s.pq);
        return false;
    }
    const XrMaterial mat = resolve_material(fa.sc, (uint32_t)pl.mat, pl.uv);
    if (bounce == 0 && fa.sc.n_tex) fa.gb_uv[p] = pl.uv;
    if (!COMPAT) {
        float3 wo = -s.d;
        if (dot(pl.geo, wo) < 0.0f) pl.geo = -pl.geo;
        if (dot(pl.normal, pl.geo) < 0.0f) pl.normal = -pl.normal;
    }
    if (mat.material_model == XR_MAT_DIFFUSE_LIGHT) {
        // reference mode: the light's own base colour, untextured, as the reference's
        // initial pass emits it (ReSTIRGIInitialSample.rgen.hlsl:117-121)
        const float* bc = COMPAT ? fa.sc.mats[pl.mat].base_color : mat.base_color;
        float3 base = f3(bc[0], bc[1], bc[2]);
        float3 term = s.thr * base * 4.0f;
        if (bounce == 0) {
            write_invalid<COMPAT>(fa, p, pl.pos, pl.normal, base * 4.0f);
        } else if (bounce == 1) {
            float3 L = f3(0.0f, 0.0f, 0.0f) + term;
            write_sample<COMPAT>(fa, p, pl.pos, pl.normal, L, s.pq);
        } else {
            float3 add = term;
            if (!COMPAT && fa.cache_on) {
                // balance heuristic against the previous vertex's next-event estimate
                // (its sampling pdf is carried in the p_q slot)
                const float lp = fa.sc.n_lights ? fa.sc.prim_light_pdf[h.prim] : 0.0f;   // no tables without lights
                const float cos_l = fabsf(dot(pl.geo, s.d));
                const float pdf_l = (lp > 0.0f && cos_l > 1e-6f && pl.t > 0.05f) ? lp * (pl.t * pl.t) / cos_l : 0.0f;
                add = term * (s.pq / (s.pq + pdf_l));
            }
            add_suffix_radiance<COMPAT>(fa, s, add);
        }
        return false;
    }
    float pdf = 0.0f, cos_theta = 0.0f;
    float3 wi;
    const float3 wo = -s.d;
    const float3 x_s = pl.pos, n_s = pl.normal;
    const uint32_t seed_this = s.rng;
    if (!COMPAT && fa.cache_on && bounce >= 1u && bounce + 1u < nb &&
        (bounce >= 2u || cache_training_pixel(fa, p)))
        ce.nee = next_event(fa.sc, mat, pl.pos, pl.normal, pl.geo, wo, s.thr, s.rng);
    // Corrected mode without the cache: at the last bounce (past bounce 1) the path
    // ends and nothing below reads the sampled direction, its pdf or the throughput,
    // so the BSDF is not sampled (the path's random state is not used again).
    const bool last = !COMPAT && !fa.cache_on && bounce >= 2u && bounce + 1u >= nb;
    float3 f = f3(0.0f, 0.0f, 0.0f);
    if (!last) f = sample_bsdf<COMPAT>(pl.normal, mat, wo, &wi, &pdf, &cos_theta, s.rng);
    float3 factor = div3(f * cos_theta, pdf);
    if (!COMPAT && !(pdf > 0.0f)) factor = f3(0.0f, 0.0f, 0.0f);
    bool alive = COMPAT ? true : (pdf > 0.0f);
    if (bounce == 0) {
        if (COMPAT) {
            fa.s_xv[p] = f4(pl.pos, __uint_as_float((uint32_t)pl.mat));
            fa.s_nv[p] = f4(pl.normal, __uint_as_float(seed_this));
        } else {
            fa.gb_pos_cur[p] = f4(pl.pos, __uint_as_float(oct_encode(pl.normal, 16)));
            fa.gb_mat_cur[p] = (uint32_t)pl.mat;
            // the temporal pass's reprojection, done here where the visible point is
            // known so that the temporal pass can gather the previous frame at once
            if (fa.temporal_on) {
                const PixView pv = pix_view(fa, p);
                fa.reproj[p] = reproject(pl.pos, u, pv.W, pv.H, pv.base);
            }
        }
        if (fa.write_pt) fa.thr0[p] = f4(factor, 0.0f);
        s.pq = pdf;
    } else {
        s.thr = s.thr * factor;
    }
    if (alive && bounce > 3) {
        float pr = fmaxf(s.thr.x, fmaxf(s.thr.y, s.thr.z));
        if (random_float(s.rng) > pr) alive = false;
        else s.thr = s.thr * (1.0f / pr);
    }
    if (bounce + 1 >= nb) alive = false;   // the next iteration would hit the depth limit
    if (bounce == 1) write_sample<COMPAT>(fa, p, x_s, n_s, f3(0.0f, 0.0f, 0.0f), s.pq);
    if (!COMPAT && fa.cache_on && bounce == 1) {
        ce.query = true;
        ce.train = cache_training_pixel(fa, p);
        ce.ra = f4(x_s, __uint_as_float(p));
        ce.rb = nrc::pack_b(n_s, wo, f3(mat.base_color[0], mat.base_color[1], mat.base_color[2]),
                            mat.material_model, mat.fuzziness);
    }
    if (bounce == 0 && !alive) {
        if (COMPAT) {
            fa.s_xs[p] = make_float4(0.0f, 0.0f, 0.0f, pdf);
            fa.s_ns[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            fa.s_L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            fa.cand_a[p] = make_float4(0.0f, 0.0f, 0.0f, pdf);
            fa.cand_b[p] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0u));
        }
    }
    if (alive) {
        float3 hit_pos = s.o + s.d * pl.t;
        float3 off = dot(wi, pl.geo) > 0.0f ? pl.geo : -pl.geo;
        s.o = hit_pos + off * 0.01f;
        s.d = wi;
        if (bounce == 0) s.thr = f3(1.0f, 1.0f, 1.0f);
        // training paths of the cache carry their sampling pdf for the MIS weight
        // of an emitter at the next vertex (p_q was written with the sample above)
        if (!COMPAT && fa.cache_on && bounce >= 1u) s.pq = pdf;
    }
    return alive;
}

// Appends the alive paths of a whole block to the next bounce's queue (all threads
// of the block call it): one atomic per block -- appends from all warps of the grid
// go to the same counter, whose atomics serialise.
template <int BLOCK>
__device__ __forceinline__ void push_path_block(const FrameArgs& fa, bool alive, const PathState& s, uint32_t qslot) {
    constexpr int kWarps = BLOCK / 32;
    __shared__ uint32_t warp_base[kWarps + 1];
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, alive);
    if (lane == 0u) warp_base[warp] = (uint32_t)__popc(mask);
    __syncthreads();
    if (threadIdx.x == 0u) {
        uint32_t run = 0u;
        for (int w = 0; w < kWarps; w++) { const uint32_t c = warp_base[w]; warp_base[w] = run; run += c; }
        warp_base[kWarps] = run ? atomicAdd(&fa.counters[qslot], run) : 0u;
    }
    __syncthreads();
    if (alive) {
        const uint32_t i = warp_base[kWarps] + warp_base[warp] + (uint32_t)__popc(mask & ((1u << lane) - 1u));
        fa.q_out[0][i] = f4(s.o, __uint_as_float(s.pixel));
        fa.q_out[1][i] = f4(s.d, __uint_as_float(s.rng));
        fa.q_out[2][i] = f4(s.thr, s.pq);
    }
    __syncthreads();   // warp_base is reused by the next call
}

// Radiance-cache records of bounce 1 (all lanes of the warp call this): one
// query per surface x_s, appended with one atomic per warp; training pixels also
// take a training record (target zero, filled by the rest of the path) and keep
// their path alive with the record index in the p_q slot; every other path ends.
// Appends the valid next-event rays of the warp (all lanes call this) for the
// training record `rec`.
__device__ __forceinline__ void push_nee(const FrameArgs& fa, bool valid, const NeeRay& r, uint32_t rec) {
    const uint32_t lane = lane_id();
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, valid);
    if (mask == 0u) return;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&fa.counters[kCntCacheNee], (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (valid) {
        const uint32_t i = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
        if (i < fa.cache_t_cap) {
            fa.cache_nee[(size_t)i * 3u] = f4(r.o, __uint_as_float(rec));
            fa.cache_nee[(size_t)i * 3u + 1u] = f4(r.d, r.tmax);
            fa.cache_nee[(size_t)i * 3u + 2u] = f4(r.contrib, 0.0f);
        } else {
            flag_error(fa, XR_DEVFLAG_QUEUE_OVERFLOW);
        }
    }
}

__device__ __forceinline__ bool cache_emit(const FrameArgs& fa, const CacheEmit& ce, bool alive, PathState& s) {
    const uint32_t lane = lane_id();
    const uint32_t qmask = __ballot_sync(0xFFFFFFFFu, ce.query);
    if (qmask) {
        const int leader = __ffs(qmask) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&fa.counters[kCntCacheQuery], (uint32_t)__popc(qmask));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (ce.query) {
            const uint32_t q = base + (uint32_t)__popc(qmask & ((1u << lane) - 1u));
            if (q < fa.N) {
                fa.cache_q[(size_t)q * 2u] = make_uint4(__float_as_uint(ce.ra.x), __float_as_uint(ce.ra.y),
                                                        __float_as_uint(ce.ra.z), __float_as_uint(ce.ra.w));
                fa.cache_q[(size_t)q * 2u + 1u] = ce.rb;
            } else {
                flag_error(fa, XR_DEVFLAG_QUEUE_OVERFLOW);
            }
        }
    }
    const bool want = ce.query && ce.train;
    const uint32_t tmask = __ballot_sync(0xFFFFFFFFu, want);
    bool trained = false;
    if (tmask) {
        const int leader = __ffs(tmask) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&fa.counters[kCntCacheTrain], (uint32_t)__popc(tmask));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (want) {
            const uint32_t t = base + (uint32_t)__popc(tmask & ((1u << lane) - 1u));
            if (t < fa.cache_t_cap) {
                fa.cache_t[(size_t)t * 3u] = make_uint4(__float_as_uint(ce.ra.x), __float_as_uint(ce.ra.y),
                                                        __float_as_uint(ce.ra.z), __float_as_uint(ce.ra.w));
                fa.cache_t[(size_t)t * 3u + 1u] = ce.rb;
                fa.cache_t[(size_t)t * 3u + 2u] = make_uint4(0u, 0u, 0u, 0u);
                s.pixel = t;
                trained = true;
            }
        }
    }
    push_nee(fa, trained && ce.nee.valid, ce.nee, s.pixel);
    return alive && trained;
}

// Z-order of a pixel in an 8 x 4 block (x bits 0..2, y bits 0..1 interleaved from x):
// runs of 8 consecutive slots are 4 x 2 pixel squares.
__device__ __forceinline__ uint32_t morton_8x4(uint32_t x, uint32_t y) {
    return (x & 1u) | ((y & 1u) << 1) | ((x & 2u) << 1) | ((y & 2u) << 2) | ((x & 4u) << 2);
}

// Camera rays (ReSTIRGIInitialSample.rgen.hlsl:41-52) for a 16 x 8 pixel tile per
// block, appended to the queue of bounce 0 in tile order.
template <bool COMPAT>
__global__ void __launch_bounds__(kBlock) k_raygen(FrameArgs fa, const XrUniformBufferObject* __restrict__ ubos, uint32_t nb) {
    // tile -> view (tiles of every view in one 1-D grid, view by view)
    uint32_t v = 0;
    if (fa.n_views > 1u) {
        uint32_t lo = 0, hi = fa.n_views - 1u;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1u) >> 1;
            if (fa.views[mid].tile_off <= blockIdx.x) lo = mid;
            else hi = mid - 1u;
        }
        v = lo;
    }
    uint32_t VW = fa.W, VH = fa.H, base = 0u, lt = blockIdx.x;
    if (fa.n_views > 1u) {
        const ViewInfo vi = fa.views[v];
        VW = vi.W; VH = vi.H; base = vi.pix_off; lt = blockIdx.x - vi.tile_off;
    }
    const XrUniformBufferObject* __restrict__ u = ubos + v;
    const uint32_t tiles_x = (VW + 15u) / 16u;
    const uint32_t tx = lt % tiles_x, ty = lt / tiles_x;
    const uint32_t x = tx * 16u + (threadIdx.x & 15u);
    const uint32_t y = ty * 8u + (threadIdx.x >> 4);
    const bool inside = x < VW && y < VH;
    PathState s;
    bool alive = false;
    if (inside) {
        s.pixel = base + y * VW + x;
        s.rng = pass_rng(COMPAT, x, y, VW, u->current_frame, kPassInitial, fa.seed);
        float ox = random_float(s.rng);
        float oy = random_float(s.rng);
        float px = (float)x + ox, py = (float)y + oy;
        float uvx = (px / (float)VW) * 2.0f - 1.0f, uvy = (py / (float)VH) * 2.0f - 1.0f;
        float4 origin = mat_mul(u->view_inverse, make_float4(0.0f, 0.0f, 0.0f, 1.0f));
        float4 target = mat_mul(u->projection_inverse, make_float4(uvx, uvy, 1.0f, 1.0f));
        float3 tn = normalize(xyz(target));
        s.d = normalize(xyz(mat_mul(u->view_inverse, make_float4(tn.x, tn.y, tn.z, 0.0f))));
        s.o = xyz(origin);
        s.thr = f3(1.0f, 1.0f, 1.0f);
        s.pq = 0.0f;
        if (nb == 0u) write_invalid<COMPAT>(fa, s.pixel, f3(0, 0, 0), f3(0, 0, 0), f3(0, 0, 0));
        else alive = true;
    }
    // Every pixel starts a path, so its queue slot is its index in tile order: the
    // view's first pixel, the full tile rows above (only the last can be short),
    // the tiles to the left in this row, the position inside the (possibly cut) tile.
    // In a full tile the 32 slots a warp fetches first cover an 8 x 4 block (four blocks
    // per tile) rather than two 16-pixel rows: squarer bundles of camera rays (the
    // default bundle; the tuner may pick 16 x 2 rows or 4 x 8 blocks instead).
    if (alive) {
        const uint32_t rows = min(8u, VH - ty * 8u), cols = min(16u, VW - tx * 16u);
        const uint32_t xi = threadIdx.x & 15u, yi = threadIdx.x >> 4;
        uint32_t in_tile = yi * cols + xi;   // a cut tile, and bundle 1 (16 x 2 rows): row order
        if (rows == 8u && cols == 16u) {
            if (fa.ray_bundle == 0u) in_tile = ((yi >> 2) * 2u + (xi >> 3)) * 32u + morton_8x4(xi & 7u, yi & 3u);
            else if (fa.ray_bundle == 2u) in_tile = (xi >> 2) * 32u + yi * 4u + (xi & 3u);   // 4 x 8 blocks
        }
        const uint32_t i = base + ty * 8u * VW + tx * 16u * rows + in_tile;
        fa.q_out[0][i] = f4(s.o, __uint_as_float(s.pixel));
        fa.q_out[1][i] = f4(s.d, __uint_as_float(s.rng));
        // corrected mode: bounce 0's shading starts from unit throughput itself (k_shade)
        if (COMPAT) fa.q_out[2][i] = f4(s.thr, s.pq);
    }
    if (blockIdx.x == 0u && threadIdx.x == 0u) fa.counters[0] = nb ? fa.N : 0u;   // the paths of bounce 0
}

// Camera rays search first up to this multiple of the distance from the camera to
// the pixel's visible point of the previous frame (0: off).  On the 1080p benchmark
// path 1.4% of the rays find nothing inside it and are traced again; node visits per
// camera ray drop from 14.3 to 11.4 and triangle tests from 5.9 to 3.5.
#ifndef XR_CAMERA_BOUND_MARGIN
#define XR_CAMERA_BOUND_MARGIN 1.02f
#endif
// In a BVH of fewer nodes the bound has little to cull and its G-buffer reads cost more
// than it saves (Cornell box, 4 nodes: 0.192 -> 0.196-0.203 ms per 256 x 256 frame).
constexpr uint32_t kCameraBoundMinNodes = 256;

// Closest hits of the paths of one bounce (TMin 1e-4, TMax 1e4,
// ReSTIRGIInitialSample.rgen.hlsl:79-80), one 16-byte hit record per queue slot.
// With several scenes each ray starts at its view's root; a path whose pixel slot
// holds a cache training record (pixel_is_record) finds its pixel in the record.
// BOUND (corrected mode, bounce 0): each camera ray first searches up to
// just past its pixel's previous visible point, then (on a miss) up to TMax, with the
// same hits (trace_persistent's RETRY).
template <bool INST, bool BOUND>
__global__ void __launch_bounds__(trace_block<INST>(), 1) k_trace_paths(FrameArgs fa, const float4* __restrict__ q0,
                                                        const float4* __restrict__ q1, uint4* __restrict__ hits,
                                                        const uint32_t* count_ptr, uint32_t* next, uint32_t* err,
                                                        uint32_t* nonfinite, uint32_t pixel_is_record) {
    const uint32_t count = *(volatile const uint32_t*)count_ptr;
    trace_persistent<false, INST, BOUND>(
        fa.sc, count, next,
        [&](uint32_t i) {
            float4 a = q0[i], b = q1[i];
            RayIn r;
            r.o = xyz(a); r.d = xyz(b); r.tmin = 0.0001f; r.tmax = 10000.0f;
            r.root = 0u;
            if (fa.multi_root) {
                uint32_t p = __float_as_uint(a.w);
                if (pixel_is_record) p = fa.cache_t[(size_t)p * 3u].w;
                r.root = root_of_pixel(fa, p);
            }
            if (BOUND) {
                const uint32_t p = __float_as_uint(a.w);
                if (fa.gb_mat_prev[p] != kInvalid) {
                    const float3 dx = xyz(fa.gb_pos_prev[p]) - r.o;
                    const float bound = sqrtf(dot(dx, dx)) * XR_CAMERA_BOUND_MARGIN;
                    if (bound > r.tmin && bound < r.tmax) r.tmax = bound;   // false for NaN
                }
            }
            return r;
        },
        [&](uint32_t i, const HitRec& h) {
            hits[i] = make_uint4((uint32_t)h.prim, __float_as_uint(h.t), __float_as_uint(h.b1), __float_as_uint(h.b2));
            if (INST) fa.hit_inst[i] = h.inst;
        },
        err, nullptr, nonfinite, 10000.0f);
}

// Shading of one bounce over the queue (persistent grid): coherent per-path
// work after the divergent traversal.
template <bool COMPAT>
// Shading is bound by its dependent gathers (hit -> indices -> vertices ->
// material): 8 CTAs per SM (64 registers, 100 bytes spilled) hide them better than
// the 5 that 96 registers allow (1080p frame 2.68 -> 2.64 ms).
#ifndef XR_SHADE_MIN_BLOCKS
#define XR_SHADE_MIN_BLOCKS 8
#endif
__global__ void __launch_bounds__(kShadeBlock, XR_SHADE_MIN_BLOCKS * 128 / kShadeBlock) k_shade(FrameArgs fa, const XrUniformBufferObject* __restrict__ u, uint32_t bounce,
                                                  uint32_t nb) {
    const uint32_t count = *(volatile const uint32_t*)&fa.counters[bounce];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
        uint32_t i = base + threadIdx.x;
        PathState s;
        bool alive = false;
        CacheEmit ce;
        ce.query = false;
        ce.train = false;
        ce.nee.valid = false;
        if (i < count) {
            float4 a = fa.q_in[0][i], b = fa.q_in[1][i];
            // corrected mode: a camera path's throughput is 1 and its p_q 0 (raygen's values), not read back
            const float4 c = (COMPAT || bounce > 0u) ? fa.q_in[2][i] : make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            uint4 hr = fa.hits[i];
            s.o = xyz(a); s.pixel = __float_as_uint(a.w);
            s.d = xyz(b); s.rng = __float_as_uint(b.w);
            s.thr = xyz(c); s.pq = c.w;
            HitRec h;
            h.prim = (int32_t)hr.x; h.t = __uint_as_float(hr.y); h.b1 = __uint_as_float(hr.z); h.b2 = __uint_as_float(hr.w);
            h.inst = fa.sc.n_inst ? fa.hit_inst[i] : -1;
            const XrUniformBufferObject* __restrict__ uv = u;
            if (fa.n_views > 1u) {
                uint32_t p = s.pixel;
                if (!COMPAT && fa.cache_on && bounce >= 2u) p = fa.cache_t[(size_t)p * 3u].w;
                uv = u + view_index(fa, p);
            }
            alive = shade_step<COMPAT>(fa, uv, bounce, nb, s, h, ce);
        }
        if (!COMPAT && fa.cache_on && bounce == 1u) alive = cache_emit(fa, ce, alive, s);
        if (!COMPAT && fa.cache_on && bounce >= 2u) push_nee(fa, ce.nee.valid, ce.nee, s.pixel);
        push_path_block<kShadeBlock>(fa, alive, s, bounce + 1u);
    }
}

// ---------------------------------------------------------------------------
// reservoir passes
// ---------------------------------------------------------------------------
struct Res {            // one reservoir in registers (selected sample + weights)
    float3 xs, L, ns, f;
    uint32_t code;      // corrected layout: oct12 code of ns
    float w_sum, W;
    uint32_t m;
};
__device__ __forceinline__ void res_init(Res& r) {
    r.xs = f3(0, 0, 0); r.L = f3(0, 0, 0); r.ns = f3(0, 0, 0); r.f = f3(0, 0, 0);
    r.code = 0u; r.w_sum = 0.0f; r.W = 0.0f; r.m = 0u;
}
// UpdateReservoir (ReSTIRGICommon.hlsl:52-61): candidate fields passed by value
// Returns whether the candidate replaced the reservoir's sample.
__device__ __forceinline__ bool res_update(Res& r, const Res& cand, float w_new, uint32_t& seed) {
    r.w_sum += w_new;
    r.m++;
    if (random_float(seed) < w_new / fmaxf(1e-10f, r.w_sum)) {
        r.xs = cand.xs; r.L = cand.L; r.ns = cand.ns; r.f = cand.f; r.code = cand.code;
        return true;
    }
    return false;
}
// MergeReservoir (ReSTIRGICommon.hlsl:63-73)
__device__ __forceinline__ bool res_merge(Res& t, const Res& src, float p_hat, uint32_t& seed) {
    uint32_t M0 = t.m;
    float w_new = p_hat * src.W * (float)src.m;
    const bool took = res_update(t, src, w_new, seed);
    t.m = M0 + src.m;
    return took;
}
// ReSTIRGITemporalReuse.rgen.hlsl:33-40
__device__ __forceinline__ float eval_target(float3 xs, float3 L, float3 x_curr, float3 n_curr) {
    float3 wi = normalize(xs - x_curr);
    float c = dot(n_curr, wi);
    if (c <= 0.0f) return 0.0f;
    return length(L);
}

__device__ __forceinline__ void load_wide(const FrameArgs& fa, float4* const* planes, uint32_t i, Res& r) {
    float4 a = planes[0][i], b = planes[1][i], c = planes[2][i], d = planes[3][i];
    r.xs = xyz(a); r.W = a.w;
    r.L = xyz(b); r.w_sum = b.w;
    r.ns = xyz(c); r.m = __float_as_uint(c.w);
    r.f = xyz(d); r.code = 0u;
}
__device__ __forceinline__ void store_wide(float4* const* planes, uint32_t i, const Res& r) {
    planes[0][i] = f4(r.xs, r.W);
    planes[1][i] = f4(r.L, r.w_sum);
    planes[2][i] = f4(r.ns, __uint_as_float(r.m));
    planes[3][i] = f4(r.f, 0.0f);
}
// with_normal = false leaves ns zero: the passes that never read the sample normal
// (temporal; resolve, whose Jacobians were evaluated by select) skip its decode.
__device__ __forceinline__ void decode_packed(float4 a, float4 b, Res& r, bool with_normal = true) {
    uint32_t w = __float_as_uint(b.w);
    r.xs = xyz(a); r.W = a.w;
    r.L = xyz(b);
    r.code = w & 0x00FFFFFFu;
    r.m = w >> 24;
    r.ns = with_normal ? oct_decode(r.code, 12) : f3(0, 0, 0);
    r.f = f3(0, 0, 0);
    r.w_sum = 0.0f;
}
__device__ __forceinline__ void load_packed(const float4* p0, const float4* p1, uint32_t i, Res& r,
                                            bool with_normal = true) {
    decode_packed(p0[i], p1[i], r, with_normal);
}
__device__ __forceinline__ void store_packed(float4* p0, float4* p1, uint32_t i, const Res& r) {
    p0[i] = f4(r.xs, r.W);
    p1[i] = f4(r.L, __uint_as_float((r.code & 0x00FFFFFFu) | (r.m << 24)));
}

__device__ __forceinline__ void write_out(const FrameArgs& fa, uint32_t p, float3 c, bool tonemap) {
    if (fa.out_hdr) fa.out_hdr[p] = f4(c, 1.0f);
    if (tonemap) {
        fa.out_ldr[p] = tonemap_ldr(c);
    } else {
        fa.out_ldr[p] = make_uchar4(unorm8(c.x), unorm8(c.y), unorm8(c.z), 255);
    }
}

__device__ __forceinline__ float3 mat_albedo_over_pi(const FrameArgs& fa, uint32_t m, uint32_t p) {
    if (m >= fa.sc.n_mats) return f3(0.0f, 0.0f, 0.0f);
    const XrMaterial mm = resolve_material(fa.sc, m, fa.sc.n_tex ? fa.gb_uv[p] : make_float2(0.0f, 0.0f));
    return f3(mm.base_color[0], mm.base_color[1], mm.base_color[2]) * XR_INV_PI_F;
}

// ---- temporal, compat layout (the reference's fields and quirks) ----
__global__ void __launch_bounds__(256) k_temporal_compat(FrameArgs fa, const XrUniformBufferObject* __restrict__ u, bool out_here) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    const PixView pv = pix_view(fa, p);
    u += pv.v;
    const uint32_t x = pv.x, y = pv.y, N = fa.N;
    uint32_t rng = pass_rng(true, x, y, pv.W, u->current_frame, kPassTemporal, fa.seed);
    const uint32_t pp = u->current_frame % 2u;
    const uint32_t cur = pp * N, prev = (1u - pp) * N;
    float4 xv = fa.s_xv[p], nv = fa.s_nv[p], xs = fa.s_xs[p], ns = fa.s_ns[p], Lv = fa.s_L[p];
    const uint32_t mat = __float_as_uint(xv.w);
    if (fa.write_pt) {
        float3 v = mat != kInvalid ? xyz(fa.thr0[p]) * xyz(Lv) : xyz(fa.le0[p]);
        fa.out_pt[p] = f4(v, 1.0f);
    }
    if (length(xyz(ns)) == 0.0f) {
        Res e; res_init(e);
        store_wide(fa.rw, cur + p, e);
        store_wide(fa.rsw, cur + p, e);
        return;
    }
    bool found = false;
    Res r_prev; res_init(r_prev);
    {
        float2 cuv = make_float2(((float)x + 0.5f) / (float)pv.W, ((float)y + 0.5f) / (float)pv.H);
        float2 puv0 = world_to_screen_uv(xyz(xv), u->view_prev, u->projection_prev);
        float mvx = half_round(cuv.x - puv0.x), mvy = half_round(cuv.y - puv0.y);
        float fx = (cuv.x - mvx) * (float)pv.W, fy = (cuv.y - mvy) * (float)pv.H;
        if (fx > -1.0f && fx < (float)pv.W && fy > -1.0f && fy < (float)pv.H) {
            uint32_t q = pv.base + (uint32_t)(int)fy * pv.W + (uint32_t)(int)fx;
            // previous G-buffer aliases the current one: validity of this frame at q
            if (__float_as_uint(fa.s_xv[q].w) != kInvalid) {
                load_wide(fa, fa.rw, prev + q, r_prev);
                found = true;
            } else {
                Res e; res_init(e);
                store_wide(fa.rsw, cur + p, e);
            }
        }
    }
    if (!fa.temporal_on) found = false;
    Res s_new;
    s_new.xs = xyz(xs); s_new.L = xyz(Lv); s_new.ns = xyz(ns); s_new.f = mat_albedo_over_pi(fa, mat, p); s_new.code = 0u;
    const float3 x_curr = xyz(xv);
    const float3 n_curr = normalize(xyz(nv));
    Res r; res_init(r);
    r.code = 0u;
    float tp_new = eval_target(s_new.xs, s_new.L, x_curr, n_curr);
    float w_new = (xs.w > 1e-6f) ? (tp_new / xs.w) : 0.0f;
    res_update(r, s_new, w_new, rng);
    if (found) {
        float tp_prev = eval_target(r_prev.xs, r_prev.L, x_curr, n_curr);
        res_merge(r, r_prev, tp_prev, rng);
    } else {
        r.m = 1u;
    }
    if (r.m > 30u) {
        r.w_sum *= (float)30u / (float)r.m;
        r.m = 30u;
    }
    float tpf = eval_target(r.xs, r.L, x_curr, n_curr);
    r.W = (tpf > 1e-6f && r.m > 0u) ? r.w_sum / ((float)r.m * tpf) : 0.0f;
    store_wide(fa.rw, cur + p, r);
    if (out_here) {
        float3 c = f3(0, 0, 0);
        if (r.W > 0.0f) {
            float3 wi = normalize(r.xs - x_curr);
            float ct = fmaxf(0.0f, dot(xyz(nv), wi));
            c = r.L * r.W * r.f * ct;
        }
        write_out(fa, p, c, true);
    }
}

__device__ __forceinline__ uint32_t neighbor_index(uint32_t x, uint32_t y, uint32_t W, uint32_t H, float max_r, uint32_t& seed) {
    float randa = random_float(seed) * 2.0f * XR_PI_F;
    float randr = sqrtf(random_float(seed)) * max_r;
    float s, c;
    sincos_xr(randa, &s, &c);
    int32_t ox = (int32_t)floorf(c * randr), oy = (int32_t)floorf(s * randr);
    int32_t cx = min(max((int32_t)x + ox, 0), (int32_t)W - 1);
    int32_t cy = min(max((int32_t)y + oy, 0), (int32_t)H - 1);
    return (uint32_t)cy * W + (uint32_t)cx;
}

__device__ __forceinline__ float jacobian_of(float3 x_nb_view, float3 x_view, float3 xs, float3 ns) {
    float3 v_orig = x_nb_view - xs;
    float d2o = dot(v_orig, v_orig);
    float3 v_curr = x_view - xs;
    float d2c = dot(v_curr, v_curr);
    float jac = 1.0f;
    if (d2o > 1e-6f && d2c > 1e-6f) {
        float3 dir_o = v_orig * (1.0f / sqrtf(d2o));
        float3 dir_c = v_curr * (1.0f / sqrtf(d2c));
        float cpo = fmaxf(0.0f, dot(ns, dir_o));
        float cpc = fmaxf(0.0f, dot(ns, dir_c));
        if (cpo > 1e-6f) jac = (cpc * d2o) / (cpo * d2c);
    }
    return fminf(fmaxf(jac, 0.1f), 10.0f);
}

// ---- spatial, compat layout ----
__global__ void __launch_bounds__(256) k_spatial_compat(FrameArgs fa, const XrUniformBufferObject* __restrict__ u) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    const PixView pv = pix_view(fa, p);
    u += pv.v;
    const uint32_t x = pv.x, y = pv.y, N = fa.N;
    uint32_t rng = pass_rng(true, x, y, pv.W, u->current_frame, kPassSpatial, fa.seed);
    const uint32_t pp = u->current_frame % 2u;
    const uint32_t read_off = pp * N, write_off = (1u - pp) * N;
    const bool reuse = u->reuse != 0u;
    float4 xv = fa.s_xv[p], nv = fa.s_nv[p], ns = fa.s_ns[p];
    // background black, lights white: written whatever `reuse` says (ReSTIRGISpatialReuse.rgen.hlsl:80-89)
    if (length(xyz(nv)) == 0.0f) { write_out(fa, p, f3(0, 0, 0), false); return; }
    if (length(xyz(ns)) == 0.0f) { write_out(fa, p, f3(1, 1, 1), false); return; }
    const uint32_t mat = __float_as_uint(xv.w);
    Res center; load_wide(fa, fa.rw, read_off + p, center);
    Res r; res_init(r);
    res_merge(r, center, length(center.L), rng);
    for (int i = 0; i < 6; i++) {
        uint32_t nbi = pv.base + neighbor_index(x, y, pv.W, pv.H, 5.0f, rng);
        float4 nxv = fa.s_xv[nbi], nnv = fa.s_nv[nbi];
        if (length(xyz(nnv)) == 0.0f) continue;
        float3 dd = xyz(xv) - xyz(nxv);
        if (dot(dd, dd) > 0.1f) continue;
        if (dot(xyz(nv), xyz(nnv)) < 0.8f) continue;
        if (mat != __float_as_uint(nxv.w)) continue;
        Res rn; load_wide(fa, fa.rw, read_off + nbi, rn);
        float jac = jacobian_of(xyz(nxv), xyz(xv), rn.xs, rn.ns);
        float ph = length(rn.L) * jac;
        res_merge(r, rn, ph, rng);
        if (ph == 0.0f) r.m -= rn.m;
    }
    r.m = min(r.m, 300u);
    float phf = length(r.L);
    r.W = (phf > 1e-6f && r.m > 0u) ? r.w_sum / ((float)r.m * phf) : 0.0f;
    store_wide(fa.rsw, write_off + p, r);
    if (reuse) {
        float3 c = f3(0, 0, 0);
        if (r.W > 0.0f) {
            float3 wi = normalize(r.xs - xyz(xv));
            float ct = fmaxf(0.0f, dot(xyz(nv), wi));
            c = r.L * r.W * r.f * ct;
        }
        write_out(fa, p, c, true);
    }
}

// ---- corrected mode ----
// Target function: |L f(wo, wi) cos| with the BSDF of the pixel's visible point
// (position, normal, material, wo towards the camera) -- the factor the
// reservoir's estimate is shaded with, so W absorbs it and a glossy lobe cannot
// turn the resampled estimate into fireflies.  Reference mode keeps the
// reference's |L| (ReSTIRGITemporalReuse.rgen.hlsl:33-40), exact for its
// Lambertian-only scenes up to the cosine.
// Near-specular visible points (GGX conductor or plastic coat with roughness
// below this) take no temporal or spatial reuse: a reconnection sample from
// another pixel lands in their sharp lobe with a target far above the one it
// was resampled for, and the 1/M-weighted merge turns that into fireflies; their
// reservoir is the initial candidate alone, i.e. the path-traced estimate.
constexpr float kReuseMinRoughness = 0.25f;

struct PixelShading {
    XrMaterial m;
    float3 x, n, wo, T, B;
    bool reuse;
};
__device__ __forceinline__ PixelShading pixel_shading(const FrameArgs& fa, const XrUniformBufferObject* __restrict__ u,
                                                      float3 x, float3 n, uint32_t mat, uint32_t p) {
    PixelShading P;
    P.m = resolve_material(fa.sc, mat, fa.sc.n_tex ? fa.gb_uv[p] : make_float2(0.0f, 0.0f));
    P.x = x;
    P.n = n;
    // the camera position: the translation column of view_inverse (column-major)
    const float3 cam = f3(u->view_inverse[12], u->view_inverse[13], u->view_inverse[14]);
    P.wo = normalize(cam - x);
    branchless_onb(n, &P.T, &P.B);
    const bool glossy = (P.m.material_model == XR_MAT_METALLIC || P.m.material_model == XR_MAT_PLASTIC) &&
                        P.m.fuzziness < kReuseMinRoughness;
    P.reuse = !glossy;
    return P;
}
__device__ __forceinline__ float target_corrected(const PixelShading& P, float3 xs, float3 L) {
    const float3 wi = normalize(xs - P.x);
    const float c = dot(P.n, wi);
    if (c <= 0.0f) return 0.0f;
    const float3 f = eval_material(P.m, to_local(P.wo, P.T, P.B, P.n), to_local(wi, P.T, P.B, P.n)).f;
    return length(L * f * c);
}

// The final target of a reservoir's sample and its shading, from one BSDF
// evaluation (target_corrected's lobe at the same direction).  `tp_known` >= 0 is
// the target when the caller already has it (the selected candidate's), else < 0.
// Shading: L W f cos along the reconnection direction.  A near-specular pixel (no
// reuse: its reservoir is its own candidate) is shaded with the path tracer's
// ratio f cos / pdf at that one direction instead: the reconnection direction from
// the visible point differs slightly from the sampled one (the path left from a
// point offset along the normal), and in a lobe that sharp f alone changes by
// orders of magnitude over that angle while the ratio stays bounded.
__device__ __forceinline__ float3 finish_corrected(const PixelShading& P, Res& r, float tp_known, uint32_t m_cap,
                                                   bool shade) {
    const float3 wi = normalize(r.xs - P.x);
    const float c = dot(P.n, wi);
    Lobe lb;
    lb.f = f3(0, 0, 0);
    lb.pdf = 0.0f;
    const bool front = c > 0.0f;
    if (front && (tp_known < 0.0f || shade))
        lb = eval_material(P.m, to_local(P.wo, P.T, P.B, P.n), to_local(wi, P.T, P.B, P.n));
    const float tpf = tp_known >= 0.0f ? tp_known : (front ? length(r.L * lb.f * c) : 0.0f);
    if (r.m > m_cap) {
        r.w_sum *= (float)m_cap / (float)r.m;
        r.m = m_cap;
    }
    r.W = (tpf > 1e-6f && r.m > 0u) ? r.w_sum / ((float)r.m * tpf) : 0.0f;
    float3 col = f3(0, 0, 0);
    if (shade && r.W > 0.0f) {
        const float ct = fmaxf(0.0f, c);
        if (P.reuse) col = r.L * r.W * lb.f * ct;
        else if (lb.pdf > 0.0f) col = r.L * lb.f * (ct / lb.pdf);
    }
    return col;
}

// Neighbours of the corrected spatial pass: the first 2 n draws of the pixel's
// spatial stream pick the n neighbours (two per pick, in order) and the merges
// draw after them.
__device__ __forceinline__ void rng_skip(uint32_t& st, uint32_t n) {
    for (uint32_t k = 0; k < n; k++) st = st * 747796405u + 2891336453u;   // the state step of next_random
}

// 64-thread blocks: finer scheduling of a latency-bound pass (swept 64 / 128 / 256 /
// 512: 69.7 / 71.2 / 73.7 / 77.3 us at 1080p, CUDA events).
#ifndef XR_TEMPORAL_BLOCK
#define XR_TEMPORAL_BLOCK 64
#endif
// launch bounds: blocks of up to 256 threads (the block size is a tuning parameter, default XR_TEMPORAL_BLOCK)
__global__ void __launch_bounds__(256) k_temporal(FrameArgs fa, const XrUniformBufferObject* __restrict__ u, bool out_here) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    const PixView pv = pix_view(fa, p);
    u += pv.v;
    const uint32_t x = pv.x, y = pv.y;
    float4 g = fa.gb_pos_cur[p];
    uint32_t mat = fa.gb_mat_cur[p];
    float4 a = fa.cand_a[p], b = fa.cand_b[p];
    const uint32_t q = (fa.temporal_on && mat != kInvalid) ? fa.reproj[p] : kInvalid;   // set by bounce 0's shading
    const uint32_t bw = __float_as_uint(b.w);
    const bool valid = mat != kInvalid, has = (bw >> 31) != 0u;
    if (fa.write_pt) {
        float3 v = valid ? xyz(fa.thr0[p]) * (has ? xyz(b) : f3(0, 0, 0)) : xyz(b);
        fa.out_pt[p] = f4(v, 1.0f);
    }
    if (!valid || !has) {
        Res e; res_init(e);
        store_packed(fa.rt_cur0, fa.rt_cur1, p, e);
        if (out_here) write_out(fa, p, valid ? f3(0, 0, 0) : xyz(b), true);
        return;
    }
    uint32_t rng = pass_rng(false, x, y, pv.W, u->current_frame, kPassTemporal, fa.seed);
    const float3 x_view = xyz(g);
    const float3 n_view = oct_decode(__float_as_uint(g.w), 16);
    Res s_new;
    s_new.xs = xyz(a); s_new.L = xyz(b); s_new.code = bw & 0x00FFFFFFu; s_new.ns = f3(0, 0, 0);   // travels as its code
    s_new.f = f3(0, 0, 0);
    // Every previous-frame word of the reprojected pixel gathered at once (material,
    // position, reservoir): one memory round trip after the coalesced loads; the
    // tests below decide what is used.
    bool in_prev = false;
    uint32_t pmat = kInvalid;
    float4 pg = make_float4(0, 0, 0, 0), rp0 = pg, rp1 = pg;
    if (q != kInvalid) {
        pmat = fa.gb_mat_prev[q];
        pg = fa.gb_pos_prev[q];
        rp0 = fa.rt_prev0[q];
        rp1 = fa.rt_prev1[q];
        in_prev = true;
    }
    const PixelShading P = pixel_shading(fa, u, x_view, n_view, mat, p);
    bool found = false;
    Res r_prev; res_init(r_prev);
    if (in_prev && P.reuse && pmat == mat) {
        float3 pn = oct_decode(__float_as_uint(pg.w), 16);
        float3 dd = x_view - xyz(pg);
        if (!(dot(n_view, pn) < 0.8f) && !(dot(dd, dd) > 0.1f)) {
            decode_packed(rp0, rp1, r_prev, false);
            found = true;
        }
    }
    Res r; res_init(r);
    const float tp_new = target_corrected(P, s_new.xs, s_new.L);
    float w_new = (a.w > 1e-6f) ? (tp_new / a.w) : 0.0f;
    // the target of the sample the reservoir ends with, when it is one already evaluated
    float tp_sel = res_update(r, s_new, w_new, rng) ? tp_new : -1.0f;
    if (found) {
        const float tp_prev = target_corrected(P, r_prev.xs, r_prev.L);
        if (res_merge(r, r_prev, tp_prev, rng)) tp_sel = tp_prev;
    } else {
        r.m = 1u;
    }
    const float3 col = finish_corrected(P, r, tp_sel, fa.m_cap_t, out_here);
    store_packed(fa.rt_cur0, fa.rt_cur1, p, r);
    if (out_here) write_out(fa, p, col, true);
}

// Spatial reuse, step 1 of 3 (corrected mode): picks each pixel's neighbours,
// tests their similarity, evaluates the target of each similar neighbour's
// sample at the pixel times the Jacobian of the reconnection (p-hat) and stores
// {neighbour, p-hat} per slot for the resolve step; with shadow rays on, queues
// one ray {pixel << 5 | slot, neighbour} per neighbour with p-hat > 0.  Every
// pixel clears its occlusion bits.
// Like shading, spatial select and resolve wait on neighbour gathers: 4 CTAs of 256
// per SM for select (64 registers, 16 bytes spilled) and 5 for resolve (48
// registers, 44 bytes spilled) beat the occupancy their register counts allow
// (spatial pass 0.76 -> 0.66 ms at 1080p, measured twice in one session).
#ifndef XR_SELECT_MIN_BLOCKS
#define XR_SELECT_MIN_BLOCKS 4
#endif
// Spatial select and resolve run in 128-thread blocks (twice the CTAs per SM of the
// 256-thread figures above, the same register budget): spatial 0.662 -> 0.648 ms.
#ifndef XR_SPATIAL_BLOCK
#define XR_SPATIAL_BLOCK 128
#endif
// launch bounds: blocks of up to 256 threads (the block size is a tuning parameter, default XR_SPATIAL_BLOCK),
// XR_SELECT_MIN_BLOCKS x 256 threads resident per SM
__global__ void __launch_bounds__(256, XR_SELECT_MIN_BLOCKS) k_spatial_select(FrameArgs fa, const XrUniformBufferObject* __restrict__ u) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = lane_id();
    uint32_t emit_mask = 0u;
    uint32_t nb_of[32];
    if (p < fa.N) {
        fa.occ[p] = 0u;
        const PixView pv = pix_view(fa, p);
        const XrUniformBufferObject* __restrict__ uv = u + pv.v;
        const uint32_t x = pv.x, y = pv.y;
        const float4 g = fa.gb_pos_cur[p];
        const uint32_t mat = fa.gb_mat_cur[p];
        const float4 b = fa.cand_b[p];
        if (mat != kInvalid && (__float_as_uint(b.w) >> 31) != 0u) {
            uint32_t rng_pick = pass_rng(false, x, y, pv.W, uv->current_frame, kPassSpatial, fa.seed);
            const float3 x_view = xyz(g);
            const float3 n_view = oct_decode(__float_as_uint(g.w), 16);
            const PixelShading P = pixel_shading(fa, uv, x_view, n_view, mat, p);
            const uint32_t nn = P.reuse ? fa.n_nb : 0u;
            // the picks do not depend on the merges: the next neighbour's G-buffer
            // words are gathered while this one is tested and evaluated
            uint32_t nx_i = 0u, nx_mat = kInvalid;
            float4 nx_g = make_float4(0, 0, 0, 0);
            if (nn) {
                nx_i = pv.base + neighbor_index(x, y, pv.W, pv.H, fa.radius, rng_pick);
                nx_mat = fa.gb_mat_cur[nx_i];
                nx_g = fa.gb_pos_cur[nx_i];
            }
            for (uint32_t i = 0; i < nn; i++) {
                uint2 slot = make_uint2(kInvalid, 0u);
                const uint32_t nbi = nx_i, nmat = nx_mat;
                const float4 ng = nx_g;
                if (i + 1u < nn) {
                    nx_i = pv.base + neighbor_index(x, y, pv.W, pv.H, fa.radius, rng_pick);
                    nx_mat = fa.gb_mat_cur[nx_i];
                    nx_g = fa.gb_pos_cur[nx_i];
                }
                uint32_t nm = 0u;
                if (nmat != kInvalid && nmat == mat) {
                    const float3 dd = x_view - xyz(ng);
                    if (!(dot(dd, dd) > 0.1f) && !(dot(n_view, oct_decode(__float_as_uint(ng.w), 16)) < 0.8f)) {
                        Res rn;
                        load_packed(fa.rt_cur0, fa.rt_cur1, nbi, rn);
                        const float ph = target_corrected(P, rn.xs, rn.L) * jacobian_of(xyz(ng), x_view, rn.xs, rn.ns);
                        // the merge weight of MergeReservoir (ReSTIRGICommon.hlsl:68): resolve merges
                        // from the slots and gathers only the reservoir that wins
                        slot = make_uint2(nbi, __float_as_uint(ph * rn.W * (float)rn.m));
                        nm = rn.m;
                        if (fa.visibility && ph > 0.0f) { emit_mask |= 1u << i; nb_of[i] = nbi; }
                    }
                }
                fa.nb_slot[(size_t)i * fa.N + p] = slot;
                fa.nb_m[(size_t)i * fa.N + p] = (uint8_t)nm;
            }
        }
    }
    // one atomic per warp: exclusive scan of the per-lane ray counts
    const uint32_t cnt = __popc(emit_mask);
    uint32_t incl = cnt;
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if ((int)lane >= off) incl += v;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(&fa.counters[32], total);
    base = __shfl_sync(0xFFFFFFFFu, base, 31);
    uint32_t pos = base + incl - cnt;
    while (emit_mask) {
        const uint32_t i = __ffs(emit_mask) - 1u;
        emit_mask &= emit_mask - 1u;
        fa.shadow_q[pos++] = make_uint2((p << 5) | i, nb_of[i]);
    }
}

// Spatial reuse, step 2 of 3: any-hit traversal of the queued shadow rays
// (ReSTIRGISpatialReuse.rgen.hlsl:44-62 with the centre pixel's visible point as
// origin); an occluded ray sets its slot's bit in the pixel's occlusion word.
template <bool INST>
__global__ void __launch_bounds__(trace_block<INST>(), 1) k_trace_shadow(FrameArgs fa) {
    const uint32_t count = *(volatile const uint32_t*)&fa.counters[32];
    trace_persistent<true, INST>(
        fa.sc, count, &fa.counters[kCntFetchShadow],
        [&](uint32_t i) {
            const uint2 e = fa.shadow_q[i];
            const float4 g = fa.gb_pos_cur[e.x >> 5];
            const float3 from = xyz(g);
            const float3 n = oct_decode(__float_as_uint(g.w), 16);
            const float3 to = xyz(fa.rt_cur0[e.y]);
            const float3 dir = to - from;
            RayIn r;
            r.root = root_of_pixel(fa, e.x >> 5);
            r.o = from + n * 0.01f;
            r.d = normalize(dir);
            r.tmin = 0.0f;
            r.tmax = length(dir) - 0.01f;
            return r;
        },
        [&](uint32_t i, const HitRec& h) {
            if (h.prim >= 0) {
                const uint32_t owner = fa.shadow_q[i].x;
                atomicOr(&fa.occ[owner >> 5], 1u << (owner & 31u));
            }
        },
        &fa.counters[kCntError], nullptr, &fa.counters[kCntNonFinite]);
}

// Next-event rays of the cache's training paths (one bounce): any-hit
// traversal; an unoccluded ray adds its contribution to its record's target.
__global__ void __launch_bounds__(kTraceBlock, 1) k_trace_nee(FrameArgs fa) {
    const uint32_t count = *(volatile const uint32_t*)&fa.counters[kCntCacheNee];
    trace_persistent<true>(
        fa.sc, count < fa.cache_t_cap ? count : fa.cache_t_cap, &fa.counters[kCntFetchNee],
        [&](uint32_t i) {
            const float4 a = fa.cache_nee[(size_t)i * 3u], b = fa.cache_nee[(size_t)i * 3u + 1u];
            RayIn r;
            r.root = fa.multi_root ? root_of_pixel(fa, fa.cache_t[(size_t)__float_as_uint(a.w) * 3u].w) : 0u;
            r.o = xyz(a);
            r.d = xyz(b);
            r.tmin = 0.0f;
            r.tmax = b.w;
            return r;
        },
        [&](uint32_t i, const HitRec& h) {
            if (h.prim < 0) {
                const uint32_t rec = __float_as_uint(fa.cache_nee[(size_t)i * 3u].w);
                const float4 c = fa.cache_nee[(size_t)i * 3u + 2u];
                float4* tgt = reinterpret_cast<float4*>(fa.cache_t + (size_t)rec * 3u + 2u);
                const float4 v = *tgt;
                *tgt = make_float4(v.x + c.x, v.y + c.y, v.z + c.z, v.w);
            }
        },
        &fa.counters[kCntError], nullptr, &fa.counters[kCntNonFinite]);
}

// Spatial reuse, step 3 of 3: the merge of ReSTIRGISpatialReuse.rgen.hlsl:91-176
// over the similar neighbours and p-hat values of step 1, with the visibility of
// step 2, M cap, W, shading and tone mapping.
#ifndef XR_RESOLVE_MIN_BLOCKS
#define XR_RESOLVE_MIN_BLOCKS 5
#endif
__global__ void __launch_bounds__(256, XR_RESOLVE_MIN_BLOCKS) k_spatial_resolve(FrameArgs fa, const XrUniformBufferObject* __restrict__ u) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    const PixView pv = pix_view(fa, p);
    u += pv.v;
    const uint32_t x = pv.x, y = pv.y;
    float4 g = fa.gb_pos_cur[p];
    uint32_t mat = fa.gb_mat_cur[p];
    float4 b = fa.cand_b[p];
    const bool valid = mat != kInvalid, has = (__float_as_uint(b.w) >> 31) != 0u;
    if (!valid || !has) {
        Res e; res_init(e);
        store_packed(fa.rs0, fa.rs1, p, e);
        write_out(fa, p, valid ? f3(0, 0, 0) : xyz(b), true);
        return;
    }
    uint32_t rng = pass_rng(false, x, y, pv.W, u->current_frame, kPassSpatial, fa.seed);
    const float3 x_view = xyz(g);
    const float3 n_view = oct_decode(__float_as_uint(g.w), 16);
    const uint32_t occ = fa.visibility ? fa.occ[p] : 0u;
    const PixelShading P = pixel_shading(fa, u, x_view, n_view, mat, p);
    Res center; load_packed(fa.rt_cur0, fa.rt_cur1, p, center, false);
    const uint32_t nn = P.reuse ? fa.n_nb : 0u;   // the neighbours k_spatial_select picked and tested
    rng_skip(rng, 2u * nn);                         // the merges draw after the picks
    Res r; res_init(r);
    const float tp_center = target_corrected(P, center.xs, center.L);
    float tp_sel = res_merge(r, center, tp_center, rng) ? tp_center : -1.0f;
    // MergeReservoir of every similar neighbour with its weight from step 1 (0 when its
    // shadow ray was occluded); only the winning neighbour's reservoir is gathered, after the loop
    uint32_t win = kInvalid;
    for (uint32_t i = 0; i < nn; i++) {
        const uint2 slot = fa.nb_slot[(size_t)i * fa.N + p];
        if (slot.x == kInvalid) continue;   // not similar: no merge, no draw
        const uint32_t mi = fa.nb_m[(size_t)i * fa.N + p];
        const bool occluded = (occ >> i) & 1u;   // set only for the rays step 1 emitted (weight > 0)
        const float w_new = occluded ? 0.0f : __uint_as_float(slot.y);
        const uint32_t M0 = r.m;
        r.w_sum += w_new;
        r.m++;
        if (random_float(rng) < w_new / fmaxf(1e-10f, r.w_sum)) {
            win = slot.x;
            tp_sel = -1.0f;   // a neighbour's sample: its target is re-evaluated
        }
        r.m = M0 + mi;
        // every similar neighbour counts towards M (1/M normalisation) except one
        // whose sample is occluded; the reference also drops zero-weight neighbours
        // (ReSTIRGISpatialReuse.rgen.hlsl:140-143), which biases the estimate upwards
        if (occluded) r.m -= mi;
    }
    if (win != kInvalid) {
        Res rn;
        load_packed(fa.rt_cur0, fa.rt_cur1, win, rn, false);
        r.xs = rn.xs; r.L = rn.L; r.ns = rn.ns; r.f = rn.f; r.code = rn.code;
    }
    const float3 col = finish_corrected(P, r, tp_sel, fa.m_cap_s, true);
    store_packed(fa.rs0, fa.rs1, p, r);
    write_out(fa, p, col, true);
}

// ---------------------------------------------------------------------------
// conversion to and from the reference layouts (ReSTIRGICommon.hlsl:6-30)
// ---------------------------------------------------------------------------
// FP64 accumulation of one sample of the plain path tracer: the initial-sample
// path's radiance, throughput0 * L_out for a surface seen directly, the emission
// (or sky) otherwise -- the pixel value the reservoir passes estimate.
__global__ void k_accumulate_sample(FrameArgs fa, double* __restrict__ acc) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    float3 v;
    if (fa.compat) {
        const bool valid = __float_as_uint(fa.s_xv[p].w) != kInvalid;
        v = valid ? xyz(fa.thr0[p]) * xyz(fa.s_L[p]) : xyz(fa.le0[p]);
    } else {
        const float4 b = fa.cand_b[p];
        const bool valid = fa.gb_mat_cur[p] != kInvalid, has = (__float_as_uint(b.w) >> 31) != 0u;
        v = valid ? xyz(fa.thr0[p]) * (has ? xyz(b) : f3(0, 0, 0)) : xyz(b);
    }
    acc[3u * p + 0u] += (double)v.x;
    acc[3u * p + 1u] += (double)v.y;
    acc[3u * p + 2u] += (double)v.z;
}

__global__ void k_export_samples(FrameArgs fa, uint32_t* __restrict__ out) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    uint32_t w[24];
    for (int i = 0; i < 24; i++) w[i] = 0u;
    auto put3 = [&](int at, float3 v) { w[at] = __float_as_uint(v.x); w[at + 1] = __float_as_uint(v.y); w[at + 2] = __float_as_uint(v.z); };
    if (fa.compat) {
        float4 xv = fa.s_xv[p], nv = fa.s_nv[p], xs = fa.s_xs[p], ns = fa.s_ns[p], L = fa.s_L[p];
        uint32_t mat = __float_as_uint(xv.w);
        put3(0, xyz(xv)); w[3] = mat;
        put3(4, xyz(nv)); w[7] = __float_as_uint(nv.w);
        put3(8, xyz(xs)); w[11] = __float_as_uint(xs.w);
        put3(12, xyz(ns));
        put3(16, xyz(L));
        if (mat != kInvalid && mat < fa.sc.n_mats) put3(20, mat_albedo_over_pi(fa, mat, p));
    } else {
        float4 g = fa.gb_pos_cur[p], a = fa.cand_a[p], b = fa.cand_b[p];
        uint32_t mat = fa.gb_mat_cur[p], bw = __float_as_uint(b.w);
        bool valid = mat != kInvalid, has = (bw >> 31) != 0u;
        w[3] = mat;
        if (valid) {
            uint32_t c16 = __float_as_uint(g.w);
            put3(0, xyz(g));
            put3(4, oct_decode(c16, 16));
            w[7] = c16;
            w[11] = __float_as_uint(a.w);
        }
        if (has) {
            put3(8, xyz(a));
            put3(12, oct_decode(bw & 0x00FFFFFFu, 12));
            w[15] = bw;
            put3(16, xyz(b));
        }
    }
    uint4* o = reinterpret_cast<uint4*>(out + 24u * p);
    for (int i = 0; i < 6; i++) o[i] = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
}

struct Planes4 { float4* p[4]; };

__global__ void k_export_res_wide(Planes4 pl, uint32_t n, uint32_t* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = pl.p[0][i], b = pl.p[1][i], c = pl.p[2][i], d = pl.p[3][i];
    uint32_t w[28];
    for (int k = 0; k < 28; k++) w[k] = 0u;
    w[0] = __float_as_uint(b.w); w[1] = __float_as_uint(a.w); w[2] = __float_as_uint(c.w);
    w[12] = __float_as_uint(a.x); w[13] = __float_as_uint(a.y); w[14] = __float_as_uint(a.z);
    w[16] = __float_as_uint(c.x); w[17] = __float_as_uint(c.y); w[18] = __float_as_uint(c.z);
    w[20] = __float_as_uint(b.x); w[21] = __float_as_uint(b.y); w[22] = __float_as_uint(b.z);
    w[24] = __float_as_uint(d.x); w[25] = __float_as_uint(d.y); w[26] = __float_as_uint(d.z);
    uint4* o = reinterpret_cast<uint4*>(out + 28u * i);
    for (int k = 0; k < 7; k++) o[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
}

__global__ void k_export_res_packed(const float4* __restrict__ p0, const float4* __restrict__ p1, uint32_t n,
                                    uint32_t* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Res r;
    load_packed(p0, p1, i, r);
    uint32_t w[28];
    for (int k = 0; k < 28; k++) w[k] = 0u;
    w[1] = __float_as_uint(r.W); w[2] = r.m;
    w[12] = __float_as_uint(r.xs.x); w[13] = __float_as_uint(r.xs.y); w[14] = __float_as_uint(r.xs.z);
    w[16] = __float_as_uint(r.ns.x); w[17] = __float_as_uint(r.ns.y); w[18] = __float_as_uint(r.ns.z);
    w[19] = r.code;
    w[20] = __float_as_uint(r.L.x); w[21] = __float_as_uint(r.L.y); w[22] = __float_as_uint(r.L.z);
    uint4* o = reinterpret_cast<uint4*>(out + 28u * i);
    for (int k = 0; k < 7; k++) o[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
}

// The reprojection of every valid pixel from the stored G-buffer (a temporal pass
// run on its own, after imported samples; frames get it from bounce 0's shading).
__global__ void k_reproject(FrameArgs fa, const XrUniformBufferObject* __restrict__ u) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    if (fa.gb_mat_cur[p] == kInvalid) return;
    const PixView pv = pix_view(fa, p);
    fa.reproj[p] = reproject(xyz(fa.gb_pos_cur[p]), u + pv.v, pv.W, pv.H, pv.base);
}

__global__ void k_import_samples(FrameArgs fa, const uint32_t* __restrict__ in) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fa.N) return;
    const uint32_t* w = in + 24u * p;
    auto get3 = [&](int at) { return f3(__uint_as_float(w[at]), __uint_as_float(w[at + 1]), __uint_as_float(w[at + 2])); };
    if (fa.compat) {
        fa.s_xv[p] = f4(get3(0), __uint_as_float(w[3]));
        fa.s_nv[p] = f4(get3(4), __uint_as_float(w[7]));
        fa.s_xs[p] = f4(get3(8), __uint_as_float(w[11]));
        fa.s_ns[p] = f4(get3(12), 0.0f);
        fa.s_L[p] = f4(get3(16), 0.0f);
    } else {
        uint32_t mat = w[3];
        bool valid = mat != kInvalid, has = (w[15] >> 31) != 0u;
        fa.gb_pos_cur[p] = valid ? f4(get3(0), __uint_as_float(w[7])) : make_float4(0, 0, 0, 0);
        fa.gb_mat_cur[p] = mat;
        fa.cand_a[p] = valid ? f4(has ? get3(8) : f3(0, 0, 0), __uint_as_float(w[11])) : make_float4(0, 0, 0, 0);
        fa.cand_b[p] = has ? f4(get3(16), __uint_as_float(w[15])) : make_float4(0, 0, 0, 0);
    }
}

__global__ void k_import_res_wide(Planes4 pl, uint32_t n, const uint32_t* __restrict__ in) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* w = in + 28u * i;
    auto g = [&](int k) { return __uint_as_float(w[k]); };
    pl.p[0][i] = make_float4(g(12), g(13), g(14), g(1));
    pl.p[1][i] = make_float4(g(20), g(21), g(22), g(0));
    pl.p[2][i] = make_float4(g(16), g(17), g(18), __uint_as_float(w[2]));
    pl.p[3][i] = make_float4(g(24), g(25), g(26), 0.0f);
}

__global__ void k_import_res_packed(float4* __restrict__ p0, float4* __restrict__ p1, uint32_t n, const uint32_t* __restrict__ in) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* w = in + 28u * i;
    auto g = [&](int k) { return __uint_as_float(w[k]); };
    p0[i] = make_float4(g(12), g(13), g(14), g(1));
    p1[i] = make_float4(g(20), g(21), g(22), __uint_as_float((w[19] & 0x00FFFFFFu) | (min(w[2], 255u) << 24)));
}

}  // namespace

// Resident blocks per SM of the persistent kernels (queried once per process).
uint32_t persistent_grid(int sm_count, bool compat) {
    static int occ[2] = {0, 0};
    int& o = occ[compat ? 1 : 0];
    if (o == 0) {
        int v = 0;
        if (compat) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_shade<true>, kShadeBlock, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_shade<false>, kShadeBlock, 0);
        o = v > 0 ? v : 4;
    }
    return (uint32_t)(o * sm_count);
}

uint32_t trace_grid(int sm_count, bool instances) {
    static int occ[2] = {0, 0};
    int& o = occ[instances ? 1 : 0];
    if (o == 0) {
        int v = 0;
        if (instances) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_trace_paths<true, false>, kTraceBlockInst, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_trace_paths<false, false>, kTraceBlock, 0);
        o = v > 0 ? v : 4;
    }
    return (uint32_t)(o * sm_count);
}

void launch_initial(const FrameArgs& fa, uint32_t nb, cudaStream_t st, void (*after_bounce1)(void*), void* arg) {
    const uint32_t grid0 = fa.n_tiles;
    FrameArgs a = fa;
    if (fa.compat) k_raygen<true><<<grid0, kBlock, 0, st>>>(a, fa.ubo, nb);
    else k_raygen<false><<<grid0, kBlock, 0, st>>>(a, fa.ubo, nb);
    const bool cache = !fa.compat && fa.cache_on;
    for (uint32_t b = 0; b < nb; b++) {
        // queues alternate: bounce b reads what raygen / bounce b-1 appended
        for (int k = 0; k < 3; k++) std::swap(a.q_in[k], a.q_out[k]);
        const uint32_t rec = (cache && b >= 2u) ? 1u : 0u;
        const bool bound = XR_CAMERA_BOUND_MARGIN > 0.0f && !fa.compat && b == 0u && fa.sc.n_nodes >= kCameraBoundMinNodes;
        if (fa.sc.n_inst && bound)
            k_trace_paths<true, true><<<fa.grid_trace, kTraceBlockInst, 0, st>>>(a, a.q_in[0], a.q_in[1], fa.hits, fa.counters + b,
                                                                    fa.counters + kCntFetchPath + b, fa.counters + kCntError,
                                                                    fa.counters + kCntNonFinite, rec);
        else if (fa.sc.n_inst)
            k_trace_paths<true, false><<<fa.grid_trace, kTraceBlockInst, 0, st>>>(a, a.q_in[0], a.q_in[1], fa.hits, fa.counters + b,
                                                                     fa.counters + kCntFetchPath + b, fa.counters + kCntError,
                                                                     fa.counters + kCntNonFinite, rec);
        else if (bound)
            k_trace_paths<false, true><<<fa.grid_trace, kTraceBlock, 0, st>>>(a, a.q_in[0], a.q_in[1], fa.hits, fa.counters + b,
                                                                     fa.counters + kCntFetchPath + b, fa.counters + kCntError,
                                                                     fa.counters + kCntNonFinite, rec);
        else
            k_trace_paths<false, false><<<fa.grid_trace, kTraceBlock, 0, st>>>(a, a.q_in[0], a.q_in[1], fa.hits, fa.counters + b,
                                                                      fa.counters + kCntFetchPath + b, fa.counters + kCntError,
                                                                      fa.counters + kCntNonFinite, rec);
        const bool nee = cache && b >= 1u && b + 1u < nb;
        if (nee) cudaMemsetAsync(fa.counters + kCntCacheNee, 0, 2 * sizeof(uint32_t), st);   // count + fetch
        if (fa.compat) k_shade<true><<<fa.grid_persistent, kShadeBlock, 0, st>>>(a, fa.ubo, b, nb);
        else k_shade<false><<<fa.grid_persistent, kShadeBlock, 0, st>>>(a, fa.ubo, b, nb);
        if (b == 1u && after_bounce1) after_bounce1(arg);   // bounce 1's records are complete
        if (nee) k_trace_nee<<<fa.grid_trace, kTraceBlock, 0, st>>>(a);
    }
    if (nb < 2u && after_bounce1) after_bounce1(arg);
}

void launch_temporal(const FrameArgs& fa, bool write_image, cudaStream_t st) {
    uint32_t blocks = (fa.N + 255u) / 256u;
    if (fa.compat) k_temporal_compat<<<blocks, 256, 0, st>>>(fa, fa.ubo, write_image);
    else {
        const uint32_t tb = fa.blk_temporal ? fa.blk_temporal : (uint32_t)XR_TEMPORAL_BLOCK;
        k_temporal<<<(fa.N + tb - 1u) / tb, tb, 0, st>>>(fa, fa.ubo, write_image);
    }
}

void launch_export_samples(const FrameArgs& fa, uint32_t* out, cudaStream_t st) {
    k_export_samples<<<(fa.N + 255u) / 256u, 256, 0, st>>>(fa, out);
}
void launch_reproject(const FrameArgs& fa, cudaStream_t st) {
    k_reproject<<<(fa.N + 255u) / 256u, 256, 0, st>>>(fa, fa.ubo);
}
void launch_import_samples(const FrameArgs& fa, const uint32_t* in, cudaStream_t st) {
    k_import_samples<<<(fa.N + 255u) / 256u, 256, 0, st>>>(fa, in);
}
void launch_export_res_wide(float4* const planes[4], uint32_t n, uint32_t* out, cudaStream_t st) {
    Planes4 pl{{planes[0], planes[1], planes[2], planes[3]}};
    k_export_res_wide<<<(n + 255u) / 256u, 256, 0, st>>>(pl, n, out);
}
void launch_export_res_packed(const float4* p0, const float4* p1, uint32_t n, uint32_t* out, cudaStream_t st) {
    k_export_res_packed<<<(n + 255u) / 256u, 256, 0, st>>>(p0, p1, n, out);
}
void launch_import_res_wide(float4* const planes[4], uint32_t n, const uint32_t* in, cudaStream_t st) {
    Planes4 pl{{planes[0], planes[1], planes[2], planes[3]}};
    k_import_res_wide<<<(n + 255u) / 256u, 256, 0, st>>>(pl, n, in);
}
void launch_import_res_packed(float4* p0, float4* p1, uint32_t n, const uint32_t* in, cudaStream_t st) {
    k_import_res_packed<<<(n + 255u) / 256u, 256, 0, st>>>(p0, p1, n, in);
}

void launch_accumulate_sample(const FrameArgs& fa, double* acc, cudaStream_t st) {
    k_accumulate_sample<<<(fa.N + 255u) / 256u, 256, 0, st>>>(fa, acc);
}

void launch_spatial(const FrameArgs& fa, cudaStream_t st) {
    uint32_t blocks = (fa.N + 255u) / 256u;
    if (fa.compat) {
        k_spatial_compat<<<blocks, 256, 0, st>>>(fa, fa.ubo);
        return;
    }
    const uint32_t sb = fa.blk_spatial ? fa.blk_spatial : (uint32_t)XR_SPATIAL_BLOCK;
    const uint32_t sblocks = (fa.N + sb - 1u) / sb;
    k_spatial_select<<<sblocks, sb, 0, st>>>(fa, fa.ubo);
    if (fa.visibility) {
        if (fa.sc.n_inst) k_trace_shadow<true><<<fa.grid_trace, kTraceBlockInst, 0, st>>>(fa);
        else k_trace_shadow<false><<<fa.grid_trace, kTraceBlock, 0, st>>>(fa);
    }
    k_spatial_resolve<<<sblocks, sb, 0, st>>>(fa, fa.ubo);
}

}  // namespace xr
