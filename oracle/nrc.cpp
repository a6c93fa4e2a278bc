// nrc.cpp -- CPU oracle of the learned radiance cache (TEST INFRASTRUCTURE).
//
// Only the tests and the benchmark's checks use this file, as the checker of
// the CUDA cache kernels.  The reference renderer has no learned cache; what is
// restated here are the published methods the cache follows:
//   * multiresolution hash encoding: Mueller, Evans, Schied, Keller, "Instant
//     Neural Graphics Primitives with a Multiresolution Hash Encoding" (SIGGRAPH
//     2022), section 3: L levels of resolution N_min * b^l, trilinear
//     interpolation of F features stored at the 8 cell corners, corners indexed
//     densely where the level's grid fits the table and by the spatial hash
//     (x * 1 xor y * 2654435761 xor z * 805459861) mod T otherwise;
//   * the radiance cache: Mueller, Rousselle, Novak, Keller, "Real-time Neural
//     Radiance Caching for Path Tracing" (SIGGRAPH 2021): inputs position,
//     normal, direction, roughness, albedo; ReLU MLP without biases; relative
//     L2 loss (y - t)^2 / (sg(y)^2 + 0.01);
//   * Adam: Kingma and Ba, ICLR 2015, with bias correction.
//
// Two arithmetic modes.  "GPU mode" rounds exactly where the CUDA kernels round
// (network inputs, weights and hidden activations to bfloat16, output-layer
// gradients and hidden-layer gradients to bfloat16, the hash table to binary16)
// and accumulates dot products in double, so the only differences from the
// tensor-core kernels are the FP32 accumulation order inside the MMAs and the
// order of the atomic gradient sums.  "Exact mode" keeps everything in double
// without rounding and is the one the finite-difference checks use.
#include "xr_oracle.h"
#include "common.h"

#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <vector>

namespace {
using namespace xro;

constexpr int kLevels = 16;
constexpr uint32_t kLog2T = 19, kT = 1u << kLog2T;
constexpr int kIn = 64, kWidth = 64, kOut = 16, kHidden = 4;
constexpr int kMlpParams = kHidden * kWidth * kIn + kOut * kWidth;   // 17,408
constexpr size_t kGridParams = (size_t)kLevels * kT * 2;            // 16,777,216
// N_l = floor(16 * 2^(7 l / 15)): 16 ... 2048 (per-level growth b = 128^(1/15))
constexpr uint32_t kRes[kLevels] = {16, 22, 30, 42, 58, 80, 111, 153, 212, 294, 406, 561, 776, 1072, 1482, 2048};

inline uint32_t unorm8(float x) { return (uint32_t)(fminf(fmaxf(x, 0.0f), 1.0f) * 255.0f + 0.5f); }

// counter-based uniform in [0, 1) for parameter initialisation
inline float init_u01(uint32_t i, uint32_t seed, uint32_t salt) {
    uint32_t h = wang(i ^ wang(seed * 0x85EBCA6Bu + salt));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

struct Decoded {
    f3 pos, n, wo, albedo;
    float rough;
    uint32_t kind;
};

inline Decoded decode(const uint32_t* r) {
    Decoded d;
    d.pos = {f32_from(r[0]), f32_from(r[1]), f32_from(r[2])};
    d.n = oct_decode(r[4], 16);
    d.wo = oct_decode(r[5], 16);
    d.albedo = {(float)(r[6] & 255u) / 255.0f, (float)((r[6] >> 8) & 255u) / 255.0f,
                (float)((r[6] >> 16) & 255u) / 255.0f};
    d.kind = r[6] >> 24;
    d.rough = f32_from(r[7]);
    return d;
}

struct Corner {
    uint32_t idx[8];
    float w[8];
};

// Cell corners and trilinear weights of one level (same operations as the kernel).
inline void level_corners(int l, f3 p, Corner& c) {
    const uint32_t res = kRes[l];
    const float fr = (float)res;
    float s[3] = {p.x * fr, p.y * fr, p.z * fr};
    uint32_t i0[3];
    float f[3];
    for (int a = 0; a < 3; ++a) {
        int ii = (int)floorf(s[a]);
        if (ii > (int)res - 1) ii = (int)res - 1;
        if (ii < 0) ii = 0;
        i0[a] = (uint32_t)ii;
        f[a] = s[a] - (float)ii;
    }
    const bool dense = (uint64_t)(res + 1u) * (res + 1u) * (res + 1u) <= (uint64_t)kT;
    const uint32_t st = res + 1u;
    for (int k = 0; k < 8; ++k) {
        const uint32_t cx = i0[0] + (k & 1), cy = i0[1] + ((k >> 1) & 1), cz = i0[2] + ((k >> 2) & 1);
        const float wx = (k & 1) ? f[0] : 1.0f - f[0];
        const float wy = (k & 2) ? f[1] : 1.0f - f[1];
        const float wz = (k & 4) ? f[2] : 1.0f - f[2];
        c.w[k] = (wx * wy) * wz;
        c.idx[k] = dense ? cx + st * (cy + st * cz) : ((cx * 1u) ^ (cy * 2654435761u) ^ (cz * 805459861u)) & (kT - 1u);
    }
}

struct Nrc {
    float lo[3] = {0, 0, 0};
    float inv_ext = 1.0f;
    std::vector<float> mlp, grid, mlp_grad, grid_grad, mlp_m, mlp_v, grid_m, grid_v;

    explicit Nrc(uint32_t seed)
        : mlp(kMlpParams), grid(kGridParams), mlp_grad(kMlpParams, 0.0f), grid_grad(kGridParams, 0.0f),
          mlp_m(kMlpParams, 0.0f), mlp_v(kMlpParams, 0.0f), grid_m(kGridParams, 0.0f), grid_v(kGridParams, 0.0f) {
        for (size_t e = 0; e < kGridParams; ++e) grid[e] = (init_u01((uint32_t)e, seed, 1u) * 2.0f - 1.0f) * 1e-4f;
        for (int l = 0; l <= kHidden; ++l) {
            const int rows = l < kHidden ? kWidth : kOut;
            const float a = sqrtf(6.0f / (float)(kIn + rows));
            for (int o = 0; o < rows; ++o)
                for (int i = 0; i < kIn; ++i) {
                    const uint32_t idx = (uint32_t)(l * kWidth * kIn + o * kIn + i);
                    mlp[idx] = (l == kHidden && o >= 3) ? 0.0f : (init_u01(idx, seed, 2u) * 2.0f - 1.0f) * a;
                }
        }
    }

    f3 unit_pos(f3 x) const {
        f3 p = {(x.x - lo[0]) * inv_ext, (x.y - lo[1]) * inv_ext, (x.z - lo[2]) * inv_ext};
        p.x = fminf(fmaxf(p.x, 0.0f), 1.0f);
        p.y = fminf(fmaxf(p.y, 0.0f), 1.0f);
        p.z = fminf(fmaxf(p.z, 0.0f), 1.0f);
        return p;
    }
    float table(size_t e, bool exact) const { return exact ? grid[e] : half_value(half_bits(grid[e])); }
    double weight(int l, int o, int i, bool exact) const {
        const float w = mlp[(size_t)l * kWidth * kIn + (size_t)o * kIn + i];
        return exact ? (double)w : (double)bf16_round(w);
    }

    // network input vector (64 values) of one packed record
    void inputs(const uint32_t* rec, double* x, bool exact) const {
        const Decoded d = decode(rec);
        const f3 p = unit_pos(d.pos);
        float v[kIn];
        for (int l = 0; l < kLevels; ++l) {
            Corner c;
            level_corners(l, p, c);
            float a0 = 0.0f, a1 = 0.0f;
            double e0 = 0.0, e1 = 0.0;
            for (int k = 0; k < 8; ++k) {
                const size_t e = ((size_t)l * kT + c.idx[k]) * 2;
                a0 = a0 + c.w[k] * table(e, exact);
                a1 = a1 + c.w[k] * table(e + 1, exact);
                e0 += (double)c.w[k] * grid[e];
                e1 += (double)c.w[k] * grid[e + 1];
            }
            v[2 * l] = a0;
            v[2 * l + 1] = a1;
            if (exact) { x[2 * l] = e0; x[2 * l + 1] = e1; }
        }
        const float ndw = dot(d.n, d.wo);
        const f3 refl = d.n * (2.0f * ndw) - d.wo;
        const float tail[16] = {d.n.x, d.n.y, d.n.z, d.wo.x, d.wo.y, d.wo.z, refl.x, refl.y, refl.z,
                                d.albedo.x, d.albedo.y, d.albedo.z, d.rough,
                                d.kind == 1u ? 1.0f : 0.0f, d.kind == 5u ? 1.0f : 0.0f, 1.0f};
        for (int j = 0; j < 16; ++j) v[32 + j] = tail[j];
        for (int j = 48; j < kIn; ++j) v[j] = 0.0f;
        for (int j = exact ? 32 : 0; j < kIn; ++j) x[j] = exact ? (double)v[j] : (double)bf16_round(v[j]);
    }

    // forward pass: h[0..4] activations (64 each), out[16]
    void forward(const double* x, double h[kHidden + 1][kWidth], double* out, bool exact) const {
        for (int i = 0; i < kIn; ++i) h[0][i] = x[i];
        for (int l = 0; l < kHidden; ++l)
            for (int o = 0; o < kWidth; ++o) {
                double z = 0.0;
                for (int i = 0; i < kIn; ++i) z += h[l][i] * weight(l, o, i, exact);
                if (exact) h[l + 1][o] = z > 0.0 ? z : 0.0;
                else {
                    const float zf = (float)z;
                    h[l + 1][o] = (double)bf16_round(zf > 0.0f ? zf : 0.0f);
                }
            }
        for (int o = 0; o < kOut; ++o) {
            double z = 0.0;
            for (int i = 0; i < kWidth; ++i) z += h[kHidden][i] * weight(kHidden, o, i, exact);
            out[o] = exact ? z : (double)(float)z;
        }
    }
};

}  // namespace

extern "C" {

void* or_nrc_create(uint32_t seed) { return new Nrc(seed); }
void or_nrc_destroy(void* p) { delete (Nrc*)p; }

void or_nrc_set_bounds(void* p, const float* lo, float inv_extent) {
    Nrc& N = *(Nrc*)p;
    for (int a = 0; a < 3; ++a) N.lo[a] = lo[a];
    N.inv_ext = inv_extent;
}

float* or_nrc_params(void* p, int which, size_t* count) {
    Nrc& N = *(Nrc*)p;
    std::vector<float>* v[] = {&N.mlp, &N.grid, &N.mlp_grad, &N.grid_grad, &N.mlp_m, &N.mlp_v, &N.grid_m, &N.grid_v};
    if (which < 0 || which > 7) return nullptr;
    if (count) *count = v[which]->size();
    return v[which]->data();
}

// XrCacheSample -> 8-word record {pos.xyz, pixel, oct16(n), oct16(wo), rgb8 | kind << 24, roughness}
void or_nrc_pack(const OrCacheSample* s, uint32_t n, uint32_t* rec) {
    for (uint32_t i = 0; i < n; ++i) {
        const OrCacheSample& q = s[i];
        uint32_t* r = rec + (size_t)i * 8;
        r[0] = f32_bits(q.pos[0]); r[1] = f32_bits(q.pos[1]); r[2] = f32_bits(q.pos[2]);
        r[3] = q.pixel;
        r[4] = oct_encode(f3{q.normal[0], q.normal[1], q.normal[2]}, 16);
        r[5] = oct_encode(f3{q.wo[0], q.wo[1], q.wo[2]}, 16);
        r[6] = unorm8(q.albedo[0]) | (unorm8(q.albedo[1]) << 8) | (unorm8(q.albedo[2]) << 16) | ((q.kind & 255u) << 24);
        r[7] = f32_bits(q.roughness);
    }
}

void or_nrc_inputs(void* p, const uint32_t* rec, uint32_t n, float* x64, int exact) {
    const Nrc& N = *(const Nrc*)p;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        double x[kIn];
        N.inputs(rec + (size_t)i * 8, x, exact != 0);
        for (int j = 0; j < kIn; ++j) x64[(size_t)i * kIn + j] = (float)x[j];
    }
}

void or_nrc_infer(void* p, const uint32_t* rec, uint32_t n, float* out3, int exact) {
    const Nrc& N = *(const Nrc*)p;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        double x[kIn], h[kHidden + 1][kWidth], out[kOut];
        N.inputs(rec + (size_t)i * 8, x, exact != 0);
        N.forward(x, h, out, exact != 0);
        for (int c = 0; c < 3; ++c) out3[(size_t)i * 3 + c] = (float)out[c];
    }
}

// Gradients of the mean loss over the n samples (3 channels each) with respect
// to every MLP weight and hash-table value; overwrites the gradient buffers and
// returns the loss.  loss_kind 0: relative L2 (y - t)^2 / (sg(y)^2 + 0.01);
// 1: plain L2 (y - t)^2 (finite-difference checks, whose loss has no stop-gradient).
double or_nrc_backward(void* p, const uint32_t* rec, const float* target3, uint32_t n, int exact, int loss_kind) {
    Nrc& N = *(Nrc*)p;
    const bool ex = exact != 0;
    std::fill(N.mlp_grad.begin(), N.mlp_grad.end(), 0.0f);
    std::fill(N.grid_grad.begin(), N.grid_grad.end(), 0.0f);
    std::vector<double> gW((size_t)kMlpParams, 0.0);
    std::unordered_map<size_t, double> gG;   // touched hash-table values only
    double loss = 0.0;
    const float inv_count = 1.0f / (float)(3u * n);
    for (uint32_t s = 0; s < n; ++s) {
        double x[kIn], h[kHidden + 1][kWidth], out[kOut];
        N.inputs(rec + (size_t)s * 8, x, ex);
        N.forward(x, h, out, ex);
        double dz[kWidth] = {0};   // gradient w.r.t. the current layer's pre-activation output
        for (int c = 0; c < 3; ++c) {
            const float y = (float)out[c], t = target3[(size_t)s * 3 + c];
            if (ex) {
                const double yd = out[c], d = yd - (double)t;
                const double den = loss_kind == 0 ? yd * yd + 0.01 : 1.0;
                loss += d * d / den / (3.0 * n);
                dz[c] = 2.0 * d / den / (3.0 * n);
            } else {
                const float d = y - t;
                const float den = loss_kind == 0 ? y * y + 0.01f : 1.0f;
                loss += (double)(d * d / den) / (3.0 * n);
                dz[c] = (double)bf16_round(2.0f * d / den * inv_count);
            }
        }
        // layers kHidden .. 0: W_l maps h[l] (64) -> z (rows_l)
        for (int l = kHidden; l >= 0; --l) {
            const int rows = l < kHidden ? kWidth : kOut;
            double dh[kWidth] = {0};
            for (int o = 0; o < rows; ++o) {
                if (dz[o] == 0.0) continue;
                for (int i = 0; i < kIn; ++i) {
                    gW[(size_t)l * kWidth * kIn + (size_t)o * kIn + i] += dz[o] * h[l][i];
                    dh[i] += dz[o] * N.weight(l, o, i, ex);
                }
            }
            if (l > 0) {
                for (int i = 0; i < kWidth; ++i) {
                    const bool on = h[l][i] > 0.0;
                    if (ex) dz[i] = on ? dh[i] : 0.0;
                    else dz[i] = on ? (double)bf16_round((float)dh[i]) : 0.0;
                }
            } else {
                // hash-table gradients through the trilinear interpolation
                const Decoded d = decode(rec + (size_t)s * 8);
                const f3 pu = N.unit_pos(d.pos);
                for (int lv = 0; lv < kLevels; ++lv) {
                    Corner c;
                    level_corners(lv, pu, c);
                    const double g0 = ex ? dh[2 * lv] : (double)(float)dh[2 * lv];
                    const double g1 = ex ? dh[2 * lv + 1] : (double)(float)dh[2 * lv + 1];
                    for (int k = 0; k < 8; ++k) {
                        const size_t e = ((size_t)lv * kT + c.idx[k]) * 2;
                        gG[e] += (double)c.w[k] * g0;
                        gG[e + 1] += (double)c.w[k] * g1;
                    }
                }
            }
        }
    }
    for (size_t i = 0; i < gW.size(); ++i) N.mlp_grad[i] = (float)gW[i];
    for (const auto& kv : gG) N.grid_grad[kv.first] = (float)kv.second;
    return loss;
}

// Mean loss only (forward passes), same modes as or_nrc_backward.
double or_nrc_loss(void* p, const uint32_t* rec, const float* target3, uint32_t n, int exact, int loss_kind) {
    const Nrc& N = *(const Nrc*)p;
    const bool ex = exact != 0;
    double loss = 0.0;
    for (uint32_t s = 0; s < n; ++s) {
        double x[kIn], h[kHidden + 1][kWidth], out[kOut];
        N.inputs(rec + (size_t)s * 8, x, ex);
        N.forward(x, h, out, ex);
        for (int c = 0; c < 3; ++c) {
            const double d = out[c] - (double)target3[(size_t)s * 3 + c];
            const double den = loss_kind == 0 ? out[c] * out[c] + 0.01 : 1.0;
            loss += d * d / den / (3.0 * n);
        }
    }
    return loss;
}

// One Adam step on the current gradients; bc1 = 1 - b1^t and bc2 = 1 - b2^t.
// The MLP is updated densely; a hash-table value only where its gradient is
// non-zero (entries no sample touched keep their value and moments).
void or_nrc_adam(void* p, float lr, float b1, float b2, float eps, float bc1, float bc2) {
    Nrc& N = *(Nrc*)p;
    auto step = [&](float& w, float& m, float& v, float g) {
        m = b1 * m + (1.0f - b1) * g;
        v = b2 * v + (1.0f - b2) * (g * g);
        const float mh = m / bc1, vh = v / bc2;
        w = w - lr * mh / (sqrtf(vh) + eps);
    };
    for (size_t i = 0; i < N.mlp.size(); ++i) step(N.mlp[i], N.mlp_m[i], N.mlp_v[i], N.mlp_grad[i]);
    for (size_t i = 0; i < N.grid.size(); ++i)
        if (N.grid_grad[i] != 0.0f) step(N.grid[i], N.grid_m[i], N.grid_v[i], N.grid_grad[i]);
}

}  // extern "C"
