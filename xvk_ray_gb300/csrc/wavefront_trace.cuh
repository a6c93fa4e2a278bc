// wavefront_trace.cuh -- persistent CWBVH traversal with dynamic ray fetching.
//
// Software replacement of the hardware TraceRay (opaque triangles, no culling,
// closest hit with ties to the lowest primitive id, or first hit for shadow
// rays).  Each warp keeps 32 rays in flight; once at least refill_min lanes have
// finished (or all have), the warp refills them from the ray queue with one
// atomic (Aila and Laine, "Understanding the Efficiency of Ray Traversal on
// GPUs", HPG 2009): the per-ray set-up (reciprocals, shear constants) then runs
// for many lanes at once instead of one or two.  The loop follows Ylitie,
// Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through
// Compressed Wide BVHs" (HPG 2017): a lane holds one group of internal children
// still to visit (base index, hit bits in near-to-far order, internal-child
// mask) and one group of triangles; each iteration visits at most one node,
// then tests triangles while enough lanes of the warp have some, and postpones
// the rest onto the lane's stack otherwise.
//
// The triangle test and the box test are those of traverse.cuh (same arithmetic
// as the CPU oracle); only the order of the work differs, which the closest-hit
// rule makes irrelevant for the result.
#pragma once
#include "traverse.cuh"

namespace xr {

constexpr uint32_t kTriGroupBit = 0x80000000u;   // stack entry holds a triangle group
constexpr uint32_t kLevelBit = 0x40000000u;      // stack entry marks the return to the top-level BVH
#ifndef XR_POSTPONE_BELOW
#define XR_POSTPONE_BELOW 8
#endif
#ifndef XR_REFILL_MIN
#define XR_REFILL_MIN 8
#endif
constexpr int kPostponeBelow = XR_POSTPONE_BELOW;  // default: lanes; fewer testing triangles -> postpone
constexpr int kRefillMin = XR_REFILL_MIN;          // default: idle lanes before a refill (swept 1..16: 1 is 9% slower)
constexpr float kMinDir = 1e-20f;                 // smallest direction component seen by the box test

struct RayIn {
    float3 o, d;
    float tmin, tmax;
    uint32_t root;   // first node of the ray's scene (0 unless several scenes share the node array)
};

// Byte k of `word` placed in mantissa bits 8..15 of 1.0f by one byte permute:
// the result is exactly 1 + q / 32768.  A plane at q cells is then
// t = q s + a = fma(1 + q / 32768, 32768 s, a - 32768 s), one instruction per
// plane after the per-node constants; the extra rounding of a - 32768 s is
// below 2^-9 of a cell, inside the 1/32-cell slack of the stored boxes.
__device__ __forceinline__ float qplane(uint32_t word, uint32_t k) {
    return __uint_as_float(__byte_perm(word, 0x3F800000u, 0x7604u | (k << 4)));
}

// Three-input minimum / maximum (PTX min.f32 / max.f32 with three sources,
// sm_100 and later); like the two-input forms they return a non-NaN operand
// when there is one, so a NaN plane drops out of the slab test.
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// LoadRay(i) -> RayIn; StoreHit(i, const HitRec&).  `next` is the fetch counter
// (zeroed before the launch), `count` the number of rays, `err` the error word.
// With `work` non-null (query kernels only) the node visits and triangle tests
// are summed into work[0] and work[1]; with `nonfinite` non-null, the rays ended
// early for a non-finite origin or direction are counted there.
//
// INST: two-level traversal of a scene with instances.  Rays start at the root of
// the top-level BVH (sc.tlas_nodes), whose leaf slots are instances; "testing" one
// saves the rest of the lane's top-level work on its stack under a level marker,
// maps the ray into the instance's object space (origin and direction by its
// world-to-object rows; t is unchanged) and continues at the root of its
// bottom-level BVH in sc.nodes.  Popping the marker restores the world-space ray
// (kept in the lane's registers or local memory since the ray's start).  Hits compare t, then instance, then primitive.
//
// RETRY (closest hit): a ray whose tmax is below retry_tmax treats its tmax
// as a guess at where it hits.  Boxes beyond it are culled from the start; a ray that
// ends without a hit inside it is traced again up to retry_tmax.  The result is the
// same either way: when a hit lies within tmax, the closest hit (and every hit tied
// with it) does too.
template <bool ANY, bool INST = false, bool RETRY = false, typename LoadRay, typename StoreHit>
__device__ __forceinline__ void trace_persistent(const DeviceScene& sc, uint32_t count, uint32_t* next,
                                                 LoadRay load, StoreHit store, uint32_t* err,
                                                 unsigned long long* work = nullptr, uint32_t* nonfinite = nullptr,
                                                 float retry_tmax = 0.0f) {
    static_assert(!RETRY || !ANY, "the retry is for closest-hit traversal");
    const uint32_t FULL = 0xFFFFFFFFu;
    uint32_t n_visits = 0, n_tests = 0, n_nonfinite = 0;
    // queue tuning of the context (0: the defaults kRefillMin / kPostponeBelow)
    const int refill_min = sc.refill_min ? (int)sc.refill_min : kRefillMin;
    const int postpone_below = sc.postpone_below ? (int)sc.postpone_below : kPostponeBelow;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    bool active = false, drained = false;
    bool retry = false;   // RETRY: the lane's ray is traced again up to retry_tmax on a miss
    uint32_t ray_id = 0;
    float3 o = f3(0, 0, 0);
    float idx = 0, idy = 0, idz = 0, tmin = 0, tmin_box = 0;
    RayTri rt;
    uint32_t flip = 0;
    HitRec h;
    h.prim = -1; h.t = 0; h.b1 = 0; h.b2 = 0;
    uint2 stack[kStackSize];
    int sp = 0;
    uint32_t ng_base = 0, ng_bits = 0;   // bits 0..7 hits (near-to-far), 8..15 internal-child mask
    uint32_t tg_base = 0, tg_mask = 0;
    uint32_t visits_left = 0;
    bool bad = false;
    bool in_blas = !INST;    // INST: the lane's ray is in an instance's object space
    int32_t cur_inst = -1;   // that instance
    h.inst = -1;
    // INST: the world-space ray and its box-test state, kept for instance entries
    // and for the return to the top level (no reload, no reciprocals recomputed)
    float3 wo = f3(0, 0, 0), wd = f3(0, 0, 0);
    float widx = 0, widy = 0, widz = 0;
    uint32_t wflip = 0;
    // box-test reciprocals and sign bits of a direction (see the comment at the ray start)
    auto set_dir = [&](float3 d) {
        idx = 1.0f / copysignf(fmaxf(fabsf(d.x), kMinDir), d.x);
        idy = 1.0f / copysignf(fmaxf(fabsf(d.y), kMinDir), d.y);
        idz = 1.0f / copysignf(fmaxf(fabsf(d.z), kMinDir), d.z);
        flip = (__float_as_uint(d.x) >> 31) | ((__float_as_uint(d.y) >> 31) << 1) | ((__float_as_uint(d.z) >> 31) << 2);
    };

    while (true) {
        // ---- refill idle lanes ----
        const uint32_t idle = __ballot_sync(FULL, !active);
        if (idle && !drained && (__popc(idle) >= refill_min || idle == FULL)) {
            const uint32_t n_idle = __popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(next, n_idle);
            base = __shfl_sync(FULL, base, 0);
            if (base + n_idle >= count) drained = true;
            if (!active) {
                const uint32_t my = base + __popc(idle & lt_mask);
                if (my < count) {
                    RayIn r = load(my);
                    ray_id = my;
                    active = true;
                    o = r.o;
                    tmin = r.tmin;
                    tmin_box = r.tmin * (1.0f - 1e-6f) - 1e-30f;
                    // Box-test reciprocals of the direction with each component kept at
                    // least kMinDir in magnitude (sign kept): an exactly zero component
                    // would give an infinite reciprocal, and inf - inf in the per-node
                    // plane constants below is NaN, which drops that axis from every slab
                    // test and walks the whole tree.  The box test then follows a ray that
                    // departs from the true one by at most kMinDir * t, far inside the
                    // slack of the stored boxes, so no box holding a hit is culled;
                    // the triangle test uses the true direction.
                    // The sign bits select the near planes (so that -0 picks the same
                    // planes as its infinite reciprocal).
                    set_dir(r.d);
                    rt = prep_ray(r.o, r.d);
                    if (INST) { wo = r.o; wd = r.d; widx = idx; widy = idy; widz = idz; wflip = flip; }
                    if constexpr (RETRY) retry = r.tmax < retry_tmax;
                    h.prim = -1; h.t = r.tmax; h.b1 = 0.0f; h.b2 = 0.0f; h.inst = -1;
                    sp = 0;
                    tg_mask = 0;
                    if (INST) {
                        // every instance may be entered once: bound the visits accordingly
                        const unsigned long long lim = ((unsigned long long)sc.n_nodes + sc.n_tlas_nodes) *
                                                       (unsigned long long)max(sc.n_inst, 1u);
                        visits_left = lim > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)lim;
                        in_blas = false;
                        cur_inst = -1;
                        ng_base = 0u;   // the top-level root
                        ng_bits = sc.n_tlas_nodes ? (1u | ((1u << flip) << 8)) : 0u;
                    } else {
                        visits_left = sc.n_nodes;
                        // a virtual group whose only child is the root (node 0)
                        ng_base = r.root;
                        ng_bits = (r.root < sc.n_nodes) ? (1u | ((1u << flip) << 8)) : 0u;   // no root: a miss
                    }
                    // A non-finite origin or direction (or a zero direction) can hit
                    // nothing -- every triangle test fails -- but would make every box
                    // test pass through NaN slabs and walk the whole tree: end it as a miss.
                    const float chk = r.o.x + r.o.y + r.o.z + r.d.x + r.d.y + r.d.z;
                    if (!isfinite(chk) || (r.d.x == 0.0f && r.d.y == 0.0f && r.d.z == 0.0f)) {
                        ng_bits = 0u;
                        n_nonfinite++;
                        if constexpr (RETRY) retry = false;
                    }
                }
            }
        }
        if (!__any_sync(FULL, active)) break;

        // ---- node phase: visit the nearest remaining child of the current group ----
        if (active && tg_mask == 0u && (ng_bits & 0xFFu)) {
            const uint32_t k = __ffs(ng_bits & 0xFFu) - 1u;
            ng_bits &= ~(1u << k);
            const uint32_t slot = k ^ flip;
            const uint32_t node = ng_base + __popc((ng_bits >> 8) & ((1u << slot) - 1u));
            if (ng_bits & 0xFFu) {
                if (sp < kStackSize) stack[sp++] = make_uint2(ng_base, ng_bits);
                else bad = true;
            }
            const WideNode* level_nodes = (INST && !in_blas) ? sc.tlas_nodes : sc.nodes;
            const uint32_t level_count = (INST && !in_blas) ? sc.n_tlas_nodes : sc.n_nodes;
            if (node >= level_count || visits_left == 0u) {
                bad = true;
                ng_bits = 0;
            } else {
                visits_left--;
                n_visits++;
                const uint4* np = reinterpret_cast<const uint4*>(level_nodes + node);
                const uint4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
                            w4 = __ldg(np + 4);
                // per axis: S = 32768 * 2^e / d and A = (p - o) / d - S (see qplane)
                const float sx = __uint_as_float((w0.w & 0xFFu) << 23) * idx * 32768.0f;
                const float sy = __uint_as_float(((w0.w >> 8) & 0xFFu) << 23) * idy * 32768.0f;
                const float sz = __uint_as_float(((w0.w >> 16) & 0xFFu) << 23) * idz * 32768.0f;
                const float ax = (__uint_as_float(w0.x) - o.x) * idx - sx;
                const float ay = (__uint_as_float(w0.y) - o.y) * idy - sy;
                const float az = (__uint_as_float(w0.z) - o.z) * idz - sz;
                const float tlimit = h.t * (1.0f + 1e-6f) + 1e-30f;
                // near and far quantised planes per axis, chosen once per node from the
                // sign bits of the direction (a negative axis enters through the high plane)
                const bool nx = (flip & 1u) != 0u, ny = (flip & 2u) != 0u, nz = (flip & 4u) != 0u;
                const uint32_t xn0 = nx ? w3.z : w2.x, xn1 = nx ? w3.w : w2.y;
                const uint32_t xf0 = nx ? w2.x : w3.z, xf1 = nx ? w2.y : w3.w;
                const uint32_t yn0 = ny ? w4.x : w2.z, yn1 = ny ? w4.y : w2.w;
                const uint32_t yf0 = ny ? w2.z : w4.x, yf1 = ny ? w2.w : w4.y;
                const uint32_t zn0 = nz ? w4.z : w3.x, zn1 = nz ? w4.w : w3.y;
                const uint32_t zf0 = nz ? w3.x : w4.z, zf1 = nz ? w3.y : w4.w;
                uint32_t hm = 0;   // bits 0..23 triangles, 24..31 internal children by slot
#pragma unroll
                for (uint32_t i = 0; i < 8; i++) {
                    const uint32_t meta = __byte_perm(i < 4 ? w1.z : w1.w, 0u, 0x4440u | (i & 3u));
                    const float txn = __fmaf_rn(qplane(i < 4 ? xn0 : xn1, i & 3u), sx, ax);
                    const float txf = __fmaf_rn(qplane(i < 4 ? xf0 : xf1, i & 3u), sx, ax);
                    const float tyn = __fmaf_rn(qplane(i < 4 ? yn0 : yn1, i & 3u), sy, ay);
                    const float tyf = __fmaf_rn(qplane(i < 4 ? yf0 : yf1, i & 3u), sy, ay);
                    const float tzn = __fmaf_rn(qplane(i < 4 ? zn0 : zn1, i & 3u), sz, az);
                    const float tzf = __fmaf_rn(qplane(i < 4 ? zf0 : zf1, i & 3u), sz, az);
                    const float tn = fmaxf(max3f(txn, tyn, tzn), tmin_box);
                    const float tf = fminf(min3f(txf, tyf, tzf), tlimit);
                    if (tn <= __fmaf_rn(tf, 1.0f + 2e-6f, 1e-30f)) hm |= __funnelshift_l(0u, meta >> 5, meta);
                }
                // internal hits from slot order to near-to-far order (bit k = slot k ^ flip)
                uint32_t ih = hm >> 24;
                if (flip & 1u) ih = ((ih & 0x55u) << 1) | ((ih >> 1) & 0x55u);
                if (flip & 2u) ih = ((ih & 0x33u) << 2) | ((ih >> 2) & 0x33u);
                if (flip & 4u) ih = ((ih & 0x0Fu) << 4) | ((ih >> 4) & 0x0Fu);
                ng_base = w1.x;
                ng_bits = ih | ((w0.w >> 24) << 8);
                tg_base = w1.y;
                tg_mask = hm & 0x00FFFFFFu;
            }
        }

        // ---- triangle phase: test while enough lanes have triangles ----
        bool first = true;
        while (true) {
            const bool want = active && tg_mask != 0u;
            const uint32_t m = __ballot_sync(FULL, want);
            if (!m) break;
            if (!first && (int)__popc(m) < postpone_below) {
                if (want && sp < kStackSize) {
                    stack[sp++] = make_uint2(tg_base, tg_mask | kTriGroupBit);
                    tg_mask = 0u;
                }
                break;
            }
            first = false;
            if (want && INST && !in_blas) {
                // an instance: enter its bottom-level BVH in object space
                const uint32_t bit = __ffs(tg_mask) - 1u;
                tg_mask &= tg_mask - 1u;
                if (tg_base + bit >= sc.n_inst_slots || sp + 3 > kStackSize) {
                    bad = true;
                    tg_mask = 0u;
                    ng_bits = 0u;
                } else {
                    const float4* ip = sc.inst_slots + 4u * (tg_base + bit);
                    const float4 m0 = __ldg(ip), m1 = __ldg(ip + 1), m2 = __ldg(ip + 2), m3 = __ldg(ip + 3);
                    // the rest of the top-level work, then the level marker
                    if (ng_bits & 0xFFu) stack[sp++] = make_uint2(ng_base, ng_bits);
                    if (tg_mask) stack[sp++] = make_uint2(tg_base, tg_mask | kTriGroupBit);
                    stack[sp++] = make_uint2(0u, kLevelBit);
                    tg_mask = 0u;
                    o = xform_point(m0, m1, m2, wo);
                    const float3 od = xform_dir(m0, m1, m2, wd);
                    set_dir(od);
                    rt = prep_ray(o, od);
                    cur_inst = (int32_t)__float_as_uint(m3.x);
                    in_blas = true;
                    ng_base = __float_as_uint(m3.y);
                    const float chk = o.x + o.y + o.z + od.x + od.y + od.z;
                    const bool ok = ng_base < sc.n_nodes && isfinite(chk) && !(od.x == 0.0f && od.y == 0.0f && od.z == 0.0f);
                    ng_bits = ok ? (1u | ((1u << flip) << 8)) : 0u;
                }
            } else if (want) {
                const uint32_t bit = __ffs(tg_mask) - 1u;
                n_tests++;
                tg_mask &= tg_mask - 1u;
                if (tg_base + bit >= sc.n_tri_slots) {
                    bad = true;
                } else {
                    const float4* tp = sc.tri + 3u * (tg_base + bit);
                    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                    const int32_t prim = (int32_t)__float_as_uint(a.w);
                    float tt, b1, b2;
                    const bool tie_wins = INST ? (cur_inst < h.inst || (cur_inst == h.inst && prim < h.prim))
                                               : prim < h.prim;
                    if (hit_triangle(rt, xyz(a), xyz(b), xyz(c), tmin, h.t, &tt, &b1, &b2) &&
                        (h.prim < 0 || tt < h.t || (tt == h.t && tie_wins))) {
                        h.prim = prim; h.t = tt; h.b1 = b1; h.b2 = b2; h.inst = cur_inst;
                        if (ANY) { tg_mask = 0u; ng_bits = 0u; sp = 0; }
                    }
                }
            }
        }

        // ---- pop or finish ----
        if (active && tg_mask == 0u && !(ng_bits & 0xFFu)) {
            if (INST && sp > 0 && stack[sp - 1].y == kLevelBit) {
                // back to the top level: the world-space ray, then (same step) the
                // top-level work saved under the marker -- markers are never adjacent
                --sp;
                o = wo;
                idx = widx; idy = widy; idz = widz;
                flip = wflip;
                in_blas = false;
                cur_inst = -1;
            }
            bool again = false;
            if constexpr (RETRY) again = sp == 0 && retry && h.prim < 0;
            if (again) {
                // nothing within the first tmax: the same ray again from the root, up to
                // retry_tmax.  The lane holds the world-space ray here (an emptied stack
                // has popped every level marker), so its direction state is kept; the
                // triangle-test set-up of a one-level ray is kept too, and a two-level
                // ray sets it up again at each instance it enters.
                retry = false;
                h.t = retry_tmax;
                if (INST) {
                    const unsigned long long lim = ((unsigned long long)sc.n_nodes + sc.n_tlas_nodes) *
                                                   (unsigned long long)max(sc.n_inst, 1u);
                    visits_left = lim > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)lim;
                    in_blas = false;
                    cur_inst = -1;
                    ng_base = 0u;   // the top-level root
                    ng_bits = sc.n_tlas_nodes ? (1u | ((1u << flip) << 8)) : 0u;
                } else {
                    visits_left = sc.n_nodes;
                    const uint32_t root = load(ray_id).root;
                    ng_base = root;
                    ng_bits = (root < sc.n_nodes) ? (1u | ((1u << flip) << 8)) : 0u;
                }
            } else if (sp == 0) {
                store(ray_id, h);
                active = false;
            } else {
                const uint2 e = stack[--sp];
                if (e.y & kTriGroupBit) { tg_base = e.x; tg_mask = e.y & 0x00FFFFFFu; ng_bits = 0u; }
                else { ng_base = e.x; ng_bits = e.y; }
            }
        }
    }
    if (__any_sync(FULL, bad) && bad) atomicOr(err, (uint32_t)XR_DEVFLAG_STACK_OVERFLOW);
    if (n_nonfinite && nonfinite) atomicAdd(nonfinite, n_nonfinite);
    if (work) {
        atomicAdd(&work[0], (unsigned long long)n_visits);
        atomicAdd(&work[1], (unsigned long long)n_tests);
    }
}

}  // namespace xr
