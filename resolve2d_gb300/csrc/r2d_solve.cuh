/*
 * r2d_solve.cuh -- per-constraint solve functions shared by the fused
 * per-world kernel and the large-world kernels.  Each function works on one
 * contact manifold or one joint through array views (SWT) that may point into
 * shared or global memory.
 */
#pragma once

#include <stdint.h>

#include "r2d_accum.h"
#include "r2d_device.cuh"
#include "r2d_world.cuh"

namespace r2d {

// Views of one world's arrays: shared memory in the fused kernel (16-bit
// manifold indices), global memory in the large-world path (32-bit).  PK:
// a body's momenta and inverse mass share one 16-byte word (mom4), so that
// the constraint loops fetch them with one load; else four arrays.
template <class IDX, bool PK = false>
struct SWT {
    float *px, *py, *ang, *mx, *my, *L, *inv_m, *inv_i, *cs, *sn, *ang_prev, *tq, *px0, *py0;
    float4* mom4;  // PK: (mx, my, L, inv_m) of each body
    bool pos0;                           // px0/py0 hold frame-start positions
    const float* __restrict__ gmass;     // this world's masses (global, read-only)
    const float* __restrict__ ginertia;  // this world's inertias
    uint8_t* kind;
    IDX *ma, *mb, *mp0;
    uint8_t *mnp, *mcol;
    float *nx, *ny, *fric;
    float *r1x, *r1y, *r2x, *r2y, *depth, *odepth, *mn, *mt, *apn, *apt, *bias;
    float *cpn, *cpt;  // compensation words of apn / apt (compensated mode, r2d_accum.h), else null

    __device__ __forceinline__ float& MX(uint32_t i) const {
        if constexpr (PK) return mom4[i].x;
        else return mx[i];
    }
    __device__ __forceinline__ float& MY(uint32_t i) const {
        if constexpr (PK) return mom4[i].y;
        else return my[i];
    }
    __device__ __forceinline__ float& AM(uint32_t i) const {  // angular momentum
        if constexpr (PK) return mom4[i].z;
        else return L[i];
    }
    __device__ __forceinline__ float& IM(uint32_t i) const {  // inverse mass
        if constexpr (PK) return mom4[i].w;
        else return inv_m[i];
    }
    // (mx, my, L, inv_m) of body i
    __device__ __forceinline__ float4 mom(uint32_t i) const {
        if constexpr (PK) return mom4[i];
        else return make_float4(mx[i], my[i], L[i], inv_m[i]);
    }
    // body i's momenta, with its inverse mass `im` (unchanged)
    __device__ __forceinline__ void put_mom(uint32_t i, float x, float y, float l, float im) const {
        if constexpr (PK) {
            mom4[i] = make_float4(x, y, l, im);
        } else {
            mx[i] = x;
            my[i] = y;
            L[i] = l;
        }
    }
    __device__ __forceinline__ float mass(uint32_t i) const { return __ldg(gmass + i); }
    __device__ __forceinline__ float inertia(uint32_t i) const { return __ldg(ginertia + i); }
    // Lever arms of point p between bodies a (reference) and b (incident).
    // Lean: middle - frame-start position, the subtraction CollisionPoint.init
    // performs (collision.zig:43-44), so the bits are those it stored.
    template <bool LEAN>
    __device__ __forceinline__ void arms(uint32_t p, uint32_t a, uint32_t b, f2* r1, f2* r2) const {
        if (LEAN) {
            const f2 mid = {r1x[p], r1y[p]};
            const float* bx = pos0 ? px0 : px;  // one substep: positions do not move before integration
            const float* by = pos0 ? py0 : py;
            *r1 = sub2(mid, f2{bx[a], by[a]});
            *r2 = sub2(mid, f2{bx[b], by[b]});
        } else {
            *r1 = f2{r1x[p], r1y[p]};
            *r2 = f2{r2x[p], r2y[p]};
        }
    }
};

// The accumulation of calculateImpulses (collision.zig:182-190): point p's
// normal impulse sum clamped at zero, its tangent sum to +-friction times
// the normal sum; the changes go to the bodies.  Compensated mode keeps each
// sum's rounding remainder in a second word (r2d_accum.h).
// The accumulator update of calculateImpulses (collision.zig:182-190) on a
// point's accumulated impulses an, at (and, compensated, their words cn, ct)
// held in registers; *applied_pn / *applied_pt get the changes.
__device__ __forceinline__ void acc_update(bool comp, float& an, float& at, float& cn, float& ct, float pn, float pt,
                                           float fr, float* applied_pn, float* applied_pt) {
    if (comp) {
        *applied_pn = r2d_acc_add_max(&an, &cn, pn, 0.0f);
        const float max_pt = fr * fabsf(an);
        *applied_pt = r2d_acc_add_clamp(&at, &ct, pt, -max_pt, max_pt);
        return;
    }
    const float nacc = zmax(0.0f, an + pn);
    *applied_pn = nacc - an;
    an = nacc;
    const float max_pt = fr * fabsf(nacc);
    const float nacct = zclamp(at + pt, -max_pt, max_pt);
    *applied_pt = nacct - at;
    at = nacct;
}

// acc_update on point p's accumulators in the world's arrays; every load
// comes before the first store.
template <class S>
__device__ __forceinline__ void accumulate(const S& s, uint32_t p, float pn, float pt, float fr,
                                           float* applied_pn, float* applied_pt) {
    const bool comp = s.cpn != nullptr;
    float an = s.apn[p], at = s.apt[p], cn = 0.f, ct = 0.f;
    if (comp) {
        cn = s.cpn[p];
        ct = s.cpt[p];
    }
    acc_update(comp, an, at, cn, ct, pn, pt, fr, applied_pn, applied_pt);
    s.apn[p] = an;
    s.apt[p] = at;
    if (comp) {
        s.cpn[p] = cn;
        s.cpt[p] = ct;
    }
}

// CollisionManifold.calculateImpulses (collision.zig:135-218).  `warm`:
// warm-starting mode, where an increment below MIN_MANIFOLD_IMPULSE is not
// skipped (the reference's skip keeps an accumulated impulse from ever
// decreasing, which a warm-started one must be able to); the sum is clamped
// at zero as written.
template <bool LEAN, class S>
__device__ __forceinline__ void solve_contact(const S& s, uint32_t m, bool warm = false) {
    const uint32_t a = s.ma[m], b = s.mb[m];
    const bool sa = s.kind[a] & K_STATIC, sb = s.kind[b] & K_STATIC;
    // the momenta, read once: no other constraint of this colour moves a or
    // b, so the sums below are the read-modify-writes the reference does
    const float4 q1 = s.mom(a), q2 = s.mom(b);
    const float mx1 = q1.x, my1 = q1.y, L1 = q1.z, inv_m1 = q1.w;
    const float mx2 = q2.x, my2 = q2.y, L2 = q2.z, inv_m2 = q2.w;
    const float inv_i1 = s.inv_i[a], inv_i2 = s.inv_i[b];
    const f2 vlinear_1 = scale2(f2{mx1, my1}, inv_m1);
    const float omega1 = L1 * inv_i1;
    const f2 vlinear_2 = scale2(f2{mx2, my2}, inv_m2);
    const float omega2 = L2 * inv_i2;
    const f2 n = {s.nx[m], s.ny[m]};
    const f2 t = cw90(n);
    const float fr = s.fric[m];
    const uint32_t p0 = s.mp0[m], np = s.mnp[m];
    const bool comp = s.cpn != nullptr;
    // Both points start from the velocities above (collision.zig:145-149),
    // so their inputs are all read before either point's accumulators are
    // written back; the impulses reach the bodies in the reference's order.
    float bias[2], mnp_[2], mtp[2], an[2], at[2], cn[2] = {0.f, 0.f}, ct[2] = {0.f, 0.f};
    f2 r1[2], r2[2];
#pragma unroll
    for (uint32_t k = 0; k < 2; ++k) {
        bias[k] = -1.f;
        if (k >= np) continue;
        const uint32_t p = p0 + k;
        bias[k] = s.bias[p];
        s.template arms<LEAN>(p, a, b, &r1[k], &r2[k]);
        mnp_[k] = s.mn[p];
        mtp[k] = s.mt[p];
        an[k] = s.apn[p];
        at[k] = s.apt[p];
        if (comp) {
            cn[k] = s.cpn[p];
            ct[k] = s.cpt[p];
        }
    }
    f2 alp1 = {0.f, 0.f}, alp2 = {0.f, 0.f};
    float arp1 = 0.f, arp2 = 0.f;
#pragma unroll
    for (uint32_t k = 0; k < 2; ++k) {
        if (bias[k] < 0.0f) continue;  // depth >= 0 (or no point): accumulators stay 0 (collision.zig:154-158)
        const f2 v1 = add2(vlinear_1, f2{-r1[k].y * omega1, r1[k].x * omega1});
        const f2 v2 = add2(vlinear_2, f2{-r2[k].y * omega2, r2[k].x * omega2});
        const f2 dv = sub2(v1, v2);
        float num = dot2(dv, n) + bias[k];  // BAUMGARTE*max(0,-depth-SLOP)/h (collision.zig:172)
        const float pn = num * mnp_[k];
        if (!warm && pn < MIN_MANIFOLD_IMPULSE) continue;
        num = dot2(dv, t);
        const float pt = num * mtp[k];
        float applied_pn, applied_pt;
        acc_update(comp, an[k], at[k], cn[k], ct[k], pn, pt, fr, &applied_pn, &applied_pt);
        const uint32_t p = p0 + k;
        s.apn[p] = an[k];
        s.apt[p] = at[k];
        if (comp) {
            s.cpn[p] = cn[k];
            s.cpt[p] = ct[k];
        }
        const f2 dp = add2(scale2(n, applied_pn), scale2(t, applied_pt));
        if (!sa) {
            alp1 = sub2(alp1, dp);
            arp1 -= cross2(r1[k], dp);
        }
        if (!sb) {
            alp2 = add2(alp2, dp);
            arp2 += cross2(r2[k], dp);
        }
    }
    // A static body receives exactly +0 in the reference; its state is left alone.
    if (!sa) s.put_mom(a, mx1 + alp1.x, my1 + alp1.y, L1 + arp1, inv_m1);
    if (!sb) s.put_mom(b, mx2 + alp2.x, my2 + alp2.y, L2 + arp2, inv_m2);
}

// calculateImpulses with two lanes per manifold: lane 2q + h of a warp takes
// contact point h.  Both points start from the velocities read once per
// manifold (collision.zig:145-149), so they are independent until their
// impulses reach the bodies; the even lane adds them in the reference's
// order, point 0 then point 1, which keeps every sum bit-identical to
// solve_contact.  Every lane of the warp must call this (it shuffles);
// `valid` says whether the lane pair holds a manifold.
template <bool LEAN, class S>
__device__ __forceinline__ void solve_contact_lanes(const S& s, uint32_t m, bool valid, uint32_t lane,
                                                    bool warm = false) {
    const uint32_t half = lane & 1u;
    uint32_t a = 0, b = 0;
    bool sa = true, sb = true, hit = false;
    f2 dp = {0.f, 0.f};
    float c1 = 0.f, c2 = 0.f;
    // the momenta, read once (no other constraint of this colour moves a or
    // b): the even lane's write-back below adds to these values
    float mx1 = 0.f, my1 = 0.f, L1 = 0.f, inv_m1 = 0.f, mx2 = 0.f, my2 = 0.f, L2 = 0.f, inv_m2 = 0.f;
    if (valid) {
        a = s.ma[m];
        b = s.mb[m];
        sa = s.kind[a] & K_STATIC;
        sb = s.kind[b] & K_STATIC;
        const float4 q1 = s.mom(a), q2 = s.mom(b);
        mx1 = q1.x;
        my1 = q1.y;
        L1 = q1.z;
        inv_m1 = q1.w;
        mx2 = q2.x;
        my2 = q2.y;
        L2 = q2.z;
        inv_m2 = q2.w;
        if (half < (uint32_t)s.mnp[m]) {
            const uint32_t p = s.mp0[m] + half;
            const float bias = s.bias[p];
            if (!(bias < 0.0f)) {  // bias < 0: depth >= 0, accumulators stay 0 (collision.zig:154-158)
                const float inv_i1 = s.inv_i[a], inv_i2 = s.inv_i[b];
                const f2 vlinear_1 = scale2(f2{mx1, my1}, inv_m1);
                const float omega1 = L1 * inv_i1;
                const f2 vlinear_2 = scale2(f2{mx2, my2}, inv_m2);
                const float omega2 = L2 * inv_i2;
                const f2 n = {s.nx[m], s.ny[m]};
                const f2 t = cw90(n);
                f2 r1, r2;
                s.template arms<LEAN>(p, a, b, &r1, &r2);
                const f2 v1 = add2(vlinear_1, f2{-r1.y * omega1, r1.x * omega1});
                const f2 v2 = add2(vlinear_2, f2{-r2.y * omega2, r2.x * omega2});
                const f2 dv = sub2(v1, v2);
                float num = dot2(dv, n) + bias;
                const float pn = num * s.mn[p];
                if (warm || !(pn < MIN_MANIFOLD_IMPULSE)) {  // as solve_contact's skip, NaN included
                    num = dot2(dv, t);
                    const float pt = num * s.mt[p];
                    float applied_pn, applied_pt;
                    accumulate(s, p, pn, pt, s.fric[m], &applied_pn, &applied_pt);
                    dp = add2(scale2(n, applied_pn), scale2(t, applied_pt));
                    c1 = cross2(r1, dp);
                    c2 = cross2(r2, dp);
                    hit = true;
                }
            }
        }
    }
    const float dqx = __shfl_down_sync(0xffffffffu, dp.x, 1);
    const float dqy = __shfl_down_sync(0xffffffffu, dp.y, 1);
    const float q1 = __shfl_down_sync(0xffffffffu, c1, 1);
    const float q2 = __shfl_down_sync(0xffffffffu, c2, 1);
    const bool hit1 = __shfl_down_sync(0xffffffffu, hit ? 1 : 0, 1) != 0;
    if (!valid || half) return;
    f2 alp1 = {0.f, 0.f}, alp2 = {0.f, 0.f};
    float arp1 = 0.f, arp2 = 0.f;
    if (hit) {
        if (!sa) {
            alp1 = sub2(alp1, dp);
            arp1 -= c1;
        }
        if (!sb) {
            alp2 = add2(alp2, dp);
            arp2 += c2;
        }
    }
    if (hit1) {
        const f2 d1 = {dqx, dqy};
        if (!sa) {
            alp1 = sub2(alp1, d1);
            arp1 -= q1;
        }
        if (!sb) {
            alp2 = add2(alp2, d1);
            arp2 += q2;
        }
    }
    // A static body receives exactly +0 in the reference; its state is left alone.
    if (!sa) s.put_mom(a, mx1 + alp1.x, my1 + alp1.y, L1 + arp1, inv_m1);
    if (!sb) s.put_mom(b, mx2 + alp2.x, my2 + alp2.y, L2 + arp2, inv_m2);
}

// ---- warm starting (an extension; off in reference mode) ----
// Each world keeps last frame's accumulated impulses in an open-addressing
// table in HBM: key (reference id << 32 | incident id), the bodies' stable
// ids, so the table outlives changes to the body store; value (pn0, pt0,
// pn1, pt1), and in compensated mode their compensation words beside it.
__host__ __device__ __forceinline__ uint32_t warm_hash(uint32_t k) {
    k ^= k >> 16;
    k *= 0x7FEB352Du;
    k ^= k >> 15;
    k *= 0x846CA68Bu;
    k ^= k >> 16;
    return k;
}

// 64-bit keys (the grid pipeline: reference << 32 | incident)
__host__ __device__ __forceinline__ uint32_t warm_hash(unsigned long long k) {
    return warm_hash((uint32_t)k ^ (warm_hash((uint32_t)(k >> 32)) * 0x9E3779B1u));
}

// Slot of `key` in a table of `hs` slots (a power of two), or -1; all-ones
// keys mark empty slots.
template <class K>
__device__ __forceinline__ int warm_find(const K* __restrict__ keys, uint32_t hs, K key) {
    const uint32_t mask = hs - 1u, h = warm_hash(key);
    for (uint32_t probe = 0; probe < hs; ++probe) {
        const uint32_t slot = (h + probe) & mask;
        const K k = keys[slot];
        if (k == key) return (int)slot;
        if (k == ~K(0)) return -1;
    }
    return -1;
}

// Claims the slot of a key that is not in the table yet (keys are unique
// per frame) and returns it; the table holds at most half its slots, so a
// free slot is always found (-1 only for a full table).
template <class K>
__device__ __forceinline__ int warm_claim(K* keys, uint32_t hs, K key) {
    const uint32_t mask = hs - 1u, h = warm_hash(key);
    for (uint32_t probe = 0; probe < hs; ++probe) {
        const uint32_t slot = (h + probe) & mask;
        if (atomicCAS(&keys[slot], ~K(0), key) == ~K(0)) return (int)slot;
    }
    return -1;
}

// The warm-start key of a manifold: its bodies' stable ids.
__device__ __forceinline__ unsigned long long warm_key_ids(uint32_t ref_id, uint32_t inc_id) {
    return ((unsigned long long)ref_id << 32) | inc_id;
}

// Applies a manifold's (warm-started) accumulated impulses to its bodies,
// summed as calculateImpulses sums its applied ones; a point with depth >= 0
// (bias < 0) starts from zero instead.
template <bool LEAN, class S>
__device__ __forceinline__ void warm_apply_contact(const S& s, uint32_t m) {
    const uint32_t a = s.ma[m], b = s.mb[m];
    const bool sa = s.kind[a] & K_STATIC, sb = s.kind[b] & K_STATIC;
    const f2 n = {s.nx[m], s.ny[m]};
    const f2 t = cw90(n);
    f2 alp1 = {0.f, 0.f}, alp2 = {0.f, 0.f};
    float arp1 = 0.f, arp2 = 0.f;
    const uint32_t p0 = s.mp0[m], np = s.mnp[m];
    for (uint32_t k = 0; k < np; ++k) {
        const uint32_t p = p0 + k;
        if (s.bias[p] < 0.0f) {
            s.apn[p] = 0.f;
            s.apt[p] = 0.f;
            if (s.cpn) {
                s.cpn[p] = 0.f;
                s.cpt[p] = 0.f;
            }
            continue;
        }
        f2 r1, r2;
        s.template arms<LEAN>(p, a, b, &r1, &r2);
        const f2 dp = add2(scale2(n, s.apn[p]), scale2(t, s.apt[p]));
        if (!sa) {
            alp1 = sub2(alp1, dp);
            arp1 -= cross2(r1, dp);
        }
        if (!sb) {
            alp2 = add2(alp2, dp);
            arp2 += cross2(r2, dp);
        }
    }
    if (!sa) {
        s.MX(a) += alp1.x;
        s.MY(a) += alp1.y;
        s.AM(a) += arp1;
    }
    if (!sb) {
        s.MX(b) += alp2.x;
        s.MY(b) += alp2.y;
        s.AM(b) += arp2;
    }
}

// Constraint solve functions (src/core/Constraints/*.zig).
template <class S>
__device__ __forceinline__ void solve_joint(const S& s, uint8_t type, uint32_t i1, uint32_t i2,
                                            const float* __restrict__ prm, float h) {
    const float pmax = __ldg(prm + 0), pmin = __ldg(prm + 1), beta = __ldg(prm + 2);
    if (type == J_DISTANCE) {  // DistanceJoint.zig:40-75
        const float epsilon = CONSTRAINT_GRADIENT_DIVISION_LIMIT;
        const float target = __ldg(prm + 3);
        const bool st1 = s.kind[i1] & K_STATIC, st2 = s.kind[i2] & K_STATIC;
        const float w1 = st1 ? 0.f : 1.0f / s.mass(i1);
        const float w2 = st2 ? 0.f : 1.0f / s.mass(i2);
        const f2 v1 = scale2(f2{s.MX(i1), s.MY(i1)}, w1);
        const f2 v2 = scale2(f2{s.MX(i2), s.MY(i2)}, w2);
        const f2 rel = sub2(v2, v1);
        const f2 d = sub2(f2{s.px[i2], s.py[i2]}, f2{s.px[i1], s.py[i1]});
        const f2 normal = normalize2(d);
        const float dist_error = length2(d) - target;
        const float pc = beta * dist_error / zmax(target, 0.001f);
        float J = -(dot2(rel, normal) + pc) / (w1 + w2);
        const float ndv = dot2(normal, rel);
        const float den = 1.0f / zmax(fabsf(ndv), epsilon);
        J = zclamp(J, pmin * den, pmax * den);
        const f2 dp = scale2(normal, J);
        s.MX(i1) -= dp.x;
        s.MY(i1) -= dp.y;
        s.MX(i2) += dp.x;
        s.MY(i2) += dp.y;
    } else if (type == J_OFFSET) {  // OffsetDistanceJoint.zig:44-105
        const float epsilon = CONSTRAINT_GRADIENT_DIVISION_LIMIT;
        const f2 r1 = {__ldg(prm + 3), __ldg(prm + 4)}, r2 = {__ldg(prm + 5), __ldg(prm + 6)};
        const float target = __ldg(prm + 7);
        const bool st1 = s.kind[i1] & K_STATIC, st2 = s.kind[i2] & K_STATIC;
        const f2 rr1 = rot(r1, s.cs[i1], s.sn[i1]);
        const f2 rr2 = rot(r2, s.cs[i2], s.sn[i2]);
        const f2 a1 = add2(rr1, f2{s.px[i1], s.py[i1]});
        const f2 a2 = add2(rr2, f2{s.px[i2], s.py[i2]});
        const f2 normal = normalize2(sub2(a2, a1));
        const float inv_m1 = st1 ? 0.f : 1.0f / s.mass(i1);
        const float inv_m2 = st2 ? 0.f : 1.0f / s.mass(i2);
        const float inv_i1 = st1 ? 0.f : 1.0f / s.inertia(i1);
        const float inv_i2 = st2 ? 0.f : 1.0f / s.inertia(i2);
        const f2 vl1 = scale2(f2{s.MX(i1), s.MY(i1)}, inv_m1);
        const float om1 = s.AM(i1) * inv_i1;
        const f2 vl2 = scale2(f2{s.MX(i2), s.MY(i2)}, inv_m2);
        const float om2 = s.AM(i2) * inv_i2;
        const f2 v1 = add2(vl1, f2{-rr1.y * om1, rr1.x * om1});
        const f2 v2 = add2(vl2, f2{-rr2.y * om2, rr2.x * om2});
        const f2 dv = sub2(v2, v1);
        const float dist_error = length2(sub2(a2, a1)) - target;
        const float pc = beta * dist_error / zmax(target, epsilon);
        const float num = dot2(normal, dv) + pc;
        const float r1xn = cross2(rr1, normal);
        const float r2xn = cross2(rr2, normal);
        const float den = inv_m1 + inv_m2 + r1xn * r1xn * inv_i1 + r2xn * r2xn * inv_i2;
        float J = -num / den;
        const float ndv = dot2(normal, dv);
        const float den2 = 1.0f / zmax(fabsf(ndv), epsilon);
        J = zclamp(J, pmin * den2, pmax * den2);
        const f2 dp = scale2(normal, J);
        s.MX(i1) -= dp.x;
        s.MY(i1) -= dp.y;
        s.AM(i1) -= J * r1xn;
        s.MX(i2) += dp.x;
        s.MY(i2) += dp.y;
        s.AM(i2) += J * r2xn;
    } else if (type == J_FIXED) {  // FixedPositionJoint.zig:38-72
        if (s.kind[i1] & K_STATIC) return;
        const float epsilon = ALLOWED_CONSTRAINT_VALUE;
        const f2 target = {__ldg(prm + 3), __ldg(prm + 4)};
        const float w = 1.0f / s.mass(i1);
        const f2 v = scale2(f2{s.MX(i1), s.MY(i1)}, w);
        const f2 delta = sub2(target, f2{s.px[i1], s.py[i1]});
        const float dist = length2(delta);
        if (dist < ALLOWED_CONSTRAINT_VALUE) return;
        const f2 normal = scale2(delta, 1.0f / dist);
        const float bias = beta * dist;
        const float relv = dot2(v, normal);
        float J = -(relv - bias) / w;
        const float den = 1.0f / zmax(fabsf(relv), epsilon);
        J = zclamp(J, pmin * den, pmax * den);
        const f2 dp = scale2(normal, J);
        s.MX(i1) += dp.x;
        s.MY(i1) += dp.y;
    } else {  // MotorJoint.zig:38-64
        if (s.kind[i1] & K_STATIC) return;
        const float epsilon = ALLOWED_CONSTRAINT_VALUE;
        const float target = __ldg(prm + 3);
        const float I = s.inertia(i1);
        const float omega = s.AM(i1) / I;
        const float C = omega - target;
        if (fabsf(C) < ALLOWED_CONSTRAINT_VALUE) return;
        const float bias = beta * C;
        const float torque = s.tq[i1];
        float J = torque - bias;
        const float relv = torque / I;
        const float den = 1.0f / zmax(fabsf(relv), epsilon);
        J = zclamp(J, pmin * den, pmax * den);
        s.AM(i1) += J * h;
    }
}

__device__ __forceinline__ bool joint_two_bodies(uint8_t type) {
    return type == J_DISTANCE || type == J_OFFSET;
}

}  // namespace r2d
