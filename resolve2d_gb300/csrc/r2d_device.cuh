/*
 * r2d_device.cuh -- per-constraint and per-shape device arithmetic of the
 * resolve2d step, written for structure-of-arrays state.
 *
 * Every function reproduces one reference function's f32 arithmetic in the
 * reference's evaluation order (paths relative to the reference project):
 * the build compiles with --fmad=false and IEEE division / square root, so
 * the results are the bits the reference's own formulas give.  Rotation
 * values come from r2d_sincos.h; a body's sin/cos is computed once per
 * angle and reused, which gives the same bits as the reference calling
 * std.math.sin/cos at every rotate2 (src/core/nmath.zig:129-136).
 */
#pragma once

#include <stdint.h>

#include "r2d_colour.h"
#include "r2d_sincos.h"

namespace r2d {

// ---- constants (src/core/simulation_constants.zig:3-22) ----
constexpr float MIN_MANIFOLD_IMPULSE = 1e-4f;
constexpr float BAUMGARTE = 0.02f;
constexpr float BAUMGARTE_SLOP = 0.005f;
constexpr float SAT_OVERLAP_THRESHOLD = 1e-4f;
constexpr float COLLISION_MARGIN = 0.01f;
constexpr float NMATH_WARN_DIVIDING_BELOW = 1e-3f;
constexpr float AABB_EPS_OVERLAP = 0.01f;
constexpr float CONSTRAINT_GRADIENT_DIVISION_LIMIT = 1e-4f;
constexpr float ALLOWED_CONSTRAINT_VALUE = 1e-6f;

#define R2D_DF __device__ __forceinline__

struct f2 {
    float x, y;
};

// ---- nmath (src/core/nmath.zig) ----
R2D_DF f2 add2(f2 a, f2 b) { return {a.x + b.x, a.y + b.y}; }
R2D_DF f2 sub2(f2 a, f2 b) { return {a.x - b.x, a.y - b.y}; }
R2D_DF f2 scale2(f2 a, float s) { return {a.x * s, a.y * s}; }
R2D_DF float dot2(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
R2D_DF float cross2(f2 a, f2 b) { return a.x * b.y - a.y * b.x; }
R2D_DF float length2(f2 a) { return sqrtf(dot2(a, a)); }
R2D_DF f2 normalize2(f2 a) {  // nmath.zig:95-103
    float len = length2(a);
    if (len < NMATH_WARN_DIVIDING_BELOW) return {0.f, 0.f};
    return scale2(a, 1.0f / len);
}
R2D_DF f2 negate2(f2 a) { return {-a.x, -a.y}; }
R2D_DF f2 neg_by_mul(f2 a) { return {a.x * -1.0f, a.y * -1.0f}; }  // Vector2.negate (:48-51)
R2D_DF f2 addmult2(f2 a, f2 b, float s) { return add2(a, scale2(b, s)); }
R2D_DF bool approx_eql(float a, float b, float eps) { return a > b - eps && a < b + eps; }
R2D_DF bool approx_eql2(f2 a, f2 b, float eps) {
    return approx_eql(a.x, b.x, eps) && approx_eql(a.y, b.y, eps);
}
R2D_DF f2 rot(f2 a, float c, float s) { return {a.x * c - a.y * s, a.x * s + a.y * c}; }
R2D_DF f2 cw90(f2 a) { return {a.y, -a.x}; }
R2D_DF f2 ccw90(f2 a) { return {-a.y, a.x}; }

// Zig @max / @min on floats: the non-NaN operand wins.
// Written as selects (no branches); same results as: a NaN -> b,
// else b NaN -> a, else the larger (smaller) with b on ties.
R2D_DF float zmax(float a, float b) {
    float r = a > b ? a : b;
    r = (b != b) ? a : r;
    return (a != a) ? b : r;
}
R2D_DF float zmin(float a, float b) {
    float r = a < b ? a : b;
    r = (b != b) ? a : r;
    return (a != a) ? b : r;
}
R2D_DF float zclamp(float v, float lo, float hi) { return zmax(lo, zmin(v, hi)); }

// ---- spatial hash (src/core/SpatialHash.zig:78-81) ----
// u64 % table_size without a 64-bit division: Barrett reduction with
// recip = floor((2^64 - 1) / table_size), then at most two corrections.
// Exact for every 64-bit hash and every table size >= 1.
struct BucketMod {
    uint64_t recip;
    uint32_t size;
};
__host__ __device__ __forceinline__ uint64_t bucket_recip(uint32_t table_size) {
    return table_size ? 0xFFFFFFFFFFFFFFFFull / (uint64_t)table_size : 0ull;
}
R2D_DF uint32_t cell_bucket(int64_t xi, int64_t yi, const BucketMod& m) {
    const uint64_t h = ((uint64_t)xi * 92837111ull) ^ ((uint64_t)yi * 689287499ull);
    const uint64_t q = __umul64hi(h, m.recip);
    uint64_t r = h - q * (uint64_t)m.size;
    if (r >= m.size) r -= m.size;
    if (r >= m.size) r -= m.size;
    return (uint32_t)r;
}

// floor(c / cell) as the reference's @intFromFloat(@floor(..)) (SpatialHash.zig:93-96);
// false when the value is not a representable cell index.
R2D_DF bool cell_index(float c, float cell, int32_t* out) {
    float v = floorf(c / cell);
    if (!(v > -2.0e9f && v < 2.0e9f)) return false;
    *out = (int32_t)v;
    return true;
}

// ---- AABB (src/core/aabb.zig:12-19; Disc.zig:63-66; Rectangle.zig:71-86) ----
R2D_DF bool aabb_intersects(f2 p1, float hw1, float hh1, f2 p2, float hw2, float hh2) {
    float dx = fabsf(p2.x - p1.x);
    float dy = fabsf(p2.y - p1.y);
    return (dx <= (hw1 + hw2) + AABB_EPS_OVERLAP) && (dy <= (hh1 + hh2) + AABB_EPS_OVERLAP);
}

// Local rectangle vertices (Rectangle.zig:38-40): (-w,-h), (-w,h), (w,h), (w,-h).
R2D_DF f2 rect_local(int i, float w, float h) {
    return {(i < 2) ? -w : w, (i == 0 || i == 3) ? -h : h};
}

R2D_DF void rect_half_extents(float width, float height, float c, float s, float* hw, float* hh) {
    const float w = width / 2.0f, h = height / 2.0f;
    float ew = 0.f, eh = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f2 r = rot(rect_local(i, w, h), c, s);
        if (r.x > ew) ew = r.x;
        if (r.y > eh) eh = r.y;
    }
    *hw = ew;
    *hh = eh;
}

// a[i] for a runtime i without dynamic indexing (keeps a[] in registers)
template <int N>
R2D_DF f2 selv(const f2 (&a)[N], uint32_t i) {
    f2 r = a[0];
#pragma unroll
    for (int k = 1; k < N; ++k) r = i == (uint32_t)k ? a[k] : r;
    return r;
}

// ---- narrowphase geometry ----
// One body as the SAT sees it.  For a rectangle (or, on the grid pipeline, a
// convex polygon of up to MAXV vertices) the world vertices
// (Rectangle.zig:88-98) and edge normals (Rectangle.zig:132-151) are computed
// once; the reference recomputes the same values at every use.  A polygon is
// the rectangle's code over its own vertex ring, the rectangle's winding
// (clockwise, so that the counter-clockwise turn of an edge points out).
template <int MAXV>
struct GeoT {
    f2 pos;
    float radius;  // disc
    bool rect;     // has vertices: a rectangle or a polygon
    uint32_t nv_;  // vertices (MAXV > 4 only)
    f2 wv[MAXV];   // world vertices
    f2 en[MAXV];   // edge normals (ccw90 of the normalised edge)
    R2D_DF uint32_t nv() const { return MAXV == 4 ? 4u : nv_; }
    R2D_DF uint32_t next(uint32_t i) const { return i + 1u == nv() ? 0u : i + 1u; }
};
using Geo = GeoT<4>;
constexpr int MAX_POLY_VERTS = 8;
using GeoPoly = GeoT<MAX_POLY_VERTS>;

template <int MAXV>
R2D_DF void geo_make(GeoT<MAXV>& g, f2 pos, bool rect, float d0, float d1, float c, float s) {
    g.pos = pos;
    g.nv_ = 4u;
    g.rect = rect;
    g.radius = d0;
    if (!rect) return;
    const float w = d0 / 2.0f, h = d1 / 2.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) g.wv[i] = add2(rot(rect_local(i, w, h), c, s), pos);
#pragma unroll
    for (int i = 0; i < 4; ++i) g.en[i] = ccw90(normalize2(sub2(g.wv[(i + 1) & 3], g.wv[i])));
}

// A convex polygon of nv (3..MAX_POLY_VERTS) local vertices `local`.
R2D_DF void geo_make_polygon(GeoPoly& g, f2 pos, const float2* __restrict__ local, uint32_t nv, float c, float s) {
    g.pos = pos;
    g.rect = true;
    g.radius = 0.f;
    g.nv_ = nv;
#pragma unroll
    for (int i = 0; i < MAX_POLY_VERTS; ++i) {
        if ((uint32_t)i >= nv) break;
        const float2 v = local[i];
        g.wv[i] = add2(rot(f2{v.x, v.y}, c, s), pos);
    }
#pragma unroll
    for (int i = 0; i < MAX_POLY_VERTS; ++i) {
        if ((uint32_t)i >= nv) break;
        g.en[i] = ccw90(normalize2(sub2(selv(g.wv, g.next(i)), g.wv[i])));
    }
}

// A polygon's AABB half extents: Rectangle.updateAABB (Rectangle.zig:71-86)
// over its vertices, from 0.
R2D_DF void polygon_half_extents(const float2* __restrict__ local, uint32_t nv, float c, float s, float* hw,
                                 float* hh) {
    float ew = 0.f, eh = 0.f;
    for (uint32_t i = 0; i < nv; ++i) {
        const float2 v = local[i];
        const f2 r = rot(f2{v.x, v.y}, c, s);
        if (r.x > ew) ew = r.x;
        if (r.y > eh) eh = r.y;
    }
    *hw = ew;
    *hh = eh;
}

// geo_make with a rectangle's edge normals taken from `en` (two float4:
// normals 0, 1 then 2, 3) as geo_make computed them for the same pose, so
// the values are the same bits; the vertices are recomputed (no division).
R2D_DF void geo_make_cached(Geo& g, f2 pos, bool rect, float d0, float d1, float c, float s, const float4* en) {
    g.pos = pos;
    g.nv_ = 4u;
    g.rect = rect;
    g.radius = d0;
    if (!rect) return;
    const float w = d0 / 2.0f, h = d1 / 2.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) g.wv[i] = add2(rot(rect_local(i, w, h), c, s), pos);
    const float4 a = en[0], b = en[1];
    g.en[0] = f2{a.x, a.y};
    g.en[1] = f2{a.z, a.w};
    g.en[2] = f2{b.x, b.y};
    g.en[3] = f2{b.z, b.w};
}

// closestPoint (Disc.zig:80-84; Rectangle.zig:114-130 -- the nearest vertex)
template <int MAXV>
R2D_DF f2 closest_point(const GeoT<MAXV>& g, f2 p) {
    if (!g.rect) {
        f2 n = normalize2(sub2(p, g.pos));
        return addmult2(g.pos, n, g.radius);
    }
    float best = __int_as_float(0x7f800000);
    f2 bp = p;
#pragma unroll
    for (int i = 0; i < MAXV; ++i) {
        if ((uint32_t)i >= g.nv()) break;
        f2 d = sub2(g.wv[i], p);
        float d2 = dot2(d, d);
        if (d2 < best) {
            best = d2;
            bp = g.wv[i];
        }
    }
    return bp;
}

// projectAlongAxis (Disc.zig:92-97; Rectangle.zig:153-169)
template <int MAXV>
R2D_DF void project(const GeoT<MAXV>& g, f2 n, float* lo, float* hi) {
    if (!g.rect) {
        float mid = dot2(g.pos, n);
        *lo = mid - g.radius;
        *hi = mid + g.radius;
        return;
    }
    float l = __int_as_float(0x7f800000), h = __int_as_float(0xff800000);
#pragma unroll
    for (int i = 0; i < MAXV; ++i) {
        if ((uint32_t)i >= g.nv()) break;
        float d = dot2(g.wv[i], n);
        if (d < l) l = d;
        if (d > h) h = d;
    }
    *lo = l;
    *hi = h;
}

struct SatState {
    f2 normal;
    float penetration;
    uint32_t refid;
    bool ref_is_first;  // key.ref_body == the body passed first to performNarrowSAT's o1
};

// overlapSAT (collision.zig:228-289) with `reference` = R, `incident` = I.
template <int MAXV>
R2D_DF bool overlap_sat(SatState& ret, const GeoT<MAXV>& R, const GeoT<MAXV>& I, bool r_is_o1) {
    const float EPS = SAT_OVERLAP_THRESHOLD;
    const int nn = R.rect ? (int)R.nv() : 1;
    f2 disc_axis = {0.f, 0.f};
    if (!R.rect) disc_axis = normalize2(sub2(closest_point(I, R.pos), R.pos));  // Disc.zig:86-90
#pragma unroll
    for (int it = 0; it < MAXV; ++it) {
        if (it >= nn) break;
        f2 normal = R.rect ? R.en[it] : disc_axis;
        bool flipped = false;
        if (dot2(normal, sub2(I.pos, R.pos)) < 0.0f) {  // normalShouldFlipSAT (:221-226)
            normal = neg_by_mul(normal);
            flipped = true;
        }
        float p1lo, p1hi, p2lo, p2hi;
        project(R, normal, &p1lo, &p1hi);
        project(I, normal, &p2lo, &p2hi);
        float d1 = p1hi - p2lo;
        float d2 = p2hi - p1lo;
        float d = zmin(d1, d2);
        if (d <= -COLLISION_MARGIN) return false;
        if (!flipped && approx_eql2(normal, ret.normal, EPS)) {
            float tref = dot2(R.pos, normal);
            float tinc = dot2(I.pos, normal);
            if (tref < tinc - EPS) {
                ret.penetration = d;
                ret.normal = normal;
                ret.refid = it;
                ret.ref_is_first = r_is_o1;
            }
        }
        if (!flipped && approx_eql2(normal, negate2(ret.normal), EPS)) {
            f2 diff = sub2(I.pos, R.pos);
            if (dot2(diff, normal) > dot2(diff, ret.normal) + EPS) {
                ret.penetration = d;
                ret.normal = normal;
                ret.refid = it;
                ret.ref_is_first = r_is_o1;
            }
        }
        if (d + EPS < ret.penetration) {
            ret.penetration = d;
            ret.normal = normal;
            ret.refid = it;
            ret.ref_is_first = r_is_o1;
        }
    }
    return true;
}

// performNarrowSAT (collision.zig:299-320): o1 = lower id.  The reference
// leaves ret.normal/key undefined until the first axis writes them; the
// start value here is normal (0,0), reference = o1, edge 0.
template <int MAXV>
R2D_DF bool perform_narrow_sat(const GeoT<MAXV>& o1, const GeoT<MAXV>& o2, SatState& ret) {
    ret.normal = {0.f, 0.f};
    ret.penetration = __int_as_float(0x7f800000);
    ret.refid = 0;
    ret.ref_is_first = true;
    if (!overlap_sat(ret, o1, o2, true)) return false;
    if (!overlap_sat(ret, o2, o1, false)) return false;
    return true;
}

struct NewPoint {
    f2 ref_r, inc_r, mid;
    float depth;
};

// CollisionPoint.init (collision.zig:38-51)
R2D_DF NewPoint make_point(f2 pos, float depth, f2 ref_pos, f2 inc_pos, f2 normal) {
    f2 middle = sub2(pos, scale2(normal, depth / 2.0f));
    NewPoint p;
    p.mid = middle;
    p.ref_r = sub2(middle, ref_pos);
    p.inc_r = sub2(middle, inc_pos);
    p.depth = depth;
    return p;
}

// clipLineToLine (collision.zig:330-363): b clipped onto a.
R2D_DF void clip_line_to_line(f2 aa, f2 ab, f2 ba, f2 bb, f2* p1o, f2* p2o) {
    f2 delta_a = sub2(ab, aa);
    float a_len = length2(delta_a);
    f2 tang = scale2(delta_a, 1.0f / a_len);
    f2 p1 = ba, p2 = bb;
    {
        float scalar = dot2(sub2(ba, aa), tang);
        if (!(scalar > 0.0f && scalar < a_len)) {
            f2 clos = scalar < 0.5f * a_len ? aa : ab;
            f2 delta_p = sub2(ba, bb);
            float t = -dot2(tang, sub2(bb, clos)) / dot2(tang, delta_p);
            p1 = addmult2(bb, delta_p, t);
        }
    }
    {
        float scalar = dot2(sub2(bb, aa), tang);
        if (!(scalar > 0.0f && scalar < a_len)) {
            f2 clos = scalar < 0.5f * a_len ? aa : ab;
            f2 delta_p = sub2(bb, ba);
            float t = -dot2(tang, sub2(ba, clos)) / dot2(tang, delta_p);
            p2 = addmult2(ba, delta_p, t);
        }
    }
    *p1o = p1;
    *p2o = p2;
}

// identifyCollisionPoints (Disc.zig:99-123; Rectangle.zig:171-211 with
// clipAgainstEdge Disc.zig:125-130 / Rectangle.zig:213-238).  Returns the
// number of points written (0..2).
template <int MAXV>
R2D_DF int identify_points(const GeoT<MAXV>& ref, const GeoT<MAXV>& inc, uint32_t refid, NewPoint out[2]) {
    if (!ref.rect) {
        f2 pos = closest_point(inc, ref.pos);
        f2 normal = normalize2(sub2(pos, ref.pos));  // Disc.getNormal recomputes the same point
        if (dot2(normal, sub2(inc.pos, ref.pos)) < 0.0f) normal = neg_by_mul(normal);
        float dot = dot2(normal, sub2(pos, ref.pos));
        float depth = dot - ref.radius;
        out[0] = make_point(pos, depth, ref.pos, inc.pos, normal);
        return 1;
    }
    const f2 ea = selv(ref.wv, refid);
    const f2 eb = selv(ref.wv, ref.next(refid));
    const f2 ndir = selv(ref.en, refid);
    if (!inc.rect) {
        f2 pos = addmult2(inc.pos, ndir, -inc.radius);
        float dot = dot2(sub2(pos, ea), ndir);
        out[0] = make_point(pos, dot, ref.pos, inc.pos, ndir);
        return 1;
    }
    uint32_t best = 0;
    bool found = false;
    float best_dot = __int_as_float(0x7f800000);
#pragma unroll
    for (int i = 0; i < MAXV; ++i) {
        if ((uint32_t)i >= inc.nv()) break;
        float d = dot2(ndir, inc.en[i]);
        if (d < best_dot) {
            best_dot = d;
            best = i;
            found = true;
        }
    }
    if (!found) best = 0;  // every dot NaN: the reference reads an undefined edge
    f2 pa, pb;
    clip_line_to_line(ea, eb, selv(inc.wv, best), selv(inc.wv, inc.next(best)), &pa, &pb);
    const float dot_a = dot2(sub2(pa, ea), ndir);
    const float dot_b = dot2(sub2(pb, eb), ndir);
    const bool ha = dot_a < COLLISION_MARGIN, hb = dot_b < COLLISION_MARGIN;
    if (ha) {
        out[0] = make_point(pa, dot_a, ref.pos, inc.pos, ndir);
        if (hb) out[1] = make_point(pb, dot_b, ref.pos, inc.pos, ndir);
    } else if (hb) {
        out[0] = make_point(pb, dot_b, ref.pos, inc.pos, ndir);
    }
    return (ha ? 1 : 0) + (hb ? 1 : 0);
}

// A set of colours 0..255 held in eight registers.
// Integration of a dynamic body's pose in the FP64-positions mode: the
// f32 step's arithmetic (lib.zig:238-243: pos += momentum * (h / mass),
// angle += ang_momentum * h / inertia) in double on a double pose kept in
// HBM (pos64[f * NB + g], f = x, y, angle); the f32 pose becomes its
// rounding.  Momenta and everything else stay f32.
R2D_DF void integrate_pose64(double* __restrict__ pos64, size_t NB, uint32_t g, float mx, float my, float L,
                             float h, float mass, float inertia, float* px, float* py, float* ang) {
    const double sm = (double)h / (double)mass;
    const double x = pos64[g] + (double)mx * sm;
    const double y = pos64[NB + g] + (double)my * sm;
    const double a = pos64[2 * NB + g] + (double)L * (double)h / (double)inertia;
    pos64[g] = x;
    pos64[NB + g] = y;
    pos64[2 * NB + g] = a;
    *px = (float)x;
    *py = (float)y;
    *ang = (float)a;
}

struct ColourSet {
    uint32_t w0 = 0u, w1 = 0u, w2 = 0u, w3 = 0u, w4 = 0u, w5 = 0u, w6 = 0u, w7 = 0u;
    R2D_DF void add(uint32_t c) {
        const uint32_t bit = 1u << (c & 31u), wd = c >> 5;
        w0 |= wd == 0u ? bit : 0u;
        w1 |= wd == 1u ? bit : 0u;
        w2 |= wd == 2u ? bit : 0u;
        w3 |= wd == 3u ? bit : 0u;
        w4 |= wd == 4u ? bit : 0u;
        w5 |= wd == 5u ? bit : 0u;
        w6 |= wd == 6u ? bit : 0u;
        w7 |= wd == 7u ? bit : 0u;
    }
    // lowest colour not in the set; >= limit means none is free below limit
    R2D_DF uint32_t first_free() const {
        if (w0 != 0xFFFFFFFFu) return (uint32_t)__ffs(~w0) - 1u;
        if (w1 != 0xFFFFFFFFu) return 32u + (uint32_t)__ffs(~w1) - 1u;
        if (w2 != 0xFFFFFFFFu) return 64u + (uint32_t)__ffs(~w2) - 1u;
        if (w3 != 0xFFFFFFFFu) return 96u + (uint32_t)__ffs(~w3) - 1u;
        if (w4 != 0xFFFFFFFFu) return 128u + (uint32_t)__ffs(~w4) - 1u;
        if (w5 != 0xFFFFFFFFu) return 160u + (uint32_t)__ffs(~w5) - 1u;
        if (w6 != 0xFFFFFFFFu) return 192u + (uint32_t)__ffs(~w6) - 1u;
        if (w7 != 0xFFFFFFFFu) return 224u + (uint32_t)__ffs(~w7) - 1u;
        return 256u;
    }
};

}  // namespace r2d
