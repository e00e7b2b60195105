/*
 * r2d_oracle.hpp -- CPU restatement of resolve2d's simulation step
 * (nilsblix/resolve2d, Zig source; every function below cites the
 * reference file:line it follows, paths relative to the reference project).
 *
 * TEST INFRASTRUCTURE.  This is the parity oracle and the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and
 * its --impl reference arm) may load it; the product library never does.
 *
 * It keeps the reference's structure on purpose: bodies are stored by value
 * in insertion order (std.AutoArrayHashMap, src/core/lib.zig:135), manifolds
 * are keyed by the (reference, incident) body pair and kept in discovery order
 * (lib.zig:137,294), the spatial hash is the reference's dense counting sort
 * (src/core/SpatialHash.zig:19-71) and the step is Solver.process
 * (lib.zig:189-251).  Shape behaviour goes through per-type functions that
 * stand in for the RigidBody vtable (src/core/Bodies/RigidBody.zig:33-42).
 *
 * Templated on the arithmetic type: R = float is the reference's f32
 * arithmetic; R = double is the same algorithm in double precision (the
 * FP64 oracle for drift studies).
 *
 * Floating-point rules that make R = float bit-identical to the CUDA path:
 * every expression is written in the reference's evaluation order, the build
 * uses -ffp-contract=off (no fused multiply-add, like Zig's default strict
 * float mode), division and sqrt are IEEE, sin/cos come from r2d_sincos.h,
 * and Zig's @min/@max are restated as NaN-ignoring min/max (zmin/zmax).
 *
 * Two solve orders:
 *   ORDER_REFERENCE: joints in insertion order, manifolds in discovery order,
 *                    exactly as lib.zig:226-236 (the reference's behaviour).
 *   ORDER_COLOUR:    the same per-constraint arithmetic replayed in the GPU's
 *                    colour-major order (r2d_colour.h defines the colouring).
 *
 * What pins it.  The reference ships two unit tests, the Vector2 operations
 * (nmath.zig:157-176) and three AABB overlaps (aabb.zig:34-45); the oracle
 * reproduces both (tests/test_oracle_reference_tests.py).  Contacts,
 * rectangle and disc manifolds, friction and joints are also checked on
 * cases worked by hand from the reference source
 * (tests/test_oracle_behaviour.py, test_oracle_manifolds.py,
 * test_oracle_friction.py, test_oracle_joints.py, test_oracle_quirks.py).  The reference cannot be
 * built or run here and ships no golden outputs, so beyond those cases
 * parity is unpinned: the oracle is trusted because it follows the source
 * line by line.
 *
 * Deviations, all documented where they occur:
 *   - body ids are u32 (the reference's RigidBody.Id is u16,
 *     RigidBody.zig:15), so scenes above 65,536 bodies are representable;
 *   - the SAT result starts from normal (0,0), reference normal 0 and key
 *     (o1,o2) where the reference leaves them `undefined`
 *     (collision.zig:300); only a zero-length axis can observe the choice.
 */
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#include "../resolve2d_gb300/csrc/r2d_accum.h"
#include "../resolve2d_gb300/csrc/r2d_colour.h"
#include "../resolve2d_gb300/csrc/r2d_sincos.h"
#include "../resolve2d_gb300/csrc/r2d_sleep.h"

namespace r2o {

enum Status : int {
    OK = 0,
    ERR_INVALID_BODY_ID = -2,  // error.InvalidRigidBodyId (DistanceJoint.zig:44-47)
    ERR_NONFINITE_AABB = -7,   // @intFromFloat of NaN/inf is undefined in the reference
    ERR_CAPACITY = -5,         // a body covers more spatial-hash cells than the oracle will allocate
    ERR_INTERNAL = -4,         // an exception escaped (allocation failure)
};

// More cells than any sane scene covers (the reference would allocate them;
// the oracle reports the blow-up instead of exhausting host memory).
constexpr int64_t MAX_CELLS = 64ll << 20;

enum Order : int { ORDER_REFERENCE = 0, ORDER_COLOUR = 1 };

// Phases of one step, for the optional wall-clock split (Solver::time_phases):
// updateManifolds (broadphase and narrowphase, lib.zig:194, 253-299), the
// colouring of the colour-major order, forces and velocities (lib.zig:199-216),
// the TGS update and preStep (lib.zig:218-224), the iterations
// (lib.zig:226-236) and integration (lib.zig:238-249).
enum Phase : int {
    PH_MANIFOLDS = 0,
    PH_COLOURING,
    PH_FORCES,
    PH_PRESTEP,
    PH_SOLVE,
    PH_INTEGRATE,
    PH_COUNT
};

// ---------------------------------------------------------------------------
// Constants (src/core/simulation_constants.zig:3-22)
// ---------------------------------------------------------------------------
template <class R>
struct C {
    static constexpr R MIN_MANIFOLD_IMPULSE = R(1e-4);
    static constexpr R BAUMGARTE = R(0.02);
    static constexpr R BAUMGARTE_SLOP = R(0.005);
    static constexpr R SAT_OVERLAP_THRESHOLD = R(1e-4);
    static constexpr R COLLISION_MARGIN = R(0.01);
    static constexpr R NMATH_WARN_DIVIDING_BELOW = R(1e-3);
    static constexpr R AABB_EPS_OVERLAP = R(0.01);
    static constexpr R CONSTRAINT_GRADIENT_DIVISION_LIMIT = R(1e-4);
    static constexpr R ALLOWED_CONSTRAINT_VALUE = R(1e-6);
};

// ---------------------------------------------------------------------------
// nmath (src/core/nmath.zig)
// ---------------------------------------------------------------------------
template <class R>
struct V2 {
    R x = 0, y = 0;
};

// Zig @max / @min on floats return the non-NaN operand when one is NaN.
template <class R>
inline R zmax(R a, R b) {
    if (a != a) return b;
    if (b != b) return a;
    return a > b ? a : b;
}
template <class R>
inline R zmin(R a, R b) {
    if (a != a) return b;
    if (b != b) return a;
    return a < b ? a : b;
}
// std.math.clamp(val, lower, upper) = @max(lower, @min(val, upper))
template <class R>
inline R zclamp(R v, R lo, R hi) {
    return zmax(lo, zmin(v, hi));
}

template <class R>
inline bool approx_eql(R a, R b, R eps) {  // nmath.zig:5-7
    return a > b - eps && a < b + eps;
}
template <class R>
inline V2<R> add2(V2<R> a, V2<R> b) { return {a.x + b.x, a.y + b.y}; }  // :58-60
template <class R>
inline V2<R> sub2(V2<R> a, V2<R> b) { return {a.x - b.x, a.y - b.y}; }  // :62-64
template <class R>
inline V2<R> scale2(V2<R> a, R s) { return {a.x * s, a.y * s}; }  // :66-68
template <class R>
inline V2<R> multelem2(V2<R> a, V2<R> b) { return {a.x * b.x, a.y * b.y}; }  // :70-72
template <class R>
inline V2<R> divelem2(V2<R> a, V2<R> b) { return {a.x / b.x, a.y / b.y}; }  // :74-77
template <class R>
inline R dot2(V2<R> a, V2<R> b) { return a.x * b.x + a.y * b.y; }  // :79-81
template <class R>
inline R cross2(V2<R> a, V2<R> b) { return a.x * b.y - a.y * b.x; }  // :83-85
template <class R>
inline R length2(V2<R> a) { return std::sqrt(dot2(a, a)); }  // :87-93
template <class R>
inline V2<R> normalize2(V2<R> a) {  // :95-103
    R len = length2(a);
    if (len < C<R>::NMATH_WARN_DIVIDING_BELOW) return V2<R>{};
    return scale2(a, R(1) / len);
}
template <class R>
inline V2<R> negate2(V2<R> a) { return {-a.x, -a.y}; }  // :105-107
template <class R>
inline V2<R> addmult2(V2<R> a, V2<R> b, R s) { return add2(a, scale2(b, s)); }  // :109-111
template <class R>
inline bool approx_eql2(V2<R> a, V2<R> b, R eps) {  // :121-123
    return approx_eql(a.x, b.x, eps) && approx_eql(a.y, b.y, eps);
}
// Vector2.negate multiplies by -1 (nmath.zig:48-51)
template <class R>
inline void negate_in_place(V2<R>& a) {
    a.x *= R(-1);
    a.y *= R(-1);
}

inline void sincos_r(float a, float* s, float* c) { r2d_sincosf(a, s, c); }
inline void sincos_r(double a, double* s, double* c) { r2d_sincos_d(a, s, c); }

template <class R>
inline V2<R> rotate2(V2<R> a, R angle) {  // nmath.zig:129-136
    R s, c;
    sincos_r(angle, &s, &c);
    return {a.x * c - a.y * s, a.x * s + a.y * c};
}
template <class R>
inline V2<R> rotate90clockwise(V2<R> a) { return {a.y, -a.x}; }  // :142-144
template <class R>
inline V2<R> rotate90counterclockwise(V2<R> a) { return {-a.y, a.x}; }  // :146-148

// ---------------------------------------------------------------------------
// AABB (src/core/aabb.zig)
// ---------------------------------------------------------------------------
template <class R>
struct AABB {
    V2<R> pos;
    R half_width = 0, half_height = 0;
    bool intersects(const AABB& other) const {  // aabb.zig:12-19
        const R EPS = C<R>::AABB_EPS_OVERLAP;
        R dx = std::fabs(other.pos.x - pos.x);
        R dy = std::fabs(other.pos.y - pos.y);
        return (dx <= (half_width + other.half_width) + EPS) &&
               (dy <= (half_height + other.half_height) + EPS);
    }
    V2<R> vertex_min() const { return {pos.x - half_width, pos.y - half_height}; }  // :25-32 [0]
    V2<R> vertex_max() const { return {pos.x + half_width, pos.y + half_height}; }  // :25-32 [2]
};

// ---------------------------------------------------------------------------
// Bodies (src/core/Bodies/{RigidBody,Disc,Rectangle}.zig)
// ---------------------------------------------------------------------------
// RigidBody.zig:28-31, plus a convex polygon: the roadmap's next shape
// (README.md:64-67), behind the same vtable (RigidBody.zig:33-42).  A
// polygon is the rectangle's code over its own vertex ring: local vertices
// about its origin in the rectangle's winding (Rectangle.zig:40 lists
// (-w,-h), (-w,h), (w,h), (w,-h): clockwise, so that the counter-clockwise
// turn of an edge points outwards), 3 to MAX_POLY_VERTS of them.
enum BodyType : uint8_t { DISC = 0, RECTANGLE = 1, POLYGON = 2 };
constexpr uint32_t MAX_POLY_VERTS = 8;

template <class R>
struct Props {  // RigidBody.zig:69-81
    V2<R> pos, momentum, force;
    R mass = 0;
    R angle = 0, ang_momentum = 0, torque = 0, inertia = 0;
    R mu = 0;
};

template <class R>
struct Body {  // RigidBody.zig:83-91 with the Disc / Rectangle payloads inlined
    uint32_t id = 0;
    AABB<R> aabb;
    bool is_static = false;
    uint32_t num_normals = 0;
    BodyType type = DISC;
    Props<R> props;
    R radius = 0;                // Disc.zig:8
    R width = 0, height = 0;     // Rectangle.zig:17-18 (a polygon: the two dims it was given)
    uint32_t nverts = 4;         // vertices of a rectangle or polygon
    V2<R> local_vertices[MAX_POLY_VERTS];  // Rectangle.zig:20
};

template <class R>
struct Line {  // collision.zig:322-325
    V2<R> a, b;
};

template <class R>
struct Edge {  // RigidBody.zig:22-26
    V2<R> dir;
    bool has_edge = false;
    Line<R> edge;
};

template <class R>
struct Incident {  // RigidBody.zig:17-20
    bool is_edge = false;
    Line<R> edge;
    V2<R> point;
};

template <class R>
V2<R> local_to_world(const Body<R>& b, V2<R> p) {  // RigidBody.zig:113-117
    V2<R> r = rotate2(p, b.props.angle);
    return add2(r, b.props.pos);
}

template <class R>
void update_aabb(Body<R>& b) {
    if (b.type == DISC) {  // Disc.zig:63-66
        b.aabb = AABB<R>{b.props.pos, b.radius, b.radius};
        return;
    }
    // Rectangle.zig:71-86 (a polygon: over its vertices)
    R width = 0, height = 0;
    for (uint32_t i = 0; i < b.nverts; ++i) {
        V2<R> rot = rotate2(b.local_vertices[i], b.props.angle);
        if (rot.x > width) width = rot.x;
        if (rot.y > height) height = rot.y;
    }
    b.aabb = AABB<R>{b.props.pos, width, height};
}

template <class R>
void world_vertices(const Body<R>& b, V2<R> out[MAX_POLY_VERTS]) {  // Rectangle.zig:88-98
    for (uint32_t i = 0; i < b.nverts; ++i) {
        V2<R> r = rotate2(b.local_vertices[i], b.props.angle);
        out[i] = add2(r, b.props.pos);
    }
}

template <class R>
V2<R> closest_point(const Body<R>& b, V2<R> pos) {
    if (b.type == DISC) {  // Disc.zig:80-84
        V2<R> normal = normalize2(sub2(pos, b.props.pos));
        return addmult2(b.props.pos, normal, b.radius);
    }
    // Rectangle.zig:114-130: the nearest VERTEX, not the nearest surface point.
    R best_dist2 = std::numeric_limits<R>::infinity();
    V2<R> best_pos = pos;
    V2<R> wv[MAX_POLY_VERTS];
    world_vertices(b, wv);
    for (uint32_t i = 0; i < b.nverts; ++i) {
        V2<R> d = sub2(wv[i], pos);
        R dist2 = dot2(d, d);
        if (dist2 < best_dist2) {
            best_dist2 = dist2;
            best_pos = wv[i];
        }
    }
    return best_pos;
}

template <class R>
Edge<R> get_normal(const Body<R>& self, const Body<R>& other, uint32_t iter) {
    Edge<R> e;
    if (self.type == DISC) {  // Disc.zig:86-90
        V2<R> closest = closest_point(other, self.props.pos);
        e.dir = normalize2(sub2(closest, self.props.pos));
        return e;
    }
    // Rectangle.zig:132-151
    uint32_t next_iter = iter + 1 == self.nverts ? 0 : iter + 1;
    V2<R> r1 = rotate2(self.local_vertices[iter], self.props.angle);
    V2<R> a1 = add2(r1, self.props.pos);
    V2<R> r2 = rotate2(self.local_vertices[next_iter], self.props.angle);
    V2<R> a2 = add2(r2, self.props.pos);
    V2<R> dir = normalize2(sub2(a2, a1));
    e.dir = rotate90counterclockwise(dir);
    e.has_edge = true;
    e.edge = Line<R>{a1, a2};
    return e;
}

template <class R>
void project_along_axis(const Body<R>& b, V2<R> normal, R out[2]) {
    if (b.type == DISC) {  // Disc.zig:92-97
        R middle = dot2(b.props.pos, normal);
        out[0] = middle - b.radius;
        out[1] = middle + b.radius;
        return;
    }
    // Rectangle.zig:153-169
    R best_low = std::numeric_limits<R>::infinity();
    R best_high = -std::numeric_limits<R>::infinity();
    for (uint32_t i = 0; i < b.nverts; ++i) {
        V2<R> r = rotate2(b.local_vertices[i], b.props.angle);
        V2<R> world = add2(r, b.props.pos);
        R dot = dot2(world, normal);
        if (dot < best_low) best_low = dot;
        if (dot > best_high) best_high = dot;
    }
    out[0] = best_low;
    out[1] = best_high;
}

// ---------------------------------------------------------------------------
// Contacts (src/core/collision.zig)
// ---------------------------------------------------------------------------
template <class R>
struct CollisionPoint {  // collision.zig:22-36
    R accumulated_pn = 0, accumulated_pt = 0;
    R comp_pn = 0, comp_pt = 0;  // compensation words (compensated mode, r2d_accum.h)
    V2<R> ref_r, inc_r, pos;
    R depth = 0, original_depth = 0;
    R mass_n = 0, mass_t = 0;
};

template <class R>
CollisionPoint<R> make_point(V2<R> pos, R depth, const Body<R>& ref, const Body<R>& inc,
                             V2<R> normal) {  // collision.zig:38-51
    V2<R> middle = sub2(pos, scale2(normal, depth / R(2)));
    CollisionPoint<R> p;
    p.ref_r = sub2(middle, ref.props.pos);
    p.inc_r = sub2(middle, inc.props.pos);
    p.pos = middle;
    p.depth = depth;
    p.original_depth = depth;
    return p;
}

template <class R>
struct Manifold {  // collision.zig:54-69
    V2<R> normal, tangent;
    bool has_point[2] = {false, false};
    CollisionPoint<R> points[2];
    R prev_angle_1 = 0, prev_angle_2 = 0;
    V2<R> applied_linear_p1, applied_linear_p2;
    R applied_rot_p_1 = 0, applied_rot_p_2 = 0;
    R friction = 0;
};

template <class R>
Line<R> clip_line_to_line(Line<R> a, Line<R> b) {  // collision.zig:330-363
    V2<R> delta_a = sub2(a.b, a.a);
    R a_len = length2(delta_a);
    V2<R> tang = scale2(delta_a, R(1) / a_len);
    V2<R> p1 = b.a, p2 = b.b;
    {
        R scalar = dot2(sub2(b.a, a.a), tang);
        if (!(scalar > 0 && scalar < a_len)) {
            V2<R> clos = scalar < R(0.5) * a_len ? a.a : a.b;
            V2<R> delta_p = sub2(b.a, b.b);
            R t = -dot2(tang, sub2(b.b, clos)) / dot2(tang, delta_p);
            p1 = addmult2(b.b, delta_p, t);
        }
    }
    {
        R scalar = dot2(sub2(b.b, a.a), tang);
        if (!(scalar > 0 && scalar < a_len)) {
            V2<R> clos = scalar < R(0.5) * a_len ? a.a : a.b;
            V2<R> delta_p = sub2(b.b, b.a);
            R t = -dot2(tang, sub2(b.a, clos)) / dot2(tang, delta_p);
            p2 = addmult2(b.a, delta_p, t);
        }
    }
    return Line<R>{p1, p2};
}

template <class R>
Incident<R> clip_against_edge(const Body<R>& self, Line<R> edge, V2<R> normal) {
    Incident<R> out;
    if (self.type == DISC) {  // Disc.zig:125-130
        out.point = addmult2(self.props.pos, normal, -self.radius);
        return out;
    }
    // Rectangle.zig:213-238
    Line<R> best_edge;
    bool found = false;
    R best_dot = std::numeric_limits<R>::infinity();
    V2<R> curr_world = local_to_world(self, self.local_vertices[0]);
    for (uint32_t i = 0; i < self.nverts; ++i) {
        uint32_t next_idx = i + 1 == self.nverts ? 0 : i + 1;
        V2<R> next_world = local_to_world(self, self.local_vertices[next_idx]);
        V2<R> tangent = normalize2(sub2(next_world, curr_world));
        V2<R> tentative_normal = rotate90counterclockwise(tangent);
        R dot = dot2(normal, tentative_normal);
        if (dot < best_dot) {
            best_edge = Line<R>{curr_world, next_world};
            best_dot = dot;
            found = true;
        }
        curr_world = next_world;
    }
    if (!found) {  // every dot NaN: the reference reads an undefined edge; use edge 0
        best_edge = Line<R>{local_to_world(self, self.local_vertices[0]),
                            local_to_world(self, self.local_vertices[1])};
    }
    Line<R> clipped = clip_line_to_line(edge, best_edge);
    out.is_edge = true;
    out.edge = clipped;
    return out;
}

template <class R>
bool normal_should_flip(V2<R> normal, const Body<R>& reference,
                        const Body<R>& incident) {  // collision.zig:221-226
    return dot2(normal, sub2(incident.props.pos, reference.props.pos)) < R(0);
}

// identifyCollisionPoints: Disc.zig:99-123, Rectangle.zig:171-211
template <class R>
void identify_collision_points(const Body<R>& self, const Body<R>& incident,
                               uint32_t active_normal_iter, bool has[2],
                               CollisionPoint<R> pts[2]) {
    has[0] = has[1] = false;
    if (self.type == DISC) {
        V2<R> pos = closest_point(incident, self.props.pos);
        Edge<R> edge = get_normal(self, incident, active_normal_iter);
        V2<R> normal = edge.dir;
        if (normal_should_flip(normal, self, incident)) negate_in_place(normal);
        R dot = dot2(normal, sub2(pos, self.props.pos));
        R depth = dot - self.radius;
        has[0] = true;
        pts[0] = make_point(pos, depth, self, incident, normal);
        return;
    }
    Edge<R> n = get_normal(self, incident, active_normal_iter);
    Incident<R> inc_edge = clip_against_edge(incident, n.edge, n.dir);
    if (inc_edge.is_edge) {
        V2<R> a = inc_edge.edge.a, b = inc_edge.edge.b;
        int i = 0;
        R dot = dot2(sub2(a, n.edge.a), n.dir);
        if (dot < C<R>::COLLISION_MARGIN) {
            has[i] = true;
            pts[i] = make_point(inc_edge.edge.a, dot, self, incident, n.dir);
            i += 1;
        }
        dot = dot2(sub2(b, n.edge.b), n.dir);
        if (dot < C<R>::COLLISION_MARGIN) {
            has[i] = true;
            pts[i] = make_point(inc_edge.edge.b, dot, self, incident, n.dir);
        }
    } else {
        V2<R> pos = inc_edge.point;
        R dot = dot2(sub2(pos, n.edge.a), n.dir);
        has[0] = true;
        pts[0] = make_point(pos, dot, self, incident, n.dir);
    }
}

template <class R>
struct SATResult {  // collision.zig:291-297
    bool collides = false;
    V2<R> normal;
    R penetration = 0;
    uint32_t reference_normal_id = 0;
    size_t ref = 0, inc = 0;
};

// ---------------------------------------------------------------------------
// Joints (src/core/Constraints/*.zig)
// ---------------------------------------------------------------------------
enum JointType : uint8_t {  // Constraint.zig:15-20
    DISTANCE_JOINT = 0,
    OFFSET_DISTANCE_JOINT = 1,
    FIXED_POSITION_JOINT = 2,
    MOTOR_JOINT = 3,
};

template <class R>
struct Joint {
    JointType type = DISTANCE_JOINT;
    R power_max = std::numeric_limits<R>::infinity();   // Constraint.zig:27-31
    R power_min = -std::numeric_limits<R>::infinity();
    R beta = R(10);
    uint32_t id1 = 0, id2 = 0;
    V2<R> r1, r2;            // OffsetDistanceJoint.zig:14-15
    R target_distance = 0;   // Distance / OffsetDistance
    V2<R> target_position;   // FixedPositionJoint.zig:13
    R target_omega = 0;      // MotorJoint.zig:13
};

// ---------------------------------------------------------------------------
// Solver (src/core/lib.zig:132-315)
// ---------------------------------------------------------------------------
template <class R>
class Solver {
public:
    struct Key {  // collision.zig:12-15 (pointer pair -> index pair)
        size_t ref, inc;
    };

    // Warm starting (an extension, off in reference mode): a manifold found
    // again the next frame with the same (reference, incident) pair starts
    // from last frame's accumulated impulses, which are applied to the
    // bodies once, after the first substep's preStep.  Pairs are keyed by
    // the bodies' stable ids, so the table survives changes to the body
    // store (r2o_copy_warm hands it to a rebuilt solver).
    bool warm_start = false;
    // (ref id << 32 | inc id) -> pn0, pt0, pn1, pt1, then their compensation words
    std::unordered_map<uint64_t, std::array<R, 8>> warm_prev;
    // Compensated accumulation of every point's impulses (an extension, off
    // in reference mode): r2d_accum.h.
    bool compensated = false;

    // Sleeping (an extension, off in reference mode; r2d_sleep.h): after
    // R2D_SLEEP_FRAMES consecutive still frames the world is not stepped
    // until its state is written again.
    bool sleep_enabled = false;
    uint32_t sleep_frames = 0;

    // A measurement aid: with time_phases set, step() adds each phase's wall
    // time to phase_seconds.  Off, it reads no clock.
    bool time_phases = false;
    double phase_seconds[PH_COUNT] = {};

    std::vector<Body<R>> bodies;  // insertion order
    std::unordered_map<uint32_t, size_t> index_of_id;
    std::vector<R> gravity;       // one DownwardsGravity per entry (ForceGen list)
    std::vector<Joint<R>> constraints;
    std::unordered_set<uint64_t> exclude_collision_pairs;
    std::vector<std::pair<Key, Manifold<R>>> manifolds;  // discovery order
    std::unordered_set<uint64_t> manifold_keys;
    // A checking aid: with record_pairs set, update_manifolds keeps every
    // pair that reaches performNarrowSAT (lib.zig:282-284) as (lower, higher)
    // body indices, sorted and unique.  Off, it records nothing.
    bool record_pairs = false;
    std::vector<uint64_t> candidate_pairs;
    R cell_size = R(4);        // lib.zig:255 hard-codes 4.0
    size_t table_mult = 2;     // lib.zig:255 hard-codes 2 * bodies.count()

    // colour-major replay (ORDER_COLOUR)
    std::vector<uint32_t> contact_colour, joint_colour;
    std::vector<size_t> contact_order, joint_order;

    static uint64_t pair_key(uint64_t a, uint64_t b) { return (a << 32) | b; }

    // EntityFactory.makeDiscBody (lib.zig:73-82, Disc.zig:29-56)
    size_t make_disc(uint32_t id, V2<R> pos, V2<R> vel, R angle, R omega, R mu,
                     bool by_density, R mass_prop, R radius) {
        R mass = by_density ? R(3.14159265358979323846) * radius * radius * mass_prop : mass_prop;
        Body<R> b;
        b.id = id;
        b.type = DISC;
        b.num_normals = 1;
        b.radius = radius;
        b.props.pos = pos;
        b.props.angle = angle;
        b.props.mass = mass;
        b.props.inertia = R(0.5) * mass * radius * radius;
        b.props.mu = mu;
        update_aabb(b);
        b.props.momentum = scale2(vel, mass);
        b.props.ang_momentum = omega * b.props.inertia;
        return append(b);
    }

    // EntityFactory.makeRectangleBody (lib.zig:84-93, Rectangle.zig:33-64)
    size_t make_rectangle(uint32_t id, V2<R> pos, V2<R> vel, R angle, R omega, R mu,
                          bool by_density, R mass_prop, R width, R height) {
        R mass = by_density ? width * height * mass_prop : mass_prop;
        Body<R> b;
        b.id = id;
        b.type = RECTANGLE;
        b.num_normals = 4;
        b.width = width;
        b.height = height;
        R w = width / R(2), h = height / R(2);
        b.local_vertices[0] = {-w, -h};
        b.local_vertices[1] = {-w, h};
        b.local_vertices[2] = {w, h};
        b.local_vertices[3] = {w, -h};
        b.props.pos = pos;
        b.props.angle = angle;
        b.props.mass = mass;
        b.props.inertia = mass * (width * width + height * height) / R(12);
        b.props.mu = mu;
        update_aabb(b);
        b.props.momentum = scale2(vel, mass);
        b.props.ang_momentum = omega * b.props.inertia;
        return append(b);
    }

    // A convex polygon (no counterpart in the reference; its roadmap's next
    // shape): `nverts` local vertices (x, y pairs, clockwise about the body's
    // origin, as the rectangle's), with its mass and inertia given (the
    // caller integrates them over its shape); d0, d1 are kept as its dims.
    size_t make_polygon(uint32_t id, V2<R> pos, V2<R> vel, R angle, R omega, R mu, R mass, R inertia,
                        uint32_t nverts, const float* verts, R d0, R d1) {
        Body<R> b;
        b.id = id;
        b.type = POLYGON;
        b.nverts = nverts;
        b.num_normals = nverts;
        b.width = d0;
        b.height = d1;
        for (uint32_t k = 0; k < nverts; ++k) b.local_vertices[k] = {R(verts[2 * k]), R(verts[2 * k + 1])};
        b.props.pos = pos;
        b.props.angle = angle;
        b.props.mass = mass;
        b.props.inertia = inertia;
        b.props.mu = mu;
        update_aabb(b);
        b.props.momentum = scale2(vel, mass);
        b.props.ang_momentum = omega * inertia;
        return append(b);
    }

    size_t append(const Body<R>& b) {  // lib.zig:66-71
        index_of_id[b.id] = bodies.size();
        bodies.push_back(b);
        return bodies.size() - 1;
    }

    void exclude_pair(uint32_t id1, uint32_t id2) {  // lib.zig:124-129
        exclude_collision_pairs.insert(pair_key(id1, id2));
        exclude_collision_pairs.insert(pair_key(id2, id1));
    }

    // ---- SAT (collision.zig:228-320) ----
    bool overlap_sat(SATResult<R>& ret, size_t ri, size_t ii) const {
        const R EPS = C<R>::SAT_OVERLAP_THRESHOLD;
        const Body<R>& reference = bodies[ri];
        const Body<R>& incident = bodies[ii];
        for (uint32_t it = 0; it < reference.num_normals; ++it) {
            Edge<R> edge = get_normal(reference, incident, it);
            V2<R> normal = edge.dir;
            bool flipped = false;
            if (normal_should_flip(normal, reference, incident)) {
                negate_in_place(normal);
                flipped = true;
            }
            R p1[2], p2[2];
            project_along_axis(reference, normal, p1);
            project_along_axis(incident, normal, p2);
            R d1 = p1[1] - p2[0];
            R d2 = p2[1] - p1[0];
            R d = zmin(d1, d2);
            if (d <= -C<R>::COLLISION_MARGIN) return false;

            if (!flipped && approx_eql2(normal, ret.normal, EPS)) {
                R tref = dot2(reference.props.pos, normal);
                R tinc = dot2(incident.props.pos, normal);
                if (tref < tinc - EPS) {
                    ret.penetration = d;
                    ret.normal = normal;
                    ret.reference_normal_id = it;
                    ret.ref = ri;
                    ret.inc = ii;
                }
            }
            if (!flipped && approx_eql2(normal, negate2(ret.normal), EPS)) {
                V2<R> diff = sub2(incident.props.pos, reference.props.pos);
                if (dot2(diff, normal) > dot2(diff, ret.normal) + EPS) {
                    ret.penetration = d;
                    ret.normal = normal;
                    ret.reference_normal_id = it;
                    ret.ref = ri;
                    ret.inc = ii;
                }
            }
            if (d + EPS < ret.penetration) {
                ret.penetration = d;
                ret.normal = normal;
                ret.reference_normal_id = it;
                ret.ref = ri;
                ret.inc = ii;
            }
        }
        return true;
    }

    SATResult<R> perform_narrow_sat(size_t b1, size_t b2) const {  // collision.zig:299-320
        SATResult<R> ret;
        ret.collides = false;
        ret.penetration = std::numeric_limits<R>::infinity();
        size_t o1 = bodies[b1].id < bodies[b2].id ? b1 : b2;
        size_t o2 = o1 == b1 ? b2 : b1;
        ret.ref = o1;
        ret.inc = o2;
        if (!overlap_sat(ret, o1, o2)) return ret;
        if (!overlap_sat(ret, o2, o1)) return ret;
        ret.collides = true;
        return ret;
    }

    // ---- spatial hash (SpatialHash.zig) ----
    static size_t hash_cell(size_t table_size, int64_t xi, int64_t yi) {  // :78-81
        uint64_t h = ((uint64_t)xi * 92837111ull) ^ ((uint64_t)yi * 689287499ull);
        return (size_t)(h % (uint64_t)table_size);
    }

    bool cell_range(const AABB<R>& a, int64_t out[4]) const {  // :83-96
        V2<R> mn = a.vertex_min(), mx = a.vertex_max();
        R v[4] = {std::floor(mn.x / cell_size), std::floor(mn.y / cell_size),
                  std::floor(mx.x / cell_size), std::floor(mx.y / cell_size)};
        for (int i = 0; i < 4; ++i) {
            if (!(v[i] > R(-9.0e18) && v[i] < R(9.0e18))) return false;
            out[i] = (int64_t)v[i];
        }
        return true;
    }

    int update_manifolds() {  // lib.zig:253-299
        const size_t n = bodies.size();
        const size_t table_size = table_mult * n;
        manifolds.clear();
        manifold_keys.clear();
        contact_colour.clear();
        contact_order.clear();
        candidate_pairs.clear();
        if (n == 0) return OK;

        // SpatialHash.init (SpatialHash.zig:19-71)
        std::vector<size_t> table(table_size + 1, 0);
        std::vector<std::array<int64_t, 4>> ranges(n);
        int64_t total_cells = 0;
        for (size_t b = 0; b < n; ++b) {
            int64_t r[4];
            if (!cell_range(bodies[b].aabb, r)) return ERR_NONFINITE_AABB;
            std::copy(r, r + 4, ranges[b].begin());
            if (r[2] >= r[0] && r[3] >= r[1]) {
                const double c = (double(r[2]) - double(r[0]) + 1.0) * (double(r[3]) - double(r[1]) + 1.0);
                if (c > double(MAX_CELLS)) return ERR_CAPACITY;
                total_cells += (int64_t)c;
                if (total_cells > MAX_CELLS) return ERR_CAPACITY;
            }
            for (int64_t yi = r[1]; yi <= r[3]; ++yi)
                for (int64_t xi = r[0]; xi <= r[2]; ++xi) table[hash_cell(table_size, xi, yi)] += 1;
        }
        size_t start = 0;
        for (size_t id = 0; id < table_size; ++id) {
            start += table[id];
            table[id] = start;
        }
        table[table_size] = start;
        std::vector<size_t> body_indices(start);
        for (size_t b = 0; b < n; ++b) {
            const auto& r = ranges[b];
            for (int64_t yi = r[1]; yi <= r[3]; ++yi)
                for (int64_t xi = r[0]; xi <= r[2]; ++xi) {
                    size_t& val = table[hash_cell(table_size, xi, yi)];
                    val -= 1;
                    body_indices[val] = b;
                }
        }

        std::vector<size_t> queries;
        for (size_t b1 = 0; b1 < n; ++b1) {
            queries.clear();
            const auto& r = ranges[b1];  // SpatialHash.query (:108-137)
            for (int64_t yi = r[1]; yi <= r[3]; ++yi)
                for (int64_t xi = r[0]; xi <= r[2]; ++xi) {
                    size_t id = hash_cell(table_size, xi, yi);
                    for (size_t idx = table[id]; idx < table[id + 1]; ++idx)
                        queries.push_back(body_indices[idx]);
                }
            const Body<R>& body1 = bodies[b1];
            for (size_t b2 : queries) {
                const Body<R>& body2 = bodies[b2];
                if (body1.is_static && body2.is_static) continue;
                if (b1 == b2) continue;
                if (exclude_collision_pairs.count(pair_key(body1.id, body2.id))) continue;
                if (exclude_collision_pairs.count(pair_key(body2.id, body1.id))) continue;
                if (manifold_keys.count(pair_key(b1, b2))) continue;
                if (manifold_keys.count(pair_key(b2, b1))) continue;
                if (!body1.aabb.intersects(body2.aabb)) continue;
                if (record_pairs) candidate_pairs.push_back(pair_key(std::min(b1, b2), std::max(b1, b2)));
                SATResult<R> sat = perform_narrow_sat(b1, b2);
                if (!sat.collides) continue;
                Manifold<R> m;
                m.normal = sat.normal;
                identify_collision_points(bodies[sat.ref], bodies[sat.inc], sat.reference_normal_id,
                                          m.has_point, m.points);
                m.prev_angle_1 = bodies[sat.ref].props.angle;
                m.prev_angle_2 = bodies[sat.inc].props.angle;
                manifolds.push_back({Key{sat.ref, sat.inc}, m});
                manifold_keys.insert(pair_key(sat.ref, sat.inc));
            }
        }
        if (record_pairs) {
            std::sort(candidate_pairs.begin(), candidate_pairs.end());
            candidate_pairs.erase(std::unique(candidate_pairs.begin(), candidate_pairs.end()), candidate_pairs.end());
        }
        return OK;
    }

    // ---- manifold per-substep work (collision.zig:73-218) ----
    void update_tgs_depth(Manifold<R>& m, const Key& k) {  // :73-100
        const Body<R>& b1 = bodies[k.ref];
        const Body<R>& b2 = bodies[k.inc];
        for (int i = 0; i < 2; ++i) {
            if (!m.has_point[i]) continue;
            CollisionPoint<R>& point = m.points[i];
            if (approx_eql(point.depth, point.original_depth, R(1e-4))) continue;
            V2<R> r_rot_1 = rotate2(point.ref_r, b1.props.angle - m.prev_angle_1);
            V2<R> r_rot_2 = rotate2(point.inc_r, b2.props.angle - m.prev_angle_2);
            V2<R> a1 = add2(r_rot_1, b1.props.pos);
            V2<R> a2 = add2(r_rot_2, b2.props.pos);
            R depth = dot2(m.normal, sub2(a2, a1));
            point.depth = depth + point.original_depth;
            point.ref_r = r_rot_1;
            point.inc_r = r_rot_2;
        }
        m.prev_angle_1 = b1.props.angle;
        m.prev_angle_2 = b2.props.angle;
    }

    void pre_step(Manifold<R>& m, const Key& k) {  // :102-133
        const Body<R>& b1 = bodies[k.ref];
        const Body<R>& b2 = bodies[k.inc];
        R inv_m1 = b1.is_static ? R(0) : R(1) / b1.props.mass;
        R inv_m2 = b2.is_static ? R(0) : R(1) / b2.props.mass;
        R inv_mass = inv_m1 + inv_m2;
        R inv_i1 = b1.is_static ? R(0) : R(1) / b1.props.inertia;
        R inv_i2 = b2.is_static ? R(0) : R(1) / b2.props.inertia;
        m.tangent = rotate90clockwise(m.normal);
        m.friction = std::sqrt(b1.props.mu * b2.props.mu);
        for (int i = 0; i < 2; ++i) {
            if (!m.has_point[i]) continue;
            CollisionPoint<R>& point = m.points[i];
            V2<R> r1 = point.ref_r, r2 = point.inc_r;
            R r1n = cross2(r1, m.normal);
            R r2n = cross2(r2, m.normal);
            R kn = inv_mass + inv_i1 * (r1n * r1n) + inv_i2 * (r2n * r2n);
            R r1t = cross2(r1, m.tangent);
            R r2t = cross2(r2, m.tangent);
            R kt = inv_mass + inv_i1 * (r1t * r1t) + inv_i2 * (r2t * r2t);
            point.mass_n = kn > R(0) ? R(1) / kn : R(0);
            point.mass_t = kt > R(0) ? R(1) / kt : R(0);
        }
    }

    void calculate_impulses(Manifold<R>& m, const Key& k, R dt) {  // :135-218
        Body<R>& b1 = bodies[k.ref];
        Body<R>& b2 = bodies[k.inc];
        R inv_m1 = b1.is_static ? R(0) : R(1) / b1.props.mass;
        R inv_m2 = b2.is_static ? R(0) : R(1) / b2.props.mass;
        R inv_i1 = b1.is_static ? R(0) : R(1) / b1.props.inertia;
        R inv_i2 = b2.is_static ? R(0) : R(1) / b2.props.inertia;
        V2<R> vlinear_1 = scale2(b1.props.momentum, inv_m1);
        R omega1 = b1.props.ang_momentum * inv_i1;
        V2<R> vlinear_2 = scale2(b2.props.momentum, inv_m2);
        R omega2 = b2.props.ang_momentum * inv_i2;
        for (int i = 0; i < 2; ++i) {
            if (!m.has_point[i]) continue;
            CollisionPoint<R>& point = m.points[i];
            if (point.depth >= R(0)) {
                point.accumulated_pn = 0;
                point.accumulated_pt = 0;
                point.comp_pn = 0;
                point.comp_pt = 0;
                continue;
            }
            V2<R> r1 = point.ref_r, r2 = point.inc_r;
            V2<R> vrot_1{-r1.y * omega1, r1.x * omega1};
            V2<R> v1 = add2(vlinear_1, vrot_1);
            V2<R> vrot_2{-r2.y * omega2, r2.x * omega2};
            V2<R> v2 = add2(vlinear_2, vrot_2);
            V2<R> dv = sub2(v1, v2);
            R bias = C<R>::BAUMGARTE *
                     zmax(R(0), (-point.depth) - C<R>::BAUMGARTE_SLOP) / dt;
            R num = dot2(dv, m.normal) + bias;
            R pn = num * point.mass_n;
            // The reference skips small or negative impulses, so an
            // accumulated impulse never decreases; a warm-started one must be
            // able to, so warm starting clamps the sum instead (below).
            if (!warm_start && pn < C<R>::MIN_MANIFOLD_IMPULSE) continue;
            num = dot2(dv, m.tangent);
            R pt = num * point.mass_t;
            R applied_pn, applied_pt;
            if (compensated) {  // r2d_accum.h: the same clamps on s + c
                applied_pn = r2d_acc_add_max(&point.accumulated_pn, &point.comp_pn, pn, R(0));
                R max_pt = m.friction * std::fabs(point.accumulated_pn);
                applied_pt = r2d_acc_add_clamp(&point.accumulated_pt, &point.comp_pt, pt, -max_pt, max_pt);
            } else {
                R new_accumulated_pn = zmax(R(0), point.accumulated_pn + pn);
                applied_pn = new_accumulated_pn - point.accumulated_pn;
                point.accumulated_pn = new_accumulated_pn;
                R max_pt = m.friction * std::fabs(point.accumulated_pn);
                R new_accumulated_pt = zclamp(point.accumulated_pt + pt, -max_pt, max_pt);
                applied_pt = new_accumulated_pt - point.accumulated_pt;
                point.accumulated_pt = new_accumulated_pt;
            }
            V2<R> pn_vec = scale2(m.normal, applied_pn);
            V2<R> pt_vec = scale2(m.tangent, applied_pt);
            V2<R> dp = add2(pn_vec, pt_vec);
            if (!b1.is_static) {
                m.applied_linear_p1 = sub2(m.applied_linear_p1, dp);
                m.applied_rot_p_1 -= cross2(r1, dp);
            }
            if (!b2.is_static) {
                m.applied_linear_p2 = add2(m.applied_linear_p2, dp);
                m.applied_rot_p_2 += cross2(r2, dp);
            }
        }
        b1.props.momentum = add2(b1.props.momentum, m.applied_linear_p1);
        b1.props.ang_momentum += m.applied_rot_p_1;
        b2.props.momentum = add2(b2.props.momentum, m.applied_linear_p2);
        b2.props.ang_momentum += m.applied_rot_p_2;
        m.applied_linear_p1 = V2<R>{};
        m.applied_rot_p_1 = 0;
        m.applied_linear_p2 = V2<R>{};
        m.applied_rot_p_2 = 0;
    }

    // ---- warm starting ----
    uint64_t warm_key(const Key& k) const {
        return ((uint64_t)bodies[k.ref].id << 32) | (uint64_t)bodies[k.inc].id;
    }

    void warm_load() {
        for (auto& km : manifolds) {
            auto it = warm_prev.find(warm_key(km.first));
            if (it == warm_prev.end()) continue;
            for (int i = 0; i < 2; ++i) {
                if (!km.second.has_point[i]) continue;
                km.second.points[i].accumulated_pn = it->second[2 * i];
                km.second.points[i].accumulated_pt = it->second[2 * i + 1];
                km.second.points[i].comp_pn = it->second[4 + 2 * i];
                km.second.points[i].comp_pt = it->second[4 + 2 * i + 1];
            }
        }
    }

    // Applies a manifold's accumulated impulses, summed like calculateImpulses
    // sums its applied ones; a point with depth >= 0 starts from zero.
    void warm_apply(Manifold<R>& m, const Key& k) {
        Body<R>& b1 = bodies[k.ref];
        Body<R>& b2 = bodies[k.inc];
        V2<R> alp1{}, alp2{};
        R arp1 = 0, arp2 = 0;
        for (int i = 0; i < 2; ++i) {
            if (!m.has_point[i]) continue;
            CollisionPoint<R>& point = m.points[i];
            if (point.depth >= R(0)) {
                point.accumulated_pn = 0;
                point.accumulated_pt = 0;
                point.comp_pn = 0;
                point.comp_pt = 0;
                continue;
            }
            V2<R> dp = add2(scale2(m.normal, point.accumulated_pn), scale2(m.tangent, point.accumulated_pt));
            if (!b1.is_static) {
                alp1 = sub2(alp1, dp);
                arp1 -= cross2(point.ref_r, dp);
            }
            if (!b2.is_static) {
                alp2 = add2(alp2, dp);
                arp2 += cross2(point.inc_r, dp);
            }
        }
        if (!b1.is_static) {
            b1.props.momentum = add2(b1.props.momentum, alp1);
            b1.props.ang_momentum += arp1;
        }
        if (!b2.is_static) {
            b2.props.momentum = add2(b2.props.momentum, alp2);
            b2.props.ang_momentum += arp2;
        }
    }

    void warm_store() {
        warm_prev.clear();
        for (auto& km : manifolds) {
            std::array<R, 8> a{};
            for (int i = 0; i < 2; ++i) {
                if (!km.second.has_point[i]) continue;
                a[2 * i] = km.second.points[i].accumulated_pn;
                a[2 * i + 1] = km.second.points[i].accumulated_pt;
                a[4 + 2 * i] = km.second.points[i].comp_pn;
                a[4 + 2 * i + 1] = km.second.points[i].comp_pt;
            }
            warm_prev[warm_key(km.first)] = a;
        }
    }

    // ---- joint solves ----
    int lookup(uint32_t id, size_t* out) const {
        auto it = index_of_id.find(id);
        if (it == index_of_id.end()) return ERR_INVALID_BODY_ID;
        *out = it->second;
        return OK;
    }

    int solve_joint(Joint<R>& j, R dt) {
        switch (j.type) {
        case DISTANCE_JOINT: {  // DistanceJoint.zig:40-75
            const R epsilon = C<R>::CONSTRAINT_GRADIENT_DIVISION_LIMIT;
            size_t i1, i2;
            if (lookup(j.id1, &i1) || lookup(j.id2, &i2)) return ERR_INVALID_BODY_ID;
            Body<R>& b1 = bodies[i1];
            Body<R>& b2 = bodies[i2];
            R w1 = b1.is_static ? R(0) : R(1) / b1.props.mass;
            R w2 = b2.is_static ? R(0) : R(1) / b2.props.mass;
            V2<R> v1 = scale2(b1.props.momentum, w1);
            V2<R> v2 = scale2(b2.props.momentum, w2);
            V2<R> relative_v = sub2(v2, v1);
            V2<R> normal = normalize2(sub2(b2.props.pos, b1.props.pos));
            R dist_error = length2(sub2(b2.props.pos, b1.props.pos)) - j.target_distance;
            R position_correction = j.beta * dist_error / zmax(j.target_distance, R(0.001));
            R J = -(dot2(relative_v, normal) + position_correction) / (w1 + w2);
            R ndv = dot2(normal, relative_v);
            R den = R(1) / zmax(std::fabs(ndv), epsilon);
            R J_max = j.power_max * den;
            R J_min = j.power_min * den;
            J = zclamp(J, J_min, J_max);
            V2<R> dp = scale2(normal, J);
            b1.props.momentum = sub2(b1.props.momentum, dp);
            b2.props.momentum = add2(b2.props.momentum, dp);
            return OK;
        }
        case OFFSET_DISTANCE_JOINT: {  // OffsetDistanceJoint.zig:44-105
            const R epsilon = C<R>::CONSTRAINT_GRADIENT_DIVISION_LIMIT;
            size_t i1, i2;
            if (lookup(j.id1, &i1) || lookup(j.id2, &i2)) return ERR_INVALID_BODY_ID;
            Body<R>& b1 = bodies[i1];
            Body<R>& b2 = bodies[i2];
            V2<R> a1 = local_to_world(b1, j.r1);
            V2<R> a2 = local_to_world(b2, j.r2);
            V2<R> normal = normalize2(sub2(a2, a1));
            R inv_m1 = b1.is_static ? R(0) : R(1) / b1.props.mass;
            R inv_m2 = b2.is_static ? R(0) : R(1) / b2.props.mass;
            R inv_i1 = b1.is_static ? R(0) : R(1) / b1.props.inertia;
            R inv_i2 = b2.is_static ? R(0) : R(1) / b2.props.inertia;
            V2<R> vlinear_1 = scale2(b1.props.momentum, inv_m1);
            R omega1 = b1.props.ang_momentum * inv_i1;
            V2<R> vlinear_2 = scale2(b2.props.momentum, inv_m2);
            R omega2 = b2.props.ang_momentum * inv_i2;
            V2<R> rotated_r1 = rotate2(j.r1, b1.props.angle);
            V2<R> v_at_a1{-rotated_r1.y * omega1, rotated_r1.x * omega1};
            V2<R> v1 = add2(vlinear_1, v_at_a1);
            V2<R> rotated_r2 = rotate2(j.r2, b2.props.angle);
            V2<R> v_at_a2{-rotated_r2.y * omega2, rotated_r2.x * omega2};
            V2<R> v2 = add2(vlinear_2, v_at_a2);
            V2<R> dv = sub2(v2, v1);
            R dist_error = length2(sub2(a2, a1)) - j.target_distance;
            R position_correction = j.beta * dist_error / zmax(j.target_distance, epsilon);
            R num = dot2(normal, dv) + position_correction;
            R r1xn = cross2(rotated_r1, normal);
            R r2xn = cross2(rotated_r2, normal);
            R den = inv_m1 + inv_m2 + r1xn * r1xn * inv_i1 + r2xn * r2xn * inv_i2;
            R J = -num / den;
            R ndv = dot2(normal, dv);
            R den2 = R(1) / zmax(std::fabs(ndv), epsilon);
            R J_max = j.power_max * den2;
            R J_min = j.power_min * den2;
            J = zclamp(J, J_min, J_max);
            V2<R> dp = scale2(normal, J);
            b1.props.momentum = sub2(b1.props.momentum, dp);
            b1.props.ang_momentum -= J * r1xn;
            b2.props.momentum = add2(b2.props.momentum, dp);
            b2.props.ang_momentum += J * r2xn;
            return OK;
        }
        case FIXED_POSITION_JOINT: {  // FixedPositionJoint.zig:38-72
            const R epsilon = C<R>::ALLOWED_CONSTRAINT_VALUE;
            size_t i1;
            if (lookup(j.id1, &i1)) return ERR_INVALID_BODY_ID;
            Body<R>& b = bodies[i1];
            if (b.is_static) return OK;
            R w = R(1) / b.props.mass;
            V2<R> v = scale2(b.props.momentum, w);
            V2<R> delta_pos = sub2(j.target_position, b.props.pos);
            R dist = length2(delta_pos);
            if (dist < C<R>::ALLOWED_CONSTRAINT_VALUE) return OK;
            V2<R> normal = scale2(delta_pos, R(1) / dist);
            R bias = j.beta * dist;
            R relative_velocity = dot2(v, normal);
            R J = -(relative_velocity - bias) / w;
            R den = R(1) / zmax(std::fabs(relative_velocity), epsilon);
            R J_max = j.power_max * den;
            R J_min = j.power_min * den;
            J = zclamp(J, J_min, J_max);
            V2<R> dp = scale2(normal, J);
            b.props.momentum = add2(b.props.momentum, dp);
            return OK;
        }
        case MOTOR_JOINT: {  // MotorJoint.zig:38-64
            const R epsilon = C<R>::ALLOWED_CONSTRAINT_VALUE;
            size_t i1;
            if (lookup(j.id1, &i1)) return ERR_INVALID_BODY_ID;
            Body<R>& b = bodies[i1];
            if (b.is_static) return OK;
            R omega = b.props.ang_momentum / b.props.inertia;
            R Cv = omega - j.target_omega;
            if (std::fabs(Cv) < C<R>::ALLOWED_CONSTRAINT_VALUE) return OK;
            R bias = j.beta * Cv;
            R J = b.props.torque - bias;
            R relative_velocity = b.props.torque / b.props.inertia;
            R den = R(1) / zmax(std::fabs(relative_velocity), epsilon);
            R J_max = j.power_max * den;
            R J_min = j.power_min * den;
            J = zclamp(J, J_min, J_max);
            b.props.ang_momentum += J * dt;
            return OK;
        }
        }
        return OK;
    }

    // ---- colour-major replay order (r2d_colour.h) ----
    // First-fit greedy colouring in ascending (mix(key), key) order.
    static uint32_t first_fit(const std::vector<uint32_t>& used_a, const std::vector<uint32_t>* used_b) {
        for (uint32_t c = 0;; ++c) {
            bool taken = std::find(used_a.begin(), used_a.end(), c) != used_a.end();
            if (!taken && used_b)
                taken = std::find(used_b->begin(), used_b->end(), c) != used_b->end();
            if (!taken) return c;
        }
    }

    int compute_colouring() {
        const size_t n = bodies.size();
        // contacts
        struct P {
            uint32_t h, lo, hi;
            size_t m;
        };
        std::vector<P> pr(manifolds.size());
        for (size_t m = 0; m < manifolds.size(); ++m) {
            uint32_t a = (uint32_t)manifolds[m].first.ref, b = (uint32_t)manifolds[m].first.inc;
            uint32_t lo = std::min(a, b), hi = std::max(a, b);
            pr[m] = P{r2d_colour_mix(lo, hi), lo, hi, m};
        }
        std::sort(pr.begin(), pr.end(), [](const P& x, const P& y) {
            if (x.h != y.h) return x.h < y.h;
            if (x.lo != y.lo) return x.lo < y.lo;
            return x.hi < y.hi;
        });
        std::vector<std::vector<uint32_t>> used(n);
        contact_colour.assign(manifolds.size(), 0);
        static const std::vector<uint32_t> none;
        for (const P& p : pr) {
            bool dyn_lo = !bodies[p.lo].is_static, dyn_hi = !bodies[p.hi].is_static;
            const std::vector<uint32_t>& ua = dyn_lo ? used[p.lo] : none;
            const std::vector<uint32_t>* ub = dyn_hi ? &used[p.hi] : nullptr;
            uint32_t c = first_fit(ua, ub);
            contact_colour[p.m] = c;
            if (dyn_lo) used[p.lo].push_back(c);
            if (dyn_hi) used[p.hi].push_back(c);
        }
        // joints: every named body is a conflict node
        struct Q {
            uint32_t h;
            size_t j;
        };
        std::vector<Q> jq(constraints.size());
        for (size_t j = 0; j < constraints.size(); ++j)
            jq[j] = Q{r2d_colour_mix((uint32_t)j, R2D_COLOUR_JOINT_SALT), j};
        std::sort(jq.begin(), jq.end(), [](const Q& x, const Q& y) {
            if (x.h != y.h) return x.h < y.h;
            return x.j < y.j;
        });
        for (auto& u : used) u.clear();
        joint_colour.assign(constraints.size(), 0);
        for (const Q& q : jq) {
            const Joint<R>& jt = constraints[q.j];
            size_t i1 = 0, i2 = 0;
            if (lookup(jt.id1, &i1)) return ERR_INVALID_BODY_ID;
            bool two = jt.type == DISTANCE_JOINT || jt.type == OFFSET_DISTANCE_JOINT;
            if (two && lookup(jt.id2, &i2)) return ERR_INVALID_BODY_ID;
            if (two && i2 == i1) two = false;
            uint32_t c = first_fit(used[i1], two ? &used[i2] : nullptr);
            joint_colour[q.j] = c;
            used[i1].push_back(c);
            if (two) used[i2].push_back(c);
        }
        // colour-major orders (insertion / discovery order inside a colour)
        auto make_order = [](const std::vector<uint32_t>& col, std::vector<size_t>& order) {
            order.resize(col.size());
            for (size_t i = 0; i < col.size(); ++i) order[i] = i;
            std::stable_sort(order.begin(), order.end(),
                             [&](size_t x, size_t y) { return col[x] < col[y]; });
        };
        make_order(contact_colour, contact_order);
        make_order(joint_colour, joint_order);
        return OK;
    }

    // ---- Solver.process (lib.zig:189-251) ----
    int process(R dt, size_t sub_steps, size_t collision_iters, int order = ORDER_REFERENCE) {
        if (sleep_enabled && sleep_frames >= R2D_SLEEP_FRAMES) return OK;  // asleep: nothing moves
        const int st = step(dt, sub_steps, collision_iters, order);
        if (st == OK && sleep_enabled) {
            bool still = true;
            for (const Body<R>& b : bodies) {
                if (b.is_static) continue;
                const float inv_m = 1.0f / float(b.props.mass), inv_i = 1.0f / float(b.props.inertia);
                still = still && r2d_body_still(float(b.props.momentum.x), float(b.props.momentum.y),
                                                float(b.props.ang_momentum), inv_m, inv_i);
            }
            sleep_frames = r2d_sleep_next(sleep_frames, still);
        }
        return st;
    }

    int step(R dt, size_t sub_steps, size_t collision_iters, int order) {
        const R f32_sub = R(sub_steps);
        const R sub_dt = dt / f32_sub;
        using clock = std::chrono::steady_clock;
        clock::time_point t_mark = time_phases ? clock::now() : clock::time_point{};
        auto mark = [&](int phase) {  // charge the time since the last mark to `phase`
            if (!time_phases) return;
            const clock::time_point now = clock::now();
            phase_seconds[phase] += std::chrono::duration<double>(now - t_mark).count();
            t_mark = now;
        };

        // joints resolve their ids on every solve in the reference; validate
        // once up front so that an invalid id leaves the state untouched.
        for (const Joint<R>& j : constraints) {
            size_t t;
            if (lookup(j.id1, &t)) return ERR_INVALID_BODY_ID;
            bool two = j.type == DISTANCE_JOINT || j.type == OFFSET_DISTANCE_JOINT;
            if (two && lookup(j.id2, &t)) return ERR_INVALID_BODY_ID;
        }

        int st = update_manifolds();
        if (st != OK) return st;
        mark(PH_MANIFOLDS);
        if (order == ORDER_COLOUR) {
            st = compute_colouring();
            if (st != OK) return st;
        }
        if (warm_start) warm_load();
        mark(PH_COLOURING);

        for (size_t s = 0; s < sub_steps; ++s) {
            for (R g : gravity) {  // DownwardsGravity.apply (DownwardsGravity.zig:35-39)
                V2<R> g_vec{R(0), -g};
                for (Body<R>& b : bodies) {
                    if (b.is_static) continue;
                    b.props.force.x += g_vec.x * b.props.mass;
                    b.props.force.y += g_vec.y * b.props.mass;
                }
            }
            for (Body<R>& b : bodies) {  // lib.zig:207-216
                update_aabb(b);
                if (b.is_static) continue;
                b.props.momentum.x += b.props.force.x * sub_dt;
                b.props.momentum.y += b.props.force.y * sub_dt;
                b.props.ang_momentum += b.props.torque * sub_dt;
            }
            mark(PH_FORCES);
            for (auto& km : manifolds) {  // lib.zig:218-224
                update_tgs_depth(km.second, km.first);
                pre_step(km.second, km.first);
            }
            mark(PH_PRESTEP);
            if (warm_start && s == 0) {
                if (order == ORDER_COLOUR) {
                    for (size_t m : contact_order) warm_apply(manifolds[m].second, manifolds[m].first);
                } else {
                    for (auto& km : manifolds) warm_apply(km.second, km.first);
                }
            }
            for (size_t it = 0; it < collision_iters; ++it) {  // lib.zig:226-236
                if (order == ORDER_COLOUR) {
                    for (size_t j : joint_order) {
                        st = solve_joint(constraints[j], sub_dt);
                        if (st != OK) return st;
                    }
                    for (size_t m : contact_order)
                        calculate_impulses(manifolds[m].second, manifolds[m].first, sub_dt);
                } else {
                    for (Joint<R>& j : constraints) {
                        st = solve_joint(j, sub_dt);
                        if (st != OK) return st;
                    }
                    for (auto& km : manifolds) calculate_impulses(km.second, km.first, sub_dt);
                }
            }
            mark(PH_SOLVE);
            for (Body<R>& b : bodies) {  // lib.zig:238-249
                if (b.is_static) continue;
                R sm = sub_dt / b.props.mass;
                b.props.pos.x += b.props.momentum.x * sm;
                b.props.pos.y += b.props.momentum.y * sm;
                b.props.angle += b.props.ang_momentum * sub_dt / b.props.inertia;
                b.props.force = V2<R>{};
                b.props.torque = 0;
            }
            mark(PH_INTEGRATE);
        }
        if (warm_start) warm_store();
        mark(PH_INTEGRATE);
        return OK;
    }
};

}  // namespace r2o
