/*
 * oracle_capi.cpp -- C entry points of the CPU oracle (r2d_oracle.hpp) for
 * the Python test harness and the benchmark's CPU arms.
 *
 * TEST INFRASTRUCTURE: loaded only by tests/, __graft_entry__.smoke() and
 * bench.py (cpu_baseline / --impl reference).  Never linked into the product.
 *
 * Array layouts match the product C-ABI (include/r2d_gb300.h) so that a test
 * hands the same numpy buffers to both sides:
 *   body options  float[10][n]: pos_x pos_y angle vel_x vel_y omega mu
 *                               mass_prop dim0 dim1 (EntityFactory.BodyOptions,
 *                               src/core/lib.zig:35-60)
 *   kind          u8[n]: bit0 rectangle, bit1 static, bit2 mass_prop is a density
 *   state         float[13][n]: pos_x pos_y angle mom_x mom_y ang_mom force_x
 *                               force_y torque aabb_x aabb_y aabb_hw aabb_hh
 *   props         float[5][n]:  mass inertia mu dim0 dim1
 *   joint params  float[8] per joint: power_max power_min beta p0..p4
 */
#include <atomic>
#include <chrono>
#include <iterator>
#include <cstring>
#include <memory>
#include <thread>

#include "r2d_oracle.hpp"

using namespace r2o;

namespace {

enum { NOPT = 10, NSTATE = 13, NPROP = 5, NJP = 8, MF = 33 };

struct Handle {
    int precision;
    std::unique_ptr<Solver<float>> f;
    std::unique_ptr<Solver<double>> d;
};

// kind bits: 1 rectangle, 2 static, 4 mass by density, 8 polygon (mass
// MASS_PROP, inertia DIM1, vertices nverts[i] pairs at verts[i][MAX_POLY_VERTS][2]).
template <class R>
void add_bodies(Solver<R>& s, uint32_t n, const uint32_t* ids, const uint8_t* kind,
                const float* opt, const uint8_t* nverts = nullptr, const float* verts = nullptr) {
    for (uint32_t i = 0; i < n; ++i) {
        auto o = [&](int f) { return R(opt[(size_t)f * n + i]); };
        V2<R> pos{o(0), o(1)}, vel{o(3), o(4)};
        bool by_density = (kind[i] & 4) != 0;
        size_t idx;
        if ((kind[i] & 8) && nverts && verts)
            idx = s.make_polygon(ids[i], pos, vel, o(2), o(5), o(6), o(7), o(9), nverts[i],
                                 verts + (size_t)i * 2 * MAX_POLY_VERTS, o(8), o(9));
        else if (kind[i] & 1)
            idx = s.make_rectangle(ids[i], pos, vel, o(2), o(5), o(6), by_density, o(7), o(8), o(9));
        else
            idx = s.make_disc(ids[i], pos, vel, o(2), o(5), o(6), by_density, o(7), o(8));
        if (kind[i] & 2) s.bodies[idx].is_static = true;  // body_unwrap().static = true
    }
}

template <class R, class T>
void get_state(const Solver<R>& s, T* out) {
    const size_t n = s.bodies.size();
    for (size_t i = 0; i < n; ++i) {
        const Body<R>& b = s.bodies[i];
        T v[NSTATE] = {T(b.props.pos.x),      T(b.props.pos.y),      T(b.props.angle),
                       T(b.props.momentum.x), T(b.props.momentum.y), T(b.props.ang_momentum),
                       T(b.props.force.x),    T(b.props.force.y),    T(b.props.torque),
                       T(b.aabb.pos.x),       T(b.aabb.pos.y),       T(b.aabb.half_width),
                       T(b.aabb.half_height)};
        for (int f = 0; f < NSTATE; ++f) out[(size_t)f * n + i] = v[f];
    }
}

template <class R>
void set_state(Solver<R>& s, const float* in) {
    const size_t n = s.bodies.size();
    for (size_t i = 0; i < n; ++i) {
        Body<R>& b = s.bodies[i];
        auto v = [&](int f) { return R(in[(size_t)f * n + i]); };
        b.props.pos = {v(0), v(1)};
        b.props.angle = v(2);
        b.props.momentum = {v(3), v(4)};
        b.props.ang_momentum = v(5);
        b.props.force = {v(6), v(7)};
        b.props.torque = v(8);
        b.aabb.pos = {v(9), v(10)};
        b.aabb.half_width = v(11);
        b.aabb.half_height = v(12);
    }
}

template <class R>
void get_props(const Solver<R>& s, float* out) {
    const size_t n = s.bodies.size();
    for (size_t i = 0; i < n; ++i) {
        const Body<R>& b = s.bodies[i];
        float v[NPROP] = {float(b.props.mass), float(b.props.inertia), float(b.props.mu),
                          float(b.type == DISC ? b.radius : b.width),
                          float(b.type == DISC ? R(0) : b.height)};
        for (int f = 0; f < NPROP; ++f) out[(size_t)f * n + i] = v[f];
    }
}

template <class R>
void add_joints(Solver<R>& s, uint32_t n, const uint8_t* type, const uint32_t* id1,
                const uint32_t* id2, const float* prm) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* p = prm + (size_t)i * NJP;
        Joint<R> j;
        j.type = (JointType)type[i];
        j.power_max = R(p[0]);
        j.power_min = R(p[1]);
        j.beta = R(p[2]);
        j.id1 = id1[i];
        j.id2 = id2[i];
        switch (j.type) {
        case DISTANCE_JOINT: j.target_distance = R(p[3]); break;
        case OFFSET_DISTANCE_JOINT:
            j.r1 = {R(p[3]), R(p[4])};
            j.r2 = {R(p[5]), R(p[6])};
            j.target_distance = R(p[7]);
            break;
        case FIXED_POSITION_JOINT: j.target_position = {R(p[3]), R(p[4])}; break;
        case MOTOR_JOINT: j.target_omega = R(p[3]); break;
        }
        s.constraints.push_back(j);
    }
}

template <class R>
void get_manifolds(const Solver<R>& s, uint32_t* keys, float* data) {
    for (size_t m = 0; m < s.manifolds.size(); ++m) {
        const auto& km = s.manifolds[m];
        keys[2 * m] = (uint32_t)km.first.ref;
        keys[2 * m + 1] = (uint32_t)km.first.inc;
        const Manifold<R>& M = km.second;
        float* d = data + m * MF;
        d[0] = float(M.normal.x);
        d[1] = float(M.normal.y);
        d[2] = float(M.tangent.x);
        d[3] = float(M.tangent.y);
        d[4] = float(M.friction);
        d[5] = M.has_point[0] ? 1.f : 0.f;
        d[6] = M.has_point[1] ? 1.f : 0.f;
        d[7] = float(M.prev_angle_1);
        d[8] = float(M.prev_angle_2);
        for (int p = 0; p < 2; ++p) {
            const CollisionPoint<R>& P = M.points[p];
            float* q = d + 9 + 12 * p;
            q[0] = float(P.pos.x);
            q[1] = float(P.pos.y);
            q[2] = float(P.ref_r.x);
            q[3] = float(P.ref_r.y);
            q[4] = float(P.inc_r.x);
            q[5] = float(P.inc_r.y);
            q[6] = float(P.depth);
            q[7] = float(P.original_depth);
            q[8] = float(P.mass_n);
            q[9] = float(P.mass_t);
            q[10] = float(P.accumulated_pn);
            q[11] = float(P.accumulated_pt);
        }
    }
}

#define DISPATCH(h, expr)                 \
    do {                                  \
        if ((h)->precision == 64) {       \
            auto& S = *(h)->d;            \
            expr;                         \
        } else {                          \
            auto& S = *(h)->f;            \
            expr;                         \
        }                                 \
    } while (0)

}  // namespace

/* Flags of r2o_batch_run_checkpoints. */
enum { BR_WARM = 1, BR_COMPENSATED = 2, BR_PERTURB_ULP = 4, BR_PERTURB_F32_ULP = 8 };

/* Perturbs every dynamic body's x by one ulp of the solver's own precision
 * (BR_PERTURB_ULP) or by one f32 ulp (BR_PERTURB_F32_ULP), upwards. */
template <class R>
void perturb_x(Solver<R>& s, int flags) {
    for (auto& b : s.bodies) {
        if (b.is_static) continue;
        if (flags & BR_PERTURB_F32_ULP) {
            const float x = (float)b.props.pos.x;
            b.props.pos.x = R(std::nextafter(x, std::numeric_limits<float>::infinity()));
        } else if (flags & BR_PERTURB_ULP) {
            b.props.pos.x = std::nextafter(b.props.pos.x, std::numeric_limits<R>::infinity());
        }
    }
}

extern "C" {

void* r2o_create(int precision) {
    Handle* h = new Handle();
    h->precision = precision == 64 ? 64 : 32;
    if (h->precision == 64)
        h->d.reset(new Solver<double>());
    else
        h->f.reset(new Solver<float>());
    return h;
}

void r2o_destroy(void* hp) { delete (Handle*)hp; }

int r2o_add_bodies(void* hp, uint32_t n, const uint32_t* ids, const uint8_t* kind,
                   const float* opt) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, add_bodies(S, n, ids, kind, opt));
    return 0;
}

/* r2o_add_bodies with polygons among them (kind bit 8): nverts [n],
 * verts [n][MAX_POLY_VERTS][2]. */
int r2o_add_bodies_poly(void* hp, uint32_t n, const uint32_t* ids, const uint8_t* kind, const float* opt,
                        const uint8_t* nverts, const float* verts) {
    Handle* h = (Handle*)hp;
    for (uint32_t i = 0; i < n; ++i)
        if ((kind[i] & 8) && (nverts[i] < 3 || nverts[i] > MAX_POLY_VERTS)) return -1;
    DISPATCH(h, add_bodies(S, n, ids, kind, opt, nverts, verts));
    return 0;
}

uint32_t r2o_num_bodies(void* hp) {
    Handle* h = (Handle*)hp;
    uint32_t n = 0;
    DISPATCH(h, n = (uint32_t)S.bodies.size());
    return n;
}

void r2o_add_gravity(void* hp, float g) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, S.gravity.push_back(g));
}

void r2o_exclude_pair(void* hp, uint32_t id1, uint32_t id2) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, S.exclude_pair(id1, id2));
}

void r2o_add_joints(void* hp, uint32_t n, const uint8_t* type, const uint32_t* id1,
                    const uint32_t* id2, const float* prm) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, add_joints(S, n, type, id1, id2, prm));
}

void r2o_set_hash_config(void* hp, float cell_size, uint32_t table_mult) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, (S.cell_size = cell_size, S.table_mult = table_mult));
}

void r2o_set_warm_start(void* hp, int on) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, (S.warm_start = on != 0, S.warm_prev.clear()));
}

/* n increments x[k] accumulated from (s, c) = (s0, 0) with the clamped
 * compensated update of r2d_accum.h (lower bound lo, no upper bound when
 * hi is NaN); out = {s, c, sum of the applied changes}. */
void r2o_acc_sum(uint32_t n, const float* x, float s0, float lo, float hi, float* out) {
    float s = s0, c = 0.f, applied = 0.f;
    for (uint32_t k = 0; k < n; ++k)
        applied += (hi == hi) ? r2d_acc_add_clamp(&s, &c, x[k], lo, hi) : r2d_acc_add_max(&s, &c, x[k], lo);
    out[0] = s;
    out[1] = c;
    out[2] = applied;
}

void r2o_set_compensated(void* hp, int on) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, S.compensated = on != 0);
}

/* Hands src's last-frame warm-start table (keyed by body ids) to dst, as an
 * engine keeps it when its body store is replaced.  Both of one precision. */
int r2o_copy_warm(void* dst, const void* src) {
    Handle* d = (Handle*)dst;
    const Handle* s = (const Handle*)src;
    if (d->precision != s->precision) return -1;
    if (d->precision == 64)
        d->d->warm_prev = s->d->warm_prev;
    else
        d->f->warm_prev = s->f->warm_prev;
    return 0;
}

void r2o_get_state(void* hp, float* out) {
    Handle* h = (Handle*)hp;
    if (h->precision == 64)
        get_state<double, float>(*h->d, out);
    else
        get_state<float, float>(*h->f, out);
}

void r2o_get_state_f64(void* hp, double* out) {
    Handle* h = (Handle*)hp;
    if (h->precision == 64)
        get_state<double, double>(*h->d, out);
    else
        get_state<float, double>(*h->f, out);
}

void r2o_set_state(void* hp, const float* in) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, (set_state(S, in), S.sleep_frames = 0u));  // a write wakes the world
}

/* Per-phase wall time of the step (a measurement aid; r2o::Phase order).
 * Switching it on or off clears the sums. */
void r2o_set_phase_timing(void* hp, int on) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, (S.time_phases = on != 0, std::fill(std::begin(S.phase_seconds), std::end(S.phase_seconds), 0.0)));
}

void r2o_phase_seconds(void* hp, double* out) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, std::copy(std::begin(S.phase_seconds), std::end(S.phase_seconds), out));
}

void r2o_set_sleep(void* hp, int on) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, (S.sleep_enabled = on != 0, S.sleep_frames = 0u));
}

uint32_t r2o_sleep_frames(void* hp) {
    Handle* h = (Handle*)hp;
    return h->precision == 64 ? h->d->sleep_frames : h->f->sleep_frames;
}

void r2o_get_props(void* hp, float* out) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, get_props(S, out));
}

int r2o_process(void* hp, float dt, uint32_t sub_steps, uint32_t iters, int order) {
    Handle* h = (Handle*)hp;
    int st = 0;
    try {
        if (h->precision == 64)
            st = h->d->process(double(dt), sub_steps, iters, order);
        else
            st = h->f->process(dt, sub_steps, iters, order);
    } catch (...) {
        st = ERR_INTERNAL;
    }
    return st;
}

/* Broadphase + narrowphase only (Solver.updateManifolds, lib.zig:253-299),
 * plus the colouring when order == ORDER_COLOUR. */
int r2o_update_manifolds(void* hp, int order) {
    Handle* h = (Handle*)hp;
    int st = 0;
    try {
        DISPATCH(h, (st = S.update_manifolds(), st = (st == 0 && order == ORDER_COLOUR) ? S.compute_colouring() : st));
    } catch (...) {
        st = ERR_INTERNAL;
    }
    return st;
}

uint32_t r2o_num_manifolds(void* hp) {
    Handle* h = (Handle*)hp;
    uint32_t n = 0;
    DISPATCH(h, n = (uint32_t)S.manifolds.size());
    return n;
}

void r2o_get_manifolds(void* hp, uint32_t* keys, float* data) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, get_manifolds(S, keys, data));
}

/* Candidate pairs of the last narrowphase (recorded once enabled): (lower,
 * higher) body indices, sorted; at most cap pairs written, count returned. */
void r2o_set_record_pairs(void* hp, int on) {
    Handle* h = (Handle*)hp;
    DISPATCH(h, S.record_pairs = on != 0);
}

uint32_t r2o_get_pairs(void* hp, uint32_t cap, uint32_t* out) {
    Handle* h = (Handle*)hp;
    uint32_t n = 0;
    DISPATCH(h, (n = (uint32_t)S.candidate_pairs.size(), [&] {
                     for (uint32_t q = 0; q < n && q < cap; ++q) {
                         out[2 * q] = (uint32_t)(S.candidate_pairs[q] >> 32);
                         out[2 * q + 1] = (uint32_t)S.candidate_pairs[q];
                     }
                 }()));
    return n;
}

/* Colours of the manifolds (discovery order) and joints (insertion order)
 * from the last colouring; at most ncap / jcap entries are written.
 * Returns the number of manifold colours available. */
uint32_t r2o_get_colours(void* hp, uint32_t ncap, uint32_t* contact, uint32_t jcap, uint32_t* joint) {
    Handle* h = (Handle*)hp;
    uint32_t n = 0;
    DISPATCH(h, (n = (uint32_t)S.contact_colour.size(),
                 std::copy_n(S.contact_colour.begin(), std::min<size_t>(ncap, S.contact_colour.size()), contact),
                 std::copy_n(S.joint_colour.begin(), std::min<size_t>(jcap, S.joint_colour.size()), joint)));
    return n;
}

/* Many independent worlds stepped on host threads (one world per task,
 * dynamic scheduling).  Bodies of world w are [body_off[w], body_off[w+1]) of
 * the concatenated arrays; each world gets one gravity generator of
 * magnitude gravity[w] (none when 0).  state_in (optional) and state_out use
 * the global field-major layout [NSTATE][total bodies].  Returns the wall
 * seconds of the stepping alone; status_out gets the first non-zero status. */
double r2o_batch_run(int precision, uint32_t nworlds, const uint32_t* body_off, const uint32_t* ids,
                     const uint8_t* kind, const float* opt_all, const float* gravity, float dt,
                     uint32_t sub_steps, uint32_t iters, uint32_t steps, int order, int nthreads,
                     const float* state_in, float* state_out, int* status_out) {
    std::vector<std::unique_ptr<Handle>> worlds(nworlds);
    const uint32_t ntot = body_off[nworlds];
    for (uint32_t w = 0; w < nworlds; ++w) {
        uint32_t b0 = body_off[w], n = body_off[w + 1] - b0;
        std::vector<float> opt((size_t)NOPT * n);
        for (int f = 0; f < NOPT; ++f)
            for (uint32_t i = 0; i < n; ++i) opt[(size_t)f * n + i] = opt_all[(size_t)f * ntot + b0 + i];
        worlds[w].reset((Handle*)r2o_create(precision));
        r2o_add_bodies(worlds[w].get(), n, ids + b0, kind + b0, opt.data());
        if (gravity[w] != 0.f) r2o_add_gravity(worlds[w].get(), gravity[w]);
        if (state_in) {
            std::vector<float> st((size_t)NSTATE * n);
            for (int f = 0; f < NSTATE; ++f)
                for (uint32_t i = 0; i < n; ++i) st[(size_t)f * n + i] = state_in[(size_t)f * ntot + b0 + i];
            r2o_set_state(worlds[w].get(), st.data());
        }
    }
    std::atomic<uint32_t> next(0);
    std::atomic<int> first_err(0);
    auto work = [&]() {
        for (;;) {
            uint32_t w = next.fetch_add(1);
            if (w >= nworlds) break;
            for (uint32_t s = 0; s < steps; ++s) {
                int st = r2o_process(worlds[w].get(), dt, sub_steps, iters, order);
                if (st != 0) {
                    int z = 0;
                    first_err.compare_exchange_strong(z, st);
                    break;
                }
            }
        }
    };
    if (nthreads < 1) nthreads = 1;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    auto t1 = std::chrono::steady_clock::now();
    if (state_out) {
        for (uint32_t w = 0; w < nworlds; ++w) {
            uint32_t b0 = body_off[w], n = body_off[w + 1] - b0;
            std::vector<float> st((size_t)NSTATE * n);
            r2o_get_state(worlds[w].get(), st.data());
            for (int f = 0; f < NSTATE; ++f)
                for (uint32_t i = 0; i < n; ++i) state_out[(size_t)f * ntot + b0 + i] = st[(size_t)f * n + i];
        }
    }
    if (status_out) *status_out = first_err.load();
    return std::chrono::duration<double>(t1 - t0).count();
}

/* Every world of a scene stepped on host threads from its initial state
 * (r2o_batch_run without state_in), in the given mode (flags above), and
 * its full state kept in f64 at each of the ncheck ascending step counts:
 * out [ncheck][NSTATE][ntot].  Returns the first non-zero status. */
int r2o_batch_run_checkpoints(int precision, uint32_t nworlds, const uint32_t* body_off, const uint32_t* ids,
                              const uint8_t* kind, const float* opt_all, const float* gravity, float dt,
                              uint32_t sub_steps, uint32_t iters, int order, int nthreads, int flags,
                              uint32_t ncheck, const uint32_t* checks, double* out) {
    const uint32_t ntot = body_off[nworlds];
    std::atomic<uint32_t> next(0);
    std::atomic<int> first_err(0);
    auto work = [&]() {
        for (;;) {
            const uint32_t w = next.fetch_add(1);
            if (w >= nworlds) break;
            const uint32_t b0 = body_off[w], n = body_off[w + 1] - b0;
            std::vector<float> opt((size_t)NOPT * n);
            for (int f = 0; f < NOPT; ++f)
                for (uint32_t i = 0; i < n; ++i) opt[(size_t)f * n + i] = opt_all[(size_t)f * ntot + b0 + i];
            std::unique_ptr<Handle> h((Handle*)r2o_create(precision));
            r2o_add_bodies(h.get(), n, ids + b0, kind + b0, opt.data());
            if (gravity[w] != 0.f) r2o_add_gravity(h.get(), gravity[w]);
            DISPATCH(h, (S.warm_start = (flags & BR_WARM) != 0, S.compensated = (flags & BR_COMPENSATED) != 0,
                         perturb_x(S, flags)));
            std::vector<double> st((size_t)NSTATE * n);
            uint32_t done = 0;
            for (uint32_t c = 0; c < ncheck; ++c) {
                for (; done < checks[c]; ++done) {
                    const int e = r2o_process(h.get(), dt, sub_steps, iters, order);
                    if (e != 0) {
                        int z = 0;
                        first_err.compare_exchange_strong(z, e);
                        break;
                    }
                }
                r2o_get_state_f64(h.get(), st.data());
                for (int f = 0; f < NSTATE; ++f)
                    for (uint32_t i = 0; i < n; ++i)
                        out[((size_t)c * NSTATE + f) * ntot + b0 + i] = st[(size_t)f * n + i];
            }
        }
    };
    if (nthreads < 1) nthreads = 1;
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    return first_err.load();
}

/* Known-answer hooks for the reference's own unit tests:
 * src/core/nmath.zig:157-176 ("vector2") and src/core/aabb.zig:34-45
 * ("sanity check aabb overlapping"). */
void r2o_nmath_kat(const float* a, const float* b, float* out) {
    V2<float> A{a[0], a[1]}, B{b[0], b[1]};
    V2<float> s = add2(A, B), d = sub2(A, B), m = multelem2(A, B), q = divelem2(A, B);
    float v[12] = {s.x, s.y, d.x, d.y, m.x, m.y, q.x, q.y, dot2(A, B), cross2(A, B), dot2(A, A), length2(A)};
    for (int i = 0; i < 12; ++i) out[i] = v[i];
}

int r2o_aabb_intersects(float x1, float y1, float hw1, float hh1, float x2, float y2, float hw2, float hh2) {
    AABB<float> s1{{x1, y1}, hw1, hh1}, s2{{x2, y2}, hw2, hh2};
    return s1.intersects(s2) ? 1 : 0;
}

/* The shared f32 sin/cos (r2d_sincos.h) for accuracy tests. */
void r2o_sincosf(uint32_t n, const float* x, float* s, float* c) {
    for (uint32_t i = 0; i < n; ++i) r2d_sincosf(x[i], &s[i], &c[i]);
}

}  // extern "C"
