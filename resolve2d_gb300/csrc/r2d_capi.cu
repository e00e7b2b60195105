/*
 * r2d_capi.cu -- host runtime behind include/r2d_gb300.h.
 *
 * An Engine owns the device copy of one or many worlds (field-major state
 * and properties in HBM, world descriptors, joints, exclusions) and steps
 * them with the fused per-world kernel (r2d_world_kernel.cu).  Worlds are
 * grouped into size classes; each class is one launch whose per-world
 * shared-memory budget is sized from that class's capacities, so small
 * worlds pack many CTAs per SM and large ones still fit.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <exception>
#include <memory>
#include <new>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/r2d_gb300.h"
#include "r2d_device.cuh"
#include "r2d_large.h"
#include "r2d_sincos.h"
#include "r2d_solve.cuh"
#include "r2d_validate.h"
#include "r2d_world.cuh"

namespace r2d {
cudaError_t launch_world_step(const StepParams& P, const Caps& C, int threads, const LayoutOpts& opts,
                              cudaStream_t stream, int priority = 0);
cudaError_t allow_world_step_smem(int bytes);
cudaError_t launch_count_call(uint32_t* counter, cudaStream_t stream);
cudaError_t launch_migrate_warm(uint32_t nworlds, const WarmTables& old_t, const uint32_t* old_cur,
                                const WarmTables& new_t, cudaStream_t stream);
}  // namespace r2d

using namespace r2d;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (expr);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            if (e_ == cudaErrorMemoryAllocation) return fail(R2D_ERR_OUT_OF_MEMORY, #expr);  \
            return fail(R2D_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
        }                                                                                    \
    } while (0)

template <class T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

template <class T>
cudaError_t dalloc(T*& p, size_t count) {
    dfree(p);
    if (count == 0) count = 1;
    return cudaMalloc((void**)&p, count * sizeof(T));
}

// AABB of a freshly created body (Disc.zig:63-66, Rectangle.zig:71-86).
void init_aabb(uint8_t kind, float x, float y, float angle, float d0, float d1, float out[4]) {
    out[0] = x;
    out[1] = y;
    if (!(kind & K_RECT)) {
        out[2] = d0;
        out[3] = d0;
        return;
    }
    float s, c;
    r2d_sincosf(angle, &s, &c);
    const float w = d0 / 2.0f, h = d1 / 2.0f;
    const float lx[4] = {-w, -w, w, w}, ly[4] = {-h, h, h, -h};
    float ew = 0.f, eh = 0.f;
    for (int i = 0; i < 4; ++i) {
        float rx = lx[i] * c - ly[i] * s;
        float ry = lx[i] * s + ly[i] * c;
        if (rx > ew) ew = rx;
        if (ry > eh) eh = ry;
    }
    out[2] = ew;
    out[3] = eh;
}

// A polygon's first AABB: its largest rotated vertex in x and y, from 0
// (Rectangle.updateAABB over its vertices, Rectangle.zig:71-86).
void init_aabb_polygon(float x, float y, float angle, const float* verts, uint32_t nv, float out[4]) {
    float s, c;
    r2d_sincosf(angle, &s, &c);
    float ew = 0.f, eh = 0.f;
    for (uint32_t i = 0; i < nv; ++i) {
        const float lx = verts[2 * i], ly = verts[2 * i + 1];
        const float rx = lx * c - ly * s;
        const float ry = lx * s + ly * c;
        if (rx > ew) ew = rx;
        if (ry > eh) eh = ry;
    }
    out[0] = x;
    out[1] = y;
    out[2] = ew;
    out[3] = eh;
}

struct KClass {
    Caps caps{};
    int threads = 128;
    LayoutOpts opts{true, false, false, false};
    std::vector<uint32_t> worlds;
    uint32_t* d_list = nullptr;
    uint32_t smem = 0;
    uint32_t boost = 0;  // the capacity boosts its worlds carry
    int priority = 0;    // launch priority (plan(): large and small bounds paired, from the top)
};

// Size-class launch priorities on (R2D_CLASS_PRIORITY=0 leaves them all at
// the default) and auxiliary streams, one per class.
#ifndef R2D_CLASS_PRIORITY
#define R2D_CLASS_PRIORITY 1
#endif
#ifndef R2D_NAUX
#define R2D_NAUX 32
#endif
#ifndef R2D_REPLAN_TWICE
#define R2D_REPLAN_TWICE 1
#endif

struct Engine {
    r2d_config cfg{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // Size classes run concurrently on auxiliary streams forked from and
    // joined back into `stream`, so one class's tail overlaps the others.
    // Classes sharing a stream would run one after the other, so there is a
    // stream for each of the size classes (body bounds x capacity boosts) a step
    // normally has.
    static constexpr int NAUX = R2D_NAUX;
    cudaStream_t aux[NAUX] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[NAUX] = {};
    bool verbose = false;
    float cell = 4.0f;
    uint32_t table_mult = 2;

    uint32_t nworlds = 0, nbodies = 0;
    std::vector<WorldDesc> worlds_h;
    std::vector<uint32_t> ids_h;
    std::vector<uint8_t> kind_h;
    std::vector<float> props_h;
    std::vector<float> state_h;  // last uploaded (for capacity planning)
    // Convex polygons (K_POLY bodies, stepped by the grid pipeline): vertex
    // counts [nbodies] and local vertices [nbodies][MAX_POLY_VERTS][2]; the
    // bodies whose first AABB waits for their vertices.
    bool has_poly = false;
    std::vector<uint8_t> poly_nv_h, poly_aabb_pending;
    std::vector<float> poly_v_h;
    uint8_t* d_poly_nv = nullptr;
    float2* d_poly_v = nullptr;

    float* d_state = nullptr;
    double* d_pos64 = nullptr;  // [3][nbodies] f64 x, y, angle (R2D_FLAG_FP64_POSITIONS)
    float* d_props = nullptr;
    uint8_t* d_kind = nullptr;
    uint32_t* d_ids = nullptr;
    WorldDesc* d_worlds = nullptr;
    int* d_status = nullptr;
    int* d_err = nullptr;
    int* h_err = nullptr;  // pinned

    // joints / exclusions (resolved to world-local indices)
    uint32_t njoints = 0, nexcl = 0;
    uint8_t* d_jtype = nullptr;
    uint32_t* d_jb1 = nullptr;
    uint64_t joint_epoch = 0;  // bumped by every upload of the joint arrays
    uint32_t* d_jb2 = nullptr;
    float* d_jprm = nullptr;
    unsigned long long* d_excl = nullptr;

    std::vector<KClass> classes;
    bool plan_dirty = true;
    // After capacity replays the plan is made again at the next call, and once
    // more at the call after it (R2D_REPLAN_TWICE): measured on the 4,096-world
    // batch, the step graph captured right after a round of replays ran 5 %
    // slower than the same plan captured one call later.
    uint32_t replan_in = 0;
    bool plan_multi_substep = false;  // layouts keep frame-start positions

    // debug taps
    DebugOut dbg{};
    uint32_t* d_dbg_nman = nullptr;
    uint32_t* d_dbg_keys = nullptr;
    float* d_dbg_data = nullptr;
    uint32_t* d_dbg_col = nullptr;
    uint32_t* d_dbg_jcol = nullptr;
    uint32_t* d_dbg_npairs = nullptr;
    uint32_t* d_dbg_pairs = nullptr;

    std::vector<int> status_h;
    bool pending = false;

    // Calls enqueued since the last sync; a world that outgrows its class is
    // frozen on the device and replayed from its failing call at sync.
    struct CallRec {
        float dt;
        uint32_t sub_steps, iters;
    };
    std::vector<CallRec> calls;
    uint32_t* d_fail_call = nullptr;
    uint32_t* d_one = nullptr;          // single-world list for replays
    uint32_t* d_capbits = nullptr;      // [nworlds] which buffers overflowed
    unsigned long long* d_timers = nullptr;  // phase timers (R2D_PHASE_TIMERS builds)
    // Doublings of each per-world buffer a world has needed (manifolds,
    // points, cell entries, candidate pairs), packed one byte each.
    std::vector<uint32_t> world_boost;
    static uint32_t boost_of(uint32_t b, int i) { return (b >> (8 * i)) & 0x7Fu; }
    static constexpr uint32_t BOOST_FULL = 0x80000000u;  // world needs the full point layout

    // Worlds above the largest fused class, or that outgrew its shared
    // memory, step through the grid-wide pipeline of r2d_large.cu on their
    // own stream while the fused classes run.
    static constexpr uint32_t FUSED_MAX_BODIES = 520;
    // Size classes of the fused kernel, by body count (a class's shared
    // memory is sized for its bound).
    static constexpr uint32_t CLASS_BOUNDS[] = {32, 64, 96, 128, 160, 192, 256, 320, 384, 448, 520};
    static constexpr int NBOUNDS = sizeof(CLASS_BOUNDS) / sizeof(CLASS_BOUNDS[0]);
    // Largest spatial-hash table (table_mult x bodies) of one world.
    static constexpr unsigned long long MAX_TABLE_BUCKETS = 1ull << 31;
    std::vector<uint8_t> world_large;                 // [nworlds] routed to the large path
    std::vector<uint32_t> large_list;                 // those worlds, in index order
    std::vector<std::unique_ptr<LargeWorld>> large;   // [nworlds] scratch of each large world
    std::vector<int> large_status;                    // [nworlds] status of its last step
    std::vector<uint8_t> large_frozen;                // failed since the last sync
    std::string large_msg;
    cudaStream_t lstream = nullptr;
    cudaEvent_t ev_ljoin = nullptr;

    // The fused step of one call, captured once as a CUDA graph and replayed
    // while the plan and (dt, sub_steps, iters) stay the same.  Calls count
    // themselves on the device (d_call), so the graph needs no per-call
    // parameters.
    uint32_t* d_call = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // threads per CTA chosen by autotune() for each size class (0 = the
    // default policy), by index into the class bounds
    int thread_override[16] = {};

    // Warm starting (R2D_FLAG_WARM_START): each fused world's two tables of
    // warm_hs slots (WorldDesc::warm_off), sized from its class's manifold
    // capacity; d_warm_cur[w] names the table holding last frame.
    unsigned long long* d_warm_keys = nullptr;
    float4* d_warm_vals = nullptr;
    float4* d_warm_cvals = nullptr;  // compensation words (R2D_FLAG_COMPENSATED)
    uint32_t* d_warm_cur = nullptr;
    // Last frame's warm-start entries of each world, taken when the body
    // store is replaced and put into the new tables at the next plan: keys
    // are body ids, so they stay valid; entries naming a vanished id are dropped.
    struct WarmEntry {
        unsigned long long key;
        float4 val, cval;
    };
    std::vector<std::vector<WarmEntry>> warm_carry;
    uint32_t* d_sleep = nullptr;  // [nworlds] consecutive still frames (R2D_FLAG_SLEEP)
    // A frame call's host rows (process_io): the device copy the kernels read
    // (StepParams::ext) and the value last copied there.
    ExtIO* d_ext = nullptr;
    ExtIO ext_cur{};
    ExtIO ext_src{};  // pageable source of the copy: free to change once the copy call returns
    uint32_t* d_warm_off = nullptr;  // [nworlds] copies of WorldDesc::warm_off / warm_hs for migration
    uint32_t* d_warm_hs = nullptr;
    std::vector<uint32_t> warm_hs_h, warm_off_h;
    float g_dt = 0.f;
    uint32_t g_sub = 0, g_iters = 0;
    bool use_graph = true;
    uint32_t colour_round_limit = 0;  // R2D_COLOUR_ROUND_LIMIT (0 = the colouring's own bound)
    // Tuning: the binning grid's cell as a multiple of the largest dynamic
    // body's diameter (R2D_FINE_CELL_SCALE, default 1).  Pairs do not depend
    // on it; candidates and entries per body do.
    float fine_scale = 1.0f;
    // Tuning: launch priorities by body bound (R2D_CLASS_PRIORITIES, e.g.
    // "520:-5,448:-4"; bounds not named get 0), in place of the pairing.
    std::vector<std::pair<uint32_t, int>> priority_map;
    bool priority_map_set = false;

    ~Engine() {
        large.clear();
        if (gexec) cudaGraphExecDestroy(gexec);
        dfree(d_call);
        dfree(d_ext);
        dfree(d_warm_keys); dfree(d_warm_vals); dfree(d_warm_cvals); dfree(d_warm_cur); dfree(d_warm_off);
        dfree(d_warm_hs);
        dfree(d_sleep);
        dfree(d_state); dfree(d_pos64); dfree(d_props); dfree(d_kind); dfree(d_ids); dfree(d_worlds);
        dfree(d_poly_nv); dfree(d_poly_v);
        dfree(d_status); dfree(d_err);
        if (h_err) cudaFreeHost(h_err);
        dfree(d_jtype); dfree(d_jb1); dfree(d_jb2); dfree(d_jprm); dfree(d_excl);
        for (auto& c : classes) dfree(c.d_list);
        dfree(d_dbg_nman); dfree(d_dbg_keys); dfree(d_dbg_data); dfree(d_dbg_col); dfree(d_dbg_jcol);
        dfree(d_dbg_npairs); dfree(d_dbg_pairs);
        dfree(d_fail_call); dfree(d_one); dfree(d_capbits); dfree(d_timers);
        for (int a = 0; a < NAUX; ++a) {
            if (aux[a]) cudaStreamDestroy(aux[a]);
            if (ev_join[a]) cudaEventDestroy(ev_join[a]);
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (lstream) cudaStreamDestroy(lstream);
        if (ev_ljoin) cudaEventDestroy(ev_ljoin);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    int init(const r2d_config* c) {
        if (c) cfg = *c;
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(R2D_ERR_NO_DEVICE, "no CUDA device");
        cell = cfg.spatialhash_cell_width > 0.f ? cfg.spatialhash_cell_width : 4.0f;
        table_mult = cfg.spatialhash_table_size_mult ? cfg.spatialhash_table_size_mult : 2u;
        if (cfg.stream) {
            stream = (cudaStream_t)cfg.stream;
        } else {
            CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
            own_stream = true;
        }
        CUDA_TRY(cudaMallocHost((void**)&h_err, sizeof(int)));
        CUDA_TRY(dalloc(d_err, 1));
        for (int a = 0; a < NAUX; ++a) {
            CUDA_TRY(cudaStreamCreateWithFlags(&aux[a], cudaStreamNonBlocking));
            CUDA_TRY(cudaEventCreateWithFlags(&ev_join[a], cudaEventDisableTiming));
        }
        CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        CUDA_TRY(cudaStreamCreateWithFlags(&lstream, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&ev_ljoin, cudaEventDisableTiming));
        const char* v = getenv("R2D_VERBOSE");
        verbose = v && v[0] && v[0] != '0';
        const char* ng = getenv("R2D_NO_GRAPH");
        use_graph = !(ng && ng[0] && ng[0] != '0');
        // Test hook: a small limit on the grid pipeline's colouring rounds
        // makes its one bounded device loop give up (R2D_ERR_TIMEOUT).
        const char* rl = getenv("R2D_COLOUR_ROUND_LIMIT");
        colour_round_limit = rl ? (uint32_t)strtoul(rl, nullptr, 10) : 0u;
        const char* fs = getenv("R2D_FINE_CELL_SCALE");
        if (fs && strtof(fs, nullptr) > 0.f) fine_scale = strtof(fs, nullptr);
        // "bound:value,bound:value,..." lists (bounds in bodies)
        auto parse_map = [](const char* q, std::vector<std::pair<uint32_t, int>>* out) {
            while (*q) {
                char* e1 = nullptr;
                const unsigned long nb = strtoul(q, &e1, 10);
                if (e1 == q || *e1 != ':') break;
                char* e2 = nullptr;
                const long v = strtol(e1 + 1, &e2, 10);
                if (e2 == e1 + 1) break;
                out->push_back({(uint32_t)nb, (int)v});
                q = *e2 == ',' ? e2 + 1 : e2;
            }
        };
        if (const char* pm = getenv("R2D_CLASS_PRIORITIES")) {
            priority_map_set = true;
            parse_map(pm, &priority_map);
        }
        // Tuning: threads per CTA by body bound (R2D_CLASS_THREADS, e.g.
        // "448:128,520:256"), as if the autotuner had chosen them.
        if (const char* tm = getenv("R2D_CLASS_THREADS")) {
            std::vector<std::pair<uint32_t, int>> tmap;
            parse_map(tm, &tmap);
            for (const auto& kv : tmap)
                for (int k = 0; k < NBOUNDS; ++k)
                    if (CLASS_BOUNDS[k] == kv.first &&
                        (kv.second == 32 || kv.second == 64 || kv.second == 128 || kv.second == 256 ||
                         kv.second == 512))
                        thread_override[k] = kv.second;
        }
        CUDA_TRY(dalloc(d_call, 1));
        CUDA_TRY(dalloc(d_ext, 1));
        CUDA_TRY(cudaMemsetAsync(d_ext, 0, sizeof(ExtIO), stream));
        CUDA_TRY(cudaMemsetAsync(d_call, 0, sizeof(uint32_t), stream));
        CUDA_TRY(allow_world_step_smem(smem_optin()));
        return R2D_OK;
    }

    int set_bodies(uint32_t nw, const uint32_t* body_off, const uint32_t* ids, const uint8_t* kind,
                   const float* props, const float* state, const float* gravity, uint32_t ngrav_each,
                   int do_init_aabb) {
        const uint32_t n = body_off[nw];
        for (uint32_t w = 0; w < nw; ++w)
            if (body_off[w + 1] < body_off[w]) return fail(R2D_ERR_INVALID_ARGUMENT, "body_off not monotonic");
        // the bucket count table_mult x n is 32-bit on the device: refuse a
        // product that would wrap before anything is uploaded
        for (uint32_t w = 0; w < nw; ++w) {
            const unsigned long long T = (unsigned long long)table_mult * (body_off[w + 1] - body_off[w]);
            if (T > MAX_TABLE_BUCKETS)
                return fail(R2D_ERR_CAPACITY, "world " + std::to_string(w) + ": a spatial-hash table of " +
                                                  std::to_string(T) + " buckets exceeds the maximum of " +
                                                  std::to_string(MAX_TABLE_BUCKETS));
        }
        uint32_t dup = 0;
        const int64_t dw = r2d_first_duplicate_id(nw, body_off, ids, &dup);
        if (dw >= 0)
            return fail(R2D_ERR_INVALID_ARGUMENT,
                        "world " + std::to_string(dw) + " holds two bodies with id " + std::to_string(dup));
        // warm starting: last frame's impulses outlive the body store (their
        // keys are ids); world w of the new store takes world w's
        if (warm_start()) {
            if (int st = take_warm_entries()) return st;
            warm_carry.resize(nw);
            for (uint32_t w = 0; w < nw; ++w) {
                std::unordered_set<uint32_t> live(ids + body_off[w], ids + body_off[w + 1]);
                auto& v = warm_carry[w];
                v.erase(std::remove_if(v.begin(), v.end(),
                                       [&](const WarmEntry& e) {
                                           return !live.count((uint32_t)(e.key >> 32)) ||
                                                  !live.count((uint32_t)e.key);
                                       }),
                        v.end());
            }
        }
        for (uint32_t i = 0; i < n; ++i)
            if ((kind[i] & K_RECT) && (kind[i] & K_POLY))
                return fail(R2D_ERR_INVALID_ARGUMENT, "body " + std::to_string(i) + " is both a rectangle and a polygon");
        nworlds = nw;
        nbodies = n;
        ids_h.assign(ids, ids + n);
        kind_h.assign(kind, kind + n);
        props_h.assign(props, props + (size_t)P_NFIELDS * n);
        state_h.assign(state, state + (size_t)S_NFIELDS * n);
        if (do_init_aabb) {
            for (uint32_t i = 0; i < n; ++i) {
                float ab[4];
                init_aabb(kind_h[i], state_h[(size_t)S_POS_X * n + i], state_h[(size_t)S_POS_Y * n + i],
                          state_h[(size_t)S_ANGLE * n + i], props_h[(size_t)P_DIM0 * n + i],
                          props_h[(size_t)P_DIM1 * n + i], ab);
                for (int k = 0; k < 4; ++k) state_h[(size_t)(S_AABB_X + k) * n + i] = ab[k];
            }
        }
        worlds_h.assign(nw, WorldDesc{});
        for (uint32_t w = 0; w < nw; ++w) {
            WorldDesc& d = worlds_h[w];
            d.body_off = body_off[w];
            d.n = body_off[w + 1] - body_off[w];
            d.ngrav = 0;
            for (uint32_t k = 0; k < ngrav_each && k < (uint32_t)MAX_GRAVITY; ++k) {
                d.g[k] = gravity[(size_t)w * ngrav_each + k];
                d.ngrav++;
            }
        }
        CUDA_TRY(dalloc(d_state, (size_t)S_NFIELDS * n));
        CUDA_TRY(dalloc(d_props, (size_t)P_NFIELDS * n));
        CUDA_TRY(dalloc(d_kind, n));
        CUDA_TRY(dalloc(d_ids, n));
        CUDA_TRY(dalloc(d_status, nw));
        CUDA_TRY(dalloc(d_fail_call, nw));
        CUDA_TRY(dalloc(d_capbits, nw));
#ifdef R2D_PHASE_TIMERS
        CUDA_TRY(dalloc(d_timers, (size_t)nw * PHASE_SLOTS));
        CUDA_TRY(cudaMemsetAsync(d_timers, 0, sizeof(unsigned long long) * nw * PHASE_SLOTS, stream));
#endif
        CUDA_TRY(cudaMemsetAsync(d_fail_call, 0xFF, sizeof(uint32_t) * nw, stream));
        CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int) * nw, stream));
        world_boost.assign(nw, 0);
        world_large.assign(nw, 0);
        const bool grid_all = (cfg.flags & R2D_FLAG_GRID_PIPELINE) != 0;
        for (uint32_t w = 0; w < nw; ++w) world_large[w] = grid_all || worlds_h[w].n > FUSED_MAX_BODIES;
        // polygons: a world holding one steps on the grid pipeline; vertices
        // come with r2d_*_set_polygons, and so do their first AABBs
        has_poly = false;
        poly_nv_h.assign(n, 0);
        poly_aabb_pending.assign(n, 0);
        poly_v_h.assign((size_t)n * 2 * MAX_POLY_VERTS, 0.f);
        dfree(d_poly_nv);
        dfree(d_poly_v);
        for (uint32_t w = 0; w < nw; ++w)
            for (uint32_t i = body_off[w]; i < body_off[w + 1]; ++i)
                if (kind_h[i] & K_POLY) {
                    has_poly = true;
                    world_large[w] = 1;
                    poly_aabb_pending[i] = do_init_aabb ? 1 : 0;
                }
        large.clear();
        large.resize(nw);
        large_status.assign(nw, 0);
        large_frozen.assign(nw, 0);
        dfree(d_warm_keys); dfree(d_warm_vals); dfree(d_warm_cvals); dfree(d_warm_cur); dfree(d_warm_off);
        dfree(d_warm_hs);
        warm_hs_h.assign(nw, 0);
        warm_off_h.assign(nw, 0);
        if (warm_start()) {
            CUDA_TRY(dalloc(d_warm_cur, nw));
            CUDA_TRY(cudaMemsetAsync(d_warm_cur, 0, sizeof(uint32_t) * nw, stream));
        }
        dfree(d_sleep);
        if (sleeping()) {
            CUDA_TRY(dalloc(d_sleep, nw));
            CUDA_TRY(cudaMemsetAsync(d_sleep, 0, sizeof(uint32_t) * nw, stream));
        }
        calls.clear();
        pending = false;
        CUDA_TRY(cudaMemcpyAsync(d_state, state_h.data(), sizeof(float) * S_NFIELDS * n, cudaMemcpyHostToDevice, stream));
        if (fp64_positions()) {
            CUDA_TRY(dalloc(d_pos64, (size_t)3 * n));
            CUDA_TRY(upload_pose64(state_h.data()));
        }
        CUDA_TRY(cudaMemcpyAsync(d_props, props_h.data(), sizeof(float) * P_NFIELDS * n, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(d_kind, kind_h.data(), n, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(d_ids, ids_h.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        plan_dirty = true;
        return R2D_OK;
    }

    // Vertices of polygon bodies (global body indices): nverts 3..8 local
    // vertices each, clockwise; a body whose first AABB was asked for at
    // upload gets it now.
    int set_polygons(uint32_t n, const uint32_t* body, const uint8_t* nverts, const float* verts) {
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t i = body[k];
            if (i >= nbodies) return fail(R2D_ERR_INVALID_ARGUMENT, "polygon body index " + std::to_string(i) + " out of range");
            if (!(kind_h[i] & K_POLY))
                return fail(R2D_ERR_INVALID_ARGUMENT, "body " + std::to_string(i) + " is not a polygon (R2D_KIND_POLYGON)");
            if (nverts[k] < 3 || nverts[k] > MAX_POLY_VERTS)
                return fail(R2D_ERR_INVALID_ARGUMENT, "a polygon has 3 to 8 vertices, body " + std::to_string(i));
        }
        CUDA_TRY(wake());
        CUDA_TRY(cudaStreamSynchronize(stream));
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t i = body[k];
            poly_nv_h[i] = nverts[k];
            std::copy(verts + (size_t)k * 2 * MAX_POLY_VERTS, verts + (size_t)(k + 1) * 2 * MAX_POLY_VERTS,
                      poly_v_h.begin() + (size_t)i * 2 * MAX_POLY_VERTS);
            if (poly_aabb_pending[i]) {
                float ab[4];
                const size_t N = nbodies;
                init_aabb_polygon(state_h[(size_t)S_POS_X * N + i], state_h[(size_t)S_POS_Y * N + i],
                                  state_h[(size_t)S_ANGLE * N + i], verts + (size_t)k * 2 * MAX_POLY_VERTS, nverts[k],
                                  ab);
                for (int f = 0; f < 4; ++f) {
                    state_h[(size_t)(S_AABB_X + f) * N + i] = ab[f];
                    CUDA_TRY(cudaMemcpy(d_state + (size_t)(S_AABB_X + f) * N + i, &ab[f], sizeof(float),
                                        cudaMemcpyHostToDevice));
                }
                poly_aabb_pending[i] = 0;
            }
        }
        if (!d_poly_nv) {
            CUDA_TRY(dalloc(d_poly_nv, nbodies));
            CUDA_TRY(dalloc(d_poly_v, (size_t)nbodies * MAX_POLY_VERTS));
        }
        CUDA_TRY(cudaMemcpy(d_poly_nv, poly_nv_h.data(), nbodies, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_poly_v, poly_v_h.data(), sizeof(float) * poly_v_h.size(), cudaMemcpyHostToDevice));
        return R2D_OK;
    }

    // Any host write wakes every sleeping world (R2D_FLAG_SLEEP).
    cudaError_t wake() {
        return d_sleep ? cudaMemsetAsync(d_sleep, 0, sizeof(uint32_t) * nworlds, stream) : cudaSuccess;
    }

    int sleep_frames(uint32_t* out) {
        if (!d_sleep) {
            std::fill(out, out + nworlds, 0u);
            return R2D_OK;
        }
        CUDA_TRY(cudaStreamSynchronize(stream));
        CUDA_TRY(cudaMemcpy(out, d_sleep, sizeof(uint32_t) * nworlds, cudaMemcpyDeviceToHost));
        return R2D_OK;
    }

    int write_state(const float* state) {
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        CUDA_TRY(wake());
        CUDA_TRY(cudaMemcpyAsync(d_state, state, sizeof(float) * S_NFIELDS * nbodies, cudaMemcpyHostToDevice, stream));
        if (d_pos64) CUDA_TRY(upload_pose64(state));  // the f64 pose restarts from the written f32 one
        return R2D_OK;
    }

    // Rows [first, first + count) of the field-major state: one contiguous
    // copy each way.
    int write_fields(uint32_t first, uint32_t count, const float* rows) {
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        if (first > (uint32_t)S_NFIELDS || count > (uint32_t)S_NFIELDS - first)
            return fail(R2D_ERR_INVALID_ARGUMENT, "field range beyond the 13 state fields");
        if (!count || !nbodies) return R2D_OK;
        CUDA_TRY(wake());
        CUDA_TRY(cudaMemcpyAsync(d_state + (size_t)first * nbodies, rows, sizeof(float) * count * nbodies,
                                 cudaMemcpyHostToDevice, stream));
        if (d_pos64 && first < 3) {  // the f64 pose restarts from the written f32 pose rows
            const uint32_t end = std::min(3u, first + count);
            std::vector<double> p((size_t)(end - first) * nbodies);
            for (size_t k = 0; k < p.size(); ++k) p[k] = (double)rows[k];
            CUDA_TRY(cudaMemcpyAsync(d_pos64 + (size_t)first * nbodies, p.data(), sizeof(double) * p.size(),
                                     cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaStreamSynchronize(stream));
        }
        return R2D_OK;
    }

    int read_fields(uint32_t first, uint32_t count, float* rows) {
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        if (first > (uint32_t)S_NFIELDS || count > (uint32_t)S_NFIELDS - first)
            return fail(R2D_ERR_INVALID_ARGUMENT, "field range beyond the 13 state fields");
        if (!count || !nbodies) return R2D_OK;
        CUDA_TRY(cudaMemcpyAsync(rows, d_state + (size_t)first * nbodies, sizeof(float) * count * nbodies,
                                 cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return R2D_OK;
    }

    bool fp64_positions() const { return (cfg.flags & R2D_FLAG_FP64_POSITIONS) != 0; }
    bool warm_start() const { return (cfg.flags & R2D_FLAG_WARM_START) != 0; }
    bool sleeping() const { return (cfg.flags & R2D_FLAG_SLEEP) != 0; }
    bool compensated() const { return (cfg.flags & R2D_FLAG_COMPENSATED) != 0; }

    static uint32_t pow2_at_least(uint32_t v) {
        uint32_t p = 1;
        while (p < v) p <<= 1;
        return p;
    }

    // (Re)lays out the fused worlds' warm tables for the capacities `nm`
    // of their classes (0 for grid-pipeline worlds), carrying last frame's
    // entries over; a no-op when nothing changed.
    int layout_warm(const std::vector<uint32_t>& nm) {
        std::vector<uint32_t> hs(nworlds, 0), off(nworlds, 0);
        size_t total = 0;
        for (uint32_t w = 0; w < nworlds; ++w) {
            hs[w] = nm[w] ? pow2_at_least(2u * nm[w] + 2u) : 0u;
            off[w] = (uint32_t)total;
            total += 2ull * hs[w];
        }
        if (hs == warm_hs_h && d_warm_keys) return R2D_OK;
        unsigned long long* keys = nullptr;
        uint32_t *doff = nullptr, *dhs = nullptr;
        float4 *vals = nullptr, *cvals = nullptr;
        CUDA_TRY(dalloc(keys, std::max<size_t>(total, 1)));
        CUDA_TRY(dalloc(vals, std::max<size_t>(total, 1)));
        if (compensated()) CUDA_TRY(dalloc(cvals, std::max<size_t>(total, 1)));
        CUDA_TRY(dalloc(doff, nworlds));
        CUDA_TRY(dalloc(dhs, nworlds));
        CUDA_TRY(cudaMemcpyAsync(doff, off.data(), 4 * nworlds, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(dhs, hs.data(), 4 * nworlds, cudaMemcpyHostToDevice, stream));
        const WarmTables old_t{d_warm_keys, d_warm_vals, d_warm_cvals, d_warm_off, d_warm_keys ? d_warm_hs : nullptr};
        const WarmTables new_t{keys, vals, cvals, doff, dhs};
        CUDA_TRY(launch_migrate_warm(nworlds, old_t, d_warm_cur, new_t, stream));
        CUDA_TRY(cudaMemsetAsync(d_warm_cur, 0, sizeof(uint32_t) * nworlds, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        dfree(d_warm_keys); dfree(d_warm_vals); dfree(d_warm_cvals); dfree(d_warm_off); dfree(d_warm_hs);
        d_warm_keys = keys;
        d_warm_vals = vals;
        d_warm_cvals = cvals;
        d_warm_off = doff;
        d_warm_hs = dhs;
        warm_hs_h = hs;
        warm_off_h = off;
        for (uint32_t w = 0; w < nworlds; ++w) {
            worlds_h[w].warm_hs = hs[w];
            worlds_h[w].warm_off = off[w];
        }
        return R2D_OK;
    }

    // Every world's last-frame warm-start entries, from the device tables
    // of the current store (fused tables and grid-pipeline worlds alike),
    // into warm_carry[w] (world w of the current store).
    int take_warm_entries() {
        // entries taken at an earlier upload and not yet placed (no step
        // since) are still the last frame's: keep them
        if (!warm_carry.empty()) return R2D_OK;
        warm_carry.assign(nworlds, {});
        if (nworlds == 0) return R2D_OK;
        CUDA_TRY(cudaStreamSynchronize(stream));
        std::vector<unsigned long long> k;
        std::vector<float4> v, c;
        std::vector<uint32_t> cur(nworlds, 0);
        if (d_warm_keys && d_warm_cur) {
            size_t total = 0;
            for (uint32_t w = 0; w < nworlds; ++w) total = std::max<size_t>(total, (size_t)warm_off_h[w] + 2ull * warm_hs_h[w]);
            k.resize(total);
            v.resize(total);
            c.assign(total, make_float4(0.f, 0.f, 0.f, 0.f));
            CUDA_TRY(cudaMemcpy(cur.data(), d_warm_cur, 4 * nworlds, cudaMemcpyDeviceToHost));
            CUDA_TRY(cudaMemcpy(k.data(), d_warm_keys, 8 * total, cudaMemcpyDeviceToHost));
            CUDA_TRY(cudaMemcpy(v.data(), d_warm_vals, 16 * total, cudaMemcpyDeviceToHost));
            if (d_warm_cvals) CUDA_TRY(cudaMemcpy(c.data(), d_warm_cvals, 16 * total, cudaMemcpyDeviceToHost));
        }
        for (uint32_t w = 0; w < nworlds; ++w) {
            auto& out = warm_carry[w];
            if (w < world_large.size() && world_large[w]) {
                if (!large[w]) continue;
                std::vector<unsigned long long> lk;
                std::vector<float4> lv, lc;
                std::string msg;
                if (const int r = large[w]->read_warm(&lk, &lv, &lc, stream, &msg)) return fail(r, msg);
                for (size_t q = 0; q < lk.size(); ++q)
                    if (lk[q] != ~0ull) out.push_back(WarmEntry{lk[q], lv[q], lc[q]});
            } else if (w < warm_hs_h.size() && warm_hs_h[w] && !k.empty()) {
                const size_t at = (size_t)warm_off_h[w] + (size_t)cur[w] * warm_hs_h[w];
                for (size_t q = at; q < at + warm_hs_h[w]; ++q)
                    if (k[q] != ~0ull) out.push_back(WarmEntry{k[q], v[q], c[q]});
            }
        }
        return R2D_OK;
    }

    // The carried entries into the new store's tables (after plan has laid
    // them out, table 0 current): a fused world's are inserted on the host
    // with the device's hash and probing and uploaded; a grid-pipeline
    // world's are seeded into its own tables.
    int put_warm_entries() {
        if (warm_carry.empty()) return R2D_OK;
        auto build = [](const std::vector<WarmEntry>& es, uint32_t hs, std::vector<unsigned long long>& k,
                        std::vector<float4>& v, std::vector<float4>& c) {
            k.assign(hs, ~0ull);
            v.assign(hs, make_float4(0.f, 0.f, 0.f, 0.f));
            c.assign(hs, make_float4(0.f, 0.f, 0.f, 0.f));
            uint32_t taken = 0;
            for (const WarmEntry& e : es) {
                if (2 * (taken + 1) > hs) break;  // at most half full, as the device keeps it
                const uint32_t mask = hs - 1u;
                for (uint32_t probe = 0, h = warm_hash(e.key); probe < hs; ++probe) {
                    const uint32_t slot = (h + probe) & mask;
                    if (k[slot] != ~0ull) continue;
                    k[slot] = e.key;
                    v[slot] = e.val;
                    c[slot] = e.cval;
                    ++taken;
                    break;
                }
            }
        };
        std::vector<unsigned long long> k;
        std::vector<float4> v, c;
        for (uint32_t w = 0; w < nworlds && w < warm_carry.size(); ++w) {
            const auto& es = warm_carry[w];
            if (es.empty()) continue;
            if (world_large[w]) {
                const uint32_t hs = pow2_at_least(2u * (uint32_t)es.size() + 2u);
                build(es, hs, k, v, c);
                unsigned long long* dk = nullptr;
                float4 *dv = nullptr, *dc = nullptr;
                CUDA_TRY(dalloc(dk, hs));
                CUDA_TRY(dalloc(dv, hs));
                CUDA_TRY(dalloc(dc, hs));
                CUDA_TRY(cudaMemcpy(dk, k.data(), 8ull * hs, cudaMemcpyHostToDevice));
                CUDA_TRY(cudaMemcpy(dv, v.data(), 16ull * hs, cudaMemcpyHostToDevice));
                CUDA_TRY(cudaMemcpy(dc, c.data(), 16ull * hs, cudaMemcpyHostToDevice));
                std::string msg;
                const int r = large[w]->seed_warm(dk, dv, compensated() ? dc : nullptr, hs, stream, &msg);
                dfree(dk);
                dfree(dv);
                dfree(dc);
                if (r) return fail(r, msg);
            } else if (warm_hs_h[w] && d_warm_keys) {
                const uint32_t hs = warm_hs_h[w];
                build(es, hs, k, v, c);
                const size_t at = warm_off_h[w];  // table 0: plan left every world's current table at 0
                CUDA_TRY(cudaMemcpy(d_warm_keys + at, k.data(), 8ull * hs, cudaMemcpyHostToDevice));
                CUDA_TRY(cudaMemcpy(d_warm_vals + at, v.data(), 16ull * hs, cudaMemcpyHostToDevice));
                if (d_warm_cvals) CUDA_TRY(cudaMemcpy(d_warm_cvals + at, c.data(), 16ull * hs, cudaMemcpyHostToDevice));
            }
        }
        warm_carry.clear();
        return R2D_OK;
    }

    // d_pos64 = the pose fields of a host f32 state, widened.
    cudaError_t upload_pose64(const float* state) {
        std::vector<double> p((size_t)3 * nbodies);
        for (size_t f = 0; f < 3; ++f)
            for (size_t i = 0; i < nbodies; ++i) p[f * nbodies + i] = (double)state[f * nbodies + i];
        cudaError_t e = cudaMemcpyAsync(d_pos64, p.data(), sizeof(double) * p.size(), cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return e;
        return cudaStreamSynchronize(stream);  // p is released on return
    }

    int read_pose64(double* out) {
        if (!d_pos64) return fail(R2D_ERR_INVALID_ARGUMENT, "FP64 positions are off (R2D_FLAG_FP64_POSITIONS)");
        CUDA_TRY(cudaStreamSynchronize(stream));
        CUDA_TRY(cudaMemcpy(out, d_pos64, sizeof(double) * 3 * nbodies, cudaMemcpyDeviceToHost));
        return R2D_OK;
    }

    int read_state(float* state) {
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        CUDA_TRY(cudaMemcpyAsync(state, d_state, sizeof(float) * S_NFIELDS * nbodies, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return R2D_OK;
    }

    // Joints / exclusions already resolved to world-local indices.
    int set_constraints(const std::vector<uint32_t>& jworld, const std::vector<uint8_t>& jtype,
                        const std::vector<uint32_t>& jb1, const std::vector<uint32_t>& jb2,
                        const std::vector<float>& jprm, const std::vector<uint32_t>& xworld,
                        const std::vector<unsigned long long>& xkey) {
        // joints are grouped per world in the order given (insertion order inside a world)
        njoints = (uint32_t)jtype.size();
        ++joint_epoch;  // the grid pipeline's cached joint colourings are stale
        CUDA_TRY(wake());
        std::vector<uint32_t> order(njoints);
        for (uint32_t j = 0; j < njoints; ++j) order[j] = j;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return jworld[a] < jworld[b]; });
        std::vector<uint8_t> t(njoints);
        std::vector<uint32_t> b1(njoints), b2(njoints);
        std::vector<float> p((size_t)njoints * JOINT_PARAMS);
        for (auto& d : worlds_h) {
            d.joint_off = 0;
            d.nj = 0;
            d.excl_off = 0;
            d.nexcl = 0;
            d.flags &= ~W_DISC_ROTATION;
        }
        for (uint32_t k = 0; k < njoints; ++k) {
            const uint32_t j = order[k];
            t[k] = jtype[j];
            b1[k] = jb1[j];
            b2[k] = jb2[j];
            std::copy(jprm.begin() + (size_t)j * JOINT_PARAMS, jprm.begin() + (size_t)(j + 1) * JOINT_PARAMS,
                      p.begin() + (size_t)k * JOINT_PARAMS);
            WorldDesc& d = worlds_h[jworld[j]];
            if (d.nj == 0) d.joint_off = k;
            d.nj++;
            if (jtype[j] == J_OFFSET) d.flags |= W_DISC_ROTATION;
        }
        nexcl = (uint32_t)xkey.size();
        std::vector<std::pair<uint32_t, unsigned long long>> xs(nexcl);
        for (uint32_t k = 0; k < nexcl; ++k) xs[k] = {xworld[k], xkey[k]};
        std::sort(xs.begin(), xs.end());
        xs.erase(std::unique(xs.begin(), xs.end()), xs.end());
        nexcl = (uint32_t)xs.size();
        std::vector<unsigned long long> xk(nexcl);
        for (uint32_t k = 0; k < nexcl; ++k) {
            const uint32_t w = xs[k].first;
            xk[k] = xs[k].second;
            WorldDesc& d = worlds_h[w];
            if (d.nexcl == 0) d.excl_off = k;
            d.nexcl++;
        }
        CUDA_TRY(dalloc(d_jtype, njoints));
        CUDA_TRY(dalloc(d_jb1, njoints));
        CUDA_TRY(dalloc(d_jb2, njoints));
        CUDA_TRY(dalloc(d_jprm, (size_t)njoints * JOINT_PARAMS));
        CUDA_TRY(dalloc(d_excl, nexcl));
        if (njoints) {
            CUDA_TRY(cudaMemcpyAsync(d_jtype, t.data(), njoints, cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaMemcpyAsync(d_jb1, b1.data(), 4 * njoints, cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaMemcpyAsync(d_jb2, b2.data(), 4 * njoints, cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaMemcpyAsync(d_jprm, p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice, stream));
        }
        if (nexcl) CUDA_TRY(cudaMemcpyAsync(d_excl, xk.data(), 8 * nexcl, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        plan_dirty = true;
        return R2D_OK;
    }

    // Capacity of a world class sized from the worlds it holds.  Settled
    // piles of the benchmark worlds peak near 2.8 manifolds and 3.1 contact
    // points per body; a world that still outgrows a buffer is replayed with
    // every capacity doubled (see sync), so these are sizes, not limits.
    Caps caps_for(uint32_t nb, uint32_t max_nj, float rect_frac, uint32_t max_cells, uint32_t boost) const {
        const double base = cfg.capacity_scale > 0.f ? cfg.capacity_scale : 1.0;
        auto sz = [&](double v, int which) {
            const double k = base * std::pow(1.25, (double)boost_of(boost, which));
            return (uint32_t)std::min(65535.0, std::max(4.0, std::ceil(v * k)));
        };
        Caps c{};
        c.nb = nb;
        c.nm = sz(2.25 * nb + 16.0, 0);
        const double ppm = 1.08 + 0.92 * (double)rect_frac * rect_frac;
        c.npt = sz((2.25 * nb + 16.0) * ppm + 16.0, 1);
        c.ne = sz(std::max(2.5 * nb + 64.0, max_cells * 1.25 + 64.0), 2);
        c.np = sz(3.25 * nb + 32.0, 3);
        c.hs = c.np;
        c.nj = max_nj;
        // a class bound times a large multiplier may pass 32 bits: such a
        // layout cannot fit shared memory, and the world takes the grid pipeline
        c.nt = (uint32_t)std::min<unsigned long long>((unsigned long long)table_mult * nb, 1ull << 28);
        return c;
    }

    // Cell width of a world's binning grid (WorldDesc::fine_cell): the
    // largest dynamic body's diameter plus twice the binning margin, so that
    // such a body covers at most 2 x 2 cells; between 1/16 of the spatial
    // hash's cell and that cell.
    float fine_cell_of(uint32_t w) const {
        const WorldDesc& d = worlds_h[w];
        const uint32_t n = nbodies;
        float dmax = 0.f;
        for (uint32_t i = d.body_off; i < d.body_off + d.n; ++i) {
            if (kind_h[i] & K_STATIC) continue;
            const float d0 = props_h[(size_t)P_DIM0 * n + i], d1 = props_h[(size_t)P_DIM1 * n + i];
            const float dia = (kind_h[i] & K_RECT) ? std::sqrt(d0 * d0 + d1 * d1) : 2.0f * d0;
            if (dia > dmax) dmax = dia;
        }
        if (!(dmax > 0.f)) return cell;
        return std::min(cell, std::max(cell / 16.0f, fine_scale * (dmax + 0.05f)));
    }

    // Expected binning-grid cells of world w: a dynamic body covers 1-4
    // cells (2.25 on average is planned for; more replays), a static body
    // its AABB's span.
    uint32_t fine_cells_of_world(uint32_t w) const {
        const WorldDesc& d = worlds_h[w];
        const uint32_t n = nbodies;
        const float g = d.fine_cell > 0.f ? d.fine_cell : fine_cell_of(w);
        double total = 0.0;
        for (uint32_t i = d.body_off; i < d.body_off + d.n; ++i) {
            if (!(kind_h[i] & K_STATIC)) {
                total += 2.25;
                continue;
            }
            const double hw = state_h[(size_t)S_AABB_HW * n + i], hh = state_h[(size_t)S_AABB_HH * n + i];
            total += (std::floor(2.0 * hw / g) + 2.0) * (std::floor(2.0 * hh / g) + 2.0);
        }
        return total > 65535.0 ? 65535u : (uint32_t)std::ceil(total);
    }

    LayoutOpts layout_opts(bool lean, bool multi_substep) const {
        const bool debug = (cfg.flags & R2D_FLAG_DEBUG_TAPS) != 0;
        // debug taps report lever arms after integration: keep frame-start positions
        return LayoutOpts{lean, debug, multi_substep || debug, debug, compensated()};
    }

    // Shared memory a CTA may have (opt-in maximum) ...
    int smem_optin() const {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        return v;
    }
    // ... and the part a class's layout may take: the fused kernel's own
    // static shared memory (under 2 KB) comes off the top.
    int smem_limit() const { return smem_optin() - 2048; }

    KClass* class_of(uint32_t w) {
        for (auto& c : classes)
            if (std::find(c.worlds.begin(), c.worlds.end(), w) != c.worlds.end()) return &c;
        return nullptr;
    }

    // Threads per CTA for a class of `nb` bodies: a world's phases rarely
    // have more parallel items than this, and smaller CTAs let more worlds
    // share an SM.
    // Threads per CTA of a size class before autotuning: small worlds run
    // fastest as many small CTAs an SM (registers, not work, limit them).
    static int default_threads(uint32_t nb) { return nb <= 64 ? 32 : (nb <= 128 ? 64 : (nb <= 256 ? 128 : 256)); }

    // Picks each size class's threads per CTA by timing whole steps (all
    // classes running together, as in use) from the current state, which is
    // restored after every trial and at the end: two coordinate-descent passes
    // over the classes, candidates 32..512 threads, a candidate replacing the
    // standing choice only when 1.5 % faster.  Results do not depend on the
    // choice (the colouring, scans and solve order do not), only speed.
    int autotune(float dt, uint32_t sub_steps, uint32_t iters, uint32_t trial_steps) {
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        if (sub_steps == 0 || trial_steps == 0) return fail(R2D_ERR_INVALID_ARGUMENT, "sub_steps and trial steps >= 1");
        if (int st = sync()) return st;
        if (plan_dirty)
            if (int st = plan()) return st;
        float* saved = nullptr;
        double* saved64 = nullptr;
        CUDA_TRY(dalloc(saved, (size_t)S_NFIELDS * nbodies));
        if (d_pos64) CUDA_TRY(dalloc(saved64, (size_t)3 * nbodies));
        CUDA_TRY(cudaMemcpyAsync(saved, d_state, sizeof(float) * S_NFIELDS * nbodies, cudaMemcpyDeviceToDevice, stream));
        if (d_pos64)
            CUDA_TRY(cudaMemcpyAsync(saved64, d_pos64, sizeof(double) * 3 * nbodies, cudaMemcpyDeviceToDevice, stream));
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        int status = R2D_OK;
        auto restore = [&]() -> cudaError_t {
            cudaError_t e = cudaMemcpyAsync(d_state, saved, sizeof(float) * S_NFIELDS * nbodies,
                                            cudaMemcpyDeviceToDevice, stream);
            if (e == cudaSuccess && d_pos64)
                e = cudaMemcpyAsync(d_pos64, saved64, sizeof(double) * 3 * nbodies, cudaMemcpyDeviceToDevice, stream);
            return e;
        };
        // seconds per step of the current plan (best of three runs), or < 0 on error
        auto time_steps = [&]() -> float {
            float best = -1.f;
            for (int run = 0; run < 4; ++run) {
                if (restore() != cudaSuccess) return -1.f;
                if (run == 0) {  // plan, graph capture, capacity replays: untimed
                    if (process(dt, sub_steps, iters) || sync()) return -1.f;
                    continue;
                }
                if (cudaEventRecord(e0, stream) != cudaSuccess) return -1.f;
                for (uint32_t k = 0; k < trial_steps; ++k)
                    if (process(dt, sub_steps, iters)) return -1.f;
                if (cudaEventRecord(e1, stream) != cudaSuccess || sync()) return -1.f;
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) return -1.f;
                const float per = ms / 1e3f / (float)trial_steps;
                if (best < 0.f || per < best) best = per;
            }
            return best;
        };
        if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            status = fail(R2D_ERR_CUDA, "autotune events");
        } else {
            const uint32_t* bnd = CLASS_BOUNDS;
            static constexpr int cand[] = {32, 64, 128, 256, 512};
            std::vector<int> used(NBOUNDS, 0);
            for (const auto& c : classes)
                for (int k = 0; k < NBOUNDS; ++k)
                    if (c.caps.nb == bnd[k]) used[k] = 1;
            // two passes: a class's best tile depends on the others' (they
            // share the SMs), so the second pass revisits every class
            for (int pass = 0; pass < 2; ++pass)
            for (int k = 0; k < NBOUNDS && status == R2D_OK; ++k) {
                if (!used[k]) continue;
                const int start = thread_override[k] ? thread_override[k] : default_threads(bnd[k]);
                thread_override[k] = start;
                plan_dirty = true;
                float best_t = time_steps();
                int best = start;
                for (int nt : cand) {
                    if (nt == start || (bnd[k] > 192 && nt < 64) || (bnd[k] <= 64 && nt > 128) ||
                        (bnd[k] <= 256 && nt > 256))
                        continue;
                    thread_override[k] = nt;
                    plan_dirty = true;
                    const float t = time_steps();
                    // a change must beat the standing choice by more than the timing noise
                    if (t > 0.f && (best_t < 0.f || t < 0.985f * best_t)) {
                        best_t = t;
                        best = nt;
                    }
                }
                thread_override[k] = best;
                if (verbose) fprintf(stderr, "r2d: autotune class %u bodies -> %d threads (%.1f us/step)\n", bnd[k], best, best_t * 1e6f);
            }
            plan_dirty = true;
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        const cudaError_t er = restore();
        const cudaError_t es = cudaStreamSynchronize(stream);
        dfree(saved);
        dfree(saved64);
        if (status) return status;
        if (er != cudaSuccess || es != cudaSuccess) return fail(R2D_ERR_CUDA, "autotune: restoring the state");
        return R2D_OK;
    }

    void drop_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }

    int plan() {
        drop_graph();
        for (auto& c : classes) dfree(c.d_list);
        classes.clear();
        // size classes by body count: bounds in bodies
        const uint32_t* bounds = CLASS_BOUNDS;
        constexpr int nbnd = NBOUNDS;
        static_assert(CLASS_BOUNDS[NBOUNDS - 1] == FUSED_MAX_BODIES, "largest fused class");
        auto bound_of = [&](uint32_t n) {
            int k = 0;
            while (k < nbnd - 1 && n > bounds[k]) ++k;
            return k;
        };
        const int smem_optin = smem_limit();
        for (uint32_t w = 0; w < nworlds; ++w) worlds_h[w].fine_cell = fine_cell_of(w);
        // A world whose own buffers do not fit one CTA's shared memory (many
        // spatial-hash cells, say) takes the grid-wide pipeline.
        for (uint32_t w = 0; w < nworlds; ++w) {
            if (world_large[w]) continue;
            const WorldDesc& d = worlds_h[w];
            uint32_t rects = 0;
            for (uint32_t i = d.body_off; i < d.body_off + d.n; ++i) rects += (kind_h[i] & K_RECT) ? 1u : 0u;
            const uint32_t cells = fine_cells_of_world(w);
            const float rf = d.n ? (float)rects / (float)d.n : 0.f;
            const Caps c = caps_for(bounds[bound_of(d.n)], d.nj, rf, cells, world_boost[w]);
            if ((int)make_layout(c, layout_opts(!(world_boost[w] & BOOST_FULL), plan_multi_substep)).total > smem_optin)
                world_large[w] = 1;
        }
        std::vector<uint32_t> boosts;  // distinct boost patterns in use
        for (uint32_t w = 0; w < nworlds; ++w) {
            if (world_large[w]) continue;
            if (std::find(boosts.begin(), boosts.end(), world_boost[w]) == boosts.end()) boosts.push_back(world_boost[w]);
        }
        std::sort(boosts.begin(), boosts.end());
        const int NBOOST = (int)boosts.size();
        std::vector<std::vector<uint32_t>> groups(nbnd * NBOOST);
        for (uint32_t w = 0; w < nworlds; ++w) {
            if (world_large[w]) continue;
            const int k = bound_of(worlds_h[w].n);
            const int bi = (int)(std::find(boosts.begin(), boosts.end(), world_boost[w]) - boosts.begin());
            groups[k * NBOOST + bi].push_back(w);
        }
        for (int gk = 0; gk < nbnd * NBOOST; ++gk) {
            const int k = gk / NBOOST;
            const uint32_t boost = boosts[gk % NBOOST];
            if (groups[gk].empty()) continue;
            KClass kc;
            uint32_t max_nj = 0, max_cells = 0;
            float rect_frac = 0.f;
            for (uint32_t w : groups[gk]) {
                const WorldDesc& d = worlds_h[w];
                max_nj = std::max(max_nj, d.nj);
                uint32_t rects = 0;
                for (uint32_t i = d.body_off; i < d.body_off + d.n; ++i) rects += (kind_h[i] & K_RECT) ? 1u : 0u;
                const uint32_t cells = fine_cells_of_world(w);
                max_cells = std::max(max_cells, cells);
                if (d.n) rect_frac = std::max(rect_frac, (float)rects / (float)d.n);
            }
            kc.caps = caps_for(bounds[k], max_nj, rect_frac, max_cells, boost);
            kc.boost = boost;
            kc.opts = layout_opts(!(boost & BOOST_FULL), plan_multi_substep);
            // A world's phases rarely have more parallel items than this many
            // threads; smaller CTAs let more worlds share an SM.
            kc.threads = thread_override[k] ? thread_override[k] : default_threads(bounds[k]);
            kc.smem = make_layout(kc.caps, kc.opts).total;
            if ((int)kc.smem > smem_optin) {
                // each world fits alone, their maxima together do not
                for (uint32_t w : groups[gk]) world_large[w] = 1;
                continue;
            }
            // largest worlds first: the longest tasks start earliest
            std::stable_sort(groups[gk].begin(), groups[gk].end(),
                             [&](uint32_t a, uint32_t b) { return worlds_h[a].n > worlds_h[b].n; });
            kc.worlds = groups[gk];
            CUDA_TRY(dalloc(kc.d_list, kc.worlds.size()));
            CUDA_TRY(cudaMemcpyAsync(kc.d_list, kc.worlds.data(), 4 * kc.worlds.size(), cudaMemcpyHostToDevice, stream));
            classes.push_back(std::move(kc));
        }
        std::stable_sort(classes.begin(), classes.end(),
                         [](const KClass& a, const KClass& b) { return a.caps.nb > b.caps.nb; });
        // The block scheduler hands out every CTA of one launch before the
        // next launch's, in an order of its own, unless priorities say
        // otherwise.  Each priority level pairs a large body bound (the
        // longest CTAs, 70-150 KB of shared memory) with a small one (short
        // CTAs of 10-30 KB that fill the shared memory the large CTAs leave
        // on an SM): bounds ranked largest first, k-th and k-th from last on
        // level k, from the device's highest priority down.
        {
            int least = 0, greatest = 0;
            if (priority_map_set) {
                for (auto& c : classes) {
                    c.priority = 0;
                    for (const auto& kv : priority_map)
                        if (kv.first == c.caps.nb) c.priority = kv.second;
                }
            } else if (R2D_CLASS_PRIORITY && cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess &&
                       least > greatest) {
                std::vector<uint32_t> nbs;
                for (const auto& c : classes)
                    if (nbs.empty() || nbs.back() != c.caps.nb) nbs.push_back(c.caps.nb);
                const int D = (int)nbs.size();
                for (auto& c : classes) {
                    const int r = (int)(std::find(nbs.begin(), nbs.end(), c.caps.nb) - nbs.begin());
                    c.priority = std::min(greatest + std::min(r, D - 1 - r), least);
                }
            }
        }
        if (verbose) {
            fprintf(stderr, "r2d: plan: %zu classes (bound/boost: worlds, threads, shared B, priority):", classes.size());
            for (const auto& c : classes)
                fprintf(stderr, " %u/%u: %zu %d %u %d;", c.caps.nb, c.boost, c.worlds.size(), c.threads, c.smem,
                        c.priority);
            fprintf(stderr, "\n");
        }
        large_list.clear();
        for (uint32_t w = 0; w < nworlds; ++w) {
            if (!world_large[w]) continue;
            large_list.push_back(w);
            if (!large[w]) large[w].reset(new LargeWorld());
        }
        if (warm_start()) {
            std::vector<uint32_t> nm(nworlds, 0);
            for (const auto& c : classes)
                for (uint32_t w : c.worlds) nm[w] = c.caps.nm;
            if (int st = layout_warm(nm)) return st;
            if (int st = put_warm_entries()) return st;
        }
        for (auto& d : worlds_h) d.bucket_recip = bucket_recip(table_mult * d.n);
        CUDA_TRY(dalloc(d_worlds, nworlds));
        CUDA_TRY(cudaMemcpyAsync(d_worlds, worlds_h.data(), sizeof(WorldDesc) * nworlds, cudaMemcpyHostToDevice, stream));
        // debug taps
        dbg = DebugOut{};
        if (cfg.flags & R2D_FLAG_DEBUG_TAPS) {
            uint32_t cap = 0, jcap = 0, pcap = 0;
            for (auto& c : classes) {
                cap = std::max(cap, c.caps.nm);
                jcap = std::max(jcap, c.caps.nj);
                pcap = std::max(pcap, c.caps.np);
            }
            CUDA_TRY(dalloc(d_dbg_npairs, nworlds));
            CUDA_TRY(dalloc(d_dbg_pairs, (size_t)nworlds * (pcap ? pcap : 1) * 2));
            CUDA_TRY(cudaMemsetAsync(d_dbg_npairs, 0, 4 * nworlds, stream));
            dbg.pcap = pcap;
            dbg.npairs = d_dbg_npairs;
            dbg.pairs = d_dbg_pairs;
            CUDA_TRY(dalloc(d_dbg_nman, nworlds));
            CUDA_TRY(dalloc(d_dbg_keys, (size_t)nworlds * cap * 2));
            CUDA_TRY(dalloc(d_dbg_data, (size_t)nworlds * cap * DEBUG_MF));
            CUDA_TRY(dalloc(d_dbg_col, (size_t)nworlds * cap));
            CUDA_TRY(dalloc(d_dbg_jcol, (size_t)nworlds * (jcap ? jcap : 1)));
            CUDA_TRY(cudaMemsetAsync(d_dbg_nman, 0, 4 * nworlds, stream));
            dbg.cap = cap;
            dbg.nman = d_dbg_nman;
            dbg.keys = d_dbg_keys;
            dbg.data = d_dbg_data;
            dbg.colour = d_dbg_col;
            dbg.jcolour = d_dbg_jcol;
            dbg.jcap = jcap;
        }
        CUDA_TRY(cudaStreamSynchronize(stream));
        plan_dirty = false;
        return R2D_OK;
    }

    // The host rows the next steps read and write (null: none).  The device
    // copy changes between calls on `stream`, so a replayed graph reads it.
    cudaError_t set_ext(const float* force, float* out) {
        if (ext_cur.force == force && ext_cur.out == out) return cudaSuccess;
        ext_src.force = force;
        ext_src.out = out;
        const cudaError_t e = cudaMemcpyAsync(d_ext, &ext_src, sizeof(ExtIO), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) ext_cur = ext_src;
        return e;
    }

    // The address kernels use for a host buffer they may read or write
    // directly (pinned or managed), else null.
    static void* device_view(const void* p) {
        if (!p) return nullptr;
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;
        }
        if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeDevice)
            return a.devicePointer;
        return nullptr;
    }

    // One frame (r2d_*_process_io): the force/torque rows in, a step, the pose
    // and momentum rows out, synchronised.  Fused worlds read and write pinned
    // host rows directly over the CPU-GPU link; otherwise (pageable buffers,
    // grid-pipeline worlds, sleeping) the rows are copied around the step.
    int process_io(float dt, uint32_t sub_steps, uint32_t iters, const float* force, float* out) {
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        const float* dforce = static_cast<const float*>(device_view(force));
        float* dout = static_cast<float*>(device_view(out));
        const bool direct = (!force || dforce) && (!out || dout) && !sleeping() &&
                            std::none_of(world_large.begin(), world_large.end(), [](uint8_t v) { return v != 0; });
        if (!direct) {
            if (force) {
                if (int st = write_fields(S_FORCE_X, 3, force)) return st;
            }
            if (int st = process(dt, sub_steps, iters)) return st;
            if (int st = sync()) return st;
            return out ? read_fields(0, 6, out) : R2D_OK;
        }
        CUDA_TRY(set_ext(dforce, dout));
        if (int st = process_step(dt, sub_steps, iters)) return st;
        return sync();
    }

    int process(float dt, uint32_t sub_steps, uint32_t iters) {
        CUDA_TRY(set_ext(nullptr, nullptr));
        return process_step(dt, sub_steps, iters);
    }

    int process_step(float dt, uint32_t sub_steps, uint32_t iters) {
        if (sub_steps == 0) return fail(R2D_ERR_INVALID_ARGUMENT, "sub_steps must be >= 1");
        if (!d_state) return fail(R2D_ERR_INVALID_ARGUMENT, "no bodies");
        if (has_poly)
            for (uint32_t i = 0; i < nbodies; ++i)
                if ((kind_h[i] & K_POLY) && poly_nv_h[i] < 3)
                    return fail(R2D_ERR_INVALID_ARGUMENT,
                                "polygon body " + std::to_string(i) + " has no vertices (r2d_*_set_polygons)");
        if ((sub_steps > 1) != plan_multi_substep) {
            plan_multi_substep = sub_steps > 1;
            plan_dirty = true;
        }
        if (replan_in && --replan_in == 0) plan_dirty = true;
        if (plan_dirty) {
            int st = plan();
            if (st) return st;
        }
        if (!pending) CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), stream));
        calls.push_back(CallRec{dt, sub_steps, iters});
        pending = true;
        if (large_list.empty() && use_graph) {
            // the fused step alone: replay (or first capture) the graph
            if (!gexec || g_dt != dt || g_sub != sub_steps || g_iters != iters) {
                drop_graph();
                cudaGraph_t graph = nullptr;
                CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                const int st = enqueue_fused(dt, sub_steps, iters);
                const cudaError_t ec = cudaStreamEndCapture(stream, &graph);
                if (st) {
                    if (graph) cudaGraphDestroy(graph);
                    return st;
                }
                CUDA_TRY(ec);
                const cudaError_t ei = cudaGraphInstantiate(&gexec, graph, cudaGraphInstantiateFlagUseNodePriority);
                cudaGraphDestroy(graph);
                CUDA_TRY(ei);
                g_dt = dt;
                g_sub = sub_steps;
                g_iters = iters;
            }
            CUDA_TRY(cudaGraphLaunch(gexec, stream));
            return R2D_OK;
        }
        if (int st = enqueue_fused(dt, sub_steps, iters)) return st;
        if (!large_list.empty()) {
            // the fused launches above are queued: the large worlds' host-driven
            // pipelines run while they execute
            CUDA_TRY(cudaStreamWaitEvent(lstream, ev_fork, 0));
            for (uint32_t w : large_list) {
                int st = step_large(w, dt, sub_steps, iters, lstream);
                if (st) return st;
            }
            CUDA_TRY(cudaEventRecord(ev_ljoin, lstream));
            CUDA_TRY(cudaStreamWaitEvent(stream, ev_ljoin, 0));
        }
        return R2D_OK;
    }

    // One call of the fused kernel classes, forked from `stream` onto the
    // auxiliary streams and joined back; ev_fork also marks the point the
    // grid pipeline's stream waits for.
    int enqueue_fused(float dt, uint32_t sub_steps, uint32_t iters) {
        StepParams P = params(dt, sub_steps, iters, 0u);
        P.call_counter = d_call;
        CUDA_TRY(launch_count_call(d_call, stream));
        const int nused = (int)std::min<size_t>(classes.size(), (size_t)NAUX);
        CUDA_TRY(cudaEventRecord(ev_fork, stream));
        if (classes.size() == 1) {
            P.world_list = classes[0].d_list;
            P.nlist = (uint32_t)classes[0].worlds.size();
            cudaError_t e =
                launch_world_step(P, classes[0].caps, classes[0].threads, classes[0].opts, stream, classes[0].priority);
            if (e != cudaSuccess) return fail(R2D_ERR_CUDA, std::string("world step launch: ") + cudaGetErrorString(e));
        } else if (nused > 1) {
            for (int a = 0; a < nused; ++a) CUDA_TRY(cudaStreamWaitEvent(aux[a], ev_fork, 0));
            // one stream per class (classes beyond NAUX share): all run at once
            for (size_t i = 0; i < classes.size(); ++i) {
                const KClass& c = classes[i];
                P.world_list = c.d_list;
                P.nlist = (uint32_t)c.worlds.size();
                cudaError_t e = launch_world_step(P, c.caps, c.threads, c.opts, aux[i % NAUX], c.priority);
                if (e != cudaSuccess) return fail(R2D_ERR_CUDA, std::string("world step launch: ") + cudaGetErrorString(e));
            }
            for (int a = 0; a < nused; ++a) {
                CUDA_TRY(cudaEventRecord(ev_join[a], aux[a]));
                CUDA_TRY(cudaStreamWaitEvent(stream, ev_join[a], 0));
            }
        }
        return R2D_OK;
    }

    LargeInputs large_inputs(uint32_t w) const {
        const WorldDesc& d = worlds_h[w];
        LargeInputs in{};
        in.state = d_state;
        in.props = d_props;
        in.kind = d_kind;
        in.ids = d_ids;
        in.NB = nbodies;
        in.base = d.body_off;
        in.n = d.n;
        in.jtype = d_jtype + d.joint_off;
        in.jb1 = d_jb1 + d.joint_off;
        in.jb2 = d_jb2 + d.joint_off;
        in.jprm = d_jprm + (size_t)d.joint_off * JOINT_PARAMS;
        in.nj = d.nj;
        in.joint_epoch = joint_epoch;
        in.excl = d_excl + d.excl_off;
        in.nexcl = d.nexcl;
        in.ngrav = d.ngrav;
        for (int k = 0; k < MAX_GRAVITY; ++k) in.g[k] = d.g[k];
        in.cell = cell;
        in.table_mult = table_mult;
        in.disc_rot = (d.flags & W_DISC_ROTATION) != 0;
        in.pos64 = d_pos64;
        in.warm = warm_start();
        in.comp = compensated();
        in.verbose = verbose;
        in.sleep = d_sleep ? d_sleep + w : nullptr;
        in.colour_round_limit = colour_round_limit;
        in.poly_v = has_poly ? d_poly_v : nullptr;
        in.poly_nv = has_poly ? d_poly_nv : nullptr;
        return in;
    }

    // One call of a large world.  A world whose step fails (a non-finite
    // AABB, more than MAX_COLOURS colours) keeps the state before that call
    // and stays frozen until sync reports it, as a fused world does; CUDA
    // errors are returned at once.
    int step_large(uint32_t w, float dt, uint32_t sub_steps, uint32_t iters, cudaStream_t st) {
        if (large_frozen[w]) return R2D_OK;
        std::string msg;
        const int r = large[w]->step(large_inputs(w), dt, sub_steps, iters, st, &msg);
        large_status[w] = r;
        if (r == R2D_ERR_CUDA || r == R2D_ERR_OUT_OF_MEMORY) return fail(r, "world " + std::to_string(w) + ": " + msg);
        if (r != R2D_OK) {
            large_frozen[w] = 1;
            if (large_msg.empty()) large_msg = "world " + std::to_string(w) + ": " + msg;
        }
        return R2D_OK;
    }

    // First error of a large world since the last sync (0 if none); unfreezes them.
    int take_large_error(std::string* msg) {
        int first = R2D_OK;
        for (uint32_t w : large_list) {
            if (large_frozen[w] && first == R2D_OK) first = large_status[w];
            large_frozen[w] = 0;
        }
        *msg = large_msg;
        large_msg.clear();
        return first;
    }

    StepParams params(float dt, uint32_t sub_steps, uint32_t iters, uint32_t call_index) const {
        StepParams P{};
        P.worlds = d_worlds;
        P.state = d_state;
        P.props = d_props;
        P.kind = d_kind;
        P.ids = d_ids;
        P.nbodies = nbodies;
        P.jtype = d_jtype;
        P.jb1 = d_jb1;
        P.jb2 = d_jb2;
        P.jprm = d_jprm;
        P.excl = d_excl;
        P.world_status = d_status;
        P.error_count = d_err;
        P.dt = dt;
        P.sub_steps = sub_steps;
        P.iters = iters;
        P.cell = cell;
        P.table_mult = table_mult;
        P.dbg = dbg;
        P.world_fail_call = d_fail_call;
        P.world_capbits = d_capbits;
        P.call_index = call_index;
        P.timers = d_timers;
        P.pos64 = d_pos64;
        P.sleep = d_sleep;
        P.ext = d_ext;
        if (warm_start()) {
            P.warm_keys = d_warm_keys;
            P.warm_vals = d_warm_vals;
            P.warm_cvals = d_warm_cvals;
            P.warm_cur = d_warm_cur;
        }
        return P;
    }

    int sync() {
        CUDA_TRY(cudaStreamSynchronize(stream));
#ifdef R2D_PHASE_TIMERS
        dump_timers();
#endif
        if (!pending) return R2D_OK;
        pending = false;
        std::string lmsg;
        const int lerr = take_large_error(&lmsg);
        CUDA_TRY(cudaMemcpy(h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (*h_err == 0) {
            calls.clear();
            CUDA_TRY(cudaMemsetAsync(d_call, 0, sizeof(uint32_t), stream));
            if (lerr != R2D_OK) return fail(lerr, lmsg);
            return R2D_OK;
        }
        std::vector<uint32_t> fail_call(nworlds);
        status_h.resize(nworlds);
        CUDA_TRY(cudaMemcpy(status_h.data(), d_status, sizeof(int) * nworlds, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(fail_call.data(), d_fail_call, sizeof(uint32_t) * nworlds, cudaMemcpyDeviceToHost));
        int first_err = R2D_OK;
        std::string first_msg;
        for (uint32_t w = 0; w < nworlds && first_err == R2D_OK; ++w) {
            if (fail_call[w] == 0xFFFFFFFFu) continue;
            if (status_h[w] != DS_CAPACITY) {
                first_err = status_h[w];
                first_msg = "world " + std::to_string(w) + " failed with status " + std::to_string(status_h[w]);
                break;
            }
            int st = replay_escalated(w, fail_call[w]);
            if (st != R2D_OK) {
                first_err = st;
                first_msg = g_last_error;
            }
        }
        calls.clear();
        CUDA_TRY(cudaMemsetAsync(d_call, 0, sizeof(uint32_t), stream));
        plan_dirty = true;  // boosted worlds move to larger classes from the next call
        replan_in = R2D_REPLAN_TWICE ? 2u : 0u;
        if (first_err != R2D_OK) return fail(first_err, first_msg);
        if (lerr != R2D_OK) return fail(lerr, lmsg);
        return R2D_OK;
    }

#ifdef R2D_PHASE_TIMERS
    // Per size class: mean cycles per world-step of each phase, and counts.
    void dump_timers() {
        std::vector<unsigned long long> t((size_t)nworlds * PHASE_SLOTS);
        if (cudaMemcpy(t.data(), d_timers, 8 * t.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return;
        for (auto& c : classes) {
            double acc[PHASE_SLOTS] = {0};
            for (uint32_t w : c.worlds)
                for (int k = 0; k < PHASE_SLOTS; ++k) acc[k] += (double)t[(size_t)w * PHASE_SLOTS + k];
            const double steps = acc[11] > 0 ? acc[11] : 1;
            fprintf(stderr, "r2d timers nb=%u thr=%d worlds=%zu smem=%u | load %.0f bp %.0f [cells %.0f sort %.0f "
                            "cand %.0f compact %.0f] np %.0f col %.0f [sort %.0f walk %.0f] jcol %.0f solve %.0f "
                            "[forces %.0f prestep %.0f] wb %.0f | entries %.1f candidates %.1f pairs %.1f man %.1f "
                            "colours %.1f\n",
                    c.caps.nb, c.threads, c.worlds.size(), c.smem, acc[0] / steps, acc[1] / steps, acc[12] / steps,
                    acc[13] / steps, acc[14] / steps, acc[17] / steps, acc[2] / steps, acc[3] / steps,
                    acc[15] / steps, acc[16] / steps, acc[4] / steps, acc[5] / steps, acc[PT_FORCES] / steps,
                    acc[PT_PRESTEP] / steps, acc[6] / steps,
                    acc[19] / steps, acc[18] / steps, acc[7] / steps, acc[8] / steps, acc[9] / steps);
        }
        dump_timeline(t);
        cudaMemset(d_timers, 0, 8 * t.size());
    }

    // The last step's CTA timeline: when each size class started and ended,
    // how busy the SMs were over the step, and how long its tail was.
    void dump_timeline(const std::vector<unsigned long long>& t) {
        struct Cta {
            unsigned long long s, e;
            uint32_t sm;
        };
        std::vector<Cta> ctas;
        unsigned long long t0 = ~0ull, t1 = 0;
        for (uint32_t w = 0; w < nworlds; ++w) {
            const unsigned long long* r = &t[(size_t)w * PHASE_SLOTS];
            if (r[PT_END] <= r[PT_START] || !r[PT_START]) continue;
            ctas.push_back({r[PT_START], r[PT_END], (uint32_t)r[PT_SM]});
            t0 = std::min(t0, r[PT_START]);
            t1 = std::max(t1, r[PT_END]);
        }
        if (ctas.empty()) return;
        const double span = (double)(t1 - t0) * 1e-3;  // us
        for (auto& c : classes) {
            unsigned long long fs = ~0ull, ls = 0, le = 0;
            double dur = 0;
            size_t k = 0;
            for (uint32_t w : c.worlds) {
                const unsigned long long* r = &t[(size_t)w * PHASE_SLOTS];
                if (r[PT_END] <= r[PT_START] || !r[PT_START]) continue;
                fs = std::min(fs, r[PT_START]);
                ls = std::max(ls, r[PT_START]);
                le = std::max(le, r[PT_END]);
                dur += (double)(r[PT_END] - r[PT_START]);
                ++k;
            }
            if (!k) continue;
            fprintf(stderr, "r2d timeline nb=%u thr=%d worlds=%zu | first start %.1f us, last start %.1f, last end %.1f, "
                            "mean CTA %.1f us\n",
                    c.caps.nb, c.threads, k, (fs - t0) * 1e-3, (ls - t0) * 1e-3, (le - t0) * 1e-3, dur / k * 1e-3);
        }
        int nsm = 0;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        // per SM: the union of its CTAs' intervals, and its last end
        std::vector<std::vector<std::pair<unsigned long long, unsigned long long>>> per((size_t)std::max(nsm, 1));
        for (const Cta& c : ctas)
            if (c.sm < per.size()) per[c.sm].push_back({c.s, c.e});
        double busy = 0;
        std::vector<double> last;
        for (auto& v : per) {
            if (v.empty()) {
                last.push_back(0);
                continue;
            }
            std::sort(v.begin(), v.end());
            unsigned long long cs = v[0].first, ce = v[0].second, le = 0;
            for (auto& iv : v) {
                le = std::max(le, iv.second);
                if (iv.first > ce) {
                    busy += (double)(ce - cs);
                    cs = iv.first;
                    ce = iv.second;
                } else {
                    ce = std::max(ce, iv.second);
                }
            }
            busy += (double)(ce - cs);
            last.push_back((le - t0) * 1e-3);
        }
        std::sort(last.begin(), last.end());
        std::vector<double> ends;
        for (const Cta& c : ctas) ends.push_back((c.e - t0) * 1e-3);
        std::sort(ends.begin(), ends.end());
        const auto q = [](const std::vector<double>& v, double f) { return v[(size_t)(f * (v.size() - 1))]; };
        fprintf(stderr, "r2d timeline step: %.1f us from first CTA start to last end, %zu CTAs on %d SMs | SM busy %.1f %% "
                        "of SM-time | SM last end min %.1f median %.1f max %.1f us | 90 %% of CTAs ended by %.1f us, "
                        "99 %% by %.1f\n",
                span, ctas.size(), nsm, 100.0 * busy * 1e-3 / (span * std::max(nsm, 1)), last.front(),
                q(last, 0.5), last.back(), q(ends, 0.9), q(ends, 0.99));
    }
#endif

    // Debug taps hold `dbg.cap` manifolds per world; a world replayed with
    // larger buffers needs more.  Re-pitch every world's slots to the new cap.
    int grow_debug(uint32_t cap) {
        if (!dbg.cap || cap <= dbg.cap) return R2D_OK;
        uint32_t *keys = nullptr, *col = nullptr;
        float* data = nullptr;
        CUDA_TRY(dalloc(keys, (size_t)nworlds * cap * 2));
        CUDA_TRY(dalloc(data, (size_t)nworlds * cap * DEBUG_MF));
        CUDA_TRY(dalloc(col, (size_t)nworlds * cap));
        const size_t o = dbg.cap, h = nworlds;
        CUDA_TRY(cudaMemcpy2DAsync(keys, 8 * (size_t)cap, d_dbg_keys, 8 * o, 8 * o, h, cudaMemcpyDeviceToDevice, stream));
        CUDA_TRY(cudaMemcpy2DAsync(data, 4 * DEBUG_MF * (size_t)cap, d_dbg_data, 4 * DEBUG_MF * o, 4 * DEBUG_MF * o, h,
                                   cudaMemcpyDeviceToDevice, stream));
        CUDA_TRY(cudaMemcpy2DAsync(col, 4 * (size_t)cap, d_dbg_col, 4 * o, 4 * o, h, cudaMemcpyDeviceToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        dfree(d_dbg_keys);
        dfree(d_dbg_data);
        dfree(d_dbg_col);
        d_dbg_keys = keys;
        d_dbg_data = data;
        d_dbg_col = col;
        dbg.cap = cap;
        dbg.keys = keys;
        dbg.data = data;
        dbg.colour = col;
        return R2D_OK;
    }

    // Re-run world w from call `from` to the last logged call with every
    // capacity doubled, up to three times.  The world's state is exactly the
    // state before its failing call (a failing world writes nothing back).
    int replay_escalated(uint32_t w, uint32_t from) {
        KClass* kc = class_of(w);
        if (!kc) return fail(R2D_ERR_CAPACITY, "world " + std::to_string(w) + " has no class");
        if (!d_one) CUDA_TRY(dalloc(d_one, 1));
        CUDA_TRY(cudaMemcpyAsync(d_one, &w, sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        const WorldDesc& d = worlds_h[w];
        uint32_t rects = 0;
        for (uint32_t i = d.body_off; i < d.body_off + d.n; ++i) rects += (kind_h[i] & K_RECT) ? 1u : 0u;
        const uint32_t cells = fine_cells_of_world(w);
        const float rf = d.n ? (float)rects / (float)d.n : 0.f;
        uint32_t capbits = 0;
        CUDA_TRY(cudaMemcpy(&capbits, d_capbits + w, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        uint32_t boost = world_boost[w];
        for (int attempt = 0; attempt < 24; ++attempt) {
            if (capbits & (CAP_BODIES | CAP_JOINTS | CAP_COLOURS)) break;  // not a buffer size
            if (capbits & CAP_TGS) boost |= BOOST_FULL;
            const int which[4] = {CAP_MANIFOLDS, CAP_POINTS, CAP_ENTRIES, CAP_PAIRS};
            for (int i = 0; i < 4; ++i)
                // manifolds and points grow together (the colouring's sort
                // scratch lives in the point arrays)
                if ((capbits & which[i]) || (which[i] == CAP_MANIFOLDS && (capbits & CAP_POINTS)) ||
                    (which[i] == CAP_POINTS && (capbits & CAP_MANIFOLDS)))
                    boost += 1u << (8 * i);
            Caps c = caps_for(kc->caps.nb, kc->caps.nj, rf, cells, boost);
            const LayoutOpts opts = layout_opts(!(boost & BOOST_FULL), kc->opts.pos0);
            if (verbose)
                fprintf(stderr, "r2d: world %u (%u bodies) outgrew buffers 0x%x at call %u; replaying with "
                                "manifolds %u points %u entries %u pairs %u, %s layout (%u B shared)\n",
                        w, d.n, capbits, from, c.nm, c.npt, c.ne, c.np, opts.lean ? "lean" : "full",
                        make_layout(c, opts).total);
            if ((int)make_layout(c, opts).total > smem_limit()) break;
            if (int st = grow_debug(c.nm)) return st;
            if (warm_start() && warm_hs_h[w] < pow2_at_least(2u * c.nm + 2u)) {
                // the world's warm table must hold the larger manifold capacity
                std::vector<uint32_t> nm(nworlds, 0);
                for (const auto& kc2 : classes)
                    for (uint32_t w2 : kc2.worlds) nm[w2] = kc2.caps.nm;
                nm[w] = std::max(nm[w], c.nm);
                if (int st = layout_warm(nm)) return st;
                CUDA_TRY(cudaMemcpyAsync(d_worlds, worlds_h.data(), sizeof(WorldDesc) * nworlds,
                                         cudaMemcpyHostToDevice, stream));
            }
            CUDA_TRY(cudaMemsetAsync(d_fail_call + w, 0xFF, sizeof(uint32_t), stream));
            CUDA_TRY(cudaMemsetAsync(d_capbits + w, 0, sizeof(uint32_t), stream));
            CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), stream));
            for (uint32_t k = from; k < calls.size(); ++k) {
                StepParams P = params(calls[k].dt, calls[k].sub_steps, calls[k].iters, k);
                P.world_list = d_one;
                P.nlist = 1;
                cudaError_t e = launch_world_step(P, c, kc->threads, opts, stream);
                if (e != cudaSuccess) return fail(R2D_ERR_CUDA, std::string("replay launch: ") + cudaGetErrorString(e));
            }
            CUDA_TRY(cudaStreamSynchronize(stream));
            CUDA_TRY(cudaMemcpy(h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost));
            if (*h_err == 0) {
                world_boost[w] = boost;
                return R2D_OK;
            }
            int st = 0;
            uint32_t fc = 0;
            CUDA_TRY(cudaMemcpy(&st, d_status + w, sizeof(int), cudaMemcpyDeviceToHost));
            CUDA_TRY(cudaMemcpy(&fc, d_fail_call + w, sizeof(uint32_t), cudaMemcpyDeviceToHost));
            CUDA_TRY(cudaMemcpy(&capbits, d_capbits + w, sizeof(uint32_t), cudaMemcpyDeviceToHost));
            if (st != DS_CAPACITY)
                return fail(st, "world " + std::to_string(w) + " failed with status " + std::to_string(st));
            from = fc;
        }
        if (capbits & CAP_COLOURS)
            return fail(R2D_ERR_CAPACITY, "world " + std::to_string(w) + " needs more than " +
                                              std::to_string(MAX_COLOURS) + " colours");
        // Outgrew the largest shared-memory budget: from now on the world
        // steps through the large-world pipeline, starting with the calls
        // it has not done yet.
        if (verbose)
            fprintf(stderr, "r2d: world %u (%u bodies) moves to the large-world path at call %u\n", w, d.n, from);
        world_large[w] = 1;
        large[w].reset(new LargeWorld());
        if (warm_start() && d_warm_keys && warm_hs_h[w]) {
            // last frame's impulses go with the world
            uint32_t cur = 0;
            CUDA_TRY(cudaMemcpy(&cur, d_warm_cur + w, sizeof(uint32_t), cudaMemcpyDeviceToHost));
            const size_t at = (size_t)warm_off_h[w] + (size_t)cur * warm_hs_h[w];
            std::string msg;
            const int r = large[w]->seed_warm(d_warm_keys + at, d_warm_vals + at,
                                              d_warm_cvals ? d_warm_cvals + at : nullptr, warm_hs_h[w], stream, &msg);
            if (r) return fail(r, msg);
        }
        for (uint32_t k = from; k < calls.size(); ++k) {
            std::string msg;
            const int r = large[w]->step(large_inputs(w), calls[k].dt, calls[k].sub_steps, calls[k].iters, stream, &msg);
            large_status[w] = r;
            if (r != R2D_OK) return fail(r, "world " + std::to_string(w) + ": " + msg);
        }
        CUDA_TRY(cudaMemsetAsync(d_status + w, 0, sizeof(int), stream));
        return R2D_OK;
    }

    int world_status(int* out) {
        int st = sync();
        (void)st;
        status_h.assign(nworlds, 0);
        if (nworlds) CUDA_TRY(cudaMemcpy(status_h.data(), d_status, sizeof(int) * nworlds, cudaMemcpyDeviceToHost));
        for (uint32_t w = 0; w < nworlds; ++w)
            if (world_large[w]) status_h[w] = large_status[w];
        std::copy(status_h.begin(), status_h.end(), out);
        return R2D_OK;
    }

    bool debug_taps() const { return (cfg.flags & R2D_FLAG_DEBUG_TAPS) != 0; }

    int num_manifolds(uint32_t w, uint32_t* out) {
        if (!debug_taps()) return fail(R2D_ERR_INVALID_ARGUMENT, "debug taps are off (R2D_FLAG_DEBUG_TAPS)");
        if (w >= nworlds) return fail(R2D_ERR_INVALID_ARGUMENT, "world index out of range");
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (world_large[w]) {
            *out = large[w] ? large[w]->num_manifolds() : 0u;
            return R2D_OK;
        }
        CUDA_TRY(cudaMemcpy(out, d_dbg_nman + w, 4, cudaMemcpyDeviceToHost));
        return R2D_OK;
    }

    int get_manifolds(uint32_t w, uint32_t cap, uint32_t* keys, float* data, uint32_t* colours) {
        uint32_t m = 0;
        int st = num_manifolds(w, &m);
        if (st) return st;
        if (world_large[w]) {
            if (!large[w]) return R2D_OK;
            std::string msg;
            const int r = large[w]->dump(cap, keys, data, colours, stream, &msg);
            return r ? fail(r, msg) : R2D_OK;
        }
        m = std::min(m, std::min(cap, dbg.cap));
        const size_t o = (size_t)w * dbg.cap;
        if (keys) CUDA_TRY(cudaMemcpy(keys, d_dbg_keys + 2 * o, 8 * (size_t)m, cudaMemcpyDeviceToHost));
        if (data) CUDA_TRY(cudaMemcpy(data, d_dbg_data + o * DEBUG_MF, 4 * (size_t)m * DEBUG_MF, cudaMemcpyDeviceToHost));
        if (colours) CUDA_TRY(cudaMemcpy(colours, d_dbg_col + o, 4 * (size_t)m, cudaMemcpyDeviceToHost));
        return R2D_OK;
    }

    int num_pairs(uint32_t w, uint32_t* out) {
        if (!debug_taps()) return fail(R2D_ERR_INVALID_ARGUMENT, "debug taps are off (R2D_FLAG_DEBUG_TAPS)");
        if (w >= nworlds) return fail(R2D_ERR_INVALID_ARGUMENT, "world index out of range");
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (world_large[w]) {
            *out = large[w] ? large[w]->num_pairs() : 0u;
            return R2D_OK;
        }
        CUDA_TRY(cudaMemcpy(out, d_dbg_npairs + w, 4, cudaMemcpyDeviceToHost));
        return R2D_OK;
    }

    // The last frame's candidate pairs of world w, (lower, higher) world-local
    // body indices, sorted ascending (the device finds them in no fixed order).
    int get_pairs(uint32_t w, uint32_t cap, uint32_t* out) {
        uint32_t m = 0;
        if (int st = num_pairs(w, &m)) return st;
        if (world_large[w]) {
            m = std::min(m, cap);
            if (large[w] && m) {
                std::string msg;
                if (const int r = large[w]->dump_pairs(m, out, stream, &msg)) return fail(r, msg);
            }
        } else {
            m = std::min(m, std::min(cap, dbg.pcap));
            if (m)
                CUDA_TRY(cudaMemcpy(out, d_dbg_pairs + 2 * (size_t)w * dbg.pcap, 8 * (size_t)m,
                                    cudaMemcpyDeviceToHost));
        }
        std::vector<unsigned long long> k(m);
        for (uint32_t q = 0; q < m; ++q) k[q] = ((unsigned long long)out[2 * q] << 32) | out[2 * q + 1];
        std::sort(k.begin(), k.end());
        for (uint32_t q = 0; q < m; ++q) {
            out[2 * q] = (uint32_t)(k[q] >> 32);
            out[2 * q + 1] = (uint32_t)k[q];
        }
        return R2D_OK;
    }

    int get_joint_colours(uint32_t w, uint32_t cap, uint32_t* colours) {
        if (!debug_taps()) return fail(R2D_ERR_INVALID_ARGUMENT, "debug taps are off (R2D_FLAG_DEBUG_TAPS)");
        if (w >= nworlds) return fail(R2D_ERR_INVALID_ARGUMENT, "world index out of range");
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (world_large[w]) {
            if (!large[w]) return R2D_OK;
            std::string msg;
            const int r = large[w]->joint_colours(cap, colours, stream, &msg);
            return r ? fail(r, msg) : R2D_OK;
        }
        const uint32_t m = std::min(std::min(cap, dbg.jcap), worlds_h[w].nj);
        if (m) CUDA_TRY(cudaMemcpy(colours, d_dbg_jcol + (size_t)w * dbg.jcap, 4 * (size_t)m, cudaMemcpyDeviceToHost));
        return R2D_OK;
    }
};

// No C++ exception may cross the C ABI: allocation failures become statuses.
template <class F>
int guarded(F f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(R2D_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(R2D_ERR_INVALID_ARGUMENT, e.what());
    } catch (...) {
        return fail(R2D_ERR_INVALID_ARGUMENT, "unexpected exception");
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// single world
// ---------------------------------------------------------------------------
struct r2d_solver {
    Engine eng;
    std::vector<float> gravity;
    std::vector<uint8_t> jtype;
    std::vector<uint32_t> jid1, jid2;
    std::vector<float> jprm;
    std::vector<uint32_t> xpairs;
    bool constraints_dirty = false;
};

struct r2d_batch {
    Engine eng;
};

extern "C" {

R2D_API int r2d_version(void) { return 1; }

R2D_API const char* r2d_last_error_string(void) { return g_last_error.c_str(); }

R2D_API int r2d_solver_create(const r2d_config* cfg, r2d_solver** out) {
    if (!out) return fail(R2D_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    r2d_solver* s = new (std::nothrow) r2d_solver();
    if (!s) return fail(R2D_ERR_OUT_OF_MEMORY, "host allocation");
    int st = s->eng.init(cfg);
    if (st) {
        delete s;
        return st;
    }
    *out = s;
    return R2D_OK;
}

R2D_API int r2d_solver_destroy(r2d_solver* s) {
    if (!s) return fail(R2D_ERR_INVALID_ARGUMENT, "solver is NULL");
    cudaStreamSynchronize(s->eng.stream);
    delete s;
    return R2D_OK;
}

R2D_API int r2d_solver_set_bodies(r2d_solver* s, uint32_t n, const uint32_t* ids, const uint8_t* kind,
                                  const float* props, const float* state, int init_aabb) {
    if (!s || (n && (!ids || !kind || !props || !state))) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    const uint32_t off[2] = {0, n};
    const float* g = s->gravity.empty() ? nullptr : s->gravity.data();
    int st = guarded([&] { return s->eng.set_bodies(1, off, ids, kind, props, state, g, (uint32_t)s->gravity.size(), init_aabb); });
    if (st) return st;
    s->constraints_dirty = true;
    return R2D_OK;
}

R2D_API int r2d_solver_write_state(r2d_solver* s, const float* state) {
    if (!s || !state) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return s->eng.write_state(state); });
}

R2D_API int r2d_solver_read_state(r2d_solver* s, float* state) {
    if (!s || !state) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return s->eng.read_state(state); });
}

R2D_API int r2d_solver_set_gravity(r2d_solver* s, uint32_t n, const float* g) {
    if (!s || (n && !g)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n > (uint32_t)MAX_GRAVITY) return fail(R2D_ERR_INVALID_ARGUMENT, "at most 4 gravity generators");
    s->gravity.assign(g, g + n);
    if (!s->eng.worlds_h.empty()) {
        WorldDesc& d = s->eng.worlds_h[0];
        d.ngrav = n;
        for (uint32_t k = 0; k < n; ++k) d.g[k] = g[k];
        s->eng.plan_dirty = true;
        if (s->eng.wake() != cudaSuccess) return fail(R2D_ERR_CUDA, "waking the world failed");
    }
    return R2D_OK;
}

R2D_API int r2d_solver_set_joints(r2d_solver* s, uint32_t n, const uint8_t* type, const uint32_t* id1,
                                  const uint32_t* id2, const float* params) {
    if (!s || (n && (!type || !id1 || !id2 || !params))) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    for (uint32_t j = 0; j < n; ++j)
        if (type[j] > J_MOTOR) return fail(R2D_ERR_INVALID_ARGUMENT, "unknown joint type");
    s->jtype.assign(type, type + n);
    s->jid1.assign(id1, id1 + n);
    s->jid2.assign(id2, id2 + n);
    s->jprm.assign(params, params + (size_t)n * JOINT_PARAMS);
    s->constraints_dirty = true;
    return R2D_OK;
}

R2D_API int r2d_solver_set_exclusions(r2d_solver* s, uint32_t n, const uint32_t* pairs) {
    if (!s || (n && !pairs)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    s->xpairs.assign(pairs, pairs + 2 * (size_t)n);
    s->constraints_dirty = true;
    return R2D_OK;
}

static int solver_resolve(r2d_solver* s) {
    Engine& e = s->eng;
    std::unordered_map<uint32_t, uint32_t> idx;
    idx.reserve(e.nbodies * 2 + 1);
    for (uint32_t i = 0; i < e.nbodies; ++i) idx[e.ids_h[i]] = i;
    const uint32_t nj = (uint32_t)s->jtype.size();
    std::vector<uint32_t> jw(nj, 0);
    std::vector<uint32_t> b1(nj), b2(nj);
    for (uint32_t j = 0; j < nj; ++j) {
        auto a = idx.find(s->jid1[j]);
        if (a == idx.end()) return fail(R2D_ERR_INVALID_BODY_ID, "joint " + std::to_string(j) + " names an unknown body id");
        b1[j] = a->second;
        b2[j] = b1[j];
        if (s->jtype[j] == J_DISTANCE || s->jtype[j] == J_OFFSET) {
            auto b = idx.find(s->jid2[j]);
            if (b == idx.end())
                return fail(R2D_ERR_INVALID_BODY_ID, "joint " + std::to_string(j) + " names an unknown body id");
            b2[j] = b->second;
        }
    }
    const uint32_t nx = (uint32_t)(s->xpairs.size() / 2);
    std::vector<uint32_t> xw;
    std::vector<unsigned long long> xk;
    for (uint32_t k = 0; k < nx; ++k) {
        auto a = idx.find(s->xpairs[2 * k]), b = idx.find(s->xpairs[2 * k + 1]);
        if (a == idx.end() || b == idx.end()) continue;  // an exclusion of a missing body excludes nothing
        const uint32_t lo = std::min(a->second, b->second), hi = std::max(a->second, b->second);
        if (lo == hi) continue;
        xw.push_back(0);
        xk.push_back(((unsigned long long)lo << 32) | hi);
    }
    return e.set_constraints(jw, s->jtype, b1, b2, s->jprm, xw, xk);
}

R2D_API int r2d_solver_process(r2d_solver* s, float dt, uint32_t sub_steps, uint32_t collision_iters) {
    if (!s) return fail(R2D_ERR_INVALID_ARGUMENT, "solver is NULL");
    if (s->eng.nworlds == 0) return R2D_OK;  // no bodies: nothing to step
    if (s->constraints_dirty) {
        int st = guarded([&] { return solver_resolve(s); });
        if (st) return st;
        s->constraints_dirty = false;
    }
    return guarded([&] { return s->eng.process(dt, sub_steps, collision_iters); });
}

R2D_API int r2d_solver_process_io(r2d_solver* s, float dt, uint32_t sub_steps, uint32_t collision_iters,
                                  const float* force_rows, float* out_rows) {
    if (!s) return fail(R2D_ERR_INVALID_ARGUMENT, "solver is NULL");
    if (s->eng.nworlds == 0) return R2D_OK;
    if (s->constraints_dirty) {
        int st = guarded([&] { return solver_resolve(s); });
        if (st) return st;
        s->constraints_dirty = false;
    }
    return guarded([&] { return s->eng.process_io(dt, sub_steps, collision_iters, force_rows, out_rows); });
}

R2D_API int r2d_solver_sync(r2d_solver* s) {
    if (!s) return fail(R2D_ERR_INVALID_ARGUMENT, "solver is NULL");
    return guarded([&] { return s->eng.sync(); });
}

R2D_API int r2d_solver_num_manifolds(r2d_solver* s, uint32_t* out) {
    if (!s || !out) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return s->eng.num_manifolds(0, out); });
}

R2D_API int r2d_solver_get_manifolds(r2d_solver* s, uint32_t cap, uint32_t* keys, float* data, uint32_t* colours) {
    if (!s) return fail(R2D_ERR_INVALID_ARGUMENT, "solver is NULL");
    return guarded([&] { return s->eng.get_manifolds(0, cap, keys, data, colours); });
}

R2D_API int r2d_solver_write_state_fields(r2d_solver* s, uint32_t first, uint32_t count, const float* rows) {
    if (!s || (count && !rows)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return s->eng.write_fields(first, count, rows); });
}

R2D_API int r2d_solver_read_state_fields(r2d_solver* s, uint32_t first, uint32_t count, float* rows) {
    if (!s || (count && !rows)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return s->eng.read_fields(first, count, rows); });
}

R2D_API int r2d_solver_read_positions_f64(r2d_solver* s, double* pose) {
    if (!s || !pose) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return s->eng.read_pose64(pose); });
}

R2D_API int r2d_solver_set_polygons(r2d_solver* s, uint32_t n, const uint32_t* body, const uint8_t* nverts,
                                    const float* verts) {
    if (!s || (n && (!body || !nverts || !verts))) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL handle or array");
    return guarded([&] { return s->eng.set_polygons(n, body, nverts, verts); });
}

R2D_API int r2d_solver_num_pairs(r2d_solver* s, uint32_t* out) {
    if (!s || !out) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL handle or out pointer");
    return guarded([&] { return s->eng.num_pairs(0, out); });
}

R2D_API int r2d_solver_get_pairs(r2d_solver* s, uint32_t cap, uint32_t* pairs) {
    if (!s || (cap && !pairs)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL handle or pairs buffer");
    return guarded([&] { return s->eng.get_pairs(0, cap, pairs); });
}

R2D_API int r2d_solver_get_joint_colours(r2d_solver* s, uint32_t cap, uint32_t* colours) {
    if (!s || !colours) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return s->eng.get_joint_colours(0, cap, colours); });
}

// ---------------------------------------------------------------------------
// batch
// ---------------------------------------------------------------------------
R2D_API int r2d_batch_create(const r2d_config* cfg, r2d_batch** out) {
    if (!out) return fail(R2D_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    r2d_batch* b = new (std::nothrow) r2d_batch();
    if (!b) return fail(R2D_ERR_OUT_OF_MEMORY, "host allocation");
    int st = b->eng.init(cfg);
    if (st) {
        delete b;
        return st;
    }
    *out = b;
    return R2D_OK;
}

R2D_API int r2d_batch_destroy(r2d_batch* b) {
    if (!b) return fail(R2D_ERR_INVALID_ARGUMENT, "batch is NULL");
    cudaStreamSynchronize(b->eng.stream);
    delete b;
    return R2D_OK;
}

R2D_API int r2d_batch_set_worlds(r2d_batch* b, uint32_t nworlds, const uint32_t* body_off, const uint32_t* ids,
                                 const uint8_t* kind, const float* props, const float* state, const float* gravity,
                                 int init_aabb) {
    if (!b || !body_off || (nworlds && (!gravity))) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    const uint32_t n = body_off[nworlds];
    if (n && (!ids || !kind || !props || !state)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    int st = guarded([&] { return b->eng.set_bodies(nworlds, body_off, ids, kind, props, state, gravity, 1, init_aabb); });
    if (st) return st;
    for (auto& d : b->eng.worlds_h) {  // gravity 0 means no generator
        if (d.g[0] == 0.f) d.ngrav = 0;
    }
    std::vector<uint32_t> e32;
    std::vector<uint8_t> e8;
    std::vector<float> ef;
    std::vector<unsigned long long> e64;
    return guarded([&] { return b->eng.set_constraints(e32, e8, e32, e32, ef, e32, e64); });
}

R2D_API int r2d_batch_write_state(r2d_batch* b, const float* state) {
    if (!b || !state) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.write_state(state); });
}

R2D_API int r2d_batch_read_state(r2d_batch* b, float* state) {
    if (!b || !state) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.read_state(state); });
}

R2D_API int r2d_batch_write_state_fields(r2d_batch* b, uint32_t first, uint32_t count, const float* rows) {
    if (!b || (count && !rows)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.write_fields(first, count, rows); });
}

R2D_API int r2d_batch_read_state_fields(r2d_batch* b, uint32_t first, uint32_t count, float* rows) {
    if (!b || (count && !rows)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.read_fields(first, count, rows); });
}

R2D_API int r2d_batch_read_positions_f64(r2d_batch* b, double* pose) {
    if (!b || !pose) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.read_pose64(pose); });
}

R2D_API int r2d_batch_process(r2d_batch* b, float dt, uint32_t sub_steps, uint32_t collision_iters) {
    if (!b) return fail(R2D_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (b->eng.nworlds == 0) return R2D_OK;
    return guarded([&] { return b->eng.process(dt, sub_steps, collision_iters); });
}

R2D_API int r2d_batch_process_io(r2d_batch* b, float dt, uint32_t sub_steps, uint32_t collision_iters,
                                 const float* force_rows, float* out_rows) {
    if (!b) return fail(R2D_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (b->eng.nworlds == 0) return R2D_OK;
    return guarded([&] { return b->eng.process_io(dt, sub_steps, collision_iters, force_rows, out_rows); });
}

R2D_API int r2d_batch_sync(r2d_batch* b) {
    if (!b) return fail(R2D_ERR_INVALID_ARGUMENT, "batch is NULL");
    return guarded([&] { return b->eng.sync(); });
}

R2D_API int r2d_batch_autotune(r2d_batch* b, float dt, uint32_t sub_steps, uint32_t collision_iters,
                               uint32_t trial_steps) {
    if (!b) return fail(R2D_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (b->eng.nworlds == 0) return R2D_OK;
    return guarded([&] { return b->eng.autotune(dt, sub_steps, collision_iters, trial_steps); });
}

// One kernel per size class, plus the call counter of the step, plus what
// each grid-pipeline world launched in its latest step.
static int launches_of(Engine& eng, uint32_t* out) {
    if (eng.plan_dirty && eng.nworlds) {
        int st = eng.plan();
        if (st) return st;
    }
    uint32_t n = (uint32_t)eng.classes.size() + (eng.classes.empty() ? 0u : 1u);
    for (uint32_t w : eng.large_list)
        if (eng.large[w]) n += eng.large[w]->launches();
    *out = n;
    return R2D_OK;
}

R2D_API int r2d_batch_launches_per_step(r2d_batch* b, uint32_t* out) {
    if (!b || !out) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return launches_of(b->eng, out);
}

R2D_API int r2d_solver_launches_per_step(r2d_solver* s, uint32_t* out) {
    if (!s || !out) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return launches_of(s->eng, out);
}

R2D_API int r2d_solver_sleep_frames(r2d_solver* s, uint32_t* frames) {
    if (!s || !frames) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->eng.nworlds == 0) {
        *frames = 0;
        return R2D_OK;
    }
    return guarded([&] { return s->eng.sleep_frames(frames); });
}

R2D_API int r2d_batch_sleep_frames(r2d_batch* b, uint32_t* frames) {
    if (!b || (!frames && b->eng.nworlds)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.sleep_frames(frames); });
}

R2D_API int r2d_batch_world_status(r2d_batch* b, int* status) {
    if (!b || !status) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.world_status(status); });
}

R2D_API int r2d_batch_num_manifolds(r2d_batch* b, uint32_t w, uint32_t* out) {
    if (!b || !out) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded([&] { return b->eng.num_manifolds(w, out); });
}

R2D_API int r2d_batch_get_manifolds(r2d_batch* b, uint32_t w, uint32_t cap, uint32_t* keys, float* data,
                                    uint32_t* colours) {
    if (!b) return fail(R2D_ERR_INVALID_ARGUMENT, "batch is NULL");
    return guarded([&] { return b->eng.get_manifolds(w, cap, keys, data, colours); });
}

R2D_API int r2d_batch_set_polygons(r2d_batch* b, uint32_t n, const uint32_t* body, const uint8_t* nverts,
                                   const float* verts) {
    if (!b || (n && (!body || !nverts || !verts))) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL handle or array");
    return guarded([&] { return b->eng.set_polygons(n, body, nverts, verts); });
}

R2D_API int r2d_batch_num_pairs(r2d_batch* b, uint32_t w, uint32_t* out) {
    if (!b || !out) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL handle or out pointer");
    return guarded([&] { return b->eng.num_pairs(w, out); });
}

R2D_API int r2d_batch_get_pairs(r2d_batch* b, uint32_t w, uint32_t cap, uint32_t* pairs) {
    if (!b || (cap && !pairs)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL handle or pairs buffer");
    return guarded([&] { return b->eng.get_pairs(w, cap, pairs); });
}

// The allocation-free world step: validation here, the pipeline over the
// static scratch array in r2d_large.cu.
R2D_API int r2d_world_step_static(float* state, const float* props, const uint8_t* kind, const uint32_t* ids,
                                  uint32_t n, const float* gravity, uint32_t ngrav, float dt, uint32_t sub_steps,
                                  uint32_t collision_iters, float cell_width, uint32_t table_mult, void* stream) {
    if (n && (!state || !props || !kind || !ids)) return fail(R2D_ERR_INVALID_ARGUMENT, "NULL device buffer");
    if (ngrav > (uint32_t)MAX_GRAVITY || (ngrav && !gravity))
        return fail(R2D_ERR_INVALID_ARGUMENT, "at most 4 gravity generators, passed by a host array");
    if (sub_steps == 0) return fail(R2D_ERR_INVALID_ARGUMENT, "sub_steps must be >= 1");
    StaticStepArgs a{};
    a.state = state;
    a.props = props;
    a.kind = kind;
    a.ids = ids;
    a.n = n;
    a.ngrav = ngrav;
    for (uint32_t k = 0; k < ngrav; ++k) a.g[k] = gravity[k];
    a.dt = dt;
    a.sub_steps = sub_steps;
    a.iters = collision_iters;
    a.cell = cell_width > 0.f ? cell_width : 4.0f;
    a.table_mult = table_mult ? table_mult : 2u;
    std::string msg;
    const int r = static_world_step(a, (cudaStream_t)stream, &msg);
    return r ? fail(r, msg) : R2D_OK;
}

}  // extern "C"
