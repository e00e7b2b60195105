/*
 * r2d_world.cuh -- data layout shared by the host runtime and the fused
 * per-world step kernel.
 */
#pragma once

#include <stdint.h>

namespace r2d {

// Field-major f32 state: field f of body g lives at state[f * nbodies + g].
enum StateField : int {
    S_POS_X = 0, S_POS_Y, S_ANGLE, S_MOM_X, S_MOM_Y, S_ANG_MOM,
    S_FORCE_X, S_FORCE_Y, S_TORQUE, S_AABB_X, S_AABB_Y, S_AABB_HW, S_AABB_HH,
    S_NFIELDS
};
enum PropField : int { P_MASS = 0, P_INERTIA, P_MU, P_DIM0, P_DIM1, P_NFIELDS };
// K_POLY: a convex polygon (grid pipeline only; its vertices live beside the props)
enum KindBits : uint8_t { K_RECT = 1, K_STATIC = 2, K_POLY = 4, K_FORCED = 0x80 /* device-only: force/torque to clear */ };
enum JointTypes : uint8_t { J_DISTANCE = 0, J_OFFSET = 1, J_FIXED = 2, J_MOTOR = 3 };
enum WorldFlags : uint32_t { W_DISC_ROTATION = 2u };

constexpr int MAX_GRAVITY = 4;
constexpr int JOINT_PARAMS = 8;
constexpr int DEBUG_MF = 33;     // floats per manifold in the debug dump (oracle layout)
constexpr int MAX_COLOURS = 128; // per-body colour masks hold 128 colours

struct WorldDesc {
    uint32_t body_off, n;
    uint32_t joint_off, nj;
    uint32_t excl_off, nexcl;
    uint32_t ngrav, flags;
    float g[MAX_GRAVITY];
    // floor((2^64 - 1) / (table_mult * n)): Barrett reciprocal of the
    // spatial-hash table size, so the kernel needs no 64-bit division
    unsigned long long bucket_recip;
    // Cell width of the binning grid that finds candidate pairs: about one
    // body diameter, so a bucket holds a few bodies (the spatial hash's own
    // cells still decide which pairs are candidates).
    float fine_cell;
    // warm starting: this world's two tables of warm_hs slots start at
    // entry warm_off (table b at warm_off + b * warm_hs)
    uint32_t warm_hs;
    uint32_t warm_off;
    uint32_t pad_;
};

// Per-world capacities of one kernel class; every buffer below is sized
// from them, and a world that outgrows one is reported, never overrun.
struct Caps {
    uint32_t nb;   // bodies
    uint32_t nm;   // manifolds
    uint32_t npt;  // contact points
    uint32_t ne;   // (cell, body) entries of the spatial hash
    uint32_t np;   // candidate pairs that passed the AABB test
    uint32_t hs;   // candidate-pair list slots before the pairs are grouped (= np)
    uint32_t nj;   // joints
    uint32_t nt;   // spatial-hash buckets (table_mult * bodies)
};

// Byte offsets into the dynamic shared memory of one CTA.
struct Layout {
    // bodies (whole step)
    uint32_t px, py, ang, mom, inv_i, cs, sn, ang_prev, tq, px0, py0, kind;  // mom: (mx, my, L, inv_m) float4
    // manifolds + points (narrowphase .. end) -- aliased by the broadphase scratch
    uint32_t ma, mb, mp0, mnp, mcol, nx, ny, fric;
    uint32_t r1x, r1y, r2x, r2y, depth, odepth, mn, mt, apn, apt, bias;
    uint32_t cpn, cpt;  // compensation words (compensated mode; offset 0 = absent)
    // broadphase scratch (inside the manifold region)
    uint32_t ax, ay, ahw, ahh, rx0, ry0, rx1, ry1, fx0, fy0, fx1, fy1, bcnt, ebucket, ebody, eslot, sbody, table, hset;
    // colouring scratch: sort keys, per-body colour masks
    uint32_t skey, cmask;
    // optional arrays (offset 0 = absent)
    bool has_depth, has_pos0, has_prev, has_comp;
    // orders
    uint32_t corder, coff, jorder, joff, jcol;
    // pairs
    uint32_t pairs;
    uint32_t total;
};

__host__ __device__ inline uint32_t r2d_align(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

// Shared-memory layout of one world.
//   lean:  contact points keep their midpoint (8 B) instead of both lever arms
//          and the original depth; the lever arms are recomputed from the
//          frame-start positions.  Worlds with a TGS-live point use the full
//          layout (the kernel detects them).
//   depth: keep each point's depth (full layout, or debug taps)
//   pos0:  keep frame-start positions (lean with more than one substep;
//          with one substep the positions do not move before integration)
//   prev:  keep each body's previous-substep angle (full layout, debug taps)
//   comp:  keep a compensation word beside each accumulated impulse
//          (R2D_FLAG_COMPENSATED)
struct LayoutOpts {
    bool lean, depth, pos0, prev, comp;
};

__host__ __device__ inline Layout make_layout(const Caps& c, const LayoutOpts& f) {
    Layout L{};
    uint32_t o = 0;
    auto take = [&](uint32_t bytes) {
        uint32_t at = o;
        o = r2d_align(o + bytes, 16);
        return at;
    };
    const uint32_t nb4 = 4 * c.nb;
    L.has_depth = f.depth || !f.lean;
    L.has_pos0 = f.lean && f.pos0;
    L.has_prev = f.prev || !f.lean;
    L.has_comp = f.comp;
    L.px = take(nb4); L.py = take(nb4); L.ang = take(nb4);
    L.mom = take(4 * nb4); L.inv_i = take(nb4);
    L.cs = take(nb4); L.sn = take(nb4); L.tq = take(nb4);
    if (L.has_prev) L.ang_prev = take(nb4);
    if (L.has_pos0) {
        L.px0 = take(nb4);
        L.py0 = take(nb4);
    }
    L.kind = take(c.nb);

    // region X: manifolds + points, aliased by the broadphase scratch
    const uint32_t xbase = o;
    const uint32_t nm4 = 4 * c.nm, np4 = 4 * c.npt;
    L.ma = take(2 * c.nm); L.mb = take(2 * c.nm); L.mp0 = take(2 * c.nm);
    L.mnp = take(c.nm); L.mcol = take(c.nm);
    L.nx = take(nm4); L.ny = take(nm4); L.fric = take(nm4);
    L.r1x = take(np4); L.r1y = take(np4);  // lean: the contact midpoint
    if (!f.lean) {
        L.r2x = take(np4);
        L.r2y = take(np4);
        L.odepth = take(np4);
    }
    if (L.has_depth) L.depth = take(np4);
    L.bias = take(np4);
    // mn .. apt (.. cpt) are contiguous: the colouring sorts its keys there
    L.mn = take(np4); L.mt = take(np4);
    L.apn = take(np4); L.apt = take(np4);
    if (L.has_comp) {
        L.cpn = take(np4);
        L.cpt = take(np4);
    }
    const uint32_t xend_m = o;
    o = xbase;
    L.ax = take(nb4); L.ay = take(nb4); L.ahw = take(nb4); L.ahh = take(nb4);
    L.rx0 = take(nb4); L.ry0 = take(nb4); L.rx1 = take(nb4); L.ry1 = take(nb4);
    L.fx0 = take(nb4); L.fy0 = take(nb4); L.fx1 = take(nb4); L.fy1 = take(nb4);
    L.bcnt = take(4 * (c.nb + 1));
    L.ebucket = take(4 * c.ne); L.ebody = take(2 * c.ne); L.eslot = take(2 * c.ne);
    L.sbody = take(2 * c.ne);
    L.table = take(4 * (c.nt + 2));
    L.hset = take(4 * c.hs);
    const uint32_t xend_bp = o;
    o = xend_m > xend_bp ? xend_m : xend_bp;

    // orders
    L.corder = take(2 * c.nm);
    L.coff = take(2 * (MAX_COLOURS + 2));
    L.jorder = take(2 * (c.nj ? c.nj : 1));
    L.joff = take(2 * (MAX_COLOURS + 2));
    L.jcol = take(c.nj ? c.nj : 1);
    // candidate pairs (broadphase -> narrowphase); after the narrowphase the
    // per-body colour masks reuse them
    L.pairs = take(4 * c.np);
    L.cmask = (20 * c.nb <= 4 * c.np) ? L.pairs : take(20 * c.nb);  // 4 colour words + lane bits
    // sort keys of the colouring (8 B a constraint): the point arrays mn ..
    // apt are not live until after the colouring
    const uint32_t ncon = c.nm > c.nj ? c.nm : c.nj;
    L.skey = (8 * ncon <= (L.has_comp ? 6u : 4u) * np4) ? L.mn : take(8 * ncon);
    L.total = o;
    return L;
}

// Every fused world's warm-start tables: world w owns slots
// [off[w], off[w] + 2 * hs[w]) (two tables of hs[w] slots, a power of two).
struct WarmTables {
    unsigned long long* keys;  // (ref id << 32 | inc id); all ones = empty
    float4* vals;              // (pn0, pt0, pn1, pt1)
    float4* cvals;             // their compensation words, or null
    const uint32_t* off;       // [nworlds]
    const uint32_t* hs;        // [nworlds]
};

struct DebugOut {
    uint32_t cap;        // manifolds per world slot (0 = no dump)
    uint32_t* nman;      // [world]
    uint32_t* keys;      // [world][cap][2]  (reference, incident) world-local indices
    float* data;         // [world][cap][DEBUG_MF]
    uint32_t* colour;    // [world][cap]
    uint32_t* jcolour;   // [world][jcap]
    uint32_t jcap;
    // candidate pairs: the pairs that reach the narrowphase (every filter of
    // updateManifolds passed, lib.zig:264-282), in no particular order
    uint32_t pcap;       // pairs per world slot
    uint32_t* npairs;    // [world]
    uint32_t* pairs;     // [world][pcap][2]  (lower, higher) world-local indices
};

// Host rows a frame call reads and writes directly over the coherent
// CPU-GPU link (r2d_*_process_io): the frame's force and torque [3][nbodies]
// and the pose and momenta it returns [6][nbodies], field-major like the
// state.  Null pointers: the state rows are the only inputs and outputs.
struct ExtIO {
    const float* force;
    float* out;
};

struct StepParams {
    const WorldDesc* worlds;
    const uint32_t* world_list;  // worlds handled by this launch
    uint32_t nlist;
    float* state;                // [S_NFIELDS][nbodies]
    const float* props;          // [P_NFIELDS][nbodies]
    const uint8_t* kind;         // [nbodies]
    const uint32_t* ids;         // [nbodies]
    uint32_t nbodies;
    const uint8_t* jtype;        // [njoints]
    const uint32_t* jb1;         // world-local body index
    const uint32_t* jb2;
    const float* jprm;           // [njoints][JOINT_PARAMS]
    const unsigned long long* excl;  // sorted ((u64)lo << 32 | hi) per world
    int* world_status;           // [nworlds]
    uint32_t* world_fail_call;   // [nworlds] first call a world failed in; ~0u = healthy
    uint32_t* world_capbits;     // [nworlds] CAP_* bits of the buffers that overflowed
    int* error_count;
    uint32_t call_index;         // position of this launch in the calls since the last sync ...
    const uint32_t* call_counter;  // ... or, when set, *call_counter - 1 (bumped on the device per call)
    unsigned long long* timers;  // [nworlds][PHASE_SLOTS] when built with R2D_PHASE_TIMERS
    double* pos64;               // [3][nbodies] x, y, angle in f64 (FP64-positions mode), else null
    unsigned long long* warm_keys;  // warm-start tables (WorldDesc::warm_off): (ref id << 32 | inc id), else null
    float4* warm_vals;           // (pn0, pt0, pn1, pt1)
    float4* warm_cvals;          // their compensation words (compensated mode), else null
    uint32_t* warm_cur;          // [nworlds] which of a world's two tables holds last frame
    uint32_t* sleep;             // [nworlds] consecutive still frames (sleeping mode, r2d_sleep.h), else null
    const ExtIO* ext;            // this call's host rows (device copy, read per call), else null
    float dt;
    uint32_t sub_steps, iters;
    float cell;
    uint32_t table_mult;
    DebugOut dbg;
};

// Phase timer slots (cycles, R2D_PHASE_TIMERS builds only): load,
// broadphase, narrowphase, contact colouring, joint colouring, solve,
// write-back, then counts: pairs, manifolds, colours, colouring rounds.
// 12..19: sub-phases (cells, bucket sort, colour sort, colour walk) and
// counts.  20..22: the CTA's timeline in the last step (not summed):
// %globaltimer at its start and end, in ns, and the SM it ran on.  23, 24:
// the solve phase's forces and prestep passes (cycles).
constexpr int PHASE_SLOTS = 25;
constexpr int PT_START = 20, PT_END = 21, PT_SM = 22, PT_FORCES = 23, PT_PRESTEP = 24;

// Which per-world buffer overflowed (reported with DS_CAPACITY).
enum CapBits : uint32_t {
    CAP_BODIES = 1u, CAP_MANIFOLDS = 2u, CAP_POINTS = 4u, CAP_ENTRIES = 8u,
    CAP_PAIRS = 16u, CAP_COLOURS = 32u, CAP_JOINTS = 64u,
    CAP_TGS = 128u  // a TGS-live contact point: the world needs the full layout
};

enum DeviceStatus : int {
    DS_OK = 0,
    DS_CAPACITY = -5,
    DS_TIMEOUT = -6,   // a bounded device-side loop gave up (R2D_ERR_TIMEOUT)
    DS_NONFINITE = -7,
};

}  // namespace r2d
