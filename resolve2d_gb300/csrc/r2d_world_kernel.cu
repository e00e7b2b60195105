/*
 * r2d_world_kernel.cu -- one CTA steps one whole world: the body state is
 * loaded into shared memory once, and the spatial-hash broadphase
 * (src/core/SpatialHash.zig), the SAT narrowphase and manifold build
 * (src/core/collision.zig:221-363, Bodies/{Disc,Rectangle,RigidBody}.zig), the constraint colouring,
 * the substep loop of Solver.process (src/core/lib.zig:189-251: forces,
 * velocities, prestep, joint + contact impulses, integration) and the state
 * write-back all run from shared memory.  HBM sees each body's state once in
 * and once out per step.
 *
 * Constraint order.  The reference solves joints then manifolds one at a
 * time (lib.zig:226-236).  Here each set is coloured into body-disjoint
 * batches (first-fit greedy in the priority order of r2d_colour.h, computed
 * by Jones-Plassmann rounds), and one colour is solved per barrier phase.
 * Inside a colour no two constraints share a non-static body, so the result
 * equals the reference's per-constraint arithmetic replayed colour by colour.
 * No floating-point atomics are used anywhere: every run is bit-reproducible.
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "r2d_device.cuh"
#include "r2d_sleep.h"
#include "r2d_solve.cuh"
#include "r2d_world.cuh"

namespace r2d {

namespace cg = cooperative_groups;

template <int NT>
__device__ uint32_t block_scan_excl(uint32_t* a, uint32_t n, uint32_t* wsum) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
    const uint32_t per = (n + NT - 1) / NT;
    const uint32_t beg = min(n, (uint32_t)tid * per), end = min(n, beg + per);
    uint32_t s = 0;
    for (uint32_t i = beg; i < end; ++i) s += a[i];
    uint32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < NW ? wsum[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane < NW) wsum[lane] = v;
    }
    __syncthreads();
    uint32_t run = (warp ? wsum[warp - 1] : 0u) + x - s;
    const uint32_t total = wsum[NW - 1];
    for (uint32_t i = beg; i < end; ++i) {
        uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
    return total;
}

// Exclusive scan of one u64 value per thread across the block; *total gets
// the block's sum.  Shared scratch: 32 words.
template <int NT>
__device__ unsigned long long block_scan_value_u64(unsigned long long v, unsigned long long* wsum,
                                                   unsigned long long* total) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < NW ? wsum[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < NW) wsum[lane] = w;
    }
    __syncthreads();
    const unsigned long long before = (warp ? wsum[warp - 1] : 0ull) + x - v;
    *total = wsum[NW - 1];
    __syncthreads();
    return before;
}

// Cell of entry e of body i: entries are emitted row by row over the body's
// cell range, starting at its prefix offset `start`.
__device__ __forceinline__ void entry_cell(uint32_t e, uint32_t start, int32_t x0, int32_t x1, int32_t y0,
                                           int32_t* x, int32_t* y) {
    const uint32_t t = e - start, wx = (uint32_t)(x1 - x0) + 1u;
    if (wx == 1u) {
        *x = x0;
        *y = y0 + (int32_t)t;
    } else if (wx == 2u) {
        *x = x0 + (int32_t)(t & 1u);
        *y = y0 + (int32_t)(t >> 1);
    } else {
        *x = x0 + (int32_t)(t % wx);
        *y = y0 + (int32_t)(t / wx);
    }
}

// Whether bodies i and j share a bucket of the reference's spatial hash,
// given their cell ranges (SpatialHash.zig:78-137): a common cell, or two
// cells whose buckets collide.
__device__ __forceinline__ bool shares_bucket(uint32_t i, uint32_t j, const int32_t* rx0, const int32_t* ry0,
                                              const int32_t* rx1, const int32_t* ry1, const BucketMod& bmod) {
    if (max(rx0[i], rx0[j]) <= min(rx1[i], rx1[j]) && max(ry0[i], ry0[j]) <= min(ry1[i], ry1[j])) return true;
    for (int32_t yi = ry0[i]; yi <= ry1[i]; ++yi)
        for (int32_t xi = rx0[i]; xi <= rx1[i]; ++xi) {
            const uint32_t bi = cell_bucket(xi, yi, bmod);
            for (int32_t yj = ry0[j]; yj <= ry1[j]; ++yj)
                for (int32_t xj = rx0[j]; xj <= rx1[j]; ++xj)
                    if (cell_bucket(xj, yj, bmod) == bi) return true;
        }
    return false;
}

__device__ __forceinline__ bool excluded(const unsigned long long* ex, uint32_t n, unsigned long long key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        unsigned long long v = __ldg(ex + mid);
        if (v == key) return true;
        if (v < key) lo = mid + 1;
        else hi = mid;
    }
    return false;
}

__device__ __forceinline__ void set_err(int* s_err, int code) { atomicCAS(s_err, 0, code); }
__device__ __forceinline__ void cap_fail(int* err, uint32_t* s_capbits, uint32_t bit) {
    *err = DS_CAPACITY;
    atomicOr(s_capbits, bit);
}

// Orders constraints 0..count-1 into skey[0..count) by (mix, tie): a
// counting sort on the top 8 bits of the mix (mixes are uniform hashes, so
// each of the 256 buckets holds a few constraints), then an insertion sort of
// each bucket by the full (mix, tie) key.  skey[k] = mix << 32 | index.
template <int NT, class Mix, class Tie>
__device__ void priority_order(uint32_t count, Mix mix, Tie tie, unsigned long long* skey, uint32_t* bucket,
                               uint32_t* wsum) {
    const int tid = threadIdx.x;
    if (count <= 128u && count <= (uint32_t)NT) {
        // Few constraints: each thread ranks its own against all the others
        // (the keys are distinct), one pass and two barriers instead of the
        // counting sort's scans.  The 256-word bucket array holds the keys.
        unsigned long long* keys = reinterpret_cast<unsigned long long*>(bucket);
        uint32_t h = 0, tv = 0;
        if ((uint32_t)tid < count) {
            h = mix((uint32_t)tid);
            tv = tie((uint32_t)tid);
            keys[tid] = ((unsigned long long)h << 32) | tv;
        }
        __syncthreads();
        if ((uint32_t)tid < count) {
            const unsigned long long mine = ((unsigned long long)h << 32) | tv;
            uint32_t rank = 0;
            for (uint32_t j = 0; j < count; ++j) rank += keys[j] < mine ? 1u : 0u;
            skey[rank] = ((unsigned long long)h << 32) | (uint32_t)tid;
        }
        __syncthreads();
        return;
    }
    for (uint32_t b = tid; b < 256; b += NT) bucket[b] = 0u;
    __syncthreads();
    for (uint32_t i = tid; i < count; i += NT) atomicAdd(&bucket[mix(i) >> 24], 1u);
    __syncthreads();
    block_scan_excl<NT>(bucket, 256, wsum);  // bucket[b] = first slot of bucket b
    for (uint32_t i = tid; i < count; i += NT) {
        const uint32_t h = mix(i);
        skey[atomicAdd(&bucket[h >> 24], 1u)] = ((unsigned long long)h << 32) | i;
    }
    __syncthreads();  // bucket[b] = one past the last slot of bucket b
    for (uint32_t b = tid; b < 256; b += NT) {
        const uint32_t lo = b ? bucket[b - 1] : 0u, hi = bucket[b];
        for (uint32_t x = lo + 1; x < hi; ++x) {
            const unsigned long long v = skey[x];
            const uint32_t hv = (uint32_t)(v >> 32), tv = tie((uint32_t)v);
            uint32_t y = x;
            while (y > lo) {
                const unsigned long long u = skey[y - 1];
                const uint32_t hu = (uint32_t)(u >> 32);
                if (hu < hv || (hu == hv && tie((uint32_t)u) < tv)) break;
                skey[y] = u;
                --y;
            }
            skey[y] = v;
        }
    }
    __syncthreads();
}

// Colours `count` constraints by first-fit greedy in ascending priority
// order (mix(i), then tie(i); unique per constraint; r2d_colour.h).  The
// constraints are put in priority order (priority_order); then one warp walks
// the sorted list 32 at a time.  A lane takes the lowest colour absent from
// its nodes' colour masks once every earlier lane of its chunk that shares a
// node is coloured, so the result is exactly the sequential greedy colouring,
// computed with warp shuffles instead of block-wide rounds.  ends(i, &a, &b)
// names constraint i's conflict nodes (values >= 0x10000 mean "no node").
// Returns true on every thread when some constraint would need more than
// MAX_COLOURS colours; *ncolours (shared) gets the number of colours used.
// bucket: 256 words of shared scratch.
template <int NT, class Ends, class Mix, class Tie, class Hook>
__device__ bool colour_greedy_sorted(uint32_t count, uint32_t n, Ends ends, Mix mix, Tie tie, uint8_t* colour,
                                     unsigned long long* skey, uint32_t* cmask, uint32_t* bucket, uint32_t* wsum,
                                     uint32_t* ncolours, Hook SUBPHASE_HOOK) {
    const int tid = threadIdx.x, lane = tid & 31;
    for (uint32_t i = tid; i < 5 * n; i += NT) cmask[i] = 0u;
    priority_order<NT>(count, mix, tie, skey, bucket, wsum);
    SUBPHASE_HOOK();
    int overflow = 0;
    if (tid < 32) {
        uint32_t used = 0;  // colours this lane handed out: the highest + 1
        uint32_t* lanebits = cmask + 4 * n;  // per node: lanes of this chunk that name it
        auto fetch = [&](uint32_t base, uint32_t* ci, uint32_t* a, uint32_t* b, bool* valid) {
            const uint32_t i = base + lane;
            *valid = i < count;
            *ci = *valid ? (uint32_t)skey[i] : 0u;
            *a = 0x10000u + 2u * lane;
            *b = 0x10001u + 2u * lane;
            if (*valid) ends(*ci, a, b);
        };
        uint32_t ci, a, b;
        bool valid;
        fetch(0, &ci, &a, &b, &valid);
        for (uint32_t base = 0; base < count; base += 32) {
            const bool na = a < 0x10000u, nb2 = b < 0x10000u;
            if (na) atomicOr(&lanebits[a], 1u << lane);
            if (nb2) atomicOr(&lanebits[b], 1u << lane);
            __syncwarp();
            // earlier lanes of this chunk sharing a node
            const uint32_t earlier = ((na ? lanebits[a] : 0u) | (nb2 ? lanebits[b] : 0u)) & ((1u << lane) - 1u);
            __syncwarp();
            if (na) lanebits[a] = 0u;
            if (nb2) lanebits[b] = 0u;
            uint32_t nci, nxa, nxb;  // the next chunk, fetched while this one resolves
            bool nvalid;
            fetch(base + 32, &nci, &nxa, &nxb, &nvalid);
            bool done = !valid;
            for (int round = 0; round < 32; ++round) {
                const uint32_t pending = __ballot_sync(0xffffffffu, !done);
                if (!pending) break;
                if (!done && !(earlier & pending)) {
                    // the lowest free colour, reading a mask word only when
                    // every colour below it is taken (colours are nearly
                    // always below 32)
                    // (the words read are current -- no other lane of this
                    // round names a or b -- so they are written back without
                    // being read again)
                    uint32_t c = 128u, wa = 0u, wb = 0u;
                    for (uint32_t q = 0; q < 4; ++q) {
                        wa = na ? cmask[q * n + a] : 0u;
                        wb = nb2 ? cmask[q * n + b] : 0u;
                        if ((wa | wb) != 0xFFFFFFFFu) {
                            c = 32u * q + (uint32_t)__ffs(~(wa | wb)) - 1u;
                            break;
                        }
                    }
                    if (c >= (uint32_t)MAX_COLOURS) {
                        overflow = 1;
                        colour[ci] = 0u;
                    } else {
                        colour[ci] = (uint8_t)c;
                        if (na) cmask[(c >> 5) * n + a] = wa | (1u << (c & 31u));
                        if (nb2) cmask[(c >> 5) * n + b] = wb | (1u << (c & 31u));
                        used = max(used, c + 1u);
                    }
                    done = true;
                }
                __syncwarp();
            }
            ci = nci;
            a = nxa;
            b = nxb;
            valid = nvalid;
        }
        used = __reduce_max_sync(0xffffffffu, used);
        if (lane == 0) *ncolours = used;
    }
    return __syncthreads_or(overflow) != 0;
}

using SW = SWT<uint16_t, true>;

// Worlds of at most this many bodies test every pair of bodies directly
// instead of binning them (the same pairs; fewer scans and barriers).
#ifndef R2D_BRUTE_MAX_BODIES
#define R2D_BRUTE_MAX_BODIES 96
#endif

// Bodies with more spatial-hash entries than this are emitted by the whole
// block (up to MAX_BIG_BODIES of them; more fall back to their own thread).
constexpr uint32_t BIG_BODY_ENTRIES = 16, MAX_BIG_BODIES = 16;

// Register budget per thread: low enough that several worlds share an SM
// (the kernel is latency-bound; concurrency hides it).
#ifndef R2D_REG_TARGET
#define R2D_REG_TARGET 96
#endif
// One-warp CTAs keep 96 registers: below that they spill.
constexpr int reg_target_for(int nt) { return nt <= 32 ? 96 : R2D_REG_TARGET; }
constexpr int min_blocks_for(int nt) {
    return 65536 / (nt * reg_target_for(nt)) > 0 ? 65536 / (nt * reg_target_for(nt)) : 1;
}

template <int NT, bool LEAN>
__global__ void __launch_bounds__(NT, min_blocks_for(NT)) world_step_kernel(const StepParams P, const Caps C,
                                                                               const Layout Lo) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ uint32_t s_wsum[32];
    __shared__ __align__(16) uint32_t s_ccnt[256];  // also 128 u64 sort keys (priority_order)
    __shared__ int s_err;
    __shared__ uint32_t s_capbits;
    __shared__ uint32_t s_cnt[4];  // pairs, manifolds, points
    __shared__ unsigned long long s_wsum64[32];
    __shared__ uint32_t s_big[MAX_BIG_BODIES];  // bodies whose cell entries the whole block emits
    __shared__ uint32_t s_nbig;
    __shared__ uint32_t s_ncol;  // colours of the last colouring

    const int tid = threadIdx.x;
    if (blockIdx.x >= P.nlist) return;
    const uint32_t w = P.world_list[blockIdx.x];
    const WorldDesc wd = P.worlds[w];
    const uint32_t n = wd.n, base = wd.body_off, NB = P.nbodies;
    const uint32_t T = P.table_mult * n;
    // A world that failed earlier in this batch of calls stays frozen (its
    // state untouched) until the host replays it with larger capacities.
    if (P.world_fail_call[w] != 0xFFFFFFFFu) return;
    // a sleeping world is not stepped (r2d_sleep.h); a frame call still gets its pose
    if (P.sleep && P.sleep[w] >= R2D_SLEEP_FRAMES) {
        float* out = P.ext ? P.ext->out : nullptr;
        for (uint32_t i = tid; out && i < n; i += NT)
            for (int f = 0; f < 6; ++f) out[(size_t)f * NB + base + i] = P.state[(size_t)f * NB + base + i];
        if (tid == 0) P.world_status[w] = DS_OK;
        return;
    }
    if (n > C.nb || wd.nj > C.nj || T > C.nt || n > 65535u) {
        if (tid == 0) {
            P.world_status[w] = DS_CAPACITY;
            P.world_capbits[w] = (n > C.nb || T > C.nt || n > 65535u ? CAP_BODIES : 0u) | (wd.nj > C.nj ? CAP_JOINTS : 0u);
            P.world_fail_call[w] = P.call_counter ? *P.call_counter - 1u : P.call_index;
            atomicAdd(P.error_count, 1);
        }
        return;
    }
    if (tid == 0) {
        s_err = 0;
        s_capbits = 0u;
        s_cnt[0] = s_cnt[1] = s_cnt[2] = s_cnt[3] = 0;
    }
    int err = 0;
#ifdef R2D_PHASE_TIMERS
    if (tid == 0 && P.timers) {
        unsigned long long gt;
        uint32_t sm;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(gt));
        asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
        P.timers[(size_t)w * PHASE_SLOTS + PT_START] = gt;
        P.timers[(size_t)w * PHASE_SLOTS + PT_SM] = sm;
    }
    long long t_mark = clock64();
    const uint32_t jp_rounds = 0;
    long long t_sub = t_mark;
#define PHASE(k)                                                              \
    do {                                                                      \
        __syncthreads();                                                      \
        if (tid == 0 && P.timers) {                                           \
            const long long t_now = clock64();                                \
            P.timers[(size_t)w * PHASE_SLOTS + (k)] += (unsigned long long)(t_now - t_mark); \
            t_mark = t_now;                                                   \
            t_sub = t_now;                                                    \
        }                                                                     \
    } while (0)
#define SUBPHASE(k)                                                           \
    do {                                                                      \
        __syncthreads();                                                      \
        if (tid == 0 && P.timers) {                                           \
            const long long t_now = clock64();                                \
            P.timers[(size_t)w * PHASE_SLOTS + (k)] += (unsigned long long)(t_now - t_sub); \
            t_sub = t_now;                                                    \
        }                                                                     \
    } while (0)
#else
#define PHASE(k) \
    do {         \
    } while (0)
#define SUBPHASE(k) \
    do {            \
    } while (0)
#endif

#define SMF(off) reinterpret_cast<float*>(sm + (off))
#define SMU32(off) reinterpret_cast<uint32_t*>(sm + (off))
#define SMU16(off) reinterpret_cast<uint16_t*>(sm + (off))
#define SMU8(off) reinterpret_cast<uint8_t*>(sm + (off))
#define SMI32(off) reinterpret_cast<int32_t*>(sm + (off))

    SW s;
    s.px = SMF(Lo.px); s.py = SMF(Lo.py); s.ang = SMF(Lo.ang);
    s.mx = s.my = s.L = s.inv_m = nullptr;
    s.mom4 = reinterpret_cast<float4*>(sm + Lo.mom);
    s.inv_i = SMF(Lo.inv_i);
    s.cs = SMF(Lo.cs); s.sn = SMF(Lo.sn); s.ang_prev = SMF(Lo.ang_prev); s.tq = SMF(Lo.tq);
    s.px0 = SMF(Lo.px0); s.py0 = SMF(Lo.py0);
    s.pos0 = Lo.has_pos0;
    s.gmass = P.props + (size_t)P_MASS * NB + base;
    s.ginertia = P.props + (size_t)P_INERTIA * NB + base;
    s.kind = SMU8(Lo.kind);
    s.ma = SMU16(Lo.ma); s.mb = SMU16(Lo.mb); s.mp0 = SMU16(Lo.mp0);
    s.mnp = SMU8(Lo.mnp); s.mcol = SMU8(Lo.mcol);
    s.nx = SMF(Lo.nx); s.ny = SMF(Lo.ny); s.fric = SMF(Lo.fric);
    s.r1x = SMF(Lo.r1x); s.r1y = SMF(Lo.r1y); s.r2x = SMF(Lo.r2x); s.r2y = SMF(Lo.r2y);
    s.depth = SMF(Lo.depth); s.odepth = SMF(Lo.odepth); s.mn = SMF(Lo.mn); s.mt = SMF(Lo.mt);
    s.apn = SMF(Lo.apn); s.apt = SMF(Lo.apt); s.bias = SMF(Lo.bias);
    s.cpn = Lo.has_comp ? SMF(Lo.cpn) : nullptr;
    s.cpt = Lo.has_comp ? SMF(Lo.cpt) : nullptr;

    float *ax = SMF(Lo.ax), *ay = SMF(Lo.ay), *ahw = SMF(Lo.ahw), *ahh = SMF(Lo.ahh);
    int32_t *rx0 = SMI32(Lo.rx0), *ry0 = SMI32(Lo.ry0), *rx1 = SMI32(Lo.rx1), *ry1 = SMI32(Lo.ry1);
    int32_t *fx0 = SMI32(Lo.fx0), *fy0 = SMI32(Lo.fy0), *fx1 = SMI32(Lo.fx1), *fy1 = SMI32(Lo.fy1);
    uint32_t* bcnt = SMU32(Lo.bcnt);
    uint32_t* ebucket = SMU32(Lo.ebucket);
    uint16_t *ebody = SMU16(Lo.ebody), *eslot = SMU16(Lo.eslot), *sbody = SMU16(Lo.sbody);
    uint32_t* table = SMU32(Lo.table);
    uint32_t* cand = SMU32(Lo.hset);  // candidate pairs before they are grouped by shape type
    unsigned long long* skey = reinterpret_cast<unsigned long long*>(sm + Lo.skey);
    uint32_t* cmask = SMU32(Lo.cmask);
    uint16_t *corder = SMU16(Lo.corder), *coff = SMU16(Lo.coff);
    uint16_t *jorder = SMU16(Lo.jorder), *joff = SMU16(Lo.joff);
    uint8_t* jcol = SMU8(Lo.jcol);
    uint32_t* pairs = SMU32(Lo.pairs);

    const bool disc_rot = (wd.flags & W_DISC_ROTATION) != 0;
    const float* __restrict__ st = P.state;
    const float* __restrict__ pr = P.props;


    // ---------------- load the world ----------------
    // Two bodies a thread per round, every global load of both issued before
    // either is used, so a round waits for memory once.
    struct RawBody {
        uint8_t k;
        float px, py, a, mx, my, L, m, I, ax, ay, ahw, ahh;
    };
    auto fetch = [&](uint32_t i) {
        const uint32_t g = base + i;
        RawBody r;
        r.k = __ldg(P.kind + g);
        r.a = st[(size_t)S_ANGLE * NB + g];
        r.px = st[(size_t)S_POS_X * NB + g];
        r.py = st[(size_t)S_POS_Y * NB + g];
        r.mx = st[(size_t)S_MOM_X * NB + g];
        r.my = st[(size_t)S_MOM_Y * NB + g];
        r.L = st[(size_t)S_ANG_MOM * NB + g];
        r.m = __ldg(pr + (size_t)P_MASS * NB + g);
        r.I = __ldg(pr + (size_t)P_INERTIA * NB + g);
        r.ax = st[(size_t)S_AABB_X * NB + g];
        r.ay = st[(size_t)S_AABB_Y * NB + g];
        r.ahw = st[(size_t)S_AABB_HW * NB + g];
        r.ahh = st[(size_t)S_AABB_HH * NB + g];
        return r;
    };
    auto put = [&](uint32_t i, const RawBody& r) {
        s.px[i] = r.px;
        s.py[i] = r.py;
        s.ang[i] = r.a;
        s.put_mom(i, r.mx, r.my, r.L, (r.k & K_STATIC) ? 0.f : 1.0f / r.m);
        if (Lo.has_pos0) {
            s.px0[i] = r.px;
            s.py0[i] = r.py;
        }
        s.inv_i[i] = (r.k & K_STATIC) ? 0.f : 1.0f / r.I;
        s.kind[i] = r.k;
        float c = 1.f, sn = 0.f;
        if ((r.k & K_RECT) || disc_rot) r2d_sincosf(r.a, &sn, &c);
        s.cs[i] = c;
        s.sn[i] = sn;
        if (Lo.has_prev) s.ang_prev[i] = r.a;
        s.tq[i] = 0.f;
        ax[i] = r.ax;
        ay[i] = r.ay;
        ahw[i] = r.ahw;
        ahh[i] = r.ahh;
    };
    for (uint32_t i = tid; i < n; i += 2 * NT) {
        const bool two = i + NT < n;
        const RawBody r0 = fetch(i);
        RawBody r1 = r0;
        if (two) r1 = fetch(i + NT);
        put(i, r0);
        if (two) put(i + NT, r1);
    }
    for (uint32_t b = tid; b < T + 1; b += NT) table[b] = 0u;
    __syncthreads();
    PHASE(0);

    // ---------------- broadphase (SpatialHash.zig:19-137, lib.zig:264-282) ----------------
    // The reference pairs every two bodies that share a bucket of its spatial
    // hash (cells 4.0 wide: dense piles put ~30 bodies in one bucket) and
    // keeps those whose AABBs intersect.  An intersecting pair shares a
    // bucket exactly when its cell ranges overlap or two of its cells hash
    // alike, so the kernel finds the intersecting pairs on a finer grid
    // (boxes grown past the 0.01 overlap margin) and applies that test: the
    // same pair set from a few candidates per body.
    const float gfine = wd.fine_cell;
    for (uint32_t i = tid; i < n; i += NT) {
        int32_t x0 = 0, y0 = 0, x1 = -1, y1 = -1;
        uint32_t cnt = 0;
        const bool ok = cell_index(ax[i] - ahw[i], P.cell, &x0) && cell_index(ay[i] - ahh[i], P.cell, &y0) &&
                        cell_index(ax[i] + ahw[i], P.cell, &x1) && cell_index(ay[i] + ahh[i], P.cell, &y1);
        int32_t u0 = 0, v0 = 0, u1 = -1, v1 = -1;
        if (!ok) {
            err = DS_NONFINITE;
            x1 = x0 - 1;
        } else {
            // margin: the overlap epsilon, plus slack for the rounding of
            // the intersection test at this magnitude
            const float m = AABB_EPS_OVERLAP + 1e-6f * (fabsf(ax[i]) + fabsf(ay[i]) + ahw[i] + ahh[i]);
            const bool okf = cell_index((ax[i] - ahw[i]) - m, gfine, &u0) &&
                             cell_index((ay[i] - ahh[i]) - m, gfine, &v0) &&
                             cell_index((ax[i] + ahw[i]) + m, gfine, &u1) &&
                             cell_index((ay[i] + ahh[i]) + m, gfine, &v1);
            if (!okf) {
                cap_fail(&err, &s_capbits, CAP_ENTRIES);  // the grid pipeline bins on the coarse cells
                u1 = u0 - 1;
            } else if (u1 >= u0 && v1 >= v0) {
                const int64_t c64 = ((int64_t)u1 - (int64_t)u0 + 1) * ((int64_t)v1 - (int64_t)v0 + 1);
                if (c64 > (int64_t)C.ne) cap_fail(&err, &s_capbits, CAP_ENTRIES);
                else cnt = (uint32_t)c64;
            }
        }
        rx0[i] = x0; ry0[i] = y0; rx1[i] = x1; ry1[i] = y1;
        fx0[i] = u0; fy0[i] = v0; fx1[i] = u1; fy1[i] = v1;
        bcnt[i] = cnt;
    }
    if (err) set_err(&s_err, err);
    if (__syncthreads_or(err != 0)) goto fail;
    if (n <= (uint32_t)R2D_BRUTE_MAX_BODIES) {
        // Few bodies: every pair is tested directly, in equal shares of the
        // n(n-1)/2 pairs per thread, with the filters and the shared-bucket
        // test below -- the same pair set without the binning grid's scans.
        const BucketMod bmod = {wd.bucket_recip, T};
        const uint32_t total = n * (n - 1u) / 2u;
        const uint32_t per = (total + NT - 1) / NT;
        const uint32_t p0 = min(total, (uint32_t)tid * per), p1 = min(total, p0 + per);
        if (p0 < p1) {
            uint32_t i = 0, rem = p0;  // pair p0 = (i, i + 1 + rem), rows of decreasing length
            while (rem >= n - 1u - i) {
                rem -= n - 1u - i;
                ++i;
            }
            uint32_t j = i + 1u + rem;
            f2 pi = {ax[i], ay[i]};
            float hwi = ahw[i], hhi = ahh[i];
            bool sti = (s.kind[i] & K_STATIC) != 0;
            for (uint32_t q = p0; q < p1; ++q, ++j) {
                if (j >= n) {  // next row
                    ++i;
                    j = i + 1u;
                    pi = f2{ax[i], ay[i]};
                    hwi = ahw[i];
                    hhi = ahh[i];
                    sti = (s.kind[i] & K_STATIC) != 0;
                }
                if (sti && (s.kind[j] & K_STATIC)) continue;
                if (!aabb_intersects(pi, hwi, hhi, f2{ax[j], ay[j]}, ahw[j], ahh[j])) continue;
                if (!shares_bucket(i, j, rx0, ry0, rx1, ry1, bmod)) continue;
                if (wd.nexcl && excluded(P.excl + wd.excl_off, wd.nexcl, ((unsigned long long)i << 32) | j)) continue;
                const cg::coalesced_group g = cg::coalesced_threads();
                uint32_t at = 0;
                if (g.thread_rank() == 0) at = atomicAdd(&s_cnt[0], g.size());
                const uint32_t slot = g.shfl(at, 0) + g.thread_rank();
                if (slot < C.hs) cand[slot] = (i << 16) | j;
            }
        }
        __syncthreads();
    } else {
        SUBPHASE(12);
        const uint32_t E = block_scan_excl<NT>(bcnt, n, s_wsum);
        if (E > C.ne) {
            if (tid == 0) {
                s_err = DS_CAPACITY;
                s_capbits |= CAP_ENTRIES;
            }
            __syncthreads();
            goto fail;
        }
        const BucketMod bmod = {wd.bucket_recip, T};
        // A body's entries, row by row over its cells; a body with many
        // (a static ground or wall spans dozens of cells) is left to the
        // whole block below, so that no thread walks a long row alone while
        // the others wait at the barrier.
        if (tid == 0) s_nbig = 0u;
        __syncthreads();
        for (uint32_t i = tid; i < n; i += NT) {
            const uint32_t wx = (uint32_t)(fx1[i] - fx0[i] + 1);
            if (fx1[i] >= fx0[i] && fy1[i] >= fy0[i] && wx * (uint32_t)(fy1[i] - fy0[i] + 1) > BIG_BODY_ENTRIES) {
                const uint32_t q = atomicAdd(&s_nbig, 1u);
                if (q < MAX_BIG_BODIES) {
                    s_big[q] = i;
                    continue;
                }
            }
            uint32_t k = bcnt[i];
            for (int32_t yi = fy0[i]; yi <= fy1[i]; ++yi)
                for (int32_t xi = fx0[i]; xi <= fx1[i]; ++xi) {
                    const uint32_t bk = cell_bucket(xi, yi, bmod);
                    ebucket[k] = bk;
                    ebody[k] = (uint16_t)i;
                    atomicAdd(&table[bk], 1u);
                    ++k;
                }
        }
        __syncthreads();
        const uint32_t nbig = min(s_nbig, (uint32_t)MAX_BIG_BODIES);
        for (uint32_t q = 0; q < nbig; ++q) {
            const uint32_t i = s_big[q], k0 = bcnt[i];
            const uint32_t wx = (uint32_t)(fx1[i] - fx0[i] + 1), cnt = wx * (uint32_t)(fy1[i] - fy0[i] + 1);
            for (uint32_t t = tid; t < cnt; t += NT) {  // entry t: row t / wx, column t % wx
                const uint32_t bk = cell_bucket(fx0[i] + (int32_t)(t % wx), fy0[i] + (int32_t)(t / wx), bmod);
                ebucket[k0 + t] = bk;
                ebody[k0 + t] = (uint16_t)i;
                atomicAdd(&table[bk], 1u);
            }
        }
        __syncthreads();
        block_scan_excl<NT>(table, T, s_wsum);  // table[b] = first slot of bucket b
        for (uint32_t e = tid; e < E; e += NT) {
            const uint32_t slot = atomicAdd(&table[ebucket[e]], 1u);
            sbody[slot] = (uint16_t)e;  // the entry: body and cell
            eslot[e] = (uint16_t)slot;
        }
        __syncthreads();  // table[b] = one past the last slot of bucket b
        SUBPHASE(13);

        // Candidates: every two entries of one fine bucket.  Entries of other
        // cells that hash to the same bucket are skipped, and a pair is
        // reported only from the first cell the two cover in common, so each
        // pair comes out once (the reference's "manifold already exists"
        // test, lib.zig:278-281, without a set).  Then the filters of
        // lib.zig:273-282 and the shared-bucket test.  Entry e pairs with the
        // entries after it in its bucket; a prefix sum over those counts deals
        // the candidates out to the threads in equal contiguous ranges.
        for (uint32_t e = tid; e < E; e += NT) ebucket[e] = table[ebucket[e]] - (uint32_t)eslot[e] - 1u;
        __syncthreads();
        const uint32_t W = block_scan_excl<NT>(ebucket, E, s_wsum);  // ebucket[e] = first candidate of e
        const uint32_t k0 = (uint32_t)(((unsigned long long)W * (uint32_t)tid) / NT);
        const uint32_t k1 = (uint32_t)(((unsigned long long)W * (uint32_t)(tid + 1)) / NT);
        if (k0 < k1) {
            uint32_t lo = 0, hi = E;  // the entry holding candidate k0: ebucket[lo] <= k0 < ebucket[hi]
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (ebucket[mid] <= k0) lo = mid;
                else hi = mid;
            }
            uint32_t e = lo, first = ebucket[e], next = e + 1 < E ? ebucket[e + 1] : W;
            uint32_t i = ebody[e];
            int32_t fx0i = fx0[i], fy0i = fy0[i], cxe, cye;
            entry_cell(e, bcnt[i], fx0i, fx1[i], fy0i, &cxe, &cye);
            f2 pi = {ax[i], ay[i]};
            float hwi = ahw[i], hhi = ahh[i];
            bool sti = (s.kind[i] & K_STATIC) != 0;
            uint32_t sb0 = (uint32_t)eslot[e] + 1u - first;  // candidate k pairs e with sorted entry sb0 + k
            for (uint32_t k = k0; k < k1; ++k) {
                if (k >= next) {
                    do {
                        ++e;
                        first = next;
                        next = e + 1 < E ? ebucket[e + 1] : W;
                    } while (k >= next);
                    i = ebody[e];
                    fx0i = fx0[i];
                    fy0i = fy0[i];
                    entry_cell(e, bcnt[i], fx0i, fx1[i], fy0i, &cxe, &cye);
                    pi = f2{ax[i], ay[i]};
                    hwi = ahw[i];
                    hhi = ahh[i];
                    sti = (s.kind[i] & K_STATIC) != 0;
                    sb0 = (uint32_t)eslot[e] + 1u - first;
                }
                const uint32_t e2 = sbody[sb0 + k];
                const uint32_t j = ebody[e2];
                // everything the tests below read of j, in one round of loads
                const int32_t fx0j = fx0[j], fy0j = fy0[j], fx1j = fx1[j];
                const uint32_t bj = bcnt[j];
                const f2 pj = {ax[j], ay[j]};
                const float hwj = ahw[j], hhj = ahh[j];
                const bool stj = (s.kind[j] & K_STATIC) != 0;
                // a pair is reported from the first cell the two cover in common
                if (max(fx0i, fx0j) != cxe || max(fy0i, fy0j) != cye) continue;
                int32_t cx2, cy2;
                entry_cell(e2, bj, fx0j, fx1j, fy0j, &cx2, &cy2);
                if (cx2 != cxe || cy2 != cye) continue;  // another cell hashed to this bucket
                if (sti && stj) continue;
                // symmetric in the two bodies: |dx|, |dy| and the sums commute
                if (!aabb_intersects(pi, hwi, hhi, pj, hwj, hhj)) continue;
                if (!shares_bucket(i, j, rx0, ry0, rx1, ry1, bmod)) continue;
                const uint32_t plo = min(i, j), phi = max(i, j);
                if (wd.nexcl && excluded(P.excl + wd.excl_off, wd.nexcl, ((unsigned long long)plo << 32) | phi)) continue;
                const cg::coalesced_group g = cg::coalesced_threads();
                uint32_t at = 0;
                if (g.thread_rank() == 0) at = atomicAdd(&s_cnt[0], g.size());
                const uint32_t slot = g.shfl(at, 0) + g.thread_rank();
                if (slot < C.hs) cand[slot] = (plo << 16) | phi;
            }
        }
        __syncthreads();
        SUBPHASE(14);
#ifdef R2D_PHASE_TIMERS
        if (tid == 0 && P.timers) {
            P.timers[(size_t)w * PHASE_SLOTS + 18] += W;
            P.timers[(size_t)w * PHASE_SLOTS + 19] += E;
        }
#endif
    }
    {
        // The pair list, grouped by shape type (rectangle-rectangle,
        // disc-rectangle, disc-disc) so that the narrowphase's warps mostly
        // follow one code path.
        {
            const uint32_t found = s_cnt[0];
            if (found > C.np) {
                if (tid == 0) {
                    s_err = DS_CAPACITY;
                    s_capbits |= CAP_PAIRS;
                }
                __syncthreads();
                goto fail;
            }
            const uint32_t per = (found + NT - 1) / NT;
            const uint32_t s0 = min(found, (uint32_t)tid * per), s1 = min(found, s0 + per);
            unsigned long long mine = 0;
            for (uint32_t q = s0; q < s1; ++q) {
                const uint32_t key = cand[q];
                mine += 1ull << (21u * ((s.kind[key >> 16] & K_RECT) + (s.kind[key & 0xFFFFu] & K_RECT)));
            }
            unsigned long long total = 0;
            const unsigned long long before = block_scan_value_u64<NT>(mine, s_wsum64, &total);
            constexpr unsigned long long F = (1ull << 21) - 1ull;
            // heaviest first: rectangle-rectangle, disc-rectangle, disc-disc,
            // so that the warps drawing the costly SAT pairs start with them
            const uint32_t t1 = (uint32_t)((total >> 21) & F), t2 = (uint32_t)(total >> 42);
            uint32_t at[3] = {t2 + t1 + (uint32_t)(before & F), t2 + (uint32_t)((before >> 21) & F),
                              (uint32_t)(before >> 42)};
            for (uint32_t q = s0; q < s1; ++q) {
                const uint32_t key = cand[q];
                const uint32_t t = (s.kind[key >> 16] & K_RECT) + (s.kind[key & 0xFFFFu] & K_RECT);
                const uint32_t slot = t == 0 ? at[0]++ : (t == 1 ? at[1]++ : at[2]++);
                pairs[slot] = key;
            }
        }
        SUBPHASE(17);
    }
    __syncthreads();
    if (P.dbg.pcap) {  // debug tap: the candidate pairs, before the narrowphase reuses nothing of them
        const uint32_t found = s_cnt[0];
        if (tid == 0) P.dbg.npairs[w] = found;
        uint32_t* out = P.dbg.pairs + 2 * (size_t)w * P.dbg.pcap;
        for (uint32_t q = tid; q < found && q < P.dbg.pcap; q += NT) {
            const uint32_t key = pairs[q];
            out[2 * q] = key >> 16;
            out[2 * q + 1] = key & 0xFFFFu;
        }
    }

    PHASE(1);
    // ---------------- narrowphase (collision.zig:299-320, lib.zig:284-294) ----------------
    {
        // Each rectangle's edge normals (a square root and two divisions per
        // edge), once per body instead of once per pair it is in: held in the
        // point arrays mn .. apt, which the narrowphase leaves alone (they
        // hold 16 B a point, at least 2.4 points a body; 32 B a body needed).
        float4* gen = reinterpret_cast<float4*>(sm + Lo.mn);
        const bool en_cached = 32u * n <= 16u * C.npt;
        if (en_cached) {
            for (uint32_t i = tid; i < n; i += NT) {
                if (!(s.kind[i] & K_RECT)) continue;
                Geo g;
                geo_make(g, f2{s.px[i], s.py[i]}, true, __ldg(pr + (size_t)P_DIM0 * NB + base + i),
                         __ldg(pr + (size_t)P_DIM1 * NB + base + i), s.cs[i], s.sn[i]);
                gen[2 * i] = make_float4(g.en[0].x, g.en[0].y, g.en[1].x, g.en[1].y);
                gen[2 * i + 1] = make_float4(g.en[2].x, g.en[2].y, g.en[3].x, g.en[3].y);
            }
            __syncthreads();
        }
        const float h = P.dt / (float)P.sub_steps;
        const uint32_t npairs = s_cnt[0];
        const uint32_t lane = tid & 31u;
        // every thread runs the same number of rounds, so whole warps claim
        // manifold and point slots together (one atomic per warp and round)
        for (uint32_t b0 = 0; b0 < npairs; b0 += NT) {
            const uint32_t pi = b0 + tid;
            bool hit = false;
            int npt = 0;
            uint32_t ref = 0, inc = 0;
            float mulo = 0.f, muhi = 0.f;  // friction coefficients of the pair's lower and higher body
            SatState sat;
            NewPoint pts[2];
            if (pi < npairs) {
                const uint32_t key = pairs[pi];
                const uint32_t lo = key >> 16, hi = key & 0xFFFFu;
                // both bodies' ids and dimensions in one round trip to L2
                const uint32_t idlo = __ldg(P.ids + base + lo), idhi = __ldg(P.ids + base + hi);
                const float alo = __ldg(pr + (size_t)P_DIM0 * NB + base + lo);
                const float blo = __ldg(pr + (size_t)P_DIM1 * NB + base + lo);
                const float ahi = __ldg(pr + (size_t)P_DIM0 * NB + base + hi);
                const float bhi = __ldg(pr + (size_t)P_DIM1 * NB + base + hi);
                mulo = __ldg(pr + (size_t)P_MU * NB + base + lo);
                muhi = __ldg(pr + (size_t)P_MU * NB + base + hi);
                const bool lo_first = idlo < idhi;
                const uint32_t o1 = lo_first ? lo : hi;
                const uint32_t o2 = lo_first ? hi : lo;
                Geo g1, g2;
                if (en_cached) {
                    geo_make_cached(g1, f2{s.px[o1], s.py[o1]}, s.kind[o1] & K_RECT, lo_first ? alo : ahi,
                                    lo_first ? blo : bhi, s.cs[o1], s.sn[o1], gen + 2 * o1);
                    geo_make_cached(g2, f2{s.px[o2], s.py[o2]}, s.kind[o2] & K_RECT, lo_first ? ahi : alo,
                                    lo_first ? bhi : blo, s.cs[o2], s.sn[o2], gen + 2 * o2);
                } else {
                    geo_make(g1, f2{s.px[o1], s.py[o1]}, s.kind[o1] & K_RECT, lo_first ? alo : ahi,
                             lo_first ? blo : bhi, s.cs[o1], s.sn[o1]);
                    geo_make(g2, f2{s.px[o2], s.py[o2]}, s.kind[o2] & K_RECT, lo_first ? ahi : alo,
                             lo_first ? bhi : blo, s.cs[o2], s.sn[o2]);
                }
                hit = perform_narrow_sat(g1, g2, sat);
                if (hit) {
                    ref = sat.ref_is_first ? o1 : o2;
                    inc = sat.ref_is_first ? o2 : o1;
                    npt = sat.ref_is_first ? identify_points(g1, g2, sat.refid, pts)
                                           : identify_points(g2, g1, sat.refid, pts);
                }
            }
            // inclusive warp scan of (manifolds, points) packed 16:16
            const uint32_t mine = (hit ? 1u : 0u) | ((uint32_t)npt << 16);
            uint32_t incl = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            uint32_t mbase = 0, pbase = 0;
            if (lane == 31u && incl) {
                mbase = atomicAdd(&s_cnt[1], incl & 0xFFFFu);
                pbase = atomicAdd(&s_cnt[2], incl >> 16);
            }
            mbase = __shfl_sync(0xffffffffu, mbase, 31);
            pbase = __shfl_sync(0xffffffffu, pbase, 31);
            if (!hit) continue;
            const uint32_t before = incl - mine;
            const uint32_t m = mbase + (before & 0xFFFFu);
            const uint32_t p0 = pbase + (before >> 16);
            if (m >= C.nm) {
                cap_fail(&err, &s_capbits, CAP_MANIFOLDS);
                continue;
            }
            if (p0 + npt > C.npt) {
                cap_fail(&err, &s_capbits, CAP_POINTS);
                continue;
            }
            s.ma[m] = (uint16_t)ref;
            s.mb[m] = (uint16_t)inc;
            s.mp0[m] = (uint16_t)p0;
            s.mnp[m] = (uint8_t)npt;
            s.nx[m] = sat.normal.x;
            s.ny[m] = sat.normal.y;
            // the preStep's friction, sqrt(mu_ref * mu_inc) (collision.zig:114), fixed for the frame
            s.fric[m] = sqrtf(mulo * muhi);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (k >= npt) break;
                const float d = pts[k].depth;
                if (LEAN) {
                    s.r1x[p0 + k] = pts[k].mid.x;
                    s.r1y[p0 + k] = pts[k].mid.y;
                    // a depth for which approxEql(depth, depth, 1e-4) fails
                    // (|depth| >= 2048 or NaN) makes updateTGSDepth rotate the
                    // lever arms (collision.zig:80-95): full layout needed
                    if (!approx_eql(d, d, 1e-4f)) cap_fail(&err, &s_capbits, CAP_TGS);
                    // otherwise the depth is fixed for the frame, and so is the
                    // bias of calculateImpulses (collision.zig:154-172); a
                    // negative bias marks a point with depth >= 0
                    s.bias[p0 + k] = d >= 0.0f ? -1.0f : BAUMGARTE * zmax(0.0f, (-d) - BAUMGARTE_SLOP) / h;
                } else {
                    s.r1x[p0 + k] = pts[k].ref_r.x;
                    s.r1y[p0 + k] = pts[k].ref_r.y;
                    s.r2x[p0 + k] = pts[k].inc_r.x;
                    s.r2y[p0 + k] = pts[k].inc_r.y;
                    s.odepth[p0 + k] = d;
                }
                if (Lo.has_depth) s.depth[p0 + k] = d;
            }
        }
    }
    if (err) set_err(&s_err, err);
    if (__syncthreads_or(err != 0)) goto fail;

    PHASE(2);
    {
        const uint32_t M = min(s_cnt[1], C.nm);
        const uint32_t NJ = wd.nj;
        uint32_t ncol = 0, njcol = 0;

        // ---------------- contact colouring (r2d_colour.h) ----------------
        // Conflict nodes of a contact: its non-static bodies.
        auto contact_ends = [&](uint32_t m, uint32_t* a, uint32_t* b) {
            const uint32_t x = s.ma[m], y = s.mb[m];
            if (!(s.kind[x] & K_STATIC)) *a = x;
            if (!(s.kind[y] & K_STATIC)) *b = y;
        };
        auto contact_mix = [&](uint32_t m) {
            const uint32_t x = s.ma[m], y = s.mb[m];
            return r2d_colour_mix(min(x, y), max(x, y));
        };
        auto contact_tie = [&](uint32_t m) {
            const uint32_t x = s.ma[m], y = s.mb[m];
            return (min(x, y) << 16) | max(x, y);
        };
        if (colour_greedy_sorted<NT>(M, n, contact_ends, contact_mix, contact_tie, s.mcol, skey, cmask, s_ccnt,
                                     s_wsum, &s_ncol, [&]() { SUBPHASE(15); })) {
            if (tid == 0) {
                s_err = DS_CAPACITY;
                s_capbits |= CAP_COLOURS;
            }
            __syncthreads();
            goto fail;
        }
        SUBPHASE(16);
        // colour-major order
        ncol = s_ncol;
        for (uint32_t c = tid; c < ncol; c += NT) s_ccnt[c] = 0u;
        __syncthreads();
        for (uint32_t m = tid; m < M; m += NT) atomicAdd(&s_ccnt[s.mcol[m]], 1u);
        __syncthreads();
        block_scan_excl<NT>(s_ccnt, ncol, s_wsum);
        for (uint32_t c = tid; c <= ncol; c += NT) coff[c] = (uint16_t)(c < ncol ? s_ccnt[c] : M);
        __syncthreads();
        for (uint32_t m = tid; m < M; m += NT) corder[atomicAdd(&s_ccnt[s.mcol[m]], 1u)] = (uint16_t)m;

        PHASE(3);
        // ---------------- joint colouring ----------------
        if (NJ) {
            const uint32_t j0 = wd.joint_off;
            __syncthreads();
            // every body a joint names is a conflict node, static or not
            auto joint_ends = [&](uint32_t j, uint32_t* a, uint32_t* b) {
                const uint8_t ty = __ldg(P.jtype + j0 + j);
                const uint32_t b1 = __ldg(P.jb1 + j0 + j), b2 = __ldg(P.jb2 + j0 + j);
                *a = b1;
                if (joint_two_bodies(ty) && b2 != b1) *b = b2;
            };
            auto joint_mix = [&](uint32_t j) { return r2d_colour_mix(j, R2D_COLOUR_JOINT_SALT); };
            auto joint_tie = [&](uint32_t j) { return j; };
            if (colour_greedy_sorted<NT>(NJ, n, joint_ends, joint_mix, joint_tie, jcol, skey, cmask, s_ccnt, s_wsum,
                                         &s_ncol, [&]() {})) {
                if (tid == 0) {
                    s_err = DS_CAPACITY;
                    s_capbits |= CAP_COLOURS;
                }
                __syncthreads();
                goto fail;
            }
            njcol = s_ncol;
            for (uint32_t c = tid; c < njcol; c += NT) s_ccnt[c] = 0u;
            __syncthreads();
            for (uint32_t j = tid; j < NJ; j += NT) atomicAdd(&s_ccnt[jcol[j]], 1u);
            __syncthreads();
            block_scan_excl<NT>(s_ccnt, njcol, s_wsum);
            for (uint32_t c = tid; c <= njcol; c += NT) joff[c] = (uint16_t)(c < njcol ? s_ccnt[c] : NJ);
            __syncthreads();
            for (uint32_t j = tid; j < NJ; j += NT) jorder[atomicAdd(&s_ccnt[jcol[j]], 1u)] = (uint16_t)j;
        }
        __syncthreads();
        // the sort scratch overlapped the accumulators: they start at zero
        for (uint32_t p = tid; p < s_cnt[2] && p < C.npt; p += NT) {
            s.apn[p] = 0.f;
            s.apt[p] = 0.f;
            if (Lo.has_comp) {
                s.cpn[p] = 0.f;
                s.cpt[p] = 0.f;
            }
        }
        const bool warm = P.warm_keys != nullptr;
        const uint32_t wcur = warm ? P.warm_cur[w] : 0u;
        if (warm) {
            // a manifold of last frame's pair starts from its impulses
            __syncthreads();
            const size_t at = (size_t)wd.warm_off + (size_t)wcur * wd.warm_hs;
            const unsigned long long* keys = P.warm_keys + at;
            for (uint32_t m = tid; m < M; m += NT) {
                const unsigned long long key = warm_key_ids(__ldg(P.ids + base + s.ma[m]), __ldg(P.ids + base + s.mb[m]));
                const int slot = warm_find(keys, wd.warm_hs, key);
                if (slot < 0) continue;
                const float4 v = P.warm_vals[at + slot];
                const uint32_t p0 = s.mp0[m], np = s.mnp[m];
                if (np > 0) {
                    s.apn[p0] = v.x;
                    s.apt[p0] = v.y;
                }
                if (np > 1) {
                    s.apn[p0 + 1] = v.z;
                    s.apt[p0 + 1] = v.w;
                }
                if (Lo.has_comp && P.warm_cvals) {
                    const float4 c = P.warm_cvals[at + slot];
                    if (np > 0) {
                        s.cpn[p0] = c.x;
                        s.cpt[p0] = c.y;
                    }
                    if (np > 1) {
                        s.cpn[p0 + 1] = c.z;
                        s.cpt[p0 + 1] = c.w;
                    }
                }
            }
        }
        __syncthreads();

        PHASE(4);
        // ---------------- substeps (lib.zig:199-250) ----------------
        const uint32_t S = P.sub_steps;
        const float h = P.dt / (float)S;
        for (uint32_t sub = 0; sub < S; ++sub) {
            const bool last = sub + 1 == S;
            // forces (DownwardsGravity.zig:35-39), AABB, velocities (lib.zig:200-216)
            for (uint32_t i = tid; i < n; i += NT) {
                const uint32_t g = base + i;
                const uint8_t k = s.kind[i];
                float fx = 0.f, fy = 0.f, tq = 0.f;
                if (sub == 0) {  // user-set force / torque (RigidBody.Props, RigidBody.zig:73,78)
                    // a frame call's host rows (r2d_*_process_io), read over the CPU-GPU link
                    const float* ext_force = P.ext ? P.ext->force : nullptr;
                    if (ext_force) {
                        fx = ext_force[g];
                        fy = ext_force[(size_t)NB + g];
                        tq = ext_force[2 * (size_t)NB + g];
                    } else {
                        fx = st[(size_t)S_FORCE_X * NB + g];
                        fy = st[(size_t)S_FORCE_Y * NB + g];
                        tq = st[(size_t)S_TORQUE * NB + g];
                    }
                    // a dynamic body's force / torque is cleared after integration (lib.zig:247-248)
                    if (!(k & K_STATIC) && (fx != 0.f || fy != 0.f || tq != 0.f)) s.kind[i] = k | K_FORCED;
                }
                if (!(k & K_STATIC)) {
                    for (uint32_t gg = 0; gg < wd.ngrav; ++gg) {
                        fx += 0.0f * s.mass(i);
                        fy += (-wd.g[gg]) * s.mass(i);
                    }
                }
                if (last) {
                    float hw, hh;
                    if (k & K_RECT) {
                        rect_half_extents(__ldg(pr + (size_t)P_DIM0 * NB + g), __ldg(pr + (size_t)P_DIM1 * NB + g),
                                          s.cs[i], s.sn[i], &hw, &hh);
                    } else {
                        hw = hh = __ldg(pr + (size_t)P_DIM0 * NB + g);
                    }
                    P.state[(size_t)S_AABB_X * NB + g] = s.px[i];
                    P.state[(size_t)S_AABB_Y * NB + g] = s.py[i];
                    P.state[(size_t)S_AABB_HW * NB + g] = hw;
                    P.state[(size_t)S_AABB_HH * NB + g] = hh;
                }
                if (k & K_STATIC) continue;
                s.MX(i) += fx * h;
                s.MY(i) += fy * h;
                s.AM(i) += tq * h;
                s.tq[i] = tq;
            }
            __syncthreads();
            SUBPHASE(PT_FORCES);
            // updateTGSDepth + preStep (collision.zig:73-133)
            for (uint32_t m = tid; m < M; m += NT) {
                const uint32_t a = s.ma[m], b = s.mb[m];
                const f2 n2 = {s.nx[m], s.ny[m]};
                const uint32_t p0 = s.mp0[m], np = s.mnp[m];
                for (uint32_t k = 0; k < np && !LEAN; ++k) {
                    const uint32_t p = p0 + k;
                    if (approx_eql(s.depth[p], s.odepth[p], 1e-4f)) continue;
                    float sa_, ca_, sb_, cb_;
                    r2d_sincosf(s.ang[a] - s.ang_prev[a], &sa_, &ca_);
                    r2d_sincosf(s.ang[b] - s.ang_prev[b], &sb_, &cb_);
                    const f2 rr1 = rot(f2{s.r1x[p], s.r1y[p]}, ca_, sa_);
                    const f2 rr2 = rot(f2{s.r2x[p], s.r2y[p]}, cb_, sb_);
                    const f2 a1 = add2(rr1, f2{s.px[a], s.py[a]});
                    const f2 a2 = add2(rr2, f2{s.px[b], s.py[b]});
                    const float d = dot2(n2, sub2(a2, a1));
                    s.depth[p] = d + s.odepth[p];
                    s.r1x[p] = rr1.x;
                    s.r1y[p] = rr1.y;
                    s.r2x[p] = rr2.x;
                    s.r2y[p] = rr2.y;
                }
                const float inv_m1 = s.IM(a), inv_m2 = s.IM(b);
                const float inv_mass = inv_m1 + inv_m2;
                const float inv_i1 = s.inv_i[a], inv_i2 = s.inv_i[b];
                const f2 t2 = cw90(n2);
                for (uint32_t k = 0; k < np; ++k) {
                    const uint32_t p = p0 + k;
                    f2 r1, r2;
                    s.arms<LEAN>(p, a, b, &r1, &r2);
                    const float r1n = cross2(r1, n2), r2n = cross2(r2, n2);
                    const float kn = inv_mass + inv_i1 * (r1n * r1n) + inv_i2 * (r2n * r2n);
                    const float r1t = cross2(r1, t2), r2t = cross2(r2, t2);
                    const float kt = inv_mass + inv_i1 * (r1t * r1t) + inv_i2 * (r2t * r2t);
                    s.mn[p] = kn > 0.0f ? 1.0f / kn : 0.0f;
                    s.mt[p] = kt > 0.0f ? 1.0f / kt : 0.0f;
                    if (!LEAN) {  // bias of calculateImpulses (collision.zig:154-172); depth fixed in a substep
                        const float d = s.depth[p];
                        s.bias[p] = d >= 0.0f ? -1.0f : BAUMGARTE * zmax(0.0f, (-d) - BAUMGARTE_SLOP) / h;
                    }
                }
            }
            __syncthreads();
            SUBPHASE(PT_PRESTEP);
            if (warm && sub == 0) {  // the warm-started impulses, colour by colour
                for (uint32_t c = 0; c < ncol; ++c) {
                    for (uint32_t k = coff[c] + tid; k < coff[c + 1]; k += NT) warm_apply_contact<LEAN>(s, corder[k]);
                    __syncthreads();
                }
            }
            // impulse iterations (lib.zig:226-236): joints, then contacts
            for (uint32_t it = 0; it < P.iters; ++it) {
                for (uint32_t c = 0; c < njcol; ++c) {
                    const uint32_t k0 = joff[c], k1 = joff[c + 1];
                    for (uint32_t k = k0 + tid; k < k1; k += NT) {
                        const uint32_t j = jorder[k];
                        const uint32_t gj = wd.joint_off + j;
                        solve_joint(s, __ldg(P.jtype + gj), __ldg(P.jb1 + gj), __ldg(P.jb2 + gj),
                                    P.jprm + (size_t)gj * JOINT_PARAMS, h);
                    }
                    __syncthreads();
                }
                // A colour that fits the block twice over takes two lanes per
                // manifold (one per contact point); a larger one, one lane.
                for (uint32_t c = 0; c < ncol; ++c) {
                    const uint32_t k0 = coff[c], k1 = coff[c + 1];
                    if (k1 - k0 <= (uint32_t)(NT / 2)) {
                        const uint32_t k = k0 + ((uint32_t)tid >> 1);
                        solve_contact_lanes<LEAN>(s, k < k1 ? (uint32_t)corder[k] : 0u, k < k1, (uint32_t)tid & 31u,
                                                  warm);
                    } else {
                        for (uint32_t k = k0 + tid; k < k1; k += NT) solve_contact<LEAN>(s, corder[k], warm);
                    }
                    __syncthreads();
                }
            }
            // integration (lib.zig:238-249)
            for (uint32_t i = tid; i < n; i += NT) {
                if (Lo.has_prev) s.ang_prev[i] = s.ang[i];
                const uint8_t k = s.kind[i];
                if (k & K_STATIC) continue;
                if (P.pos64) {
                    integrate_pose64(P.pos64, NB, base + i, s.MX(i), s.MY(i), s.AM(i), h, s.mass(i), s.inertia(i),
                                     &s.px[i], &s.py[i], &s.ang[i]);
                } else {
                    const float sm_ = h / s.mass(i);
                    s.px[i] += s.MX(i) * sm_;
                    s.py[i] += s.MY(i) * sm_;
                    s.ang[i] += s.AM(i) * h / s.inertia(i);
                }
                s.tq[i] = 0.f;
                if (!last && ((k & K_RECT) || disc_rot)) {
                    float c, sn;
                    r2d_sincosf(s.ang[i], &sn, &c);
                    s.cs[i] = c;
                    s.sn[i] = sn;
                }
            }
            __syncthreads();
        }

        if (warm) {
            // this frame's impulses go to the world's other table, which then
            // becomes the one the next frame reads
            const size_t at = (size_t)wd.warm_off + (size_t)(1u - wcur) * wd.warm_hs;
            unsigned long long* keys = P.warm_keys + at;
            for (uint32_t q = tid; q < wd.warm_hs; q += NT) keys[q] = ~0ull;
            __syncthreads();
            for (uint32_t m = tid; m < M; m += NT) {
                const uint32_t p0 = s.mp0[m], np = s.mnp[m];
                const unsigned long long key = warm_key_ids(__ldg(P.ids + base + s.ma[m]), __ldg(P.ids + base + s.mb[m]));
                const int slot = warm_claim(keys, wd.warm_hs, key);
                if (slot < 0) continue;
                P.warm_vals[at + slot] = make_float4(np > 0 ? s.apn[p0] : 0.f, np > 0 ? s.apt[p0] : 0.f,
                                                     np > 1 ? s.apn[p0 + 1] : 0.f, np > 1 ? s.apt[p0 + 1] : 0.f);
                if (P.warm_cvals)
                    P.warm_cvals[at + slot] =
                        Lo.has_comp ? make_float4(np > 0 ? s.cpn[p0] : 0.f, np > 0 ? s.cpt[p0] : 0.f,
                                                  np > 1 ? s.cpn[p0 + 1] : 0.f, np > 1 ? s.cpt[p0 + 1] : 0.f)
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            __syncthreads();
            if (tid == 0) P.warm_cur[w] = 1u - wcur;
        }

        PHASE(5);
        // ---------------- write back ----------------
        bool moving = false;
        const float* ext_force = P.ext ? P.ext->force : nullptr;
        float* ext_out = P.ext ? P.ext->out : nullptr;
        for (uint32_t i = tid; i < n; i += NT) {
            const uint32_t g = base + i;
            P.state[(size_t)S_POS_X * NB + g] = s.px[i];
            P.state[(size_t)S_POS_Y * NB + g] = s.py[i];
            P.state[(size_t)S_ANGLE * NB + g] = s.ang[i];
            P.state[(size_t)S_MOM_X * NB + g] = s.MX(i);
            P.state[(size_t)S_MOM_Y * NB + g] = s.MY(i);
            P.state[(size_t)S_ANG_MOM * NB + g] = s.AM(i);
            // consumed forces are cleared (lib.zig:247-248); a frame call's
            // forces replace the state's rows as if written before the step:
            // cleared for a dynamic body, kept (unused) for a static one
            if (ext_force) {
                const bool keep = (s.kind[i] & K_STATIC) != 0;
                P.state[(size_t)S_FORCE_X * NB + g] = keep ? ext_force[g] : 0.f;
                P.state[(size_t)S_FORCE_Y * NB + g] = keep ? ext_force[(size_t)NB + g] : 0.f;
                P.state[(size_t)S_TORQUE * NB + g] = keep ? ext_force[2 * (size_t)NB + g] : 0.f;
            } else if (s.kind[i] & K_FORCED) {
                P.state[(size_t)S_FORCE_X * NB + g] = 0.f;
                P.state[(size_t)S_FORCE_Y * NB + g] = 0.f;
                P.state[(size_t)S_TORQUE * NB + g] = 0.f;
            }
            if (ext_out) {
                ext_out[g] = s.px[i];
                ext_out[(size_t)NB + g] = s.py[i];
                ext_out[2 * (size_t)NB + g] = s.ang[i];
                ext_out[3 * (size_t)NB + g] = s.MX(i);
                ext_out[4 * (size_t)NB + g] = s.MY(i);
                ext_out[5 * (size_t)NB + g] = s.AM(i);
            }
            if (P.sleep && !(s.kind[i] & K_STATIC))
                moving = moving || !r2d_body_still(s.MX(i), s.MY(i), s.AM(i), s.IM(i), s.inv_i[i]);
        }
        if (P.sleep) {
            const bool any_moving = __syncthreads_or(moving) != 0;
            if (tid == 0) P.sleep[w] = r2d_sleep_next(P.sleep[w], !any_moving);
        }
        if (P.dbg.cap) {
            const uint32_t cap = P.dbg.cap;
            if (tid == 0) P.dbg.nman[w] = M;
            for (uint32_t m = tid; m < M && m < cap; m += NT) {
                const size_t o = (size_t)w * cap + m;
                P.dbg.keys[2 * o] = s.ma[m];
                P.dbg.keys[2 * o + 1] = s.mb[m];
                P.dbg.colour[o] = s.mcol[m];
                float* d = P.dbg.data + o * DEBUG_MF;
                const f2 nn = {s.nx[m], s.ny[m]};
                const f2 tt = cw90(nn);
                const uint32_t np = s.mnp[m], p0 = s.mp0[m];
                d[0] = nn.x; d[1] = nn.y; d[2] = tt.x; d[3] = tt.y; d[4] = s.fric[m];
                d[5] = np > 0 ? 1.f : 0.f;
                d[6] = np > 1 ? 1.f : 0.f;
                d[7] = Lo.has_prev ? s.ang_prev[s.ma[m]] : __int_as_float(0x7fc00000);
                d[8] = Lo.has_prev ? s.ang_prev[s.mb[m]] : __int_as_float(0x7fc00000);
                for (uint32_t k = 0; k < 2; ++k) {
                    float* q = d + 9 + 12 * k;
                    const bool has = k < np;
                    const uint32_t p = p0 + k;
                    q[0] = __int_as_float(0x7fc00000);
                    q[1] = __int_as_float(0x7fc00000);
                    f2 r1 = {0.f, 0.f}, r2 = {0.f, 0.f};
                    if (has) s.arms<LEAN>(p, s.ma[m], s.mb[m], &r1, &r2);
                    q[2] = r1.x;
                    q[3] = r1.y;
                    q[4] = r2.x;
                    q[5] = r2.y;
                    const float dd = Lo.has_depth ? s.depth[p] : __int_as_float(0x7fc00000);
                    q[6] = has ? dd : 0.f;
                    q[7] = has ? (LEAN ? dd : s.odepth[p]) : 0.f;
                    q[8] = has ? s.mn[p] : 0.f;
                    q[9] = has ? s.mt[p] : 0.f;
                    q[10] = has ? s.apn[p] : 0.f;
                    q[11] = has ? s.apt[p] : 0.f;
                }
            }
            if (P.dbg.jcap) {
                for (uint32_t j = tid; j < NJ && j < P.dbg.jcap; j += NT)
                    P.dbg.jcolour[(size_t)w * P.dbg.jcap + j] = jcol[j];
            }
        }
        PHASE(6);
#ifdef R2D_PHASE_TIMERS
        if (tid == 0 && P.timers) {
            unsigned long long* t = P.timers + (size_t)w * PHASE_SLOTS;
            t[7] += s_cnt[0];
            t[8] += M;
            t[9] += ncol;
            t[10] += jp_rounds;
            t[11] += 1;
            unsigned long long gt;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(gt));
            t[PT_END] = gt;
        }
#endif
        if (tid == 0) P.world_status[w] = DS_OK;
        return;
    }

fail:
    if (tid == 0) {
        P.world_status[w] = s_err ? s_err : DS_CAPACITY;
        P.world_capbits[w] = s_capbits;
        P.world_fail_call[w] = P.call_counter ? *P.call_counter - 1u : P.call_index;
        atomicAdd(P.error_count, 1);
    }
#undef SMF
#undef SMU32
#undef SMU16
#undef SMU8
#undef SMI32
}

// One call of the step begins by counting itself (StepParams::call_counter).
__global__ void count_call_kernel(uint32_t* counter) { *counter += 1u; }

// ---------------------------------------------------------------------------
// host-side launch helpers
// ---------------------------------------------------------------------------
template <int NT, bool LEAN>
cudaError_t launch_world_step_nt(const StepParams& P, const Caps& C, const LayoutOpts& opts, cudaStream_t stream,
                                 int priority) {
    const Layout L = make_layout(C, opts);
    if (P.nlist == 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(P.nlist);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = L.total;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = priority;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, world_step_kernel<NT, LEAN>, P, C, L);
}

template <int NT, bool LEAN>
cudaError_t allow_smem_nt(int bytes) {
    cudaFuncAttributes fa;
    const cudaError_t e = cudaFuncGetAttributes(&fa, world_step_kernel<NT, LEAN>);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(world_step_kernel<NT, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                bytes - (int)fa.sharedSizeBytes);
}

// Lets every instantiation use all the shared memory a CTA may have (`bytes`,
// static included) as dynamic shared memory; set once, before any launch,
// so that launches (and graph capture) set nothing.
cudaError_t allow_world_step_smem(int bytes) {
    const cudaError_t es[] = {allow_smem_nt<32, true>(bytes),  allow_smem_nt<32, false>(bytes),
                              allow_smem_nt<64, true>(bytes),  allow_smem_nt<64, false>(bytes),
                              allow_smem_nt<128, true>(bytes), allow_smem_nt<128, false>(bytes),
                              allow_smem_nt<256, true>(bytes), allow_smem_nt<256, false>(bytes),
                              allow_smem_nt<512, true>(bytes), allow_smem_nt<512, false>(bytes)};
    for (cudaError_t e : es)
        if (e != cudaSuccess) return e;
    return cudaSuccess;
}

// Moves each world's last-frame warm-start table into a new layout (one CTA
// per world): entries of the old table `old_cur[w]` are inserted into table 0
// of the new one, at most half its slots.  Old sizes of 0 slots mean "no
// table"; compensation words move when both layouts keep them.
__global__ void migrate_warm_kernel(WarmTables o, const uint32_t* old_cur, WarmTables n) {
    const uint32_t w = blockIdx.x;
    const uint32_t nh = n.hs[w], oh = o.hs ? o.hs[w] : 0u;
    unsigned long long* nk = n.keys + n.off[w];
    for (uint32_t q = threadIdx.x; q < 2u * nh; q += blockDim.x) nk[q] = ~0ull;
    __syncthreads();
    if (!oh || !nh) return;
    const size_t base = (size_t)o.off[w] + (size_t)old_cur[w] * oh;
    __shared__ uint32_t taken;
    if (threadIdx.x == 0) taken = 0u;
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < oh; q += blockDim.x) {
        const unsigned long long key = o.keys[base + q];
        if (key == ~0ull || atomicAdd(&taken, 1u) >= nh / 2u) continue;
        const int slot = warm_claim(nk, nh, key);
        if (slot < 0) continue;
        n.vals[n.off[w] + slot] = o.vals[base + q];
        if (n.cvals) n.cvals[n.off[w] + slot] = o.cvals ? o.cvals[base + q] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

cudaError_t launch_migrate_warm(uint32_t nworlds, const WarmTables& old_t, const uint32_t* old_cur,
                                const WarmTables& new_t, cudaStream_t stream) {
    if (nworlds == 0) return cudaSuccess;
    migrate_warm_kernel<<<nworlds, 256, 0, stream>>>(old_t, old_cur, new_t);
    return cudaGetLastError();
}

cudaError_t launch_count_call(uint32_t* counter, cudaStream_t stream) {
    count_call_kernel<<<1, 1, 0, stream>>>(counter);
    return cudaGetLastError();
}

// `priority` is the launch's stream priority (cudaDeviceGetStreamPriorityRange):
// when several size classes run at once, the block scheduler hands out the
// CTAs of a higher-priority launch first.
cudaError_t launch_world_step(const StepParams& P, const Caps& C, int threads, const LayoutOpts& opts,
                              cudaStream_t stream, int priority) {
#define R2D_LAUNCH(NT)                                                                  \
    return opts.lean ? launch_world_step_nt<NT, true>(P, C, opts, stream, priority) \
                     : launch_world_step_nt<NT, false>(P, C, opts, stream, priority)
    switch (threads) {
    case 32: R2D_LAUNCH(32);
    case 64: R2D_LAUNCH(64);
    case 128: R2D_LAUNCH(128);
    case 256: R2D_LAUNCH(256);
    case 512: R2D_LAUNCH(512);
    default: return cudaErrorInvalidValue;
    }
#undef R2D_LAUNCH
}

}  // namespace r2d
