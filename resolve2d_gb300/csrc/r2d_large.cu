/*
 * r2d_large.cu -- the step of one world too large for a single CTA's shared
 * memory (a 12,001-body pyramid, a 200,004-body box with chains and motors).
 *
 * The stages of the fused per-world kernel run as grid-wide and
 * cluster-resident kernels over global scratch buffers.  Every per-item
 * computation is the fused kernel's own device function (r2d_device.cuh,
 * r2d_solve.cuh) or, for the contact solve on packed records, its arithmetic
 * in the same order, so both paths produce the same bits for the same world:
 *
 *   cells, entries, bucket sort    SpatialHash.zig:19-137 (a counting sort)
 *   candidate pairs                lib.zig:264-282 (bucket sharing, filters,
 *                                  "manifold already exists" as a hash set)
 *   narrowphase + manifolds        collision.zig:299-363, Bodies/{Disc,Rectangle,RigidBody}.zig
 *   colouring                      Jones-Plassmann rounds: a constraint takes
 *                                  its colour once every neighbour that comes
 *                                  before it in priority order has one, which
 *                                  is exactly the sequential first-fit
 *                                  colouring of r2d_colour.h; all rounds in
 *                                  one thread-block cluster
 *   substeps                       lib.zig:199-250 on colour-major packed
 *                                  records: every substep in one resident
 *                                  cluster, or one kernel per phase and per
 *                                  colour of each iteration
 *
 * Buffer sizes are exact where they can be (cell entries are counted before
 * they are written; a manifold needs a candidate pair; a manifold has at most
 * two points).  Only the candidate-pair set is guessed; when it overflows,
 * the pair search reruns with a larger set, which is exact because nothing
 * writes the world's state before the substeps.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

#include "r2d_device.cuh"
#include "r2d_large.h"
#include "r2d_sleep.h"
#include "r2d_solve.cuh"
#include "r2d_world.cuh"

namespace r2d {

namespace {

constexpr int LT = 256;                                       // threads per block
constexpr unsigned long long MAX_CELL_ENTRIES = 64ull << 20;  // spatial-hash entries of one step

enum LargeCounter : int {
    LC_PAIRS = 0,      // candidate pairs found
    LC_MANIFOLDS,      // manifolds built
    LC_POINTS,         // contact points built
    LC_PAIR_OVERFLOW,  // the pair set or list was full
    LC_NONFINITE,      // a body's AABB has no cell index
    LC_COLOURS,        // a constraint needed more than MAX_COLOURS colours
    LC_BIG,            // one body covers more than MAX_CELL_ENTRIES cells
    LC_PEND0,          // three rotating "still uncoloured" counters of the colouring rounds
    LC_PEND1,
    LC_PEND2,
    LC_ROUNDS,         // the rounds that colouring needed
    LC_MOVING,         // some non-static body ended the step moving (sleeping mode)
    LC_STUCK,          // a colouring ran more rounds than it has constraints (cannot happen)
    LC_NOPOLY,         // a polygon body where no vertices are given (the allocation-free step)
    LC_N
};

// pinned host words of a grid step: the counters, the 64-bit entry total,
// then the colourings' counters and result blocks
constexpr uint32_t H_COLOUR = LC_N + 2;

inline uint32_t blocks(uint64_t n) { return (uint32_t)std::max<uint64_t>(1, (n + LT - 1) / LT); }

// Exclusive scan of one value per thread over a block of SCAN_THREADS
// threads; *total receives the block's sum.
constexpr int SCAN_THREADS = 1024;
constexpr uint32_t SCAN_TILE = 4 * SCAN_THREADS;        // elements per block of the multi-block scan
constexpr uint32_t SCAN_ONE_BLOCK = 4 * SCAN_TILE;      // longer arrays take the multi-block scan
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t wsum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        wsum[lane] = w;
    }
    __syncthreads();
    const uint32_t r = (warp ? wsum[warp - 1] : 0u) + x - v;
    *total = wsum[31];
    __syncthreads();  // wsum is reused by the next call
    return r;
}

// In-place exclusive scan of a[0..n) by one block, SCAN_THREADS consecutive
// elements at a time; a[n] receives the total.
__global__ void __launch_bounds__(SCAN_THREADS) lk_scan(uint32_t* a, uint32_t n) {
    uint32_t carry = 0;
    for (uint32_t at = 0; at < n; at += SCAN_THREADS) {
        const uint32_t i = at + threadIdx.x;
        const uint32_t v = i < n ? a[i] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(v, &tot);
        if (i < n) a[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) a[n] = carry;
}

// Multi-block scan, first pass: each block scans its SCAN_TILE elements in
// place and leaves the tile's sum in tsum[tile].
__global__ void __launch_bounds__(SCAN_THREADS) lk_scan_tiles(uint32_t* a, uint32_t n, uint32_t* tsum) {
    const uint32_t base = blockIdx.x * SCAN_TILE;
    uint32_t carry = 0;
#pragma unroll 1
    for (uint32_t k = 0; k < SCAN_TILE; k += SCAN_THREADS) {
        const uint32_t i = base + k + threadIdx.x;
        const uint32_t v = i < n ? a[i] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(v, &tot);
        if (i < n) a[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) tsum[blockIdx.x] = carry;
}

// Last pass, after tsum[0..tiles) has been scanned (its total at tsum[tiles]).
__global__ void lk_scan_add(uint32_t* a, uint32_t n, const uint32_t* tsum, uint32_t tiles) {
    const uint32_t i = blockIdx.x * 256 + threadIdx.x;
    if (i < n) a[i] += tsum[i / SCAN_TILE];
    if (i == n) a[n] = tsum[tiles];
}

// ---------------------------------------------------------------------------
// one-cluster resident kernels
// ---------------------------------------------------------------------------
// The colouring rounds and the colour-by-colour solve are chains of short
// dependent phases.  One thread-block cluster runs a whole chain and the
// hardware cluster barrier separates the phases: no launch per phase, no host
// round trip per few colouring rounds.  The barrier's release/acquire makes
// each phase's global-memory writes visible to the whole cluster.
constexpr int RT = 512;                     // threads per CTA of the resident kernels
constexpr uint32_t RESIDENT_MAX_PASSES = 4;  // colour sizes (in cluster threads) the resident solve takes

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// ---------------------------------------------------------------------------
// broadphase + narrowphase
// ---------------------------------------------------------------------------
struct Phase1 {
    SWT<uint32_t> s;
    const float* state;  // field-major, stride NB
    const float* props;
    const uint8_t* kind_in;
    const uint32_t* ids;
    uint32_t NB, base, n;
    float cell;
    BucketMod bmod;
    bool disc_rot;
    int32_t *rx0, *ry0, *rx1, *ry1;
    uint32_t *bcnt, *ebucket, *ebody, *eslot, *sbody, *table;
    unsigned long long* hset;  // pair set, ~0 = empty
    unsigned long long* pairs;
    uint32_t np, hs, nm, npt;
    const unsigned long long* excl;
    uint32_t nexcl;
    uint32_t* cnt;
    unsigned long long* entries;  // total cell entries (64-bit)
    // convex polygons of the engine (K_POLY bodies): local vertices
    // [NB][MAX_POLY_VERTS] and counts [NB]; null when it has none
    const float2* poly_v;
    const uint8_t* poly_nv;

    __device__ float st(int f, uint32_t i) const { return state[(size_t)f * NB + base + i]; }
    __device__ float pr(int f, uint32_t i) const { return __ldg(props + (size_t)f * NB + base + i); }
};

// per body: derived quantities, and the cells its stored AABB covers;
// returns its cell count
__device__ __forceinline__ uint32_t load_body(const Phase1& A, uint32_t i) {
    const uint8_t k = __ldg(A.kind_in + A.base + i);
    const float a = A.st(S_ANGLE, i);
    A.s.kind[i] = k;
    if ((k & K_POLY) && !A.poly_v) atomicExch(&A.cnt[LC_NOPOLY], 1u);
    const float inv_m = (k & K_STATIC) ? 0.f : 1.0f / A.pr(P_MASS, i);
    const float inv_i = (k & K_STATIC) ? 0.f : 1.0f / A.pr(P_INERTIA, i);
    A.s.inv_m[i] = inv_m;
    A.s.inv_i[i] = inv_i;
    float c = 1.f, sn = 0.f;
    if ((k & (K_RECT | K_POLY)) || A.disc_rot) r2d_sincosf(a, &sn, &c);
    A.s.cs[i] = c;
    A.s.sn[i] = sn;
    A.s.ang_prev[i] = a;
    A.s.tq[i] = 0.f;
    const float ax = A.st(S_AABB_X, i), ay = A.st(S_AABB_Y, i);
    const float hw = A.st(S_AABB_HW, i), hh = A.st(S_AABB_HH, i);
    int32_t x0 = 0, y0 = 0, x1 = -1, y1 = -1;
    uint32_t count = 0;
    const bool ok = cell_index(ax - hw, A.cell, &x0) && cell_index(ay - hh, A.cell, &y0) &&
                    cell_index(ax + hw, A.cell, &x1) && cell_index(ay + hh, A.cell, &y1);
    if (!ok) {
        atomicExch(&A.cnt[LC_NONFINITE], 1u);
        x1 = x0 - 1;
    } else if (x1 >= x0 && y1 >= y0) {
        const unsigned long long c64 =
            (unsigned long long)((int64_t)x1 - (int64_t)x0 + 1) * (unsigned long long)((int64_t)y1 - (int64_t)y0 + 1);
        if (c64 > MAX_CELL_ENTRIES) {
            atomicExch(&A.cnt[LC_BIG], 1u);
            x1 = x0 - 1;
        } else {
            count = (uint32_t)c64;
        }
    }
    A.rx0[i] = x0; A.ry0[i] = y0; A.rx1[i] = x1; A.ry1[i] = y1;
    A.bcnt[i] = count;
    return count;
}

// The cell-entry total is summed per warp first: one atomic per warp
// instead of one per body on a single counter.
__global__ void lk_load(Phase1 A) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    unsigned long long sum = i < A.n ? load_body(A, i) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31u) == 0 && sum) atomicAdd(A.entries, sum);
}

// One thread per cell entry (a wall can cover hundreds of cells): after the
// scan of the counts, entry e belongs to the last body whose first entry is
// at most e, and is that body's (e - first)-th cell in row-major order.
__global__ void lk_emit(Phase1 A, uint32_t E) {
    const uint32_t e = blockIdx.x * LT + threadIdx.x;
    if (e >= E) return;
    uint32_t lo = 0, hi = A.n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (A.bcnt[mid] <= e) lo = mid;
        else hi = mid;
    }
    const uint32_t i = lo, r = e - A.bcnt[i];
    const uint32_t w = (uint32_t)(A.rx1[i] - A.rx0[i] + 1);
    const int32_t xi = A.rx0[i] + (int32_t)(r % w), yi = A.ry0[i] + (int32_t)(r / w);
    const uint32_t bk = cell_bucket(xi, yi, A.bmod);
    A.ebucket[e] = bk;
    A.ebody[e] = i;
    atomicAdd(&A.table[bk], 1u);
}

// after the scan: table[b] = first slot of bucket b; afterwards one past its last
__global__ void lk_scatter(Phase1 A, uint32_t E) {
    const uint32_t e = blockIdx.x * LT + threadIdx.x;
    if (e >= E) return;
    const uint32_t slot = atomicAdd(&A.table[A.ebucket[e]], 1u);
    A.sbody[slot] = A.ebody[e];
    A.eslot[e] = slot;
}

__device__ __forceinline__ bool lk_excluded(const unsigned long long* ex, uint32_t n, unsigned long long key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        const unsigned long long v = __ldg(ex + mid);
        if (v == key) return true;
        if (v < key) lo = mid + 1;
        else hi = mid;
    }
    return false;
}

// Candidates: every two entries of one bucket, filtered as lib.zig:273-282,
// deduplicated like its "manifold already exists" test (lib.zig:278-281).
// PAIR_GROUP lanes per entry take the bucket's later entries PAIR_GROUP at a
// time (a pyramid cell holds ~16 entries, a sparse box's ~3).
constexpr uint32_t PAIR_GROUP = 8;
__global__ void lk_pairs(Phase1 A, uint32_t E) {
    const uint64_t w = ((uint64_t)blockIdx.x * LT + threadIdx.x) / PAIR_GROUP;
    if (w >= E) return;
    const uint32_t e = (uint32_t)w, lane = threadIdx.x % PAIR_GROUP;
    const uint32_t i = A.ebody[e];
    const uint32_t end = A.table[A.ebucket[e]];
    const f2 pi = {A.st(S_AABB_X, i), A.st(S_AABB_Y, i)};
    const float hwi = A.st(S_AABB_HW, i), hhi = A.st(S_AABB_HH, i);
    const bool sti = (A.s.kind[i] & K_STATIC) != 0;
    const unsigned long long mask = (unsigned long long)A.hs - 1ull;
    for (uint32_t q = A.eslot[e] + 1u + lane; q < end; q += PAIR_GROUP) {
        const uint32_t j = A.sbody[q];
        if (j == i) continue;
        if (sti && (A.s.kind[j] & K_STATIC)) continue;
        if (!aabb_intersects(pi, hwi, hhi, f2{A.st(S_AABB_X, j), A.st(S_AABB_Y, j)}, A.st(S_AABB_HW, j),
                             A.st(S_AABB_HH, j)))
            continue;
        const uint32_t lo = min(i, j), hi = max(i, j);
        const unsigned long long key = ((unsigned long long)lo << 32) | hi;
        if (A.nexcl && lk_excluded(A.excl, A.nexcl, key)) continue;
        unsigned long long h = key * 0x9E3779B97F4A7C15ull;
        h ^= h >> 31;
        bool fresh = false, placed = false;
        for (unsigned long long probe = 0; probe <= mask; ++probe) {
            const unsigned long long slot = (h + probe) & mask;
            const unsigned long long prev = atomicCAS(&A.hset[slot], ~0ull, key);
            if (prev == ~0ull || prev == key) {
                fresh = prev == ~0ull;
                placed = true;
                break;
            }
        }
        if (!placed) {
            atomicExch(&A.cnt[LC_PAIR_OVERFLOW], 1u);
            return;
        }
        if (fresh) {
            const uint32_t idx = atomicAdd(&A.cnt[LC_PAIRS], 1u);
            if (idx < A.np) A.pairs[idx] = key;
            else atomicExch(&A.cnt[LC_PAIR_OVERFLOW], 1u);
        }
    }
}

// Body i as the polygon-capable SAT sees it: a disc, a rectangle (its four
// vertices) or a polygon (its own ring).
__device__ __forceinline__ void narrow_geo(const Phase1& A, uint32_t i, GeoPoly& g) {
    const SWT<uint32_t>& s = A.s;
    const uint8_t k = s.kind[i];
    if (k & K_POLY) {
        const size_t gi = (size_t)A.base + i;
        geo_make_polygon(g, f2{s.px[i], s.py[i]}, A.poly_v + gi * MAX_POLY_VERTS, A.poly_nv[gi], s.cs[i], s.sn[i]);
    } else {
        geo_make(g, f2{s.px[i], s.py[i]}, k & K_RECT, A.pr(P_DIM0, i), A.pr(P_DIM1, i), s.cs[i], s.sn[i]);
    }
}

// performNarrowSAT + manifold build (collision.zig:299-320, lib.zig:284-294)
// One pair's manifold and contact points into the solver arrays.
__device__ void narrow_write(const Phase1& A, uint32_t o1, uint32_t o2, const SatState& sat, const NewPoint* pts,
                             int npt) {
    const SWT<uint32_t>& s = A.s;
    const uint32_t ref = sat.ref_is_first ? o1 : o2, inc = sat.ref_is_first ? o2 : o1;
    const uint32_t m = atomicAdd(&A.cnt[LC_MANIFOLDS], 1u);
    const uint32_t p0 = atomicAdd(&A.cnt[LC_POINTS], (uint32_t)npt);
    if (m >= A.nm || p0 + npt > A.npt) return;  // cannot happen: sized from the pair count
    s.ma[m] = ref;
    s.mb[m] = inc;
    s.mp0[m] = p0;
    s.mnp[m] = (uint8_t)npt;
    s.nx[m] = sat.normal.x;
    s.ny[m] = sat.normal.y;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (k >= npt) break;
        const uint32_t p = p0 + k;
        s.r1x[p] = pts[k].ref_r.x;
        s.r1y[p] = pts[k].ref_r.y;
        s.r2x[p] = pts[k].inc_r.x;
        s.r2y[p] = pts[k].inc_r.y;
        s.depth[p] = pts[k].depth;
        s.odepth[p] = pts[k].depth;
        s.apn[p] = 0.f;
        s.apt[p] = 0.f;
        if (s.cpn) {
            s.cpn[p] = 0.f;
            s.cpt[p] = 0.f;
        }
    }
}

// SAT and contact points of pair pi, o1 = the lower id (performNarrowSAT,
// collision.zig:299-320), on one thread.
__device__ void narrow_pair(const Phase1& A, uint32_t pi) {
    const SWT<uint32_t>& s = A.s;
    const unsigned long long key = A.pairs[pi];
    const uint32_t lo = (uint32_t)(key >> 32), hi = (uint32_t)key;
    const uint32_t o1 = __ldg(A.ids + A.base + lo) < __ldg(A.ids + A.base + hi) ? lo : hi;
    const uint32_t o2 = o1 == lo ? hi : lo;
    SatState sat;
    NewPoint pts[2];
    int npt = 0;
    if (A.poly_v) {  // an engine with polygons: every pair through the polygon-capable geometry
        GeoPoly g1, g2;
        narrow_geo(A, o1, g1);
        narrow_geo(A, o2, g2);
        if (!perform_narrow_sat(g1, g2, sat)) return;
        npt = sat.ref_is_first ? identify_points(g1, g2, sat.refid, pts) : identify_points(g2, g1, sat.refid, pts);
    } else {
        Geo g1, g2;
        geo_make(g1, f2{s.px[o1], s.py[o1]}, s.kind[o1] & K_RECT, A.pr(P_DIM0, o1), A.pr(P_DIM1, o1), s.cs[o1],
                 s.sn[o1]);
        geo_make(g2, f2{s.px[o2], s.py[o2]}, s.kind[o2] & K_RECT, A.pr(P_DIM0, o2), A.pr(P_DIM1, o2), s.cs[o2],
                 s.sn[o2]);
        if (!perform_narrow_sat(g1, g2, sat)) return;
        npt = sat.ref_is_first ? identify_points(g1, g2, sat.refid, pts) : identify_points(g2, g1, sat.refid, pts);
    }
    narrow_write(A, o1, o2, sat, pts, npt);
}

__global__ void lk_narrow(Phase1 A, uint32_t npairs) {
    const uint32_t pi = blockIdx.x * LT + threadIdx.x;
    if (pi >= npairs) return;
    narrow_pair(A, pi);
}

// ---------------------------------------------------------------------------
// colouring (r2d_colour.h) by Jones-Plassmann rounds
// ---------------------------------------------------------------------------
constexpr uint32_t NO_NODE = 0xFFFFFFFFu;
constexpr uint32_t PRED_ROW = 64;  // earlier neighbours kept per constraint (two 21-contact bodies: 36)

struct Colouring {
    uint32_t count;
    bool joints;  // joints: every named body is a node; contacts: non-static bodies
    const uint8_t* jtype;
    const uint32_t* jb1;
    const uint32_t* jb2;
    const uint32_t* ma;
    const uint32_t* mb;
    const uint8_t* kind;
    uint8_t* colour;  // 0xFF = not yet coloured
    uint32_t *adj, *adjl, *prio, *cursor;
    uint32_t* cnt;
    uint32_t* npred;  // earlier neighbours of each constraint (null: rounds walk the adjacency)
    uint32_t* preds;  // their indices, PRED_ROW a constraint (those with more walk the adjacency)
    uint32_t* wl[2];  // worklists of the constraints a round left uncoloured (null: rounds scan all)
    // Rounds allowed before the colouring gives up (LC_STUCK); 0 = count + 1,
    // more than the count ever needs, since every round colours at least one.
    uint32_t round_limit;

    __device__ void ends(uint32_t i, uint32_t* a, uint32_t* b) const {
        *a = NO_NODE;
        *b = NO_NODE;
        if (joints) {
            const uint32_t b1 = __ldg(jb1 + i), b2 = __ldg(jb2 + i);
            *a = b1;
            if (joint_two_bodies(__ldg(jtype + i)) && b2 != b1) *b = b2;
        } else {
            const uint32_t x = ma[i], y = mb[i];
            if (!(kind[x] & K_STATIC)) *a = x;
            if (!(kind[y] & K_STATIC)) *b = y;
        }
    }
    // the order among equal mixes: the joint index, or the contact's (lo, hi)
    __device__ unsigned long long tie(uint32_t i) const {
        if (joints) return i;
        const uint32_t x = ma[i], y = mb[i];
        return ((unsigned long long)min(x, y) << 32) | max(x, y);
    }
};

__global__ void lk_col_count(Colouring C) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i >= C.count) return;
    uint32_t a, b;
    C.ends(i, &a, &b);
    if (a != NO_NODE) atomicAdd(&C.adj[a], 1u);
    if (b != NO_NODE) atomicAdd(&C.adj[b], 1u);
}

__global__ void lk_col_fill(Colouring C) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i >= C.count) return;
    uint32_t a, b;
    C.ends(i, &a, &b);
    if (a != NO_NODE) C.adjl[atomicAdd(&C.cursor[a], 1u)] = i;
    if (b != NO_NODE) C.adjl[atomicAdd(&C.cursor[b], 1u)] = i;
    if (C.joints) {
        C.prio[i] = r2d_colour_mix(i, R2D_COLOUR_JOINT_SALT);
    } else {
        const uint32_t x = C.ma[i], y = C.mb[i];
        C.prio[i] = r2d_colour_mix(min(x, y), max(x, y));
    }
    C.colour[i] = 0xFFu;
}

// Constraint i's neighbours that come before it in priority order, into its
// row of preds (PRED_ROW entries); npred[i] is their number, which may
// exceed the row (the rounds then walk the adjacency instead).  A neighbour
// through both ends is listed twice, which changes no colour.
__global__ void lk_col_preds(Colouring C) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i >= C.count) return;
    uint32_t ends[2];
    C.ends(i, &ends[0], &ends[1]);
    const uint32_t pi = C.prio[i];
    const unsigned long long ti = C.tie(i);
    uint32_t* row = C.preds + (size_t)i * PRED_ROW;
    uint32_t k = 0;
    for (int e2 = 0; e2 < 2; ++e2) {
        const uint32_t x = ends[e2];
        if (x == NO_NODE) continue;
        const uint32_t q1 = C.adj[x + 1];
#pragma unroll 4
        for (uint32_t q = C.adj[x]; q < q1; ++q) {
            const uint32_t o = C.adjl[q];
            if (o == i) continue;
            const uint32_t po = C.prio[o];
            if (po > pi || (po == pi && C.tie(o) > ti)) continue;  // comes later
            if (k < PRED_ROW) row[k] = o;
            ++k;
        }
    }
    C.npred[i] = k;
}

// One round's test of constraint i: if every earlier neighbour (in priority
// order) has a colour, i takes the lowest colour none of them holds.  Returns
// 1 while i stays uncoloured.  A colour, once written, is final, so reading
// one written in this same round is as good as reading it next round, and a
// stale read only defers i by a round: the colours are read from L2
// (ld.global.cg), which sees every earlier round's writes.  (A volatile load
// here would be a system-scope access, several microseconds apiece on a
// coherent CPU-GPU node.)
__device__ uint32_t colour_try(const Colouring& C, uint32_t i) {
    const uint8_t* col = C.colour;
    if (__ldcg(col + i) != 0xFFu) return 0u;
    const uint32_t np = C.npred ? C.npred[i] : NO_NODE;
    if (np <= PRED_ROW) {  // the listed earlier neighbours: independent loads, no walk
        const uint32_t* row = C.preds + (size_t)i * PRED_ROW;
        ColourSet used;
        bool ready = true;
#pragma unroll 4
        for (uint32_t q = 0; q < np; ++q) {
            const uint8_t c = __ldcg(col + row[q]);
            if (c == 0xFFu) ready = false;
            else used.add(c);
        }
        if (!ready) return 1u;
        uint32_t c = used.first_free();
        if (c >= (uint32_t)MAX_COLOURS) {
            atomicExch(&C.cnt[LC_COLOURS], 1u);
            c = 0u;
        }
        C.colour[i] = (uint8_t)c;
        return 0u;
    }
    uint32_t ends[2];
    C.ends(i, &ends[0], &ends[1]);
    const uint32_t pi = C.prio[i];
    const unsigned long long ti = C.tie(i);
    ColourSet used;
    for (int e2 = 0; e2 < 2; ++e2) {
        const uint32_t x = ends[e2];
        if (x == NO_NODE) continue;
        const uint32_t q1 = C.adj[x + 1];
        for (uint32_t q = C.adj[x]; q < q1; ++q) {
            const uint32_t o = C.adjl[q];
            if (o == i) continue;
            const uint32_t po = C.prio[o];
            if (po > pi || (po == pi && C.tie(o) > ti)) continue;  // comes later
            const uint8_t c = __ldcg(col + o);
            if (c == 0xFFu) return 1u;
            used.add(c);
        }
    }
    uint32_t c = used.first_free();
    if (c >= (uint32_t)MAX_COLOURS) {
        atomicExch(&C.cnt[LC_COLOURS], 1u);
        c = 0u;
    }
    C.colour[i] = (uint8_t)c;
    return 0u;
}

// colour_try for a constraint known to be open whose earlier neighbours fit
// its row, read 16 at a time: a chunk's used 16-byte pieces, then all its
// neighbours' colours, are loaded at once (two memory round trips a chunk;
// most constraints need one chunk).  It stops at the first chunk that holds
// an uncoloured neighbour.
__device__ __forceinline__ uint32_t colour_try_row(const Colouring& C, uint32_t i) {
    const uint32_t np = C.npred[i];
    if (np > PRED_ROW) return colour_try(C, i);
    const uint4* row4 = reinterpret_cast<const uint4*>(C.preds + (size_t)i * PRED_ROW);
    // colours below 32 (nearly always): one word of the set, one shift and OR each
    uint32_t w0 = 0u, high = 0u;
    for (uint32_t at = 0; at < np; at += 16) {
        uint32_t o[16];
#pragma unroll
        for (uint32_t v = 0; v < 4; ++v) {
            const uint4 r = at + 4 * v < np ? __ldcg(row4 + at / 4 + v) : make_uint4(0u, 0u, 0u, 0u);
            o[4 * v] = r.x;
            o[4 * v + 1] = r.y;
            o[4 * v + 2] = r.z;
            o[4 * v + 3] = r.w;
        }
        uint32_t c[16];
#pragma unroll
        for (uint32_t q = 0; q < 16; ++q) c[q] = at + q < np ? (uint32_t)__ldcg(C.colour + o[q]) : 0u;
        uint32_t any_open = 0u;
#pragma unroll
        for (uint32_t q = 0; q < 16; ++q) {
            if (at + q >= np) break;
            any_open |= c[q] == 0xFFu;
            high |= c[q] >> 5;
            w0 |= 1u << (c[q] & 31u);
        }
        if (any_open) return 1u;
    }
    uint32_t col;
    if (high == 0u) {
        col = w0 == 0xFFFFFFFFu ? 32u : (uint32_t)__ffs(~w0) - 1u;
    } else {  // a colour of 32 or more: the full set, from the row again
        ColourSet used;
        const uint32_t* row = C.preds + (size_t)i * PRED_ROW;
        for (uint32_t q = 0; q < np; ++q) used.add(__ldcg(C.colour + __ldcg(row + q)));
        col = used.first_free();
    }
    if (col >= (uint32_t)MAX_COLOURS) {
        atomicExch(&C.cnt[LC_COLOURS], 1u);
        col = 0u;
    }
    C.colour[i] = (uint8_t)col;
    return 0u;
}

// Every Jones-Plassmann round, in one cluster of CT-thread CTAs
// (r2d_colour.h's order).  With worklists, each thread keeps the constraints
// it holds that are still open in its own slots of the round's list (slot
// t + j * nt of wl[r & 1] for its j-th), so rounds need no atomics: round 0
// holds constraint t + j * nt, round r re-tries what the thread kept from
// round r - 1.  Without them every round re-scans all constraints.  A thread
// that leaves one open sets flag slot r % 3; the flag of round r + 1 is
// cleared in round r, and each thread reads slot r % 3 between the barrier
// after round r and the next barrier, two rounds before the slot is cleared
// again, so all threads see the same flag and leave the loop together.
// Expects flag slot 0 zeroed.
constexpr int CT = 1024;  // threads per CTA of the colouring cluster
__global__ void __launch_bounds__(CT, 1) lk_colour_cluster(Colouring C) {
    const uint32_t t0 = blockIdx.x * CT + threadIdx.x, nt = gridDim.x * CT;
    const bool listed = C.wl[0] != nullptr && C.npred != nullptr;
    uint32_t* cnt = C.cnt;
    uint32_t held = C.count > t0 ? (C.count - t0 - 1) / nt + 1 : 0u;  // constraints this thread holds
    const uint32_t limit = C.round_limit ? C.round_limit : C.count + 1u;
    for (uint32_t round = 0;; ++round) {
        if (t0 == 0) cnt[LC_PEND0 + (round + 1) % 3] = 0u;
        bool open = false;
        if (listed) {
            const uint32_t* in = round > 0 ? C.wl[(round + 1) & 1] : nullptr;
            uint32_t* out = C.wl[round & 1];
            uint32_t kept = 0;
            for (uint32_t j = 0; j < held; ++j) {
                const uint32_t i = in ? __ldcg(in + t0 + j * nt) : t0 + j * nt;
                if (colour_try_row(C, i)) out[t0 + (kept++) * nt] = i;
            }
            held = kept;
            open = kept > 0;
        } else {
            for (uint32_t i = t0; i < C.count; i += nt) open |= colour_try(C, i) != 0u;
        }
        if (open) cnt[LC_PEND0 + round % 3] = 1u;
        cluster_sync_all();
        if (__ldcg(cnt + LC_PEND0 + round % 3) == 0u) {
            if (t0 == 0) cnt[LC_ROUNDS] = round + 1;
            break;
        }
        // each round colours at least the highest-priority uncoloured
        // constraint, so only a limit below the count can end here
        if (round + 1u >= limit) {
            if (t0 == 0) cnt[LC_STUCK] = 1u;
            break;
        }
    }
}

// A colouring's result block (words): per-colour counts, cursors, offsets
// (colour c is order[off[c], off[c+1])) and the number of colours.
constexpr uint32_t CB_HIST = 0, CB_CURSOR = MAX_COLOURS, CB_OFF = 2 * MAX_COLOURS, CB_NCOL = 3 * MAX_COLOURS + 1,
                   CB_WORDS = 4 * MAX_COLOURS;
constexpr uint32_t H_WORDS = H_COLOUR + 2 * LC_N + 2 * CB_WORDS;
static_assert(MAX_COLOURS == 128, "the offsets warp scans four colours a lane");

// per-colour counts, one global add per block and colour
__global__ void lk_col_hist(Colouring C, uint32_t* cb) {
    __shared__ uint32_t h[MAX_COLOURS];
    for (uint32_t c = threadIdx.x; c < (uint32_t)MAX_COLOURS; c += LT) h[c] = 0u;
    __syncthreads();
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i < C.count) {
        const uint32_t c = C.colour[i];
        if (c < (uint32_t)MAX_COLOURS) atomicAdd(&h[c], 1u);
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < (uint32_t)MAX_COLOURS; c += LT)
        if (h[c]) atomicAdd(&cb[CB_HIST + c], h[c]);
}

// exclusive offsets of the colours (one warp, four colours a lane)
__global__ void lk_col_offsets(uint32_t* cb) {
    const uint32_t lane = threadIdx.x;
    uint32_t h[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        h[k] = cb[CB_HIST + 4 * lane + k];
        sum += h[k];
    }
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    uint32_t run = x - sum, top = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        cb[CB_OFF + 4 * lane + k] = run;
        cb[CB_CURSOR + 4 * lane + k] = run;
        run += h[k];
        if (h[k]) top = 4 * lane + k + 1;
    }
    top = __reduce_max_sync(0xffffffffu, top);
    if (lane == 31) cb[CB_OFF + MAX_COLOURS] = x;
    if (lane == 0) cb[CB_NCOL] = top;
}

// colour-major order; inside a colour the order is free (body-disjoint), so
// a block reserves one range per colour and fills it in any order
__global__ void lk_col_order(Colouring C, uint32_t* cb, uint32_t* order) {
    __shared__ uint32_t h[MAX_COLOURS], base[MAX_COLOURS];
    for (uint32_t c = threadIdx.x; c < (uint32_t)MAX_COLOURS; c += LT) h[c] = 0u;
    __syncthreads();
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    uint32_t c = 0xFFu, rank = 0;
    if (i < C.count) {
        c = C.colour[i];
        if (c < (uint32_t)MAX_COLOURS) rank = atomicAdd(&h[c], 1u);
    }
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < (uint32_t)MAX_COLOURS; q += LT)
        if (h[q]) base[q] = atomicAdd(&cb[CB_CURSOR + q], h[q]);
    __syncthreads();
    if (c < (uint32_t)MAX_COLOURS) order[base[c] + rank] = i;
}

// Manifolds and their points in colour-major order: manifold k of dst is
// manifold order[k] of src, and its points are 2k and 2k + 1.  Each colour
// then is one contiguous range, read with coalesced loads and no index
// indirection.  Fields the pre-step derives (friction, masses, bias) are not
// copied.
__global__ void lk_permute(SWT<uint32_t> src, SWT<uint32_t> dst, const uint32_t* order, uint32_t M) {
    const uint32_t k = blockIdx.x * LT + threadIdx.x;
    if (k >= M) return;
    const uint32_t m = order[k];
    const uint32_t p0 = src.mp0[m], np = src.mnp[m];
    dst.ma[k] = src.ma[m];
    dst.mb[k] = src.mb[m];
    dst.mp0[k] = 2 * k;
    dst.mnp[k] = (uint8_t)np;
    dst.mcol[k] = src.mcol[m];
    dst.nx[k] = src.nx[m];
    dst.ny[k] = src.ny[m];
    for (uint32_t j = 0; j < np; ++j) {
        const uint32_t p = p0 + j, q = 2 * k + j;
        dst.r1x[q] = src.r1x[p];
        dst.r1y[q] = src.r1y[p];
        dst.r2x[q] = src.r2x[p];
        dst.r2y[q] = src.r2y[p];
        dst.depth[q] = src.depth[p];
        dst.odepth[q] = src.odepth[p];
        dst.apn[q] = src.apn[p];
        dst.apt[q] = src.apt[p];
        if (src.cpn) {
            dst.cpn[q] = src.cpn[p];
            dst.cpt[q] = src.cpt[p];
        }
    }
}

// The contact solve's records: per colour-major manifold seven float4 (v0 =
// bodies and normal, v1 = friction, point count and static flags, biases,
// v2 / v3 = the lever arms of points 0 / 1, v4 = their effective masses,
// v5 = their accumulated impulses, live during the step, v6 = both bodies'
// 1/mass and 1/inertia).  A warp reads each with one coalesced 16-byte load
// instead of a scalar load per field, and the per-body constants come with
// the manifold instead of from two scattered bodies.  mom4, when set, holds
// each body's live momentum {px, py, L, 0} during the step (one scattered
// load and store per body instead of three); worlds with joints or warm
// starting keep it in the state rows, which their other solvers use.
struct Packed {
    float4 *v0, *v1, *v2, *v3, *v4, *v5, *v6;
    float4* mom4;
    float4* v7;  // compensated mode: the accumulators' compensation words, as v5; else null
};
constexpr uint32_t PK_NP = 0xFFu, PK_STATIC_A = 0x100u, PK_STATIC_B = 0x200u;  // v1.y bits

// calculateImpulses (collision.zig:135-218) of colour-major manifold m from
// its packed record: solve_contact's arithmetic in the same order.  Seven
// coalesced record loads are issued together, then the two bodies'
// momenta; the accumulators go back as one store.
struct MRec {  // one manifold's packed record
    float4 v0, v1, v2, v3, v4, v5, v6;
};

__device__ __forceinline__ MRec load_rec(const Packed& pk, uint32_t m) {
    return MRec{pk.v0[m], pk.v1[m], pk.v2[m], pk.v3[m], pk.v4[m], pk.v5[m], pk.v6[m]};
}

template <bool MOM4>
__device__ __forceinline__ void solve_contact_rec(const Packed& pk, const MRec& rec, float* mx, float* my, float* L,
                                                  uint32_t m, bool warm) {
    const float4 v0 = rec.v0, v1 = rec.v1, v2 = rec.v2, v3 = rec.v3, v4 = rec.v4, v5 = rec.v5, v6 = rec.v6;
    const uint32_t a = __float_as_uint(v0.x), b = __float_as_uint(v0.y), flags = __float_as_uint(v1.y);
    const uint32_t np = flags & PK_NP;
    const bool sa = flags & PK_STATIC_A, sb = flags & PK_STATIC_B;
    const f2 n = {v0.z, v0.w};
    const float fr = v1.x;
    const float bias[2] = {v1.z, v1.w};
    const f2 r1s[2] = {{v2.x, v2.y}, {v3.x, v3.y}}, r2s[2] = {{v2.z, v2.w}, {v3.z, v3.w}};
    const float mn[2] = {v4.x, v4.z}, mt[2] = {v4.y, v4.w};
    float apn[2] = {v5.x, v5.z}, apt[2] = {v5.y, v5.w};
    float4 v7 = pk.v7 ? pk.v7[m] : make_float4(0.f, 0.f, 0.f, 0.f);
    float cpn[2] = {v7.x, v7.z}, cpt[2] = {v7.y, v7.w};
    const float inv_m1 = v6.x, inv_i1 = v6.y, inv_m2 = v6.z, inv_i2 = v6.w;
    float4 ma4, mb4;
    if (MOM4) {
        ma4 = pk.mom4[a];
        mb4 = pk.mom4[b];
    } else {
        ma4 = make_float4(mx[a], my[a], L[a], 0.f);
        mb4 = make_float4(mx[b], my[b], L[b], 0.f);
    }
    const f2 vlinear_1 = scale2(f2{ma4.x, ma4.y}, inv_m1);
    const float omega1 = ma4.z * inv_i1;
    const f2 vlinear_2 = scale2(f2{mb4.x, mb4.y}, inv_m2);
    const float omega2 = mb4.z * inv_i2;
    const f2 t = cw90(n);
    f2 alp1 = {0.f, 0.f}, alp2 = {0.f, 0.f};
    float arp1 = 0.f, arp2 = 0.f;
#pragma unroll
    for (uint32_t k = 0; k < 2; ++k) {
        if (k >= np) break;
        if (bias[k] < 0.0f) continue;  // depth >= 0: accumulators stay 0 (collision.zig:154-158)
        const f2 r1 = r1s[k], r2 = r2s[k];
        const f2 v1 = add2(vlinear_1, f2{-r1.y * omega1, r1.x * omega1});
        const f2 v2 = add2(vlinear_2, f2{-r2.y * omega2, r2.x * omega2});
        const f2 dv = sub2(v1, v2);
        float num = dot2(dv, n) + bias[k];
        const float pn = num * mn[k];
        if (!warm && pn < MIN_MANIFOLD_IMPULSE) continue;
        num = dot2(dv, t);
        const float pt = num * mt[k];
        float applied_pn, applied_pt;
        if (pk.v7) {  // compensated (r2d_accum.h), as accumulate() in r2d_solve.cuh
            applied_pn = r2d_acc_add_max(&apn[k], &cpn[k], pn, 0.0f);
            const float max_pt = fr * fabsf(apn[k]);
            applied_pt = r2d_acc_add_clamp(&apt[k], &cpt[k], pt, -max_pt, max_pt);
        } else {
            const float acc = apn[k];
            const float nacc = zmax(0.0f, acc + pn);
            applied_pn = nacc - acc;
            apn[k] = nacc;
            const float max_pt = fr * fabsf(nacc);
            const float acct = apt[k];
            const float nacct = zclamp(acct + pt, -max_pt, max_pt);
            applied_pt = nacct - acct;
            apt[k] = nacct;
        }
        const f2 dp = add2(scale2(n, applied_pn), scale2(t, applied_pt));
        if (!sa) {
            alp1 = sub2(alp1, dp);
            arp1 -= cross2(r1, dp);
        }
        if (!sb) {
            alp2 = add2(alp2, dp);
            arp2 += cross2(r2, dp);
        }
    }
    pk.v5[m] = make_float4(apn[0], apt[0], apn[1], apt[1]);
    if (pk.v7) pk.v7[m] = make_float4(cpn[0], cpt[0], cpn[1], cpt[1]);
    if (!sa) {
        if (MOM4) {
            pk.mom4[a] = make_float4(ma4.x + alp1.x, ma4.y + alp1.y, ma4.z + arp1, 0.f);
        } else {
            mx[a] = ma4.x + alp1.x;
            my[a] = ma4.y + alp1.y;
            L[a] = ma4.z + arp1;
        }
    }
    if (!sb) {
        if (MOM4) {
            pk.mom4[b] = make_float4(mb4.x + alp2.x, mb4.y + alp2.y, mb4.z + arp2, 0.f);
        } else {
            mx[b] = mb4.x + alp2.x;
            my[b] = mb4.y + alp2.y;
            L[b] = mb4.z + arp2;
        }
    }
}

__device__ __forceinline__ void solve_contact_rec(const Packed& pk, const MRec& rec, float* mx, float* my, float* L,
                                                  uint32_t m, bool warm) {
    if (pk.mom4) solve_contact_rec<true>(pk, rec, mx, my, L, m, warm);
    else solve_contact_rec<false>(pk, rec, mx, my, L, m, warm);
}

__device__ __forceinline__ void solve_contact_packed(const Packed& pk, float* mx, float* my, float* L, uint32_t m,
                                                     bool warm) {
    solve_contact_rec(pk, load_rec(pk, m), mx, my, L, m, warm);
}

// ---------------------------------------------------------------------------
// substeps (lib.zig:199-250)
// ---------------------------------------------------------------------------
struct Phase2 {
    SWT<uint32_t> s;
    Packed pk;
    float* state;
    const float* props;
    uint32_t NB, base, n, nman;
    float h;
    bool first, last, disc_rot;
    uint32_t ngrav;
    float g[MAX_GRAVITY];
    const uint4* jhead;     // colour-major joints: {type, body 1, body 2, -}
    const float* jprm_cm;   // and their parameters, [k][JOINT_PARAMS]
    uint32_t k0, k1;        // the colour-major constraints one per-colour launch solves
    double* pos64;          // f64 pose (FP64-positions mode), else null
    const float2* poly_v;   // polygons (as Phase1), else null
    const uint8_t* poly_nv;
    bool warm;              // warm starting

    __device__ float& st(int f, uint32_t i) const { return state[(size_t)f * NB + base + i]; }
    __device__ float pr(int f, uint32_t i) const { return __ldg(props + (size_t)f * NB + base + i); }
};

// forces (DownwardsGravity.zig:35-39), AABB (last substep), velocities (lib.zig:200-216)
__device__ __forceinline__ void forces_one(const Phase2& A, uint32_t i, bool first, bool last) {
    const SWT<uint32_t>& s = A.s;
    const uint8_t k = s.kind[i];
    float fx = 0.f, fy = 0.f, tq = 0.f;
    if (first) {  // user-set force / torque (RigidBody.zig:73,78)
        fx = A.st(S_FORCE_X, i);
        fy = A.st(S_FORCE_Y, i);
        tq = A.st(S_TORQUE, i);
        // a dynamic body's force / torque is cleared after integration (lib.zig:247-248)
        if (!(k & K_STATIC) && (fx != 0.f || fy != 0.f || tq != 0.f)) s.kind[i] = k | K_FORCED;
    }
    if (!(k & K_STATIC)) {
        for (uint32_t gg = 0; gg < A.ngrav; ++gg) {
            fx += 0.0f * s.mass(i);
            fy += (-A.g[gg]) * s.mass(i);
        }
    }
    if (last) {
        float hw, hh;
        if (k & K_POLY) {
            const size_t gi = (size_t)A.base + i;
            polygon_half_extents(A.poly_v + gi * MAX_POLY_VERTS, A.poly_nv[gi], s.cs[i], s.sn[i], &hw, &hh);
        } else if (k & K_RECT) {
            rect_half_extents(A.pr(P_DIM0, i), A.pr(P_DIM1, i), s.cs[i], s.sn[i], &hw, &hh);
        } else {
            hw = hh = A.pr(P_DIM0, i);
        }
        A.st(S_AABB_X, i) = s.px[i];
        A.st(S_AABB_Y, i) = s.py[i];
        A.st(S_AABB_HW, i) = hw;
        A.st(S_AABB_HH, i) = hh;
    }
    if (!(k & K_STATIC)) {
        s.mx[i] += fx * A.h;
        s.my[i] += fy * A.h;
        s.L[i] += tq * A.h;
        s.tq[i] = tq;
    }
    if (A.pk.mom4) A.pk.mom4[i] = make_float4(s.mx[i], s.my[i], s.L[i], 0.f);
}

__global__ void lk_forces(Phase2 A) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i < A.n) forces_one(A, i, A.first, A.last);
}

// updateTGSDepth + preStep (collision.zig:73-133)
__device__ __forceinline__ void prestep_one(const Phase2& A, uint32_t m) {
    const SWT<uint32_t>& s = A.s;
    const uint32_t a = s.ma[m], b = s.mb[m];
    const f2 n2 = {s.nx[m], s.ny[m]};
    const uint32_t p0 = s.mp0[m], np = s.mnp[m];
    for (uint32_t k = 0; k < np; ++k) {
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
    const float inv_m1 = s.inv_m[a], inv_m2 = s.inv_m[b];
    const float inv_mass = inv_m1 + inv_m2;
    const float inv_i1 = s.inv_i[a], inv_i2 = s.inv_i[b];
    const f2 t2 = cw90(n2);
    s.fric[m] = sqrtf(A.pr(P_MU, a) * A.pr(P_MU, b));
    for (uint32_t k = 0; k < np; ++k) {
        const uint32_t p = p0 + k;
        const f2 r1 = {s.r1x[p], s.r1y[p]}, r2 = {s.r2x[p], s.r2y[p]};
        const float r1n = cross2(r1, n2), r2n = cross2(r2, n2);
        const float kn = inv_mass + inv_i1 * (r1n * r1n) + inv_i2 * (r2n * r2n);
        const float r1t = cross2(r1, t2), r2t = cross2(r2, t2);
        const float kt = inv_mass + inv_i1 * (r1t * r1t) + inv_i2 * (r2t * r2t);
        s.mn[p] = kn > 0.0f ? 1.0f / kn : 0.0f;
        s.mt[p] = kt > 0.0f ? 1.0f / kt : 0.0f;
        // bias of calculateImpulses (collision.zig:154-172); the depth is fixed within a substep
        const float d = s.depth[p];
        s.bias[p] = d >= 0.0f ? -1.0f : BAUMGARTE * zmax(0.0f, (-d) - BAUMGARTE_SLOP) / A.h;
    }
}

// The solve's record of colour-major manifold m (points 2m, 2m + 1), from
// the fields the pre-step just wrote (slot 1 of a one-point manifold carries
// whatever it holds, unused).  The first substep also starts the live
// accumulators from the manifold's stored ones, except that a point with
// depth >= 0 (bias < 0) starts from zero, as the warm start leaves it.
__device__ __forceinline__ void pack_one(const Phase2& A, uint32_t m, bool first) {
    const SWT<uint32_t>& s = A.s;
    const uint32_t p = 2 * m;
    const float b0 = s.bias[p], b1 = s.bias[p + 1];
    const uint32_t a = s.ma[m], b = s.mb[m];
    const uint32_t flags = (uint32_t)s.mnp[m] | ((s.kind[a] & K_STATIC) ? PK_STATIC_A : 0u) |
                           ((s.kind[b] & K_STATIC) ? PK_STATIC_B : 0u);
    A.pk.v0[m] = make_float4(__uint_as_float(a), __uint_as_float(b), s.nx[m], s.ny[m]);
    A.pk.v1[m] = make_float4(s.fric[m], __uint_as_float(flags), b0, b1);
    A.pk.v6[m] = make_float4(s.inv_m[a], s.inv_i[a], s.inv_m[b], s.inv_i[b]);
    A.pk.v2[m] = make_float4(s.r1x[p], s.r1y[p], s.r2x[p], s.r2y[p]);
    A.pk.v3[m] = make_float4(s.r1x[p + 1], s.r1y[p + 1], s.r2x[p + 1], s.r2y[p + 1]);
    A.pk.v4[m] = make_float4(s.mn[p], s.mt[p], s.mn[p + 1], s.mt[p + 1]);
    if (first) {
        const bool z0 = b0 < 0.0f, z1 = b1 < 0.0f;
        A.pk.v5[m] = make_float4(z0 ? 0.f : s.apn[p], z0 ? 0.f : s.apt[p], z1 ? 0.f : s.apn[p + 1],
                                 z1 ? 0.f : s.apt[p + 1]);
        if (A.pk.v7)
            A.pk.v7[m] = make_float4(z0 ? 0.f : s.cpn[p], z0 ? 0.f : s.cpt[p], z1 ? 0.f : s.cpn[p + 1],
                                     z1 ? 0.f : s.cpt[p + 1]);
    }
}

// the live accumulators back into the manifold's fields (end of the step)
__device__ __forceinline__ void unpack_one(const Phase2& A, uint32_t m) {
    const float4 v = A.pk.v5[m];
    const uint32_t p = 2 * m, np = A.s.mnp[m];
    A.s.apn[p] = v.x;
    A.s.apt[p] = v.y;
    if (np > 1) {
        A.s.apn[p + 1] = v.z;
        A.s.apt[p + 1] = v.w;
    }
    if (A.pk.v7) {
        const float4 c = A.pk.v7[m];
        A.s.cpn[p] = c.x;
        A.s.cpt[p] = c.y;
        if (np > 1) {
            A.s.cpn[p + 1] = c.z;
            A.s.cpt[p + 1] = c.w;
        }
    }
}

__global__ void lk_prestep(Phase2 A) {
    const uint32_t m = blockIdx.x * LT + threadIdx.x;
    if (m >= A.nman) return;
    prestep_one(A, m);
    pack_one(A, m, A.first);
}

__global__ void lk_unpack(Phase2 A) {
    const uint32_t m = blockIdx.x * LT + threadIdx.x;
    if (m < A.nman) unpack_one(A, m);
}

__global__ void lk_contacts(Phase2 A) {
    const uint32_t k = A.k0 + blockIdx.x * LT + threadIdx.x;
    if (k >= A.k1) return;
    solve_contact_packed(A.pk, A.s.mx, A.s.my, A.s.L, k, A.warm);
}

// ---- warm starting: the world's tables of last frame's impulses ----
// Keys are the bodies' stable ids (warm_key_ids); `ids` is this world's id array.
__global__ void lk_warm_load(SWT<uint32_t> s, const uint32_t* ids, uint32_t M, const unsigned long long* keys,
                             const float4* vals, const float4* cvals, uint32_t hs) {
    const uint32_t m = blockIdx.x * LT + threadIdx.x;
    if (m >= M) return;
    const int slot = warm_find(keys, hs, warm_key_ids(__ldg(ids + s.ma[m]), __ldg(ids + s.mb[m])));
    if (slot < 0) return;
    const float4 v = vals[slot];
    const uint32_t p0 = s.mp0[m], np = s.mnp[m];
    if (np > 0) {
        s.apn[p0] = v.x;
        s.apt[p0] = v.y;
    }
    if (np > 1) {
        s.apn[p0 + 1] = v.z;
        s.apt[p0 + 1] = v.w;
    }
    if (s.cpn && cvals) {
        const float4 c = cvals[slot];
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

__global__ void lk_warm_apply(Phase2 A) {
    const uint32_t k = A.k0 + blockIdx.x * LT + threadIdx.x;
    if (k >= A.k1) return;
    warm_apply_contact<false>(A.s, k);
}

__global__ void lk_warm_clear(unsigned long long* keys, uint32_t hs) {
    const uint32_t q = blockIdx.x * LT + threadIdx.x;
    if (q < hs) keys[q] = ~0ull;
}

__global__ void lk_warm_store(SWT<uint32_t> s, const uint32_t* ids, uint32_t M, unsigned long long* keys,
                              float4* vals, float4* cvals, uint32_t hs) {
    const uint32_t m = blockIdx.x * LT + threadIdx.x;
    if (m >= M) return;
    const uint32_t p0 = s.mp0[m], np = s.mnp[m];
    const int slot = warm_claim(keys, hs, warm_key_ids(__ldg(ids + s.ma[m]), __ldg(ids + s.mb[m])));
    if (slot < 0) return;
    vals[slot] = make_float4(np > 0 ? s.apn[p0] : 0.f, np > 0 ? s.apt[p0] : 0.f, np > 1 ? s.apn[p0 + 1] : 0.f,
                             np > 1 ? s.apt[p0 + 1] : 0.f);
    if (cvals)
        cvals[slot] = s.cpn ? make_float4(np > 0 ? s.cpn[p0] : 0.f, np > 0 ? s.cpt[p0] : 0.f,
                                          np > 1 ? s.cpn[p0 + 1] : 0.f, np > 1 ? s.cpt[p0 + 1] : 0.f)
                            : make_float4(0.f, 0.f, 0.f, 0.f);
}

// another table of the same format (a fused world's, or one the host built)
// into this path's
__global__ void lk_warm_copy(const unsigned long long* keys, const float4* vals, const float4* cvals, uint32_t hs,
                             unsigned long long* nkeys, float4* nvals, float4* ncvals, uint32_t nhs) {
    const uint32_t q = blockIdx.x * LT + threadIdx.x;
    if (q >= hs) return;
    const unsigned long long key = keys[q];
    if (key == ~0ull) return;
    const int slot = warm_claim(nkeys, nhs, key);
    if (slot < 0) return;
    nvals[slot] = vals[q];
    if (ncvals) ncvals[slot] = cvals ? cvals[q] : make_float4(0.f, 0.f, 0.f, 0.f);
}

// the joint at colour-major position k (one coalesced head, 32 B of parameters)
__device__ __forceinline__ void joint_one(const Phase2& A, uint32_t k) {
    const uint4 h = A.jhead[k];
    solve_joint(A.s, (uint8_t)h.x, h.y, h.z, A.jprm_cm + (size_t)k * JOINT_PARAMS, A.h);
}

__global__ void lk_joints(Phase2 A) {
    const uint32_t k = A.k0 + blockIdx.x * LT + threadIdx.x;
    if (k < A.k1) joint_one(A, k);
}

// joints in colour-major order: position k holds joint order[k]
__global__ void lk_joint_pack(const uint8_t* jtype, const uint32_t* jb1, const uint32_t* jb2, const float* jprm,
                              const uint32_t* order, uint32_t nj, uint4* jhead, float* jprm_cm) {
    const uint32_t k = blockIdx.x * LT + threadIdx.x;
    if (k >= nj) return;
    const uint32_t j = order[k];
    jhead[k] = make_uint4(jtype[j], jb1[j], jb2[j], 0u);
    const float4* src = reinterpret_cast<const float4*>(jprm + (size_t)j * JOINT_PARAMS);
    float4* dst = reinterpret_cast<float4*>(jprm_cm + (size_t)k * JOINT_PARAMS);
    dst[0] = src[0];
    dst[1] = src[1];
}

// integration (lib.zig:238-249); the last substep clears consumed forces
__device__ __forceinline__ void integrate_one(const Phase2& A, uint32_t i, bool last) {
    const SWT<uint32_t>& s = A.s;
    s.ang_prev[i] = s.ang[i];
    const uint8_t k = s.kind[i];
    if (k & K_STATIC) return;
    if (A.pk.mom4) {  // the solve's momentum back into the state rows
        const float4 q = A.pk.mom4[i];
        s.mx[i] = q.x;
        s.my[i] = q.y;
        s.L[i] = q.z;
    }
    if (A.pos64) {
        integrate_pose64(A.pos64, A.NB, A.base + i, s.mx[i], s.my[i], s.L[i], A.h, s.mass(i), s.inertia(i), &s.px[i],
                         &s.py[i], &s.ang[i]);
    } else {
        const float sm_ = A.h / s.mass(i);
        s.px[i] += s.mx[i] * sm_;
        s.py[i] += s.my[i] * sm_;
        s.ang[i] += s.L[i] * A.h / s.inertia(i);
    }
    s.tq[i] = 0.f;
    if (!last && ((k & (K_RECT | K_POLY)) || A.disc_rot)) {
        float c, sn;
        r2d_sincosf(s.ang[i], &sn, &c);
        s.cs[i] = c;
        s.sn[i] = sn;
    }
    if (last && (k & K_FORCED)) {
        A.st(S_FORCE_X, i) = 0.f;
        A.st(S_FORCE_Y, i) = 0.f;
        A.st(S_TORQUE, i) = 0.f;
    }
}

__global__ void lk_integrate(Phase2 A) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i < A.n) integrate_one(A, i, A.last);
}

// The colour offsets of one step: contact colour c is manifolds [coff[c],
// coff[c+1]), joint colour c is packed joints [joff[c], joff[c+1]) (both
// colour-major).
struct ResidentPlan {
    const uint32_t* coff;
    const uint32_t* joff;
    uint32_t ncol, njcol, sub_steps, iters;
};

// Every substep of the step in one cluster (lib.zig:199-250): the same
// per-item functions as the one-launch-per-phase kernels, in the same order.
// A body's integration and its next substep's forces touch only that body,
// so they share a phase; so do the forces and the pre-step (the pre-step
// reads no momentum).
__global__ void __launch_bounds__(RT, 1) lk_substeps_resident(Phase2 A, ResidentPlan R) {
    const uint32_t t0 = blockIdx.x * RT + threadIdx.x, nt = gridDim.x * RT;
    for (uint32_t sub = 0; sub < R.sub_steps; ++sub) {
        const bool first = sub == 0, last = sub + 1 == R.sub_steps;
        if (first)
            for (uint32_t i = t0; i < A.n; i += nt) forces_one(A, i, true, last);
        for (uint32_t m = t0; m < A.nman; m += nt) {
            prestep_one(A, m);
            pack_one(A, m, first);
        }
        cluster_sync_all();
        if (A.warm && first) {
            for (uint32_t c = 0; c < R.ncol; ++c) {
                const uint32_t k1 = R.coff[c + 1];
                for (uint32_t k = R.coff[c] + t0; k < k1; k += nt) warm_apply_contact<false>(A.s, k);
                cluster_sync_all();
            }
        }
        MRec cur;
        for (uint32_t it = 0; it < R.iters; ++it) {
            for (uint32_t c = 0; c < R.njcol; ++c) {
                const uint32_t k1 = R.joff[c + 1];
                for (uint32_t k = R.joff[c] + t0; k < k1; k += nt) joint_one(A, k);
                cluster_sync_all();
            }
            // Software-pipelined: the thread's first manifold of the next
            // contact colour (the next iteration's first colour after the
            // last) is loaded before this colour is solved.  Within a
            // substep a record changes only in its accumulators, which only
            // the manifold's own thread writes (manifold k of colour c is
            // always thread (k - coff[c]) mod nt's), so the early load sees
            // their latest values, unless the next manifold is this one
            // (a single colour), whose accumulators are then reloaded.
            for (uint32_t c = 0; c < R.ncol; ++c) {
                const uint32_t k0 = R.coff[c] + t0, k1 = R.coff[c + 1];
                const uint32_t cn = c + 1 < R.ncol ? c + 1 : 0u;
                const bool more = c + 1 < R.ncol || it + 1 < R.iters;
                const uint32_t kn = R.coff[cn] + t0;
                MRec next;
                if (more && kn < R.coff[cn + 1]) next = load_rec(A.pk, kn);
                if (k0 < k1) {
                    if (c > 0 || it > 0) {
                        if (R.ncol == 1) cur.v5 = A.pk.v5[k0];
                    } else {
                        cur = load_rec(A.pk, k0);
                    }
                    solve_contact_rec(A.pk, cur, A.s.mx, A.s.my, A.s.L, k0, A.warm);
                }
                for (uint32_t k = k0 + nt; k < k1; k += nt)
                    solve_contact_packed(A.pk, A.s.mx, A.s.my, A.s.L, k, A.warm);
                cur = next;
                cluster_sync_all();
            }
        }
        for (uint32_t i = t0; i < A.n; i += nt) {
            integrate_one(A, i, last);
            if (!last) forces_one(A, i, false, sub + 2 == R.sub_steps);
        }
        if (!last) cluster_sync_all();
    }
    for (uint32_t m = t0; m < A.nman; m += nt) unpack_one(A, m);
}

// One iteration's contact colours in one cluster, a cluster barrier between
// colours: for worlds whose joint colours are too large for the resident
// kernel but whose contact colours are not.
__global__ void __launch_bounds__(RT, 1) lk_contacts_cluster(Phase2 A, const uint32_t* coff, uint32_t ncol) {
    const uint32_t t0 = blockIdx.x * RT + threadIdx.x, nt = gridDim.x * RT;
    for (uint32_t c = 0; c < ncol; ++c) {
        const uint32_t k1 = coff[c + 1];
        for (uint32_t k = coff[c] + t0; k < k1; k += nt) solve_contact_packed(A.pk, A.s.mx, A.s.my, A.s.L, k, A.warm);
        if (c + 1 < ncol) cluster_sync_all();
    }
}

// sleeping mode (r2d_sleep.h): is any non-static body still moving?
__global__ void lk_still(SWT<uint32_t> s, uint32_t n, uint32_t* moving) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    bool m = false;
    if (i < n && !(s.kind[i] & K_STATIC)) m = !r2d_body_still(s.mx[i], s.my[i], s.L[i], s.inv_m[i], s.inv_i[i]);
    if (__any_sync(0xffffffffu, m) && (threadIdx.x & 31u) == 0) atomicOr(moving, 1u);
}

__global__ void lk_sleep_update(const uint32_t* moving, uint32_t* frames) {
    *frames = r2d_sleep_next(*frames, *moving == 0u);
}

// debug taps in the oracle's manifold layout (DebugOut)
__global__ void lk_dump(SWT<uint32_t> s, uint32_t m_count, uint32_t* keys, float* data, uint32_t* colours) {
    const uint32_t m = blockIdx.x * LT + threadIdx.x;
    if (m >= m_count) return;
    keys[2 * m] = s.ma[m];
    keys[2 * m + 1] = s.mb[m];
    colours[m] = s.mcol[m];
    float* d = data + (size_t)m * DEBUG_MF;
    const f2 nn = {s.nx[m], s.ny[m]};
    const f2 tt = cw90(nn);
    const uint32_t np = s.mnp[m], p0 = s.mp0[m];
    d[0] = nn.x; d[1] = nn.y; d[2] = tt.x; d[3] = tt.y; d[4] = s.fric[m];
    d[5] = np > 0 ? 1.f : 0.f;
    d[6] = np > 1 ? 1.f : 0.f;
    d[7] = s.ang_prev[s.ma[m]];
    d[8] = s.ang_prev[s.mb[m]];
    for (uint32_t k = 0; k < 2; ++k) {
        float* q = d + 9 + 12 * k;
        const bool has = k < np;
        const uint32_t p = p0 + k;
        q[0] = __int_as_float(0x7fc00000);
        q[1] = __int_as_float(0x7fc00000);
        q[2] = has ? s.r1x[p] : 0.f;
        q[3] = has ? s.r1y[p] : 0.f;
        q[4] = has ? s.r2x[p] : 0.f;
        q[5] = has ? s.r2y[p] : 0.f;
        q[6] = has ? s.depth[p] : 0.f;
        q[7] = has ? s.odepth[p] : 0.f;
        q[8] = has ? s.mn[p] : 0.f;
        q[9] = has ? s.mt[p] : 0.f;
        q[10] = has ? s.apn[p] : 0.f;
        q[11] = has ? s.apt[p] : 0.f;
    }
}

__global__ void lk_widen(const uint8_t* in, uint32_t n, uint32_t* out) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i < n) out[i] = in[i];
}

// A group of device arrays that share one element capacity.
struct Buf {
    void** p;
    size_t elem;
};
#define LB(x) Buf{(void**)&(x), sizeof(*(x))}

cudaError_t regrow(size_t& cap, size_t need, std::initializer_list<Buf> bufs) {
    if (need <= cap) return cudaSuccess;
    const size_t c = need + need / 4 + 64;
    for (const Buf& b : bufs) {
        if (*b.p) cudaFree(*b.p);
        *b.p = nullptr;
    }
    cap = 0;
    for (const Buf& b : bufs) {
        cudaError_t e = cudaMalloc(b.p, c * b.elem);
        if (e != cudaSuccess) return e;
    }
    cap = c;
    return cudaSuccess;
}

constexpr int MAX_DEVICES = 64;
std::atomic<int> g_cluster_size[3][MAX_DEVICES];  // [resident kernel][device]; 0 = not known yet

// The cluster size of a resident kernel: 16 CTAs where the device can hold
// such a cluster with the kernel's resources, else the portable 8.  Found
// once per device and kernel.
template <class... P>
cudaError_t resident_cluster(int which, void (*kernel)(P...), int threads, int* out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    int cl = g_cluster_size[which][dev].load();
    if (cl == 0) {
        cl = 8;
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(16);
            cfg.blockDim = dim3(threads);
            cudaLaunchAttribute at{};
            at.id = cudaLaunchAttributeClusterDimension;
            at.val.clusterDim.x = 16;
            at.val.clusterDim.y = 1;
            at.val.clusterDim.z = 1;
            cfg.attrs = &at;
            cfg.numAttrs = 1;
            int nc = 0;
            if (cudaOccupancyMaxActiveClusters(&nc, kernel, &cfg) == cudaSuccess && nc > 0) cl = 16;
        }
        (void)cudaGetLastError();  // a refused probe leaves no error behind
        g_cluster_size[which][dev].store(cl);
    }
    *out = cl;
    return cudaSuccess;
}

// One cluster of `cl` CTAs: the whole grid of a resident kernel.
template <class... P, class... A>
cudaError_t launch_resident(void (*kernel)(P...), int cl, int threads, cudaStream_t st, A... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(cl);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at{};
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = cl;
    at.val.clusterDim.y = 1;
    at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Exclusive scan of a[0..n) (a[n] = total): one block for short arrays, else
// tiles, their sums (tsum, ceil(n / SCAN_TILE) + 1 words) and a fix-up.
cudaError_t scan(uint32_t* a, uint32_t n, uint32_t* tsum, cudaStream_t st, uint32_t* nlaunch) {
    if (n <= SCAN_ONE_BLOCK || !tsum) {
        lk_scan<<<1, SCAN_THREADS, 0, st>>>(a, n);
        *nlaunch += 1;
    } else {
        const uint32_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
        lk_scan_tiles<<<tiles, SCAN_THREADS, 0, st>>>(a, n, tsum);
        lk_scan<<<1, SCAN_THREADS, 0, st>>>(tsum, tiles);
        lk_scan_add<<<(n + 256) / 256, 256, 0, st>>>(a, n, tsum, tiles);
        *nlaunch += 3;
    }
    return cudaGetLastError();
}

// Whether the substeps run as one resident cluster, or as one launch per
// phase and colour, with an iteration's contact colours then in one cluster
// launch when they fit.  The cluster wins while its threads cover a colour in
// a few passes.  R2D_RESIDENT forces a choice: 1 the resident cluster, 0 one
// launch per colour throughout, 2 per-colour joints with clustered contacts.
int resident_override() {
    static const int forced = [] {
        const char* e = getenv("R2D_RESIDENT");
        return e && *e ? atoi(e) : -1;
    }();
    return forced;
}

bool use_resident_substeps(uint32_t largest_colour, int cl) {
    const int o = resident_override();
    if (o >= 0) return o == 1;
    return largest_colour <= RESIDENT_MAX_PASSES * (uint32_t)cl * RT;
}

bool use_contacts_cluster(uint32_t largest_contact_colour, int cl) {
    const int o = resident_override();
    if (o >= 0) return o == 2;
    return largest_contact_colour <= RESIDENT_MAX_PASSES * (uint32_t)cl * RT;
}

}  // namespace

struct LargeWorld::Impl {
    size_t cap_n = 0, cap_t = 0, cap_e = 0, cap_hs = 0, cap_p = 0, cap_m = 0, cap_pt = 0, cap_c = 0, cap_j = 0,
           cap_d = 0, cap_dd = 0;
    // bodies
    float *inv_m = nullptr, *inv_i = nullptr, *cs = nullptr, *sn = nullptr, *tq = nullptr, *ang_prev = nullptr;
    uint8_t* kind = nullptr;
    int32_t *rx0 = nullptr, *ry0 = nullptr, *rx1 = nullptr, *ry1 = nullptr;
    uint32_t *bcnt = nullptr, *adj = nullptr, *cursor = nullptr;
    // spatial hash
    uint32_t* table = nullptr;
    uint32_t *ebucket = nullptr, *ebody = nullptr, *eslot = nullptr, *sbody = nullptr;
    unsigned long long *hset = nullptr, *pairs = nullptr;
    // manifolds and points
    uint32_t *ma = nullptr, *mb = nullptr, *mp0 = nullptr, *corder = nullptr;
    uint8_t *mnp = nullptr, *mcol = nullptr;
    float *nx = nullptr, *ny = nullptr, *fric = nullptr;
    float *r1x = nullptr, *r1y = nullptr, *r2x = nullptr, *r2y = nullptr, *depth = nullptr, *odepth = nullptr;
    float *mn = nullptr, *mt = nullptr, *apn = nullptr, *apt = nullptr, *bias = nullptr;
    float *cpn = nullptr, *cpt = nullptr;  // compensation words (compensated mode)
    float4* pk[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // Packed records
    float4* mom4 = nullptr;
    // the permutation's second copy of the fields it moves (swapped with the first after each step's permutation)
    uint32_t *ma2 = nullptr, *mb2 = nullptr, *mp02 = nullptr;
    uint8_t *mnp2 = nullptr, *mcol2 = nullptr;
    float *nx2 = nullptr, *ny2 = nullptr;
    float *r1x2 = nullptr, *r1y2 = nullptr, *r2x2 = nullptr, *r2y2 = nullptr, *depth2 = nullptr, *odepth2 = nullptr,
          *apn2 = nullptr, *apt2 = nullptr, *cpn2 = nullptr, *cpt2 = nullptr;
    // colouring
    uint32_t *adjl = nullptr, *prio = nullptr;
    uint32_t *jadj = nullptr, *jadjl = nullptr, *jprio = nullptr;  // the joints' own adjacency
    uint32_t *npred = nullptr, *jnpred = nullptr, *preds = nullptr, *jpreds = nullptr;
    uint32_t *wl0 = nullptr, *wl1 = nullptr, *jwl0 = nullptr, *jwl1 = nullptr;  // colouring worklists
    // colour-major joints, and the joint arrays they were coloured from
    uint4* jhead = nullptr;
    float* jprm_cm = nullptr;
    size_t cap_jh = 0, cap_jp = 0;
    uint64_t joint_epoch = 0;
    uint32_t joint_nj = 0;
    size_t cap_pr = 0, cap_prr = 0;
    uint8_t* jcol = nullptr;
    uint32_t* jorder = nullptr;
    uint32_t* cnt = nullptr;                // LargeCounter; a second block for the joint colouring
    unsigned long long* entries = nullptr;  // total cell entries
    uint32_t* hist = nullptr;               // two colouring result blocks (contacts, joints)
    uint32_t* tsum = nullptr;               // tile sums of the multi-block scan
    size_t cap_ts = 0;
    int cl_solve = 0, cl_colour = 0, cl_contacts = 0;  // cluster sizes of the resident kernels
    uint32_t* h_cnt = nullptr;              // pinned: counters, then the entry total
    // debug taps
    uint32_t *dk = nullptr, *dc = nullptr;
    float* dd = nullptr;

    // warm starting: two tables (last frame's = wcur), sizes in slots
    unsigned long long* wkeys[2] = {nullptr, nullptr};
    float4* wvals[2] = {nullptr, nullptr};
    float4* wcvals[2] = {nullptr, nullptr};  // compensated mode
    size_t wcap[2] = {0, 0};
    uint32_t whs[2] = {0, 0};
    int wcur = 0;

    double pair_scale = 1.0;  // grows when the candidate-pair set overflows
    uint32_t nman = 0, nj = 0, nlaunch = 0, npairs = 0;
    std::vector<uint32_t> coff, joff;

    ~Impl() {
        void* ps[] = {inv_m, inv_i, cs, sn, tq, ang_prev, kind, rx0, ry0, rx1, ry1, bcnt, adj, cursor,
                      table, ebucket, ebody, eslot, sbody, hset, pairs, ma, mb, mp0, corder, mnp, mcol,
                      nx, ny, fric, r1x, r1y, r2x, r2y, depth, odepth, mn, mt, apn, apt, bias, adjl, prio,
                      jcol, jorder, cnt, entries, hist, tsum, dk, dc, dd, ma2, mb2, mp02, mnp2, mcol2, nx2, ny2,
                      r1x2, r1y2, r2x2, r2y2, depth2, odepth2, apn2, apt2, jadj, jadjl, jprio, npred, jnpred,
                      preds, jpreds, pk[0], pk[1], pk[2], pk[3], pk[4], pk[5], pk[6], pk[7], mom4, wl0, wl1, jwl0,
                      jwl1, jhead, jprm_cm, cpn, cpt, cpn2, cpt2};
        for (void* p : ps)
            if (p) cudaFree(p);
        for (int b = 0; b < 2; ++b) {
            if (wkeys[b]) cudaFree(wkeys[b]);
            if (wvals[b]) cudaFree(wvals[b]);
            if (wcvals[b]) cudaFree(wcvals[b]);
        }
        if (h_cnt) cudaFreeHost(h_cnt);
    }

    SWT<uint32_t> views(const LargeInputs& in) const {
        SWT<uint32_t> s{};
        float* S = in.state;
        const size_t NB = in.NB;
        s.px = S + (size_t)S_POS_X * NB + in.base;
        s.py = S + (size_t)S_POS_Y * NB + in.base;
        s.ang = S + (size_t)S_ANGLE * NB + in.base;
        s.mx = S + (size_t)S_MOM_X * NB + in.base;
        s.my = S + (size_t)S_MOM_Y * NB + in.base;
        s.L = S + (size_t)S_ANG_MOM * NB + in.base;
        s.inv_m = inv_m; s.inv_i = inv_i; s.cs = cs; s.sn = sn; s.ang_prev = ang_prev; s.tq = tq;
        s.px0 = nullptr; s.py0 = nullptr; s.pos0 = false;
        s.gmass = in.props + (size_t)P_MASS * NB + in.base;
        s.ginertia = in.props + (size_t)P_INERTIA * NB + in.base;
        s.kind = kind;
        s.ma = ma; s.mb = mb; s.mp0 = mp0; s.mnp = mnp; s.mcol = mcol;
        s.nx = nx; s.ny = ny; s.fric = fric;
        s.r1x = r1x; s.r1y = r1y; s.r2x = r2x; s.r2y = r2y;
        s.depth = depth; s.odepth = odepth; s.mn = mn; s.mt = mt; s.apn = apn; s.apt = apt; s.bias = bias;
        s.cpn = in.comp ? cpn : nullptr;
        s.cpt = in.comp ? cpt : nullptr;
        return s;
    }
    // the permutation's destination: views() with the second copies
    SWT<uint32_t> shadow_views(const LargeInputs& in) const {
        SWT<uint32_t> s = views(in);
        s.ma = ma2; s.mb = mb2; s.mp0 = mp02; s.mnp = mnp2; s.mcol = mcol2; s.nx = nx2; s.ny = ny2;
        s.r1x = r1x2; s.r1y = r1y2; s.r2x = r2x2; s.r2y = r2y2; s.depth = depth2; s.odepth = odepth2;
        s.apn = apn2; s.apt = apt2;
        s.cpn = in.comp ? cpn2 : nullptr;
        s.cpt = in.comp ? cpt2 : nullptr;
        return s;
    }
    void swap_shadow() {
        std::swap(ma, ma2); std::swap(mb, mb2); std::swap(mp0, mp02); std::swap(mnp, mnp2); std::swap(mcol, mcol2);
        std::swap(nx, nx2); std::swap(ny, ny2); std::swap(r1x, r1x2); std::swap(r1y, r1y2); std::swap(r2x, r2x2);
        std::swap(r2y, r2y2); std::swap(depth, depth2); std::swap(odepth, odepth2); std::swap(apn, apn2);
        std::swap(apt, apt2); std::swap(cpn, cpn2); std::swap(cpt, cpt2);
    }
};

LargeWorld::LargeWorld() : impl(new Impl()) {}
LargeWorld::~LargeWorld() { delete impl; }

#define LTRY(expr)                                                     \
    do {                                                               \
        cudaError_t e_ = (expr);                                       \
        if (e_ != cudaSuccess) {                                       \
            *msg = std::string(#expr) + ": " + cudaGetErrorString(e_); \
            return e_ == cudaErrorMemoryAllocation ? -3 : -4;          \
        }                                                              \
    } while (0)
#define LAUNCH(kernel, grid, ...)                   \
    do {                                            \
        kernel<<<(grid), LT, 0, st>>>(__VA_ARGS__); \
        ++I.nlaunch;                                \
    } while (0)
#define SCAN(a, n) LTRY(scan((a), (n), I.tsum, st, &I.nlaunch))

int LargeWorld::step(const LargeInputs& in, float dt, uint32_t sub_steps, uint32_t iters, cudaStream_t st,
                     std::string* msg) {
    Impl& I = *impl;
    const uint32_t n = in.n;
    const auto t_start = std::chrono::steady_clock::now();
    double t_ms[5] = {0, 0, 0, 0, 0};  // cells+entries, pairs, narrowphase, colouring, substeps (verbose)
    auto mark = [&](int k) {
        t_ms[k] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    };
    if (!I.h_cnt) LTRY(cudaMallocHost((void**)&I.h_cnt, sizeof(uint32_t) * H_WORDS));
    if (in.sleep && n) {  // a sleeping world is not stepped; its last frame's manifolds stay (r2d_sleep.h)
        LTRY(cudaMemcpyAsync(I.h_cnt, in.sleep, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        LTRY(cudaStreamSynchronize(st));
        if (I.h_cnt[0] >= R2D_SLEEP_FRAMES) {
            I.nlaunch = 0;
            return 0;
        }
    }
    I.nman = 0;
    I.nj = 0;
    I.nlaunch = 0;
    I.npairs = 0;
    I.coff.assign(1, 0u);
    I.joff.assign(1, 0u);
    if (n == 0) return 0;
    const uint32_t T = in.table_mult * n;
    if (!I.cnt) {
        LTRY(cudaMalloc((void**)&I.cnt, sizeof(uint32_t) * 2 * LC_N));
        LTRY(cudaMalloc((void**)&I.entries, sizeof(unsigned long long)));
        LTRY(cudaMalloc((void**)&I.hist, sizeof(uint32_t) * 2 * CB_WORDS));
        LTRY(resident_cluster(0, lk_substeps_resident, RT, &I.cl_solve));
        LTRY(resident_cluster(1, lk_colour_cluster, CT, &I.cl_colour));
        LTRY(resident_cluster(2, lk_contacts_cluster, RT, &I.cl_contacts));
    }
    LTRY(regrow(I.cap_n, (size_t)n + 1,
                {LB(I.inv_m), LB(I.inv_i), LB(I.cs), LB(I.sn), LB(I.tq), LB(I.ang_prev), LB(I.kind), LB(I.rx0),
                 LB(I.ry0), LB(I.rx1), LB(I.ry1), LB(I.bcnt), LB(I.adj), LB(I.jadj), LB(I.cursor),
                 LB(I.mom4)}));
    LTRY(regrow(I.cap_t, (size_t)T + 1, {LB(I.table)}));
    LTRY(regrow(I.cap_ts, std::max(n, T) / SCAN_TILE + 2, {LB(I.tsum)}));

    Phase1 A{};
    A.s = I.views(in);
    A.state = in.state; A.props = in.props; A.kind_in = in.kind; A.ids = in.ids;
    A.poly_v = in.poly_v; A.poly_nv = in.poly_nv;
    A.NB = in.NB; A.base = in.base; A.n = n; A.cell = in.cell;
    A.bmod = BucketMod{bucket_recip(T), T};
    A.disc_rot = in.disc_rot;
    A.rx0 = I.rx0; A.ry0 = I.ry0; A.rx1 = I.rx1; A.ry1 = I.ry1; A.bcnt = I.bcnt; A.table = I.table;
    A.excl = in.excl; A.nexcl = in.nexcl;
    A.cnt = I.cnt; A.entries = I.entries;

    // ---- cells: count them, then size the entry arrays exactly ----
    LTRY(cudaMemsetAsync(I.cnt, 0, sizeof(uint32_t) * LC_N, st));
    LTRY(cudaMemsetAsync(I.entries, 0, sizeof(unsigned long long), st));
    LTRY(cudaMemsetAsync(I.table, 0, sizeof(uint32_t) * ((size_t)T + 1), st));
    LAUNCH(lk_load, blocks(n), A);
    LTRY(cudaMemcpyAsync(I.h_cnt, I.cnt, sizeof(uint32_t) * LC_N, cudaMemcpyDeviceToHost, st));
    LTRY(cudaMemcpyAsync(I.h_cnt + LC_N, I.entries, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    LTRY(cudaStreamSynchronize(st));
    if (I.h_cnt[LC_NONFINITE]) {
        *msg = "a body's AABB is not finite (it has no spatial-hash cell)";
        return DS_NONFINITE;
    }
    unsigned long long E64 = 0;
    memcpy(&E64, I.h_cnt + LC_N, sizeof(E64));
    if (I.h_cnt[LC_BIG] || E64 > MAX_CELL_ENTRIES) {
        *msg = "the bodies cover more than 64Mi spatial-hash cells";
        return DS_CAPACITY;
    }
    const uint32_t E = (uint32_t)E64;
    mark(0);
    LTRY(regrow(I.cap_e, (size_t)E + 1, {LB(I.ebucket), LB(I.ebody), LB(I.eslot), LB(I.sbody)}));
    A.ebucket = I.ebucket; A.ebody = I.ebody; A.eslot = I.eslot; A.sbody = I.sbody;
    SCAN(I.bcnt, n);
    LAUNCH(lk_emit, blocks(E), A, E);
    SCAN(I.table, T);
    LAUNCH(lk_scatter, blocks(E), A, E);

    // ---- candidate pairs (the set grows until it holds them all) ----
    uint32_t npairs = 0;
    for (;;) {
        const double want = (3.25 * n + 64.0) * I.pair_scale;
        if (want > 1.0e9) {
            *msg = "more than 1e9 candidate pairs";
            return DS_CAPACITY;
        }
        const uint32_t np = (uint32_t)want;
        uint32_t hs = 1;
        while (hs < np + np / 2) hs <<= 1;
        LTRY(regrow(I.cap_p, np, {LB(I.pairs)}));
        LTRY(regrow(I.cap_hs, hs, {LB(I.hset)}));
        A.pairs = I.pairs; A.hset = I.hset; A.np = np; A.hs = hs;
        LTRY(cudaMemsetAsync(I.hset, 0xFF, sizeof(unsigned long long) * hs, st));
        LTRY(cudaMemsetAsync(I.cnt, 0, sizeof(uint32_t) * LC_N, st));
        LAUNCH(lk_pairs, blocks((uint64_t)PAIR_GROUP * E), A, E);
        LTRY(cudaMemcpyAsync(I.h_cnt, I.cnt, sizeof(uint32_t) * LC_N, cudaMemcpyDeviceToHost, st));
        LTRY(cudaStreamSynchronize(st));
        if (!I.h_cnt[LC_PAIR_OVERFLOW]) {
            npairs = I.h_cnt[LC_PAIRS];
            break;
        }
        I.pair_scale *= std::max(1.5, 1.25 * (double)I.h_cnt[LC_PAIRS] / (double)np);
    }

    mark(1);
    // ---- narrowphase: at most one manifold per pair, two points per manifold ----
    LTRY(regrow(I.cap_m, (size_t)npairs + 1,
                {LB(I.ma), LB(I.mb), LB(I.mp0), LB(I.corder), LB(I.mnp), LB(I.mcol), LB(I.nx), LB(I.ny),
                 LB(I.fric), LB(I.ma2), LB(I.mb2), LB(I.mp02), LB(I.mnp2), LB(I.mcol2), LB(I.nx2), LB(I.ny2),
                 LB(I.pk[0]), LB(I.pk[1]), LB(I.pk[2]), LB(I.pk[3]), LB(I.pk[4]), LB(I.pk[5]), LB(I.pk[6]),
                 LB(I.pk[7])}));
    LTRY(regrow(I.cap_pt, 2 * (size_t)npairs + 1,
                {LB(I.r1x), LB(I.r1y), LB(I.r2x), LB(I.r2y), LB(I.depth), LB(I.odepth), LB(I.mn), LB(I.mt),
                 LB(I.apn), LB(I.apt), LB(I.bias), LB(I.r1x2), LB(I.r1y2), LB(I.r2x2), LB(I.r2y2), LB(I.depth2),
                 LB(I.odepth2), LB(I.apn2), LB(I.apt2), LB(I.cpn), LB(I.cpt), LB(I.cpn2), LB(I.cpt2)}));
    A.s = I.views(in);
    I.npairs = npairs;
    A.nm = npairs;
    A.npt = 2 * npairs;
    LTRY(cudaMemsetAsync(I.cnt, 0, sizeof(uint32_t) * LC_N, st));
    LAUNCH(lk_narrow, blocks(npairs), A, npairs);
    LTRY(cudaMemcpyAsync(I.h_cnt, I.cnt, sizeof(uint32_t) * LC_N, cudaMemcpyDeviceToHost, st));
    LTRY(cudaStreamSynchronize(st));
    const uint32_t M = I.h_cnt[LC_MANIFOLDS];
    mark(2);

    // ---- colouring: contacts, then joints (Jones-Plassmann rounds) ----
    // Each colouring queues the rounds its previous step needed, then its
    // counts, offsets and order; one round trip then checks both, and only a
    // colouring that needed more rounds queues more.
    LTRY(regrow(I.cap_c, 2 * (size_t)std::max(M, in.nj) + 2,
                {LB(I.adjl), LB(I.prio), LB(I.jadjl), LB(I.jprio)}));
    LTRY(regrow(I.cap_j, (size_t)in.nj + 1, {LB(I.jcol), LB(I.jorder)}));
    LTRY(regrow(I.cap_pr, (size_t)std::max(M, in.nj) + 1,
                {LB(I.npred), LB(I.jnpred), LB(I.wl0), LB(I.wl1), LB(I.jwl0), LB(I.jwl1)}));
    LTRY(regrow(I.cap_prr, ((size_t)std::max(M, in.nj) + 1) * PRED_ROW, {LB(I.preds), LB(I.jpreds)}));
    LTRY(cudaMemsetAsync(I.cnt, 0, sizeof(uint32_t) * 2 * LC_N, st));
    uint32_t* cb_c = I.hist;
    uint32_t* cb_j = I.hist + CB_WORDS;
    uint32_t rounds[2] = {0, 0};
    // adjacency, earlier-neighbour rows, every round (one cluster), then the
    // colour counts, offsets and colour-major order
    auto colour = [&](bool joints, uint32_t count, uint8_t* col, uint32_t* order, uint32_t* cb, uint32_t* cnt,
                      uint32_t* adj, uint32_t* adjl, uint32_t* prio, uint32_t* npred, uint32_t* preds, uint32_t* wl0,
                      uint32_t* wl1) -> int {
        LTRY(cudaMemsetAsync(cb, 0, sizeof(uint32_t) * CB_WORDS, st));
        if (count == 0) return 0;
        Colouring C{};
        C.count = count;
        C.joints = joints;
        C.jtype = in.jtype; C.jb1 = in.jb1; C.jb2 = in.jb2;
        C.ma = I.ma; C.mb = I.mb; C.kind = I.kind; C.colour = col;
        C.adj = adj; C.adjl = adjl; C.prio = prio; C.cursor = I.cursor; C.cnt = cnt;
        C.npred = npred; C.preds = preds;
        C.wl[0] = wl0; C.wl[1] = wl1;
        C.round_limit = in.colour_round_limit;
        LTRY(cudaMemsetAsync(adj, 0, sizeof(uint32_t) * ((size_t)n + 1), st));
        LAUNCH(lk_col_count, blocks(count), C);
        SCAN(adj, n);
        LTRY(cudaMemcpyAsync(I.cursor, adj, sizeof(uint32_t) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
        LAUNCH(lk_col_fill, blocks(count), C);
        LAUNCH(lk_col_preds, blocks(count), C);
        LTRY(launch_resident(lk_colour_cluster, I.cl_colour, CT, st, C));
        ++I.nlaunch;
        LAUNCH(lk_col_hist, blocks(count), C, cb);
        lk_col_offsets<<<1, 32, 0, st>>>(cb);
        ++I.nlaunch;
        LAUNCH(lk_col_order, blocks(count), C, cb, order);
        return 0;
    };
    if (int r = colour(false, M, I.mcol, I.corder, cb_c, I.cnt, I.adj, I.adjl, I.prio, I.npred, I.preds, I.wl0,
                       I.wl1))
        return r;
    // The joint colouring depends on the joint arrays alone: it is kept while
    // their epoch stays the same.
    const bool joints_kept = in.nj && in.joint_epoch && in.joint_epoch == I.joint_epoch && in.nj == I.joint_nj;
    if (!joints_kept) {
        I.joint_epoch = 0;
        if (int r = colour(true, in.nj, I.jcol, I.jorder, cb_j, I.cnt + LC_N, I.jadj, I.jadjl, I.jprio, I.jnpred,
                           I.jpreds, I.jwl0, I.jwl1))
            return r;
        if (in.nj) {
            LTRY(regrow(I.cap_jh, in.nj, {LB(I.jhead)}));
            LTRY(regrow(I.cap_jp, (size_t)in.nj * JOINT_PARAMS, {LB(I.jprm_cm)}));
            LAUNCH(lk_joint_pack, blocks(in.nj), in.jtype, in.jb1, in.jb2, in.jprm, I.jorder, in.nj, I.jhead,
                   I.jprm_cm);
        }
    }
    // one round trip for both colourings: their flags and colour offsets
    uint32_t* hc = I.h_cnt + H_COLOUR;  // both counter blocks, then both result blocks
    LTRY(cudaMemcpyAsync(hc, I.cnt, sizeof(uint32_t) * 2 * LC_N, cudaMemcpyDeviceToHost, st));
    LTRY(cudaMemcpyAsync(hc + 2 * LC_N, I.hist, sizeof(uint32_t) * 2 * CB_WORDS, cudaMemcpyDeviceToHost, st));
    LTRY(cudaStreamSynchronize(st));
    for (int j = 0; j < 2; ++j) {
        const uint32_t* h = hc + j * LC_N;
        if (h[LC_COLOURS]) {
            *msg = "a constraint needs more than " + std::to_string(MAX_COLOURS) + " colours";
            return DS_CAPACITY;
        }
        if (h[LC_STUCK]) {
            *msg = "the colouring did not finish within its round limit";
            return DS_TIMEOUT;
        }
        rounds[j] = h[LC_ROUNDS];
    }
    if (in.nj && !joints_kept) {
        I.joint_epoch = in.joint_epoch;
        I.joint_nj = in.nj;
    }
    auto offsets = [&](const uint32_t* cb, std::vector<uint32_t>& off) {
        const uint32_t ncol = cb[CB_NCOL];
        off.assign(cb + CB_OFF, cb + CB_OFF + ncol + 1);
        uint32_t big = 0;
        for (uint32_t c = 0; c < ncol; ++c) big = std::max(big, off[c + 1] - off[c]);
        return big;
    };
    const uint32_t largest_contacts = offsets(hc + 2 * LC_N, I.coff);
    const uint32_t largest = std::max(largest_contacts, offsets(hc + 2 * LC_N + CB_WORDS, I.joff));
    I.nman = M;
    I.nj = in.nj;
    // manifolds in colour-major order: colour c is manifolds [coff[c], coff[c+1])
    if (M) {
        LAUNCH(lk_permute, blocks(M), I.views(in), I.shadow_views(in), I.corder, M);
        I.swap_shadow();
    }
    mark(3);

    const uint32_t* wids = in.ids + in.base;
    if (in.warm && M && I.whs[I.wcur]) {
        LAUNCH(lk_warm_load, blocks(M), I.views(in), wids, M, I.wkeys[I.wcur], I.wvals[I.wcur],
               in.comp ? I.wcvals[I.wcur] : nullptr, I.whs[I.wcur]);
    }
    // the table this call writes, sized for its manifolds (at most half full)
    const int wnext = 1 - I.wcur;
    uint32_t whs_next = 1;
    while (whs_next < 2u * M + 2u) whs_next <<= 1;
    if (in.warm) {
        LTRY(regrow(I.wcap[wnext], whs_next, {LB(I.wkeys[wnext]), LB(I.wvals[wnext]), LB(I.wcvals[wnext])}));
    }

    // ---- substeps: the world's state changes from here on ----
    Phase2 S{};
    S.s = I.views(in);
    S.state = in.state; S.props = in.props; S.NB = in.NB; S.base = in.base; S.n = n; S.nman = M;
    S.poly_v = in.poly_v; S.poly_nv = in.poly_nv;
    S.h = dt / (float)sub_steps;
    S.disc_rot = in.disc_rot;
    S.ngrav = in.ngrav;
    for (int k = 0; k < MAX_GRAVITY; ++k) S.g[k] = in.g[k];
    S.jhead = I.jhead; S.jprm_cm = I.jprm_cm;
    S.pos64 = in.pos64;
    S.warm = in.warm;
    S.pk = Packed{I.pk[0], I.pk[1], I.pk[2], I.pk[3], I.pk[4], I.pk[5], I.pk[6],
                  in.nj == 0 && !in.warm ? I.mom4 : nullptr, in.comp ? I.pk[7] : nullptr};
    const bool resident = use_resident_substeps(largest, I.cl_solve);
    // on the per-colour path, an iteration's contact colours may still share one cluster launch
    const bool contacts_clustered = !resident && M && I.coff.size() > 2 &&
                                    use_contacts_cluster(largest_contacts, I.cl_contacts);
    if (resident) {
        ResidentPlan R{};
        R.coff = cb_c + CB_OFF; R.joff = cb_j + CB_OFF;
        R.ncol = (uint32_t)I.coff.size() - 1; R.njcol = (uint32_t)I.joff.size() - 1;
        R.sub_steps = sub_steps; R.iters = iters;
        LTRY(launch_resident(lk_substeps_resident, I.cl_solve, RT, st, S, R));
        ++I.nlaunch;
    }
    for (uint32_t sub = 0; sub < sub_steps && !resident; ++sub) {
        S.first = sub == 0;
        S.last = sub + 1 == sub_steps;
        LAUNCH(lk_forces, blocks(n), S);
        if (M) LAUNCH(lk_prestep, blocks(M), S);
        if (in.warm && sub == 0) {  // the warm-started impulses, colour by colour
            for (size_t c = 0; c + 1 < I.coff.size(); ++c) {
                S.k0 = I.coff[c];
                S.k1 = I.coff[c + 1];
                LAUNCH(lk_warm_apply, blocks(S.k1 - S.k0), S);
            }
        }
        for (uint32_t it = 0; it < iters; ++it) {
            for (size_t c = 0; c + 1 < I.joff.size(); ++c) {
                S.k0 = I.joff[c];
                S.k1 = I.joff[c + 1];
                LAUNCH(lk_joints, blocks(S.k1 - S.k0), S);
            }
            if (contacts_clustered) {
                LTRY(launch_resident(lk_contacts_cluster, I.cl_contacts, RT, st, S, cb_c + CB_OFF,
                                     (uint32_t)I.coff.size() - 1));
                ++I.nlaunch;
                continue;
            }
            for (size_t c = 0; c + 1 < I.coff.size(); ++c) {
                S.k0 = I.coff[c];
                S.k1 = I.coff[c + 1];
                LAUNCH(lk_contacts, blocks(S.k1 - S.k0), S);
            }
        }
        LAUNCH(lk_integrate, blocks(n), S);
    }
    if (!resident && M) LAUNCH(lk_unpack, blocks(M), S);
    if (in.warm) {  // this call's impulses become the next call's start
        LAUNCH(lk_warm_clear, blocks(whs_next), I.wkeys[wnext], whs_next);
        if (M)
            LAUNCH(lk_warm_store, blocks(M), S.s, wids, M, I.wkeys[wnext], I.wvals[wnext],
                   in.comp ? I.wcvals[wnext] : nullptr, whs_next);
        I.whs[wnext] = whs_next;
        I.wcur = wnext;
    }
    if (in.sleep) {
        LTRY(cudaMemsetAsync(I.cnt + LC_MOVING, 0, sizeof(uint32_t), st));
        LAUNCH(lk_still, blocks(n), I.views(in), n, I.cnt + LC_MOVING);
        lk_sleep_update<<<1, 1, 0, st>>>(I.cnt + LC_MOVING, in.sleep);
        ++I.nlaunch;
    }
    LTRY(cudaGetLastError());
    if (in.verbose) {
        LTRY(cudaStreamSynchronize(st));
        mark(4);
        fprintf(stderr,
                "r2d grid step: %u bodies, %u entries, %u pairs, %u manifolds, %zu contact colours, %zu joint colours, "
                "largest colour %u, colouring rounds %u + %u, %s substeps, %u launches | ms: cells %.3f pairs %.3f "
                "narrow %.3f colour %.3f substeps %.3f\n",
                n, E, npairs, M, I.coff.size() - 1, I.joff.size() - 1, largest, rounds[0], rounds[1],
                resident ? "resident" : "per-colour", I.nlaunch, t_ms[0], t_ms[1] - t_ms[0], t_ms[2] - t_ms[1],
                t_ms[3] - t_ms[2], t_ms[4] - t_ms[3]);
    }
    return 0;
}

int LargeWorld::seed_warm(const unsigned long long* keys, const float4* vals, const float4* cvals, uint32_t hs,
                          cudaStream_t st, std::string* msg) {
    Impl& I = *impl;
    LTRY(regrow(I.wcap[0], hs, {LB(I.wkeys[0]), LB(I.wvals[0]), LB(I.wcvals[0])}));
    lk_warm_clear<<<blocks(hs), LT, 0, st>>>(I.wkeys[0], hs);
    lk_warm_copy<<<blocks(hs), LT, 0, st>>>(keys, vals, cvals, hs, I.wkeys[0], I.wvals[0], I.wcvals[0], hs);
    LTRY(cudaStreamSynchronize(st));
    I.whs[0] = hs;
    I.whs[1] = 0;
    I.wcur = 0;
    return 0;
}

int LargeWorld::read_warm(std::vector<unsigned long long>* keys, std::vector<float4>* vals,
                          std::vector<float4>* cvals, cudaStream_t st, std::string* msg) {
    Impl& I = *impl;
    const uint32_t hs = I.whs[I.wcur];
    keys->assign(hs, ~0ull);
    vals->assign(hs, make_float4(0.f, 0.f, 0.f, 0.f));
    cvals->assign(hs, make_float4(0.f, 0.f, 0.f, 0.f));
    if (hs == 0) return 0;
    LTRY(cudaStreamSynchronize(st));
    LTRY(cudaMemcpy(keys->data(), I.wkeys[I.wcur], 8ull * hs, cudaMemcpyDeviceToHost));
    LTRY(cudaMemcpy(vals->data(), I.wvals[I.wcur], 16ull * hs, cudaMemcpyDeviceToHost));
    if (I.wcvals[I.wcur]) LTRY(cudaMemcpy(cvals->data(), I.wcvals[I.wcur], 16ull * hs, cudaMemcpyDeviceToHost));
    return 0;
}

uint32_t LargeWorld::num_manifolds() const { return impl->nman; }
uint32_t LargeWorld::launches() const { return impl->nlaunch; }

int LargeWorld::dump(uint32_t cap, uint32_t* keys, float* data, uint32_t* colours, cudaStream_t st,
                     std::string* msg) {
    Impl& I = *impl;
    const uint32_t m = std::min(cap, I.nman);
    if (m == 0) return 0;
    LTRY(regrow(I.cap_d, 2 * (size_t)m, {LB(I.dk), LB(I.dc)}));
    LTRY(regrow(I.cap_dd, (size_t)DEBUG_MF * m, {LB(I.dd)}));
    SWT<uint32_t> s{};
    s.ma = I.ma; s.mb = I.mb; s.mp0 = I.mp0; s.mnp = I.mnp; s.mcol = I.mcol;
    s.nx = I.nx; s.ny = I.ny; s.fric = I.fric; s.ang_prev = I.ang_prev;
    s.r1x = I.r1x; s.r1y = I.r1y; s.r2x = I.r2x; s.r2y = I.r2y;
    s.depth = I.depth; s.odepth = I.odepth; s.mn = I.mn; s.mt = I.mt; s.apn = I.apn; s.apt = I.apt;
    lk_dump<<<blocks(m), LT, 0, st>>>(s, m, I.dk, I.dd, I.dc);
    LTRY(cudaStreamSynchronize(st));
    if (keys) LTRY(cudaMemcpy(keys, I.dk, 8ull * m, cudaMemcpyDeviceToHost));
    if (data) LTRY(cudaMemcpy(data, I.dd, sizeof(float) * DEBUG_MF * (size_t)m, cudaMemcpyDeviceToHost));
    if (colours) LTRY(cudaMemcpy(colours, I.dc, 4ull * m, cudaMemcpyDeviceToHost));
    return 0;
}

uint32_t LargeWorld::num_pairs() const { return impl->npairs; }

// the 64-bit (lower << 32 | higher) pair keys as two 32-bit indices each
__global__ void lk_split_pairs(const unsigned long long* keys, uint32_t n, uint32_t* out) {
    const uint32_t i = blockIdx.x * LT + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    out[2 * i] = (uint32_t)(k >> 32);
    out[2 * i + 1] = (uint32_t)k;
}

int LargeWorld::dump_pairs(uint32_t cap, uint32_t* pairs, cudaStream_t st, std::string* msg) {
    Impl& I = *impl;
    const uint32_t m = std::min(cap, I.npairs);
    if (m == 0) return 0;
    LTRY(regrow(I.cap_d, 2 * (size_t)m, {LB(I.dk), LB(I.dc)}));
    lk_split_pairs<<<blocks(m), LT, 0, st>>>(I.pairs, m, I.dk);
    LTRY(cudaStreamSynchronize(st));
    LTRY(cudaMemcpy(pairs, I.dk, 8ull * m, cudaMemcpyDeviceToHost));
    return 0;
}

int LargeWorld::joint_colours(uint32_t cap, uint32_t* colours, cudaStream_t st, std::string* msg) {
    Impl& I = *impl;
    const uint32_t m = std::min(cap, I.nj);
    if (m == 0) return 0;
    LTRY(regrow(I.cap_d, m, {LB(I.dk), LB(I.dc)}));
    lk_widen<<<blocks(m), LT, 0, st>>>(I.jcol, m, I.dc);
    LTRY(cudaStreamSynchronize(st));
    LTRY(cudaMemcpy(colours, I.dc, 4ull * m, cudaMemcpyDeviceToHost));
    return 0;
}


// ---------------------------------------------------------------------------
// The world step with no allocation (r2d_world_step_static).  Some callers
// cannot allocate device memory once they are running: a fixed-step physics
// tick inside a frame loop with a hard budget (cudaMalloc and cudaFree can
// synchronise the whole device and stall the frame), or an embedder whose
// own pool owns all device memory.  For them the same kernels run with their
// scratch carved from one file-scope device array instead of cudaMalloc'd
// buffers, and the host side keeps its counters on the stack.
// ---------------------------------------------------------------------------
namespace {

struct StaticCarve {
    size_t off = 0;
    template <class T>
    constexpr size_t take(size_t count) {
        const size_t at = off;
        off = (off + count * sizeof(T) + 255) / 256 * 256;
        return at;
    }
};

// Byte offsets of every scratch buffer for the static maxima; the same
// function sizes the array (at compile time) and hands out the pointers.
struct StaticLayout {
    size_t inv_m, inv_i, cs, sn, tq, ang_prev, kind, rx0, ry0, rx1, ry1, bcnt, adj, cursor;
    size_t table, ebucket, ebody, eslot, sbody, hset, pairs;
    size_t ma, mb, mp0, corder, mnp, mcol, nx, ny, fric;
    size_t r1x, r1y, r2x, r2y, depth, odepth, mn, mt, apn, apt, bias;
    size_t adjl, prio, jcol, jorder, cnt, entries, hist;
    size_t ma2, mb2, mp02, mnp2, mcol2, nx2, ny2, r1x2, r1y2, r2x2, r2y2, depth2, odepth2, apn2, apt2;
    size_t pk[7], mom4;
    size_t total;
};

constexpr uint32_t SX_BODIES = R2D_STATIC_MAX_BODIES;
constexpr uint32_t SX_BUCKETS = 2 * R2D_STATIC_MAX_BODIES;
constexpr uint32_t SX_ENTRIES = R2D_STATIC_MAX_CELL_ENTRIES;
constexpr uint32_t SX_PAIRS = R2D_STATIC_MAX_PAIRS;
constexpr uint32_t SX_HASH = 2 * R2D_STATIC_MAX_PAIRS;  // power of two, >= 1.5x the pairs

constexpr StaticLayout static_layout() {
    StaticLayout L{};
    StaticCarve c;
    const size_t nb = SX_BODIES + 1, np = SX_PAIRS + 1, npt = 2 * (size_t)SX_PAIRS + 1;
    L.inv_m = c.take<float>(nb); L.inv_i = c.take<float>(nb); L.cs = c.take<float>(nb); L.sn = c.take<float>(nb);
    L.tq = c.take<float>(nb); L.ang_prev = c.take<float>(nb); L.kind = c.take<uint8_t>(nb);
    L.rx0 = c.take<int32_t>(nb); L.ry0 = c.take<int32_t>(nb); L.rx1 = c.take<int32_t>(nb); L.ry1 = c.take<int32_t>(nb);
    L.bcnt = c.take<uint32_t>(nb); L.adj = c.take<uint32_t>(nb); L.cursor = c.take<uint32_t>(nb);
    L.table = c.take<uint32_t>(SX_BUCKETS + 1);
    L.ebucket = c.take<uint32_t>(SX_ENTRIES + 1); L.ebody = c.take<uint32_t>(SX_ENTRIES + 1);
    L.eslot = c.take<uint32_t>(SX_ENTRIES + 1); L.sbody = c.take<uint32_t>(SX_ENTRIES + 1);
    L.hset = c.take<unsigned long long>(SX_HASH); L.pairs = c.take<unsigned long long>(SX_PAIRS);
    L.ma = c.take<uint32_t>(np); L.mb = c.take<uint32_t>(np); L.mp0 = c.take<uint32_t>(np);
    L.corder = c.take<uint32_t>(np); L.mnp = c.take<uint8_t>(np); L.mcol = c.take<uint8_t>(np);
    L.nx = c.take<float>(np); L.ny = c.take<float>(np); L.fric = c.take<float>(np);
    L.r1x = c.take<float>(npt); L.r1y = c.take<float>(npt); L.r2x = c.take<float>(npt); L.r2y = c.take<float>(npt);
    L.depth = c.take<float>(npt); L.odepth = c.take<float>(npt); L.mn = c.take<float>(npt); L.mt = c.take<float>(npt);
    L.apn = c.take<float>(npt); L.apt = c.take<float>(npt); L.bias = c.take<float>(npt);
    L.adjl = c.take<uint32_t>(2 * (size_t)SX_PAIRS + 2); L.prio = c.take<uint32_t>(2 * (size_t)SX_PAIRS + 2);
    L.jcol = c.take<uint8_t>(1); L.jorder = c.take<uint32_t>(1);
    L.cnt = c.take<uint32_t>(LC_N); L.entries = c.take<unsigned long long>(1);
    L.hist = c.take<uint32_t>(CB_WORDS);
    L.ma2 = c.take<uint32_t>(np); L.mb2 = c.take<uint32_t>(np); L.mp02 = c.take<uint32_t>(np);
    L.mnp2 = c.take<uint8_t>(np); L.mcol2 = c.take<uint8_t>(np); L.nx2 = c.take<float>(np); L.ny2 = c.take<float>(np);
    L.r1x2 = c.take<float>(npt); L.r1y2 = c.take<float>(npt); L.r2x2 = c.take<float>(npt);
    L.r2y2 = c.take<float>(npt); L.depth2 = c.take<float>(npt); L.odepth2 = c.take<float>(npt);
    L.apn2 = c.take<float>(npt); L.apt2 = c.take<float>(npt);
    for (int k = 0; k < 7; ++k) L.pk[k] = c.take<float4>(np);
    L.mom4 = c.take<float4>(nb);
    L.total = c.off;
    return L;
}

constexpr StaticLayout SL = static_layout();
static_assert(SL.total == R2D_STATIC_SCRATCH_BYTES, "R2D_STATIC_SCRATCH_BYTES must equal the carved layout");

// The scratch of every allocation-free call on this device.  Each GPU that
// loads the library holds these R2D_STATIC_SCRATCH_BYTES until the process
// exits.  In host code the name stands for the symbol, not an address: the
// address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_static_scratch[R2D_STATIC_SCRATCH_BYTES];

constexpr int STATIC_MAX_DEVICES = 64;
std::atomic<unsigned char*> g_static_ptr[STATIC_MAX_DEVICES];

}  // namespace

int static_scratch_address(unsigned char** out, std::string* msg) {
    int dev = 0;
    LTRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= STATIC_MAX_DEVICES) {
        *msg = "device index beyond " + std::to_string(STATIC_MAX_DEVICES);
        return -1;
    }
    unsigned char* p = g_static_ptr[dev].load();
    if (!p) {
        // set-up, once per device, with that device current
        void* sym = nullptr;
        LTRY(cudaGetSymbolAddress(&sym, g_static_scratch));
        p = static_cast<unsigned char*>(sym);
        g_static_ptr[dev].store(p);
    }
    *out = p;
    return 0;
}

#undef LAUNCH
#undef SCAN
#define LAUNCH(kernel, grid, ...) kernel<<<(grid), LT, 0, st>>>(__VA_ARGS__)
#define SCAN(a, n) lk_scan<<<1, SCAN_THREADS, 0, st>>>((a), (n))

int static_world_step(const StaticStepArgs& in, cudaStream_t st, std::string* msg) {
    const uint32_t n = in.n;
    if (n == 0) return 0;
    if (n > SX_BODIES) {
        *msg = std::to_string(n) + " bodies exceed the static-scratch maximum of " + std::to_string(SX_BODIES);
        return DS_CAPACITY;
    }
    // table_mult x n in 64 bits: a product that wraps 32 bits must not pass the check
    const unsigned long long T64 = (unsigned long long)in.table_mult * n;
    if (T64 == 0 || T64 > SX_BUCKETS) {
        *msg = "spatial-hash table of " + std::to_string(T64) + " buckets exceeds the static-scratch maximum of " +
               std::to_string(SX_BUCKETS);
        return DS_CAPACITY;
    }
    const uint32_t T = (uint32_t)T64;
    unsigned char* base = nullptr;
    if (int r = static_scratch_address(&base, msg)) return r;
#define SP(T_, field) reinterpret_cast<T_*>(base + SL.field)
    uint32_t* cnt = SP(uint32_t, cnt);
    unsigned long long* entries = SP(unsigned long long, entries);
    uint32_t* hist = SP(uint32_t, hist);
    uint32_t h[LC_N + 2];  // counters read back to the host (host stack, no allocation)

    SWT<uint32_t> s{};
    float* S = in.state;
    s.px = S + (size_t)S_POS_X * n; s.py = S + (size_t)S_POS_Y * n; s.ang = S + (size_t)S_ANGLE * n;
    s.mx = S + (size_t)S_MOM_X * n; s.my = S + (size_t)S_MOM_Y * n; s.L = S + (size_t)S_ANG_MOM * n;
    s.inv_m = SP(float, inv_m); s.inv_i = SP(float, inv_i); s.cs = SP(float, cs); s.sn = SP(float, sn);
    s.ang_prev = SP(float, ang_prev); s.tq = SP(float, tq);
    s.px0 = nullptr; s.py0 = nullptr; s.pos0 = false;
    s.gmass = in.props + (size_t)P_MASS * n;
    s.ginertia = in.props + (size_t)P_INERTIA * n;
    s.kind = SP(uint8_t, kind);
    s.ma = SP(uint32_t, ma); s.mb = SP(uint32_t, mb); s.mp0 = SP(uint32_t, mp0);
    s.mnp = SP(uint8_t, mnp); s.mcol = SP(uint8_t, mcol);
    s.nx = SP(float, nx); s.ny = SP(float, ny); s.fric = SP(float, fric);
    s.r1x = SP(float, r1x); s.r1y = SP(float, r1y); s.r2x = SP(float, r2x); s.r2y = SP(float, r2y);
    s.depth = SP(float, depth); s.odepth = SP(float, odepth); s.mn = SP(float, mn); s.mt = SP(float, mt);
    s.apn = SP(float, apn); s.apt = SP(float, apt); s.bias = SP(float, bias);

    Phase1 A{};
    A.s = s;
    A.state = in.state; A.props = in.props; A.kind_in = in.kind; A.ids = in.ids;
    A.NB = n; A.base = 0; A.n = n; A.cell = in.cell;
    A.bmod = BucketMod{bucket_recip(T), T};
    A.disc_rot = false;
    A.rx0 = SP(int32_t, rx0); A.ry0 = SP(int32_t, ry0); A.rx1 = SP(int32_t, rx1); A.ry1 = SP(int32_t, ry1);
    A.bcnt = SP(uint32_t, bcnt); A.table = SP(uint32_t, table);
    A.ebucket = SP(uint32_t, ebucket); A.ebody = SP(uint32_t, ebody); A.eslot = SP(uint32_t, eslot);
    A.sbody = SP(uint32_t, sbody);
    A.hset = SP(unsigned long long, hset); A.pairs = SP(unsigned long long, pairs);
    A.np = SX_PAIRS; A.hs = SX_HASH;
    A.excl = nullptr; A.nexcl = 0;
    A.cnt = cnt; A.entries = entries;

    // The array keeps the previous call's contents: clear what starts at zero.
    LTRY(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * LC_N, st));
    LTRY(cudaMemsetAsync(entries, 0, sizeof(unsigned long long), st));
    LTRY(cudaMemsetAsync(A.table, 0, sizeof(uint32_t) * ((size_t)T + 1), st));
    LTRY(cudaMemsetAsync(A.hset, 0xFF, sizeof(unsigned long long) * SX_HASH, st));
    LAUNCH(lk_load, blocks(n), A);
    LTRY(cudaMemcpyAsync(h, cnt, sizeof(uint32_t) * LC_N, cudaMemcpyDeviceToHost, st));
    LTRY(cudaMemcpyAsync(h + LC_N, entries, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    LTRY(cudaStreamSynchronize(st));
    if (h[LC_NONFINITE]) {
        *msg = "a body's AABB is not finite (it has no spatial-hash cell)";
        return DS_NONFINITE;
    }
    if (h[LC_NOPOLY]) {
        *msg = "a polygon body (R2D_KIND_POLYGON): this step takes discs and rectangles only";
        return -1;  // R2D_ERR_INVALID_ARGUMENT
    }
    unsigned long long E64 = 0;
    memcpy(&E64, h + LC_N, sizeof(E64));
    if (h[LC_BIG] || E64 > SX_ENTRIES) {
        *msg = "the bodies cover more than the static-scratch maximum of " + std::to_string(SX_ENTRIES) +
               " spatial-hash cell entries";
        return DS_CAPACITY;
    }
    const uint32_t E = (uint32_t)E64;
    SCAN(A.bcnt, n);
    LAUNCH(lk_emit, blocks(E), A, E);
    SCAN(A.table, T);
    LAUNCH(lk_scatter, blocks(E), A, E);
    LAUNCH(lk_pairs, blocks((uint64_t)PAIR_GROUP * E), A, E);
    LTRY(cudaMemcpyAsync(h, cnt, sizeof(uint32_t) * LC_N, cudaMemcpyDeviceToHost, st));
    LTRY(cudaStreamSynchronize(st));
    if (h[LC_PAIR_OVERFLOW]) {
        *msg = "more candidate pairs than the static-scratch maximum of " + std::to_string(SX_PAIRS);
        return DS_CAPACITY;
    }
    const uint32_t npairs = h[LC_PAIRS];
    A.nm = npairs;
    A.npt = 2 * npairs;
    LTRY(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * LC_N, st));
    LAUNCH(lk_narrow, blocks(npairs), A, npairs);
    LTRY(cudaMemcpyAsync(h, cnt, sizeof(uint32_t) * LC_N, cudaMemcpyDeviceToHost, st));
    LTRY(cudaStreamSynchronize(st));
    const uint32_t M = h[LC_MANIFOLDS];

    // contact colouring (Jones-Plassmann rounds, queued STATIC_ROUNDS at a
    // time), the colour-major permutation, then the substeps in one resident
    // cluster
    int cl_solve = 0, cl_colour = 0;
    LTRY(resident_cluster(0, lk_substeps_resident, RT, &cl_solve));
    LTRY(resident_cluster(1, lk_colour_cluster, CT, &cl_colour));
    uint32_t ncol = 0;
    if (M) {
        Colouring C{};
        C.count = M;
        C.joints = false;
        C.ma = s.ma; C.mb = s.mb; C.kind = s.kind; C.colour = s.mcol;
        C.adj = SP(uint32_t, adj); C.adjl = SP(uint32_t, adjl); C.prio = SP(uint32_t, prio);
        C.cursor = SP(uint32_t, cursor); C.cnt = cnt;
        LTRY(cudaMemsetAsync(C.adj, 0, sizeof(uint32_t) * ((size_t)n + 1), st));
        LTRY(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * LC_N, st));
        LAUNCH(lk_col_count, blocks(M), C);
        SCAN(C.adj, n);
        LTRY(cudaMemcpyAsync(C.cursor, C.adj, sizeof(uint32_t) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
        LAUNCH(lk_col_fill, blocks(M), C);
        LTRY(launch_resident(lk_colour_cluster, cl_colour, CT, st, C));
        LTRY(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * CB_WORDS, st));
        LAUNCH(lk_col_hist, blocks(M), C, hist);
        lk_col_offsets<<<1, 32, 0, st>>>(hist);
        LAUNCH(lk_col_order, blocks(M), C, hist, SP(uint32_t, corder));
        LTRY(cudaMemcpyAsync(h, cnt, sizeof(uint32_t) * LC_N, cudaMemcpyDeviceToHost, st));
        LTRY(cudaMemcpyAsync(h + LC_N, hist + CB_NCOL, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        // manifolds in colour-major order (into the second copies, which the substeps then use)
        SWT<uint32_t> d = s;
        d.ma = SP(uint32_t, ma2); d.mb = SP(uint32_t, mb2); d.mp0 = SP(uint32_t, mp02); d.mnp = SP(uint8_t, mnp2);
        d.mcol = SP(uint8_t, mcol2); d.nx = SP(float, nx2); d.ny = SP(float, ny2);
        d.r1x = SP(float, r1x2); d.r1y = SP(float, r1y2); d.r2x = SP(float, r2x2); d.r2y = SP(float, r2y2);
        d.depth = SP(float, depth2); d.odepth = SP(float, odepth2); d.apn = SP(float, apn2); d.apt = SP(float, apt2);
        LAUNCH(lk_permute, blocks(M), s, d, SP(uint32_t, corder), M);
        s = d;
        LTRY(cudaStreamSynchronize(st));
        if (h[LC_COLOURS]) {
            *msg = "a contact needs more than " + std::to_string(MAX_COLOURS) + " colours";
            return DS_CAPACITY;
        }
        if (h[LC_STUCK]) {
            *msg = "the colouring did not finish within its round limit";
            return DS_TIMEOUT;
        }
        ncol = h[LC_N];
    }

    // substeps: the caller's state changes from here on
    Phase2 P{};
    P.s = s;
    P.state = in.state; P.props = in.props; P.NB = n; P.base = 0; P.n = n; P.nman = M;
    P.h = in.dt / (float)in.sub_steps;
    P.disc_rot = false;
    P.ngrav = in.ngrav;
    for (int k = 0; k < MAX_GRAVITY; ++k) P.g[k] = in.g[k];
    P.pk = Packed{reinterpret_cast<float4*>(base + SL.pk[0]), reinterpret_cast<float4*>(base + SL.pk[1]),
                  reinterpret_cast<float4*>(base + SL.pk[2]), reinterpret_cast<float4*>(base + SL.pk[3]),
                  reinterpret_cast<float4*>(base + SL.pk[4]), reinterpret_cast<float4*>(base + SL.pk[5]),
                  reinterpret_cast<float4*>(base + SL.pk[6]), SP(float4, mom4)};
    ResidentPlan R{};
    R.coff = hist + CB_OFF; R.joff = nullptr;
    R.ncol = ncol; R.njcol = 0;
    R.sub_steps = in.sub_steps; R.iters = in.iters;
    LTRY(launch_resident(lk_substeps_resident, cl_solve, RT, st, P, R));
#undef SP
    LTRY(cudaGetLastError());
    return 0;
}

}  // namespace r2d
