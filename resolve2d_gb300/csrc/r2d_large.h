/*
 * r2d_large.h -- host interface of the large-world step (r2d_large.cu): one
 * world whose bodies do not fit one CTA's shared memory, stepped by a
 * pipeline of grid-wide kernels over global scratch buffers.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "r2d_world.cuh"

namespace r2d {

// Device views of one world inside an engine's field-major arrays.
struct LargeInputs {
    float* state;          // [S_NFIELDS][NB]
    const float* props;    // [P_NFIELDS][NB]
    const uint8_t* kind;   // [NB]
    const uint32_t* ids;   // [NB]
    uint32_t NB;           // bodies of the whole engine (field stride)
    uint32_t base, n;      // this world's first body and body count
    const uint8_t* jtype;  // this world's joints (world-local body indices)
    const uint32_t* jb1;
    const uint32_t* jb2;
    const float* jprm;     // [nj][JOINT_PARAMS]
    uint32_t nj;
    uint64_t joint_epoch;  // changes whenever the joint arrays change; 0 = unknown (recolour every step)
    const unsigned long long* excl;  // sorted (lo << 32 | hi) keys of this world
    uint32_t nexcl;
    uint32_t ngrav;
    float g[MAX_GRAVITY];
    float cell;
    uint32_t table_mult;
    bool disc_rot;         // some joint reads disc orientations
    double* pos64;         // [3][NB] f64 pose (FP64-positions mode), else null
    bool warm;             // warm starting (the world keeps its impulses across calls)
    bool comp;             // compensated accumulation of the impulses (r2d_accum.h)
    bool verbose;          // print each step's phase times and counts to stderr
    uint32_t* sleep;       // this world's still-frame counter (sleeping mode, r2d_sleep.h), else null
    uint32_t colour_round_limit;  // colouring rounds before R2D_ERR_TIMEOUT (0 = never reached)
    const float2* poly_v;  // [NB][MAX_POLY_VERTS] local vertices of the engine's polygons, else null
    const uint8_t* poly_nv;  // [NB] their vertex counts
};

class LargeWorld {
public:
    LargeWorld();
    ~LargeWorld();
    LargeWorld(const LargeWorld&) = delete;
    LargeWorld& operator=(const LargeWorld&) = delete;

    // One Solver.process call.  Returns 0 or a negative r2d status (with
    // *msg set); on an error the world's state is that before the call.
    int step(const LargeInputs& in, float dt, uint32_t sub_steps, uint32_t iters, cudaStream_t st, std::string* msg);
    // Manifolds and colourings of the last step (debug taps, oracle layout).
    uint32_t num_manifolds() const;
    int dump(uint32_t cap, uint32_t* keys, float* data, uint32_t* colours, cudaStream_t st, std::string* msg);
    int joint_colours(uint32_t cap, uint32_t* colours, cudaStream_t st, std::string* msg);
    // Candidate pairs of the last step (debug tap): (lower, higher) world-local
    // indices [min(cap, count)][2], in no particular order.
    uint32_t num_pairs() const;
    int dump_pairs(uint32_t cap, uint32_t* pairs, cudaStream_t st, std::string* msg);
    // Kernel launches of the last step.
    uint32_t launches() const;
    // Warm starting: take over another table of last frame's impulses
    // (keys / values / compensation words (may be null) of `hs` slots in
    // device memory, the fused kernel's layout) when a world moves to this
    // path or its body store is replaced.
    int seed_warm(const unsigned long long* keys, const float4* vals, const float4* cvals, uint32_t hs,
                  cudaStream_t st, std::string* msg);
    // This path's last-frame table, copied to the host: keys, values and
    // compensation words (zeros when none are kept), `hs` slots.
    int read_warm(std::vector<unsigned long long>* keys, std::vector<float4>* vals, std::vector<float4>* cvals,
                  cudaStream_t st, std::string* msg);

    struct Impl;

private:
    Impl* impl;
};

// Allocation-free world step (r2d_world_step_static): maxima of the static
// scratch array and the inputs of one call.
#define R2D_STATIC_MAX_BODIES 4096u
#define R2D_STATIC_MAX_CELL_ENTRIES 65536u
#define R2D_STATIC_MAX_PAIRS 16384u
#define R2D_STATIC_SCRATCH_BYTES 7216128ull  // 6.88 MiB

struct StaticStepArgs {
    float* state;          // [S_NFIELDS][n], device
    const float* props;    // [P_NFIELDS][n], device
    const uint8_t* kind;   // [n], device
    const uint32_t* ids;   // [n], device
    uint32_t n;
    uint32_t ngrav;
    float g[MAX_GRAVITY];
    float dt;
    uint32_t sub_steps, iters;
    float cell;
    uint32_t table_mult;
};

int static_world_step(const StaticStepArgs& in, cudaStream_t st, std::string* msg);

}  // namespace r2d
