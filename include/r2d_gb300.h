/*
 * r2d_gb300.h -- C ABI of the GB300 step library (libr2d_gb300.so).
 *
 * It replaces the CPU step of nilsblix/resolve2d, Solver.process
 * (src/core/lib.zig:189-251), behind plain pointers and sizes so that the
 * reference's own host language can bind it directly (one Zig `extern fn`
 * per entry point).  Reference paths below are relative to the reference
 * project.
 *
 * Conventions
 *   - Every entry point returns an r2d_status (0 = success, negative = error).
 *     Errors never abort; the reference's error unions map onto them:
 *     error.InvalidRigidBodyId -> R2D_ERR_INVALID_BODY_ID,
 *     error.OutOfMemory        -> R2D_ERR_OUT_OF_MEMORY.
 *   - Host buffers are caller-owned; the library owns all device memory.
 *   - Per-body arrays are field-major: field f of body i is at [f * n + i].
 *   - Body ids are u32 (the reference's RigidBody.Id is u16,
 *     src/core/Bodies/RigidBody.zig:15; u32 lets one world hold more bodies).
 *   - One handle per host thread; calls on one handle are not reentrant.
 *   - `stream` in r2d_config is a cudaStream_t (NULL = a stream the library
 *     creates).  r2d_*_process only enqueues work; r2d_*_sync waits for it
 *     and returns the first device-side error.
 */
#ifndef R2D_GB300_H
#define R2D_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define R2D_API __attribute__((visibility("default")))
#else
#define R2D_API
#endif

typedef enum r2d_status {
    R2D_OK = 0,
    R2D_ERR_INVALID_ARGUMENT = -1,
    R2D_ERR_INVALID_BODY_ID = -2, /* error.InvalidRigidBodyId (src/core/Constraints/DistanceJoint.zig:44-47) */
    R2D_ERR_OUT_OF_MEMORY = -3,   /* error.OutOfMemory */
    R2D_ERR_CUDA = -4,            /* a CUDA runtime call failed (see r2d_last_error_string) */
    R2D_ERR_CAPACITY = -5,        /* a hard limit: more than 128 colours, or more than 64Mi spatial-hash cells */
    R2D_ERR_TIMEOUT = -6,         /* a bounded device-side wait gave up */
    R2D_ERR_NONFINITE = -7,       /* an AABB coordinate is not a representable spatial-hash cell */
    R2D_ERR_NO_DEVICE = -8        /* no CUDA device is visible */
} r2d_status;

/* Per-body state, f32 field-major [R2D_STATE_FIELDS][n]
 * (RigidBody.Props, src/core/Bodies/RigidBody.zig:69-81, plus the body's
 * stored AABB, RigidBody.zig:84, which the next frame's broadphase reads). */
enum {
    R2D_S_POS_X = 0, R2D_S_POS_Y, R2D_S_ANGLE,
    R2D_S_MOM_X, R2D_S_MOM_Y, R2D_S_ANG_MOM,
    R2D_S_FORCE_X, R2D_S_FORCE_Y, R2D_S_TORQUE,
    R2D_S_AABB_X, R2D_S_AABB_Y, R2D_S_AABB_HW, R2D_S_AABB_HH,
    R2D_STATE_FIELDS
};

/* Per-body constant properties, f32 field-major [R2D_PROP_FIELDS][n]:
 * mass, inertia, mu, then radius (disc) or width, height (rectangle)
 * (Disc.zig:8, Rectangle.zig:17-18). */
enum { R2D_P_MASS = 0, R2D_P_INERTIA, R2D_P_MU, R2D_P_DIM0, R2D_P_DIM1, R2D_PROP_FIELDS };

/* kind bits per body: RigidBody.Type (RigidBody.zig:28-31) and the static flag (:85).
 * R2D_KIND_POLYGON: a convex polygon, the roadmap's next shape (README.md:64-67)
 * behind the same vtable (RigidBody.zig:33-42); its vertices come with
 * r2d_*_set_polygons, its props are mass, inertia, mu and two free dims. */
enum { R2D_KIND_RECTANGLE = 1, R2D_KIND_STATIC = 2, R2D_KIND_POLYGON = 4 };
/* Vertices a polygon may have (3 .. R2D_POLY_MAX_VERTS). */
enum { R2D_POLY_MAX_VERTS = 8 };

/* Constraint.Type (src/core/Constraints/Constraint.zig:15-20) */
enum {
    R2D_JOINT_DISTANCE = 0,
    R2D_JOINT_OFFSET_DISTANCE = 1,
    R2D_JOINT_FIXED_POSITION = 2,
    R2D_JOINT_MOTOR = 3
};

/* Joint parameters, f32 [n][R2D_JOINT_PARAMS]:
 *   [0] power_max [1] power_min [2] beta   (Constraint.Parameters, Constraint.zig:27-31)
 *   distance:        [3] target_distance
 *   offset distance: [3] r1.x [4] r1.y [5] r2.x [6] r2.y [7] target_distance
 *   fixed position:  [3] target.x [4] target.y
 *   motor:           [3] target_omega */
enum { R2D_JOINT_PARAMS = 8 };

/* Floats per manifold in r2d_*_get_manifolds:
 *   [0..1] normal [2..3] tangent [4] friction [5] has point 0 [6] has point 1
 *   [7] prev_angle_1 [8] prev_angle_2, then per point (12 floats, points 0 and 1):
 *   pos.x pos.y (NaN: not kept on the device) ref_r.x ref_r.y inc_r.x inc_r.y
 *   depth original_depth mass_n mass_t accumulated_pn accumulated_pt
 *   (CollisionManifold / CollisionPoint, src/core/collision.zig:22-69). */
enum { R2D_MANIFOLD_FLOATS = 33 };

enum {
    R2D_FLAG_DEBUG_TAPS = 1u, /* keep manifolds, colours and candidate pairs for r2d_*_get_manifolds / _get_pairs */
    /* Step every world through the grid-wide pipeline that worlds above 520
     * bodies always use (global scratch, one kernel per phase and colour)
     * instead of the fused one-CTA-per-world kernel.  Same results. */
    R2D_FLAG_GRID_PIPELINE = 2u,
    /* Keep each body's x, y and angle in f64 as well and integrate them in
     * f64 (x += p * (h / m), angle += L * h / I); the f32 pose the step uses
     * is that pose rounded.  Momenta, contacts and joints stay f32.  No
     * counterpart in the reference, which is f32 throughout; it reduces
     * drift over long horizons (r2d_*_read_positions_f64 reads the pose). */
    R2D_FLAG_FP64_POSITIONS = 4u,
    /* Warm starting (no counterpart in the reference, whose manifolds are
     * cleared every frame, src/core/lib.zig:261; its roadmap asks for it,
     * README.md:60-61): a manifold whose (reference, incident) pair of body
     * ids had one last frame starts from last frame's accumulated impulses,
     * applied to the bodies after the first substep's preStep; and since
     * such a sum must be able to shrink, impulses below the reference's
     * 1e-4 skip threshold are applied (clamped at zero) instead of skipped.
     * The impulses are keyed by the stable body ids, so they survive
     * r2d_*_set_bodies / set_worlds: pairs whose two ids are still in the
     * world (world w of a batch keeps world w's) start warm. */
    R2D_FLAG_WARM_START = 8u,
    /* Sleeping (no counterpart in the reference; its roadmap lists it,
     * README.md:64-67): a world whose every non-static body ends 60
     * consecutive steps slower than 0.01 units/s and 0.01 rad/s is not
     * stepped again until the host writes to the engine (state, fields,
     * bodies, gravity, joints or exclusions), which wakes every world.
     * r2d_*_sleep_frames reads the per-world counters. */
    R2D_FLAG_SLEEP = 16u,
    /* Compensated (Kahan) accumulation of each contact point's normal and
     * tangent impulse sums (no counterpart in the reference, which adds them
     * in plain f32, src/core/collision.zig:182-190): the rounding remainder of
     * every addition is kept in a second word and carried into later ones;
     * the bodies receive the changes of the rounded sum, as in the reference.
     * With R2D_FLAG_WARM_START the remainders travel with the sums from
     * frame to frame. */
    R2D_FLAG_COMPENSATED = 32u
};

typedef struct r2d_config {
    /* Spatial hash cell width and bucket-table multiplier.  The reference
     * hard-codes 4.0 and 2 * bodies (src/core/lib.zig:254-255) and ignores
     * Solver.init's arguments (lib.zig:145); 0 selects those values. */
    float spatialhash_cell_width;
    uint32_t spatialhash_table_size_mult;
    uint32_t flags;
    void* stream;
    /* Scales the per-world buffer sizes of the fused kernel (0 = 1.0).  A
     * world that outgrows a buffer is replayed with larger sizes, so this
     * trades shared memory against replays; it never changes results. */
    float capacity_scale;
} r2d_config;

/* ---------------------------------------------------------------------------
 * One world: the drop-in for Solver (src/core/lib.zig:132-315) and the WASM
 * exports solverInit / solverDeinit / solverProcess (src/wasm_root.zig:18-43).
 * ------------------------------------------------------------------------- */
typedef struct r2d_solver r2d_solver;

/* Solver.init (lib.zig:145-157) / solverInit (wasm_root.zig:18-30) */
R2D_API int r2d_solver_create(const r2d_config* cfg, r2d_solver** out);
/* Solver.deinit (lib.zig:159-179) / solverDeinit (wasm_root.zig:32-37) */
R2D_API int r2d_solver_destroy(r2d_solver* s);

/* Replaces the body store (Solver.bodies, lib.zig:135) in its iteration
 * order.  props [R2D_PROP_FIELDS][n], state [R2D_STATE_FIELDS][n].  With
 * init_aabb != 0 every AABB is computed as RigidBody.updateAABB does when a
 * body is created (Disc.zig:63-66, Rectangle.zig:71-86) and the AABB fields
 * of `state` are ignored.  Ids are unique (the store is a map keyed by id):
 * two bodies with one id return R2D_ERR_INVALID_ARGUMENT. */
R2D_API int r2d_solver_set_bodies(r2d_solver* s, uint32_t n, const uint32_t* ids, const uint8_t* kind,
                                  const float* props, const float* state, int init_aabb);
/* The vertices of the store's R2D_KIND_POLYGON bodies (after set_bodies):
 * for each of n bodies (store indices `body`), nverts[k] (3..8) local
 * vertices about the body's origin, verts [n][R2D_POLY_MAX_VERTS][2],
 * clockwise as the rectangle's (Rectangle.zig:40), convex.  A body uploaded
 * with init_aabb gets its first AABB here.  A world holding a polygon steps
 * on the grid pipeline.  No counterpart in the reference (polygons are on
 * its roadmap, README.md:64-67). */
R2D_API int r2d_solver_set_polygons(r2d_solver* s, uint32_t n, const uint32_t* body, const uint8_t* nverts,
                                    const float* verts);
/* Per-frame mirror of the dynamic state (host -> device, device -> host). */
R2D_API int r2d_solver_write_state(r2d_solver* s, const float* state);
R2D_API int r2d_solver_read_state(r2d_solver* s, float* state);
/* Solver.force_generators (lib.zig:136): one DownwardsGravity per entry
 * (src/core/Forces/DownwardsGravity.zig:19-39), at most 4. */
R2D_API int r2d_solver_set_gravity(r2d_solver* s, uint32_t n, const float* g);
/* Solver.constraints (lib.zig:139), EntityFactory.make*Joint (lib.zig:100-122).
 * Ids refer to body ids; they are resolved at r2d_solver_process, which
 * returns R2D_ERR_INVALID_BODY_ID (state untouched) for an unknown id. */
R2D_API int r2d_solver_set_joints(r2d_solver* s, uint32_t n, const uint8_t* type, const uint32_t* id1,
                                  const uint32_t* id2, const float* params);
/* Solver.exclude_collision_pairs / EntityFactory.excludeCollisionPair
 * (lib.zig:124-129): pairs [n][2] of body ids. */
R2D_API int r2d_solver_set_exclusions(r2d_solver* s, uint32_t n, const uint32_t* pairs);
/* Solver.process (lib.zig:189-251) / solverProcess (wasm_root.zig:39-43). */
R2D_API int r2d_solver_process(r2d_solver* s, float dt, uint32_t sub_steps, uint32_t collision_iters);
R2D_API int r2d_solver_sync(r2d_solver* s);
/* One frame of a host loop in one call: the force and torque rows
 * `force_rows` [3][n] (state fields 6..8) are this frame's forces, the frame
 * is stepped, and the pose and momentum rows (fields 0..5) are written to
 * `out_rows` [6][n]; returns once they are there (with the status of
 * r2d_solver_sync).  Either pointer may be NULL.  Pinned (page-locked) or
 * managed buffers are read and written by the step itself over the coherent
 * CPU-GPU link; pageable ones are copied.  The bulk counterpart of the WASM
 * exports' per-field setters, solverProcess and getters
 * (src/wasm_root.zig:39-43,88-251). */
R2D_API int r2d_solver_process_io(r2d_solver* s, float dt, uint32_t sub_steps, uint32_t collision_iters,
                                  const float* force_rows, float* out_rows);
/* Bulk get/set of part of the state: rows [first, first + count) of the
 * field-major state (each row n floats), one contiguous copy.  The batched
 * form of the WASM exports' per-field body getters and setters
 * (src/wasm_root.zig:88-251), e.g. forces (R2D_S_FORCE_X, 3) in before a
 * step and pose and momenta (R2D_S_POS_X, 6) out after it.  Reading waits for
 * the step. */
R2D_API int r2d_solver_write_state_fields(r2d_solver* s, uint32_t first, uint32_t count, const float* rows);
R2D_API int r2d_solver_read_state_fields(r2d_solver* s, uint32_t first, uint32_t count, float* rows);
/* The f64 pose [3][n] (x, y, angle) kept under R2D_FLAG_FP64_POSITIONS;
 * writing the f32 state restarts it from that state.  No counterpart in the
 * reference. */
R2D_API int r2d_solver_read_positions_f64(r2d_solver* s, double* pose);
/* Consecutive still steps of the solver's world (R2D_FLAG_SLEEP); from 60 on
 * the world sleeps.  0 when sleeping is off. */
R2D_API int r2d_solver_sleep_frames(r2d_solver* s, uint32_t* frames);
/* Kernel launches of the solver's latest step (a world on the grid pipeline
 * launches per phase and per colouring; a fused world launches one kernel). */
R2D_API int r2d_solver_launches_per_step(r2d_solver* s, uint32_t* out);
/* Debug taps (need R2D_FLAG_DEBUG_TAPS): the last frame's manifolds
 * (Solver.manifolds, lib.zig:137) with their contact colours.  keys [cap][2]
 * are (reference, incident) body indices; data [cap][R2D_MANIFOLD_FLOATS]. */
R2D_API int r2d_solver_num_manifolds(r2d_solver* s, uint32_t* out);
R2D_API int r2d_solver_get_manifolds(r2d_solver* s, uint32_t cap, uint32_t* keys, float* data,
                                     uint32_t* colours);
/* Debug taps: the colour of each of the first `cap` joints, in insertion order,
 * from the last frame (the solve runs joint colours in ascending order). */
R2D_API int r2d_solver_get_joint_colours(r2d_solver* s, uint32_t cap, uint32_t* colours);
/* Debug taps: the last frame's candidate pairs, the pairs that reach SAT in
 * Solver.updateManifolds (src/core/lib.zig:264-282): two bodies sharing a
 * spatial-hash bucket, not both static, not excluded, AABBs intersecting.
 * pairs [cap][2] are (lower, higher) body indices in the store's order,
 * sorted ascending; each pair once. */
R2D_API int r2d_solver_num_pairs(r2d_solver* s, uint32_t* out);
R2D_API int r2d_solver_get_pairs(r2d_solver* s, uint32_t cap, uint32_t* pairs);

/* ---------------------------------------------------------------------------
 * Many independent worlds stepped by one launch per kernel class.  No
 * counterpart in the reference, which holds one global solver
 * (src/wasm_root.zig:15); each world behaves exactly like one r2d_solver.
 * ------------------------------------------------------------------------- */
typedef struct r2d_batch r2d_batch;

R2D_API int r2d_batch_create(const r2d_config* cfg, r2d_batch** out);
R2D_API int r2d_batch_destroy(r2d_batch* b);
/* Bodies of world w are [body_off[w], body_off[w+1]) of the concatenated
 * arrays (same layouts as r2d_solver_set_bodies); gravity [nworlds] is one
 * DownwardsGravity per world (0 = none).  Ids are unique within a world and
 * may repeat across worlds. */
R2D_API int r2d_batch_set_worlds(r2d_batch* b, uint32_t nworlds, const uint32_t* body_off, const uint32_t* ids,
                                 const uint8_t* kind, const float* props, const float* state,
                                 const float* gravity, int init_aabb);
/* r2d_solver_set_polygons for a batch: `body` indexes the concatenated bodies. */
R2D_API int r2d_batch_set_polygons(r2d_batch* b, uint32_t n, const uint32_t* body, const uint8_t* nverts,
                                   const float* verts);
R2D_API int r2d_batch_write_state(r2d_batch* b, const float* state);
R2D_API int r2d_batch_read_state(r2d_batch* b, float* state);
R2D_API int r2d_batch_process(r2d_batch* b, float dt, uint32_t sub_steps, uint32_t collision_iters);
R2D_API int r2d_batch_sync(r2d_batch* b);
/* r2d_solver_process_io over all worlds' bodies (rows of total-bodies length). */
R2D_API int r2d_batch_process_io(r2d_batch* b, float dt, uint32_t sub_steps, uint32_t collision_iters,
                                 const float* force_rows, float* out_rows);
/* Kernel launches one r2d_batch_process enqueues (one per occupied size class). */
R2D_API int r2d_batch_launches_per_step(r2d_batch* b, uint32_t* out);
/* Consecutive still steps of every world [nworlds] (R2D_FLAG_SLEEP; a world
 * sleeps from 60 on); zeros when sleeping is off. */
R2D_API int r2d_batch_sleep_frames(r2d_batch* b, uint32_t* frames);
/* Rows [first, first + count) of the state over all bodies (see the
 * solver's). */
R2D_API int r2d_batch_write_state_fields(r2d_batch* b, uint32_t first, uint32_t count, const float* rows);
R2D_API int r2d_batch_read_state_fields(r2d_batch* b, uint32_t first, uint32_t count, float* rows);
/* Autotuning (no counterpart in the reference): picks the threads per CTA of
 * each size class by timing `trial_steps` whole steps per candidate from the
 * current state, which is restored afterwards.  Results never depend on the
 * choice; it persists for later calls.  Takes a few hundred steps' time. */
R2D_API int r2d_batch_autotune(r2d_batch* b, float dt, uint32_t sub_steps, uint32_t collision_iters,
                               uint32_t trial_steps);
/* The f64 pose [3][total bodies] under R2D_FLAG_FP64_POSITIONS (see the
 * solver's). */
R2D_API int r2d_batch_read_positions_f64(r2d_batch* b, double* pose);
/* Per-world status of the last synced step (0 or an r2d_status). */
R2D_API int r2d_batch_world_status(r2d_batch* b, int* status);
/* Debug taps for world w (need R2D_FLAG_DEBUG_TAPS). */
R2D_API int r2d_batch_num_manifolds(r2d_batch* b, uint32_t w, uint32_t* out);
R2D_API int r2d_batch_get_manifolds(r2d_batch* b, uint32_t w, uint32_t cap, uint32_t* keys, float* data,
                                    uint32_t* colours);
/* The candidate pairs of world w (see the solver's), world-local indices. */
R2D_API int r2d_batch_num_pairs(r2d_batch* b, uint32_t w, uint32_t* out);
R2D_API int r2d_batch_get_pairs(r2d_batch* b, uint32_t w, uint32_t cap, uint32_t* pairs);

/* ---------------------------------------------------------------------------
 * One world stepped with no allocation.  No counterpart in the reference.
 *
 * For callers that must not allocate device memory once they run: a fixed-step
 * physics tick inside a game or robotics frame loop with a hard frame budget
 * (cudaMalloc and cudaFree can synchronise the whole device and stall the
 * frame), or an embedder that owns all device memory through its own pool and
 * forbids driver allocations after start-up.  The caller passes the world in
 * its own DEVICE buffers (state [13][n] and props [5][n] field-major as
 * above, kind [n], ids [n]; AABB fields initialised, e.g. from
 * r2d_solver_read_state); `state` is stepped in place, as one
 * r2d_solver_process call would step it, bit for bit.  `gravity` is a host
 * array of ngrav <= 4 magnitudes; cell_width 0 and table_mult 0 select 4.0
 * and 2.
 *
 * Scratch lives in one static device array of 7,216,128 bytes (6.88 MiB),
 * which every GPU that loads this library holds until the process exits.
 * Limits: 4,096 bodies, 65,536 spatial-hash cell entries, 16,384 candidate
 * pairs, no joints or exclusions; a world beyond them returns
 * R2D_ERR_CAPACITY with the state untouched.  The call allocates nothing
 * (no cudaMalloc, cudaFree or pinned host memory) and synchronises `stream`
 * a few times to read counters back.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  Every call on a device shares the one array and
 * overwrites it: calls that overlap on the GPU (two streams, two host threads)
 * race, so serialise them.
 * ------------------------------------------------------------------------- */
R2D_API int r2d_world_step_static(float* state, const float* props, const uint8_t* kind, const uint32_t* ids,
                                  uint32_t n, const float* gravity, uint32_t ngrav, float dt, uint32_t sub_steps,
                                  uint32_t collision_iters, float cell_width, uint32_t table_mult, void* stream);

/* Library information. */
R2D_API const char* r2d_last_error_string(void);
R2D_API int r2d_version(void);

#ifdef __cplusplus
}
#endif

#endif /* R2D_GB300_H */
