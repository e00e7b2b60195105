// Thin binding of libr2d_gb300.so (include/r2d_gb300.h): the file a
// maintainer adds to the reference as src/core/gpu/r2d.zig.  One `extern fn`
// per entry point of the header, with the same parameters; the Config struct
// lays out r2d_config field for field.  Written against the header; no Zig
// toolchain was available to compile it.
pub const Status = c_int;
pub const OK: Status = 0;
pub const ERR_INVALID_ARGUMENT: Status = -1;
pub const ERR_INVALID_BODY_ID: Status = -2;
pub const ERR_OUT_OF_MEMORY: Status = -3;
pub const ERR_CUDA: Status = -4;
pub const ERR_CAPACITY: Status = -5;
pub const ERR_TIMEOUT: Status = -6;
pub const ERR_NONFINITE: Status = -7;
pub const ERR_NO_DEVICE: Status = -8;

pub const Config = extern struct {
    spatialhash_cell_width: f32 = 0, // 0 = 4.0 (lib.zig:255)
    spatialhash_table_size_mult: u32 = 0, // 0 = 2 (lib.zig:254)
    flags: u32 = 0,
    stream: ?*anyopaque = null,
    capacity_scale: f32 = 0,
};

pub const Solver = opaque {};

pub extern "r2d_gb300" fn r2d_solver_create(cfg: *const Config, out: *?*Solver) Status;
pub extern "r2d_gb300" fn r2d_solver_destroy(s: *Solver) Status;
pub extern "r2d_gb300" fn r2d_solver_set_bodies(s: *Solver, n: u32, ids: [*]const u32, kind: [*]const u8,
    props: [*]const f32, state: [*]const f32, init_aabb: c_int) Status;
pub extern "r2d_gb300" fn r2d_solver_set_polygons(s: *Solver, n: u32, body: [*]const u32, nverts: [*]const u8,
    verts: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_solver_write_state(s: *Solver, state: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_solver_read_state(s: *Solver, state: [*]f32) Status;
pub extern "r2d_gb300" fn r2d_solver_set_gravity(s: *Solver, n: u32, g: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_solver_set_joints(s: *Solver, n: u32, jtype: [*]const u8, id1: [*]const u32,
    id2: [*]const u32, params: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_solver_set_exclusions(s: *Solver, n: u32, pairs: [*]const u32) Status;
pub extern "r2d_gb300" fn r2d_solver_process(s: *Solver, dt: f32, sub_steps: u32, iters: u32) Status;
pub extern "r2d_gb300" fn r2d_solver_sync(s: *Solver) Status;
pub extern "r2d_gb300" fn r2d_solver_process_io(s: *Solver, dt: f32, sub_steps: u32, iters: u32,
    force_rows: ?[*]const f32, out_rows: ?[*]f32) Status;
pub extern "r2d_gb300" fn r2d_solver_write_state_fields(s: *Solver, first: u32, count: u32, rows: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_solver_read_state_fields(s: *Solver, first: u32, count: u32, rows: [*]f32) Status;
pub extern "r2d_gb300" fn r2d_solver_read_positions_f64(s: *Solver, pose: [*]f64) Status;
pub extern "r2d_gb300" fn r2d_solver_sleep_frames(s: *Solver, frames: *u32) Status;
pub extern "r2d_gb300" fn r2d_solver_launches_per_step(s: *Solver, out: *u32) Status;
pub extern "r2d_gb300" fn r2d_solver_num_manifolds(s: *Solver, out: *u32) Status;
pub extern "r2d_gb300" fn r2d_solver_get_manifolds(s: *Solver, cap: u32, keys: ?[*]u32, data: ?[*]f32,
    colours: ?[*]u32) Status;
pub extern "r2d_gb300" fn r2d_solver_get_joint_colours(s: *Solver, cap: u32, colours: [*]u32) Status;
pub extern "r2d_gb300" fn r2d_solver_num_pairs(s: *Solver, out: *u32) Status;
pub extern "r2d_gb300" fn r2d_solver_get_pairs(s: *Solver, cap: u32, pairs: ?[*]u32) Status;

// many independent worlds in one engine
pub const Batch = opaque {};

pub extern "r2d_gb300" fn r2d_batch_create(cfg: *const Config, out: *?*Batch) Status;
pub extern "r2d_gb300" fn r2d_batch_destroy(b: *Batch) Status;
pub extern "r2d_gb300" fn r2d_batch_set_worlds(b: *Batch, nworlds: u32, body_off: [*]const u32, ids: [*]const u32,
    kind: [*]const u8, props: [*]const f32, state: [*]const f32, gravity: [*]const f32, init_aabb: c_int) Status;
pub extern "r2d_gb300" fn r2d_batch_set_polygons(b: *Batch, n: u32, body: [*]const u32, nverts: [*]const u8,
    verts: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_batch_write_state(b: *Batch, state: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_batch_read_state(b: *Batch, state: [*]f32) Status;
pub extern "r2d_gb300" fn r2d_batch_process(b: *Batch, dt: f32, sub_steps: u32, iters: u32) Status;
pub extern "r2d_gb300" fn r2d_batch_sync(b: *Batch) Status;
pub extern "r2d_gb300" fn r2d_batch_process_io(b: *Batch, dt: f32, sub_steps: u32, iters: u32,
    force_rows: ?[*]const f32, out_rows: ?[*]f32) Status;
pub extern "r2d_gb300" fn r2d_batch_launches_per_step(b: *Batch, out: *u32) Status;
pub extern "r2d_gb300" fn r2d_batch_sleep_frames(b: *Batch, frames: [*]u32) Status;
pub extern "r2d_gb300" fn r2d_batch_write_state_fields(b: *Batch, first: u32, count: u32, rows: [*]const f32) Status;
pub extern "r2d_gb300" fn r2d_batch_read_state_fields(b: *Batch, first: u32, count: u32, rows: [*]f32) Status;
pub extern "r2d_gb300" fn r2d_batch_autotune(b: *Batch, dt: f32, sub_steps: u32, iters: u32, trial_steps: u32) Status;
pub extern "r2d_gb300" fn r2d_batch_read_positions_f64(b: *Batch, pose: [*]f64) Status;
pub extern "r2d_gb300" fn r2d_batch_world_status(b: *Batch, status: [*]c_int) Status;
pub extern "r2d_gb300" fn r2d_batch_num_manifolds(b: *Batch, w: u32, out: *u32) Status;
pub extern "r2d_gb300" fn r2d_batch_get_manifolds(b: *Batch, w: u32, cap: u32, keys: ?[*]u32, data: ?[*]f32,
    colours: ?[*]u32) Status;
pub extern "r2d_gb300" fn r2d_batch_num_pairs(b: *Batch, w: u32, out: *u32) Status;
pub extern "r2d_gb300" fn r2d_batch_get_pairs(b: *Batch, w: u32, cap: u32, pairs: ?[*]u32) Status;

// one world stepped in caller-owned device buffers, allocating nothing
pub extern "r2d_gb300" fn r2d_world_step_static(state: [*]f32, props: [*]const f32, kind: [*]const u8,
    ids: [*]const u32, n: u32, gravity: ?[*]const f32, ngrav: u32, dt: f32, sub_steps: u32, iters: u32,
    cell_width: f32, table_mult: u32, stream: ?*anyopaque) Status;
pub extern "r2d_gb300" fn r2d_last_error_string() [*:0]const u8;
pub extern "r2d_gb300" fn r2d_version() c_int;
