/*
 * frame_loop.c -- the smallest C caller of libr2d_gb300.so: one world of n
 * bodies (field-major arrays as in include/r2d_gb300.h) stepped 600 frames
 * with gravity, then read back.  Returns the first error status, 0 if none.
 *
 *   cc -std=c99 -I include -c examples/frame_loop.c
 *   link with -L resolve2d_gb300/_build -lr2d_gb300 -lcudart
 */
#include <stdio.h>

#include "r2d_gb300.h"

int step_600_frames(uint32_t n, const uint32_t* ids, const uint8_t* kind, const float* props, float* state) {
    r2d_config cfg = {0}; /* cell 4.0, table 2N, library-owned stream */
    r2d_solver* s;
    if (r2d_solver_create(&cfg, &s) != R2D_OK) {
        puts(r2d_last_error_string());
        return 1;
    }
    float g = 9.81f;
    r2d_solver_set_gravity(s, 1, &g);
    r2d_solver_set_bodies(s, n, ids, kind, props, state, /*init_aabb=*/1);
    for (int k = 0; k < 600; ++k) r2d_solver_process(s, 1.0f / 60, 1, 8);
    int st = r2d_solver_sync(s); /* 0, or the first failure of those calls */
    r2d_solver_read_state(s, state);
    r2d_solver_destroy(s);
    return st;
}
