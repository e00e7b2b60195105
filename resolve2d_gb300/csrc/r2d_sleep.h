/*
 * r2d_sleep.h -- when a world falls asleep (R2D_FLAG_SLEEP; off in reference
 * mode).  The reference has no sleeping; its roadmap lists it
 * (README.md:64-67).  This build sleeps whole worlds: a world whose every
 * non-static body ends R2D_SLEEP_FRAMES consecutive steps with a linear speed
 * below 0.01 units/s and an angular speed below 0.01 rad/s is not stepped
 * again until the host writes to the engine (state, fields, bodies, gravity,
 * joints or exclusions), which wakes every world.  A sleeping world's state,
 * manifolds and debug taps stay as the last stepped frame left them.
 *
 * The test runs on the step's final momenta with f32 arithmetic in a fixed
 * order (no contraction), on the GPU and in the oracle alike, so both reach
 * the same decisions.
 */
#ifndef R2D_SLEEP_H
#define R2D_SLEEP_H

#include <stdint.h>

#if defined(__CUDACC__)
#define R2D_SLEEP_FN __host__ __device__ __forceinline__
#else
#define R2D_SLEEP_FN inline
#endif

#define R2D_SLEEP_FRAMES 60u     /* consecutive still steps before a world sleeps */
#define R2D_SLEEP_SPEED2 1.0e-4f /* (0.01 units/s)^2 */
#define R2D_SLEEP_SPIN2 1.0e-4f  /* (0.01 rad/s)^2 */

/* A non-static body is still when |p|^2 / m^2 and L^2 / I^2 are both below
 * the bounds (a NaN is never still). */
R2D_SLEEP_FN bool r2d_body_still(float mx, float my, float L, float inv_m, float inv_i) {
    const float v2 = (mx * mx + my * my) * (inv_m * inv_m);
    const float w2 = (L * L) * (inv_i * inv_i);
    return v2 < R2D_SLEEP_SPEED2 && w2 < R2D_SLEEP_SPIN2;
}

/* The counter after a stepped frame: one more still frame, or back to zero. */
R2D_SLEEP_FN uint32_t r2d_sleep_next(uint32_t frames, bool all_still) {
    return all_still ? (frames < R2D_SLEEP_FRAMES ? frames + 1u : frames) : 0u;
}

#endif /* R2D_SLEEP_H */
