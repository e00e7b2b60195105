/*
 * r2d_colour.h -- the priority that orders constraints for graph colouring.
 *
 * The reference solves constraints strictly one after another
 * (src/core/lib.zig:226-236): all joints in insertion order, then all
 * contact manifolds in discovery order.  The GPU path instead colours each
 * constraint set greedily into body-disjoint batches and solves colour after
 * colour; inside a colour the constraints touch disjoint bodies, so their
 * order cannot change any result.
 *
 * The colouring is defined as first-fit greedy colouring in ascending
 * priority order, where priority = (r2d_colour_mix(key), key):
 *   contacts: key = (lo, hi), the world-local indices of the two bodies,
 *             lo < hi; only non-static bodies are conflict nodes (the
 *             reference adds exactly +0 to a static body, collision.zig:197-212);
 *   joints:   key = the joint's index in insertion order; every body the
 *             joint names is a conflict node, static or not (the joint solve
 *             functions write both bodies' momenta unconditionally,
 *             e.g. DistanceJoint.zig:72-74).
 * A hashed priority keeps the dependency chains short (Jones-Plassmann
 * rounds on the GPU), and sequential greedy in the same order (the oracle)
 * gives the identical colouring by construction.
 */
#ifndef R2D_COLOUR_H
#define R2D_COLOUR_H

#include <stdint.h>

#if defined(__CUDACC__)
#define R2D_COL_FN __host__ __device__ __forceinline__
#else
#define R2D_COL_FN static inline
#endif

/* 32-bit avalanche mix of two words (multiply-xorshift finaliser with the
 * "lowbias32" constants published by C. Wellons, 2018). */
R2D_COL_FN uint32_t r2d_colour_mix(uint32_t a, uint32_t b)
{
    uint32_t h = a * 0x9E3779B1u + b * 0x85EBCA77u + 0x165667B1u;
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}

/* Joints are keyed by their insertion index; the second word separates the
 * joint hash stream from the contact one. */
#define R2D_COLOUR_JOINT_SALT 0x4A4F494Eu

#endif /* R2D_COLOUR_H */
