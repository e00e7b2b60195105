/*
 * r2d_validate.h -- host-side checks of the body arrays a caller hands to the
 * library (r2d_solver_set_bodies, r2d_batch_set_worlds).
 */
#ifndef R2D_VALIDATE_H
#define R2D_VALIDATE_H

#include <stdint.h>

#include <algorithm>
#include <vector>

/* The first world that holds two bodies with one id, or -1 if there is none;
 * *dup receives the repeated id.  The reference keeps a world's bodies in a
 * map keyed by id (src/core/lib.zig:135), so one id names one body.  Worlds
 * are body_off[w] .. body_off[w+1]; the offsets must already be monotonic. */
inline int64_t r2d_first_duplicate_id(uint32_t nworlds, const uint32_t* body_off, const uint32_t* ids,
                                      uint32_t* dup) {
    std::vector<uint32_t> sorted;
    for (uint32_t w = 0; w < nworlds; ++w) {
        const uint32_t b0 = body_off[w], b1 = body_off[w + 1];
        if (b1 - b0 < 2) continue;
        sorted.assign(ids + b0, ids + b1);
        std::sort(sorted.begin(), sorted.end());
        const auto it = std::adjacent_find(sorted.begin(), sorted.end());
        if (it != sorted.end()) {
            if (dup) *dup = *it;
            return (int64_t)w;
        }
    }
    return -1;
}

#endif /* R2D_VALIDATE_H */
