/*
 * r2d_accum.h -- compensated accumulation of a contact point's impulses
 * (R2D_FLAG_COMPENSATED; off in reference mode), shared by the CUDA kernels
 * and the CPU oracle so that both round identically.
 *
 * The reference accumulates each point's normal and tangent impulse in f32
 * and applies the change of the clamped sum to the bodies
 * (CollisionManifold.calculateImpulses, src/core/collision.zig:182-190):
 *
 *     new = clamp(acc + x);  applied = new - acc;  acc = new;
 *
 * With warm starting the sum lives across frames and grows large against its
 * per-iteration increments, so the rounding of `acc + x` drops part of every
 * increment.  Kahan's compensated summation (W. Kahan, "Further remarks on
 * reducing truncation errors", CACM 8(1):40, 1965) keeps that part in a
 * second word: the accumulated impulse is s + c, where s is the value the
 * solver reads and c holds what s could not.
 *
 *     y = x + c;  t = s + y;  c' = y - (t - s);       (t - s is what s took)
 *     new = clamp(t);  if new != t: c' = 0              (a clamped sum is exact)
 *     applied = new - s;  s = new;  c = c'
 *
 * The bodies receive the change of s, as in the reference; the part in c
 * reaches them once later increments carry it into s.  A NaN total clamps to
 * the bound (NaN-ignoring max/min, as Zig's @max/@min) and clears c.
 */
#ifndef R2D_ACCUM_H
#define R2D_ACCUM_H

#if defined(__CUDACC__)
#define R2D_ACCUM_FN __host__ __device__ __forceinline__
#else
#define R2D_ACCUM_FN inline
#endif

/* NaN-ignoring max / min: the non-NaN operand wins (Zig's @max / @min). */
template <class R>
R2D_ACCUM_FN R r2d_acc_max(R a, R b) {
    R r = a > b ? a : b;
    r = (b != b) ? a : r;
    return (a != a) ? b : r;
}
template <class R>
R2D_ACCUM_FN R r2d_acc_min(R a, R b) {
    R r = a < b ? a : b;
    r = (b != b) ? a : r;
    return (a != a) ? b : r;
}

/* acc = max(lo, acc + x), compensated; returns the change of s. */
template <class R>
R2D_ACCUM_FN R r2d_acc_add_max(R* s, R* c, R x, R lo) {
    const R y = x + *c;
    const R t = *s + y;
    R nc = y - (t - *s);
    const R nt = r2d_acc_max(lo, t);
    if (!(nt == t)) nc = R(0);
    const R applied = nt - *s;
    *s = nt;
    *c = nc;
    return applied;
}

/* acc = clamp(acc + x, lo, hi) = max(lo, min(acc + x, hi)), compensated;
 * returns the change of s. */
template <class R>
R2D_ACCUM_FN R r2d_acc_add_clamp(R* s, R* c, R x, R lo, R hi) {
    const R y = x + *c;
    const R t = *s + y;
    R nc = y - (t - *s);
    const R nt = r2d_acc_max(lo, r2d_acc_min(t, hi));
    if (!(nt == t)) nc = R(0);
    const R applied = nt - *s;
    *s = nt;
    *c = nc;
    return applied;
}

#endif /* R2D_ACCUM_H */
