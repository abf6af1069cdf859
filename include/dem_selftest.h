/*
 * dem_selftest.h -- self-tests of the device arithmetic helpers.
 * No reference counterpart: these check, on the GPU, that the exact
 * shortcuts used by the fused step return the IEEE result bit for bit.
 */
#ifndef DEM_SELFTEST_H
#define DEM_SELFTEST_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
/* Draws n seeded (a, b) pairs over several magnitude ranges, and counts the
 * pairs where the reciprocal-based division (Markstein's correction step with
 * y = RN(1/b)) differs in any bit from the compiled division a / b.        */
int dem_selftest_division(uint64_t n, uint64_t seed, uint64_t* mismatches, uint64_t* fast_path_taken);

/* Draws n seeded near-threshold cases of the polyhedron broad-phase tests
 * (kind = case % 6: 0 vertex gate / OBB::intersect, 1 filter_vv, 2 filter_ve,
 * 3 filter_vf, 4 filter_ee, 5 vertex displacement against max_displ) and
 * evaluates each with its FP32 decision and its FP64 test.
 * counts[4 * kind + k] (24 entries), k = 0: decided cases whose result differs
 * from FP64 (must be 0), 1: undecided cases, 2: decided true, 3: FP64 true.  */
int dem_selftest_poly_decisions(uint64_t n, uint64_t seed, uint64_t* counts);

/* Draws n seeded operand pairs (typical magnitudes, short significands that
 * give exact products and ties, the whole exponent range, boundaries, zeros,
 * subnormals, infinities, NaNs) and counts the results of the integer-pipe
 * binary64 multiply (emu_dmul, and the exact x*2 / x*0.5) that differ in any
 * bit from the hardware multiply; for each pair and three derived ones (the
 * negation of a, its neighbours, a gap of 0..70 binades) also the sums and
 * differences of the integer-pipe addition (emu_dadd_nb, emu_dsub_nb) that
 * differ from the hardware's, where the addition keeps its fast path.     */
int dem_selftest_emu_mul(uint64_t n, uint64_t seed, uint64_t* mismatches);

/* Draws n seeded (branch, spin, normal force, moment) cases around the range
 * bounds of the exact rolling-clip shortcut (mur = 0) and counts the moments
 * that differ in any bit from the formula (r = b.w / w.w, ... , m * t/|m|);
 * fast_path_taken counts the cases inside the shortcut's range.            */
int dem_selftest_rolling_clip(uint64_t n, uint64_t seed, uint64_t* mismatches, uint64_t* fast_path_taken);

#ifdef __cplusplus
}
#endif
#endif
