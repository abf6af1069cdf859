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
#ifdef __cplusplus
}
#endif
#endif
