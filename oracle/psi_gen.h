/*
 * psi_gen.h -- the seeded workload games, generated on the CPU without the
 * product library.  TEST INFRASTRUCTURE ONLY (bench.py's reference arm and the
 * tests).  Every function returns a negative value on bad arguments.
 */
#ifndef PSI_GEN_H
#define PSI_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Random game: edge count (offsets[n+1] filled when offsets != NULL). */
int64_t oracle_gen_random_edges(int n, int deg_lo, int deg_hi, uint64_t seed, int *offsets);
/* Random game: owner, priority and targets for the offsets above. */
int oracle_gen_random_fill(int n, int deg_lo, int deg_hi, int pri_hi, uint64_t seed, const int *offsets, int *owner,
                           int *priority, int *targets);
/* Long-path game: 2n-2 edges. */
int64_t oracle_gen_longpath_edges(int n);
int oracle_gen_longpath(int n, int pri_hi, uint64_t seed, int *owner, int *priority, int *offsets, int *targets);

#ifdef __cplusplus
}
#endif
#endif
