// psi_internal.h -- shared declarations of the native library (host side).
#ifndef PSI_INTERNAL_H
#define PSI_INTERNAL_H

#include <cstdint>
#include <string>

#include "psi.h"

namespace psi {

// Error reporting: the C-ABI returns a status code and keeps a per-thread
// message readable through psi_last_error().
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

int gen_random_offsets(int32_t n, int32_t deg_lo, int32_t deg_hi, uint64_t seed, int32_t *offsets);
int gen_random_fill(int32_t n, int32_t deg_lo, int32_t deg_hi, int32_t pri_hi, uint64_t seed,
                    const int32_t *offsets, int32_t *owner, int32_t *priority, int32_t *targets);
int gen_longpath(int32_t n, int32_t pri_hi, uint64_t seed, int32_t *owner, int32_t *priority,
                 int32_t *offsets, int32_t *targets);
int gen_batch_sizes(int32_t count, int32_t n_lo, int32_t n_hi, uint64_t seed, int32_t *sizes);
uint64_t gen_game_seed(uint64_t seed, int32_t index);

// psi_measure_random_access (measure.cu)
int measure_random_access(int32_t device, int64_t array_bytes, int32_t reps, double *gathers_per_s,
                          double *ms_per_launch, int64_t *gathers_per_launch);

}  // namespace psi

#endif
