// tune.h -- the autotuner (psi_autotune).
#ifndef PSI_TUNE_H
#define PSI_TUNE_H

#include <vector>

#include "game.h"
#include "psi.h"

namespace psi {

// Chooses sublist_len, walk_block and patch_limit for the workload `gs` (one
// game, or a batch when there are several) by timing trial solves on
// base.device; the other options are taken from base.  Writes the chosen
// options to *out and what was timed to *rep.
int autotune(const std::vector<const HostGame *> &gs, const psi_options &base, int32_t repeats, int32_t flags,
             psi_options *out, psi_tune_report *rep);

// The candidate values tried for each knob, in the order they are tried
// (the first of each is the default).
const std::vector<int32_t> &tune_sublist_lens();
const std::vector<int32_t> &tune_walk_blocks();
const std::vector<int32_t> &tune_patch_divisors();

}  // namespace psi

#endif
