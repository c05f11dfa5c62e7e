// check.h -- certificate check of a solved parity game (check.cpp).
#ifndef PSI_CHECK_H
#define PSI_CHECK_H

#include <cstdint>

#include "game.h"

namespace psi {

struct CheckReport {
    int32_t status = 0;        // PSI_CHECK_*
    int64_t vertex = -1;       // the lowest offending vertex found, if any
    int64_t edge_visits = 0;   // work of the cycle-parity check
};

// strategy[n]: each vertex's successor (-1 = the sink, Even only); infinite[n]:
// +1 where Even wins (W0), anything else where Odd wins (W1).  work_budget:
// edge visits allowed to the cycle-parity check (<= 0: unbounded).
int check_solution(const CsrView &g, const int32_t *strategy, const int32_t *infinite, int64_t work_budget,
                   CheckReport *out);

}  // namespace psi

#endif
