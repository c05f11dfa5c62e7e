/*
 * psi_sparse.h -- exact CPU restatement of the reference CPUParity solver with
 * path-based valuations, for games far beyond the dense table's reach.
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU legs of
 * bench.py as a checker or a timed baseline; never by the product path.
 */
#ifndef PSI_SPARSE_H
#define PSI_SPARSE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sparse sparse_t;

/* Game in CSR form (successors of v: targets[offsets[v] .. offsets[v+1]) in
 * file order); the arrays are copied.  threads <= 0: every online core. */
sparse_t *sparse_create(int n, const int *owner, const int *priority, const int *offsets, const int *targets,
                        int threads);
void sparse_destroy(sparse_t *o);
int sparse_max_pri(const sparse_t *o);
int sparse_threads(const sparse_t *o);

void sparse_init_strat(sparse_t *o);
void sparse_reset_opponent_strategy(sparse_t *o);
void sparse_compute_valuation(sparse_t *o);
void sparse_mark_solved(sparse_t *o, int player);
int64_t sparse_switch_strategy(sparse_t *o, int player);
int64_t sparse_get_winning(const sparse_t *o, int player, int *out);
int sparse_compare(const sparse_t *o, int v, int u);

void sparse_get_strategy(const sparse_t *o, int *out);
void sparse_set_strategy(sparse_t *o, const int *in);
void sparse_get_infinite(const sparse_t *o, int *out);
void sparse_get_solved(const sparse_t *o, int *out);
/* Per vertex after the last evaluation: the length of its strategy path to the
 * sink (0 if its valuation is infinite), the highest priority on that path and
 * how often it occurs (-1 and 0 if infinite).  Any pointer may be NULL. */
void sparse_get_summary(const sparse_t *o, int *depth, int *top, int *count);
/* Dense valuation rows [v0, v0+count) of (max_pri+1) ints each (rows of
 * infinite vertices are zero), by walking each finite vertex's path. */
void sparse_get_vals(const sparse_t *o, int v0, int count, int *out);

int sparse_solve(sparse_t *o, int reset, int *iter_count, int *br_count, int64_t max_evals);

#ifdef __cplusplus
}
#endif
#endif
