/*
 * psi_oracle.h -- C restatement of the reference CPUParity solver.
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU-baseline
 * leg of bench.py as the parity checker; never by the product path.
 */
#ifndef PSI_ORACLE_H
#define PSI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle oracle_t;

/* Game in CSR form: successors of v are targets[offsets[v] .. offsets[v+1]) in
 * file order.  The arrays are copied. */
oracle_t *oracle_create(int n, const int *owner, const int *priority,
                        const int *offsets, const int *targets);
void oracle_destroy(oracle_t *o);
int oracle_max_pri(const oracle_t *o);

void oracle_init_strat(oracle_t *o);
void oracle_reset_opponent_strategy(oracle_t *o);
void oracle_compute_valuation(oracle_t *o);
void oracle_mark_solved(oracle_t *o, int player);
int64_t oracle_switch_strategy(oracle_t *o, int player);
int64_t oracle_get_winning(const oracle_t *o, int player, int *out);
int oracle_compare(const oracle_t *o, int v, int u);

void oracle_get_strategy(const oracle_t *o, int *out);
void oracle_set_strategy(oracle_t *o, const int *in);
void oracle_get_infinite(const oracle_t *o, int *out);
void oracle_get_solved(const oracle_t *o, int *out);
void oracle_get_vals(const oracle_t *o, int v0, int count, int *out);

int oracle_solve(oracle_t *o, int reset, int *iter_count, int *br_count, int64_t max_evals);

#ifdef __cplusplus
}
#endif
#endif
