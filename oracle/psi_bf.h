/*
 * psi_bf.h -- C restatement of the reference's Bellman-Ford best-response
 * solver (CPU_BellmanFord<ArrayVal>, cpu_bf.cpp, on its base CPUBV, cpu_bv.cpp)
 * and of its driver solve_bf (main.cpp:58-76).
 * TEST INFRASTRUCTURE ONLY: an alternative evaluation of Odd's best response
 * that the tests compare the CUDA path against; never part of the product.
 */
#ifndef PSI_BF_H
#define PSI_BF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bf bf_t;

/* Game in CSR form, as oracle_create; the arrays are copied. */
bf_t *bf_create(int n, const int *owner, const int *priority, const int *offsets, const int *targets);
void bf_destroy(bf_t *b);
int bf_max_pri(const bf_t *b);

/* Status of the calls that evaluate: BF_OK, or BF_ODD_CYCLE where the
 * reference prints "Game contains an odd cycle that uses only odd nodes" and
 * exits (cpu_bv.cpp:73-85); the state is then that of the failed evaluation. */
enum { BF_OK = 0, BF_ODD_CYCLE = -1 };

void bf_init_strat(bf_t *b);                                  /* cpu_bv.cpp:220-230 */
int bf_compute_valuation(bf_t *b);                            /* cpu_bv.cpp:53-121 */
void bf_mark_solved(bf_t *b, int player);                     /* cpu_bv.cpp:208-218 */
int64_t bf_switch_strategy(bf_t *b, int player);              /* cpu_bv.cpp:176-206 */
/* One best response (cpu_bf.cpp:24-49): the first by strategy improvement for
 * Odd, every later one by Bellman-Ford (br_count += its rounds). */
int bf_best_response(bf_t *b, int *br_count);
/* solve_bf (main.cpp:58-76); max_iters > 0 stops after that many iterations. */
int bf_solve(bf_t *b, int *iter_count, int *br_count, int max_iters);
int64_t bf_get_winning(const bf_t *b, int player, int *out);  /* cpu_bv.cpp:232-241 */

void bf_get_strategy(const bf_t *b, int *out);
void bf_get_infinite(const bf_t *b, int *out);
void bf_get_solved(const bf_t *b, int *out);
void bf_get_vals(const bf_t *b, int v0, int count, int *out);

#ifdef __cplusplus
}
#endif
#endif
