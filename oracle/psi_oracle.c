/*
 * psi_oracle.c -- CPU restatement of the reference strategy-improvement solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the
 * smoke check and the CPU-baseline leg of bench.py call it to check or to time
 * against the CUDA path.  No product code path links, loads or falls back to it.
 *
 * It restates, in plain C, the semantics of the reference's CPUParity solver
 * (cpu_parity.cpp) and of its solve_si driver (main.cpp:20-55):
 *
 *   - dense valuations: vals[v][p] = number of vertices of priority p on the
 *     strategy path from v (inclusive) to the virtual sink (cpu_parity.cpp:54-114);
 *   - +inf / -inf for paths that end in a cycle, by the parity of the cycle's
 *     maximum priority (cpu_parity.cpp:35-52, 80-89);
 *   - solved (frozen) vertices from mark_solved (cpu_parity.cpp:265-274, 116-127);
 *   - the lexicographic comparison (cpu_parity.cpp:154-236);
 *   - the all-switches rule: per vertex, scan the CSR successors in file order and
 *     replace the running choice only on a strict improvement
 *     (cpu_parity.cpp:239-263).
 *
 * The recursion of cpu_parity.cpp:54-114 is written here as an explicit walk plus
 * an unwind over a path stack, so long strategy paths do not overflow the C
 * stack; the values it assigns are the same.
 *
 * Parity status: pinned.  tests/test_oracle_vs_reference.py runs this oracle
 * and the reference's own CPUParity (compiled from its sources by
 * oracle/build_ref.sh into oracle/_ref/) in lockstep on seeded random games and
 * compares every strategy, infinite flag and valuation; tests/golden/ holds
 * fixtures produced by the compiled reference (tests/golden/make_golden.py).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "psi_oracle.h"

struct oracle {
    int n;
    int max_pri;             /* d = max_pri + 1 priorities, as Game::get_max_pri */
    int64_t m;
    int *owner, *priority, *offsets, *targets;
    int *strat, *infinite, *solved, *done;
    int *vals;               /* n * d, row-major (the reference's ArrayVal layout) */
    int *zero_val;           /* d zeros: valuation of the sink */
    int *stack;              /* explicit recursion stack (n entries) */
};

static int64_t rowsz(const oracle_t *o) { return (int64_t)o->max_pri + 1; }
static int *row(const oracle_t *o, int v) { return o->vals + (int64_t)v * rowsz(o); }

oracle_t *oracle_create(int n, const int *owner, const int *priority,
                        const int *offsets, const int *targets)
{
    if (n < 0) return NULL;                       /* n = 0: the empty game (game.cpp:56 with no lines) */
    oracle_t *o = (oracle_t *)calloc(1, sizeof(oracle_t));
    if (!o) return NULL;
    const int n1 = n > 0 ? n : 1;                 /* every array gets at least one slot */
    o->n = n;
    o->m = offsets[n];
    int mp = 0;                                   /* game.cpp:18-31: max_pri >= 0 */
    for (int v = 0; v < n; v++)
        if (priority[v] > mp) mp = priority[v];
    o->max_pri = mp;
    o->owner = (int *)malloc(sizeof(int) * n1);
    o->priority = (int *)malloc(sizeof(int) * n1);
    o->offsets = (int *)malloc(sizeof(int) * (n + 1));
    o->targets = (int *)malloc(sizeof(int) * (o->m > 0 ? o->m : 1));
    o->strat = (int *)calloc(n1, sizeof(int));
    o->infinite = (int *)calloc(n1, sizeof(int));
    o->solved = (int *)calloc(n1, sizeof(int));
    o->done = (int *)calloc(n1, sizeof(int));
    o->stack = (int *)malloc(sizeof(int) * n1);
    o->vals = (int *)calloc((size_t)n1 * (size_t)rowsz(o), sizeof(int));
    o->zero_val = (int *)calloc((size_t)rowsz(o), sizeof(int));
    if (!o->owner || !o->priority || !o->offsets || !o->targets || !o->strat ||
        !o->infinite || !o->solved || !o->done || !o->stack || !o->vals || !o->zero_val) {
        oracle_destroy(o);
        return NULL;
    }
    memcpy(o->owner, owner, sizeof(int) * n);
    memcpy(o->priority, priority, sizeof(int) * n);
    memcpy(o->offsets, offsets, sizeof(int) * (n + 1));
    if (o->m > 0) memcpy(o->targets, targets, sizeof(int) * o->m);
    return o;
}

void oracle_destroy(oracle_t *o)
{
    if (!o) return;
    free(o->owner); free(o->priority); free(o->offsets); free(o->targets);
    free(o->strat); free(o->infinite); free(o->solved); free(o->done);
    free(o->stack); free(o->vals); free(o->zero_val);
    free(o);
}

int oracle_max_pri(const oracle_t *o) { return o->max_pri; }

/* cpu_parity.cpp:276-286.  The reference's solver object serves one solve
 * (its init_strat appends to strat); starting a solve here also clears what
 * a previous solve on the same object left in solved[] and infinite[], so
 * every solve runs as on a fresh CPUParity (cpu_parity.cpp:20-33). */
void oracle_init_strat(oracle_t *o)
{
    for (int v = 0; v < o->n; v++) {
        o->strat[v] = (o->owner[v] == 0) ? -1 : o->targets[o->offsets[v]];
        o->solved[v] = 0;
        o->infinite[v] = 0;
    }
}

/* cpu_parity.cpp:300-307 */
void oracle_reset_opponent_strategy(oracle_t *o)
{
    for (int v = 0; v < o->n; v++)
        if (o->owner[v] == 1) o->strat[v] = o->targets[o->offsets[v]];
}

/* cpu_parity.cpp:35-52: parity of the maximum priority on the cycle through v */
static int even_cycle(const oracle_t *o, int v)
{
    int cur = v, maxpri = 0;
    for (;;) {
        cur = o->strat[cur];
        if (o->priority[cur] > maxpri) maxpri = o->priority[cur];
        if (cur == v) break;
    }
    return maxpri % 2 == 0;
}

/* Resolve v whose successor nx = strat[v] is already done (done[nx] == 2):
 * cpu_parity.cpp:98-112. */
static void finish_from_next(oracle_t *o, int v)
{
    int nx = o->strat[v];
    if (o->infinite[nx] != 0) {
        o->infinite[v] = o->infinite[nx];
    } else {
        int64_t d = rowsz(o);
        memcpy(row(o, v), row(o, nx), sizeof(int) * d);
        row(o, v)[o->priority[v]] += 1;
    }
    o->done[v] = 2;
}

/* cpu_parity.cpp:54-114 as an explicit walk + unwind.  done: 0 untouched,
 * 1 on the current path, 2 finished. */
static void compute_valuation_from(oracle_t *o, int start)
{
    int top = 0;
    int x = start;
    for (;;) {
        if (o->infinite[x] == 1) {                 /* cpu_parity.cpp:61-65 */
            o->done[x] = 2;
            break;
        }
        if (o->strat[x] == -1) {                   /* cpu_parity.cpp:67-76 */
            int64_t d = rowsz(o);
            memset(row(o, x), 0, sizeof(int) * d);
            row(o, x)[o->priority[x]] = 1;
            o->done[x] = 2;
            break;
        }
        int nx = o->strat[x];
        if (o->done[nx] == 1) {                    /* cpu_parity.cpp:80-89 */
            o->infinite[x] = even_cycle(o, x) ? 1 : -1;
            o->done[x] = 2;
            break;
        }
        if (o->done[nx] == 0) {                    /* cpu_parity.cpp:91-96 */
            o->done[x] = 1;
            o->stack[top++] = x;
            x = nx;
            continue;
        }
        finish_from_next(o, x);                    /* done[nx] == 2 */
        break;
    }
    while (top > 0) finish_from_next(o, o->stack[--top]);
}

/* cpu_parity.cpp:116-133 */
void oracle_compute_valuation(oracle_t *o)
{
    for (int v = 0; v < o->n; v++) {
        if (!o->solved[v]) {
            o->done[v] = 0;
            o->infinite[v] = 0;
        } else {
            o->done[v] = 2;
        }
    }
    for (int v = 0; v < o->n; v++)
        if (!o->done[v]) compute_valuation_from(o, v);
}

/* cpu_parity.cpp:154-192 */
static int compare_rows(const oracle_t *o, const int *a, const int *b)
{
    int maxdiff = -1;
    for (int i = (int)rowsz(o) - 1; i >= 0; i--)
        if (a[i] != b[i]) { maxdiff = i; break; }
    if (maxdiff == -1) return 0;
    int ac = a[maxdiff], bc = b[maxdiff];
    if (maxdiff % 2 == 0) return ac > bc ? 1 : (ac == bc ? 0 : -1);
    return ac < bc ? 1 : (ac == bc ? 0 : -1);
}

/* cpu_parity.cpp:194-236: 1 if v is better for Even than u, 0 if equal, -1 if worse.
 * -1 denotes the sink. */
int oracle_compare(const oracle_t *o, int v, int u)
{
    int iv = (v != -1) ? o->infinite[v] : 0;
    int iu = (u != -1) ? o->infinite[u] : 0;
    if (v != -1 && u != -1 && iv && iu) {
        if (iv == 1 && iu == -1) return 1;
        if (iv == -1 && iu == 1) return -1;
        return 0;
    }
    if ((v != -1 && iv) && (u == -1 || !iu)) return iv == 1 ? 1 : -1;
    if ((u != -1 && iu) && (v == -1 || !iv)) return iu == 1 ? -1 : 1;
    const int *a = (v == -1) ? o->zero_val : row(o, v);
    const int *b = (u == -1) ? o->zero_val : row(o, u);
    return compare_rows(o, a, b);
}

/* cpu_parity.cpp:239-263: returns the number of replacements */
int64_t oracle_switch_strategy(oracle_t *o, int player)
{
    int64_t total = 0;
    for (int v = 0; v < o->n; v++) {
        if (o->owner[v] != player) continue;
        int cur = o->strat[v];
        for (int e = o->offsets[v]; e < o->offsets[v + 1]; e++) {
            int u = o->targets[e];
            int c = oracle_compare(o, u, cur);
            if ((player == 0 && c == 1) || (player == 1 && c == -1)) {
                o->strat[v] = u;
                cur = u;
                total++;
            }
        }
    }
    return total;
}

/* cpu_parity.cpp:265-274 */
void oracle_mark_solved(oracle_t *o, int player)
{
    for (int v = 0; v < o->n; v++) {
        if (player == 0 && o->infinite[v] == 1) o->solved[v] = 1;
        else if (player == 1 && o->infinite[v] == -1) o->solved[v] = 1;
    }
}

/* cpu_parity.cpp:288-297: writes the winning set of `player` in increasing
 * vertex order, returns its size.  out may be NULL to only count. */
int64_t oracle_get_winning(const oracle_t *o, int player, int *out)
{
    int64_t k = 0;
    for (int v = 0; v < o->n; v++) {
        int w0 = (o->infinite[v] == 1);
        if ((player == 0 && w0) || (player == 1 && !w0)) {
            if (out) out[k] = v;
            k++;
        }
    }
    return k;
}

void oracle_get_strategy(const oracle_t *o, int *out) { memcpy(out, o->strat, sizeof(int) * o->n); }
void oracle_set_strategy(oracle_t *o, const int *in) { memcpy(o->strat, in, sizeof(int) * o->n); }
void oracle_get_infinite(const oracle_t *o, int *out) { memcpy(out, o->infinite, sizeof(int) * o->n); }
void oracle_get_solved(const oracle_t *o, int *out) { memcpy(out, o->solved, sizeof(int) * o->n); }

/* Dense valuation rows [v0, v0+count) of (max_pri+1) ints each. */
void oracle_get_vals(const oracle_t *o, int v0, int count, int *out)
{
    memcpy(out, row(o, v0), sizeof(int) * (size_t)count * (size_t)rowsz(o));
}

/* main.cpp:20-55 (solve_si).  With reset != 0 it is the "cpu-reset" variant
 * (main.cpp:27-28).  Returns 0, or -1 if max_rounds evaluations were reached. */
int oracle_solve(oracle_t *o, int reset, int *iter_count, int *br_count, int64_t max_evals)
{
    int iters = 0, brs = 0, first = 1;
    oracle_init_strat(o);
    for (;;) {
        if (!first && reset) oracle_reset_opponent_strategy(o);
        for (;;) {
            oracle_compute_valuation(o);   /* compute_first_val == compute_valuation for CPUParity */
            brs++;
            oracle_mark_solved(o, 1);
            if (oracle_switch_strategy(o, 1) == 0) break;
            if (max_evals > 0 && brs >= max_evals) goto out_cap;
        }
        first = 0;
        oracle_mark_solved(o, 0);
        iters++;
        if (oracle_switch_strategy(o, 0) == 0) break;
        if (max_evals > 0 && brs >= max_evals) goto out_cap;
    }
    *iter_count = iters;
    *br_count = brs;
    return 0;
out_cap:
    *iter_count = iters;
    *br_count = brs;
    return -1;
}
