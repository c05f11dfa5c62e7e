/*
 * psi_bf.c -- CPU restatement of the reference's Bellman-Ford best-response
 * solver.
 *
 * TEST INFRASTRUCTURE ONLY.  It is an alternative evaluation of Odd's best
 * response that the tests compare the CUDA path against; no product code path
 * links, loads or falls back to it.
 *
 * It restates, in plain C with the reference's dense valuation rows (ArrayVal,
 * valuation.cpp:9-115: one count per priority), three pieces of the reference:
 *
 *   - CPUBV (cpu_bv.cpp), the base solver: its evaluation marks a strategy
 *     path that ends in a cycle +inf when the cycle's top priority is even and
 *     gives up on the whole game when it is odd (cpu_bv.cpp:73-85 print a
 *     message and exit; here BF_ODD_CYCLE is returned); its comparison,
 *     all-switches rule, mark_solved, init_strat and get_winning;
 *   - CPU_BellmanFord (cpu_bf.cpp:24-163): the first best response is Odd's
 *     strategy-improvement loop; every later one relaxes the valuations in
 *     place, vertex by vertex in id order, for at most n rounds (br_count += 1
 *     per round): an Even vertex takes its successor's valuation plus itself, an
 *     Odd vertex the least (for Even: the worst) over its successors with a
 *     finite valuation, moving only on a strict improvement; vertices never
 *     given a finite valuation become +inf, and Odd's strategy becomes the
 *     relaxation's choices;
 *   - solve_bf (main.cpp:58-76): best response, mark_solved(0), Even's switch
 *     step, until Even switches nothing.
 *
 * The recursion of cpu_bv.cpp:53-109 is an explicit walk and unwind here, so
 * long strategy paths do not overflow the C stack; the values it assigns are
 * the same.  Quirks kept as the reference has them: the relaxation starts
 * every valuation (also of solved vertices) at zero, an Odd vertex the
 * relaxation never reached takes succ's initial 0 (or its previous choice) as
 * its strategy, and infinite flags are only ever raised, never cleared, by a
 * relaxation.
 *
 * Parity status: pinned.  tests/test_bf_oracle.py runs this restatement and
 * the reference's own CPU_BellmanFord<ArrayVal> (compiled from its sources by
 * oracle/build_ref.sh into oracle/_ref/libpsi_refbf.so) in lockstep and
 * compares every strategy, infinite flag and valuation row after every best
 * response, and the golden digests in tests/golden/reference_bf_solves.json
 * were produced by that compiled reference.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "psi_bf.h"

struct bf {
    int n, max_pri;
    int64_t m;
    int *owner, *priority, *offsets, *targets;
    int *strat, *infinite, *solved, *done;   /* CPUBV state (cpu_bv.h:15-21) */
    int *bf_inf, *succ;                      /* CPU_BellmanFord state (cpu_bf.h:9-12) */
    int init;                                /* the first best response has run */
    int *vals;                               /* n rows of max_pri + 1 counts */
    int *zero_val, *tmp;                     /* the sink's valuation; one scratch row */
    int *stack;                              /* explicit recursion stack */
};

static int64_t rowsz(const bf_t *b) { return (int64_t)b->max_pri + 1; }
static int *row(const bf_t *b, int v) { return b->vals + (int64_t)v * rowsz(b); }

bf_t *bf_create(int n, const int *owner, const int *priority, const int *offsets, const int *targets)
{
    if (n < 0) return NULL;
    bf_t *b = (bf_t *)calloc(1, sizeof(bf_t));
    if (!b) return NULL;
    const int n1 = n > 0 ? n : 1;
    b->n = n;
    b->m = offsets[n];
    int mp = 0;
    for (int v = 0; v < n; v++)
        if (priority[v] > mp) mp = priority[v];
    b->max_pri = mp;
    b->owner = (int *)malloc(sizeof(int) * n1);
    b->priority = (int *)malloc(sizeof(int) * n1);
    b->offsets = (int *)malloc(sizeof(int) * (n + 1));
    b->targets = (int *)malloc(sizeof(int) * (b->m > 0 ? b->m : 1));
    b->strat = (int *)calloc(n1, sizeof(int));
    b->infinite = (int *)calloc(n1, sizeof(int));
    b->solved = (int *)calloc(n1, sizeof(int));
    b->done = (int *)calloc(n1, sizeof(int));
    b->bf_inf = (int *)malloc(sizeof(int) * n1);
    b->succ = (int *)calloc(n1, sizeof(int));   /* cpu_bf.cpp:18: succ starts at 0 */
    b->stack = (int *)malloc(sizeof(int) * n1);
    b->vals = (int *)calloc((size_t)n1 * (size_t)rowsz(b), sizeof(int));
    b->zero_val = (int *)calloc((size_t)rowsz(b), sizeof(int));
    b->tmp = (int *)calloc((size_t)rowsz(b), sizeof(int));
    if (!b->owner || !b->priority || !b->offsets || !b->targets || !b->strat || !b->infinite || !b->solved ||
        !b->done || !b->bf_inf || !b->succ || !b->stack || !b->vals || !b->zero_val || !b->tmp) {
        bf_destroy(b);
        return NULL;
    }
    memcpy(b->owner, owner, sizeof(int) * n);
    memcpy(b->priority, priority, sizeof(int) * n);
    memcpy(b->offsets, offsets, sizeof(int) * (n + 1));
    if (b->m > 0) memcpy(b->targets, targets, sizeof(int) * b->m);
    for (int v = 0; v < n; v++) b->bf_inf[v] = 1;   /* cpu_bf.cpp:14 */
    return b;
}

void bf_destroy(bf_t *b)
{
    if (!b) return;
    free(b->owner);
    free(b->priority);
    free(b->offsets);
    free(b->targets);
    free(b->strat);
    free(b->infinite);
    free(b->solved);
    free(b->done);
    free(b->bf_inf);
    free(b->succ);
    free(b->stack);
    free(b->vals);
    free(b->zero_val);
    free(b->tmp);
    free(b);
}

int bf_max_pri(const bf_t *b) { return b->max_pri; }

/* cpu_bv.cpp:220-230 (on a fresh solver: the reference appends to strat) */
void bf_init_strat(bf_t *b)
{
    for (int v = 0; v < b->n; v++) b->strat[v] = (b->owner[v] == 0) ? -1 : b->targets[b->offsets[v]];
}

/* ArrayVal::copy_and_add (valuation.cpp:48-53): dst = src + the priority of v.
 * src may be dst. */
static void copy_and_add(const bf_t *b, int *dst, const int *src, int v)
{
    if (dst != src) memcpy(dst, src, sizeof(int) * rowsz(b));
    dst[b->priority[v]] += 1;
}

/* ArrayVal::compare_valuation (valuation.cpp:70-115): +1 if a is better for
 * Even, -1 if worse, 0 if equal. */
static int compare_rows(const bf_t *b, const int *a, const int *c)
{
    for (int64_t p = rowsz(b) - 1; p >= 0; p--) {
        if (a[p] == c[p]) continue;
        if (p % 2 == 0) return a[p] > c[p] ? 1 : -1;
        return a[p] < c[p] ? 1 : -1;
    }
    return 0;
}

/* CPUBV::even_cycle (cpu_bv.cpp:29-48): v lies on a cycle of the strategy. */
static int even_cycle(const bf_t *b, int v)
{
    int cur = v, maxpri = 0;
    for (;;) {
        cur = b->strat[cur];
        if (b->priority[cur] > maxpri) maxpri = b->priority[cur];
        if (cur == v) break;
    }
    return maxpri % 2 == 0;
}

/* Valuation of a vertex y whose successor nx is done (the tail of
 * cpu_bv.cpp:97-108). */
static void take_from_successor(bf_t *b, int y, int nx)
{
    if (b->infinite[nx] != 0) b->infinite[y] = b->infinite[nx];
    else copy_and_add(b, row(b, y), row(b, nx), y);
    b->done[y] = 2;
}

/* CPUBV::compute_valuation(v) (cpu_bv.cpp:50-109) as a walk along the
 * strategy until a vertex whose valuation is known (or a cycle), then an
 * unwind assigning each vertex on the walk from its successor. */
static int valuation_from(bf_t *b, int v)
{
    int top = 0, x = v;
    for (;;) {
        if (b->infinite[x] == 1) {   /* cpu_bv.cpp:57-61 */
            b->done[x] = 2;
            break;
        }
        if (b->strat[x] == -1) {   /* cpu_bv.cpp:63-69 */
            int *r = row(b, x);
            memset(r, 0, sizeof(int) * rowsz(b));
            r[b->priority[x]] = 1;
            b->done[x] = 2;
            break;
        }
        const int nx = b->strat[x];
        if (b->done[nx] == 1) {   /* cpu_bv.cpp:73-86: a cycle closes at x */
            if (!even_cycle(b, x)) return BF_ODD_CYCLE;
            b->infinite[x] = 1;
            b->done[x] = 2;
            break;
        }
        if (b->done[nx] == 0) {   /* cpu_bv.cpp:89-93: recurse */
            b->done[x] = 1;
            b->stack[top++] = x;
            x = nx;
            continue;
        }
        take_from_successor(b, x, nx);
        break;
    }
    while (top > 0) {
        const int y = b->stack[--top];
        take_from_successor(b, y, b->strat[y]);
    }
    return BF_OK;
}

/* CPUBV::compute_valuation() (cpu_bv.cpp:111-127) */
int bf_compute_valuation(bf_t *b)
{
    for (int i = 0; i < b->n; i++) {
        if (!b->solved[i]) {
            b->done[i] = 0;
            b->infinite[i] = 0;
        } else {
            b->done[i] = 2;
        }
    }
    for (int i = 0; i < b->n; i++)
        if (!b->done[i]) {
            int rc = valuation_from(b, i);
            if (rc != BF_OK) return rc;
        }
    return BF_OK;
}

/* CPUBV::mark_solved (cpu_bv.cpp:208-218) */
void bf_mark_solved(bf_t *b, int player)
{
    for (int i = 0; i < b->n; i++) {
        if (player == 0 && b->infinite[i] == 1) b->solved[i] = 1;
        else if (player == 1 && b->infinite[i] == -1) b->solved[i] = 1;
    }
}

/* CPUBV::compare_valuation (cpu_bv.cpp:140-174); -1 is the sink */
static int compare(const bf_t *b, int v, int u)
{
    const int iv = (v != -1) ? b->infinite[v] : 0, iu = (u != -1) ? b->infinite[u] : 0;
    if (iv && iu) {
        if (iv == 1 && iu == -1) return 1;
        if (iv == -1 && iu == 1) return -1;
        return 0;
    }
    if (iv) return iv == 1 ? 1 : -1;
    if (iu) return iu == 1 ? -1 : 1;
    return compare_rows(b, v == -1 ? b->zero_val : row(b, v), u == -1 ? b->zero_val : row(b, u));
}

/* CPUBV::switch_vertex / switch_strategy (cpu_bv.cpp:176-206) */
int64_t bf_switch_strategy(bf_t *b, int player)
{
    int64_t total = 0;
    for (int v = 0; v < b->n; v++) {
        if (b->owner[v] != player) continue;
        int cur = b->strat[v];
        for (int e = b->offsets[v]; e < b->offsets[v + 1]; e++) {
            const int u = b->targets[e];
            const int c = compare(b, u, cur);
            if ((player == 0 && c == 1) || (player == 1 && c == -1)) {
                b->strat[v] = u;
                cur = u;
                total++;
            }
        }
    }
    return total;
}

/* CPU_BellmanFord::best_response_alg (cpu_bf.cpp:51-160), without negative
 * cycle detection (the reference passes false). */
static void relax(bf_t *b, int *br_count)
{
    const int n = b->n;
    const int64_t d = rowsz(b);
    memset(b->vals, 0, sizeof(int) * (size_t)n * (size_t)d);   /* cpu_bf.cpp:57-61 */
    for (int i = 0; i < n; i++) {
        (*br_count)++;
        int done = 1;
        for (int v = 0; v < n; v++) {
            if (b->solved[v]) continue;
            if (b->owner[v] == 0) {   /* cpu_bf.cpp:75-103: follow the strategy */
                const int u = b->strat[v];
                if (u != -1 && b->bf_inf[u]) continue;
                if (b->bf_inf[v]) {
                    b->bf_inf[v] = 0;
                    done = 0;
                }
                copy_and_add(b, b->tmp, u == -1 ? b->zero_val : row(b, u), v);
                if (memcmp(row(b, v), b->tmp, sizeof(int) * d) != 0) {
                    memcpy(row(b, v), b->tmp, sizeof(int) * d);
                    done = 0;
                }
                continue;
            }
            for (int e = b->offsets[v]; e < b->offsets[v + 1]; e++) {   /* cpu_bf.cpp:106-141 */
                const int u = b->targets[e];
                if (u != -1 && b->bf_inf[u]) continue;
                if (b->bf_inf[v]) {
                    copy_and_add(b, b->tmp, u != -1 ? row(b, u) : b->zero_val, v);
                    memcpy(row(b, v), b->tmp, sizeof(int) * d);
                    b->bf_inf[v] = 0;
                    b->succ[v] = u;
                    done = 0;
                    continue;
                }
                copy_and_add(b, b->tmp, row(b, u), v);
                if (compare_rows(b, row(b, v), b->tmp) == 1) {
                    memcpy(row(b, v), b->tmp, sizeof(int) * d);
                    b->succ[v] = u;
                    done = 0;
                }
            }
        }
        if (done) break;
    }
    for (int v = 0; v < n; v++) {   /* cpu_bf.cpp:150-159 */
        if (b->bf_inf[v] && !b->solved[v]) b->infinite[v] = 1;
        if (b->owner[v] == 1) b->strat[v] = b->succ[v];
    }
}

/* CPU_BellmanFord::best_response (cpu_bf.cpp:24-49) */
int bf_best_response(bf_t *b, int *br_count)
{
    if (!b->init) {   /* the first best response: Odd's improvement loop, uncounted */
        for (;;) {
            int rc = bf_compute_valuation(b);
            if (rc != BF_OK) return rc;
            bf_mark_solved(b, 1);
            if (bf_switch_strategy(b, 1) == 0) break;
        }
        b->init = 1;
        return BF_OK;
    }
    for (int v = 0; v < b->n; v++) b->bf_inf[v] = 1;
    relax(b, br_count);
    return BF_OK;
}

/* solve_bf (main.cpp:58-76) */
int bf_solve(bf_t *b, int *iter_count, int *br_count, int max_iters)
{
    *iter_count = 0;
    *br_count = 0;
    bf_init_strat(b);
    for (;;) {
        int rc = bf_best_response(b, br_count);
        if (rc != BF_OK) return rc;
        bf_mark_solved(b, 0);
        (*iter_count)++;
        if (bf_switch_strategy(b, 0) == 0) break;
        if (max_iters > 0 && *iter_count >= max_iters) break;
    }
    return BF_OK;
}

/* CPUBV::get_winning (cpu_bv.cpp:232-241) */
int64_t bf_get_winning(const bf_t *b, int player, int *out)
{
    int64_t k = 0;
    for (int i = 0; i < b->n; i++)
        if ((player == 0) ? b->infinite[i] == 1 : b->infinite[i] != 1) out[k++] = i;
    return k;
}

void bf_get_strategy(const bf_t *b, int *out) { memcpy(out, b->strat, sizeof(int) * b->n); }
void bf_get_infinite(const bf_t *b, int *out) { memcpy(out, b->infinite, sizeof(int) * b->n); }
void bf_get_solved(const bf_t *b, int *out) { memcpy(out, b->solved, sizeof(int) * b->n); }

void bf_get_vals(const bf_t *b, int v0, int count, int *out)
{
    memcpy(out, row(b, v0), sizeof(int) * (size_t)count * (size_t)rowsz(b));
}
