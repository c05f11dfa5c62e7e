/*
 * psi_sparse.c -- exact CPU restatement of the reference strategy-improvement
 * solver, with valuations kept as strategy paths instead of dense rows.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a parity oracle: the tests, the smoke
 * check and the CPU legs of bench.py call it to check or to time against the
 * CUDA path.  No product code path links, loads or falls back to it.
 *
 * It computes what the reference's CPUParity (cpu_parity.cpp) computes, step
 * for step, under the solve_si driver (main.cpp:20-55):
 *
 *   - compute_valuation (cpu_parity.cpp:54-133): the valuation of a vertex is
 *     the multiset of priorities on its strategy path to the virtual sink; a
 *     path that ends in a cycle is +inf/-inf by the parity of the cycle's top
 *     priority (cpu_parity.cpp:35-52, 80-89); a path into a solved vertex takes
 *     its frozen value (cpu_parity.cpp:98-104, 116-127);
 *   - compare_valuation (cpu_parity.cpp:154-236): the highest priority whose
 *     counts differ decides, the larger count winning at an even priority and
 *     the smaller at an odd one; +inf > finite > -inf;
 *   - switch_strategy (cpu_parity.cpp:239-263): successors in CSR order, the
 *     running choice replaced only on a strict improvement, every replacement
 *     counted;
 *   - mark_solved, get_winning, init_strat, reset_opponent_strategy
 *     (cpu_parity.cpp:265-307).
 *
 * Where CPUParity keeps one dense row of max_pri+1 counts per vertex (n*(d+1)
 * ints: 2^48 of them for 2^24 vertices with priorities up to 2^24), this
 * restatement keeps, per vertex, the path itself (the strategy snapshot of the
 * last evaluation), its length, and its top priority with that priority's
 * count.  Two finite valuations compare by those summaries when they differ;
 * otherwise both paths are walked up to their lowest common ancestor (the
 * common part cancels), the two remaining priority lists are sorted, and the
 * counts compared from the highest priority down.  That is the reference's
 * row comparison restricted to the rows' difference, so the results are
 * identical; tests/test_sparse_oracle.py checks it against the dense
 * restatement and the reference's own solves step by step.
 *
 * The evaluation builds the children lists of the sink tree (counts and
 * fills with atomic increments), walks every subtree of the sink from the
 * sink's children without a stack (each vertex keeps its next-child cursor),
 * and resolves the vertices the sink does not reach by one memoised walk each.
 * Evaluation passes and the switch step run on `threads` POSIX threads over
 * vertex ranges handed out from an atomic counter.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "psi_sparse.h"

struct sparse {
    int n, threads, max_pri;
    int64_t m;
    int8_t *owner;
    int *priority, *offsets, *targets;
    int *strat;
    int8_t *inf;      /* +1 / -1 / 0 as CPUParity's infinite[] */
    uint8_t *solved;
    /* snapshot of the last evaluation, per vertex the sink reaches */
    int *parent;      /* strategy at evaluation time (-1 = the sink) */
    int *depth;       /* path length to the sink, 0 if not reached */
    int *top, *cnt;   /* highest priority on the path, its count */
    /* children lists of the sink tree; index n is the sink */
    int *coff;        /* n+2 */
    int *cur;         /* n+1: fill cursor, then the traversal's next-child cursor */
    int *child;       /* n */
    uint8_t *mark;    /* cycle resolution: 0 open, 1 on the current walk, 2 done */
    int *walk;        /* n: the current walk */
};

/* ------------------------------------------------------------ threads */

/* f(o, a, b, scratch, arg, acc) handles items [a, b); *scratch is a pointer
 * the worker keeps across its chunks (NULL at first), released with
 * `release` when the worker ends; *acc is the worker's running sum. */
typedef void (*range_fn)(sparse_t *o, int64_t a, int64_t b, void **scratch, void *arg, int64_t *acc);

struct par_job {
    sparse_t *o;
    range_fn f;
    void *arg;
    void (*release)(void *);
    int64_t total, chunk;
    int64_t next;     /* atomic */
};

struct par_worker {
    struct par_job *job;
    int64_t acc;
};

static void *par_run(void *p)
{
    struct par_worker *w = (struct par_worker *)p;
    struct par_job *j = w->job;
    void *scratch = NULL;
    w->acc = 0;
    for (;;) {
        int64_t a = __atomic_fetch_add(&j->next, j->chunk, __ATOMIC_RELAXED);
        if (a >= j->total) break;
        int64_t b = a + j->chunk < j->total ? a + j->chunk : j->total;
        j->f(j->o, a, b, &scratch, j->arg, &w->acc);
    }
    if (scratch && j->release) j->release(scratch);
    return NULL;
}

/* Runs f over [0, total) in chunks on o->threads threads; returns the sum of
 * what the calls added to their accumulators. */
static int64_t par_for(sparse_t *o, int64_t total, int64_t chunk, range_fn f, void *arg,
                       void (*release)(void *))
{
    struct par_job job = {o, f, arg, release, total, chunk > 0 ? chunk : 1, 0};
    int t = o->threads;
    if ((int64_t)t * job.chunk > total) t = (int)((total + job.chunk - 1) / job.chunk);
    if (t < 1) t = 1;
    struct par_worker w[256];
    pthread_t th[256];
    if (t > 256) t = 256;
    for (int i = 0; i < t; i++) w[i].job = &job;
    int started = 0;
    for (int i = 1; i < t; i++) {
        if (pthread_create(&th[i], NULL, par_run, &w[i]) != 0) break;
        started = i;
    }
    par_run(&w[0]);
    int64_t sum = w[0].acc;
    for (int i = 1; i <= started; i++) {
        pthread_join(th[i], NULL);
        sum += w[i].acc;
    }
    return sum;
}

/* ------------------------------------------------------------ set-up */

sparse_t *sparse_create(int n, const int *owner, const int *priority, const int *offsets, const int *targets,
                        int threads)
{
    if (n < 0) return NULL;
    sparse_t *o = (sparse_t *)calloc(1, sizeof(sparse_t));
    if (!o) return NULL;
    const size_t n1 = n > 0 ? (size_t)n : 1;
    o->n = n;
    o->m = offsets[n];
    if (threads <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        threads = c > 0 ? (int)c : 1;
    }
    o->threads = threads > 256 ? 256 : threads;
    int mp = 0;
    for (int v = 0; v < n; v++)
        if (priority[v] > mp) mp = priority[v];
    o->max_pri = mp;
    o->owner = (int8_t *)malloc(n1);
    o->priority = (int *)malloc(sizeof(int) * n1);
    o->offsets = (int *)malloc(sizeof(int) * (n1 + 1));
    o->targets = (int *)malloc(sizeof(int) * (o->m > 0 ? (size_t)o->m : 1));
    o->strat = (int *)calloc(n1, sizeof(int));
    o->inf = (int8_t *)calloc(n1, 1);
    o->solved = (uint8_t *)calloc(n1, 1);
    o->parent = (int *)calloc(n1, sizeof(int));
    o->depth = (int *)calloc(n1, sizeof(int));
    o->top = (int *)calloc(n1, sizeof(int));
    o->cnt = (int *)calloc(n1, sizeof(int));
    o->coff = (int *)calloc(n1 + 2, sizeof(int));
    o->cur = (int *)calloc(n1 + 1, sizeof(int));
    o->child = (int *)calloc(n1, sizeof(int));
    o->mark = (uint8_t *)calloc(n1, 1);
    o->walk = (int *)calloc(n1, sizeof(int));
    if (!o->owner || !o->priority || !o->offsets || !o->targets || !o->strat || !o->inf || !o->solved ||
        !o->parent || !o->depth || !o->top || !o->cnt || !o->coff || !o->cur || !o->child || !o->mark ||
        !o->walk) {
        sparse_destroy(o);
        return NULL;
    }
    for (int v = 0; v < n; v++) o->owner[v] = (int8_t)owner[v];
    memcpy(o->priority, priority, sizeof(int) * (size_t)n);
    memcpy(o->offsets, offsets, sizeof(int) * ((size_t)n + 1));
    if (o->m > 0) memcpy(o->targets, targets, sizeof(int) * (size_t)o->m);
    return o;
}

void sparse_destroy(sparse_t *o)
{
    if (!o) return;
    free(o->owner); free(o->priority); free(o->offsets); free(o->targets);
    free(o->strat); free(o->inf); free(o->solved); free(o->parent); free(o->depth);
    free(o->top); free(o->cnt); free(o->coff); free(o->cur); free(o->child);
    free(o->mark); free(o->walk);
    free(o);
}

int sparse_max_pri(const sparse_t *o) { return o->max_pri; }
int sparse_threads(const sparse_t *o) { return o->threads; }

/* cpu_parity.cpp:276-286; like a fresh CPUParity, nothing is solved
 * (cpu_parity.cpp:20-33) */
void sparse_init_strat(sparse_t *o)
{
    for (int v = 0; v < o->n; v++) {
        o->strat[v] = (o->owner[v] == 0) ? -1 : o->targets[o->offsets[v]];
        o->solved[v] = 0;
        o->inf[v] = 0;
    }
}

/* cpu_parity.cpp:300-307 */
void sparse_reset_opponent_strategy(sparse_t *o)
{
    for (int v = 0; v < o->n; v++)
        if (o->owner[v] == 1) o->strat[v] = o->targets[o->offsets[v]];
}

/* ------------------------------------------------------------ evaluation */

/* The sink-tree parent slot of a non-solved vertex: n for the sink, -1 when
 * its successor is solved (it takes the solved vertex's value instead). */
static inline int tree_slot(const sparse_t *o, int v)
{
    int p = o->strat[v];
    if (p < 0) return o->n;
    return o->solved[p] ? -1 : p;
}

static void ev_clear(sparse_t *o, int64_t a, int64_t b, void **s, void *arg, int64_t *acc)
{
    (void)s; (void)arg; (void)acc;
    for (int64_t v = a; v < b; v++) {
        o->cur[v] = 0;
        o->coff[v] = 0;
        if (!o->solved[v]) {
            o->inf[v] = 0;
            o->depth[v] = 0;
            o->mark[v] = 0;
        }
    }
}

static void ev_count(sparse_t *o, int64_t a, int64_t b, void **s, void *arg, int64_t *acc)
{
    (void)s; (void)arg; (void)acc;
    for (int64_t v = a; v < b; v++) {
        if (o->solved[v]) continue;
        int p = tree_slot(o, (int)v);
        if (p >= 0) __atomic_fetch_add(&o->coff[p + 1], 1, __ATOMIC_RELAXED);
    }
}

static void ev_fill(sparse_t *o, int64_t a, int64_t b, void **s, void *arg, int64_t *acc)
{
    (void)s; (void)arg; (void)acc;
    for (int64_t v = a; v < b; v++) {
        if (o->solved[v]) continue;
        int p = tree_slot(o, (int)v);
        if (p >= 0) o->child[o->coff[p] + __atomic_fetch_add(&o->cur[p], 1, __ATOMIC_RELAXED)] = (int)v;
    }
}

/* Valuation summary of y from its parent x (x == -1: the sink). */
static inline void visit(sparse_t *o, int y, int x)
{
    const int p = o->priority[y];
    o->parent[y] = x;
    if (x < 0) {
        o->depth[y] = 1;
        o->top[y] = p;
        o->cnt[y] = 1;
    } else {
        o->depth[y] = o->depth[x] + 1;
        if (p > o->top[x]) {
            o->top[y] = p;
            o->cnt[y] = 1;
        } else {
            o->top[y] = o->top[x];
            o->cnt[y] = o->cnt[x] + (p == o->top[x]);
        }
    }
}

/* Subtrees of the sink's children [a, b) of its list, each traversed without
 * a stack: cur[x] is x's next child to visit, parent[] leads back up. */
static void ev_subtrees(sparse_t *o, int64_t a, int64_t b, void **s, void *arg, int64_t *acc)
{
    (void)s; (void)arg; (void)acc;
    const int base = o->coff[o->n];
    for (int64_t i = a; i < b; i++) {
        const int root = o->child[base + i];
        visit(o, root, -1);
        o->cur[root] = o->coff[root];
        int x = root;
        for (;;) {
            if (o->cur[x] < o->coff[x + 1]) {
                const int y = o->child[o->cur[x]++];
                visit(o, y, x);
                o->cur[y] = o->coff[y];
                x = y;
            } else {
                if (x == root) break;
                x = o->parent[x];
            }
        }
    }
}

/* cpu_parity.cpp:35-52: the parity of the top priority on the cycle through v */
static int even_cycle(const sparse_t *o, int v)
{
    int c = v, mx = 0;
    for (;;) {
        c = o->strat[c];
        if (o->priority[c] > mx) mx = o->priority[c];
        if (c == v) break;
    }
    return mx % 2 == 0;
}

/* The vertices the sink does not reach: each walk follows the strategy to a
 * solved vertex, to a vertex already resolved, or around a cycle, and gives
 * every vertex on it that value (cpu_parity.cpp:80-104). */
static void ev_unreached(sparse_t *o)
{
    for (int v = 0; v < o->n; v++) {
        if (o->solved[v] || o->depth[v] > 0 || o->mark[v] == 2) continue;
        int k = 0, x = v, val = 0;
        o->mark[x] = 1;
        o->walk[k++] = x;
        for (;;) {
            const int nx = o->strat[x];   /* >= 0: a vertex pointing at the sink is reached */
            if (o->solved[nx] || o->mark[nx] == 2) {
                val = o->inf[nx];
                break;
            }
            if (o->mark[nx] == 1) {
                val = even_cycle(o, x) ? 1 : -1;
                break;
            }
            o->mark[nx] = 1;
            o->walk[k++] = nx;
            x = nx;
        }
        while (k > 0) {
            const int y = o->walk[--k];
            o->inf[y] = (int8_t)val;
            o->mark[y] = 2;
        }
    }
}

/* cpu_parity.cpp:116-133 */
void sparse_compute_valuation(sparse_t *o)
{
    const int n = o->n;
    if (n == 0) return;
    o->cur[n] = 0;
    o->coff[n] = o->coff[n + 1] = 0;
    par_for(o, n, 1 << 14, ev_clear, NULL, NULL);
    par_for(o, n, 1 << 14, ev_count, NULL, NULL);
    /* exclusive prefix sum over the n+1 slots (the sink last) */
    int64_t run = 0;
    for (int i = 0; i <= n; i++) {
        const int c = o->coff[i + 1];
        o->coff[i] = (int)run;
        run += c;
    }
    o->coff[n + 1] = (int)run;
    par_for(o, n, 1 << 14, ev_fill, NULL, NULL);
    const int64_t roots = o->coff[n + 1] - o->coff[n];
    par_for(o, roots, 64, ev_subtrees, NULL, NULL);
    ev_unreached(o);
}

/* ------------------------------------------------------------ comparison */

struct walk_buf {
    int *a, *b;
    int64_t cap;
};

static int cmp_desc(const void *x, const void *y)
{
    const int a = *(const int *)x, b = *(const int *)y;
    return (a < b) - (a > b);
}

/* Decides at priority p where u has cu and w has cw (cu != cw): 1 if u is
 * better for Even (cpu_parity.cpp:154-192). */
static inline int decide(int p, int cu, int cw)
{
    if (p % 2 == 0) return cu > cw ? 1 : -1;
    return cu < cw ? 1 : -1;
}

/* Finite u != w (either may be -1, the sink) with equal summaries: walk both
 * paths to their lowest common ancestor and compare what lies below it. */
static int compare_paths(const sparse_t *o, int u, int w, struct walk_buf *buf)
{
    int du = u < 0 ? 0 : o->depth[u], dw = w < 0 ? 0 : o->depth[w];
    const int64_t need = (int64_t)du + dw + 2;
    if (need > buf->cap) {
        int64_t c = buf->cap ? buf->cap : 256;
        while (c < need) c *= 2;
        free(buf->a);
        free(buf->b);
        buf->a = (int *)malloc(sizeof(int) * (size_t)c);
        buf->b = (int *)malloc(sizeof(int) * (size_t)c);
        buf->cap = c;
    }
    int na = 0, nb = 0;
    while (du > dw) {
        buf->a[na++] = o->priority[u];
        u = o->parent[u];
        du--;
    }
    while (dw > du) {
        buf->b[nb++] = o->priority[w];
        w = o->parent[w];
        dw--;
    }
    while (u != w) {
        buf->a[na++] = o->priority[u];
        u = o->parent[u];
        buf->b[nb++] = o->priority[w];
        w = o->parent[w];
    }
    qsort(buf->a, (size_t)na, sizeof(int), cmp_desc);
    qsort(buf->b, (size_t)nb, sizeof(int), cmp_desc);
    int i = 0, j = 0;
    while (i < na || j < nb) {
        const int pa = i < na ? buf->a[i] : -1, pb = j < nb ? buf->b[j] : -1;
        const int p = pa > pb ? pa : pb;
        int ca = 0, cb = 0;
        while (i < na && buf->a[i] == p) { ca++; i++; }
        while (j < nb && buf->b[j] == p) { cb++; j++; }
        if (ca != cb) return decide(p, ca, cb);
    }
    return 0;
}

/* cpu_parity.cpp:194-236: 1 if v is better for Even than u, 0 if equal, -1 if
 * worse; -1 denotes the sink. */
static int compare_with(const sparse_t *o, int v, int u, struct walk_buf *buf)
{
    const int iv = (v != -1) ? o->inf[v] : 0;
    const int iu = (u != -1) ? o->inf[u] : 0;
    if (v != -1 && u != -1 && iv && iu) {
        if (iv == 1 && iu == -1) return 1;
        if (iv == -1 && iu == 1) return -1;
        return 0;
    }
    if (iv) return iv == 1 ? 1 : -1;
    if (iu) return iu == 1 ? -1 : 1;
    if (v == u) return 0;
    const int tv = v < 0 ? -1 : o->top[v], cv = v < 0 ? 0 : o->cnt[v];
    const int tu = u < 0 ? -1 : o->top[u], cu = u < 0 ? 0 : o->cnt[u];
    if (tv != tu) return tv > tu ? decide(tv, cv, 0) : decide(tu, 0, cu);
    if (cv != cu) return decide(tv, cv, cu);
    return compare_paths(o, v, u, buf);
}

int sparse_compare(const sparse_t *o, int v, int u)
{
    struct walk_buf buf = {NULL, NULL, 0};
    const int r = compare_with(o, v, u, &buf);
    free(buf.a);
    free(buf.b);
    return r;
}

/* ------------------------------------------------------------ switching */

static void walk_buf_release(void *p)
{
    struct walk_buf *buf = (struct walk_buf *)p;
    free(buf->a);
    free(buf->b);
    free(buf);
}

static void sw_range(sparse_t *o, int64_t a, int64_t b, void **scratch, void *arg, int64_t *acc)
{
    const int player = *(const int *)arg;
    if (!*scratch) *scratch = calloc(1, sizeof(struct walk_buf));
    struct walk_buf *buf = (struct walk_buf *)*scratch;
    int64_t total = 0;
    for (int64_t v = a; v < b; v++) {
        if (o->owner[v] != player) continue;
        int cur = o->strat[v];
        for (int e = o->offsets[v]; e < o->offsets[v + 1]; e++) {
            const int u = o->targets[e];
            const int c = compare_with(o, u, cur, buf);
            if ((player == 0 && c == 1) || (player == 1 && c == -1)) {
                cur = u;
                total++;
            }
        }
        o->strat[v] = cur;
    }
    *acc += total;
}

/* cpu_parity.cpp:239-263: returns the number of replacements.  The walks of
 * the comparisons read the evaluation's snapshot (parent[]), never the
 * strategies this step is changing. */
int64_t sparse_switch_strategy(sparse_t *o, int player)
{
    return par_for(o, o->n, 4096, sw_range, &player, walk_buf_release);
}

/* cpu_parity.cpp:265-274 */
void sparse_mark_solved(sparse_t *o, int player)
{
    for (int v = 0; v < o->n; v++) {
        if (player == 0 && o->inf[v] == 1) o->solved[v] = 1;
        else if (player == 1 && o->inf[v] == -1) o->solved[v] = 1;
    }
}

/* cpu_parity.cpp:288-297 */
int64_t sparse_get_winning(const sparse_t *o, int player, int *out)
{
    int64_t k = 0;
    for (int v = 0; v < o->n; v++) {
        const int w0 = (o->inf[v] == 1);
        if ((player == 0 && w0) || (player == 1 && !w0)) {
            if (out) out[k] = v;
            k++;
        }
    }
    return k;
}

void sparse_get_strategy(const sparse_t *o, int *out) { memcpy(out, o->strat, sizeof(int) * (size_t)o->n); }
void sparse_set_strategy(sparse_t *o, const int *in) { memcpy(o->strat, in, sizeof(int) * (size_t)o->n); }

void sparse_get_infinite(const sparse_t *o, int *out)
{
    for (int v = 0; v < o->n; v++) out[v] = o->inf[v];
}

void sparse_get_solved(const sparse_t *o, int *out)
{
    for (int v = 0; v < o->n; v++) out[v] = o->solved[v];
}

void sparse_get_summary(const sparse_t *o, int *depth, int *top, int *count)
{
    for (int v = 0; v < o->n; v++) {
        const int fin = !o->inf[v] && o->depth[v] > 0;
        if (depth) depth[v] = fin ? o->depth[v] : 0;
        if (top) top[v] = fin ? o->top[v] : -1;
        if (count) count[v] = fin ? o->cnt[v] : 0;
    }
}

void sparse_get_vals(const sparse_t *o, int v0, int count, int *out)
{
    const int64_t d = (int64_t)o->max_pri + 1;
    memset(out, 0, sizeof(int) * (size_t)count * (size_t)d);
    for (int i = 0; i < count; i++) {
        int v = v0 + i;
        if (o->inf[v] || o->depth[v] == 0) continue;
        int *row = out + (int64_t)i * d;
        for (int x = v; x >= 0; x = o->parent[x]) row[o->priority[x]]++;
    }
}

/* main.cpp:20-55 (solve_si); reset != 0 is the "cpu-reset" variant
 * (main.cpp:27-28).  Returns 0, or -1 when max_evals evaluations were reached. */
int sparse_solve(sparse_t *o, int reset, int *iter_count, int *br_count, int64_t max_evals)
{
    int iters = 0, brs = 0, first = 1, rc = 0;
    sparse_init_strat(o);
    for (;;) {
        if (!first && reset) sparse_reset_opponent_strategy(o);
        for (;;) {
            sparse_compute_valuation(o);
            brs++;
            sparse_mark_solved(o, 1);
            if (sparse_switch_strategy(o, 1) == 0) break;
            if (max_evals > 0 && brs >= max_evals) { rc = -1; goto out; }
        }
        first = 0;
        sparse_mark_solved(o, 0);
        iters++;
        if (sparse_switch_strategy(o, 0) == 0) break;
        if (max_evals > 0 && brs >= max_evals) { rc = -1; goto out; }
    }
out:
    *iter_count = iters;
    *br_count = brs;
    return rc;
}
