// check.cpp -- independent certificate check of a solved parity game.
//
// A solution is a partition of the vertices into W0 (Even wins) and W1 (Odd
// wins) with a positional strategy for each player.  It is correct iff
//   (1) every strategy entry is a successor of its vertex;
//   (2) W0 is closed under Even's strategy and a trap for Odd (every Odd vertex
//       of W0 has all its successors in W0); W1 likewise with the roles
//       swapped;
//   (3) in the graph G0 on W0 where Even's vertices keep only their strategy
//       edge and Odd's keep all edges, every cycle has an even top priority;
//       in G1 on W1 (Odd's strategy fixed, Even's edges all kept) every cycle
//       has an odd top priority.
// (2) and (3) together make each strategy winning on its region against every
// counter-strategy, so the regions are the winning regions.  Checks (1) and
// (2) take O(n + m) and run on several threads.  Check (3) decomposes each
// graph into strongly connected components: a component with a cycle whose
// top priority has the wrong parity is a violation; otherwise its vertices of
// that top priority are removed and the rest is decomposed again.  Every
// round removes at least one vertex, so it ends, but games whose components
// shrink slowly cost up to O(n * m); the caller bounds the edge visits and
// gets "incomplete" past the bound.
//
// The strategies and regions are the solver's own outputs (get_strategy,
// get_infinite); no counterpart exists in the reference, which reports only
// counts and prints the winning sets (gpumain.cpp:18-53).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

#include "check.h"
#include "game.h"
#include "psi.h"
#include "psi_internal.h"

namespace psi {

namespace {

struct Violation {
    std::mutex mu;
    int32_t kind = PSI_CHECK_OK;
    int64_t vertex = -1;
    void report(int32_t k, int64_t v)
    {
        std::lock_guard<std::mutex> lk(mu);
        if (vertex < 0 || v < vertex) {
            kind = k;
            vertex = v;
        }
    }
};

bool is_successor(const CsrView &g, int32_t v, int32_t t)
{
    for (int32_t e = g.offsets[v]; e < g.offsets[v + 1]; e++)
        if (g.targets[e] == t) return true;
    return false;
}

// One cycle-parity check: vertices in[v] != 0 form the graph; fixed[v] = the
// only successor of a vertex whose owner's strategy is fixed there, or -1 to
// keep all its edges.  bad_parity: the parity of a top priority that is a
// violation.  Returns PSI_CHECK_OK, PSI_CHECK_BAD_CYCLE (its top vertex in
// *where) or PSI_CHECK_INCOMPLETE once `budget` edge visits are spent.
int32_t cycle_check(const CsrView &g, const std::vector<uint8_t> &in, const std::vector<int32_t> &fixed,
                    int32_t bad_parity, int64_t &budget, int64_t *where)
{
    const int32_t n = g.n;
    std::vector<uint8_t> alive(in.begin(), in.end()), on_stack(n);
    std::vector<int32_t> setid(n, -1), index(n, -1), low(n);
    std::vector<int32_t> stack, frame_v, frame_e, members;
    std::vector<std::vector<int32_t>> work;   // vertex sets still to decompose
    {
        std::vector<int32_t> all;
        for (int32_t v = 0; v < n; v++)
            if (alive[v]) all.push_back(v);
        if (!all.empty()) work.push_back(std::move(all));
    }
    int32_t sid = 0;
    while (!work.empty()) {
        const std::vector<int32_t> set = std::move(work.back());
        work.pop_back();
        ++sid;
        for (int32_t v : set) {
            setid[v] = sid;
            index[v] = -1;
            on_stack[v] = 0;
        }
        // an edge counts only inside the set being decomposed
        auto inside = [&](int32_t u) { return u >= 0 && setid[u] == sid && alive[u]; };
        int32_t counter = 0;
        for (int32_t root : set) {
            if (index[root] != -1) continue;
            // iterative Tarjan; frame_e is the edge cursor (for a fixed
            // vertex: 0 before and 1 after its one edge)
            index[root] = low[root] = counter++;
            stack.push_back(root);
            on_stack[root] = 1;
            frame_v.push_back(root);
            frame_e.push_back(fixed[root] >= 0 ? 0 : g.offsets[root]);
            while (!frame_v.empty()) {
                const int32_t v = frame_v.back();
                int32_t next = -1;
                for (;;) {
                    int32_t u;
                    if (fixed[v] >= 0) {
                        if (frame_e.back() != 0) break;
                        frame_e.back() = 1;
                        u = fixed[v];
                    } else {
                        if (frame_e.back() >= g.offsets[v + 1]) break;
                        u = g.targets[frame_e.back()++];
                    }
                    if (--budget < 0) return PSI_CHECK_INCOMPLETE;
                    if (!inside(u) || index[u] == -2) continue;   // outside, or in a finished component
                    if (index[u] == -1) {
                        next = u;
                        break;
                    }
                    if (on_stack[u]) low[v] = std::min(low[v], index[u]);
                }
                if (next >= 0) {
                    index[next] = low[next] = counter++;
                    stack.push_back(next);
                    on_stack[next] = 1;
                    frame_v.push_back(next);
                    frame_e.push_back(fixed[next] >= 0 ? 0 : g.offsets[next]);
                    continue;
                }
                frame_v.pop_back();
                frame_e.pop_back();
                if (!frame_v.empty()) low[frame_v.back()] = std::min(low[frame_v.back()], low[v]);
                if (low[v] != index[v]) continue;
                // the component rooted at v
                members.clear();
                int32_t w;
                do {
                    w = stack.back();
                    stack.pop_back();
                    on_stack[w] = 0;
                    members.push_back(w);
                } while (w != v);
                for (int32_t x : members) index[x] = -2;
                bool cyclic = members.size() > 1;
                if (!cyclic) {   // one vertex is a cycle only through a self-loop
                    const int32_t x = members[0];
                    if (fixed[x] >= 0) {
                        cyclic = fixed[x] == x;
                    } else {
                        for (int32_t f = g.offsets[x]; f < g.offsets[x + 1] && !cyclic; f++) cyclic = g.targets[f] == x;
                    }
                }
                if (!cyclic) continue;
                int32_t top = -1;
                for (int32_t x : members) top = std::max(top, g.priority[x]);
                if ((top & 1) == bad_parity) {
                    int64_t at = -1;
                    for (int32_t x : members)
                        if (g.priority[x] == top && (at < 0 || x < at)) at = x;
                    *where = at;
                    return PSI_CHECK_BAD_CYCLE;
                }
                // cycles through a top vertex are fine; the rest may still hold bad ones
                std::vector<int32_t> rest;
                for (int32_t x : members) {
                    if (g.priority[x] == top) alive[x] = 0;
                    else rest.push_back(x);
                }
                if (!rest.empty()) work.push_back(std::move(rest));
            }
        }
    }
    return PSI_CHECK_OK;
}

}  // namespace

int check_solution(const CsrView &g, const int32_t *strategy, const int32_t *infinite, int64_t work_budget,
                   CheckReport *out)
{
    *out = CheckReport();
    const int32_t n = g.n;
    // (1) strategy entries, (2) closure and traps
    Violation bad;
    parallel_chunks(n, [&](int64_t lo, int64_t hi) {
        for (int64_t v64 = lo; v64 < hi; v64++) {
            const int32_t v = (int32_t)v64;
            const int32_t s = strategy[v];
            const bool w0 = infinite[v] == 1;
            const int32_t owner = g.owner[v];
            if (!(s == -1 && owner == 0) && !(s >= 0 && s < n && is_successor(g, v, s))) {
                bad.report(PSI_CHECK_BAD_STRATEGY, v);
                continue;
            }
            const bool mine = (owner == 0) == w0;   // the owner wins v
            if (mine) {
                // the winner's strategy stays in its region (Even never leaves W0 for the sink)
                if (s < 0 || (infinite[s] == 1) != w0) bad.report(PSI_CHECK_NOT_CLOSED, v);
            } else {
                for (int32_t e = g.offsets[v]; e < g.offsets[v + 1]; e++)
                    if ((infinite[g.targets[e]] == 1) != w0) {
                        bad.report(PSI_CHECK_NOT_TRAP, v);
                        break;
                    }
            }
        }
    });
    if (bad.vertex >= 0) {
        out->status = bad.kind;
        out->vertex = bad.vertex;
        return PSI_OK;
    }
    // (3) cycle parities of G0 (bad: odd top) and G1 (bad: even top)
    std::vector<uint8_t> in0(n), in1(n);
    std::vector<int32_t> fixed0(n, -1), fixed1(n, -1);
    for (int32_t v = 0; v < n; v++) {
        const bool w0 = infinite[v] == 1;
        (w0 ? in0 : in1)[v] = 1;
        if (w0 && g.owner[v] == 0) fixed0[v] = strategy[v];
        if (!w0 && g.owner[v] == 1) fixed1[v] = strategy[v];
    }
    int64_t budget = work_budget > 0 ? work_budget : INT64_MAX;
    int64_t where = -1;
    int32_t r = cycle_check(g, in0, fixed0, 1, budget, &where);
    if (r == PSI_CHECK_OK) r = cycle_check(g, in1, fixed1, 0, budget, &where);
    out->status = r;
    out->vertex = where;
    out->edge_visits = (work_budget > 0 ? work_budget : INT64_MAX) - budget;
    return PSI_OK;
}

}  // namespace psi
