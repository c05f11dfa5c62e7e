// ref_bf_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A thin C driver around the reference's own Bellman-Ford best-response solver
// (CPU_BellmanFord<ArrayVal>, cpu_bf.cpp, on CPUBV, cpu_bv.cpp, with the dense
// valuations of valuation.cpp), compiled with those sources where they lie by
// oracle/build_ref.sh into oracle/_ref/libpsi_refbf.so.  The tests use it to
// pin the C restatement in psi_bf.c and to produce its golden fixtures; it is
// never part of the product.
//
// The class below only widens access to the solver's protected state (strat,
// infinite, solved, vals; cpu_bv.h:15-21) so that each step of solve_bf
// (main.cpp:58-76) can be observed.  Games enter through the reference's own
// .gm parser (Game::parse_pgsolver, game.cpp:51-107).
//
// CPUBV's evaluation ends the whole process (exit(1), cpu_bv.cpp:73-85) when
// a strategy closes a cycle whose top priority is odd.  So a game is accepted
// only if no cycle of its graph has an odd top priority: then no strategy can
// close one, and the reference never exits under a test.
#include <sstream>
#include <string>
#include <vector>
#include <cstring>
#include <functional>
#include <algorithm>
#include <pthread.h>

#include "game.h"
#include "cpu_bf.h"
#include "valuation.h"

namespace {

class ObservedBF : public CPU_BellmanFord<ArrayVal> {
public:
    explicit ObservedBF(Game &g) : CPU_BellmanFord<ArrayVal>(g) {}
    std::vector<int> &strategy() { return this->strat; }
    std::vector<int> &inf() { return this->infinite; }
    std::vector<int> &sol() { return this->solved; }
    ArrayVal &val(int v) { return this->vals[v]; }
};

struct RefBF {
    Game game;
    ObservedBF *solver = nullptr;
};

// CPUBV::compute_valuation recurses once per vertex of a strategy path
// (cpu_bv.cpp:89-93): run such calls on a thread with a 1 GiB stack.
void *trampoline(void *f)
{
    (*static_cast<std::function<void()> *>(f))();
    return nullptr;
}

void with_big_stack(std::function<void()> f)
{
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, (size_t)1 << 30);
    pthread_t t;
    if (pthread_create(&t, &attr, trampoline, &f) != 0) {
        f();
    } else {
        pthread_join(t, nullptr);
    }
    pthread_attr_destroy(&attr);
}

// Strongly connected components of the subgraph induced by `keep`
// (Kosaraju, iterative).  comp[v] = component id, or -1 outside the subgraph.
void components(const std::vector<std::vector<int>> &adj, const std::vector<char> &keep, std::vector<int> &comp)
{
    const int n = (int)adj.size();
    std::vector<std::vector<int>> radj(n);
    for (int v = 0; v < n; v++)
        if (keep[v])
            for (int u : adj[v])
                if (keep[u]) radj[u].push_back(v);
    std::vector<int> order;
    std::vector<char> seen(n, 0);
    std::vector<std::pair<int, size_t>> st;
    for (int s = 0; s < n; s++) {
        if (!keep[s] || seen[s]) continue;
        seen[s] = 1;
        st.push_back({s, 0});
        while (!st.empty()) {
            int v = st.back().first;
            size_t &i = st.back().second;
            if (i < adj[v].size()) {
                int u = adj[v][i++];
                if (keep[u] && !seen[u]) {
                    seen[u] = 1;
                    st.push_back({u, 0});
                }
            } else {
                order.push_back(v);
                st.pop_back();
            }
        }
    }
    comp.assign(n, -1);
    int c = 0;
    std::vector<int> work;
    for (int k = (int)order.size() - 1; k >= 0; k--) {
        int s = order[k];
        if (comp[s] >= 0) continue;
        comp[s] = c;
        work.push_back(s);
        while (!work.empty()) {
            int v = work.back();
            work.pop_back();
            for (int u : radj[v])
                if (comp[u] < 0) {
                    comp[u] = c;
                    work.push_back(u);
                }
        }
        c++;
    }
}

// True if some cycle of the game graph has an odd top priority: for each odd
// priority p, a vertex of priority p on a cycle of the vertices of priority
// at most p.
bool has_odd_cycle(Game &g)
{
    const int n = g.get_n_vertices();
    std::vector<std::vector<int>> adj(n);
    std::vector<int> pris;
    for (int v = 0; v < n; v++) {
        adj[v] = g.get_edges(v);
        if (g.get_priority(v) % 2 == 1) pris.push_back(g.get_priority(v));
    }
    std::sort(pris.begin(), pris.end());
    pris.erase(std::unique(pris.begin(), pris.end()), pris.end());
    std::vector<char> keep(n);
    std::vector<int> comp, size;
    for (int p : pris) {
        for (int v = 0; v < n; v++) keep[v] = g.get_priority(v) <= p;
        components(adj, keep, comp);
        size.assign(n, 0);
        for (int v = 0; v < n; v++)
            if (comp[v] >= 0) size[comp[v]]++;
        for (int v = 0; v < n; v++) {
            if (g.get_priority(v) != p) continue;
            if (size[comp[v]] > 1) return true;
            for (int u : adj[v])
                if (u == v) return true;
        }
    }
    return false;
}

}  // namespace

extern "C" {

// Parses .gm text with the reference parser.  Returns NULL and fills err when
// the parser throws, or when a cycle of the game has an odd top priority (the
// reference solver would exit the process on such a game).
void *ref_bf_create_from_gm(const char *text, char *err, int errlen)
{
    RefBF *h = new RefBF();
    const char *why = nullptr;
    try {
        std::istringstream in(text);
        h->game.parse_pgsolver(in);
    } catch (const char *e) {
        why = e;
    }
    if (!why && has_odd_cycle(h->game)) why = "a cycle of the game has an odd top priority";
    if (why) {
        if (err && errlen > 0) {
            std::strncpy(err, why, errlen - 1);
            err[errlen - 1] = 0;
        }
        delete h;
        return nullptr;
    }
    h->solver = new ObservedBF(h->game);
    return h;
}

void ref_bf_destroy(void *p)
{
    RefBF *h = static_cast<RefBF *>(p);
    if (!h) return;
    delete h->solver;
    delete h;
}

int ref_bf_n(void *p) { return static_cast<RefBF *>(p)->game.get_n_vertices(); }
int ref_bf_max_pri(void *p) { return static_cast<RefBF *>(p)->game.get_max_pri(); }

void ref_bf_init_strat(void *p) { static_cast<RefBF *>(p)->solver->init_strat(); }

void ref_bf_best_response(void *p, int *br_count)
{
    with_big_stack([p, br_count] { static_cast<RefBF *>(p)->solver->best_response(br_count); });
}

void ref_bf_mark_solved(void *p, int player) { static_cast<RefBF *>(p)->solver->mark_solved(player); }

long long ref_bf_switch_strategy(void *p, int player)
{
    return static_cast<RefBF *>(p)->solver->switch_strategy(player);
}

long long ref_bf_get_winning(void *p, int player, int *out)
{
    std::vector<int> w;
    static_cast<RefBF *>(p)->solver->get_winning(w, player);
    if (out) std::memcpy(out, w.data(), sizeof(int) * w.size());
    return (long long)w.size();
}

void ref_bf_get_strategy(void *p, int *out)
{
    std::vector<int> &s = static_cast<RefBF *>(p)->solver->strategy();
    std::memcpy(out, s.data(), sizeof(int) * s.size());
}

void ref_bf_get_infinite(void *p, int *out)
{
    std::vector<int> &s = static_cast<RefBF *>(p)->solver->inf();
    std::memcpy(out, s.data(), sizeof(int) * s.size());
}

void ref_bf_get_solved(void *p, int *out)
{
    std::vector<int> &s = static_cast<RefBF *>(p)->solver->sol();
    std::memcpy(out, s.data(), sizeof(int) * s.size());
}

// Valuation rows through ArrayVal::to_string ("[c0 c1 ... ]"), the only
// public view of the counts.
void ref_bf_get_vals(void *p, int v0, int count, int *out)
{
    RefBF *h = static_cast<RefBF *>(p);
    const int d = h->game.get_max_pri() + 1;
    for (int i = 0; i < count; i++) {
        std::string s = h->solver->val(v0 + i).to_string();
        std::istringstream in(s.substr(1));
        for (int k = 0; k < d; k++) in >> out[(long long)i * d + k];
    }
}

}  // extern "C"
