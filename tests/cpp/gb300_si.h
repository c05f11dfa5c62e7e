// gb300_si.h -- the adapter a maintainer adds to the reference code base so
// that its driver solves through this library: a StrategyImprovement
// (si.h:6-16) whose methods call the C ABI (include/psi.h).  It is written
// against the reference's own headers (game.h, si.h), which this repository
// does not carry; tests/test_ref_adapter.py compiles it against them where
// the reference tree is present.  The GB300List constructor replaces both
// GPUGame(g) (gpu_game.cpp:11-41) and GPUList(g, gpu_g)
// (gpu_list_ranking.cu:14-36).
#ifndef GB300_SI_H
#define GB300_SI_H

#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "game.h"   // reference
#include "psi.h"    // this library
#include "si.h"     // reference

class GB300List : public StrategyImprovement {
    psi_solver *s = nullptr;
    int n;
    static void ok(int rc)
    {
        if (rc != PSI_OK) {   // the reference's solvers exit on CUDA errors (gpu_assert)
            std::cout << "psi error: " << psi_last_error() << std::endl;
            std::exit(1);
        }
    }

public:
    explicit GB300List(Game &g) : n(g.get_n_vertices())
    {
        std::vector<int32_t> owner(n), pri(n), off(n + 1), tgt;
        for (int v = 0; v < n; v++) {
            owner[v] = g.get_player(v);
            pri[v] = g.get_priority(v);
            off[v] = (int32_t)tgt.size();
            for (int u : g.get_edges(v)) tgt.push_back(u);
        }
        off[n] = (int32_t)tgt.size();
        psi_game *pg = nullptr;
        ok(psi_game_from_csr(n, owner.data(), pri.data(), off.data(), tgt.data(), &pg));
        ok(psi_solver_create(pg, nullptr, &s));   // uploads the game (GPUGame)
        psi_game_free(pg);
    }
    ~GB300List() { psi_solver_destroy(s); }   // si.h declares no virtual destructor
    void init_strat() override { ok(psi_init_strat(s)); }
    void compute_valuation() override { ok(psi_compute_valuation(s)); }
    void compute_first_val() override { ok(psi_compute_first_val(s)); }
    void mark_solved(int p) override { ok(psi_mark_solved(s, p)); }
    int switch_strategy(int p) override
    {
        int64_t k = 0;
        ok(psi_switch_strategy(s, p, &k));
        return k > 0;   // the reference GPU solvers return a 0/1 flag
    }
    void get_winning(std::vector<int> &out, int p) override
    {
        std::vector<int32_t> w(n);
        int64_t k = 0;
        ok(psi_get_winning(s, p, w.data(), n, &k));
        out.insert(out.end(), w.begin(), w.begin() + k);
    }
    void reset_opponent_strategy() override { ok(psi_reset_opponent_strategy(s)); }
};

#endif
