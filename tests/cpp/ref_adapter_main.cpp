// ref_adapter_main.cpp -- the reference driver's flow (gpumain.cpp:102-146:
// parse a .gm file with the reference's own Game::parse_pgsolver, build the
// solver, run solve_si, print "iters brs" and the size of Even's winning set),
// with the GB300List adapter (gb300_si.h) behind the reference's
// StrategyImprovement interface.  Compiled by tests/test_ref_adapter.py
// against the reference's game.h, si.h and game.cpp.
#include <cstdio>
#include <vector>

#include "game.h"
#include "gb300_si.h"
#include "si.h"

// solve_si as the reference drivers run it (main.cpp:20-55, gpumain.cpp:18-53),
// restated against the interface: Odd's best response, then Even's switch.
static void solve_si(StrategyImprovement &si, int &iters, int &brs)
{
    iters = brs = 0;
    si.init_strat();
    bool first = true;
    for (;;) {
        for (;;) {
            if (first) si.compute_first_val();
            else si.compute_valuation();
            first = false;
            brs++;
            si.mark_solved(1);
            if (!si.switch_strategy(1)) break;
        }
        si.mark_solved(0);
        iters++;
        if (!si.switch_strategy(0)) break;
    }
}

int main(int argc, char **argv)
{
    if (argc != 2) {
        std::printf("usage: %s game.gm\n", argv[0]);
        return 2;
    }
    Game g;
    g.parse_pgsolver(argv[1]);
    GB300List si(g);
    int iters = 0, brs = 0;
    solve_si(si, iters, brs);
    std::vector<int> w0;
    si.get_winning(w0, 0);
    std::printf("%d %d %zu\n", iters, brs, w0.size());
    return 0;
}
