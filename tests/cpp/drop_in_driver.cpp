// drop_in_driver.cpp -- the reference's GPU driver flow (gpumain.cpp:102-146:
// parse a .gm file, build the solver, run solve_si, print "time iters brs")
// written against include/psi_si.hpp.  Built and run by tests/test_cpp_driver.py.
//   drop_in_driver parse <game.gm>   -> "n m max_pri" (no GPU needed)
//   drop_in_driver solve <game.gm>   -> "time iters brs" then the W0 size
//   drop_in_driver serve <game.gm>   -> the same game through Batch and Server:
//                                       "iters brs" of each and the certificate status
//   drop_in_driver tune <game.gm>    -> options from psi::autotune, then solve_si with
//                                       them: "sublist_len walk_block patch_limit" then
//                                       "iters brs" 
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "psi_si.hpp"

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::printf("usage: %s parse|solve|serve|tune game.gm\n", argv[0]);
        return 1;
    }
    try {
        psi::Game g;
        g.parse_pgsolver(argv[2]);
        if (std::strcmp(argv[1], "parse") == 0) {
            std::printf("%d %lld %d\n", g.get_n_vertices(), (long long)g.get_n_edges(), g.get_max_pri());
            return 0;
        }
        if (std::strcmp(argv[1], "serve") == 0) {
            std::vector<const psi::Game *> one{&g};
            psi::Batch b(one);
            std::vector<int32_t> bi, bb;
            b.solve(bi, bb);
            psi::Server srv(2 * (int64_t)g.get_n_vertices() + 2, 2 * g.get_n_edges() + 2, 4);
            int64_t t = srv.submit(g);
            while (!srv.idle()) srv.step();
            int32_t si_ = 0, sb = 0;
            srv.finished(t, &si_, &sb);
            std::vector<int32_t> strat, inf;
            srv.take(t, strat, inf);
            std::printf("%d %d\n%d %d\n%d\n", bi[0], bb[0], si_, sb, psi::check_solution(g, strat, inf));
            return 0;
        }
        if (std::strcmp(argv[1], "tune") == 0) {
            psi_tune_report rep;
            const psi_options o = psi::autotune({&g}, nullptr, 1, &rep);
            psi::GPUList tuned(g, &o);
            int it = 0, br = 0;
            psi::solve_si(tuned, &br, &it, false);
            std::printf("%d %d %d\n%d %d\n", o.sublist_len, o.walk_block, o.patch_limit, it, br);
            return 0;
        }
        psi::GPUList si(g);
        int iters = 0, brs = 0;
        auto t0 = std::chrono::steady_clock::now();
        psi::solve_si(si, &brs, &iters, false);
        double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("%f %d %d\n", dt, iters, brs);
        std::vector<int> w0;
        si.get_winning(w0, 0);
        std::printf("%zu\n", w0.size());
    } catch (const psi::Error &e) {
        std::fprintf(stderr, "parsing error: %s\n", e.what());
        return 2;
    }
    return 0;
}
