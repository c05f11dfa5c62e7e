// psi_si.hpp -- C++ mirror of the reference solver interface over the C ABI.
//
// Header-only.  It gives C++ callers the shape of the reference's classes so
// a driver written against them keeps its structure:
//   psi::Game           ~ Game (game.h:9-34): parse_pgsolver, get_n_vertices,
//                          get_max_pri, get_player, get_priority, get_edges
//   psi::StrategyImprovement ~ StrategyImprovement (si.h:6-16)
//   psi::GPUList        ~ GPUList(Game&, GPUGame&) (gpu_list_ranking.h:11-41):
//                          the GPU solver; constructing it uploads the game
//   psi::solve_si       ~ solve_si (main.cpp:20-55, gpumain.cpp:18-53)
// and, without counterparts in the reference: psi::Batch (many games solved
// together), psi::Server (continuous batching) and psi::check_solution (a
// certificate check of a result).
// Failures become psi::Error exceptions carrying the C ABI status and message
// (the reference exits on CUDA errors, gpu_util.cpp:10-17, and throws
// const char* on parse errors, game.cpp:68-105).
#ifndef PSI_SI_HPP
#define PSI_SI_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "psi.h"

namespace psi {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string &msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc)
{
    if (rc != PSI_OK) throw Error(rc, psi_last_error());
}

class Game {
public:
    Game() = default;
    explicit Game(psi_game *h) : h_(h) { load_info(); }
    Game(const Game &) = delete;
    Game &operator=(const Game &) = delete;
    Game(Game &&o) noexcept { *this = std::move(o); }
    Game &operator=(Game &&o) noexcept
    {
        std::swap(h_, o.h_);
        n_ = o.n_;
        m_ = o.m_;
        max_pri_ = o.max_pri_;
        csr_loaded_ = false;
        return *this;
    }
    ~Game() { psi_game_free(h_); }

    // Game::parse_pgsolver(std::string filename) (game.cpp:38-50)
    void parse_pgsolver(const std::string &filename)
    {
        psi_game *h = nullptr;
        check(psi_game_load_gm(filename.c_str(), &h));
        replace(h);
    }
    // Game::parse_pgsolver(std::istream&) on text already in memory
    void parse_pgsolver_text(const std::string &text)
    {
        psi_game *h = nullptr;
        check(psi_game_parse_gm(text.data(), (int64_t)text.size(), &h));
        replace(h);
    }
    static Game from_csr(const std::vector<int32_t> &owner, const std::vector<int32_t> &priority,
                         const std::vector<int32_t> &offsets, const std::vector<int32_t> &targets)
    {
        psi_game *h = nullptr;
        check(psi_game_from_csr((int32_t)owner.size(), owner.data(), priority.data(), offsets.data(),
                                targets.data(), &h));
        return Game(h);
    }

    int get_n_vertices() const { return n_; }
    int get_max_pri() const { return max_pri_; }
    int64_t get_n_edges() const { return m_; }
    int get_player(int v) { return csr().owner[v]; }
    int get_priority(int v) { return csr().priority[v]; }
    std::vector<int> get_edges(int v)
    {
        const Csr &c = csr();
        return std::vector<int>(c.targets.begin() + c.offsets[v], c.targets.begin() + c.offsets[v + 1]);
    }
    psi_game *handle() const { return h_; }

private:
    struct Csr {
        std::vector<int32_t> owner, priority, offsets, targets;
    };
    void replace(psi_game *h)
    {
        psi_game_free(h_);
        h_ = h;
        csr_loaded_ = false;
        load_info();
    }
    void load_info() { check(psi_game_info(h_, &n_, &m_, &max_pri_)); }
    const Csr &csr()
    {
        if (!csr_loaded_) {
            csr_.owner.resize(n_);
            csr_.priority.resize(n_);
            csr_.offsets.resize((size_t)n_ + 1);
            csr_.targets.resize((size_t)m_);
            check(psi_game_copy_csr(h_, csr_.owner.data(), csr_.priority.data(), csr_.offsets.data(),
                                    csr_.targets.data()));
            csr_loaded_ = true;
        }
        return csr_;
    }
    psi_game *h_ = nullptr;
    int32_t n_ = 0, max_pri_ = 0;
    int64_t m_ = 0;
    bool csr_loaded_ = false;
    Csr csr_;
};

// si.h:6-16
class StrategyImprovement {
public:
    virtual ~StrategyImprovement() = default;
    virtual void init_strat() = 0;
    virtual void compute_valuation() = 0;
    virtual void compute_first_val() { compute_valuation(); }
    virtual void mark_solved(int player) = 0;
    virtual int switch_strategy(int player) = 0;
    virtual void get_winning(std::vector<int> &out, int player) = 0;
    virtual void reset_opponent_strategy() {}
};

class GPUList : public StrategyImprovement {
public:
    explicit GPUList(const Game &g, const psi_options *opt = nullptr) : n_(g.get_n_vertices())
    {
        check(psi_solver_create(g.handle(), opt, &s_));
    }
    GPUList(const GPUList &) = delete;
    GPUList &operator=(const GPUList &) = delete;
    ~GPUList() override { psi_solver_destroy(s_); }

    void init_strat() override { check(psi_init_strat(s_)); }
    void compute_valuation() override { check(psi_compute_valuation(s_)); }
    void compute_first_val() override { check(psi_compute_first_val(s_)); }
    void mark_solved(int player) override { check(psi_mark_solved(s_, player)); }
    // Returns the number of strict improvements, saturated to int.
    int switch_strategy(int player) override
    {
        int64_t k = 0;
        check(psi_switch_strategy(s_, player, &k));
        return k > INT32_MAX ? INT32_MAX : (int)k;
    }
    // Appends the winning set of `player` to out (gpu_parity.cu:340-354).
    void get_winning(std::vector<int> &out, int player) override
    {
        std::vector<int32_t> w((size_t)n_);
        int64_t count = 0;
        check(psi_get_winning(s_, player, w.data(), (int64_t)w.size(), &count));
        out.insert(out.end(), w.begin(), w.begin() + count);
    }
    void reset_opponent_strategy() override { check(psi_reset_opponent_strategy(s_)); }

    std::vector<int32_t> get_strategy()
    {
        std::vector<int32_t> s((size_t)n_);
        check(psi_get_strategy(s_, s.data()));
        return s;
    }
    std::vector<int32_t> get_infinite()
    {
        std::vector<int32_t> s((size_t)n_);
        check(psi_get_infinite(s_, s.data()));
        return s;
    }
    // The whole solve on the device side of the boundary (psi_solve).
    void solve(int *iter_count, int *br_count, bool reset = false)
    {
        int32_t it = 0, br = 0;
        check(psi_solve(s_, reset ? 1 : 0, &it, &br, 0));
        *iter_count = it;
        *br_count = br;
    }
    psi_solver *handle() const { return s_; }

private:
    psi_solver *s_ = nullptr;
    int32_t n_ = 0;
};

// Certificate check of a solution (psi_check_solution): PSI_CHECK_OK or the
// failed check; *vertex receives the offending vertex, if any.
inline int check_solution(const Game &g, const std::vector<int32_t> &strategy, const std::vector<int32_t> &infinite,
                          int64_t *vertex = nullptr, int64_t work_budget = 0)
{
    psi_check_report r;
    check(psi_check_solution(g.handle(), strategy.data(), infinite.data(), work_budget, &r));
    if (vertex) *vertex = r.vertex;
    return r.status;
}

// Options for a workload (one game, or several solved as a Batch) chosen by
// timing trial solves on the device (psi_autotune); base supplies the device
// and the options that are not tuned (nullptr: the defaults).
inline psi_options autotune(const std::vector<const Game *> &games, const psi_options *base = nullptr,
                            int32_t repeats = 2, psi_tune_report *report = nullptr, int32_t flags = 0)
{
    std::vector<const psi_game *> hs;
    for (const Game *g : games) hs.push_back(g->handle());
    psi_options out;
    psi_tune_report r;
    check(psi_autotune(hs.data(), (int32_t)hs.size(), base, repeats, flags, &out, &r));
    if (report) *report = r;
    return out;
}

// Many games solved together (psi_batch_*); each ends with its solo results.
class Batch {
public:
    explicit Batch(const std::vector<const Game *> &games, const psi_options *opt = nullptr)
    {
        std::vector<const psi_game *> hs;
        for (const Game *g : games) {
            hs.push_back(g->handle());
            sizes_.push_back(g->get_n_vertices());
        }
        check(psi_batch_create(hs.data(), (int32_t)hs.size(), opt, &b_));
    }
    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;
    ~Batch() { psi_batch_destroy(b_); }
    // (iteration, evaluation) counts per game
    void solve(std::vector<int32_t> &iters, std::vector<int32_t> &brs)
    {
        iters.assign(sizes_.size(), 0);
        brs.assign(sizes_.size(), 0);
        check(psi_batch_solve(b_, iters.data(), brs.data()));
    }
    std::vector<int32_t> get_strategy(int32_t game)
    {
        std::vector<int32_t> s((size_t)sizes_.at(game));
        check(psi_batch_get_strategy(b_, game, s.data()));
        return s;
    }

private:
    psi_batch *b_ = nullptr;
    std::vector<int32_t> sizes_;
};

// Continuous-batching server (psi_server_*): submit at any time, step, take.
class Server {
public:
    Server(int64_t max_vertices, int64_t max_edges, int32_t max_games, bool reset = false,
           const psi_options *opt = nullptr)
    {
        check(psi_server_create(max_vertices, max_edges, max_games, reset ? 1 : 0, opt, &s_));
    }
    Server(const Server &) = delete;
    Server &operator=(const Server &) = delete;
    ~Server() { psi_server_destroy(s_); }
    int64_t submit(const Game &g)
    {
        int64_t t = 0;
        check(psi_server_submit(s_, g.handle(), &t));
        sizes_.push_back({t, g.get_n_vertices()});
        return t;
    }
    int32_t step()
    {
        int32_t k = 0;
        check(psi_server_step(s_, &k));
        return k;
    }
    bool finished(int64_t ticket, int32_t *iters = nullptr, int32_t *brs = nullptr)
    {
        int32_t state = 0;
        check(psi_server_status(s_, ticket, &state, iters, brs));
        return state == PSI_REQ_FINISHED;
    }
    // strategy and infinity flags of a finished request, in its own vertex ids
    void take(int64_t ticket, std::vector<int32_t> &strategy, std::vector<int32_t> &infinite)
    {
        int32_t n = 0;
        for (const auto &p : sizes_)
            if (p.first == ticket) n = p.second;
        strategy.assign((size_t)n, 0);
        infinite.assign((size_t)n, 0);
        check(psi_server_take(s_, ticket, strategy.data(), infinite.data()));
    }
    bool idle()
    {
        int32_t resident = 0, queued = 0;
        check(psi_server_info(s_, &resident, &queued, nullptr, nullptr));
        return resident == 0 && queued == 0;
    }

private:
    psi_server *s_ = nullptr;
    std::vector<std::pair<int64_t, int32_t>> sizes_;
};

// The reference driver loop (main.cpp:20-55) over any StrategyImprovement.
inline void solve_si(StrategyImprovement &si, int *br_count, int *iter_count, bool reset)
{
    si.init_strat();
    bool first = true;
    while (true) {
        if (!first && reset) si.reset_opponent_strategy();
        while (true) {
            if (first) si.compute_first_val();
            else si.compute_valuation();
            (*br_count)++;
            si.mark_solved(1);
            if (si.switch_strategy(1) == 0) break;
        }
        first = false;
        si.mark_solved(0);
        (*iter_count)++;
        if (si.switch_strategy(0) == 0) break;
    }
}

}  // namespace psi

#endif
