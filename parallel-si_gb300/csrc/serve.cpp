// serve.cpp -- continuous-batching server for parity games on one GPU.
//
// Requests (games) are queued on submit.  Each step admits queued games, in
// arrival order, as far as vertex/edge ranges and game slots of the resident
// arena allow (first fit; a game that does not fit yet waits and does not
// block smaller ones behind it); then it runs one solve_si step of every
// resident game at once (Solver::arena_step); games that finished leave,
// their results are copied out and their ranges freed for the next
// admissions.  Requests that arrive while others are on the GPU therefore
// join the running set at the next step instead of waiting for a whole batch.
// A resident game advances by exactly its solo solve_si sequence, so its
// results do not depend on what else is resident.
#include <algorithm>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <set>
#include <unordered_map>
#include <vector>

#include "game.h"
#include "psi.h"
#include "psi_internal.h"
#include "serve.h"
#include "solver.h"

namespace psi {

namespace {

// First-fit allocator over [0, capacity).
class Ranges {
public:
    explicit Ranges(int64_t capacity) { free_[0] = capacity; }
    bool take(int64_t len, int64_t *start)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= len) {
                *start = it->first;
                int64_t rest = it->second - len;
                int64_t at = it->first + len;
                free_.erase(it);
                if (rest > 0) free_[at] = rest;
                return true;
            }
        }
        return false;
    }
    void give(int64_t start, int64_t len)
    {
        auto it = free_.emplace(start, len).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }

private:
    std::map<int64_t, int64_t> free_;
};

struct Request {
    int64_t ticket = 0;
    HostGame game;
    int state = 0;                 // 0 queued, 1 resident, 2 finished
    int32_t slot = -1;
    int64_t vb = 0, eb = 0;
    int32_t iters = 0, brs = 0;
    std::vector<int32_t> strategy, infinite;
};

}  // namespace

class Server {
public:
    Server(Solver *s, int64_t max_vertices, int64_t max_edges, int32_t slots, bool reset)
        : solver_(s), vranges_(max_vertices), eranges_(max_edges), slots_(slots),
          max_v_(max_vertices), max_e_(max_edges), reset_(reset)
    {
        for (int32_t k = slots - 1; k >= 0; k--) free_slots_.push_back(k);
        slot_req_.assign(slots, nullptr);
    }
    ~Server() { delete solver_; }

    int submit(const HostGame &g, int64_t *ticket)
    {
        if (g.n <= 0) return fail(PSI_ERR_INVALID, "empty game");
        if ((int64_t)g.n + 1 > max_v_ || g.m > max_e_)
            return fail(PSI_ERR_TOO_LARGE, "game larger than the server's arena");
        auto r = std::make_unique<Request>();
        r->ticket = next_ticket_++;
        r->game = g;
        *ticket = r->ticket;
        queue_.push_back(r.get());
        reqs_[r->ticket] = std::move(r);
        return PSI_OK;
    }

    int step(int32_t *finished)
    {
        *finished = 0;
        last_finished_.clear();
        bool changed = false;
        int rc = admit(&changed);
        if (rc) return rc;
        if (changed || lists_stale_) {   // one rebuild for this step's admissions and the last step's retirements
            rc = solver_->arena_rebuild_lists();
            if (rc) return rc;
            lists_stale_ = false;
        }
        if (resident_ == 0) return PSI_OK;
        std::vector<int32_t> done, iters, brs;
        rc = solver_->arena_step(reset_, done, iters, brs);
        if (rc) return rc;
        // retire the finished games together: copy their results out (in
        // game-local ids, converted on the device), then free their ranges
        std::vector<Request *> fin;
        for (size_t i = 0; i < done.size(); i++) {
            Request *r = slot_req_[done[i]];
            if (!r) continue;
            r->iters = iters[i];
            r->brs = brs[i];
            r->strategy.resize(r->game.n);
            r->infinite.resize(r->game.n);
            rc = solver_->arena_export((int32_t)r->vb, r->game.n, r->strategy.data(), r->infinite.data());
            if (rc) return rc;
            fin.push_back(r);
        }
        if (fin.empty()) return PSI_OK;
        std::vector<int32_t> vbs, counts, slots;
        for (Request *r : fin) {
            const int64_t count = (int64_t)r->game.n + 1;
            ends_.erase(ends_.find(r->vb + count));
            vbs.push_back((int32_t)r->vb);
            counts.push_back((int32_t)count);
            slots.push_back(r->slot);
        }
        rc = solver_->arena_remove(vbs, counts, slots, (int32_t)extent());
        if (rc) return rc;
        for (Request *r : fin) {
            release(r);
            r->state = 2;
            last_finished_.push_back(r->ticket);
            (*finished)++;
        }
        lists_stale_ = true;   // the player lists still hold the retired vertices
        return PSI_OK;
    }

    int status(int64_t ticket, int32_t *state, int32_t *iters, int32_t *brs)
    {
        auto it = reqs_.find(ticket);
        if (it == reqs_.end()) return fail(PSI_ERR_INVALID, "unknown ticket");
        if (state) *state = it->second->state;
        if (iters) *iters = it->second->iters;
        if (brs) *brs = it->second->brs;
        return PSI_OK;
    }

    int take(int64_t ticket, int32_t *strategy, int32_t *infinite)
    {
        auto it = reqs_.find(ticket);
        if (it == reqs_.end()) return fail(PSI_ERR_INVALID, "unknown ticket");
        Request *r = it->second.get();
        if (r->state != 2) return fail(PSI_ERR_STATE, "request not finished");
        if (strategy) std::memcpy(strategy, r->strategy.data(), 4 * r->strategy.size());
        if (infinite) std::memcpy(infinite, r->infinite.data(), 4 * r->infinite.size());
        reqs_.erase(it);
        return PSI_OK;
    }

    const std::vector<int64_t> &last_finished() const { return last_finished_; }

    void info(int32_t *resident, int32_t *queued, int64_t *used_vertices, int64_t *used_edges) const
    {
        if (resident) *resident = resident_;
        if (queued) *queued = (int32_t)queue_.size();
        if (used_vertices) *used_vertices = used_v_;
        if (used_edges) *used_edges = used_e_;
    }

private:
    // Admits queued requests in arrival order while ranges and slots allow,
    // then places them on the device together.
    int admit(bool *changed)
    {
        std::vector<Request *> in;
        for (auto it = queue_.begin(); it != queue_.end() && !free_slots_.empty();) {
            Request *r = *it;
            int64_t vb = 0, eb = 0;
            if (!vranges_.take((int64_t)r->game.n + 1, &vb)) {
                ++it;
                continue;
            }
            if (!eranges_.take(r->game.m, &eb)) {
                vranges_.give(vb, (int64_t)r->game.n + 1);
                ++it;
                continue;
            }
            r->slot = free_slots_.back();
            free_slots_.pop_back();
            r->vb = vb;
            r->eb = eb;
            ends_.insert(vb + r->game.n + 1);
            in.push_back(r);
            it = queue_.erase(it);
        }
        if (in.empty()) return PSI_OK;
        std::vector<const HostGame *> gs;
        std::vector<int32_t> vb, eb, slot;
        for (Request *r : in) {
            gs.push_back(&r->game);
            vb.push_back((int32_t)r->vb);
            eb.push_back((int32_t)r->eb);
            slot.push_back(r->slot);
        }
        int rc = solver_->arena_add(gs, vb, eb, slot, (int32_t)extent());
        if (rc) return rc;
        for (Request *r : in) {
            slot_req_[r->slot] = r;
            r->state = 1;
            resident_++;
            used_v_ += r->game.n + 1;
            used_e_ += r->game.m;
        }
        *changed = true;
        return PSI_OK;
    }

    // Host bookkeeping of a retired request (its device range is already inert).
    void release(Request *r)
    {
        const int64_t count = (int64_t)r->game.n + 1;
        vranges_.give(r->vb, count);
        eranges_.give(r->eb, r->game.m);
        slot_req_[r->slot] = nullptr;
        free_slots_.push_back(r->slot);
        resident_--;
        used_v_ -= count;
        used_e_ -= r->game.m;
        r->game = HostGame();   // the input is no longer needed
    }

    int64_t extent() const { return ends_.empty() ? 0 : *ends_.rbegin(); }

    Solver *solver_;
    Ranges vranges_, eranges_;
    int32_t slots_;
    int64_t max_v_, max_e_;
    bool reset_;
    std::vector<int32_t> free_slots_;
    std::vector<Request *> slot_req_;
    std::deque<Request *> queue_;
    std::unordered_map<int64_t, std::unique_ptr<Request>> reqs_;
    std::multiset<int64_t> ends_;
    std::vector<int64_t> last_finished_;
    int64_t next_ticket_ = 1;
    int32_t resident_ = 0;
    int64_t used_v_ = 0, used_e_ = 0;
    bool lists_stale_ = false;
};

int make_server(int64_t max_vertices, int64_t max_edges, int32_t slots, bool reset, const psi_options &opt,
                Server **out)
{
    Solver *s = nullptr;
    int rc = Solver::create_arena(max_vertices, max_edges, slots, opt, &s);
    if (rc) return rc;
    *out = new Server(s, max_vertices, max_edges, slots, reset);
    return PSI_OK;
}

int server_submit(Server *s, const HostGame &g, int64_t *ticket) { return s->submit(g, ticket); }
int server_step(Server *s, int32_t *finished) { return s->step(finished); }
int server_status(Server *s, int64_t t, int32_t *state, int32_t *iters, int32_t *brs)
{
    return s->status(t, state, iters, brs);
}
int server_take(Server *s, int64_t t, int32_t *strategy, int32_t *infinite) { return s->take(t, strategy, infinite); }
void server_info(const Server *s, int32_t *resident, int32_t *queued, int64_t *uv, int64_t *ue)
{
    s->info(resident, queued, uv, ue);
}
int server_finished(const Server *s, int64_t *tickets, int32_t cap, int32_t *count)
{
    const auto &f = s->last_finished();
    int32_t k = (int32_t)f.size();
    for (int32_t i = 0; i < k && i < cap; i++) tickets[i] = f[i];
    *count = k;
    return PSI_OK;
}
void server_destroy(Server *s) { delete s; }

}  // namespace psi
