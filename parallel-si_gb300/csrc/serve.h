// serve.h -- continuous-batching server (serve.cpp) used by the C-ABI.
#ifndef PSI_SERVE_H
#define PSI_SERVE_H

#include <cstdint>

#include "game.h"
#include "psi.h"

namespace psi {

class Server;

// An arena of max_vertices vertex slots (a game of n vertices takes n+1) and
// max_edges edges holding at most `slots` games at a time; `reset` selects the
// reset variant of solve_si.
int make_server(int64_t max_vertices, int64_t max_edges, int32_t slots, bool reset, const psi_options &opt,
                Server **out);
int server_submit(Server *s, const HostGame &g, int64_t *ticket);
// Admits what fits, runs one solve_si step of every resident game and retires
// the games that finished; *finished = how many did.
int server_step(Server *s, int32_t *finished);
// state: 0 queued, 1 resident, 2 finished (result ready).
int server_status(Server *s, int64_t ticket, int32_t *state, int32_t *iters, int32_t *brs);
// Copies a finished request's strategy and infinity flags out and forgets it.
int server_take(Server *s, int64_t ticket, int32_t *strategy, int32_t *infinite);
void server_info(const Server *s, int32_t *resident, int32_t *queued, int64_t *used_vertices, int64_t *used_edges);
// Tickets that finished in the last step (*count of them; at most cap copied).
int server_finished(const Server *s, int64_t *tickets, int32_t cap, int32_t *count);
void server_destroy(Server *s);

}  // namespace psi

#endif
