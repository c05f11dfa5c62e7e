// game.h -- host-side parity game (CSR) used by the native library.
#ifndef PSI_GAME_H
#define PSI_GAME_H

#include <cstdint>
#include <vector>

namespace psi {

// Vertices 0..n-1; owner 0 = Even, 1 = Odd; successors of v are
// targets[offsets[v] .. offsets[v+1]) in file order (the order the all-switches
// rule scans them in).  max_pri is the largest priority, at least 0.
struct HostGame {
    int32_t n = 0;
    int64_t m = 0;
    int32_t max_pri = 0;
    std::vector<int32_t> owner, priority, offsets, targets;
};

int parse_gm(const char *text, int64_t len, HostGame &g);
int load_gm(const char *path, HostGame &g);
int write_gm(const HostGame &g, const char *path);
int validate_csr(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
                 const int32_t *targets);
int make_game(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
              const int32_t *targets, HostGame &g);
int generate_random(int32_t n, int32_t deg_lo, int32_t deg_hi, int32_t pri_hi, uint64_t seed, HostGame &g);
int generate_longpath(int32_t n, int32_t pri_hi, uint64_t seed, HostGame &g);
int pack_games(const std::vector<const HostGame *> &games, HostGame &out, std::vector<int64_t> &base);

}  // namespace psi

#endif
