// game.h -- host-side parity game (CSR) used by the native library.
#ifndef PSI_GAME_H
#define PSI_GAME_H

#include <cstdint>
#include <functional>
#include <memory>
#include <new>
#include <type_traits>
#include <utility>
#include <vector>

namespace psi {

// Allocator whose resize() leaves new elements default-initialised (for
// int32: unwritten), so a large game's arrays are not zeroed just before
// they are filled.
template <class T>
struct DefaultInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = DefaultInitAlloc<U>;
    };
    DefaultInitAlloc() = default;
    template <class U>
    DefaultInitAlloc(const DefaultInitAlloc<U> &) noexcept {}
    template <class U>
    void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value)
    {
        ::new (static_cast<void *>(p)) U;
    }
    template <class U, class... A>
    void construct(U *p, A &&...a)
    {
        ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
    }
};
using IVec = std::vector<int32_t, DefaultInitAlloc<int32_t>>;

// Vertices 0..n-1; owner 0 = Even, 1 = Odd; successors of v are
// targets[offsets[v] .. offsets[v+1]) in file order (the order the all-switches
// rule scans them in).  max_pri is the largest priority, at least 0.
struct HostGame {
    int32_t n = 0;
    int64_t m = 0;
    int32_t max_pri = 0;
    IVec owner, priority, offsets, targets;
};

// Runs f(lo, hi) over [0, count) split into contiguous chunks on up to 16
// host threads (one thread below about a million items).
void parallel_chunks(int64_t count, const std::function<void(int64_t, int64_t)> &f);

// Read-only view of a CSR game in caller memory (what the solver uploads).
struct CsrView {
    int32_t n = 0;
    int64_t m = 0;
    int32_t max_pri = 0;
    const int32_t *owner = nullptr, *priority = nullptr, *offsets = nullptr, *targets = nullptr;
};
inline CsrView view_of(const HostGame &g)
{
    return CsrView{g.n, g.m, g.max_pri, g.owner.data(), g.priority.data(), g.offsets.data(), g.targets.data()};
}
// Validates caller arrays (validate_csr) and fills in m and max_pri.
int make_view(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
              const int32_t *targets, CsrView &v);

int parse_gm(const char *text, int64_t len, HostGame &g);
int load_gm(const char *path, HostGame &g);
int write_gm(const HostGame &g, const char *path);
int validate_csr(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
                 const int32_t *targets);
int make_game(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
              const int32_t *targets, HostGame &g);
int generate_random(int32_t n, int32_t deg_lo, int32_t deg_hi, int32_t pri_hi, uint64_t seed, HostGame &g);
int generate_longpath(int32_t n, int32_t pri_hi, uint64_t seed, HostGame &g);

}  // namespace psi

#endif
