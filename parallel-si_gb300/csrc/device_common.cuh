// device_common.cuh -- shared constants and helpers of the sm_103a kernels.
#ifndef PSI_DEVICE_COMMON_CUH
#define PSI_DEVICE_COMMON_CUH

#include <climits>
#include <cstdint>

#include "kernels.h"
#include <cuda_runtime.h>

namespace psi {

// Per-vertex status word written by an evaluation (and frozen for solved
// vertices):  >= 1  finite valuation, the value is the length of the strategy
// path from the vertex to the sink (its depth in the sink tree);
//             -1    valuation -inf (the path ends in a cycle won by Odd);
//             -2    valuation +inf (the path ends in a cycle won by Even);
//              0    the sink itself (never stored for a vertex).
constexpr int32_t ST_NEG_INF = -1;
constexpr int32_t ST_POS_INF = -2;
constexpr int32_t ST_UNRESOLVED = INT32_MIN;

__host__ __device__ __forceinline__ int32_t st_infinite(int32_t st)
{
    return st == ST_POS_INF ? 1 : (st == ST_NEG_INF ? -1 : 0);
}

// Snapshot of a vertex the sink reached, written by an evaluation: its parent
// in the sink tree (-1 = the sink), its priority, and a summary of its root
// path (the path from the vertex to the sink): the highest priority on it and
// how many vertices of the path carry that priority.  rmax == RM_UNKNOWN until
// the summary has been computed.  16-byte aligned so one load fetches it all
// and the (rmax, rcnt) pair is written as one 8-byte store.
struct __align__(16) PathNode {
    int32_t parent, pri, rmax, rcnt;
};
constexpr int32_t RM_UNKNOWN = INT32_MIN;

// Comparison key of a vertex after an evaluation: 4 bytes, what the switch
// step gathers per compared edge (n = 2^24 keys take 64 MiB and stay in L2).
// With (M, c) the root-path summary of a finite vertex (the highest priority
// on its path to the sink and its count), let
//   q = M < KEY_MCAP ? (M << 7 | min(c, 126)) : KEY_MCAP << 7
// and key = +q if M is even, -q if M is odd; +inf -> KEY_POS_INF, -inf ->
// KEY_NEG_INF; the sink (empty path) -> 0.  The key is a monotone function of
// the valuation order: between distinct summaries the highest priority whose
// counts differ is max(M_u, M_w), so a higher even M is better and a higher
// odd M worse, and at equal M a larger count is better if M is even, worse if
// odd -- clamping c, or M together with c, only merges neighbours.  Hence
// key_u > key_w implies u better than w, and equal keys of distinct finite
// vertices are decided by their exact summaries, then by a walk.
constexpr int32_t KEY_POS_INF = INT32_MAX;
constexpr int32_t KEY_NEG_INF = -INT32_MAX;
constexpr int32_t KEY_MCAP = (1 << 24) - 1;
__host__ __device__ __forceinline__ int32_t finite_key(int32_t m, int32_t c)
{
    int32_t q = (m < KEY_MCAP) ? ((m << 7) | (c < 126 ? c : 126)) : (KEY_MCAP << 7);
    return (m & 1) ? -q : q;
}
__host__ __device__ __forceinline__ int key_infinite(int32_t k)
{
    return k == KEY_POS_INF ? 1 : (k == KEY_NEG_INF ? -1 : 0);
}

// Value signature codes of infinite vertices (finite: (rmax, rcnt), rmax >= 0).
constexpr int32_t SIG_POS_INF = INT32_MIN + 2;
constexpr int32_t SIG_NEG_INF = INT32_MIN + 1;

// Records v's new value signature; if it changed, flags v's in-neighbours
// for their next switch step (kernels.h: ChangeTrack).
__device__ __forceinline__ void note_signature(const ChangeTrack &t, int32_t v, int2 sig)
{
    if (!t.sig) return;
    const int2 old = t.sig[v];
    if (old.x == sig.x && old.y == sig.y) return;
    t.sig[v] = sig;
    const int32_t e1 = t.rev_off[v + 1];
    for (int32_t e = t.rev_off[v]; e < e1; e++) t.need[t.rev_src[e]] = 1;
}

// Tour node ids (an Euler tour of the strategy forest, two nodes per vertex):
// node 2v is v's "down" node (leaving v's subtree toward the sink), 2v+1 its
// "up" node (entering it); 2n / 2n+1 are the sink's down / up nodes.  The list
// starts at the sink's up node and ends at the sink's down node (successor -1).
constexpr int32_t TOUR_END = -1;

// Device-side error bits (a word the host reads back at sync points).
constexpr uint32_t DERR_SUBLIST_CAP = 1u << 0;   // a sublist walk exceeded the list length
constexpr uint32_t DERR_WALK_CAP = 1u << 1;      // a valuation walk exceeded its step cap
constexpr uint32_t DERR_PASS_CAP = 1u << 2;      // a comparison exceeded its pass cap
constexpr uint32_t DERR_BAD_INPUT = 1u << 3;     // malformed strategy (target out of range)

constexpr int kBlock = 256;

__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace psi

#define PSI_CUDA_TRY(expr)                                                            \
    do {                                                                              \
        cudaError_t e__ = (expr);                                                     \
        if (e__ != cudaSuccess)                                                       \
            return ::psi::fail(PSI_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e__)); \
    } while (0)

#endif
