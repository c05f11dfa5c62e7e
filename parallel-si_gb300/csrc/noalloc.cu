// noalloc.cu -- strategy evaluation that allocates no memory.
//
// Some callers must not allocate device memory once they are running: a
// serving process that sizes its device memory up front and treats any later
// allocation as a failure (it can run out under load, and cudaMalloc/cudaFree
// can stall other work on the device while they run), or a host program whose
// device memory belongs to another allocator (a framework's caching pool)
// that it must not bypass.  psi_evaluate_strategy_noalloc serves them: it runs
// the same evaluation as psi_compute_valuation -- Euler tour of the sink tree,
// Helman-JaJa sublists, device ranking of the reduced list, depth broadcast,
// cycle parity -- on caller-provided device arrays, and takes its working
// memory from one file-scope __device__ array of fixed size instead of
// cudaMalloc.
//
// That array exists once per device in every process that loads the library,
// from load until exit, whether or not the entry point is used; its size
// bounds the games this entry point accepts (PSI_NOALLOC_MAX_VERTICES).
#include <cstring>
#include <mutex>
#include <string>

#include "device_common.cuh"
#include "kernels.h"
#include "psi_internal.h"

namespace psi {

namespace {

constexpr int32_t kMaxN = PSI_NOALLOC_MAX_VERTICES;
constexpr int32_t kStride = 64;                                   // sublist stride
constexpr int64_t kMaxL = 2 * (int64_t)kMaxN + 2;                 // tour nodes
constexpr int32_t kMaxSub = (int32_t)((kMaxL - 1 + kStride - 1) / kStride + 1);

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Layout of the scratch array (byte offsets).
struct Layout {
    static constexpr size_t words = 0;                                            // struct Words
    static constexpr size_t succ = align256(words + 32);
    static constexpr size_t vloc = align256(succ + 4 * kMaxL);                    // later: two active lists
    static constexpr size_t list = align256(vloc + 8 * (size_t)kMaxN);            // sink list, then unreached list
    static constexpr size_t node = align256(list + 4 * (size_t)kMaxN);
    static constexpr size_t solved = align256(node + sizeof(PathNode) * (size_t)kMaxN);
    static constexpr size_t ja = align256(solved + (size_t)kMaxN);
    static constexpr size_t jb = align256(ja + 16 * (size_t)kMaxN);
    static constexpr size_t redA = align256(jb + 16 * (size_t)kMaxN);
    static constexpr size_t redB = align256(redA + 8 * (size_t)kMaxSub);
    static constexpr size_t redC = align256(redB + 8 * (size_t)kMaxSub);
    static constexpr size_t total = align256(redC + 8 * (size_t)kMaxSub);
};

// The working memory of psi_evaluate_strategy_noalloc (one copy per device).
static __device__ __align__(256) unsigned char g_scratch[Layout::total];

// Device address of g_scratch per device ordinal, looked up once.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_base[kMaxDevices] = {nullptr};

struct Words {
    uint32_t err;
    int32_t ucount;
    int32_t sinkcount;
    int32_t cnt[3];
};
static_assert(sizeof(Words) <= 32, "Words must fit its slot");

inline unsigned grid_for(int64_t items, int block = kBlock)
{
    int64_t g = ceil_div(items, block);
    return (unsigned)(g < 1 ? 1 : g);
}

__global__ void k_na_init(int32_t n, int32_t *__restrict__ succ, int2 *__restrict__ vloc,
                          uint8_t *__restrict__ solved)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    succ[2 * (int64_t)i + 1] = 2 * i;
    succ[2 * (int64_t)i] = (i == n) ? TOUR_END : 2 * i + 1;
    if (i < n) {
        vloc[i] = make_int2(-1, 0);
        solved[i] = 0;
    }
}

// Children of real vertices splice into the parent's up slot with one atomic
// exchange; the sink's children are appended to a list (one atomic per warp)
// and chained by k_na_sink_chain.
__global__ void k_na_link(int32_t n, const int32_t *__restrict__ strat, int32_t *__restrict__ succ,
                          int32_t *__restrict__ sinklist, int32_t *__restrict__ sinkcount,
                          uint32_t *__restrict__ err)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    int32_t p = (v < n) ? strat[v] : 0;
    if (v < n && (p >= n || p < -1)) {           // neither a vertex nor the sink: reject
        atomicOr(err, DERR_BAD_INPUT);
        p = -1;
    }
    bool to_sink = v < n && p < 0;
    if (v < n && !to_sink) {
        int32_t old = atomicExch(&succ[2 * (int64_t)p + 1], 2 * v + 1);
        succ[2 * (int64_t)v] = old;
    }
    unsigned mask = __ballot_sync(0xffffffffu, to_sink);
    if (mask) {
        int lane = threadIdx.x & 31;
        int leader = __ffs(mask) - 1;
        int32_t base = 0;
        if (lane == leader) base = atomicAdd(sinkcount, __popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (to_sink) sinklist[base + __popc(mask & ((1u << lane) - 1))] = v;
    }
}

__global__ void k_na_sink_chain(int32_t n, const int32_t *__restrict__ sinklist,
                                const int32_t *__restrict__ sinkcount, int32_t *__restrict__ succ)
{
    int32_t k = *sinkcount;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) {
        int32_t v = sinklist[i];
        succ[2 * (int64_t)v] = (i + 1 < k) ? 2 * sinklist[i + 1] + 1 : 2 * n;
        if (i == 0) succ[2 * (int64_t)n + 1] = 2 * v + 1;
    }
}

// Looks up this device's address of g_scratch once (the device must be
// current).  In host code the name g_scratch denotes a host-side stand-in,
// never the device array, so only the address returned here is used.
int scratch_base(int dev, unsigned char **out)
{
    if (dev < 0 || dev >= kMaxDevices) return fail(PSI_ERR_INVALID, "device ordinal beyond the no-alloc table");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_base[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess)
            return fail(PSI_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_base[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_base[dev];
    return PSI_OK;
}

}  // namespace

}  // namespace psi

extern "C" int psi_evaluate_strategy_noalloc(int32_t n, const int32_t *strategy, const int32_t *priority,
                                             int32_t *status, void *stream)
{
    using namespace psi;
    if (n <= 0 || !strategy || !priority || !status) return fail(PSI_ERR_INVALID, "null or empty argument");
    if (n > kMaxN)
        return fail(PSI_ERR_TOO_LARGE, "psi_evaluate_strategy_noalloc: n = " + std::to_string(n) +
                                           " exceeds its fixed scratch capacity of " + std::to_string(kMaxN) +
                                           " vertices; use a solver handle (psi_solver_create) instead");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(PSI_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    unsigned char *base = nullptr;
    int rc = scratch_base(dev, &base);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    Words *w = reinterpret_cast<Words *>(base + Layout::words);
    int32_t *succ = reinterpret_cast<int32_t *>(base + Layout::succ);
    int2 *vloc = reinterpret_cast<int2 *>(base + Layout::vloc);
    int32_t *list = reinterpret_cast<int32_t *>(base + Layout::list);
    PathNode *node = reinterpret_cast<PathNode *>(base + Layout::node);
    uint8_t *solved = reinterpret_cast<uint8_t *>(base + Layout::solved);
    int4 *ja = reinterpret_cast<int4 *>(base + Layout::ja);
    int4 *jb = reinterpret_cast<int4 *>(base + Layout::jb);
    int2 *redA = reinterpret_cast<int2 *>(base + Layout::redA);
    int2 *redB = reinterpret_cast<int2 *>(base + Layout::redB);
    int2 *redC = reinterpret_cast<int2 *>(base + Layout::redC);

    const int64_t L = 2 * (int64_t)n + 2;
    const int32_t nsub = (int32_t)(ceil_div(L - 1, kStride) + 1);

    // the scratch keeps the previous call's contents: reset what must start at zero
    e = cudaMemsetAsync(w, 0, sizeof(Words), s);
    if (e != cudaSuccess) return fail(PSI_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e));
    count_launch();
    k_na_init<<<grid_for((int64_t)n + 1), kBlock, 0, s>>>(n, succ, vloc, solved);
    count_launch();
    k_na_link<<<grid_for(n), kBlock, 0, s>>>(n, strategy, succ, list, &w->sinkcount, &w->err);
    count_launch();
    unsigned g = grid_for(n);
    k_na_sink_chain<<<g < 1216u ? g : 1216u, kBlock, 0, s>>>(n, list, &w->sinkcount, succ);
    launch_walk_sublists(s, nsub, n, L, kStride, succ, vloc, redA, &w->err);
    const int2 *fin = nullptr;
    int re = launch_rank_reduced(s, nsub, redA, redB, redC, &fin, nullptr, &w->err);
    if (re) return fail(PSI_ERR_CUDA, std::string("reduced-list kernel launch: ") + cudaGetErrorString((cudaError_t)re));
    launch_broadcast_depth(s, n, vloc, fin, strategy, priority, solved, status, node, list, &w->ucount);
    int32_t *la = reinterpret_cast<int32_t *>(vloc), *lb = la + n;
    int ce = launch_cycles(s, &w->ucount, list, strategy, priority, solved, status, nullptr, ja, jb, la, lb, w->cnt,
                           &w->err);
    if (ce) return fail(PSI_ERR_CUDA, std::string("cycle kernel launch: ") + cudaGetErrorString((cudaError_t)ce));
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PSI_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    uint32_t err_bits = 0;
    e = cudaMemcpyAsync(&err_bits, &w->err, sizeof err_bits, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(PSI_ERR_CUDA, std::string("evaluation: ") + cudaGetErrorString(e));
    if (err_bits & DERR_BAD_INPUT) return fail(PSI_ERR_INVALID, "strategy entry out of range");
    if (err_bits) return fail(PSI_ERR_LIMIT, "device step cap reached (bits " + std::to_string(err_bits) + ")");
    return PSI_OK;
}
