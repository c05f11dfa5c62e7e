// setup_kernels.cu -- device set-up of a game and ordered selections: the
// reverse CSR (distinct in-neighbours of every vertex, in increasing order)
// that the tour build scans to link each parent's children without atomics,
// the owner narrowing and player lists built at upload, and the winning-set
// selection read back at the end of a solve.
#include <cub/block/block_reduce.cuh>
#include <cub/device/device_partition.cuh>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "device_common.cuh"
#include "kernels.h"

namespace psi {

namespace {

inline unsigned grid_for(int64_t items, int block = kBlock)
{
    int64_t g = ceil_div(items, block);
    return (unsigned)(g < 1 ? 1 : g);
}

// (target, source) of every edge, in CSR order: sources non-decreasing, so a
// stable sort by target leaves each target's sources in increasing order.
__global__ void k_edge_pairs(int32_t n, const int32_t *__restrict__ off, const int32_t *__restrict__ tgt,
                             uint32_t *__restrict__ keys, int32_t *__restrict__ vals)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        for (int32_t e = off[v]; e < off[v + 1]; e++) {
            keys[e] = (uint32_t)tgt[e];
            vals[e] = (int32_t)v;
        }
}

// Keep the first of each run of equal (target, source) pairs; count the kept
// sources per target.
__global__ void k_rev_unique(int64_t m, const uint32_t *__restrict__ keys, const int32_t *__restrict__ vals,
                             uint8_t *__restrict__ keep, int32_t *__restrict__ deg)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        const bool first = i == 0 || k != keys[i - 1] || vals[i] != vals[i - 1];
        keep[i] = first ? 1 : 0;
        if (first) atomicAdd(&deg[k], 1);
    }
}

// Checks an uploaded CSR game as validate_csr does on the host: the lowest
// failing vertex and its check (1 player not 0/1, 2 negative priority, 3 no
// successor) as min(4 v + check) in *bad_vertex, any successor outside
// [0, n) in *bad_edge, and the largest priority in *max_pri.
__global__ void k_validate(int32_t n, int64_t m, const int32_t *__restrict__ owner, const int32_t *__restrict__ pri,
                           const int32_t *__restrict__ off, const int32_t *__restrict__ tgt,
                           unsigned long long *__restrict__ bad_vertex, int32_t *__restrict__ bad_edge,
                           int32_t *__restrict__ max_pri)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int32_t top = 0;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        const int32_t o = owner[v], p = pri[v];
        const int check = (o != 0 && o != 1) ? 1 : (p < 0 ? 2 : (off[v + 1] <= off[v] ? 3 : 0));
        if (check) atomicMin(bad_vertex, (unsigned long long)v * 4 + check);
        top = max(top, p);
    }
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += stride)
        if ((uint32_t)tgt[e] >= (uint32_t)n) *bad_edge = 1;
    typedef cub::BlockReduce<int32_t, kBlock> Reduce;
    __shared__ typename Reduce::TempStorage tmp;
    const int32_t block_top = Reduce(tmp).Reduce(top, [](int32_t x, int32_t y) { return max(x, y); });
    if (threadIdx.x == 0) atomicMax(max_pri, block_top);
}

__global__ void k_narrow_owner(int32_t n, const int32_t *__restrict__ in, int8_t *__restrict__ out)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) out[v] = (int8_t)in[v];
}

struct OwnedBy {
    const int8_t *owner;
    int8_t player;
    __device__ bool operator()(int32_t v) const { return owner[v] == player; }
};

// get_winning (cpu_parity.cpp:288-297): Even wins the +inf vertices, Odd every
// other vertex.
struct WonBy {
    const int32_t *st;
    int32_t player;
    __device__ bool operator()(int32_t v) const { return (st[v] == ST_POS_INF) == (player == 0); }
};

int bits_for(int64_t x)
{
    int b = 1;
    while (((int64_t)1 << b) <= x) b++;
    return b;
}

}  // namespace

int build_reverse_csr(cudaStream_t s, int32_t n, int64_t m, const int32_t *off, const int32_t *tgt,
                      int32_t *rev_off, int32_t *rev_src, int64_t *rev_m)
{
    *rev_m = 0;
    if (m <= 0) return cudaMemsetAsync(rev_off, 0, 4 * ((size_t)n + 1), s);
    uint32_t *k0 = nullptr, *k1 = nullptr;
    int32_t *v0 = nullptr, *v1 = nullptr, *nuniq = nullptr, *deg = nullptr;
    uint8_t *keep = nullptr;
    void *tmp = nullptr;
    size_t tmp_sort = 0, tmp_sel = 0, tmp_scan = 0;
    const int end_bit = bits_for(n);   // targets < n
    cudaError_t e = cudaSuccess;
    {
        cub::DoubleBuffer<uint32_t> dk(nullptr, nullptr);
        cub::DoubleBuffer<int32_t> dv(nullptr, nullptr);
        e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, dk, dv, (int)m, 0, end_bit, s);
        if (e) return e;
    }
    e = cub::DeviceSelect::Flagged(nullptr, tmp_sel, (int32_t *)nullptr, (uint8_t *)nullptr, (int32_t *)nullptr,
                                   (int32_t *)nullptr, (int)m, s);
    if (e) return e;
    e = cub::DeviceScan::ExclusiveSum(nullptr, tmp_scan, (int32_t *)nullptr, (int32_t *)nullptr, n + 1, s);
    if (e) return e;
    size_t tmp_bytes = std::max(tmp_sort, std::max(tmp_sel, tmp_scan));
    if ((e = device_alloc((void **)&k0, 4 * (size_t)m, s))) goto out;
    if ((e = device_alloc((void **)&k1, 4 * (size_t)m, s))) goto out;
    if ((e = device_alloc((void **)&v0, 4 * (size_t)m, s))) goto out;
    if ((e = device_alloc((void **)&v1, 4 * (size_t)m, s))) goto out;
    if ((e = device_alloc((void **)&keep, (size_t)m, s))) goto out;
    if ((e = device_alloc((void **)&nuniq, sizeof(int32_t), s))) goto out;
    if ((e = device_alloc((void **)&deg, 4 * ((size_t)n + 1), s))) goto out;
    if ((e = device_alloc(&tmp, tmp_bytes, s))) goto out;
    count_launch();
    k_edge_pairs<<<grid_for(n), kBlock, 0, s>>>(n, off, tgt, k0, v0);
    {
        // stable by target: each target's sources stay in increasing order
        cub::DoubleBuffer<uint32_t> keys(k0, k1);
        cub::DoubleBuffer<int32_t> vals(v0, v1);
        size_t t = tmp_bytes;
        if ((e = cub::DeviceRadixSort::SortPairs(tmp, t, keys, vals, (int)m, 0, end_bit, s))) goto out;
        if ((e = cudaMemsetAsync(deg, 0, 4 * ((size_t)n + 1), s))) goto out;
        count_launch();
        k_rev_unique<<<1216, kBlock, 0, s>>>(m, keys.Current(), vals.Current(), keep, deg);
        t = tmp_bytes;
        if ((e = cub::DeviceSelect::Flagged(tmp, t, vals.Current(), keep, rev_src, nuniq, (int)m, s))) goto out;
        t = tmp_bytes;
        if ((e = cub::DeviceScan::ExclusiveSum(tmp, t, deg, rev_off, n + 1, s))) goto out;
        int32_t h = 0;
        if ((e = cudaMemcpyAsync(&h, nuniq, sizeof h, cudaMemcpyDeviceToHost, s))) goto out;
        if ((e = cudaStreamSynchronize(s))) goto out;
        *rev_m = h;
    }
out:
    for (void *p : {(void *)k0, (void *)k1, (void *)v0, (void *)v1, (void *)keep, (void *)nuniq, (void *)deg, tmp})
        if (p) cudaFreeAsync(p, s);
    return (int)e;
}

int validate_game(cudaStream_t s, int32_t n, int64_t m, const int32_t *owner, const int32_t *pri,
                  const int32_t *off, const int32_t *tgt, int64_t *bad_vertex, int32_t *bad_check,
                  int32_t *bad_edge, int32_t *max_pri)
{
    *bad_vertex = -1;
    *bad_check = 0;
    *bad_edge = 0;
    *max_pri = 0;
    if (n <= 0) return 0;
    struct Out {
        unsigned long long bad_vertex;
        int32_t bad_edge, max_pri;
    };
    Out *d = nullptr;
    cudaError_t e = device_alloc((void **)&d, sizeof(Out), s);
    if (e) return e;
    Out init = {~0ull, 0, 0};
    Out h = init;
    e = cudaMemcpyAsync(d, &init, sizeof init, cudaMemcpyHostToDevice, s);
    if (!e) {
        count_launch();
        unsigned g = grid_for(std::max<int64_t>(n, m));
        g = g < 2432u ? g : 2432u;
        k_validate<<<g, kBlock, 0, s>>>(n, m, owner, pri, off, tgt, &d->bad_vertex, &d->bad_edge, &d->max_pri);
        e = cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, s);
    }
    if (!e) e = cudaStreamSynchronize(s);
    cudaFreeAsync(d, s);
    if (e) return e;
    if (h.bad_vertex != ~0ull) {
        *bad_vertex = (int64_t)(h.bad_vertex / 4);
        *bad_check = (int32_t)(h.bad_vertex % 4);
    }
    *bad_edge = h.bad_edge;
    *max_pri = h.max_pri;
    return 0;
}

void launch_narrow_owner(cudaStream_t s, int32_t n, const int32_t *in, int8_t *out)
{
    if (n <= 0) return;
    count_launch();
    k_narrow_owner<<<grid_for(n), kBlock, 0, s>>>(n, in, out);
}

int partition_players(cudaStream_t s, int32_t n, const int8_t *owner, int32_t *plist, int32_t *n_even)
{
    thrust::counting_iterator<int32_t> ids(0);
    OwnedBy even{owner, 0};
    size_t bytes = 0;
    cudaError_t e = cub::DevicePartition::If(nullptr, bytes, ids, plist, n_even, n, even, s);
    if (e) return e;
    void *tmp = nullptr;
    if ((e = device_alloc(&tmp, bytes, s))) return e;
    e = cub::DevicePartition::If(tmp, bytes, ids, plist, n_even, n, even, s);
    cudaFreeAsync(tmp, s);
    return e;
}

int select_winning(cudaStream_t s, int32_t n, int32_t player, const int32_t *st, int32_t *out, int32_t *count)
{
    thrust::counting_iterator<int32_t> ids(0);
    WonBy won{st, player};
    size_t bytes = 0;
    cudaError_t e = cub::DeviceSelect::If(nullptr, bytes, ids, out, count, n, won, s);
    if (e) return e;
    void *tmp = nullptr;
    if ((e = device_alloc(&tmp, bytes, s))) return e;
    e = cub::DeviceSelect::If(tmp, bytes, ids, out, count, n, won, s);
    cudaFreeAsync(tmp, s);
    return e;
}

}  // namespace psi
