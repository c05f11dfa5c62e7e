// setup_kernels.cu -- device set-up of a game and ordered selections: the
// reverse CSR (distinct in-neighbours of every vertex, in increasing order)
// that the tour build scans to link each parent's children without atomics,
// the owner narrowing and player lists built at upload, and the winning-set
// selection read back at the end of a solve.
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

// key = (target << 32) | source for every edge
__global__ void k_edge_keys(int32_t n, const int32_t *__restrict__ off, const int32_t *__restrict__ tgt,
                            unsigned long long *__restrict__ keys)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    for (int32_t e = off[v]; e < off[v + 1]; e++)
        keys[e] = ((unsigned long long)(uint32_t)tgt[e] << 32) | (uint32_t)v;
}

__global__ void k_rev_count(const unsigned long long *__restrict__ keys, const int32_t *__restrict__ nkeys,
                            int32_t *__restrict__ deg, int32_t *__restrict__ src)
{
    int32_t k = *nkeys;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) {
        unsigned long long key = keys[i];
        atomicAdd(&deg[(int32_t)(key >> 32)], 1);
        src[i] = (int32_t)(uint32_t)(key & 0xffffffffull);
    }
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
    unsigned long long *k0 = nullptr, *k1 = nullptr;
    int32_t *nuniq = nullptr, *deg = nullptr;
    void *tmp = nullptr;
    size_t tmp_sort = 0, tmp_uniq = 0, tmp_scan = 0;
    const int end_bit = 32 + bits_for(n);
    cudaError_t e = cudaSuccess;
    cub::DoubleBuffer<unsigned long long> db(nullptr, nullptr);
    e = cub::DeviceRadixSort::SortKeys(nullptr, tmp_sort, db, (int)m, 0, end_bit, s);
    if (e) return e;
    e = cub::DeviceSelect::Unique(nullptr, tmp_uniq, (unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                  (int32_t *)nullptr, (int)m, s);
    if (e) return e;
    e = cub::DeviceScan::ExclusiveSum(nullptr, tmp_scan, (int32_t *)nullptr, (int32_t *)nullptr, n + 1, s);
    if (e) return e;
    size_t tmp_bytes = std::max(tmp_sort, std::max(tmp_uniq, tmp_scan));
    if ((e = device_alloc((void **)&k0, 8 * (size_t)m, s))) goto out;
    if ((e = device_alloc((void **)&k1, 8 * (size_t)m, s))) goto out;
    if ((e = device_alloc((void **)&nuniq, sizeof(int32_t), s))) goto out;
    if ((e = device_alloc((void **)&deg, 4 * ((size_t)n + 1), s))) goto out;
    if ((e = device_alloc(&tmp, tmp_bytes, s))) goto out;
    count_launch();
    k_edge_keys<<<grid_for(n), kBlock, 0, s>>>(n, off, tgt, k0);
    {
        cub::DoubleBuffer<unsigned long long> keys(k0, k1);
        size_t t = tmp_bytes;
        if ((e = cub::DeviceRadixSort::SortKeys(tmp, t, keys, (int)m, 0, end_bit, s))) goto out;
        unsigned long long *sorted = keys.Current(), *spare = keys.Alternate();
        t = tmp_bytes;
        if ((e = cub::DeviceSelect::Unique(tmp, t, sorted, spare, nuniq, (int)m, s))) goto out;
        if ((e = cudaMemsetAsync(deg, 0, 4 * ((size_t)n + 1), s))) goto out;
        count_launch();
        k_rev_count<<<1216, kBlock, 0, s>>>(spare, nuniq, deg, rev_src);
        t = tmp_bytes;
        if ((e = cub::DeviceScan::ExclusiveSum(tmp, t, deg, rev_off, n + 1, s))) goto out;
        int32_t h = 0;
        if ((e = cudaMemcpyAsync(&h, nuniq, sizeof h, cudaMemcpyDeviceToHost, s))) goto out;
        if ((e = cudaStreamSynchronize(s))) goto out;
        *rev_m = h;
    }
out:
    if (k0) cudaFreeAsync(k0, s);
    if (k1) cudaFreeAsync(k1, s);
    if (nuniq) cudaFreeAsync(nuniq, s);
    if (deg) cudaFreeAsync(deg, s);
    if (tmp) cudaFreeAsync(tmp, s);
    return (int)e;
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
