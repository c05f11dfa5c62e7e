// measure.cu -- the random-access bound that the evaluation and switch
// kernels are held against: how many independent 4-byte loads from uniformly
// random positions of a large device array this GPU serves per second.
//
// The sublist walk, the root-summary walks and the switch's key gathers read
// one 4-byte word per data-dependent address; each such read moves a whole
// 32-byte sector from HBM, so a plain copy's bandwidth overstates what they
// can reach.  This kernel issues the same kind of reads with no dependence
// between them (eight in flight per thread, every SM filled), which is the
// most such reads can achieve; the walks' chains of dependent loads can only
// approach it.  No counterpart in the reference.
#include <algorithm>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "kernels.h"
#include "psi_internal.h"

namespace psi {

namespace {

// splitmix64's output function (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014): a bijective 64-bit mix whose
// low bits are close to uniform for consecutive inputs.
__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

constexpr int kGatherPer = 8;        // independent loads in flight per thread
constexpr int kGatherBlock = 256;

// Every thread runs `rounds` rounds of kGatherPer loads at mixed positions
// of the array's `words` words (the high 32 bits of the mix scaled to
// [0, words) by a multiply and shift, words < 2^32) and stores the XOR of
// what it read, so no load can be dropped.
__global__ void __launch_bounds__(kGatherBlock) k_random_gather(const int32_t *__restrict__ a, uint64_t words,
                                                                int32_t rounds, uint64_t seed,
                                                                int32_t *__restrict__ sink)
{
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
    int32_t acc = 0;
    for (int32_t r = 0; r < rounds; r++) {
        int32_t v[kGatherPer];
#pragma unroll
        for (int j = 0; j < kGatherPer; j++) {
            const uint64_t k = ((uint64_t)r * kGatherPer + j) * nth + tid;
            v[j] = __ldg(&a[((mix64(k ^ seed) >> 32) * words) >> 32]);
        }
#pragma unroll
        for (int j = 0; j < kGatherPer; j++) acc ^= v[j];
    }
    sink[tid] = acc;
}

int measure_on_current(int32_t device, int64_t array_bytes, int32_t reps, double *gathers_per_s,
                       double *ms_per_launch, int64_t *gathers_per_launch);

}  // namespace

int measure_random_access(int32_t device, int64_t array_bytes, int32_t reps, double *gathers_per_s,
                          double *ms_per_launch, int64_t *gathers_per_launch)
{
    if (reps < 1) return fail(PSI_ERR_INVALID, "reps must be >= 1");
    if (array_bytes < (1 << 20) || array_bytes % 4 != 0 || array_bytes > ((int64_t)1 << 34))
        return fail(PSI_ERR_INVALID, "array_bytes must be a multiple of 4 in [2^20, 2^34]");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(PSI_ERR_NO_DEVICE, "no CUDA device available");
    if (device < 0 || device >= ndev) return fail(PSI_ERR_INVALID, "device ordinal out of range");
    int prev = 0;
    PSI_CUDA_TRY(cudaGetDevice(&prev));
    PSI_CUDA_TRY(cudaSetDevice(device));
    const int rc = measure_on_current(device, array_bytes, reps, gathers_per_s, ms_per_launch, gathers_per_launch);
    cudaSetDevice(prev);   // the caller's current device, as it was
    return rc;
}

namespace {

int measure_on_current(int32_t device, int64_t array_bytes, int32_t reps, double *gathers_per_s,
                       double *ms_per_launch, int64_t *gathers_per_launch)
{
    int sms = 0, per_sm = 0;
    PSI_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    PSI_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_random_gather, kGatherBlock, 0));
    const int blocks = sms * std::max(1, per_sm);
    const int64_t threads = (int64_t)blocks * kGatherBlock;
    // about 2^27 loads per launch: long enough for the event timer, short of a second
    const int32_t rounds = (int32_t)std::max<int64_t>(1, ((int64_t)1 << 27) / (threads * kGatherPer));
    const int64_t words = array_bytes / 4;

    // plain allocations, freed on return (the library's pool keeps what it
    // is given, and this array is needed once)
    int32_t *a = nullptr, *sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<float> ms;
    std::string err;
    auto attempt = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
        return err.empty();
    };
    if (attempt(cudaMalloc(&a, (size_t)array_bytes), "cudaMalloc(array)") &&
        attempt(cudaMalloc(&sink, (size_t)threads * 4), "cudaMalloc(sink)") &&
        attempt(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate") &&
        attempt(cudaEventCreate(&e0), "cudaEventCreate") && attempt(cudaEventCreate(&e1), "cudaEventCreate") &&
        attempt(cudaMemsetAsync(a, 0x5a, (size_t)array_bytes, s), "cudaMemsetAsync")) {
        for (int32_t r = -2; r < reps && err.empty(); r++) {   // two untimed launches first
            count_launch();
            attempt(cudaEventRecord(e0, s), "cudaEventRecord");
            k_random_gather<<<blocks, kGatherBlock, 0, s>>>(a, (uint64_t)words, rounds,
                                                             0x9e3779b97f4a7c15ull * (uint64_t)(r + 3), sink);
            attempt(cudaGetLastError(), "k_random_gather");
            attempt(cudaEventRecord(e1, s), "cudaEventRecord");
            attempt(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float t = 0.f;
            if (attempt(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime") && r >= 0) ms.push_back(t);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (sink) cudaFree(sink);
    if (a) cudaFree(a);
    if (!err.empty()) return fail(PSI_ERR_CUDA, err);
    std::sort(ms.begin(), ms.end());
    const double med = ms[ms.size() / 2];
    const int64_t loads = threads * rounds * kGatherPer;
    if (gathers_per_s) *gathers_per_s = (double)loads / (med / 1e3);
    if (ms_per_launch) *ms_per_launch = med;
    if (gathers_per_launch) *gathers_per_launch = loads;
    return PSI_OK;
}

}  // namespace

}  // namespace psi
