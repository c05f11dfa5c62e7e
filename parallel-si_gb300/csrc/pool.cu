// pool.cu -- the library's device memory: one stream-ordered memory pool per
// device, created on first use, whose release threshold keeps freed blocks
// cached in the pool.  Solvers, batches and servers allocate their arrays
// and temporaries from it, so a process that creates solvers one after
// another (a service uploading one game per request) reuses device memory
// instead of mapping it anew each time.  The process's default pool and its
// settings are left alone.
#include <cstdint>
#include <mutex>

#include "kernels.h"

namespace psi {

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

cudaError_t pool_of(cudaMemPool_t *out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        e = cudaMemPoolCreate(&p, &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = UINT64_MAX;   // never hand freed blocks back while the process runs
        e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(p);
            return e;
        }
        g_pool[dev] = p;
    }
    *out = g_pool[dev];
    return cudaSuccess;
}

}  // namespace

cudaError_t device_alloc(void **p, size_t bytes, cudaStream_t s)
{
    *p = nullptr;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = pool_of(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, s);
}

}  // namespace psi
