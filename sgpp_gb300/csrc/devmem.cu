#include "devmem.h"

#include <cstdint>
#include <mutex>
#include <vector>

namespace sgmev {

namespace {
std::mutex g_mu;
std::vector<cudaMemPool_t> g_pools;  // per device: the library's own pool (nullptr: not made yet)
std::vector<void*> g_pinned;         // recycled pinned blocks
constexpr size_t kPinnedBytes = 64;

// The library allocates from a pool of its own, not from the device's default pool: its release
// threshold is raised so that freed blocks stay for the next operator, and raising it on the
// default pool would stop every other cudaMallocAsync user of the process from returning memory.
cudaMemPool_t library_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (static_cast<int>(g_pools.size()) <= dev) g_pools.resize(dev + 1, nullptr);
  if (g_pools[dev]) return g_pools[dev];
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  uint64_t keep = UINT64_MAX;  // keep freed blocks for the next operator
  if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess)
    (void)cudaGetLastError();
  g_pools[dev] = pool;
  return pool;
}
}  // namespace

cudaError_t dev_malloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  cudaMemPool_t pool = library_pool();
  if (!pool) return cudaErrorMemoryAllocation;
  const size_t n = bytes == 0 ? 1 : bytes;
  cudaError_t e = cudaMallocFromPoolAsync(p, n, pool, s);
  if (e == cudaErrorMemoryAllocation) {
    // hand the pool's unused blocks back to the device and try once more
    (void)cudaGetLastError();
    cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocFromPoolAsync(p, n, pool, s);
  }
  if (e != cudaSuccess) {
    *p = nullptr;
    (void)cudaGetLastError();
  }
  return e;
}

void dev_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

void* pinned_block() {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_pinned.empty()) {
      void* p = g_pinned.back();
      g_pinned.pop_back();
      return p;
    }
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, kPinnedBytes) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return p;
}

void pinned_release(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_mu);
  g_pinned.push_back(p);
}

}  // namespace sgmev
