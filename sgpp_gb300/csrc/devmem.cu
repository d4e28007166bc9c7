#include "devmem.h"

#include <cstdint>
#include <mutex>
#include <vector>

namespace sgmev {

namespace {
std::mutex g_mu;
std::vector<int> g_pool_ready;  // per device: release threshold raised
std::vector<void*> g_pinned;    // recycled pinned blocks
constexpr size_t kPinnedBytes = 64;

void prepare_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (static_cast<int>(g_pool_ready.size()) <= dev) g_pool_ready.resize(dev + 1, 0);
  if (g_pool_ready[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;  // keep freed blocks for the next operator
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  (void)cudaGetLastError();
  g_pool_ready[dev] = 1;
}
}  // namespace

cudaError_t dev_malloc(void** p, size_t bytes, cudaStream_t s) {
  prepare_pool();
  *p = nullptr;
  cudaError_t e = cudaMallocAsync(p, bytes == 0 ? 1 : bytes, s);
  if (e == cudaErrorMemoryAllocation) {
    // hand the pool's unused blocks back to the device and try once more
    (void)cudaGetLastError();
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
      cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocAsync(p, bytes == 0 ? 1 : bytes, s);
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
