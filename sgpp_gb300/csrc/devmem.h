// Device memory of the operators (internal to libsgpp_gb300): stream-ordered allocations, so
// that creating and destroying operators in several host threads never synchronises the whole
// device (cudaFree does), and small pinned host blocks recycled instead of freed.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace sgmev {

// stream-ordered allocation on `s` from the library's own memory pool on the current device
// (created once per device; it keeps freed memory for reuse and is trimmed when an allocation
// fails); *p is nullptr on failure
cudaError_t dev_malloc(void** p, size_t bytes, cudaStream_t s);

template <typename T>
inline cudaError_t dev_malloc(T** p, size_t bytes, cudaStream_t s) {
  return dev_malloc(reinterpret_cast<void**>(p), bytes, s);
}

// cudaFreeAsync on `s` (nullptr is accepted); the memory is reused once `s` reaches this point
void dev_free(void* p, cudaStream_t s);

// 64-byte pinned host blocks for scalars read back from the device
void* pinned_block();
void pinned_release(void* p);

}  // namespace sgmev
