// Runtime helpers shared by the engine's translation units.
//
// Device and pinned-host allocations of the engine, routed through the
// process-wide allocation hook of gelio_set_alloc_hook (include/gelio.h):
// a hook that refuses an allocation makes it fail with
// cudaErrorMemoryAllocation without calling CUDA, exactly as an exhausted
// device would, so callers report GELIO_ERR_OUT_OF_MEMORY.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

namespace gelio {

cudaError_t dev_malloc_raw(void **p, size_t bytes);
// Record a CUDA failure as the calling thread's gelio_last_error text.
void note_cuda_error(cudaError_t e, const char *file, int line);
cudaError_t pinned_malloc_raw(void **p, size_t bytes);

template <class T> inline cudaError_t dev_malloc(T **p, size_t bytes) {
  return dev_malloc_raw(reinterpret_cast<void **>(p), bytes);
}
template <class T> inline cudaError_t pinned_malloc(T **p, size_t bytes) {
  return pinned_malloc_raw(reinterpret_cast<void **>(p), bytes);
}

}  // namespace gelio
