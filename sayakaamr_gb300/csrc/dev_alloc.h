// Device memory of the solvers, from the device's default memory pool (the
// stream-ordered allocator) with its release threshold raised: memory that a
// destroyed solver gives back stays in the pool and serves the next solver
// without a round trip through the driver (a sequence that builds a solver
// per regrid allocates and frees gigabytes each time).  Allocation is
// ordered on the legacy default stream and complete when the call returns;
// release first waits for the device to be idle, as cudaFree does, so the
// memory is usable from, and safe to release after, any stream.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace sayaka_gb300 {

cudaError_t dev_malloc_bytes(void **p, size_t bytes);
cudaError_t dev_free(void *p);

template <typename T>
inline cudaError_t dev_malloc(T **p, size_t bytes) {
  return dev_malloc_bytes(reinterpret_cast<void **>(p), bytes);
}

}  // namespace sayaka_gb300
