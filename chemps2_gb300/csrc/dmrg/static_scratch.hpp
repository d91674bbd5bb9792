// Process-wide static device scratch (static_scratch.cu): no allocation at run time.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace c2g {

// 16 MiB: two vectors of up to 1 M doubles each.
constexpr int64_t kStaticScratchDoubles = int64_t(1) << 21;
// Longest vector the allocation-free matvec takes: x, then y from the next 256-byte
// boundary, both inside the array (1 048 544 doubles).
constexpr int64_t kStaticScratchMaxVector = kStaticScratchDoubles / 2 - 32;

// Device address of the scratch on device `dev` (cudaGetSymbolAddress with that device
// current, once per device; the calling thread's current device is restored). Not
// thread-safe to *use* concurrently; see static_scratch.cu.
cudaError_t static_scratch(int dev, double** ptr);

}  // namespace c2g
