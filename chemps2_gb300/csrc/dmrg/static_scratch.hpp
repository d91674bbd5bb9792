// Process-wide static device scratch (static_scratch.cu): no allocation at run time.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace c2g {

// 16 MiB: two vectors of up to 1 M doubles each.
constexpr int64_t kStaticScratchDoubles = int64_t(1) << 21;

// Device address of the scratch on the current device (cudaGetSymbolAddress, once per
// device). Not thread-safe to *use* concurrently; see static_scratch.cu.
cudaError_t static_scratch(double** ptr);

}  // namespace c2g
