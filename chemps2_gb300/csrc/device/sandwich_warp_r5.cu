// Team-cooperative block-sandwich kernels of row class 5 (sandwich_warp.cuh).
#include "sandwich_warp.cuh"

namespace c2g {
template cudaError_t launch_sandwich_warp_class<5>(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&,
                                                   cudaStream_t, Precision);
}  // namespace c2g
