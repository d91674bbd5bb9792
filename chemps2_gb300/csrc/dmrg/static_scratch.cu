// A file-scope device array used as staging memory by the allocation-free host-buffer
// matvec (DMRG::heff_apply_noalloc). Its device address is looked up once per device with
// cudaGetSymbolAddress and cached.
//
// Races: there is one array per device for the whole process. Two calls that use it at
// the same time (two host threads, or two DMRG objects whose streams overlap) overwrite
// each other's vectors. Every user synchronises its stream before it returns, so calls
// issued one after another from any number of DMRG objects are safe; concurrent calls
// are not and must be serialised by the caller.
#include "static_scratch.hpp"

#include <mutex>

namespace c2g {

namespace {

__device__ __align__(256) double g_static_scratch[kStaticScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_addr[kMaxDevices] = {};

}  // namespace

cudaError_t static_scratch(int dev, double** ptr) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_addr[dev]) {
    // the symbol's address is per device: look it up with `dev` current
    int cur = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return e;
    if (cur != dev && (e = cudaSetDevice(dev)) != cudaSuccess) return e;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (cur != dev) {
      const cudaError_t r = cudaSetDevice(cur);
      if (e == cudaSuccess) e = r;
    }
    if (e != cudaSuccess) return e;
    g_addr[dev] = static_cast<double*>(p);
  }
  *ptr = g_addr[dev];
  return cudaSuccess;
}

}  // namespace c2g
