// Resolution of task references (slot << 48 | offset) into device pointers, for the FP64
// operands and for their FP32 copies.
#pragma once

#include "kernels.cuh"

namespace c2g {

template <typename Real>
struct Tables;
template <>
struct Tables<double> {
  __device__ static const double* get(const SlotPtrs& sp, int s) {
    switch (s) {
      case kSlotX: return sp.x;
      case kSlotY: return sp.y;
      case kSlotCombo: return sp.combo;
      case kSlotOnes: return sp.ones;
      case kSlotInter: return sp.inter;
      default: return sp.table[s];
    }
  }
};
template <>
struct Tables<float> {
  __device__ static const float* get(const SlotPtrs& sp, int s) {
    switch (s) {
      case kSlotX: return sp.x32;
      case kSlotCombo: return sp.combo32;
      case kSlotOnes: return sp.ones32;
      case kSlotInter: return sp.inter32;
      default: return sp.table32[s];
    }
  }
};

template <typename Real>
__device__ __forceinline__ const Real* resolve(const SlotPtrs& sp, Ref r) {
  const int s = static_cast<int>(r >> kRefShift);
  const int64_t off = static_cast<int64_t>(r & kRefMask);
  return Tables<Real>::get(sp, s) + off;
}

__device__ __forceinline__ double fmaR(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaR(float a, float b, float c) { return fmaf(a, b, c); }

}  // namespace c2g
