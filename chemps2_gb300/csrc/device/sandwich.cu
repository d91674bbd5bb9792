// The block-sandwich kernel: executes one stage of a task program.
//
// FP64 variant: FP64 operands and arithmetic. FP32 variant: reads the FP32 copies of the
// operands (SlotPtrs::table32, x32, combo32) and multiplies / sums in FP32 inside each
// lane, so its item loop issues no FP64 instruction (on GB300 the FP64 pipe is the
// bottleneck of the FP64 variant); the lane reduction and the update of the FP64 output
// stay in FP64.
#include "kernels.cuh"
#include "slots.cuh"

namespace c2g {

namespace {

// acc[ii][jj] (rows i0 + ii, ii < r; columns j0 + jj, jj < c) += one entry of a term.
template <typename Real>
__device__ __forceinline__ void sandwich_item(Real (&acc)[kSub][kSub], const Term& T, const Real* __restrict__ A,
                                              const Real* __restrict__ B, const Real* __restrict__ C, Real al, int i0,
                                              int j0, int r, int c) {
  const bool ha = T.flags & kHasA, hc = T.flags & kHasC;
  const bool ta = T.flags & kTransA, tb = T.flags & kTransB, tc = T.flags & kTransC;
  const int64_t lda = T.lda, ldb = T.ldb, ldc = T.ldc;
  auto opA = [&](int i, int k) { return ta ? A[k + lda * i] : A[i + lda * k]; };
  auto opB = [&](int k, int l) { return tb ? B[l + ldb * k] : B[k + ldb * l]; };
  auto opC = [&](int l, int j) { return tc ? C[j + ldc * l] : C[l + ldc * j]; };
  if (ha && hc) {
    if (T.flags & kLeftFirst) {
      for (int l = 0; l < T.k2; l++) {
        Real s[kSub];
#pragma unroll
        for (int ii = 0; ii < kSub; ii++) s[ii] = Real(0);
        for (int k = 0; k < T.k1; k++) {
          const Real b = opB(k, l);
#pragma unroll
          for (int ii = 0; ii < kSub; ii++)
            if (ii < r) s[ii] = fmaR(opA(i0 + ii, k), b, s[ii]);
        }
#pragma unroll
        for (int jj = 0; jj < kSub; jj++) {
          if (jj >= c) break;
          const Real cv = al * opC(l, j0 + jj);
#pragma unroll
          for (int ii = 0; ii < kSub; ii++)
            if (ii < r) acc[ii][jj] = fmaR(s[ii], cv, acc[ii][jj]);
        }
      }
    } else {
      for (int k = 0; k < T.k1; k++) {
        Real t[kSub];
#pragma unroll
        for (int jj = 0; jj < kSub; jj++) t[jj] = Real(0);
        for (int l = 0; l < T.k2; l++) {
          const Real b = opB(k, l);
#pragma unroll
          for (int jj = 0; jj < kSub; jj++)
            if (jj < c) t[jj] = fmaR(b, opC(l, j0 + jj), t[jj]);
        }
#pragma unroll
        for (int ii = 0; ii < kSub; ii++) {
          if (ii >= r) break;
          const Real av = al * opA(i0 + ii, k);
#pragma unroll
          for (int jj = 0; jj < kSub; jj++)
            if (jj < c) acc[ii][jj] = fmaR(av, t[jj], acc[ii][jj]);
        }
      }
    }
  } else if (ha) {
    for (int k = 0; k < T.k1; k++) {
      Real bv[kSub];
#pragma unroll
      for (int jj = 0; jj < kSub; jj++) bv[jj] = (jj < c) ? al * opB(k, j0 + jj) : Real(0);
#pragma unroll
      for (int ii = 0; ii < kSub; ii++) {
        if (ii >= r) break;
        const Real av = opA(i0 + ii, k);
#pragma unroll
        for (int jj = 0; jj < kSub; jj++)
          if (jj < c) acc[ii][jj] = fmaR(av, bv[jj], acc[ii][jj]);
      }
    }
  } else if (hc) {
    for (int l = 0; l < T.k2; l++) {
      Real cv[kSub];
#pragma unroll
      for (int jj = 0; jj < kSub; jj++) cv[jj] = (jj < c) ? al * opC(l, j0 + jj) : Real(0);
#pragma unroll
      for (int ii = 0; ii < kSub; ii++) {
        if (ii >= r) break;
        const Real b = opB(i0 + ii, l);
#pragma unroll
        for (int jj = 0; jj < kSub; jj++)
          if (jj < c) acc[ii][jj] = fmaR(b, cv[jj], acc[ii][jj]);
      }
    }
  } else {
#pragma unroll
    for (int ii = 0; ii < kSub; ii++) {
      if (ii >= r) break;
#pragma unroll
      for (int jj = 0; jj < kSub; jj++)
        if (jj < c) acc[ii][jj] = fmaR(al, opB(i0 + ii, j0 + jj), acc[ii][jj]);
    }
  }
}

template <typename Real>
__global__ void __launch_bounds__(kSandwichThreads) sandwich_kernel(const Group* __restrict__ groups,
                                                                    const Term* __restrict__ terms,
                                                                    const BatchEntry* __restrict__ entries,
                                                                    const TileDesc* __restrict__ tiles, SlotPtrs sp) {
  __shared__ double red[kSandwichThreads * kSub * kSub];
  const TileDesc td = tiles[blockIdx.x];
  const Group G = groups[td.group];
  const int row0 = (td.pos >> 16) * kTile, col0 = (td.pos & 0xffff) * kTile;
  const int tm = min(kTile, G.m - row0), tn = min(kTile, G.n - col0);
  const int sr = td.grid >> 8, sc = td.grid & 0xff;
  const int S = sr * sc;
  const int P = kSandwichThreads / S;
  const int tid = threadIdx.x;
  const int s = tid % S, lane = tid / S;
  const int si = s % sr, sj = s / sr;
  const int i0 = row0 + si * kSub, j0 = col0 + sj * kSub;
  const int r = max(0, min(kSub, row0 + tm - i0)), c = max(0, min(kSub, col0 + tn - j0));
  Real acc[kSub][kSub];
#pragma unroll
  for (int ii = 0; ii < kSub; ii++)
#pragma unroll
    for (int jj = 0; jj < kSub; jj++) acc[ii][jj] = Real(0);
  if (lane < P && r > 0 && c > 0 && G.t1 > G.t0) {
    const Term& last = terms[G.t1 - 1];
    const int total = last.item0 + last.count;
    const int chunk = (total + P - 1) / P;
    const int start = lane * chunk;
    const int stop = min(total, start + chunk);
    if (start < stop) {
      int lo = G.t0, hi = G.t1 - 1;  // last term with item0 <= start
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (terms[mid].item0 <= start) lo = mid;
        else hi = mid - 1;
      }
      int t = lo;
      Term T = terms[t];
      const Real* B = resolve<Real>(sp, T.b);
      const Real* A0 = (T.flags & kHasA) ? resolve<Real>(sp, T.a) : nullptr;
      const Real* C0 = (T.flags & kHasC) ? resolve<Real>(sp, T.c) : nullptr;
      Real alpha = static_cast<Real>(T.alpha);
      for (int item = start; item < stop; item++) {
        int p = item - T.item0;
        if (p >= T.count) {
          T = terms[++t];
          B = resolve<Real>(sp, T.b);
          A0 = (T.flags & kHasA) ? resolve<Real>(sp, T.a) : nullptr;
          C0 = (T.flags & kHasC) ? resolve<Real>(sp, T.c) : nullptr;
          alpha = static_cast<Real>(T.alpha);
          p = 0;
        }
        Real al = alpha;
        const Real* A = A0;
        const Real* C = C0;
        if (T.list >= 0) {
          const BatchEntry e = entries[T.list + p];
          if (e.ratio != 1.0) al = static_cast<Real>(T.alpha * e.ratio);
          if (A) A += e.da;
          if (C) C += e.dc;
        }
        sandwich_item<Real>(acc, T, A, B, C, al, i0, j0, r, c);
      }
    }
  }
#pragma unroll
  for (int ii = 0; ii < kSub; ii++)
#pragma unroll
    for (int jj = 0; jj < kSub; jj++) red[tid * kSub * kSub + ii * kSub + jj] = static_cast<double>(acc[ii][jj]);
  __syncthreads();
  // the output is FP64 in both variants
  double* O = const_cast<double*>(resolve<double>(sp, G.out));
  const int64_t ldo = G.ldo;
  const bool accum = (G.flags & kAccumulate) != 0;
  for (int e = tid; e < tm * tn; e += kSandwichThreads) {
    const int ii = e % tm, jj = e / tm;
    const int sub = (ii / kSub) + sr * (jj / kSub);
    const int w = (ii % kSub) * kSub + (jj % kSub);
    double v = 0.0;
    for (int l = 0; l < P; l++) v += red[(sub + S * l) * kSub * kSub + w];
    const int64_t idx = (row0 + ii) + ldo * (col0 + jj);
    O[idx] = accum ? O[idx] + v : v;
  }
}

__global__ void to_f32_kernel(float* __restrict__ dst, const double* __restrict__ src, int64_t n) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    dst[i] = static_cast<float>(src[i]);
}

}  // namespace

cudaError_t launch_sandwich(const Group* groups, const Term* terms, const BatchEntry* entries, const TileDesc* tiles,
                            int ntiles, const SlotPtrs& sp, cudaStream_t stream, Precision prec) {
  if (ntiles <= 0) return cudaSuccess;
  if (prec == Precision::kFP32)
    sandwich_kernel<float><<<ntiles, kSandwichThreads, 0, stream>>>(groups, terms, entries, tiles, sp);
  else
    sandwich_kernel<double><<<ntiles, kSandwichThreads, 0, stream>>>(groups, terms, entries, tiles, sp);
  return cudaGetLastError();
}

cudaError_t launch_to_f32(float* dst, const double* src, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  to_f32_kernel<<<static_cast<int>(blocks), 256, 0, stream>>>(dst, src, n);
  return cudaGetLastError();
}

}  // namespace c2g
