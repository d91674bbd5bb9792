// Cooperative block-sandwich kernel for groups whose output tiles and inner dimensions
// are large (typical of C1 symmetry and of converged virtual dimensions).
//
// One CTA (256 threads, 16 x 16, each thread a 2 x 2 patch) per 32 x 32 output tile. Every
// (term, entry) item is evaluated as a chain of two shared-memory tiled GEMMs in the
// cheaper association: A (B C) builds a 32-row chunk of B C_p in shared memory and
// multiplies A_p's matching columns into the tile; (A B) C builds a 32-column chunk of
// A_p B. Operand chunks are staged through shared memory with coalesced loads. Each
// item's partial tile is added to an FP64 accumulator, scaled by its coefficient, in
// the fixed item order; the FP32 variant computes the items in FP32 from the FP32
// operand copies.
#include "kernels.cuh"
#include "slots.cuh"

namespace c2g {

namespace {

constexpr int kKC = 16;
constexpr int kTT = 256;

// element (i, k) of op(M) = t ? p[k + ld i] : p[i + ld k]
template <typename Real>
struct OpRef {
  const Real* p;
  int64_t ld;
  bool t;
  __device__ __forceinline__ Real at(int i, int k) const { return t ? p[k + ld * i] : p[i + ld * k]; }
  // the operand whose (i, k) is this one's (i + di, k + dk)
  __device__ __forceinline__ OpRef shift(int di, int dk) const {
    OpRef o = *this;
    o.p = t ? p + dk + ld * di : p + di + ld * dk;
    return o;
  }
};

template <typename Real>
struct Smem {
  Real Ls[kKC][kTile + 1];
  Real Rs[kKC][kTile + 1];
  Real Ts[kTile][kTile + 1];
};

// part (rows ty, ty+16; cols tx, tx+16) += sum_{k < K} L(i, k) R(k, j), i < M, j < N.
template <typename Real>
__device__ __forceinline__ void gemm_global(Real (&part)[2][2], const OpRef<Real>& L, int M, const OpRef<Real>& R,
                                            int N, int K, Smem<Real>& sm) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int k0 = 0; k0 < K; k0 += kKC) {
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const int e = tid + kTT * s;
      int i, kk;
      if (!L.t) { i = e & 31; kk = e >> 5; } else { kk = e & 15; i = e >> 4; }
      sm.Ls[kk][i] = (i < M && k0 + kk < K) ? L.at(i, k0 + kk) : Real(0);
      int j;
      if (!R.t) { kk = e & 15; j = e >> 4; } else { j = e & 31; kk = e >> 5; }
      sm.Rs[kk][j] = (j < N && k0 + kk < K) ? R.at(k0 + kk, j) : Real(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKC; kk++) {
      const Real a0 = sm.Ls[kk][ty], a1 = sm.Ls[kk][ty + 16];
      const Real b0 = sm.Rs[kk][tx], b1 = sm.Rs[kk][tx + 16];
      part[0][0] = fmaR(a0, b0, part[0][0]);
      part[0][1] = fmaR(a0, b1, part[0][1]);
      part[1][0] = fmaR(a1, b0, part[1][0]);
      part[1][1] = fmaR(a1, b1, part[1][1]);
    }
    __syncthreads();
  }
}

// part += Ts (rows i, columns k < K) R(k, j)
template <typename Real>
__device__ __forceinline__ void gemm_left_smem(Real (&part)[2][2], const OpRef<Real>& R, int N, int K,
                                               Smem<Real>& sm) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int k0 = 0; k0 < K; k0 += kKC) {
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const int e = tid + kTT * s;
      int j, kk;
      if (!R.t) { kk = e & 15; j = e >> 4; } else { j = e & 31; kk = e >> 5; }
      sm.Rs[kk][j] = (j < N && k0 + kk < K) ? R.at(k0 + kk, j) : Real(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKC; kk++) {
      const int k = k0 + kk;
      const Real a0 = (k < kTile) ? sm.Ts[ty][k] : Real(0), a1 = (k < kTile) ? sm.Ts[ty + 16][k] : Real(0);
      const Real b0 = sm.Rs[kk][tx], b1 = sm.Rs[kk][tx + 16];
      part[0][0] = fmaR(a0, b0, part[0][0]);
      part[0][1] = fmaR(a0, b1, part[0][1]);
      part[1][0] = fmaR(a1, b0, part[1][0]);
      part[1][1] = fmaR(a1, b1, part[1][1]);
    }
    __syncthreads();
  }
}

// part += L(i, k) Ts (rows k < K, columns j)
template <typename Real>
__device__ __forceinline__ void gemm_right_smem(Real (&part)[2][2], const OpRef<Real>& L, int M, int K,
                                                Smem<Real>& sm) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int k0 = 0; k0 < K; k0 += kKC) {
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const int e = tid + kTT * s;
      int i, kk;
      if (!L.t) { i = e & 31; kk = e >> 5; } else { kk = e & 15; i = e >> 4; }
      sm.Ls[kk][i] = (i < M && k0 + kk < K) ? L.at(i, k0 + kk) : Real(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKC; kk++) {
      const int k = k0 + kk;
      const Real a0 = sm.Ls[kk][ty], a1 = sm.Ls[kk][ty + 16];
      const Real b0 = (k < kTile) ? sm.Ts[k][tx] : Real(0), b1 = (k < kTile) ? sm.Ts[k][tx + 16] : Real(0);
      part[0][0] = fmaR(a0, b0, part[0][0]);
      part[0][1] = fmaR(a0, b1, part[0][1]);
      part[1][0] = fmaR(a1, b0, part[1][0]);
      part[1][1] = fmaR(a1, b1, part[1][1]);
    }
    __syncthreads();
  }
}

template <typename Real>
__device__ __forceinline__ void store_ts(const Real (&v)[2][2], Smem<Real>& sm) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  sm.Ts[ty][tx] = v[0][0];
  sm.Ts[ty][tx + 16] = v[0][1];
  sm.Ts[ty + 16][tx] = v[1][0];
  sm.Ts[ty + 16][tx + 16] = v[1][1];
  __syncthreads();
}

template <typename Real>
__global__ void __launch_bounds__(kTT) sandwich_tile_kernel(const Group* __restrict__ groups,
                                                            const Term* __restrict__ terms,
                                                            const BatchEntry* __restrict__ entries,
                                                            const TileDesc* __restrict__ tiles, SlotPtrs sp) {
  __shared__ Smem<Real> sm;
  const TileDesc td = tiles[blockIdx.x];
  const Group G = groups[td.group];
  const int row0 = (td.pos >> 16) * kTile, col0 = (td.pos & 0xffff) * kTile;
  const int tm = min(kTile, G.m - row0), tn = min(kTile, G.n - col0);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int t = G.t0; t < G.t1; t++) {
    const Term T = terms[t];
    const bool ha = T.flags & kHasA, hc = T.flags & kHasC;
    const OpRef<Real> B0{resolve<Real>(sp, T.b), T.ldb, (T.flags & kTransB) != 0};
    const Real* A0 = ha ? resolve<Real>(sp, T.a) : nullptr;
    const Real* C0 = hc ? resolve<Real>(sp, T.c) : nullptr;
    for (int p = 0; p < T.count; p++) {
      double al = T.alpha;
      const Real* Ap = A0;
      const Real* Cp = C0;
      if (T.list >= 0) {
        const BatchEntry e = entries[T.list + p];
        al *= e.ratio;
        if (Ap) Ap += e.da;
        if (Cp) Cp += e.dc;
      }
      const OpRef<Real> A{Ap, T.lda, (T.flags & kTransA) != 0};
      const OpRef<Real> C{Cp, T.ldc, (T.flags & kTransC) != 0};
      Real part[2][2] = {{Real(0), Real(0)}, {Real(0), Real(0)}};
      if (ha && hc) {
        if (T.flags & kLeftFirst) {
          for (int l0 = 0; l0 < T.k2; l0 += kTile) {
            const int lc = min(kTile, T.k2 - l0);
            Real s[2][2] = {{Real(0), Real(0)}, {Real(0), Real(0)}};
            gemm_global(s, A.shift(row0, 0), tm, B0.shift(0, l0), lc, T.k1, sm);
            store_ts(s, sm);
            gemm_left_smem(part, C.shift(l0, col0), tn, lc, sm);
          }
        } else {
          for (int k0 = 0; k0 < T.k1; k0 += kTile) {
            const int kc = min(kTile, T.k1 - k0);
            Real s[2][2] = {{Real(0), Real(0)}, {Real(0), Real(0)}};
            gemm_global(s, B0.shift(k0, 0), kc, C.shift(0, col0), tn, T.k2, sm);
            store_ts(s, sm);
            gemm_right_smem(part, A.shift(row0, k0), tm, kc, sm);
          }
        }
      } else if (ha) {
        gemm_global(part, A.shift(row0, 0), tm, B0.shift(0, col0), tn, T.k1, sm);
      } else if (hc) {
        gemm_global(part, B0.shift(row0, 0), tm, C.shift(0, col0), tn, T.k2, sm);
      } else {
#pragma unroll
        for (int ii = 0; ii < 2; ii++)
#pragma unroll
          for (int jj = 0; jj < 2; jj++) {
            const int r = ty + 16 * ii, c = tx + 16 * jj;
            part[ii][jj] = (r < tm && c < tn) ? B0.at(row0 + r, col0 + c) : Real(0);
          }
      }
#pragma unroll
      for (int ii = 0; ii < 2; ii++)
#pragma unroll
        for (int jj = 0; jj < 2; jj++) acc[ii][jj] = fma(al, static_cast<double>(part[ii][jj]), acc[ii][jj]);
    }
  }
  double* O = const_cast<double*>(resolve<double>(sp, G.out));
  const int64_t ldo = G.ldo;
  const bool accum = (G.flags & kAccumulate) != 0;
#pragma unroll
  for (int ii = 0; ii < 2; ii++)
#pragma unroll
    for (int jj = 0; jj < 2; jj++) {
      const int r = ty + 16 * ii, c = tx + 16 * jj;
      if (r < tm && c < tn) {
        const int64_t idx = (row0 + r) + ldo * (col0 + c);
        O[idx] = accum ? O[idx] + acc[ii][jj] : acc[ii][jj];
      }
    }
}

}  // namespace

cudaError_t launch_sandwich_tiles(const Group* groups, const Term* terms, const BatchEntry* entries,
                                  const TileDesc* tiles, int ntiles, const SlotPtrs& sp, cudaStream_t stream,
                                  Precision prec) {
  if (ntiles <= 0) return cudaSuccess;
  if (prec == Precision::kFP32)
    sandwich_tile_kernel<float><<<ntiles, kTT, 0, stream>>>(groups, terms, entries, tiles, sp);
  else
    sandwich_tile_kernel<double><<<ntiles, kTT, 0, stream>>>(groups, terms, entries, tiles, sp);
  return cudaGetLastError();
}

}  // namespace c2g
