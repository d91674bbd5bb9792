// Two-pass path of large groups (declarations and the scheme in kernels.cuh).
//
// Both passes run the same CTA-level GEMM on an output tile of at most 64 x 64 placed on
// a 64 x 64 grid: 256 threads in a 16 x 16 layout, thread (ty, tx) holding rows
// ty PM .. ty PM + PM - 1 and columns tx PN .. tx PN + PN - 1 of the tile, where PM and PN
// (1 to 4) are the tile's extents in units of 16, chosen per tile on the host. The
// operands are staged through shared memory in chunks of 16 along the inner dimension,
// loaded with the unit-stride index fastest for either storage order of each operand, and
// read back as contiguous runs (16-byte reads: one per operand and step for FP32 4 x 4).
// In FP64 the GEMM is bound by the FP64 pipe (two FMAs per SM and clock on this GPU), so
// no FMA may be issued twice or on padding: every intermediate is formed once in pass 1,
// tile extents follow the block to 16 columns, and warps whose rows lie past the block
// skip the multiply-adds altogether.
#include "kernels.cuh"
#include "slots.cuh"

namespace c2g {

namespace {

constexpr int kKC = 16;

template <typename Real>
struct Opnd {
  const Real* p;
  int64_t ld;
  bool t;
  __device__ __forceinline__ Real at(int i, int k) const { return t ? p[k + ld * i] : p[i + ld * k]; }
  __device__ __forceinline__ Opnd shift(int di, int dk) const {
    Opnd o = *this;
    o.p = t ? p + dk + ld * di : p + di + ld * dk;
    return o;
  }
};

template <typename Real>
__device__ __forceinline__ Opnd<Real> opnd(const SlotPtrs& sp, const GemmOperand& g) {
  return Opnd<Real>{resolve<Real>(sp, g.ref), g.ld, g.trans != 0};
}

// rows of 68 elements keep every row 16-byte aligned for vector reads (FP32 and FP64)
constexpr int kGLd = 68;
template <typename Real>
struct __align__(16) GSmem {
  Real L[kKC][kGLd];
  Real R[kKC][kGLd];
};

// v[0 .. P) = p[0 .. P) from shared memory, in 16-byte (or 8-byte) reads where the run's
// length and alignment allow (p is aligned to P elements)
template <int P>
__device__ __forceinline__ void lds_run(float (&v)[P], const float* p) {
  if constexpr (P == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else if constexpr (P == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = t.x; v[1] = t.y;
  } else {
#pragma unroll
    for (int i = 0; i < P; i++) v[i] = p[i];
  }
}
template <int P>
__device__ __forceinline__ void lds_run(double (&v)[P], const double* p) {
  if constexpr (P == 2 || P == 4) {
#pragma unroll
    for (int i = 0; i < P; i += 2) {
      const double2 t = *reinterpret_cast<const double2*>(p + i);
      v[i] = t.x;
      v[i + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < P; i++) v[i] = p[i];
  }
}

// One 16-deep chunk of the operands of a tile GEMM, staged in registers: the global
// loads of the next chunk are issued before the current chunk's multiply-adds, so their
// latency overlaps that work (also across item boundaries in pass 2).
template <typename Real, int PM, int PN>
struct ChunkRegs {
  Real l[PM], r[PN];
};

template <typename Real, int PM, int PN>
__device__ __forceinline__ void fetch_chunk(ChunkRegs<Real, PM, PN>& g, const Opnd<Real>& L, int M, const Opnd<Real>& R,
                                            int N, int K, int k0) {
  constexpr int TM = 16 * PM, TN = 16 * PN;
  const int tid = threadIdx.x;
#pragma unroll
  for (int s = 0; s < PM; s++) {
    const int e = tid + kGemmThreads * s;
    const int i = L.t ? e / kKC : e % TM, kk = L.t ? e % kKC : e / TM;
    g.l[s] = (i < M && k0 + kk < K) ? L.at(i, k0 + kk) : Real(0);
  }
#pragma unroll
  for (int s = 0; s < PN; s++) {
    const int e = tid + kGemmThreads * s;
    const int j = R.t ? e % TN : e / kKC, kk = R.t ? e / TN : e % kKC;
    g.r[s] = (j < N && k0 + kk < K) ? R.at(k0 + kk, j) : Real(0);
  }
}

template <typename Real, int PM, int PN>
__device__ __forceinline__ void store_chunk(const ChunkRegs<Real, PM, PN>& g, bool lt, bool rt, GSmem<Real>& sm) {
  constexpr int TM = 16 * PM, TN = 16 * PN;
  const int tid = threadIdx.x;
#pragma unroll
  for (int s = 0; s < PM; s++) {
    const int e = tid + kGemmThreads * s;
    const int i = lt ? e / kKC : e % TM, kk = lt ? e % kKC : e / TM;
    sm.L[kk][i] = g.l[s];
  }
#pragma unroll
  for (int s = 0; s < PN; s++) {
    const int e = tid + kGemmThreads * s;
    const int j = rt ? e % TN : e / kKC, kk = rt ? e / TN : e % kKC;
    sm.R[kk][j] = g.r[s];
  }
}

// part (rows ty PM + ii, columns tx PN + jj) = sum_{k < K} L(i, k) R(k, j) over i < M,
// j < N (zero elsewhere); M <= 16 PM, N <= 16 PN. The next chunk's loads are in flight
// while the current chunk is multiplied.
template <typename Real, int PM, int PN>
__device__ __forceinline__ void tile_gemm(Real (&part)[PM][PN], const Opnd<Real>& L, int M, const Opnd<Real>& R,
                                          int N, int K, GSmem<Real>& sm) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  // a warp holds rows (ty & ~1) PM .. (ty | 1) PM + PM - 1
  const bool active = (ty & ~1) * PM < M;
#pragma unroll
  for (int ii = 0; ii < PM; ii++)
#pragma unroll
    for (int jj = 0; jj < PN; jj++) part[ii][jj] = Real(0);
  if (K <= 0) return;
  ChunkRegs<Real, PM, PN> g;
  fetch_chunk<Real, PM, PN>(g, L, M, R, N, K, 0);
  for (int k0 = 0; k0 < K; k0 += kKC) {
    store_chunk<Real, PM, PN>(g, L.t, R.t, sm);
    __syncthreads();
    if (k0 + kKC < K) fetch_chunk<Real, PM, PN>(g, L, M, R, N, K, k0 + kKC);
    if (active) {
      const int kn = min(kKC, K - k0);
      for (int kk = 0; kk < kn; kk++) {
        Real a[PM], b[PN];
        lds_run<PM>(a, &sm.L[kk][ty * PM]);
        lds_run<PN>(b, &sm.R[kk][tx * PN]);
#pragma unroll
        for (int ii = 0; ii < PM; ii++)
#pragma unroll
          for (int jj = 0; jj < PN; jj++) part[ii][jj] = fmaR(a[ii], b[jj], part[ii][jj]);
      }
    }
    __syncthreads();
  }
}

template <typename Real, int PM, int PN>
__device__ __forceinline__ void inter_tile(const InterJob& J, int pos, const SlotPtrs& sp, GSmem<Real>& sm) {
  constexpr int TM = 16 * PM, TN = 16 * PN;
  const int row0 = (pos >> 16) * 64, col0 = (pos & 0xffff) * 64;
  const int tm = min(TM, J.m - row0), tn = min(TN, J.n - col0);
  Real part[PM][PN];
  tile_gemm<Real, PM, PN>(part, opnd<Real>(sp, J.l).shift(row0, 0), tm, opnd<Real>(sp, J.r).shift(0, col0), tn, J.k,
                          sm);
  Real* S = const_cast<Real*>(Tables<Real>::get(sp, kSlotInter)) + J.off;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
#pragma unroll
  for (int ii = 0; ii < PM; ii++)
#pragma unroll
    for (int jj = 0; jj < PN; jj++) {
      const int r = ty * PM + ii, c = tx * PN + jj;
      if (r < tm && c < tn) S[(row0 + r) + static_cast<int64_t>(J.m) * (col0 + c)] = part[ii][jj];
    }
}

template <typename Real>
__global__ void __launch_bounds__(kGemmThreads, sizeof(Real) == 4 ? 3 : 2)
    inter_gemm_kernel(const InterJob* __restrict__ jobs, const GemmTile* __restrict__ tiles, SlotPtrs sp) {
  __shared__ GSmem<Real> sm;
  const GemmTile T = tiles[blockIdx.x];
  const InterJob J = jobs[T.idx];
  // shape = (PM - 1) | (PN - 1) << 2
#define C2G_INTER(pm, pn) \
  case (pm - 1) | ((pn - 1) << 2): inter_tile<Real, pm, pn>(J, T.pos, sp, sm); break;
  switch (T.shape) {
    C2G_INTER(1, 1) C2G_INTER(2, 1) C2G_INTER(3, 1) C2G_INTER(4, 1)
    C2G_INTER(1, 2) C2G_INTER(2, 2) C2G_INTER(3, 2) C2G_INTER(4, 2)
    C2G_INTER(1, 3) C2G_INTER(2, 3) C2G_INTER(3, 3) C2G_INTER(4, 3)
    C2G_INTER(1, 4) C2G_INTER(2, 4) C2G_INTER(3, 4) C2G_INTER(4, 4)
    default: break;
  }
#undef C2G_INTER
}

// Pass 1 for small jobs (m n <= 256): one warp per job, each lane a run of output
// elements, each element a dot product over k read straight from global memory (L1).
// A tile-shaped CTA would spend most of its time staging a few operand values; here no
// multiply-add runs on padding except in the last group of 32 elements, and in FP64 two
// loads per multiply-add stay below what the FP64 pipe consumes.
template <typename Real, int NQ>
__device__ __forceinline__ void small_job(const InterJob& J, const SlotPtrs& sp, int lane) {
  // element (i, k) of op(M) at M + i si + k sk
  const int64_t lsi = J.l.trans ? J.l.ld : 1, lsk = J.l.trans ? 1 : J.l.ld;
  const int64_t rsk = J.r.trans ? J.r.ld : 1, rsj = J.r.trans ? 1 : J.r.ld;
  const Real* L = resolve<Real>(sp, J.l.ref);
  const Real* R = resolve<Real>(sp, J.r.ref);
  const int mn = J.m * J.n;
  const Real* lp[NQ];
  const Real* rp[NQ];
  Real acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int e = min(lane + 32 * q, mn - 1);  // lanes past the end repeat the last element
    lp[q] = L + (e % J.m) * lsi;
    rp[q] = R + (e / J.m) * rsj;
    acc[q] = Real(0);
  }
  for (int k = 0; k < J.k; k++) {
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      acc[q] = fmaR(*lp[q], *rp[q], acc[q]);
      lp[q] += lsk;
      rp[q] += rsk;
    }
  }
  Real* S = const_cast<Real*>(Tables<Real>::get(sp, kSlotInter)) + J.off;
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int e = lane + 32 * q;
    if (e < mn) S[(e % J.m) + static_cast<int64_t>(J.m) * (e / J.m)] = acc[q];
  }
}

template <typename Real>
__global__ void __launch_bounds__(256, 2)
    inter_small_kernel(const InterJob* __restrict__ jobs, const int32_t* __restrict__ list, int njobs, SlotPtrs sp) {
  const int w = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (w >= njobs) return;
  const InterJob J = jobs[list[w]];
  const int lane = threadIdx.x & 31;
  switch ((J.m * J.n + 31) / 32) {
    case 1: small_job<Real, 1>(J, sp, lane); break;
    case 2: small_job<Real, 2>(J, sp, lane); break;
    case 3: small_job<Real, 3>(J, sp, lane); break;
    case 4: small_job<Real, 4>(J, sp, lane); break;
    case 5: small_job<Real, 5>(J, sp, lane); break;
    case 6: small_job<Real, 6>(J, sp, lane); break;
    case 7: small_job<Real, 7>(J, sp, lane); break;
    case 8: small_job<Real, 8>(J, sp, lane); break;
    default: break;
  }
}

template <typename Real, int PM, int PN>
__device__ __forceinline__ void sum_tile(const GemmTile& T, const SumGroup& G, const SumItem* __restrict__ items,
                                         double* partials, unsigned int* counters, const SlotPtrs& sp,
                                         GSmem<Real>& sm) {
  constexpr int TM = 16 * PM, TN = 16 * PN;
  const int row0 = (T.pos >> 16) * 64, col0 = (T.pos & 0xffff) * 64;
  const int tm = min(TM, G.m - row0), tn = min(TN, G.n - col0);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const bool active = (ty & ~1) * PM < tm;  // the warp holds rows of the block
  double acc[PM][PN];
#pragma unroll
  for (int ii = 0; ii < PM; ii++)
#pragma unroll
    for (int jj = 0; jj < PN; jj++) acc[ii][jj] = 0.0;
  // items without an inner dimension: out += alpha op(R), straight from global memory
  auto add_copy = [&](const SumItem& I) {
    const Opnd<Real> R = opnd<Real>(sp, I.r);
#pragma unroll
    for (int ii = 0; ii < PM; ii++)
#pragma unroll
      for (int jj = 0; jj < PN; jj++) {
        const int r = ty * PM + ii, c = tx * PN + jj;
        if (r < tm && c < tn) acc[ii][jj] = fma(I.alpha, static_cast<double>(R.at(row0 + r, col0 + c)), acc[ii][jj]);
      }
  };
  // the GEMM items, chunk by chunk, with the next chunk's loads in flight
  int it = T.item0;
  SumItem cur{};
  bool have = false;
  for (; it < T.item1; it++) {
    cur = items[it];
    if (cur.k > 0) {
      have = true;
      break;
    }
    add_copy(cur);
  }
  if (have) {
    Opnd<Real> cL = opnd<Real>(sp, cur.l).shift(row0, 0), cR = opnd<Real>(sp, cur.r).shift(0, col0);
    int k0 = 0;
    ChunkRegs<Real, PM, PN> g;
    fetch_chunk<Real, PM, PN>(g, cL, tm, cR, tn, cur.k, 0);
    Real part[PM][PN];
#pragma unroll
    for (int ii = 0; ii < PM; ii++)
#pragma unroll
      for (int jj = 0; jj < PN; jj++) part[ii][jj] = Real(0);
    for (;;) {
      store_chunk<Real, PM, PN>(g, cL.t, cR.t, sm);
      __syncthreads();
      const int kn = min(kKC, cur.k - k0);
      const bool last = k0 + kKC >= cur.k;
      SumItem nxt = cur;
      Opnd<Real> nL = cL, nR = cR;
      int nk0 = k0 + kKC;
      bool more = true;
      if (last) {
        more = false;
        for (int j = it + 1; j < T.item1; j++) {
          const SumItem c2 = items[j];
          if (c2.k > 0) {
            nxt = c2;
            it = j;
            more = true;
            break;
          }
          add_copy(c2);
        }
        if (more) {
          nL = opnd<Real>(sp, nxt.l).shift(row0, 0);
          nR = opnd<Real>(sp, nxt.r).shift(0, col0);
          nk0 = 0;
        }
      }
      if (more) fetch_chunk<Real, PM, PN>(g, nL, tm, nR, tn, nxt.k, nk0);
      if (active) {
        for (int kk = 0; kk < kn; kk++) {
          Real a[PM], b[PN];
          lds_run<PM>(a, &sm.L[kk][ty * PM]);
          lds_run<PN>(b, &sm.R[kk][tx * PN]);
#pragma unroll
          for (int ii = 0; ii < PM; ii++)
#pragma unroll
            for (int jj = 0; jj < PN; jj++) part[ii][jj] = fmaR(a[ii], b[jj], part[ii][jj]);
        }
      }
      if (last) {
#pragma unroll
        for (int ii = 0; ii < PM; ii++)
#pragma unroll
          for (int jj = 0; jj < PN; jj++) {
            acc[ii][jj] = fma(cur.alpha, static_cast<double>(part[ii][jj]), acc[ii][jj]);
            part[ii][jj] = Real(0);
          }
      }
      __syncthreads();
      if (!more) break;
      cur = nxt;
      cL = nL;
      cR = nR;
      k0 = nk0;
    }
  }
  if (T.nsplit > 1) {
    // store this split's partial tile; the last split to arrive adds them up in split order
    double* part = partials + T.part;
    constexpr int te = TM * TN;
#pragma unroll
    for (int ii = 0; ii < PM; ii++)
#pragma unroll
      for (int jj = 0; jj < PN; jj++)
        __stcg(part + static_cast<int64_t>(T.split) * te + (ty * PM + ii) + TM * (tx * PN + jj), acc[ii][jj]);
    __threadfence();
    __shared__ int is_last;
    __syncthreads();
    if (tid == 0) is_last = atomicAdd(counters + T.counter, 1u) == static_cast<unsigned>(T.nsplit - 1);
    __syncthreads();
    if (!is_last) return;
    __threadfence();
#pragma unroll
    for (int ii = 0; ii < PM; ii++)
#pragma unroll
      for (int jj = 0; jj < PN; jj++) {
        double v = 0.0;
        for (int s = 0; s < T.nsplit; s++)
          v += __ldcg(part + static_cast<int64_t>(s) * te + (ty * PM + ii) + TM * (tx * PN + jj));
        acc[ii][jj] = v;
      }
    if (tid == 0) counters[T.counter] = 0u;  // ready for the next launch
  }
  double* O = const_cast<double*>(resolve<double>(sp, G.out));
  const int64_t ldo = G.ldo;
  const bool accum = (G.flags & kAccumulate) != 0;
#pragma unroll
  for (int ii = 0; ii < PM; ii++)
#pragma unroll
    for (int jj = 0; jj < PN; jj++) {
      const int r = ty * PM + ii, c = tx * PN + jj;
      if (r < tm && c < tn) {
        const int64_t idx = (row0 + r) + ldo * (col0 + c);
        O[idx] = accum ? O[idx] + acc[ii][jj] : acc[ii][jj];
      }
    }
}

template <typename Real>
__global__ void __launch_bounds__(kGemmThreads, 2)
    sum_gemm_kernel(const SumGroup* __restrict__ groups, const SumItem* __restrict__ items,
                    const GemmTile* __restrict__ tiles, double* partials, unsigned int* counters, SlotPtrs sp) {
  __shared__ GSmem<Real> sm;
  const GemmTile T = tiles[blockIdx.x];
  const SumGroup G = groups[T.idx];
#define C2G_SUM(pm, pn) \
  case (pm - 1) | ((pn - 1) << 2): sum_tile<Real, pm, pn>(T, G, items, partials, counters, sp, sm); break;
  switch (T.shape) {
    C2G_SUM(1, 1) C2G_SUM(2, 1) C2G_SUM(3, 1) C2G_SUM(4, 1)
    C2G_SUM(1, 2) C2G_SUM(2, 2) C2G_SUM(3, 2) C2G_SUM(4, 2)
    C2G_SUM(1, 3) C2G_SUM(2, 3) C2G_SUM(3, 3) C2G_SUM(4, 3)
    C2G_SUM(1, 4) C2G_SUM(2, 4) C2G_SUM(3, 4) C2G_SUM(4, 4)
    default: break;
  }
#undef C2G_SUM
}

}  // namespace

cudaError_t launch_inter_gemm(const InterJob* jobs, const GemmTile* tiles, int ntiles, const SlotPtrs& sp,
                              cudaStream_t stream, Precision prec) {
  if (ntiles <= 0) return cudaSuccess;
  if (prec == Precision::kFP32)
    inter_gemm_kernel<float><<<ntiles, kGemmThreads, 0, stream>>>(jobs, tiles, sp);
  else
    inter_gemm_kernel<double><<<ntiles, kGemmThreads, 0, stream>>>(jobs, tiles, sp);
  return cudaGetLastError();
}

cudaError_t launch_inter_small(const InterJob* jobs, const int32_t* list, int njobs, const SlotPtrs& sp,
                               cudaStream_t stream, Precision prec) {
  if (njobs <= 0) return cudaSuccess;
  const int grid = (njobs + 7) / 8;
  if (prec == Precision::kFP32)
    inter_small_kernel<float><<<grid, 256, 0, stream>>>(jobs, list, njobs, sp);
  else
    inter_small_kernel<double><<<grid, 256, 0, stream>>>(jobs, list, njobs, sp);
  return cudaGetLastError();
}

cudaError_t launch_sum_gemm(const SumGroup* groups, const SumItem* items, const GemmTile* tiles, int ntiles,
                            double* partials, unsigned int* counters, const SlotPtrs& sp, cudaStream_t stream,
                            Precision prec) {
  if (ntiles <= 0) return cudaSuccess;
  if (prec == Precision::kFP32)
    sum_gemm_kernel<float><<<ntiles, kGemmThreads, 0, stream>>>(groups, items, tiles, partials, counters, sp);
  else
    sum_gemm_kernel<double><<<ntiles, kGemmThreads, 0, stream>>>(groups, items, tiles, partials, counters, sp);
  return cudaGetLastError();
}

}  // namespace c2g
