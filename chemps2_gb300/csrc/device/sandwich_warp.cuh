// Team-cooperative block-sandwich kernel for output tiles up to 16 x 16.
//
// One 128-thread CTA per (group, tile). The host picks the tile's capacity class: GR x GC
// lanes form a team, each lane owning a PR x PC patch (rows lr + GR i, columns lc + GC j)
// of an (GR PR) x (GC PC) tile; the classes cover tile edges of 2, 4, 6, 8, 12, 16 rows and
// 2, 4, 8, 12, 16 columns. A team evaluates one (term, entry) item at a time; a warp
// holds 32 / (GR GC) teams and the CTA's teams ("slots") take the group's items round
// robin (slot s: items s, s + NS, ...), so that neighbouring teams mostly evaluate items
// of one term shape. For a three-operand item the team builds its intermediate (a column
// chunk of A B, or a row chunk of B C, scaled by the item's coefficient) once in shared
// memory and multiplies it into the patch: every multiply-add of the fused contraction is
// executed once. The slots' partial tiles are summed in a fixed order at the end, so the
// result is deterministic.
#pragma once

#include "kernels.cuh"
#include "slots.cuh"

namespace c2g {

namespace {

constexpr int kWT = 128;     // threads per CTA
constexpr int kWBuf = 2048;  // doubles of shared scratch (intermediates, then the slot sums)

template <int GR_, int PR_, int GC_, int PC_>
struct Geo {
  static constexpr int PR = PR_, PC = PC_, GR = GR_, GC = GC_;
  static constexpr int RC = GR * PR, CC = GC * PC;   // tile capacity
  static constexpr int TEAM = GR * GC;               // lanes per item
  static constexpr int TEAMS = 32 / TEAM;            // teams per warp
  static constexpr int NS = (kWT / 32) * TEAMS;      // slots per CTA
  static constexpr int LDX = CC >= 8 ? CC + 1 : CC;  // row stride of a slot's intermediate
  static_assert(TEAM <= 32 && 32 % TEAM == 0, "team must divide a warp");
  static_assert(NS * RC * LDX <= kWBuf, "intermediates exceed the shared scratch");
  static_assert(NS * RC * CC <= kWBuf, "slot sums exceed the shared scratch");
};

// x(i, j) += sum_{k < K} L[ri_i * lr + k * lk] * R[k * rk + cj_j * rc] for the lane's patch
// rows ri (valid where vr) and columns cj (valid where vc); invalid rows / columns read 0.
template <typename Real, int PR, int PC>
__device__ __forceinline__ void patch_gemm(Real (&x)[PR][PC], const Real* L, int64_t lr, int64_t lk,
                                           const int (&ri)[PR], const bool (&vr)[PR], const Real* R, int64_t rk,
                                           int64_t rc, const int (&cj)[PC], const bool (&vc)[PC], int K) {
  int64_t lo[PR], ro[PC];
#pragma unroll
  for (int i = 0; i < PR; i++) lo[i] = ri[i] * lr;
#pragma unroll
  for (int j = 0; j < PC; j++) ro[j] = cj[j] * rc;
#pragma unroll 2
  for (int k = 0; k < K; k++) {
    Real a[PR], b[PC];
#pragma unroll
    for (int i = 0; i < PR; i++) a[i] = vr[i] ? L[lo[i]] : Real(0);
#pragma unroll
    for (int j = 0; j < PC; j++) b[j] = vc[j] ? R[ro[j]] : Real(0);
#pragma unroll
    for (int i = 0; i < PR; i++)
#pragma unroll
      for (int j = 0; j < PC; j++) x[i][j] = fmaR(a[i], b[j], x[i][j]);
    L += lk;
    R += rk;
  }
}

template <typename Real, int PR, int PC>
__device__ __forceinline__ void zero(Real (&x)[PR][PC]) {
#pragma unroll
  for (int i = 0; i < PR; i++)
#pragma unroll
    for (int j = 0; j < PC; j++) x[i][j] = Real(0);
}

template <typename Real, class Gm>
__device__ __forceinline__ void run_tile(const WarpLaunch& w, const WarpTile& td, const Group& G, const SlotPtrs& sp,
                                         double* smem) {
  const Term* __restrict__ terms = w.terms;
  const BatchEntry* __restrict__ entries = w.entries;
  const int row0 = (td.pos >> 16) * kWarpTile, col0 = (td.pos & 0xffff) * kWarpTile;
  constexpr int PR = Gm::PR, PC = Gm::PC, GR = Gm::GR, GC = Gm::GC, RC = Gm::RC, CC = Gm::CC;
  constexpr int TEAM = Gm::TEAM, NS = Gm::NS, LDX = Gm::LDX;
  const int tm = min(RC, G.m - row0), tn = min(CC, G.n - col0);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int team = lane / TEAM, tl = lane % TEAM;
  const int lr = tl % GR, lc = tl / GR;
  const int slot = warp * Gm::TEAMS + team;
  const unsigned mask = TEAM == 32 ? 0xffffffffu : (((1u << TEAM) - 1u) << (team * TEAM));
  Real* Xs = reinterpret_cast<Real*>(smem) + slot * RC * LDX;
  int ri[PR], cj[PC];
#pragma unroll
  for (int i = 0; i < PR; i++) ri[i] = lr + GR * i;
#pragma unroll
  for (int j = 0; j < PC; j++) cj[j] = lc + GC * j;
  bool vr_out[PR], vc_out[PC];
#pragma unroll
  for (int i = 0; i < PR; i++) vr_out[i] = ri[i] < tm;
#pragma unroll
  for (int j = 0; j < PC; j++) vc_out[j] = cj[j] < tn;

  Real acc[PR][PC];
  zero(acc);

  const int first = td.item0 + slot;
  if (first < td.item1) {
    int t = G.t0;
    {  // the term holding `first`
      int lo = G.t0, hi = G.t1 - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (terms[mid].item0 <= first) lo = mid;
        else hi = mid - 1;
      }
      t = lo;
    }
    Term T = terms[t];
    for (int item = first; item < td.item1; item += NS) {
      if (item >= T.item0 + T.count) {
        // every term holds at least one item, so the term of `item` is within NS terms
        int lo = t + 1, hi = min(t + NS, G.t1 - 1);
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (terms[mid].item0 <= item) lo = mid;
          else hi = mid - 1;
        }
        t = lo;
        T = terms[t];
      }
      double ald = T.alpha;
      int64_t da = 0, dc = 0;
      if (T.list >= 0) {
        const BatchEntry e = entries[T.list + (item - T.item0)];
        ald *= e.ratio;
        da = e.da;
        dc = e.dc;
      }
      const Real al = static_cast<Real>(ald);
      const bool ha = T.flags & kHasA, hc = T.flags & kHasC;
      // op(M)(i, j) = M[i * rs + j * cs]
      const int64_t rsb = (T.flags & kTransB) ? T.ldb : 1, csb = (T.flags & kTransB) ? 1 : T.ldb;
      const Real* B = resolve<Real>(sp, T.b);
      Real x[PR][PC];
      zero(x);
      if (ha && hc) {
        const int64_t rsa = (T.flags & kTransA) ? T.lda : 1, csa = (T.flags & kTransA) ? 1 : T.lda;
        const int64_t rsc = (T.flags & kTransC) ? T.ldc : 1, csc = (T.flags & kTransC) ? 1 : T.ldc;
        const Real* A = resolve<Real>(sp, T.a) + da + row0 * rsa;
        const Real* C = resolve<Real>(sp, T.c) + dc + col0 * csc;
        if (T.flags & kLeftFirst) {
          for (int l0 = 0; l0 < T.k2; l0 += CC) {
            const int kc = min(CC, T.k2 - l0);
            bool vc[PC];
#pragma unroll
            for (int j = 0; j < PC; j++) vc[j] = cj[j] < kc;
            if (l0 > 0) zero(x);
            // X = al op(A) [tm x k1] op(B)[:, l0 : l0 + kc]
            patch_gemm<Real, PR, PC>(x, A, rsa, csa, ri, vr_out, B + l0 * csb, rsb, csb, cj, vc, T.k1);
#pragma unroll
            for (int i = 0; i < PR; i++)
#pragma unroll
              for (int j = 0; j < PC; j++) Xs[ri[i] * LDX + cj[j]] = al * x[i][j];
            __syncwarp(mask);
            // acc += X [tm x kc] op(C)[l0 : l0 + kc, tile columns]
            patch_gemm<Real, PR, PC>(acc, Xs, LDX, 1, ri, vr_out, C + l0 * rsc, rsc, csc, cj, vc_out, kc);
            __syncwarp(mask);
          }
        } else {
          for (int k0 = 0; k0 < T.k1; k0 += RC) {
            const int kc = min(RC, T.k1 - k0);
            bool vr[PR];
#pragma unroll
            for (int i = 0; i < PR; i++) vr[i] = ri[i] < kc;
            if (k0 > 0) zero(x);
            // Y = al op(B)[k0 : k0 + kc, :] op(C) [k2 x tn]
            patch_gemm<Real, PR, PC>(x, B + k0 * rsb, rsb, csb, ri, vr, C, rsc, csc, cj, vc_out, T.k2);
#pragma unroll
            for (int i = 0; i < PR; i++)
#pragma unroll
              for (int j = 0; j < PC; j++) Xs[ri[i] * LDX + cj[j]] = al * x[i][j];
            __syncwarp(mask);
            // acc += op(A)[tile rows, k0 : k0 + kc] Y [kc x tn]
            patch_gemm<Real, PR, PC>(acc, A + k0 * csa, rsa, csa, ri, vr_out, Xs, LDX, 1, cj, vc_out, kc);
            __syncwarp(mask);
          }
        }
      } else {
        if (ha) {
          const int64_t rsa = (T.flags & kTransA) ? T.lda : 1, csa = (T.flags & kTransA) ? 1 : T.lda;
          const Real* A = resolve<Real>(sp, T.a) + da + row0 * rsa;
          patch_gemm<Real, PR, PC>(x, A, rsa, csa, ri, vr_out, B + col0 * csb, rsb, csb, cj, vc_out, T.k1);
        } else if (hc) {
          const int64_t rsc = (T.flags & kTransC) ? T.ldc : 1, csc = (T.flags & kTransC) ? 1 : T.ldc;
          const Real* C = resolve<Real>(sp, T.c) + dc + col0 * csc;
          patch_gemm<Real, PR, PC>(x, B + row0 * rsb, rsb, csb, ri, vr_out, C, rsc, csc, cj, vc_out, T.k2);
        } else {
          const Real* Bt = B + row0 * rsb + col0 * csb;
#pragma unroll
          for (int i = 0; i < PR; i++)
#pragma unroll
            for (int j = 0; j < PC; j++) x[i][j] = (vr_out[i] && vc_out[j]) ? Bt[ri[i] * rsb + cj[j] * csb] : Real(0);
        }
#pragma unroll
        for (int i = 0; i < PR; i++)
#pragma unroll
          for (int j = 0; j < PC; j++) acc[i][j] = fmaR(al, x[i][j], acc[i][j]);
      }
    }
  }
  __syncthreads();  // every team is done with its intermediate
#pragma unroll
  for (int i = 0; i < PR; i++)
#pragma unroll
    for (int j = 0; j < PC; j++) smem[(slot * RC + ri[i]) * CC + cj[j]] = static_cast<double>(acc[i][j]);
  __syncthreads();
  double* O = const_cast<double*>(resolve<double>(sp, G.out));
  const int64_t ldo = G.ldo;
  const bool accum = (G.flags & kAccumulate) != 0;
  const int te = tm * tn;
  if (td.nsplit == 1) {
    for (int e = tid; e < te; e += kWT) {
      const int r = e % tm, c = e / tm;
      double v = 0.0;
      for (int s = 0; s < NS; s++) v += smem[(s * RC + r) * CC + c];
      const int64_t idx = (row0 + r) + ldo * (col0 + c);
      O[idx] = accum ? O[idx] + v : v;
    }
    return;
  }
  // split tile: publish this CTA's partial sums; the last CTA to arrive adds all splits
  double* part = w.partials + td.part;
  for (int e = tid; e < te; e += kWT) {
    const int r = e % tm, c = e / tm;
    double v = 0.0;
    for (int s = 0; s < NS; s++) v += smem[(s * RC + r) * CC + c];
    __stcg(part + static_cast<int64_t>(td.split) * te + e, v);
  }
  __threadfence();
  __syncthreads();
  __shared__ int is_last;
  if (tid == 0) is_last = atomicAdd(w.counters + td.counter, 1u) == static_cast<unsigned>(td.nsplit - 1);
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int e = tid; e < te; e += kWT) {
    const int r = e % tm, c = e / tm;
    double v = 0.0;
    for (int s = 0; s < td.nsplit; s++) v += __ldcg(part + static_cast<int64_t>(s) * te + e);
    const int64_t idx = (row0 + r) + ldo * (col0 + c);
    O[idx] = accum ? O[idx] + v : v;
  }
  if (tid == 0) w.counters[td.counter] = 0u;  // ready for the next launch
}

// Row class R: (GR, PR) = (1, 2), (1, 4), (2, 3), (2, 4), (4, 3), (4, 4) for R = 0..5; column
// classes (GC, PC) = (1, 2), (2, 2), (4, 2), (4, 3), (8, 2) for 0..4 (warp_class_id).
template <int R>
struct RowClass;
template <> struct RowClass<0> { static constexpr int GR = 1, PR = 2; };
template <> struct RowClass<1> { static constexpr int GR = 1, PR = 4; };
template <> struct RowClass<2> { static constexpr int GR = 2, PR = 3; };
template <> struct RowClass<3> { static constexpr int GR = 2, PR = 4; };
template <> struct RowClass<4> { static constexpr int GR = 4, PR = 3; };
template <> struct RowClass<5> { static constexpr int GR = 4, PR = 4; };

// One kernel per (precision, row class); the column class is a CTA-uniform switch.
template <typename Real, int R>
__global__ void __launch_bounds__(kWT) sandwich_warp_kernel(const WarpLaunch w, const WarpTile* __restrict__ tiles,
                                                            SlotPtrs sp) {
  __shared__ double smem[kWBuf];
  const WarpTile td = tiles[blockIdx.x];
  const Group G = w.groups[td.group];
  constexpr int GR = RowClass<R>::GR, PR = RowClass<R>::PR;
  switch (td.cls - R * kWarpColClasses) {
    case 0: run_tile<Real, Geo<GR, PR, 1, 2>>(w, td, G, sp, smem); break;
    case 1: run_tile<Real, Geo<GR, PR, 2, 2>>(w, td, G, sp, smem); break;
    case 2: run_tile<Real, Geo<GR, PR, 4, 2>>(w, td, G, sp, smem); break;
    case 3: run_tile<Real, Geo<GR, PR, 4, 3>>(w, td, G, sp, smem); break;
    case 4: run_tile<Real, Geo<GR, PR, 8, 2>>(w, td, G, sp, smem); break;
    default: break;
  }
}

}  // namespace

template <int R>
cudaError_t launch_sandwich_warp_class(const WarpLaunch& w, const WarpTile* tiles, int ntiles, const SlotPtrs& sp,
                                       cudaStream_t stream, Precision prec) {
  if (ntiles <= 0) return cudaSuccess;
  if (prec == Precision::kFP32)
    sandwich_warp_kernel<float, R><<<ntiles, kWT, 0, stream>>>(w, tiles, sp);
  else
    sandwich_warp_kernel<double, R><<<ntiles, kWT, 0, stream>>>(w, tiles, sp);
  return cudaGetLastError();
}

}  // namespace c2g
