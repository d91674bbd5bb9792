// Team-cooperative block-sandwich kernel for output tiles up to 16 x 16.
//
// One 128-thread CTA per (group, tile). The host picks the tile's capacity class RC x CC
// (RC, CC in {2, 4, 8, 16}, the smallest powers of two covering the tile). A team of
// GR x GC lanes evaluates one (term, entry) item at a time, each lane owning a PR x PC
// patch (rows lr + GR i, columns lc + GC j) of the tile; a warp holds 32 / (GR GC) teams
// and the CTA's teams ("slots") take the group's items round robin (slot s: items s,
// s + NS, ...), so that neighbouring teams mostly evaluate items of one term shape. For
// a three-operand item the team builds its intermediate (a column chunk of A B, or a
// row chunk of B C) once in shared memory and multiplies it into the patch: every
// multiply-add of the fused contraction is executed once. The slots' partial tiles are
// summed in a fixed order at the end, so the result is deterministic.
#include "kernels.cuh"
#include "slots.cuh"

namespace c2g {

namespace {

constexpr int kWT = 128;        // threads per CTA
constexpr int kWBuf = 1536;     // doubles of shared scratch (intermediates, then the slot sums)

template <int RC, int CC>
struct Geo {
  static constexpr int PR = RC < 4 ? RC : 4;
  static constexpr int PC = CC < 2 ? CC : 2;
  static constexpr int GR = RC / PR, GC = CC / PC;
  static constexpr int TEAM = GR * GC;          // lanes per item
  static constexpr int TEAMS = 32 / TEAM;       // teams per warp
  static constexpr int NS = (kWT / 32) * TEAMS;  // slots per CTA
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

template <typename Real, int RC, int CC>
__device__ __forceinline__ void run_tile(const Group& G, const Term* __restrict__ terms,
                                         const BatchEntry* __restrict__ entries, const SlotPtrs& sp, int row0,
                                         int col0, double* smem) {
  using Gm = Geo<RC, CC>;
  constexpr int PR = Gm::PR, PC = Gm::PC, GR = Gm::GR, TEAM = Gm::TEAM, NS = Gm::NS, LDX = Gm::LDX;
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
  for (int j = 0; j < PC; j++) cj[j] = lc + Gm::GC * j;
  bool vr_out[PR], vc_out[PC];
#pragma unroll
  for (int i = 0; i < PR; i++) vr_out[i] = ri[i] < tm;
#pragma unroll
  for (int j = 0; j < PC; j++) vc_out[j] = cj[j] < tn;

  Real acc[PR][PC];
#pragma unroll
  for (int i = 0; i < PR; i++)
#pragma unroll
    for (int j = 0; j < PC; j++) acc[i][j] = Real(0);

  if (G.t1 > G.t0) {
    const int total = terms[G.t1 - 1].item0 + terms[G.t1 - 1].count;
    int t = G.t0;
    Term T = terms[t];
    for (int item = slot; item < total; item += NS) {
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
      const bool ha = T.flags & kHasA, hc = T.flags & kHasC;
      // op(M)(i, j) = M[i * rs + j * cs]
      const int64_t rsb = (T.flags & kTransB) ? T.ldb : 1, csb = (T.flags & kTransB) ? 1 : T.ldb;
      const Real* B = resolve<Real>(sp, T.b);
      Real tmp[PR][PC];
#pragma unroll
      for (int i = 0; i < PR; i++)
#pragma unroll
        for (int j = 0; j < PC; j++) tmp[i][j] = Real(0);
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
            Real x[PR][PC];
#pragma unroll
            for (int i = 0; i < PR; i++)
#pragma unroll
              for (int j = 0; j < PC; j++) x[i][j] = Real(0);
            // X = op(A) [tm x k1] op(B)[:, l0 : l0 + kc]
            patch_gemm<Real, PR, PC>(x, A, rsa, csa, ri, vr_out, B + l0 * csb, rsb, csb, cj, vc, T.k1);
#pragma unroll
            for (int i = 0; i < PR; i++)
#pragma unroll
              for (int j = 0; j < PC; j++) Xs[ri[i] * LDX + cj[j]] = x[i][j];
            __syncwarp(mask);
            // tmp += X [tm x kc] op(C)[l0 : l0 + kc, tile columns]
            patch_gemm<Real, PR, PC>(tmp, Xs, LDX, 1, ri, vr_out, C + l0 * rsc, rsc, csc, cj, vc_out, kc);
            __syncwarp(mask);
          }
        } else {
          for (int k0 = 0; k0 < T.k1; k0 += RC) {
            const int kc = min(RC, T.k1 - k0);
            bool vr[PR];
#pragma unroll
            for (int i = 0; i < PR; i++) vr[i] = ri[i] < kc;
            Real y[PR][PC];
#pragma unroll
            for (int i = 0; i < PR; i++)
#pragma unroll
              for (int j = 0; j < PC; j++) y[i][j] = Real(0);
            // Y = op(B)[k0 : k0 + kc, :] op(C) [k2 x tn]
            patch_gemm<Real, PR, PC>(y, B + k0 * rsb, rsb, csb, ri, vr, C, rsc, csc, cj, vc_out, T.k2);
#pragma unroll
            for (int i = 0; i < PR; i++)
#pragma unroll
              for (int j = 0; j < PC; j++) Xs[ri[i] * LDX + cj[j]] = y[i][j];
            __syncwarp(mask);
            // tmp += op(A)[tile rows, k0 : k0 + kc] Y [kc x tn]
            patch_gemm<Real, PR, PC>(tmp, A + k0 * csa, rsa, csa, ri, vr_out, Xs, LDX, 1, cj, vc_out, kc);
            __syncwarp(mask);
          }
        }
      } else if (ha) {
        const int64_t rsa = (T.flags & kTransA) ? T.lda : 1, csa = (T.flags & kTransA) ? 1 : T.lda;
        const Real* A = resolve<Real>(sp, T.a) + da + row0 * rsa;
        patch_gemm<Real, PR, PC>(tmp, A, rsa, csa, ri, vr_out, B + col0 * csb, rsb, csb, cj, vc_out, T.k1);
      } else if (hc) {
        const int64_t rsc = (T.flags & kTransC) ? T.ldc : 1, csc = (T.flags & kTransC) ? 1 : T.ldc;
        const Real* C = resolve<Real>(sp, T.c) + dc + col0 * csc;
        patch_gemm<Real, PR, PC>(tmp, B + row0 * rsb, rsb, csb, ri, vr_out, C, rsc, csc, cj, vc_out, T.k2);
      } else {
        const Real* Bt = B + row0 * rsb + col0 * csb;
#pragma unroll
        for (int i = 0; i < PR; i++)
#pragma unroll
          for (int j = 0; j < PC; j++) tmp[i][j] = (vr_out[i] && vc_out[j]) ? Bt[ri[i] * rsb + cj[j] * csb] : Real(0);
      }
      const Real al = static_cast<Real>(ald);
#pragma unroll
      for (int i = 0; i < PR; i++)
#pragma unroll
        for (int j = 0; j < PC; j++) acc[i][j] = fmaR(al, tmp[i][j], acc[i][j]);
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
  for (int e = tid; e < tm * tn; e += kWT) {
    const int r = e % tm, c = e / tm;
    double v = 0.0;
    for (int s = 0; s < NS; s++) v += smem[(s * RC + r) * CC + c];
    const int64_t idx = (row0 + r) + ldo * (col0 + c);
    O[idx] = accum ? O[idx] + v : v;
  }
}

template <typename Real>
__global__ void __launch_bounds__(kWT) sandwich_warp_kernel(const Group* __restrict__ groups,
                                                            const Term* __restrict__ terms,
                                                            const BatchEntry* __restrict__ entries,
                                                            const TileDesc* __restrict__ tiles, SlotPtrs sp) {
  __shared__ double smem[kWBuf];
  const TileDesc td = tiles[blockIdx.x];
  const Group G = groups[td.group];
  const int row0 = (td.pos >> 16) * kWarpTile, col0 = (td.pos & 0xffff) * kWarpTile;
  switch (td.grid) {
#define C2G_WARP_CASE(r, c) \
  case warp_class_id(r, c): run_tile<Real, r, c>(G, terms, entries, sp, row0, col0, smem); break;
    C2G_WARP_CASE(2, 2) C2G_WARP_CASE(2, 4) C2G_WARP_CASE(2, 8) C2G_WARP_CASE(2, 16)
    C2G_WARP_CASE(4, 2) C2G_WARP_CASE(4, 4) C2G_WARP_CASE(4, 8) C2G_WARP_CASE(4, 16)
    C2G_WARP_CASE(8, 2) C2G_WARP_CASE(8, 4) C2G_WARP_CASE(8, 8) C2G_WARP_CASE(8, 16)
    C2G_WARP_CASE(16, 2) C2G_WARP_CASE(16, 4) C2G_WARP_CASE(16, 8) C2G_WARP_CASE(16, 16)
#undef C2G_WARP_CASE
    default: break;
  }
}

}  // namespace

cudaError_t launch_sandwich_warp(const Group* groups, const Term* terms, const BatchEntry* entries,
                                 const TileDesc* tiles, int ntiles, const SlotPtrs& sp, cudaStream_t stream,
                                 Precision prec) {
  if (ntiles <= 0) return cudaSuccess;
  if (prec == Precision::kFP32)
    sandwich_warp_kernel<float><<<ntiles, kWT, 0, stream>>>(groups, terms, entries, tiles, sp);
  else
    sandwich_warp_kernel<double><<<ntiles, kWT, 0, stream>>>(groups, terms, entries, tiles, sp);
  return cudaGetLastError();
}

}  // namespace c2g
