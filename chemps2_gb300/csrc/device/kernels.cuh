// Device kernels of the DMRG hot path and their host launchers.
//
//   block sandwich     every term out += alpha sum_p ratio_p op(A_p) op(B) op(C_p) of a
//                      task-program stage, by output tiles, in three variants: the team
//                      kernel for tiles up to 16 x 16 (one launch per row class,
//                      sandwich_warp.cuh), the two-pass GEMM path for large groups
//                      (intermediates once, then split-K item sums; sandwich_gemm.cu)
//                      and, for comparison only, the one-pass cooperative and
//                      item-parallel kernels. Item sums run in a fixed order and split
//                      tiles are reduced in split order, so results are deterministic.
//   vector kernels     the Davidson eigensolver's dots, linear combinations and
//                      preconditioner, with deterministic two-pass reductions.
//   eigensolvers       one-CTA Jacobi for the <= 32 x 32 Rayleigh-Ritz matrix, and
//                      batched one-CTA Jacobi for the truncation's Gram matrices up to
//                      order 128 (FP64).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../host/tasks.hpp"

namespace c2g {

constexpr int kTile = 32;          // output tile edge of the block sandwich
constexpr int kSub = 4;            // register sub-tile edge
constexpr int kSandwichThreads = 128;
constexpr int kMaxSlots = 512;     // slot table size on the device

// Device pointers the kernels resolve references against. X, Y, Combo and Ones are per
// launch; everything else comes from the slot table.
struct SlotPtrs {
  const double* const* table;  // device array [kMaxSlots]
  double* x;
  double* y;
  double* combo;
  const double* ones;
  // FP32 copies read by the FP32 variant of the block sandwich (Y stays FP64)
  const float* const* table32;
  const float* x32;
  const float* combo32;
  const float* ones32;
  // intermediate products of the two-pass large-group path (slot kSlotInter), written in
  // the precision of the run
  double* inter;
  float* inter32;
};

// ---- Two-pass path of large groups (big output blocks with heavy items).
// A one-pass tile kernel recomputes an item's intermediate product (B C_p, or A_p B) for
// every output tile it feeds. Here pass 1 forms every intermediate once, as a plain tiled
// GEMM into the program's intermediate scratch (slot kSlotInter); pass 2 sums the items'
// products into the output tiles, out += sum_p alpha_p op(L_p) op(R_p), in the fixed item
// order, with long item lists split over several CTAs whose partial tiles the last CTA to
// finish adds up in split order. Tiles lie on a 64 x 64 grid; each is 16 PM x 16 PN
// (PM, PN = 1 .. 4) to cover its part of the block with little padding.
constexpr int kGemmThreads = 256;
constexpr int kGemmMaxSplit = 64;
constexpr int64_t kGemmCtaTarget = 1216;  // 152 SMs x 8 CTA-sized pieces per stage

struct GemmOperand {   // element (i, k) of op(M): trans ? p[k + ld i] : p[i + ld k]
  Ref ref;
  int32_t ld, trans;
};
struct InterJob {      // S (m x n, column-major, ld m) = op(L) (m x k) op(R) (k x n)
  GemmOperand l, r;
  int32_t m, n, k, pad;
  int64_t off;         // S at slot kSlotInter + off
  int64_t pad2;
};
struct SumItem {       // out += alpha op(L) (m x k) op(R) (k x n); k == 0: out += alpha op(R)
  GemmOperand l, r;
  double alpha;
  int32_t k, pad;
};
struct SumGroup {      // an output block of the path: items [i0, i1)
  Ref out;
  int32_t m, n, ldo, flags;
  int32_t i0, i1;
};
struct GemmTile {      // a CTA's work unit of either pass
  int32_t idx;         // job (pass 1) or sum group (pass 2)
  int32_t pos;         // tile row << 16 | tile column, in units of 64
  int32_t shape;       // (PM - 1) | (PN - 1) << 2: the tile is 16 PM x 16 PN
  int32_t nsplit, split;
  int32_t item0, item1;  // pass 2: this split's items (absolute indices)
  int32_t counter;       // pass 2 with nsplit > 1: arrival counter
  int64_t part;          // and its partial tiles (nsplit x 64 x 64 doubles)
};

// dst[i] = (float)src[i]
cudaError_t launch_to_f32(float* dst, const double* src, int64_t n, cudaStream_t stream);

// A CTA work unit: group index, tile position (row << 16 | col, in units of kTile) and the
// sub-tile grid (rows << 8 | cols) of the tile, chosen on the host.
struct TileDesc {
  int32_t group;
  int32_t pos;
  int32_t grid;
  int32_t pad;
};

// Choose the sub-tile grid (sr x sc, sr * sc <= kSandwichThreads) of an m x n tile.
inline int sandwich_grid(int m, int n) {
  const int sr = (m + kSub - 1) / kSub, sc = (n + kSub - 1) / kSub;
  return (sr << 8) | sc;
}

// Arithmetic of the block sandwich: FP64 throughout, or FP32 operands (the FP32 copies of
// SlotPtrs), products and per-lane sums, with the lane reduction and the FP64 output
// update in FP64. The FP32 variant issues no FP64 instruction in its item loop.
// kTC: the two-pass groups on the tensor cores as split-BF16 three-term products with FP32
// accumulation (sandwich_tc.cu), every other kernel as kFP32 (same FP32 operand copies).
enum class Precision : int { kFP64 = 0, kFP32 = 1, kTC = 2 };
// The arithmetic of the SIMT kernels of a run of precision p.
inline Precision simt_precision(Precision p) { return p == Precision::kTC ? Precision::kFP32 : p; }

cudaError_t launch_inter_gemm(const InterJob* jobs, const GemmTile* tiles, int ntiles, const SlotPtrs& sp,
                              cudaStream_t stream, Precision prec);
// Pass 1 for the jobs list[0 .. njobs) with m n <= kInterSmallElems: one warp per job.
constexpr int kInterSmallElems = 256;
cudaError_t launch_inter_small(const InterJob* jobs, const int32_t* list, int njobs, const SlotPtrs& sp,
                               cudaStream_t stream, Precision prec);
cudaError_t launch_sum_gemm(const SumGroup* groups, const SumItem* items, const GemmTile* tiles, int ntiles,
                            double* partials, unsigned int* counters, const SlotPtrs& sp, cudaStream_t stream,
                            Precision prec);


// Tensor-core variants of the two passes (sandwich_tc.cu), reading the FP32 operand copies.
// `sched`: two device counters, zero between launches (the kernels' tile scheduler resets
// them). `err` (device-visible, may be null) is or-ed with 1 when a kernel gave up a
// bounded wait.
cudaError_t launch_inter_tc(const InterJob* jobs, const GemmTile* tiles, int ntiles, const SlotPtrs& sp,
                            unsigned int* sched, int* err, cudaStream_t stream);
cudaError_t launch_sum_tc(const SumGroup* groups, const SumItem* items, const GemmTile* tiles, int ntiles,
                          double* partials, unsigned int* counters, const SlotPtrs& sp, unsigned int* sched, int* err,
                          cudaStream_t stream);

cudaError_t launch_sandwich(const Group* groups, const Term* terms, const BatchEntry* entries, const TileDesc* tiles,
                            int ntiles, const SlotPtrs& sp, cudaStream_t stream, Precision prec = Precision::kFP64);

// The one-pass cooperative variant for large output tiles (sandwich_tile.cu): one
// 256-thread CTA per 32 x 32 tile evaluating every item as shared-memory tiled GEMMs
// (kept for comparison, C2G_LARGE=tile; large groups take the two-pass path).
cudaError_t launch_sandwich_tiles(const Group* groups, const Term* terms, const BatchEntry* entries,
                                  const TileDesc* tiles, int ntiles, const SlotPtrs& sp, cudaStream_t stream,
                                  Precision prec = Precision::kFP64);

// Groups whose tiles hold at least this many elements and whose items average at least
// kLargeItemFlops are large groups (the two-pass path).
constexpr int kLargeTileElems = 256;
constexpr int64_t kLargeItemFlops = 4096;

// The team variant for tiles up to kWarpTile x kWarpTile (sandwich_warp.cuh). Its tile
// class is (row class * kWarpColClasses + column class); row capacities 2, 4, 6, 8, 12,
// 16, column capacities 2, 4, 8, 12, 16. A tile whose items are split over `nsplit` CTAs
// (split-items) has its partial sums written to `partials` (split s at part + s * rows *
// cols) and summed, in split order, by the CTA that finishes last (per-tile arrival
// counter, reset by that CTA).
constexpr int kWarpTile = 16;
constexpr int kWarpColClasses = 5;
constexpr int kWarpRowClasses = 6;
inline int warp_class_id(int rows, int cols) {
  const int rc = rows <= 2 ? 0 : rows <= 4 ? 1 : rows <= 6 ? 2 : rows <= 8 ? 3 : rows <= 12 ? 4 : 5;
  const int cc = cols <= 2 ? 0 : cols <= 4 ? 1 : cols <= 8 ? 2 : cols <= 12 ? 3 : 4;
  return rc * kWarpColClasses + cc;
}
inline int warp_row_class(int class_id) { return class_id / kWarpColClasses; }

struct WarpTile {   // 48 bytes
  int32_t group;
  int32_t pos;      // row << 16 | col, in units of kWarpTile
  int32_t cls;      // tile class
  int32_t item0, item1;  // the CTA's items [item0, item1) of the group
  int32_t nsplit, split;
  int32_t counter;  // arrival counter of a split tile
  int64_t part;     // first double of the tile's partial sums (split tiles)
  int64_t pad;
};

struct WarpLaunch {
  const Group* groups;
  const Term* terms;
  const BatchEntry* entries;
  const WarpTile* tiles;   // ordered by row class
  double* partials;
  unsigned int* counters;  // zero between launches
};

// Kernel of row class R (sandwich_warp_r<R>.cu) over `ntiles` tiles of that class.
template <int R>
cudaError_t launch_sandwich_warp_class(const WarpLaunch& w, const WarpTile* tiles, int ntiles, const SlotPtrs& sp,
                                       cudaStream_t stream, Precision prec);
extern template cudaError_t launch_sandwich_warp_class<0>(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&,
                                                          cudaStream_t, Precision);
extern template cudaError_t launch_sandwich_warp_class<1>(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&,
                                                          cudaStream_t, Precision);
extern template cudaError_t launch_sandwich_warp_class<2>(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&,
                                                          cudaStream_t, Precision);
extern template cudaError_t launch_sandwich_warp_class<3>(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&,
                                                          cudaStream_t, Precision);
extern template cudaError_t launch_sandwich_warp_class<4>(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&,
                                                          cudaStream_t, Precision);
extern template cudaError_t launch_sandwich_warp_class<5>(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&,
                                                          cudaStream_t, Precision);

// The team variant over w.tiles (counts[r] tiles of row class r, in class order); returns
// the number of kernels launched in *launched.
inline cudaError_t launch_sandwich_warp(const WarpLaunch& w, const int (&counts)[kWarpRowClasses], const SlotPtrs& sp,
                                        cudaStream_t stream, Precision prec, int* launched) {
  using Fn = cudaError_t (*)(const WarpLaunch&, const WarpTile*, int, const SlotPtrs&, cudaStream_t, Precision);
  static constexpr Fn fns[kWarpRowClasses] = {launch_sandwich_warp_class<0>, launch_sandwich_warp_class<1>,
                                              launch_sandwich_warp_class<2>, launch_sandwich_warp_class<3>,
                                              launch_sandwich_warp_class<4>, launch_sandwich_warp_class<5>};
  *launched = 0;
  int off = 0;
  for (int r = 0; r < kWarpRowClasses; r++) {
    if (counts[r] <= 0) continue;
    const cudaError_t e = fns[r](w, w.tiles + off, counts[r], sp, stream, prec);
    if (e != cudaSuccess) return e;
    off += counts[r];
    ++*launched;
  }
  return cudaSuccess;
}

// out[j] = sum_i A[i + lda * j] * x[i] for j < ncol (A has n rows). Uses `partial`
// (at least ncol * kDotBlocks doubles) as scratch.
constexpr int kDotBlocks = 152;
constexpr int kDotThreads = 256;
cudaError_t launch_multi_dot(const double* A, int64_t lda, int ncol, const double* x, int64_t n, double* partial,
                             double* out, cudaStream_t stream);
// out[i] = beta * out[i] + sum_j coef[j] * A[i + lda * j]   (coef on the device)
cudaError_t launch_combine(double* out, double beta, const double* A, int64_t lda, const double* coef, int ncol,
                           int64_t n, cudaStream_t stream);
// Sum of squares of x, written to out[0]
cudaError_t launch_norm2(const double* x, int64_t n, double* partial, double* out, cudaStream_t stream);
// x *= s (scalar on the host)
cudaError_t launch_scale(double* x, double s, int64_t n, cudaStream_t stream);
// y += a * x
cudaError_t launch_axpy(double* y, double a, const double* x, int64_t n, cudaStream_t stream);
cudaError_t launch_fill(double* x, double v, int64_t n, cudaStream_t stream);
// dst[:, j] = +-src[:, cols - 1 - j] for a rows x cols column-major matrix (ld = rows), the
// sign making the largest-magnitude entry of each column positive
cudaError_t launch_reverse_columns(double* dst, const double* src, int rows, int cols, cudaStream_t stream);

// Davidson device steps (CheMPS2/Davidson.cpp). `sc` is a small device scratch of
// scalars; layout documented in kernels.cu.
// Eigenvalues ascending in evals[0, n), eigenvectors in the columns of evecs (ld). warm:
// evecs holds the eigenvectors of the leading (n - 1) x (n - 1) block of mat (the previous
// call on the same matrix before it grew by one row and column).
cudaError_t launch_small_eig(double* mat, int n, int ld, double* evals, double* evecs, cudaStream_t stream,
                             bool warm = false);
// Batched Jacobi eigendecompositions of the Gram matrices of the truncation step, one CTA
// per job (n <= kBatchedEigMax); offsets in doubles from `base` (jobs on the device).
constexpr int kBatchedEigMax = 32;
struct EigJob {
  int32_t n, pad;
  int64_t offG, offE, offU;
};
cudaError_t launch_batched_eig(const EigJob* jobs, int njobs, double* base, cudaStream_t stream);
// The same for kBatchedEigMax < n <= kBatchedEigLargeMax: one 512-thread CTA per matrix
// with the matrix in dynamic shared memory and the eigenvector columns rotated in place
// in global memory (the Gram matrix's own slot, which the matrix is read from first).
// nmax: the largest n among the jobs (sizes the shared memory).
constexpr int kBatchedEigLargeMax = 128;
cudaError_t launch_batched_eig_large(const EigJob* jobs, int njobs, int nmax, double* base, cudaStream_t stream);
cudaError_t launch_residual(double* t, const double* u, const double* evals, int64_t n, cudaStream_t stream);
cudaError_t launch_precond_w(double* w, const double* u, const double* diag, const double* evals, double cutoff,
                             int64_t n, cudaStream_t stream);
cudaError_t launch_precond_t(double* t, const double* u, const double* diag, const double* evals,
                             const double* dots2, double cutoff, int64_t n, cudaStream_t stream);
cudaError_t launch_neg(double* c, int n, cudaStream_t stream);
cudaError_t launch_inv_sqrt_scale(double* x, const double* sumsq, int64_t n, cudaStream_t stream);
cudaError_t launch_mxm_row(double* mxm, int ld, int row, const double* dots, int ncol, cudaStream_t stream);
cudaError_t launch_lowdin(const double* overlap, int k, double* lowdin, cudaStream_t stream);

}  // namespace c2g
