// Two-pass path of large groups on the 5th-generation tensor cores (tcgen05), for the
// mixed-precision Heff: both passes of sandwich_gemm.cu with the products formed as
// split-BF16 three-term products accumulated in FP32 in tensor memory.
//
// Each FP32 operand value v (the FP32 copies of X, of the operators and of the pass-1
// intermediates, times the item's coefficient for the left operand) is split into
// hi = bf16(v) and lo = bf16(v - hi); a product is hi_a hi_b + hi_a lo_b + lo_a hi_b, which
// keeps about 16 significant bits of each factor (relative error ~1e-5 per product, the
// missing lo_a lo_b term ~2^-16 of it). Sums over the inner dimension and over the items
// accumulate in FP32 in tensor memory; the item sum of a tile is turned into FP64 in the
// epilogue (split tiles are reduced in FP64 in split order, as in the SIMT path).
//
// Persistent 256-thread CTAs (three per SM) take the output tiles of the SIMT kernels'
// tile lists (64 x 64 grid) one after another from an atomic counter. The tile is the top-left 64 x 64 of a 128 x 64 MMA (M = 128, N = 64): rows
// 64..127 of the A operand are never written and their accumulator rows never read. The
// inner dimension is staged in chunks of 16 through three shared-memory stages: all threads
// load a chunk (FP32, pairs of k per thread, 32-byte segments whichever index is
// unit-stride), scale, split and store it in the no-swizzle K-major layout of the MMA
// (8-row x 16-byte core matrices, core matrices adjacent along K 128 bytes apart, 8-row
// groups 256 bytes apart; the 4-byte stores of a warp hit 32 distinct banks); one thread
// issues the three MMAs of the chunk and commits them to the stage's mbarrier, which the
// threads wait on before they overwrite that stage three chunks later. A chunk's global
// loads are issued three chunks ahead of its shared-memory stores, so they are in flight
// while the chunks before it are stored and their MMAs issued. Items with an inner
// dimension shorter than 16 are padded with zeros. The accumulator (64 FP32 columns of tensor memory, allocated by warp 0) is read
// with tcgen05.ld by warps 0, 1, 4 and 5 (lanes 0..63 = tile rows, two column halves).
//
// Every mbarrier wait is bounded: after kTcSpinLimit polls the kernel records an error in
// the runtime's mapped error word, waits (bounded again) for its own MMAs, frees its tensor
// memory and returns without writing its tile.
#include <cuda_bf16.h>

#include <algorithm>

#include "kernels.cuh"
#include "slots.cuh"

namespace c2g {

namespace {

constexpr int kTcThreads = 256;
constexpr int kTcM = 128, kTcN = 64, kTcK = 16;
constexpr int kTcStages = 3;
constexpr int kTcABytes = kTcM * kTcK * 2;  // 4096: one BF16 A operand of a chunk
constexpr int kTcBBytes = kTcN * kTcK * 2;  // 2048: one BF16 B operand of a chunk
constexpr int kTcStageBytes = 2 * kTcABytes + 2 * kTcBBytes;  // A hi, A lo, B hi, B lo
constexpr uint32_t kTcTmemCols = 64;
constexpr long long kTcSpinLimit = 1LL << 26;

struct __align__(1024) TcSmem {
  unsigned char stage[kTcStages][kTcStageBytes];
  unsigned long long bar[kTcStages];
  uint32_t tmem_base;
};

// Instruction descriptor of kind::f16 (tcgen05.mma): D F32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t(kTcN) >> 3) << 17) |
                              ((uint32_t(kTcM) >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, no swizzle: start address, leading-dimension byte
// offset (between core matrices adjacent along K), stride-dimension byte offset (between
// 8-row groups), the descriptor version bit 46.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// byte offset of element (row, k) of a chunk operand (k < 16) in the K-major layout
__device__ __forceinline__ uint32_t kmajor_off(int row, int k) {
  return static_cast<uint32_t>((row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for phase `parity` of the barrier; false when the limit was reached
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
  for (long long i = 0; i < kTcSpinLimit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kTcIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

struct TcOpnd {  // element (i, k) of op(M): t ? p[k + ld i] : p[i + ld k]
  const float* p;
  int64_t ld;
  bool t;
};

__device__ __forceinline__ TcOpnd tc_opnd(const SlotPtrs& sp, const GemmOperand& g, int di, int dk) {
  const float* p = resolve<float>(sp, g.ref);
  const int64_t ld = g.ld;
  const bool t = g.trans != 0;
  return TcOpnd{t ? p + dk + ld * di : p + di + ld * dk, ld, t};
}

// Staging map of a 64 x 16 chunk operand (op(L) rows, or op(R)^T columns): 512 k-pairs,
// two per thread. Slot g = warp + 8 s (s = 0, 1) is the row group g & 7 and the k-pair
// half g >> 3; lane = (row & 7) + 8 (k-pair & 3). A warp thus reads eight rows at eight
// consecutive k (32-byte segments whichever index is unit-stride) and its 4-byte
// shared-memory stores of a BF16 pair fall in 32 distinct banks.
struct TcRegs {
  float a[2][2], b[2][2];  // [slot][k of the pair]
};

__device__ __forceinline__ void stage_pos(int s, int& row, int& k) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = warp + 8 * s;
  row = (g & 7) * 8 + (lane & 7);
  k = 2 * ((g >> 3) * 4 + (lane >> 3));
}

__device__ __forceinline__ void tc_fetch(TcRegs& c, const TcOpnd& L, int M, const TcOpnd& R, int N, int K, int k0,
                                         float alpha) {
#pragma unroll
  for (int s = 0; s < 2; s++) {
    int i, k;
    stage_pos(s, i, k);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int kk = k0 + k + h;
      c.a[s][h] = (i < M && kk < K) ? alpha * (L.t ? L.p[kk + L.ld * i] : L.p[i + L.ld * kk]) : 0.0f;
      c.b[s][h] = (i < N && kk < K) ? (R.t ? R.p[i + R.ld * kk] : R.p[kk + R.ld * i]) : 0.0f;
    }
  }
}

// hi = bf16(v), lo = bf16(v - hi) of a pair, packed low k first
__device__ __forceinline__ void split_pair(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(v0 - hf.x, v1 - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

__device__ __forceinline__ void tc_store(const TcRegs& c, unsigned char* stage) {
  unsigned char* ahi = stage;
  unsigned char* alo = stage + kTcABytes;
  unsigned char* bhi = stage + 2 * kTcABytes;
  unsigned char* blo = stage + 2 * kTcABytes + kTcBBytes;
#pragma unroll
  for (int s = 0; s < 2; s++) {
    int i, k;
    stage_pos(s, i, k);
    const uint32_t off = kmajor_off(i, k);
    uint32_t hi, lo;
    split_pair(c.a[s][0], c.a[s][1], hi, lo);
    *reinterpret_cast<uint32_t*>(ahi + off) = hi;
    *reinterpret_cast<uint32_t*>(alo + off) = lo;
    split_pair(c.b[s][0], c.b[s][1], hi, lo);
    *reinterpret_cast<uint32_t*>(bhi + off) = hi;
    *reinterpret_cast<uint32_t*>(blo + off) = lo;
  }
}

// The three MMAs of a staged chunk: D (+)= Ahi Bhi + Ahi Blo + Alo Bhi.
__device__ __forceinline__ void tc_issue(uint32_t tmem_d, const unsigned char* stage, bool first) {
  const uint32_t base = smem_u32(stage);
  const uint64_t ahi = smem_desc(base, 128, 256);
  const uint64_t alo = smem_desc(base + kTcABytes, 128, 256);
  const uint64_t bhi = smem_desc(base + 2 * kTcABytes, 128, 256);
  const uint64_t blo = smem_desc(base + 2 * kTcABytes + kTcBBytes, 128, 256);
  tc_mma(tmem_d, alo, bhi, first ? 0u : 1u);
  tc_mma(tmem_d, ahi, blo, 1u);
  tc_mma(tmem_d, ahi, bhi, 1u);
}

// Item sources: the (L, R, alpha, K) products a tile sums, in order.
struct InterSource {  // pass 1: one product
  const InterJob* J;
  int row0, col0;
  __device__ int count() const { return 1; }
  __device__ bool get(int, const SlotPtrs& sp, TcOpnd& L, TcOpnd& R, float& alpha, int& K) const {
    L = tc_opnd(sp, J->l, row0, 0);
    R = tc_opnd(sp, J->r, 0, col0);
    alpha = 1.0f;
    K = J->k;
    return K > 0;
  }
};

// pass 2: the GEMM items of [item0, item1) (items with k = 0 are skipped). The item
// records are read through shared memory, kTcItemBatch at a time, loaded by the whole CTA
// with 16-byte loads (the calls of get() are the same in every thread, so the refill's
// barriers are uniform): an item's operand loads do not wait behind a global load of its
// record.
constexpr int kTcItemBatch = 32;
static_assert(sizeof(SumItem) % 16 == 0, "item records are copied in 16-byte words");
struct SumSource {
  const SumItem* items;
  int item0, item1, row0, col0;
  SumItem* buf;  // shared memory, kTcItemBatch records
  int* base;     // shared: first item held in buf (-1: none)
  __device__ int count() const { return item1 - item0; }
  __device__ void refill(int q) const {
    __syncthreads();  // every thread is done with the records held so far
    const int first = item0 + q;
    const int n = min(kTcItemBatch, item1 - first);
    constexpr int kWords = static_cast<int>(sizeof(SumItem) / 16);
    const int4* src = reinterpret_cast<const int4*>(items + first);
    int4* dst = reinterpret_cast<int4*>(buf);
    for (int w = threadIdx.x; w < n * kWords; w += kTcThreads) dst[w] = src[w];
    if (threadIdx.x == 0) *base = q;
    __syncthreads();
  }
  __device__ bool get(int q, const SlotPtrs& sp, TcOpnd& L, TcOpnd& R, float& alpha, int& K) const {
    const int b = *base;
    if (b < 0 || q < b || q >= b + kTcItemBatch) refill(q);
    const SumItem& I = buf[q - *base];
    K = I.k;
    if (K <= 0) return false;
    L = tc_opnd(sp, I.l, row0, 0);
    R = tc_opnd(sp, I.r, 0, col0);
    alpha = static_cast<float>(I.alpha);
    return true;
  }
};

// Position in the chunk sequence of a tile: item q of the source, inner offset k0.
struct TcCursor {
  int q, k0, K;
  float alpha;
  TcOpnd L, R;
};

// Moves `c` to the first chunk at or after item q (k0 = 0); false when none is left.
template <class Src>
__device__ __forceinline__ bool tc_seek(const Src& src, const SlotPtrs& sp, TcCursor& c, int q) {
  const int n = src.count();
  for (; q < n; q++)
    if (src.get(q, sp, c.L, c.R, c.alpha, c.K)) {
      c.q = q;
      c.k0 = 0;
      return true;
    }
  return false;
}

// The chunk loop of tc_accumulate: kTcAhead chunks of operand loads are in flight in
// registers (one TcRegs each, held in unrolled code so that no register is moved while its
// load is pending); each step stores the oldest, issues the loads of the chunk kTcAhead
// further on, and hands the stored chunk to the MMA issuer.
constexpr int kTcAhead = 3;

struct TcPipe {
  TcCursor cur;   // the next chunk to fetch
  bool more;      // cur is valid
  int fetched, stored;
};

template <class Src>
__device__ __forceinline__ void tc_fetch_next(const Src& src, const SlotPtrs& sp, TcPipe& pp, TcRegs& r, int M,
                                              int N) {
  if (!pp.more) return;
  tc_fetch(r, pp.cur.L, M, pp.cur.R, N, pp.cur.K, pp.cur.k0, pp.cur.alpha);
  pp.fetched++;
  pp.cur.k0 += kTcK;
  if (pp.cur.k0 >= pp.cur.K) pp.more = tc_seek(src, sp, pp.cur, pp.cur.q + 1);
}

// One step: store `r` (chunk pp.stored) into its stage, refill `r` with the chunk kTcAhead
// further on, then issue the stored chunk's MMAs. False (in every thread) when a wait ran
// out.
template <class Src>
__device__ __forceinline__ bool tc_step(const Src& src, const SlotPtrs& sp, TcPipe& pp, TcRegs& r, int M, int N,
                                        TcSmem& sm, uint32_t tmem_d, uint32_t& phase, uint32_t& pending) {
  const int chunk = pp.stored;
  const int s = chunk % kTcStages;
  const uint32_t bit = 1u << s;
  bool ok = true;
  if (pending & bit) {  // the MMAs that read this stage kTcStages chunks ago
    ok = mbar_wait(&sm.bar[s], (phase >> s) & 1u);
    phase ^= bit;
    pending &= ~bit;
  }
  tc_store(r, sm.stage[s]);
  pp.stored++;
  tc_fetch_next(src, sp, pp, r, M, N);
  fence_async_smem();
  if (__syncthreads_or(!ok)) return false;
  if (threadIdx.x == 0) {
    tc_fence_after();
    tc_issue(tmem_d, sm.stage[s], chunk == 0);
    tc_commit(&sm.bar[s]);
  }
  pending |= bit;
  return true;
}

// Sums the products of `src` into the tensor-memory accumulator. Returns the number of
// chunks issued (0: the accumulator was never written), or -1 when a wait ran out (the
// decision is the same in every thread of the CTA).
template <class Src>
__device__ int tc_accumulate(const Src& src, int M, int N, const SlotPtrs& sp, TcSmem& sm, uint32_t tmem_d,
                             uint32_t& phase, uint32_t& pending) {
  TcPipe pp;
  pp.fetched = pp.stored = 0;
  pp.more = tc_seek(src, sp, pp.cur, 0);
  if (!pp.more) return 0;
  static_assert(kTcAhead == 3, "the step loop below holds three register sets");
  TcRegs r0, r1, r2;
  tc_fetch_next(src, sp, pp, r0, M, N);
  tc_fetch_next(src, sp, pp, r1, M, N);
  tc_fetch_next(src, sp, pp, r2, M, N);
  for (;;) {
    if (pp.stored == pp.fetched) break;
    if (!tc_step(src, sp, pp, r0, M, N, sm, tmem_d, phase, pending)) return -1;
    if (pp.stored == pp.fetched) break;
    if (!tc_step(src, sp, pp, r1, M, N, sm, tmem_d, phase, pending)) return -1;
    if (pp.stored == pp.fetched) break;
    if (!tc_step(src, sp, pp, r2, M, N, sm, tmem_d, phase, pending)) return -1;
  }
  return pp.stored;
}

// Waits for every committed chunk; false (in every thread) when a wait ran out.
__device__ bool tc_drain(TcSmem& sm, uint32_t& phase, uint32_t& pending) {
  bool ok = true;
  for (int s = 0; s < kTcStages; s++) {
    const uint32_t bit = 1u << s;
    if (!(pending & bit)) continue;
    if (!mbar_wait(&sm.bar[s], (phase >> s) & 1u)) ok = false;
    phase ^= bit;
    pending &= ~bit;
  }
  return !__syncthreads_or(!ok);
}

__device__ void tc_setup(TcSmem& sm) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStages; s++) mbar_init(&sm.bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kTcTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

__device__ void tc_teardown(uint32_t tmem_d) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(kTcTmemCols) : "memory");
  }
}

// The epilogue readers: warps 0, 1, 4 and 5 (warp w may read accumulator lanes
// 32 (w % 4) .. 32 (w % 4) + 31), tile row (w % 4) * 32 + lane, columns 32 (w / 4) ..
// 32 (w / 4) + 31.
__device__ __forceinline__ bool tc_reader(int& row, int& col_base) {
  const int warp = threadIdx.x >> 5;
  row = (warp & 3) * 32 + (threadIdx.x & 31);
  col_base = (warp >> 2) * 32;
  return (warp & 3) < 2;
}

// Accumulator columns c0 .. c0 + 15 of this reader's tile row; zeros when no chunk was
// issued.
__device__ __forceinline__ void tc_read16(uint32_t tmem_d, int chunks, int c0, float (&v)[16]) {
  if (chunks <= 0) {
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = 0.0f;
    return;
  }
  const int warp = threadIdx.x >> 5;
  tmem_ld16(tmem_d + (static_cast<uint32_t>((warp & 3) * 32) << 16) + static_cast<uint32_t>(c0), v);
}

__device__ __forceinline__ void record_failure(int* err) {
  if (threadIdx.x == 0 && err) atomicOr(err, 1);
}

// Persistent CTAs: each takes the next tile of the list from sched[0] until the list is
// exhausted (tiles are ordered by descending work, so the longest start first); the last
// CTA to finish resets sched[0] and sched[1] for the next launch. Tensor memory and the
// mbarriers are set up once per CTA.
__device__ __forceinline__ int tc_next_tile(unsigned int* sched, int* slot) {
  __syncthreads();  // the previous tile's epilogue is done in every thread
  if (threadIdx.x == 0) *slot = static_cast<int>(atomicAdd(sched, 1u));
  __syncthreads();
  return *slot;
}

__device__ __forceinline__ void tc_finish(unsigned int* sched) {
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(sched + 1, 1u) == gridDim.x - 1) {
    sched[0] = 0u;
    sched[1] = 0u;
  }
}

__global__ void __launch_bounds__(kTcThreads, 3)
    inter_tc_kernel(const InterJob* __restrict__ jobs, const GemmTile* __restrict__ tiles, int ntiles, SlotPtrs sp,
                    unsigned int* sched, int* err) {
  __shared__ TcSmem sm;
  __shared__ int slot;
  tc_setup(sm);
  const uint32_t tmem_d = sm.tmem_base;
  uint32_t phase = 0u, pending = 0u;  // per stage: mbarrier phase and outstanding commit
  for (;;) {
    const int t = tc_next_tile(sched, &slot);
    if (t >= ntiles) break;
    const GemmTile T = tiles[t];
    const InterJob J = jobs[T.idx];
    const int row0 = (T.pos >> 16) * 64, col0 = (T.pos & 0xffff) * 64;
    const int tm = min(64, J.m - row0), tn = min(64, J.n - col0);
    const InterSource src{&J, row0, col0};
    const int chunks = tc_accumulate(src, tm, tn, sp, sm, tmem_d, phase, pending);
    const bool ok = tc_drain(sm, phase, pending) && chunks >= 0;
    tc_fence_after();
    if (!ok) {
      record_failure(err);
      break;
    }
    int r, cb;
    if (tc_reader(r, cb)) {
      float* S = sp.inter32 + J.off;
#pragma unroll
      for (int c0 = cb; c0 < cb + 32; c0 += 16) {
        float v[16];
        tc_read16(tmem_d, chunks, c0, v);
        if (r < tm) {
#pragma unroll
          for (int c = 0; c < 16; c++)
            if (c0 + c < tn) S[(row0 + r) + static_cast<int64_t>(J.m) * (col0 + c0 + c)] = v[c];
        }
      }
    }
    tc_fence_before();  // the accumulator reads precede the next tile's MMAs
  }
  tc_finish(sched);
  tc_teardown(tmem_d);
}

__global__ void __launch_bounds__(kTcThreads, 3)
    sum_tc_kernel(const SumGroup* __restrict__ groups, const SumItem* __restrict__ items,
                  const GemmTile* __restrict__ tiles, int ntiles, double* partials, unsigned int* counters,
                  SlotPtrs sp, unsigned int* sched, int* err) {
  __shared__ TcSmem sm;
  __shared__ int slot, is_last, item_base;
  __shared__ __align__(16) SumItem item_buf[kTcItemBatch];
  tc_setup(sm);
  const uint32_t tmem_d = sm.tmem_base;
  uint32_t phase = 0u, pending = 0u;  // per stage: mbarrier phase and outstanding commit
  for (;;) {
    const int t = tc_next_tile(sched, &slot);
    if (t >= ntiles) break;
    const GemmTile T = tiles[t];
    const SumGroup G = groups[T.idx];
    const int row0 = (T.pos >> 16) * 64, col0 = (T.pos & 0xffff) * 64;
    const int tm = min(64, G.m - row0), tn = min(64, G.n - col0);
    if (threadIdx.x == 0) item_base = -1;
    __syncthreads();
    const SumSource src{items, T.item0, T.item1, row0, col0, item_buf, &item_base};
    const int chunks = tc_accumulate(src, tm, tn, sp, sm, tmem_d, phase, pending);
    const bool ok = tc_drain(sm, phase, pending) && chunks >= 0;
    tc_fence_after();
    if (!ok) {
      record_failure(err);
      break;
    }
    int r, cb;
    const bool reader = tc_reader(r, cb);
    double* O = const_cast<double*>(resolve<double>(sp, G.out));
    const int64_t ldo = G.ldo;
    const bool accum = (G.flags & kAccumulate) != 0;
    // partial tiles of a split tile: TM x TN doubles per split (the tile's 16-granular
    // extents, as planned on the host), element (row, col) at row + TM col
    const int TM = 16 * ((T.shape & 3) + 1);
    double* part = partials + T.part;
    const int64_t part_elems = static_cast<int64_t>(TM) * 16 * (((T.shape >> 2) & 3) + 1);
    if (reader) {
#pragma unroll
      for (int c0 = cb; c0 < cb + 32; c0 += 16) {
        float v[16];
        tc_read16(tmem_d, chunks, c0, v);
        double acc[16];
#pragma unroll
        for (int c = 0; c < 16; c++) acc[c] = static_cast<double>(v[c]);
        // items without an inner dimension: out += alpha op(R), straight from global memory
        if (r < tm) {
          for (int it = T.item0; it < T.item1; it++) {
            const SumItem I = items[it];
            if (I.k > 0) continue;
            const TcOpnd R = tc_opnd(sp, I.r, row0, col0 + c0);
#pragma unroll
            for (int c = 0; c < 16; c++)
              if (c0 + c < tn)
                acc[c] = fma(I.alpha, static_cast<double>(R.t ? R.p[c + R.ld * r] : R.p[r + R.ld * c]), acc[c]);
          }
        }
        if (T.nsplit > 1) {
          if (r < tm) {
#pragma unroll
            for (int c = 0; c < 16; c++)
              if (c0 + c < tn) __stcg(part + T.split * part_elems + r + TM * (c0 + c), acc[c]);
          }
        } else if (r < tm) {
#pragma unroll
          for (int c = 0; c < 16; c++) {
            if (c0 + c < tn) {
              const int64_t idx = (row0 + r) + ldo * (col0 + c0 + c);
              O[idx] = accum ? O[idx] + acc[c] : acc[c];
            }
          }
        }
      }
    }
    tc_fence_before();  // the accumulator reads precede the next tile's MMAs
    if (T.nsplit > 1) {
      // the last split to arrive adds the partial tiles up in split order
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) is_last = atomicAdd(counters + T.counter, 1u) == static_cast<unsigned>(T.nsplit - 1);
      __syncthreads();
      if (is_last) {
        __threadfence();
        if (threadIdx.x == 0) counters[T.counter] = 0u;  // ready for the next launch
        // every thread: row tid % 64, columns 16 (tid / 64) .. 16 (tid / 64) + 15
        const int rr = threadIdx.x & 63, c1 = 16 * (threadIdx.x >> 6);
        if (rr < tm) {
          for (int c = c1; c < min(tn, c1 + 16); c++) {
            double v = 0.0;
            for (int s = 0; s < T.nsplit; s++) v += __ldcg(part + s * part_elems + rr + TM * c);
            const int64_t idx = (row0 + rr) + ldo * (col0 + c);
            O[idx] = accum ? O[idx] + v : v;
          }
        }
      }
    }
  }
  tc_finish(sched);
  tc_teardown(tmem_d);
}

// Persistent grid: three CTAs per SM (the kernels' occupancy), at most one per tile.
int tc_grid(int ntiles) {
  static const int sms = [] {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    return n;
  }();
  return std::min(ntiles, 3 * sms);
}

}  // namespace

cudaError_t launch_inter_tc(const InterJob* jobs, const GemmTile* tiles, int ntiles, const SlotPtrs& sp,
                            unsigned int* sched, int* err, cudaStream_t stream) {
  if (ntiles <= 0) return cudaSuccess;
  inter_tc_kernel<<<tc_grid(ntiles), kTcThreads, 0, stream>>>(jobs, tiles, ntiles, sp, sched, err);
  return cudaGetLastError();
}

cudaError_t launch_sum_tc(const SumGroup* groups, const SumItem* items, const GemmTile* tiles, int ntiles,
                          double* partials, unsigned int* counters, const SlotPtrs& sp, unsigned int* sched, int* err,
                          cudaStream_t stream) {
  if (ntiles <= 0) return cudaSuccess;
  sum_tc_kernel<<<tc_grid(ntiles), kTcThreads, 0, stream>>>(groups, items, tiles, ntiles, partials, counters, sp,
                                                           sched, err);
  return cudaGetLastError();
}

}  // namespace c2g
