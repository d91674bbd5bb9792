// Contraction-task representation of the DMRG hot path.
//
// The reference performs every hot-path operation (Heff diagrams, operator updates,
// Join, Split, the complementary-operator sums) as BLAS calls on symmetry blocks:
//     out_block += alpha * op(A) * op(B) * op(C)        (A and/or C optional)
// where op() is an optional transpose and the operand blocks live in MPS tensors,
// operator tensors, the two-site vector or temporary "combined" blocks built with
// daxpy (e.g. CheMPS2/HeffDiagrams4.cpp:2334-2420, CheMPS2/TensorQ.cpp:113-248).
// The host task compiler walks the same loops and records these contractions here
// instead of executing them; the GPU runtime (and the CPU executor of the oracle)
// execute them as grouped launches.
//
// A Term is a fused, batched sandwich:
//     out += alpha * sum_p ratio_p * op(A + da_p) * op(B) * op(C + dc_p)
// The reference's innermost loops over an operator index (orbital pairs in diagram 2a,
// orbitals in 3C, 4B, 5A, ...) multiply the same block B of the input vector by blocks of
// different operator tensors at the same position inside their tensors; those
// contractions become one term whose batch list holds the tensor offsets (da_p, dc_p).
// The lists do not depend on the output block, so the compiler stores each distinct
// list once per program.
//
// A Program is a list of stages, one launch each: an optional combination stage
// (combined blocks = sum_i alpha_i op(block_i), run once per program preparation) and
// accumulation stages. Within a stage every output block is owned by one group; the terms
// of a group are summed in a fixed order, so results are deterministic.
#pragma once

#include <algorithm>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace c2g {

// A data reference: buffer slot in the top 16 bits, offset in doubles below.
using Ref = uint64_t;
constexpr int kRefShift = 48;
constexpr uint64_t kRefMask = (uint64_t(1) << kRefShift) - 1;
inline Ref make_ref(int slot, int64_t off) { return (uint64_t(slot) << kRefShift) | uint64_t(off); }
inline int ref_slot(Ref r) { return static_cast<int>(r >> kRefShift); }
inline int64_t ref_off(Ref r) { return static_cast<int64_t>(r & kRefMask); }

// Fixed buffer slots. X and Y are bound per launch (the Davidson input / output
// vector of a matvec); the rest are registered allocations.
enum Slot : int {
  kSlotX = 0,
  kSlotY = 1,
  kSlotInter = 2,   // intermediate products of the two-pass large-block path
  kSlotCombo = 3,   // combined blocks of the program being run
  kSlotWork = 4,    // truncation workspace (assembled sector matrices, Gram, eigvecs)
  kSlotOnes = 5,    // a vector of 1.0, at least as long as the largest sector dimension
  kSlotCorr0 = 6,   // correlation-pass tensors of alternating boundaries
  kSlotCorr1 = 7,
  kSlotMpsBase = 8, // + site: MPS tensors
};
inline int slot_ops(int L, int boundary) { return kSlotMpsBase + L + boundary; }
inline int num_slots(int L) { return kSlotMpsBase + 2 * L + 2; }

// A block operand: rows x cols, column-major with leading dimension ld.
struct Blk {
  Ref ref = 0;
  int rows = 0, cols = 0, ld = 0;
  bool valid = false;
  static Blk make(Ref r, int rows, int cols, int ld = -1) {
    Blk b;
    b.ref = r;
    b.rows = rows;
    b.cols = cols;
    b.ld = (ld < 0) ? rows : ld;
    b.valid = true;
    return b;
  }
};

enum TermFlags : int32_t {
  kHasA = 1,
  kHasC = 2,
  kTransA = 4,   // A stored k1 x m
  kTransB = 8,   // B stored k2 x k1
  kTransC = 16,  // C stored n x k2
  kLeftFirst = 32,  // with A and C: evaluate (A B) C, otherwise A (B C) (the cheaper order)
};

// out (m x n, from the group) += alpha * sum_p ratio_p op(A_p) (m x k1) op(B) (k1 x k2)
// op(C_p) (k2 x n). Without A, op(A) = I and k1 = m; without C, op(C) = I and k2 = n.
struct Term {        // 64 bytes
  Ref a, b, c;       // entry 0 (a / c are 0 when absent)
  double alpha;
  int32_t k1, k2;
  int32_t lda, ldb, ldc;
  int32_t flags;
  int32_t list;      // first entry in Program::entries, -1 for a single contraction
  int32_t count;     // entries (1 for a single contraction)
  int32_t item0;     // entries of the previous terms of the same group
};

// Entry p of a batched term: A_p = a + da, C_p = c + dc, coefficient alpha * ratio.
struct BatchEntry {  // 24 bytes
  int64_t da, dc;
  double ratio;
};

enum GroupFlags : int32_t {
  kAccumulate = 1,  // out += sum; otherwise out = sum
};

struct Group {       // 40 bytes
  Ref out;
  int32_t m, n, ldo;
  int32_t flags;
  int32_t t0, t1;    // term range [t0, t1)
  int64_t work;      // flop count, used for scheduling
};

struct Stage {
  std::vector<Group> groups;
  std::vector<Term> terms;
  std::string name;
  int64_t flops = 0;  // sum over terms and entries of the sandwich flops
  int64_t items = 0;  // sum of term entry counts
};

struct Program {
  std::vector<Stage> stages;
  std::vector<BatchEntry> entries;  // shared batch lists of all stages
  int64_t combo_size = 0;           // doubles of combined blocks (slot kSlotCombo)
  int first_repeat_stage = 0;       // stages [0, first_repeat_stage) run once (combinations)
  int64_t flops() const {
    int64_t f = 0;
    for (auto& s : stages) f += s.flops;
    return f;
  }
};

// Flops of one entry of a term (2 per multiply-add; m * n for a plain scaled copy).
int64_t term_flops(const Term& t, int m, int n);

// Open-addressing index from 64-bit keys to non-negative int32 values (several values per
// key allowed, visited in insertion order), for the compiler's large lookup tables.
class FlatIndex {
 public:
  // Calls f(value) for the values stored under key until f returns true; true if it did.
  template <class F>
  bool visit(uint64_t key, F&& f) const {
    if (vals_.empty()) return false;
    for (size_t i = slot(key);; i = (i + 1) & mask_) {
      if (vals_[i] < 0) return false;
      if (keys_[i] == key && f(vals_[i])) return true;
    }
  }
  // The first value stored under key, or -1.
  int32_t find(uint64_t key) const {
    int32_t out = -1;
    visit(key, [&](int32_t v) {
      out = v;
      return true;
    });
    return out;
  }
  void insert(uint64_t key, int32_t value) {
    if ((size_ + 1) * 2 > vals_.size()) grow();
    size_t i = slot(key);
    while (vals_[i] >= 0) i = (i + 1) & mask_;
    keys_[i] = key;
    vals_[i] = value;
    size_++;
  }
  void clear() {
    keys_.clear();
    vals_.clear();
    mask_ = 0;
    size_ = 0;
  }
  size_t size() const { return size_; }

 private:
  std::vector<uint64_t> keys_;
  std::vector<int32_t> vals_;  // -1: empty
  size_t mask_ = 0, size_ = 0;
  size_t slot(uint64_t k) const {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    return static_cast<size_t>(k) & mask_;
  }
  void grow() {
    std::vector<uint64_t> ok;
    std::vector<int32_t> ov;
    ok.swap(keys_);
    ov.swap(vals_);
    const size_t cap = std::max<size_t>(1024, ov.size() * 2);
    keys_.assign(cap, 0);
    vals_.assign(cap, -1);
    mask_ = cap - 1;
    size_ = 0;
    for (size_t i = 0; i < ov.size(); i++)  // old probe order keeps equal keys in order
      if (ov[i] >= 0) insert(ok[i], ov[i]);
  }
};

// Open-addressing table from block references (never 0: slot 0 is never tracked) to the
// largest element count seen for each: the operand footprint of a program.
class RefSizes {
 public:
  void note(Ref r, int64_t n) {
    if ((size_ + 1) * 2 > keys_.size()) grow();
    for (size_t i = slot(r);; i = (i + 1) & mask_) {
      if (keys_[i] == r) {
        if (n > vals_[i]) vals_[i] = n;
        return;
      }
      if (keys_[i] == 0) {
        keys_[i] = r;
        vals_[i] = n;
        size_++;
        return;
      }
    }
  }
  template <class F>
  void for_each(F&& f) const {
    for (size_t i = 0; i < keys_.size(); i++)
      if (keys_[i] != 0) f(keys_[i], vals_[i]);
  }
  int64_t total() const {
    int64_t s = 0;
    for_each([&](Ref, int64_t v) { s += v; });
    return s;
  }
  size_t size() const { return size_; }

 private:
  std::vector<Ref> keys_;
  std::vector<int64_t> vals_;
  size_t mask_ = 0, size_ = 0;
  size_t slot(Ref k) const {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    return static_cast<size_t>(k) & mask_;
  }
  void grow() {
    std::vector<Ref> ok;
    std::vector<int64_t> ov;
    ok.swap(keys_);
    ov.swap(vals_);
    const size_t cap = std::max<size_t>(1024, ok.size() * 2);
    keys_.assign(cap, 0);
    vals_.assign(cap, 0);
    mask_ = cap - 1;
    size_ = 0;
    for (size_t i = 0; i < ok.size(); i++)
      if (ok[i] != 0) note(ok[i], ov[i]);
  }
};

// Records contractions and lowers them into a Program.
class TaskBuilder {
 public:
  // track_operands: record the footprint of the MPS / operator blocks read (for the
  // benchmark ledger; off by default because it costs a hash insert per operand).
  explicit TaskBuilder(bool track_operands = false);

  // A block of the combination scratch holding sum_i alpha_i * op_i(block_i).
  // All parts must have the shape rows x cols after their optional transpose.
  // Returns an invalid Blk when parts is empty.
  Blk combine(const std::vector<std::pair<double, Blk>>& parts, int rows, int cols,
              const std::vector<bool>* transposed = nullptr);

  // out += alpha * op(A) * op(B) * op(C). A and C may be invalid (absent).
  void contract(const Blk& out, double alpha, const Blk& A, bool ta, const Blk& B, bool tb,
                const Blk& C, bool tc);

  // out += alpha * op(B)
  void axpy(const Blk& out, double alpha, const Blk& B, bool tb) {
    contract(out, alpha, Blk(), false, B, tb, Blk(), false);
  }

  // Makes out a zero-initialised output of the current accumulation stage even if no
  // term reaches it (so an executor writes zeros instead of leaving stale data).
  void declare_output(const Blk& out);

  // Closes the current accumulation stage; later contractions accumulate onto what
  // earlier stages wrote.
  void next_stage(const std::string& name);

  // keep_empty keeps empty stages (and an empty combination stage), so that programs of
  // disjoint shards have identical stage lists and can be merged position by position.
  Program finalize(bool keep_empty = false);

  int64_t num_contractions() const { return n_contract_; }

  // Bytes of the distinct MPS / operator blocks the recorded contractions read (each
  // block counted once, FP64), the operand traffic of one execution of the program.
  int64_t operand_bytes() const;
  const RefSizes& operands() const { return operands_; }

 private:
  // Terms and batch entries of a stage in emission order (flat arrays: no allocation
  // per term); lowering orders them by group, and entries by term, with counting sorts.
  struct StageBuf {
    std::vector<Group> groups;
    std::vector<Term> terms;
    std::vector<int32_t> term_group;
    std::vector<BatchEntry> extra;      // batch entries beyond entry 0
    std::vector<int32_t> extra_term;    // the term of each
    FlatIndex group_of;  // output reference -> group
    std::string name;
  };
  // Terms of the open group that later contractions may join, by hash of the batching
  // key (B, shapes, leading dimensions, flags, operand slots); cleared in O(1) by stamps.
  class OpenTerms {
   public:
    template <class Eq>
    int32_t find(uint64_t h, Eq&& eq) const {
      if (stamps_.empty()) return -1;
      for (size_t i = h & mask_;; i = (i + 1) & mask_) {
        if (stamps_[i] != stamp_) return -1;
        if (hashes_[i] == h && eq(terms_[i])) return terms_[i];
      }
    }
    void insert(uint64_t h, int32_t term);
    void clear() {
      n_ = 0;
      if (++stamp_ == 0) {
        std::fill(stamps_.begin(), stamps_.end(), 0u);
        stamp_ = 1;
      }
    }

   private:
    std::vector<uint32_t> stamps_;
    std::vector<uint64_t> hashes_;
    std::vector<int32_t> terms_;
    uint32_t stamp_ = 1;
    size_t mask_ = 0, n_ = 0;
  };

  StageBuf combo_;
  int64_t combo_size_ = 0;
  // Combination cache: key words of every combined block in one arena, looked up by hash
  // and compared exactly.
  struct ComboEntry {
    int64_t word0;
    int32_t nwords;
    Blk out;
  };
  FlatIndex combo_index_;
  std::vector<ComboEntry> combo_entries_;
  std::vector<uint64_t> combo_words_;
  std::vector<uint64_t> key_scratch_;
  std::vector<StageBuf> stages_;
  OpenTerms open_;                                         // open terms of the open group
  FlatIndex written_;                                      // outputs written by closed stages
  RefSizes operands_;                                      // footprint of MPS / operator operands
  // direct-mapped cache of recently noted blocks in front of operands_ (the same operator
  // blocks recur across the output blocks of a program)
  static constexpr int kOperandCache = 16384;
  std::vector<Ref> seen_ref_;
  std::vector<int64_t> seen_n_;
  int64_t n_contract_ = 0;
  bool track_operands_ = false;
  const StageBuf* open_sb_ = nullptr;  // the group whose terms are open for batching
  int open_group_ = -1;
  const StageBuf* last_sb_ = nullptr;  // output-group lookup cache
  Ref last_out_ = 0;
  int last_group_ = -1;

  void note_operand(const Blk& b);
  // The group of `out` in sb, created on first use: it accumulates onto what earlier
  // stages wrote (never in the combination stage).
  int group_for(StageBuf& sb, const Blk& out);
  void add(StageBuf& sb, bool batchable, const Blk& out, double alpha, const Blk& A, bool ta, const Blk& B, bool tb,
           const Blk& C, bool tc);
  // lists: batch lists already in `table`, by hash of their entries
  static Stage lower(StageBuf& sb, const std::string& name, std::vector<BatchEntry>& table,
                     FlatIndex& lists);
};

// Concatenates programs compiled (with keep_empty) from disjoint output shards into one
// program with the same stage structure, relocating combination-scratch references and
// batch lists. Empty stages are dropped.
Program merge_programs(std::vector<Program>& parts);

// Number of compile threads: the calling thread's own setting if it made one, else
// C2G_COMPILE_THREADS, else the hardware count.
int compile_threads();
// Sets the calling thread's compile thread count (0 clears it). Concurrent solves give
// each worker thread a share of the cores.
void set_thread_compile_threads(int n);
// While on, the calling thread's compilations use an equal share of the cores among all
// threads that have it on (re-read at every compilation, so the share grows as others
// turn it off). Concurrent solves turn it on in their worker threads.
void share_compile_threads(bool on);

}  // namespace c2g
