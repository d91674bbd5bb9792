// Contraction-task representation of the DMRG hot path.
//
// The reference performs every hot-path operation (Heff diagrams, operator updates,
// Join, the complementary-operator sums) as BLAS calls on symmetry blocks:
//     out_block += alpha * op(A) * op(B) * op(C)        (A and/or C optional)
// where op() is an optional transpose and the operand blocks live in MPS tensors,
// operator tensors, the two-site vector or temporary "combined" blocks built with
// daxpy (e.g. CheMPS2/HeffDiagrams4.cpp:2334-2420, CheMPS2/TensorQ.cpp:113-248).
// The host task compiler walks the same loops and records these contractions here
// instead of executing them; the GPU runtime (and the CPU executor of the oracle)
// then run them as grouped launches.
//
// A Program is a list of stages, each one launch:
//   * a combination stage: combined blocks = sum_i alpha_i * op(block_i);
//   * product stages: phase-1 products P = op(A) op(B) (or op(B) op(C)) for every
//     three-operand contraction, written to scratch and de-duplicated;
//   * accumulation stages: out_block (+)= sum_t alpha_t * op(U_t) * op(V_t).
// Within an accumulation stage every output block is owned by exactly one group, and
// the terms of a group are summed in emission order, so the result is deterministic
// and identical for every executor that honours the term order.
#pragma once

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
  kSlotP1 = 2,      // phase-1 products of the program being run
  kSlotCombo = 3,   // combined blocks of the program being run
  kSlotWork = 4,    // truncation workspace (assembled sector matrices, Gram, eigvecs)
  kSlotOnes = 5,    // a vector of 1.0, at least as long as the largest sector dimension
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
  kTransU = 1,   // U stored k x m (used transposed)
  kTransV = 2,   // V stored n x k (used transposed)
  kScalar = 4,   // out += alpha * op(U), no V
};

struct Term {       // 48 bytes
  Ref u, v;
  double alpha;
  int32_t k;        // inner dimension (unused for scalar terms)
  int32_t ldu, ldv;
  int32_t flags;
  int32_t pad0, pad1;
};

enum GroupFlags : int32_t {
  kAccumulate = 1,  // out += sum; otherwise out = sum
};

struct Group {      // 40 bytes
  Ref out;
  int32_t m, n, ldo;
  int32_t flags;
  int32_t t0, t1;   // term range [t0, t1)
  int64_t work;     // flop estimate, used for scheduling
};

struct Stage {
  std::vector<Group> groups;
  std::vector<Term> terms;
  std::string name;
  int64_t flops = 0;  // 2*m*n*k summed over the stage's terms (m*n for scalar terms)
};

struct Program {
  std::vector<Stage> stages;
  int64_t p1_size = 0;     // doubles of phase-1 scratch (slot kSlotP1)
  int64_t combo_size = 0;  // doubles of combined blocks (slot kSlotCombo)
  int first_repeat_stage = 0;  // stages [0, first_repeat_stage) run once (combinations)
  int64_t flops() const {
    int64_t f = 0;
    for (auto& s : stages) f += s.flops;
    return f;
  }
};

// Records contractions and lowers them into a Program.
class TaskBuilder {
 public:
  TaskBuilder();

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

  // Closes the current product/accumulation stage pair; later contractions accumulate
  // onto what earlier stages wrote.
  void next_stage(const std::string& name);

  Program finalize();

  int64_t num_terms() const { return static_cast<int64_t>(p2_terms_.size()); }

  // Bytes of the distinct MPS / operator blocks the recorded contractions read (each
  // block counted once, FP64), the operand traffic of one execution of the program.
  int64_t operand_bytes() const;

 private:
  struct PendingTerm { int group; Term t; };
  struct StageBuf {
    std::vector<Group> groups;
    std::vector<PendingTerm> terms;
    std::unordered_map<Ref, int> group_of;
    std::string name;
  };
  // combination stage
  StageBuf combo_;
  int64_t combo_size_ = 0;
  std::unordered_map<std::string, Blk> combo_cache_;
  // product / accumulation stages
  std::vector<StageBuf> p1_stages_, p2_stages_;
  std::unordered_map<std::string, Blk> p1_cache_;
  int64_t p1_size_ = 0;
  std::vector<Term> p2_terms_;  // only for counting
  std::unordered_map<Ref, bool> written_;  // outputs written by closed stages
  std::unordered_map<Ref, int64_t> operands_;  // footprint of MPS / operator operands
  void note_operand(const Blk& b);

  int group_for(StageBuf& sb, const Blk& out, bool accumulate);
  Blk product(const Blk& U, bool tu, const Blk& V, bool tv);
  void add_term(StageBuf& sb, const Blk& out, double alpha, const Blk& U, bool tu, const Blk* V,
                bool tv, bool accumulate);
  static Stage lower(StageBuf& sb, const std::string& name);
};

}  // namespace c2g
