// Renormalized operators of one boundary and the compiler of their updates.
//
// A BoundaryOps holds every operator tensor that the reference keeps for one boundary
// and sweep direction (CheMPS2/DMRGoperators.cpp:909-1145): the single creators L, the
// pair operators F0/F1/S0/S1 of the side already swept, the complementary pair operators
// A/B/C/D and the complementary triple operators Q of the other side, and the block
// Hamiltonian X. All tensors of a boundary are packed into one buffer slot.
//
// compile_update() records, as contraction tasks, exactly the work of
// DMRG::updateMovingRight / updateMovingLeft (CheMPS2/DMRGoperators.cpp:243-908): the
// generic TensorOperator::update, TensorL::create, the makenew routines of F0/F1/S0/S1,
// TensorQ::AddTerm*, TensorX::update and the complementary-operator sums.
#pragma once

#include <memory>
#include <vector>

#include "chemps2/Problem.h"
#include "chemps2/SyBookkeeper.h"
#include "layout.hpp"
#include "tasks.hpp"

namespace c2g {

struct OpT {
  const OpLayout* lay = nullptr;
  Ref base = 0;
  bool moving_right = true, prime_last = true, jw_phase = false;
  int site = -1;  // Q tensors: the orbital the complementary operator refers to

  bool valid() const { return lay != nullptr; }
  int two_j() const { return lay->two_j; }
  int n_elec() const { return lay->n_elec; }
  int irrep() const { return lay->n_irrep; }
  int64_t size() const { return lay->size(); }
  Blk blk(int n1, int s1, int i1, int n2, int s2, int i2) const {
    if (!lay) return Blk();
    const int k = lay->kappa(n1, s1, i1, n2, s2, i2);
    if (k < 0) return Blk();
    return Blk::make(base + lay->k2i[k], lay->rows[k], lay->cols[k]);
  }
  Blk blk_k(int k) const { return Blk::make(base + lay->k2i[k], lay->rows[k], lay->cols[k]); }
};

struct MpsT {
  const MpsLayout* lay = nullptr;
  Ref base = 0;
  Blk blk(int nl, int sl, int il, int nr, int sr, int ir) const {
    const int k = lay->kappa(nl, sl, il, nr, sr, ir);
    if (k < 0) return Blk();
    return Blk::make(base + lay->k2i[k], lay->rows[k], lay->cols[k]);
  }
};

struct BoundaryOps {
  int index = -1;  // the reference's index: operators live at boundary index + 1
  bool moving_right = true;
  int slot = -1;
  int64_t size = 0;  // doubles
  std::unique_ptr<OpLayoutCache> layouts;
  std::vector<OpT> L;                                   // [cnt2]
  std::vector<std::vector<OpT>> F0, F1, S0, S1;         // [cnt2][cnt3]; S1[0] empty
  std::vector<std::vector<OpT>> A, B, C, D;             // [cnt2][cnt3]; B[0] empty
  std::vector<OpT> Q;                                   // [cnt2]
  OpT X;
  std::vector<const OpT*> all;                          // every tensor, allocation order

  // Operator on orbital `site` (L), on the pair (s1 <= s2) (F/S on the swept side,
  // A/B/C/D on the other side), or Q of orbital `site`. The mapping of (cnt2, cnt3)
  // onto orbitals follows CheMPS2/DMRGoperators.cpp:921-1109.
  const OpT& Lop(int site) const;
  const OpT& Qop(int site) const;
};

// Allocates (lays out) the operator set of boundary index + 1 for the given direction,
// using the current dimensions of bk. Offsets are relative to `slot`.
void allocate_ops(BoundaryOps& ops, const CheMPS2::SyBookkeeper& bk, int L, int index,
                  bool moving_right, int slot);

struct UpdateContext {
  const CheMPS2::SyBookkeeper* bk = nullptr;
  const CheMPS2::Problem* prob = nullptr;
  int L = 0;
  int index = 0;             // reference's index of updateMovingRight/Left
  bool moving_right = true;
  const BoundaryOps* prev = nullptr;  // boundary index (right) / index + 2 (left); null at the edge
  BoundaryOps* next = nullptr;        // boundary index + 1
  MpsT mps;                            // MPS[index] (right) or MPS[index + 1] (left)
  // Sharded compilation: only the output tensors t with (allocation order of t) % nshards
  // == shard are emitted. Shards write disjoint outputs and can be compiled in parallel.
  int shard = 0, nshards = 1;
};

// The generic TensorOperator::update (CheMPS2/TensorOperator.cpp:163-405) of `out`, at the
// boundary of its layout, from `prev` at the previous boundary in out's direction, through
// the MPS tensor T of the site between them.
void emit_generic_update(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, const CheMPS2::Problem& prob,
                         const MpsT& T, int L, const OpT& out, const OpT& prev);

// Records the whole operator update of one boundary. Stage 1 builds every tensor from
// the previous boundary; stage 2 adds the freshly made pair operators into the
// complementary A/B/C/D tensors (CheMPS2/DMRGoperators.cpp:370-403, :703-736).
void compile_update(TaskBuilder& tb, const UpdateContext& ctx);

}  // namespace c2g
