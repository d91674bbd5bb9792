// Host random draws of the DMRG: the random MPS start (CheMPS2/TensorT.cpp:167-173), the
// noise of CheMPS2/Sobject.cpp:652-661 and the Davidson guess fallback
// (CheMPS2/Davidson.cpp:204-214). The reference draws them from the C library's rand().
// A DMRG solved on its own does the same. Problems solved concurrently (the batch entry
// point) each draw from a private generator instead, so their streams do not interleave.
//
// The private generator is the additive-feedback generator of the GNU C library's
// random()/rand() (degree 31, separation 3), as published: the state is seeded by
// r[i] = 16807 r[i-1] mod (2^31 - 1) with Schrage's factorisation, r[31..33] = r[0..2],
// then r[i] = r[i-31] + r[i-3] (mod 2^32), the first 310 outputs of that recurrence are
// discarded, and each draw returns r[i] >> 1. A private generator seeded with s gives the
// sequence that srand(s) followed by rand() gives on that library, so a batch member's
// numbers equal those of a sequential run after srand(s).
#pragma once

#include <cstdint>

namespace c2g {

class HostRand {
 public:
  // draws from the C library's rand()
  HostRand() = default;
  // draws from a private generator seeded with `seed`
  explicit HostRand(unsigned seed);

  int next();
  // a value in [0, 1], as rand() / RAND_MAX
  double unit();
  bool is_private() const { return own_; }

 private:
  bool own_ = false;
  uint32_t ring_[31] = {};
  int pos_ = 0;
};

}  // namespace c2g
