// Parallel task compilation: every hot-path compiler emits disjoint outputs per shard, so
// shards are compiled on host threads and merged (tasks.hpp, merge_programs).
#pragma once

#include "heff.hpp"
#include "operators.hpp"
#include "tasks.hpp"

namespace c2g {

struct Compiled {
  Program program;             // the merged program (empty when `parts` is not)
  std::vector<Program> parts;  // the unmerged shards (merge = false); Runtime::upload takes them
  int64_t operand_bytes = 0;   // distinct MPS / operator bytes the program reads
  int64_t contractions = 0;    // block contractions recorded (before batching)
};

// track_operands fills Compiled::operand_bytes (costs compile time). With merge = false
// a program compiled in several shards is left in Compiled::parts.
Compiled compile_heff_program(const HeffContext& ctx, bool track_operands = false, bool merge = true);
Compiled compile_heff_diag_program(const HeffContext& ctx, bool merge = true);
Compiled compile_update_program(const UpdateContext& ctx, bool merge = true);

}  // namespace c2g
