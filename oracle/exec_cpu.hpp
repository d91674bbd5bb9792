// ORACLE (test infrastructure, not product code): a CPU executor of task programs.
//
// Executes a c2g::Program with plain loops in the exact semantics the device kernels
// implement: for every group, out (+)= sum over its terms, in order, of
// alpha * op(U) * op(V) (or alpha * op(U)). Before executing, it checks every access of
// every term against the size of the buffer its slot is bound to, and that within one
// stage no output overlaps another output or any input (the device runs all groups of a
// stage concurrently). A violation throws, so a program is known to stay in bounds before
// it is ever launched on a GPU.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "tasks.hpp"

namespace oracle {

struct Buffer {
  double* data = nullptr;
  int64_t size = 0;  // doubles
};

class CpuExecutor {
 public:
  explicit CpuExecutor(int nslots) : slots_(nslots) {}
  void bind(int slot, double* data, int64_t size) { slots_.at(slot) = Buffer{data, size}; }
  Buffer& slot(int s) { return slots_.at(s); }

  // check() verifies p; run() executes its once stages and / or repeat stages. The
  // combination scratch is owned by the executor (prepare_scratch).
  void check(const c2g::Program& p);
  void run(const c2g::Program& p, bool once_stages, bool repeat_stages);
  void prepare_scratch(const c2g::Program& p);

  int64_t flops_done = 0;

  // Host threads that execute the groups of a stage (independent outputs); results do not
  // depend on it (each group is computed by one thread in the fixed term order).
  static void set_threads(int n);
  static int threads();

 private:
  std::vector<Buffer> slots_;
  std::vector<double> combo_;
  void check_stage(const c2g::Stage& st, const std::vector<c2g::BatchEntry>& table);
  void run_stage(const c2g::Stage& st, const std::vector<c2g::BatchEntry>& table);
  int64_t run_group(const c2g::Stage& st, const c2g::Group& G, const std::vector<c2g::BatchEntry>& table,
                    std::vector<double>& acc, std::vector<double>& tmp);
  const double* ptr(c2g::Ref r) const;
};

}  // namespace oracle
