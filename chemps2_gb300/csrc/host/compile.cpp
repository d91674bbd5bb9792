#include "compile.hpp"

#include <exception>
#include <thread>
#include <unordered_set>

namespace c2g {

namespace {

template <class F>
Compiled run_sharded(F emit, bool track, bool merge) {
  const int n = compile_threads();
  Compiled out;
  if (n <= 1) {
    TaskBuilder tb(track);
    emit(tb, 0, 1);
    out.program = tb.finalize();
    out.operand_bytes = tb.operand_bytes();
    out.contractions = tb.num_contractions();
    return out;
  }
  std::vector<Program> parts(n);
  std::vector<RefSizes> operands(n);
  std::vector<int64_t> contractions(n, 0);
  std::vector<std::exception_ptr> errors(n);
  std::vector<std::thread> threads;
  threads.reserve(n);
  for (int i = 0; i < n; i++)
    threads.emplace_back([&, i] {
      try {
        TaskBuilder tb(track);
        emit(tb, i, n);
        parts[i] = tb.finalize(true);
        operands[i] = tb.operands();
        contractions[i] = tb.num_contractions();
      } catch (...) {
        errors[i] = std::current_exception();
      }
    });
  for (auto& t : threads) t.join();
  for (auto& e : errors)
    if (e) std::rethrow_exception(e);
  if (merge) out.program = merge_programs(parts);
  else out.parts = std::move(parts);
  if (track) {
    RefSizes all;
    for (auto& m : operands) m.for_each([&](Ref r, int64_t v) { all.note(r, v); });
    out.operand_bytes = 8 * all.total();
  }
  for (int64_t c : contractions) out.contractions += c;
  return out;
}

}  // namespace

Compiled compile_heff_program(const HeffContext& ctx, bool track_operands, bool merge) {
  return run_sharded([&](TaskBuilder& tb, int shard, int n) { compile_heff(tb, ctx, shard, n); }, track_operands,
                     merge);
}

Compiled compile_heff_diag_program(const HeffContext& ctx, bool merge) {
  return run_sharded([&](TaskBuilder& tb, int shard, int n) { compile_heff_diag(tb, ctx, shard, n); }, false, merge);
}

Compiled compile_update_program(const UpdateContext& ctx, bool merge) {
  return run_sharded([&](TaskBuilder& tb, int shard, int n) {
    UpdateContext c = ctx;
    c.shard = shard;
    c.nshards = n;
    compile_update(tb, c);
  }, false, merge);
}

}  // namespace c2g
