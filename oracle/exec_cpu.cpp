// ORACLE (test infrastructure, not product code): CPU executor of task programs.
#include "exec_cpu.hpp"

#include <algorithm>
#include <atomic>
#include <sstream>
#include <thread>
#include <utility>

namespace oracle {

using c2g::BatchEntry;
using c2g::Group;
using c2g::Ref;
using c2g::Stage;
using c2g::Term;

namespace {

struct Seg {
  int64_t lo, hi;  // [lo, hi)
};

[[noreturn]] void fail(const std::string& stage, const std::string& what) {
  throw std::runtime_error("task program check failed in stage '" + stage + "': " + what);
}

// Element columns of a stored rows x cols matrix with leading dimension ld.
void add_segments(std::vector<Seg>& out, int64_t off, int rows, int cols, int ld) {
  if (rows <= 0 || cols <= 0) return;
  if (ld >= rows) {
    for (int j = 0; j < cols; j++) out.push_back({off + int64_t(ld) * j, off + int64_t(ld) * j + rows});
  } else {
    // ld < rows only happens for a single row read with unit stride (ones vector)
    out.push_back({off, off + int64_t(ld) * (cols - 1) + rows});
  }
}

inline BatchEntry entry_of(const Term& t, const std::vector<BatchEntry>& table, int p) {
  if (t.list < 0) return BatchEntry{0, 0, 1.0};
  return table[static_cast<size_t>(t.list) + p];
}

}  // namespace

const double* CpuExecutor::ptr(Ref r) const {
  const int s = c2g::ref_slot(r);
  const int64_t off = c2g::ref_off(r);
  const double* base = (s == c2g::kSlotCombo) ? combo_.data() : slots_.at(s).data;
  return base + off;
}

void CpuExecutor::prepare_scratch(const c2g::Program& p) { combo_.assign(std::max<int64_t>(p.combo_size, 1), 0.0); }

void CpuExecutor::check_stage(const Stage& st, const std::vector<BatchEntry>& table) {
  auto slot_size = [&](int s) -> int64_t {
    if (s == c2g::kSlotCombo) return static_cast<int64_t>(combo_.size());
    if (s < 0 || s >= static_cast<int>(slots_.size())) fail(st.name, "slot index out of range");
    if (!slots_[s].data) fail(st.name, "slot " + std::to_string(s) + " is not bound");
    return slots_[s].size;
  };
  auto check_access = [&](Ref r, int rows, int cols, int ld, const char* what) {
    if (rows <= 0 || cols <= 0) return;
    const int s = c2g::ref_slot(r);
    const int64_t off = c2g::ref_off(r);
    if (ld < 1) fail(st.name, std::string(what) + ": leading dimension < 1");
    if (ld < rows && cols > 1 && rows > 1) fail(st.name, std::string(what) + ": leading dimension below the row count");
    const int64_t last = off + (rows - 1) + int64_t(ld) * (cols - 1);
    const int64_t n = slot_size(s);
    if (off < 0 || last >= n) {
      std::ostringstream os;
      os << what << ": access [" << off << ", " << last << "] outside slot " << s << " of size " << n;
      fail(st.name, os.str());
    }
  };
  std::vector<std::vector<Seg>> outs(slots_.size() + 8), ins(slots_.size() + 8);
  for (const Group& G : st.groups) {
    if (G.t0 < 0 || G.t1 > static_cast<int>(st.terms.size()) || G.t0 > G.t1) fail(st.name, "term range");
    check_access(G.out, G.m, G.n, G.ldo, "output");
    add_segments(outs.at(c2g::ref_slot(G.out)), c2g::ref_off(G.out), G.m, G.n, G.ldo);
    int32_t items = 0;
    for (int t = G.t0; t < G.t1; t++) {
      const Term& T = st.terms[t];
      if (T.item0 != items) fail(st.name, "item offsets");
      items += T.count;
      if (T.count < 1) fail(st.name, "empty batch");
      if (T.list >= 0 && static_cast<size_t>(T.list) + T.count > table.size()) fail(st.name, "batch list range");
      if (T.list < 0 && T.count != 1) fail(st.name, "single term with a count");
      const bool ha = T.flags & c2g::kHasA, hc = T.flags & c2g::kHasC;
      const bool ta = T.flags & c2g::kTransA, tb = T.flags & c2g::kTransB, tc = T.flags & c2g::kTransC;
      if (!ha && T.k1 != G.m) fail(st.name, "k1 differs from m without A");
      if (!hc && T.k2 != G.n) fail(st.name, "k2 differs from n without C");
      const int br = tb ? T.k2 : T.k1, bc = tb ? T.k1 : T.k2;
      check_access(T.b, br, bc, T.ldb, "B operand");
      add_segments(ins.at(c2g::ref_slot(T.b)), c2g::ref_off(T.b), br, bc, T.ldb);
      for (int p = 0; p < T.count; p++) {
        const BatchEntry e = entry_of(T, table, p);
        if (ha) {
          const Ref a = T.a + static_cast<uint64_t>(e.da);
          if (c2g::ref_slot(a) != c2g::ref_slot(T.a)) fail(st.name, "batched A leaves its slot");
          const int ar = ta ? T.k1 : G.m, ac = ta ? G.m : T.k1;
          check_access(a, ar, ac, T.lda, "A operand");
          add_segments(ins.at(c2g::ref_slot(a)), c2g::ref_off(a), ar, ac, T.lda);
        }
        if (hc) {
          const Ref c = T.c + static_cast<uint64_t>(e.dc);
          if (c2g::ref_slot(c) != c2g::ref_slot(T.c)) fail(st.name, "batched C leaves its slot");
          const int cr = tc ? G.n : T.k2, cc = tc ? T.k2 : G.n;
          check_access(c, cr, cc, T.ldc, "C operand");
          add_segments(ins.at(c2g::ref_slot(c)), c2g::ref_off(c), cr, cc, T.ldc);
        }
      }
    }
  }
  for (size_t s = 0; s < outs.size(); s++) {
    auto& o = outs[s];
    if (o.empty()) continue;
    std::sort(o.begin(), o.end(), [](const Seg& a, const Seg& b) { return a.lo < b.lo; });
    for (size_t i = 1; i < o.size(); i++)
      if (o[i].lo < o[i - 1].hi) fail(st.name, "two outputs overlap in slot " + std::to_string(s));
    for (const Seg& in : ins[s]) {
      auto it = std::upper_bound(o.begin(), o.end(), in.lo, [](int64_t v, const Seg& g) { return v < g.lo; });
      if (it != o.begin() && std::prev(it)->hi > in.lo) fail(st.name, "an input overlaps an output in slot " + std::to_string(s));
      if (it != o.end() && it->lo < in.hi) fail(st.name, "an input overlaps an output in slot " + std::to_string(s));
    }
  }
}

void CpuExecutor::check(const c2g::Program& p) {
  if (static_cast<int64_t>(combo_.size()) < std::max<int64_t>(p.combo_size, 1)) prepare_scratch(p);
  for (const Stage& st : p.stages) check_stage(st, p.entries);
}

int64_t CpuExecutor::run_group(const Stage& st, const Group& G, const std::vector<BatchEntry>& table,
                               std::vector<double>& acc, std::vector<double>& tmp) {
  int64_t flops = 0;
  if (G.m <= 0 || G.n <= 0) return 0;
  const int m = G.m, n = G.n;
  acc.assign(static_cast<size_t>(m) * n, 0.0);
  for (int t = G.t0; t < G.t1; t++) {
    const Term& T = st.terms[t];
    const bool ha = T.flags & c2g::kHasA, hc = T.flags & c2g::kHasC;
    const bool ta = T.flags & c2g::kTransA, tb = T.flags & c2g::kTransB, tc = T.flags & c2g::kTransC;
    const double* B = ptr(T.b);
    auto opB = [&](int k, int l) { return tb ? B[l + int64_t(T.ldb) * k] : B[k + int64_t(T.ldb) * l]; };
    for (int p = 0; p < T.count; p++) {
      const BatchEntry e = entry_of(T, table, p);
      const double al = T.alpha * e.ratio;
      const double* A = ha ? ptr(T.a + static_cast<uint64_t>(e.da)) : nullptr;
      const double* C = hc ? ptr(T.c + static_cast<uint64_t>(e.dc)) : nullptr;
      auto opA = [&](int i, int k) { return ta ? A[k + int64_t(T.lda) * i] : A[i + int64_t(T.lda) * k]; };
      auto opC = [&](int l, int j) { return tc ? C[j + int64_t(T.ldc) * l] : C[l + int64_t(T.ldc) * j]; };
      if (ha && hc) {
        // tmp = op(B) op(C_p): k1 x n
        tmp.assign(static_cast<size_t>(T.k1) * n, 0.0);
        for (int j = 0; j < n; j++)
          for (int l = 0; l < T.k2; l++) {
            const double c = opC(l, j);
            if (c == 0.0) continue;
            for (int k = 0; k < T.k1; k++) tmp[k + size_t(T.k1) * j] += opB(k, l) * c;
          }
        for (int j = 0; j < n; j++)
          for (int k = 0; k < T.k1; k++) {
            const double v = al * tmp[k + size_t(T.k1) * j];
            if (v == 0.0) continue;
            for (int i = 0; i < m; i++) acc[i + size_t(m) * j] += opA(i, k) * v;
          }
        flops += term_flops(T, m, n);
      } else if (ha) {
        for (int j = 0; j < n; j++)
          for (int k = 0; k < T.k1; k++) {
            const double v = al * opB(k, j);
            if (v == 0.0) continue;
            for (int i = 0; i < m; i++) acc[i + size_t(m) * j] += opA(i, k) * v;
          }
        flops += 2 * int64_t(m) * n * T.k1;
      } else if (hc) {
        for (int j = 0; j < n; j++)
          for (int l = 0; l < T.k2; l++) {
            const double v = al * opC(l, j);
            if (v == 0.0) continue;
            for (int i = 0; i < m; i++) acc[i + size_t(m) * j] += opB(i, l) * v;
          }
        flops += 2 * int64_t(m) * n * T.k2;
      } else {
        for (int j = 0; j < n; j++)
          for (int i = 0; i < m; i++) acc[i + size_t(m) * j] += al * opB(i, j);
        flops += int64_t(m) * n;
      }
    }
  }
  double* O = const_cast<double*>(ptr(G.out));
  const bool accum = G.flags & c2g::kAccumulate;
  for (int c = 0; c < n; c++)
    for (int r = 0; r < m; r++) {
      double& o = O[r + int64_t(G.ldo) * c];
      o = accum ? o + acc[r + size_t(m) * c] : acc[r + size_t(m) * c];
    }
  return flops;
}

namespace {
std::atomic<int> g_threads{1};
}  // namespace

void CpuExecutor::set_threads(int n) { g_threads = std::max(1, std::min(n, 1024)); }
int CpuExecutor::threads() { return g_threads.load(); }

void CpuExecutor::run_stage(const Stage& st, const std::vector<BatchEntry>& table) {
  const size_t ng = st.groups.size();
  const int nt = static_cast<int>(std::min<size_t>(threads(), (ng + 15) / 16));
  if (nt <= 1) {
    std::vector<double> acc, tmp;
    for (const Group& G : st.groups) flops_done += run_group(st, G, table, acc, tmp);
    return;
  }
  std::atomic<size_t> next{0};
  std::atomic<int64_t> flops{0};
  auto work = [&] {
    std::vector<double> acc, tmp;
    int64_t f = 0;
    for (size_t g0 = next.fetch_add(32); g0 < ng; g0 = next.fetch_add(32))
      for (size_t g = g0; g < std::min(ng, g0 + 32); g++) f += run_group(st, st.groups[g], table, acc, tmp);
    flops += f;
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < nt; i++) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  flops_done += flops.load();
}

void CpuExecutor::run(const c2g::Program& p, bool once_stages, bool repeat_stages) {
  for (size_t s = 0; s < p.stages.size(); s++) {
    const bool once = static_cast<int>(s) < p.first_repeat_stage;
    if ((once && once_stages) || (!once && repeat_stages)) run_stage(p.stages[s], p.entries);
  }
}

}  // namespace oracle
