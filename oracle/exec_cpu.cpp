// ORACLE (test infrastructure, not product code): CPU executor of task programs.
#include "exec_cpu.hpp"

#include <algorithm>
#include <sstream>
#include <utility>

namespace oracle {

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

}  // namespace

const double* CpuExecutor::ptr(Ref r) const {
  const int s = c2g::ref_slot(r);
  const int64_t off = c2g::ref_off(r);
  const double* base;
  if (s == c2g::kSlotP1)
    base = p1_.data();
  else if (s == c2g::kSlotCombo)
    base = combo_.data();
  else
    base = slots_.at(s).data;
  return base + off;
}

void CpuExecutor::prepare_scratch(const c2g::Program& p) {
  p1_.assign(std::max<int64_t>(p.p1_size, 1), 0.0);
  combo_.assign(std::max<int64_t>(p.combo_size, 1), 0.0);
}

void CpuExecutor::check_stage(const Stage& st) {
  auto slot_size = [&](int s) -> int64_t {
    if (s == c2g::kSlotP1) return static_cast<int64_t>(p1_.size());
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
    for (int t = G.t0; t < G.t1; t++) {
      const Term& T = st.terms[t];
      const bool tu = T.flags & c2g::kTransU, tv = T.flags & c2g::kTransV;
      if (T.flags & c2g::kScalar) {
        const int r = tu ? G.n : G.m, c = tu ? G.m : G.n;
        check_access(T.u, r, c, T.ldu, "scalar operand");
        add_segments(ins.at(c2g::ref_slot(T.u)), c2g::ref_off(T.u), r, c, T.ldu);
      } else {
        if (T.k < 0) fail(st.name, "negative inner dimension");
        const int ur = tu ? T.k : G.m, uc = tu ? G.m : T.k;
        const int vr = tv ? G.n : T.k, vc = tv ? T.k : G.n;
        check_access(T.u, ur, uc, T.ldu, "left operand");
        check_access(T.v, vr, vc, T.ldv, "right operand");
        add_segments(ins.at(c2g::ref_slot(T.u)), c2g::ref_off(T.u), ur, uc, T.ldu);
        add_segments(ins.at(c2g::ref_slot(T.v)), c2g::ref_off(T.v), vr, vc, T.ldv);
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
  if (static_cast<int64_t>(p1_.size()) < std::max<int64_t>(p.p1_size, 1) ||
      static_cast<int64_t>(combo_.size()) < std::max<int64_t>(p.combo_size, 1))
    prepare_scratch(p);
  for (const Stage& st : p.stages) check_stage(st);
}

void CpuExecutor::run_stage(const Stage& st) {
  std::vector<double> acc;
  for (const Group& G : st.groups) {
    if (G.m <= 0 || G.n <= 0) continue;
    acc.assign(static_cast<size_t>(G.m) * G.n, 0.0);
    for (int t = G.t0; t < G.t1; t++) {
      const Term& T = st.terms[t];
      const bool tu = T.flags & c2g::kTransU, tv = T.flags & c2g::kTransV;
      const double* U = ptr(T.u);
      if (T.flags & c2g::kScalar) {
        for (int c = 0; c < G.n; c++)
          for (int r = 0; r < G.m; r++)
            acc[r + size_t(G.m) * c] += T.alpha * (tu ? U[c + int64_t(T.ldu) * r] : U[r + int64_t(T.ldu) * c]);
        flops_done += int64_t(G.m) * G.n;
        continue;
      }
      const double* V = ptr(T.v);
      for (int c = 0; c < G.n; c++)
        for (int kk = 0; kk < T.k; kk++) {
          const double v = tv ? V[c + int64_t(T.ldv) * kk] : V[kk + int64_t(T.ldv) * c];
          if (v == 0.0) continue;
          const double av = T.alpha * v;
          double* a = &acc[size_t(G.m) * c];
          if (!tu) {
            const double* u = U + int64_t(T.ldu) * kk;
            for (int r = 0; r < G.m; r++) a[r] += u[r] * av;
          } else {
            for (int r = 0; r < G.m; r++) a[r] += U[kk + int64_t(T.ldu) * r] * av;
          }
        }
      flops_done += 2 * int64_t(G.m) * G.n * T.k;
    }
    double* O = const_cast<double*>(ptr(G.out));
    const bool accum = G.flags & c2g::kAccumulate;
    for (int c = 0; c < G.n; c++)
      for (int r = 0; r < G.m; r++) {
        double& o = O[r + int64_t(G.ldo) * c];
        o = accum ? o + acc[r + size_t(G.m) * c] : acc[r + size_t(G.m) * c];
      }
  }
}

void CpuExecutor::run(const c2g::Program& p, bool once_stages, bool repeat_stages) {
  for (size_t s = 0; s < p.stages.size(); s++) {
    const bool once = static_cast<int>(s) < p.first_repeat_stage;
    if ((once && once_stages) || (!once && repeat_stages)) run_stage(p.stages[s]);
  }
}

}  // namespace oracle
