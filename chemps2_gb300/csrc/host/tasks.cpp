#include "tasks.hpp"

#include <cassert>
#include <cstring>
#include <stdexcept>

namespace c2g {

namespace {

inline int64_t align4(int64_t x) { return (x + 3) & ~int64_t(3); }

struct Shape { int r, c; };
inline Shape op_shape(const Blk& b, bool t) { return t ? Shape{b.cols, b.rows} : Shape{b.rows, b.cols}; }

[[noreturn]] void shape_error(const char* what) {
  throw std::logic_error(std::string("task compiler: inconsistent block shapes in ") + what);
}

void append_bytes(std::string& s, const void* p, size_t n) {
  s.append(static_cast<const char*>(p), n);
}

}  // namespace

TaskBuilder::TaskBuilder() {
  p1_stages_.emplace_back();
  p2_stages_.emplace_back();
  p2_stages_.back().name = "stage0";
}

int TaskBuilder::group_for(StageBuf& sb, const Blk& out, bool accumulate) {
  auto it = sb.group_of.find(out.ref);
  if (it != sb.group_of.end()) {
    const Group& g = sb.groups[it->second];
    if (g.m != out.rows || g.n != out.cols || g.ldo != out.ld) shape_error("output group");
    return it->second;
  }
  Group g{};
  g.out = out.ref;
  g.m = out.rows;
  g.n = out.cols;
  g.ldo = out.ld;
  g.flags = accumulate ? kAccumulate : 0;
  g.work = 0;
  sb.groups.push_back(g);
  const int id = static_cast<int>(sb.groups.size()) - 1;
  sb.group_of[out.ref] = id;
  return id;
}

void TaskBuilder::add_term(StageBuf& sb, const Blk& out, double alpha, const Blk& U, bool tu,
                           const Blk* V, bool tv, bool accumulate) {
  const int g = group_for(sb, out, accumulate);
  Term t{};
  t.u = U.ref;
  t.ldu = U.ld;
  t.alpha = alpha;
  t.flags = (tu ? kTransU : 0);
  if (V) {
    t.v = V->ref;
    t.ldv = V->ld;
    t.flags |= (tv ? kTransV : 0);
    t.k = op_shape(U, tu).c;
  } else {
    t.v = 0;
    t.ldv = 0;
    t.k = 0;
    t.flags |= kScalar;
  }
  sb.terms.push_back({g, t});
  Group& gr = sb.groups[g];
  gr.work += V ? int64_t(2) * gr.m * gr.n * t.k : int64_t(gr.m) * gr.n;
}

void TaskBuilder::note_operand(const Blk& b) {
  if (!b.valid || ref_slot(b.ref) < kSlotMpsBase) return;
  const int64_t n = int64_t(b.rows) * b.cols;
  int64_t& cur = operands_[b.ref];
  if (n > cur) cur = n;
}

int64_t TaskBuilder::operand_bytes() const {
  int64_t s = 0;
  for (const auto& kv : operands_) s += kv.second;
  return 8 * s;
}

Blk TaskBuilder::combine(const std::vector<std::pair<double, Blk>>& parts, int rows, int cols,
                         const std::vector<bool>* transposed) {
  if (parts.empty()) return Blk();
  std::string key;
  for (size_t i = 0; i < parts.size(); i++) {
    const bool t = transposed ? (*transposed)[i] : false;
    const Shape s = op_shape(parts[i].second, t);
    if (s.r != rows || s.c != cols) shape_error("combine");
    append_bytes(key, &parts[i].first, sizeof(double));
    append_bytes(key, &parts[i].second.ref, sizeof(Ref));
    append_bytes(key, &parts[i].second.ld, sizeof(int));
    key.push_back(t ? 'T' : 'N');
  }
  append_bytes(key, &rows, sizeof(int));
  append_bytes(key, &cols, sizeof(int));
  auto it = combo_cache_.find(key);
  if (it != combo_cache_.end()) return it->second;
  for (const auto& pr : parts) note_operand(pr.second);
  const Blk out = Blk::make(make_ref(kSlotCombo, combo_size_), rows, cols);
  combo_size_ = align4(combo_size_ + int64_t(rows) * cols);
  for (size_t i = 0; i < parts.size(); i++) {
    const bool t = transposed ? (*transposed)[i] : false;
    add_term(combo_, out, parts[i].first, parts[i].second, t, nullptr, false, false);
  }
  combo_cache_[key] = out;
  return out;
}

Blk TaskBuilder::product(const Blk& U, bool tu, const Blk& V, bool tv) {
  const Shape su = op_shape(U, tu), sv = op_shape(V, tv);
  if (su.c != sv.r) shape_error("product");
  std::string key;
  append_bytes(key, &U.ref, sizeof(Ref));
  append_bytes(key, &U.ld, sizeof(int));
  append_bytes(key, &V.ref, sizeof(Ref));
  append_bytes(key, &V.ld, sizeof(int));
  const int dims[4] = {su.r, su.c, sv.c, (tu ? 1 : 0) + (tv ? 2 : 0)};
  append_bytes(key, dims, sizeof(dims));
  auto it = p1_cache_.find(key);
  if (it != p1_cache_.end()) return it->second;
  const Blk P = Blk::make(make_ref(kSlotP1, p1_size_), su.r, sv.c);
  p1_size_ = align4(p1_size_ + int64_t(su.r) * sv.c);
  add_term(p1_stages_.back(), P, 1.0, U, tu, &V, tv, false);
  p1_cache_[key] = P;
  return P;
}

void TaskBuilder::declare_output(const Blk& out) {
  if (!out.valid || out.rows == 0 || out.cols == 0) return;
  group_for(p2_stages_.back(), out, written_.count(out.ref) > 0);
}

void TaskBuilder::contract(const Blk& out, double alpha, const Blk& A, bool ta, const Blk& B,
                           bool tb, const Blk& C, bool tc) {
  if (!out.valid || !B.valid) shape_error("contract (missing block)");
  const Shape sb = op_shape(B, tb);
  int m, n;
  if (A.valid) {
    const Shape sa = op_shape(A, ta);
    if (sa.c != sb.r) shape_error("contract (A,B)");
    m = sa.r;
  } else {
    m = sb.r;
  }
  if (C.valid) {
    const Shape sc = op_shape(C, tc);
    if (sb.c != sc.r) shape_error("contract (B,C)");
    n = sc.c;
  } else {
    n = sb.c;
  }
  if (m != out.rows || n != out.cols) shape_error("contract (out)");
  note_operand(A);
  note_operand(B);
  note_operand(C);
  const bool acc = written_.count(out.ref) > 0;
  StageBuf& sb2 = p2_stages_.back();
  // Zero-sized or zero-weight contractions add nothing; the output still exists.
  if (alpha == 0.0 || m == 0 || n == 0 || sb.r == 0 || sb.c == 0) {
    if (m > 0 && n > 0) group_for(sb2, out, acc);
    return;
  }
  if (A.valid && C.valid) {
    const Shape sa = op_shape(A, ta);
    const int k1 = sa.c, k2 = sb.c;
    const int64_t cost_ab = int64_t(m) * k1 * k2 + int64_t(m) * k2 * n;
    const int64_t cost_bc = int64_t(k1) * k2 * n + int64_t(m) * k1 * n;
    if (cost_ab <= cost_bc) {
      const Blk P = product(A, ta, B, tb);
      add_term(sb2, out, alpha, P, false, &C, tc, acc);
    } else {
      const Blk P = product(B, tb, C, tc);
      add_term(sb2, out, alpha, A, ta, &P, false, acc);
    }
  } else if (A.valid) {
    add_term(sb2, out, alpha, A, ta, &B, tb, acc);
  } else if (C.valid) {
    add_term(sb2, out, alpha, B, tb, &C, tc, acc);
  } else {
    add_term(sb2, out, alpha, B, tb, nullptr, false, acc);
  }
  p2_terms_.emplace_back();
}

void TaskBuilder::next_stage(const std::string& name) {
  for (auto& g : p2_stages_.back().groups) written_[g.out] = true;
  p1_stages_.emplace_back();
  p2_stages_.emplace_back();
  p2_stages_.back().name = name;
  p1_cache_.clear();
}

Stage TaskBuilder::lower(StageBuf& sb, const std::string& name) {
  Stage st;
  st.name = name;
  const size_t ng = sb.groups.size();
  std::vector<int32_t> count(ng + 1, 0);
  for (auto& pt : sb.terms) count[pt.group + 1]++;
  for (size_t g = 0; g < ng; g++) count[g + 1] += count[g];
  st.terms.resize(sb.terms.size());
  std::vector<int32_t> pos(count.begin(), count.end() - 1);
  for (auto& pt : sb.terms) st.terms[pos[pt.group]++] = pt.t;  // stable: keeps emission order
  st.groups = sb.groups;
  for (size_t g = 0; g < ng; g++) {
    st.groups[g].t0 = count[g];
    st.groups[g].t1 = count[g + 1];
    st.flops += st.groups[g].work;
  }
  return st;
}

Program TaskBuilder::finalize() {
  Program p;
  if (!combo_.groups.empty()) {
    p.stages.push_back(lower(combo_, "combine"));
    p.first_repeat_stage = 1;
  }
  for (size_t s = 0; s < p2_stages_.size(); s++) {
    if (!p1_stages_[s].groups.empty())
      p.stages.push_back(lower(p1_stages_[s], p2_stages_[s].name + ".products"));
    if (!p2_stages_[s].groups.empty()) p.stages.push_back(lower(p2_stages_[s], p2_stages_[s].name));
  }
  p.p1_size = p1_size_;
  p.combo_size = combo_size_;
  return p;
}

}  // namespace c2g
