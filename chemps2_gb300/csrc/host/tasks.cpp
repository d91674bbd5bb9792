#include "tasks.hpp"

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <thread>

namespace c2g {

namespace {

inline int64_t align4(int64_t x) { return (x + 3) & ~int64_t(3); }

struct Shape { int r, c; };
inline Shape op_shape(const Blk& b, bool t) { return t ? Shape{b.cols, b.rows} : Shape{b.rows, b.cols}; }

[[noreturn]] void shape_error(const char* what) {
  throw std::logic_error(std::string("task compiler: inconsistent block shapes in ") + what);
}

void append_bytes(std::string& s, const void* p, size_t n) { s.append(static_cast<const char*>(p), n); }

inline uint64_t fmix(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}
inline uint64_t mix(uint64_t h, uint64_t v) { return fmix(h ^ (v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2))); }

}  // namespace

int64_t term_flops(const Term& t, int m, int n) {
  const bool ha = t.flags & kHasA, hc = t.flags & kHasC;
  if (ha && hc) {
    const int64_t ab = int64_t(m) * t.k1 * t.k2 + int64_t(m) * t.k2 * n;
    const int64_t bc = int64_t(t.k1) * t.k2 * n + int64_t(m) * t.k1 * n;
    return 2 * std::min(ab, bc);
  }
  if (ha) return 2 * int64_t(m) * t.k1 * n;
  if (hc) return 2 * int64_t(m) * t.k2 * n;
  return int64_t(m) * n;
}

size_t TaskBuilder::BatchKeyHash::operator()(const BatchKey& k) const {
  uint64_t h = static_cast<uint64_t>(k.group);
  h = mix(h, k.b);
  h = mix(h, (uint64_t(uint32_t(k.flags)) << 32) | uint32_t(k.k1));
  h = mix(h, (uint64_t(uint32_t(k.k2)) << 32) | uint32_t(k.lda));
  h = mix(h, (uint64_t(uint32_t(k.ldc)) << 32) | (uint32_t(k.aslot) << 16) | uint32_t(k.cslot & 0xffff));
  return static_cast<size_t>(h);
}

TaskBuilder::TaskBuilder(bool track_operands) : track_operands_(track_operands) {
  stages_.emplace_back();
  stages_.back().name = "stage0";
}

void TaskBuilder::note_operand(const Blk& b) {
  if (!track_operands_ || !b.valid || ref_slot(b.ref) < kSlotMpsBase) return;
  const int64_t n = int64_t(b.rows) * b.cols;
  int64_t& cur = operands_[b.ref];
  if (n > cur) cur = n;
}

int64_t TaskBuilder::operand_bytes() const {
  int64_t s = 0;
  for (const auto& kv : operands_) s += kv.second;
  return 8 * s;
}

int TaskBuilder::group_for(StageBuf& sb, const Blk& out, bool accumulate) {
  if (&sb == last_sb_ && out.ref == last_out_) return last_group_;
  auto it = sb.group_of.find(out.ref);
  if (it != sb.group_of.end()) {
    const Group& g = sb.groups[it->second];
    if (g.m != out.rows || g.n != out.cols || g.ldo != out.ld) shape_error("output group");
    last_sb_ = &sb;
    last_out_ = out.ref;
    last_group_ = it->second;
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
  sb.terms.emplace_back();
  const int id = static_cast<int>(sb.groups.size()) - 1;
  sb.group_of[out.ref] = id;
  last_sb_ = &sb;
  last_out_ = out.ref;
  last_group_ = id;
  return id;
}

void TaskBuilder::add(StageBuf& sb, bool batchable, const Blk& out, double alpha, const Blk& A, bool ta,
                      const Blk& B, bool tb, const Blk& C, bool tc, bool accumulate) {
  const int g = group_for(sb, out, accumulate);
  Term t{};
  t.a = A.valid ? A.ref : 0;
  t.b = B.ref;
  t.c = C.valid ? C.ref : 0;
  t.alpha = alpha;
  const Shape sb_ = op_shape(B, tb);
  t.k1 = sb_.r;
  t.k2 = sb_.c;
  t.lda = A.valid ? A.ld : 0;
  t.ldb = B.ld;
  t.ldc = C.valid ? C.ld : 0;
  t.flags = (A.valid ? kHasA : 0) | (C.valid ? kHasC : 0) | (A.valid && ta ? kTransA : 0) | (tb ? kTransB : 0) |
            (C.valid && tc ? kTransC : 0);
  t.list = -1;
  t.count = 1;
  t.item0 = 0;
  auto& gt = sb.terms[g];
  Group& G = sb.groups[g];
  if (batchable) {
    // The compilers emit all contractions of one output block consecutively, so only the
    // current group's terms are kept open for batching: the map stays small.
    if (g != open_group_ || &sb != open_sb_) {
      open_.clear();
      open_group_ = g;
      open_sb_ = &sb;
    }
    const BatchKey key{g, t.b, t.flags, t.k1, t.k2, t.lda, t.ldc, A.valid ? ref_slot(A.ref) : -1,
                       C.valid ? ref_slot(C.ref) : -1};
    auto it = open_.find(key);
    if (it != open_.end()) {
      PendingTerm& pt = gt[it->second];
      BatchEntry e;
      e.da = A.valid ? static_cast<int64_t>(A.ref - pt.t.a) : 0;
      e.dc = C.valid ? static_cast<int64_t>(C.ref - pt.t.c) : 0;
      e.ratio = alpha / pt.t.alpha;
      pt.entries.push_back(e);
      G.work += term_flops(pt.t, G.m, G.n);
      return;
    }
    open_.emplace(key, static_cast<int>(gt.size()));
  }
  gt.push_back(PendingTerm{t, {}});
  G.work += term_flops(t, G.m, G.n);
}

Blk TaskBuilder::combine(const std::vector<std::pair<double, Blk>>& parts, int rows, int cols,
                         const std::vector<bool>* transposed) {
  if (parts.empty()) return Blk();
  std::string key;
  key.reserve(parts.size() * 24 + 8);
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
    add(combo_, false, out, parts[i].first, Blk(), false, parts[i].second, t, Blk(), false, false);
  }
  combo_cache_.emplace(std::move(key), out);
  return out;
}

void TaskBuilder::declare_output(const Blk& out) {
  if (!out.valid || out.rows == 0 || out.cols == 0) return;
  group_for(stages_.back(), out, written_.count(out.ref) > 0);
}

void TaskBuilder::contract(const Blk& out, double alpha, const Blk& A, bool ta, const Blk& B, bool tb, const Blk& C,
                           bool tc) {
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
  n_contract_++;
  const bool acc = written_.count(out.ref) > 0;
  StageBuf& st = stages_.back();
  // Zero-sized or zero-weight contractions add nothing; the output still exists.
  if (alpha == 0.0 || m == 0 || n == 0 || sb.r == 0 || sb.c == 0) {
    if (m > 0 && n > 0) group_for(st, out, acc);
    return;
  }
  add(st, true, out, alpha, A, ta, B, tb, C, tc, acc);
}

void TaskBuilder::next_stage(const std::string& name) {
  for (auto& g : stages_.back().groups) written_[g.out] = true;
  open_.clear();
  last_sb_ = nullptr;
  open_sb_ = nullptr;
  open_group_ = -1;
  stages_.emplace_back();
  stages_.back().name = name;
}

Stage TaskBuilder::lower(StageBuf& sb, const std::string& name, std::vector<BatchEntry>& table,
                         std::unordered_map<std::string, int32_t>& lists) {
  Stage st;
  st.name = name;
  st.groups = sb.groups;
  std::string key;
  for (size_t g = 0; g < sb.groups.size(); g++) {
    Group& G = st.groups[g];
    G.t0 = static_cast<int32_t>(st.terms.size());
    int32_t items = 0;
    for (PendingTerm& pt : sb.terms[g]) {
      Term t = pt.t;
      t.item0 = items;
      if ((t.flags & kHasA) && (t.flags & kHasC)) {
        const int64_t ab = int64_t(G.m) * t.k1 * t.k2 + int64_t(G.m) * t.k2 * G.n;
        const int64_t bc = int64_t(t.k1) * t.k2 * G.n + int64_t(G.m) * t.k1 * G.n;
        if (ab < bc) t.flags |= kLeftFirst;
      }
      if (!pt.entries.empty()) {
        key.clear();
        const BatchEntry first{0, 0, 1.0};
        append_bytes(key, &first, sizeof(BatchEntry));
        append_bytes(key, pt.entries.data(), sizeof(BatchEntry) * pt.entries.size());
        auto it = lists.find(key);
        if (it == lists.end()) {
          const int32_t off = static_cast<int32_t>(table.size());
          table.push_back(first);
          table.insert(table.end(), pt.entries.begin(), pt.entries.end());
          it = lists.emplace(key, off).first;
        }
        t.list = it->second;
        t.count = static_cast<int32_t>(pt.entries.size()) + 1;
      }
      items += t.count;
      st.items += t.count;
      st.flops += term_flops(t, G.m, G.n) * t.count;
      st.terms.push_back(t);
    }
    G.t1 = static_cast<int32_t>(st.terms.size());
    std::vector<PendingTerm>().swap(sb.terms[g]);
  }
  return st;
}

Program TaskBuilder::finalize(bool keep_empty) {
  Program p;
  std::unordered_map<std::string, int32_t> lists;
  if (!combo_.groups.empty() || keep_empty) {
    p.stages.push_back(lower(combo_, "combine", p.entries, lists));
    p.first_repeat_stage = 1;
  }
  for (auto& s : stages_)
    if (!s.groups.empty() || keep_empty) p.stages.push_back(lower(s, s.name, p.entries, lists));
  p.combo_size = combo_size_;
  if (p.entries.size() > size_t(INT32_MAX)) throw std::length_error("task compiler: batch table too large");
  return p;
}

Program merge_programs(std::vector<Program>& parts) {
  Program out;
  if (parts.empty()) return out;
  const size_t ns = parts[0].stages.size();
  for (auto& p : parts)
    if (p.stages.size() != ns) throw std::logic_error("merge_programs: shards with different stage lists");
  std::vector<int64_t> combo_base(parts.size()), entry_base(parts.size());
  int64_t cb = 0, eb = 0;
  for (size_t i = 0; i < parts.size(); i++) {
    combo_base[i] = cb;
    entry_base[i] = eb;
    cb = align4(cb + parts[i].combo_size);
    eb += static_cast<int64_t>(parts[i].entries.size());
  }
  if (eb > INT32_MAX) throw std::length_error("merge_programs: batch table too large");
  out.combo_size = cb;
  out.entries.reserve(eb);
  for (auto& p : parts) {
    out.entries.insert(out.entries.end(), p.entries.begin(), p.entries.end());
    std::vector<BatchEntry>().swap(p.entries);
  }
  auto reloc = [&](Ref r, size_t i) -> Ref {
    if (r != 0 && ref_slot(r) == kSlotCombo) return make_ref(kSlotCombo, ref_off(r) + combo_base[i]);
    return r;
  };
  for (size_t s = 0; s < ns; s++) {
    Stage st;
    st.name = parts[0].stages[s].name;
    for (size_t i = 0; i < parts.size(); i++) {
      Stage& ps = parts[i].stages[s];
      const int32_t toff = static_cast<int32_t>(st.terms.size());
      for (Group g : ps.groups) {
        g.out = reloc(g.out, i);
        g.t0 += toff;
        g.t1 += toff;
        st.groups.push_back(g);
      }
      for (Term t : ps.terms) {
        if (t.flags & kHasA) t.a = reloc(t.a, i);
        t.b = reloc(t.b, i);
        if (t.flags & kHasC) t.c = reloc(t.c, i);
        if (t.list >= 0) t.list += static_cast<int32_t>(entry_base[i]);
        st.terms.push_back(t);
      }
      st.flops += ps.flops;
      st.items += ps.items;
      std::vector<Group>().swap(ps.groups);
      std::vector<Term>().swap(ps.terms);
    }
    const bool once = (s == 0 && parts[0].first_repeat_stage == 1);
    if (st.groups.empty()) continue;
    if (once) out.first_repeat_stage = 1;
    out.stages.push_back(std::move(st));
  }
  return out;
}

int compile_threads() {
  if (const char* e = std::getenv("C2G_COMPILE_THREADS")) {
    const int n = std::atoi(e);
    if (n > 0) return std::min(n, 256);
  }
  const unsigned h = std::thread::hardware_concurrency();
  return static_cast<int>(std::max(1u, std::min(h, 64u)));
}

}  // namespace c2g
