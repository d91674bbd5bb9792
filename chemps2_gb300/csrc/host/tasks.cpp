#include "tasks.hpp"

#include <algorithm>
#include <atomic>
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

void TaskBuilder::OpenTerms::insert(uint64_t h, int32_t term) {
  if ((n_ + 1) * 2 > stamps_.size()) {
    // grow, keeping the current entries (in probe order, so equal hashes keep their order)
    std::vector<uint32_t> os;
    std::vector<uint64_t> oh;
    std::vector<int32_t> ot;
    os.swap(stamps_);
    oh.swap(hashes_);
    ot.swap(terms_);
    const size_t cap = std::max<size_t>(64, os.size() * 2);
    stamps_.assign(cap, 0u);
    hashes_.assign(cap, 0);
    terms_.assign(cap, -1);
    mask_ = cap - 1;
    const uint32_t cur = stamp_;
    stamp_ = 1;
    n_ = 0;
    for (size_t i = 0; i < os.size(); i++)
      if (os[i] == cur) insert(oh[i], ot[i]);
  }
  size_t i = h & mask_;
  while (stamps_[i] == stamp_) i = (i + 1) & mask_;
  stamps_[i] = stamp_;
  hashes_[i] = h;
  terms_[i] = term;
  n_++;
}

TaskBuilder::TaskBuilder(bool track_operands) : track_operands_(track_operands) {
  stages_.emplace_back();
  stages_.back().name = "stage0";
}

void TaskBuilder::note_operand(const Blk& b) {
  if (!track_operands_ || !b.valid || ref_slot(b.ref) < kSlotMpsBase) return;
  const int64_t n = int64_t(b.rows) * b.cols;
  if (seen_ref_.empty()) {
    seen_ref_.assign(kOperandCache, 0);
    seen_n_.assign(kOperandCache, 0);
  }
  const size_t h = static_cast<size_t>((b.ref * 0x9e3779b97f4a7c15ull) >> 50) & (kOperandCache - 1);
  if (seen_ref_[h] == b.ref) {
    if (n <= seen_n_[h]) return;  // already noted with at least this size
  } else {
    seen_ref_[h] = b.ref;
  }
  seen_n_[h] = n;
  operands_.note(b.ref, n);
}

int64_t TaskBuilder::operand_bytes() const { return 8 * operands_.total(); }

int TaskBuilder::group_for(StageBuf& sb, const Blk& out) {
  if (&sb == last_sb_ && out.ref == last_out_) return last_group_;
  const int found = sb.group_of.find(out.ref);
  if (found >= 0) {
    const Group& g = sb.groups[found];
    if (g.m != out.rows || g.n != out.cols || g.ldo != out.ld) shape_error("output group");
    last_sb_ = &sb;
    last_out_ = out.ref;
    last_group_ = found;
    return found;
  }
  const bool accumulate = (&sb != &combo_) && written_.find(out.ref) >= 0;
  Group g{};
  g.out = out.ref;
  g.m = out.rows;
  g.n = out.cols;
  g.ldo = out.ld;
  g.flags = accumulate ? kAccumulate : 0;
  g.work = 0;
  sb.groups.push_back(g);
  const int id = static_cast<int>(sb.groups.size()) - 1;
  sb.group_of.insert(out.ref, id);
  last_sb_ = &sb;
  last_out_ = out.ref;
  last_group_ = id;
  return id;
}

void TaskBuilder::add(StageBuf& sb, bool batchable, const Blk& out, double alpha, const Blk& A, bool ta,
                      const Blk& B, bool tb, const Blk& C, bool tc) {
  const int g = group_for(sb, out);
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
  const int32_t idx = static_cast<int32_t>(sb.terms.size());
  if (batchable) {
    // The compilers emit all contractions of one output block consecutively, so only the
    // current group's terms are kept open for batching: the table stays small.
    if (g != open_group_ || &sb != open_sb_) {
      open_.clear();
      open_group_ = g;
      open_sb_ = &sb;
    }
    const int aslot = A.valid ? ref_slot(A.ref) : -1, cslot = C.valid ? ref_slot(C.ref) : -1;
    // multiply-xor combination of the key words (independent multiplies), high bits folded
    // down for the table index
    uint64_t h = (t.b * 0x9e3779b97f4a7c15ull) ^
                 (((uint64_t(uint32_t(t.flags)) << 32) | uint32_t(t.k1)) * 0xc2b2ae3d27d4eb4full) ^
                 (((uint64_t(uint32_t(t.k2)) << 32) | uint32_t(t.lda)) * 0x165667b19e3779f9ull) ^
                 (((uint64_t(uint32_t(t.ldc)) << 32) | (uint32_t(aslot & 0xffff) << 16) | uint32_t(cslot & 0xffff)) *
                  0x27d4eb2f165667c5ull);
    h ^= h >> 29;
    const int32_t hit = open_.find(h, [&](int32_t k) {
      const Term& o = sb.terms[k];
      return o.b == t.b && o.flags == t.flags && o.k1 == t.k1 && o.k2 == t.k2 && o.lda == t.lda && o.ldc == t.ldc &&
             ((o.flags & kHasA) ? ref_slot(o.a) : -1) == aslot && ((o.flags & kHasC) ? ref_slot(o.c) : -1) == cslot;
    });
    if (hit >= 0) {
      const Term& o = sb.terms[hit];
      BatchEntry e;
      e.da = A.valid ? static_cast<int64_t>(A.ref - o.a) : 0;
      e.dc = C.valid ? static_cast<int64_t>(C.ref - o.c) : 0;
      e.ratio = alpha / o.alpha;
      sb.extra.push_back(e);
      sb.extra_term.push_back(hit);
      return;
    }
    open_.insert(h, idx);
  }
  sb.terms.push_back(t);
  sb.term_group.push_back(g);
}

Blk TaskBuilder::combine(const std::vector<std::pair<double, Blk>>& parts, int rows, int cols,
                         const std::vector<bool>* transposed) {
  if (parts.empty()) return Blk();
  std::vector<uint64_t>& key = key_scratch_;
  key.clear();
  for (size_t i = 0; i < parts.size(); i++) {
    const bool t = transposed ? (*transposed)[i] : false;
    const Shape s = op_shape(parts[i].second, t);
    if (s.r != rows || s.c != cols) shape_error("combine");
    uint64_t a;
    std::memcpy(&a, &parts[i].first, sizeof(a));
    key.push_back(a);
    key.push_back(parts[i].second.ref);
    key.push_back((uint64_t(uint32_t(parts[i].second.ld)) << 1) | (t ? 1u : 0u));
  }
  key.push_back((uint64_t(uint32_t(rows)) << 32) | uint32_t(cols));
  uint64_t h = 0x243f6a8885a308d3ull;
  for (uint64_t w : key) h = mix(h, w);
  int32_t hit = -1;
  combo_index_.visit(h, [&](int32_t idx) {
    const ComboEntry& e = combo_entries_[idx];
    if (e.nwords == static_cast<int32_t>(key.size()) &&
        std::memcmp(combo_words_.data() + e.word0, key.data(), sizeof(uint64_t) * key.size()) == 0) {
      hit = idx;
      return true;
    }
    return false;
  });
  if (hit >= 0) return combo_entries_[hit].out;
  for (const auto& pr : parts) note_operand(pr.second);
  const Blk out = Blk::make(make_ref(kSlotCombo, combo_size_), rows, cols);
  combo_size_ = align4(combo_size_ + int64_t(rows) * cols);
  for (size_t i = 0; i < parts.size(); i++) {
    const bool t = transposed ? (*transposed)[i] : false;
    add(combo_, false, out, parts[i].first, Blk(), false, parts[i].second, t, Blk(), false);
  }
  combo_index_.insert(h, static_cast<int32_t>(combo_entries_.size()));
  combo_entries_.push_back(ComboEntry{static_cast<int64_t>(combo_words_.size()), static_cast<int32_t>(key.size()), out});
  combo_words_.insert(combo_words_.end(), key.begin(), key.end());
  return out;
}

void TaskBuilder::declare_output(const Blk& out) {
  if (!out.valid || out.rows == 0 || out.cols == 0) return;
  group_for(stages_.back(), out);
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
  StageBuf& st = stages_.back();
  // Zero-sized or zero-weight contractions add nothing; the output still exists.
  if (alpha == 0.0 || m == 0 || n == 0 || sb.r == 0 || sb.c == 0) {
    if (m > 0 && n > 0) group_for(st, out);
    return;
  }
  add(st, true, out, alpha, A, ta, B, tb, C, tc);
}

void TaskBuilder::next_stage(const std::string& name) {
  for (auto& g : stages_.back().groups)
    if (written_.find(g.out) < 0) written_.insert(g.out, 1);
  open_.clear();
  last_sb_ = nullptr;
  open_sb_ = nullptr;
  open_group_ = -1;
  stages_.emplace_back();
  stages_.back().name = name;
}

Stage TaskBuilder::lower(StageBuf& sb, const std::string& name, std::vector<BatchEntry>& table,
                         FlatIndex& lists) {
  Stage st;
  st.name = name;
  st.groups = std::move(sb.groups);
  const size_t ng = st.groups.size(), nt = sb.terms.size(), ne = sb.extra.size();
  // terms by group, entries by term, both in emission order (counting sorts)
  std::vector<int32_t> gstart(ng + 1, 0), order(nt);
  for (size_t k = 0; k < nt; k++) gstart[sb.term_group[k] + 1]++;
  for (size_t g = 0; g < ng; g++) gstart[g + 1] += gstart[g];
  {
    std::vector<int32_t> fill(gstart.begin(), gstart.end() - 1);
    for (size_t k = 0; k < nt; k++) order[fill[sb.term_group[k]]++] = static_cast<int32_t>(k);
  }
  std::vector<int32_t> estart(nt + 1, 0);
  std::vector<BatchEntry> ebuf(ne);
  for (size_t q = 0; q < ne; q++) estart[sb.extra_term[q] + 1]++;
  for (size_t k = 0; k < nt; k++) estart[k + 1] += estart[k];
  {
    std::vector<int32_t> fill(estart.begin(), estart.end() - 1);
    for (size_t q = 0; q < ne; q++) ebuf[fill[sb.extra_term[q]]++] = sb.extra[q];
  }
  std::vector<BatchEntry>().swap(sb.extra);
  std::vector<int32_t>().swap(sb.extra_term);
  st.terms.reserve(nt);
  for (size_t g = 0; g < ng; g++) {
    Group& G = st.groups[g];
    G.t0 = static_cast<int32_t>(st.terms.size());
    int32_t items = 0;
    for (int32_t j = gstart[g]; j < gstart[g + 1]; j++) {
      const int32_t k = order[j];
      Term t = sb.terms[k];
      t.item0 = items;
      if ((t.flags & kHasA) && (t.flags & kHasC)) {
        const int64_t ab = int64_t(G.m) * t.k1 * t.k2 + int64_t(G.m) * t.k2 * G.n;
        const int64_t bc = int64_t(t.k1) * t.k2 * G.n + int64_t(G.m) * t.k1 * G.n;
        if (ab < bc) t.flags |= kLeftFirst;
      }
      const size_t n = static_cast<size_t>(estart[k + 1] - estart[k]);
      if (n > 0) {
        // the list is entry 0 (the term itself) followed by the term's further entries
        const BatchEntry* pe = ebuf.data() + estart[k];
        const BatchEntry first{0, 0, 1.0};
        uint64_t h = 0x13198a2e03707344ull ^ (n * 0x9e3779b97f4a7c15ull);
        for (size_t q = 0; q < n; q++) {
          uint64_t r;
          std::memcpy(&r, &pe[q].ratio, sizeof(r));
          h = (h ^ (static_cast<uint64_t>(pe[q].da) * 0xc2b2ae3d27d4eb4full) ^
               (static_cast<uint64_t>(pe[q].dc) * 0x165667b19e3779f9ull) ^ (r * 0x27d4eb2f165667c5ull)) *
              0xff51afd7ed558ccdull;
          h ^= h >> 32;
        }
        int32_t found = -1;
        lists.visit(h, [&](int32_t off) {
          if (off + 1 + n > table.size()) return false;
          const BatchEntry* l = table.data() + off;
          bool same = l[0].da == 0 && l[0].dc == 0 && l[0].ratio == 1.0;
          for (size_t q = 0; same && q < n; q++)
            same = l[q + 1].da == pe[q].da && l[q + 1].dc == pe[q].dc &&
                   std::memcmp(&l[q + 1].ratio, &pe[q].ratio, sizeof(double)) == 0;
          if (same) found = off;
          return same;
        });
        if (found < 0) {
          found = static_cast<int32_t>(table.size());
          table.push_back(first);
          table.insert(table.end(), pe, pe + n);
          lists.insert(h, found);
        }
        t.list = found;
        t.count = static_cast<int32_t>(n) + 1;
      }
      items += t.count;
      st.items += t.count;
      const int64_t f = term_flops(t, G.m, G.n) * t.count;
      st.flops += f;
      G.work += f;
      st.terms.push_back(t);
    }
    G.t1 = static_cast<int32_t>(st.terms.size());
  }
  std::vector<Term>().swap(sb.terms);
  std::vector<int32_t>().swap(sb.term_group);
  return st;
}

Program TaskBuilder::finalize(bool keep_empty) {
  Program p;
  FlatIndex lists;
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
  out.entries.resize(eb);
  {
    auto copy_entries = [&](size_t i) {
      std::copy(parts[i].entries.begin(), parts[i].entries.end(), out.entries.begin() + entry_base[i]);
      std::vector<BatchEntry>().swap(parts[i].entries);
    };
    std::vector<std::thread> th;
    for (size_t i = 0; i < parts.size(); i++) {
      if (eb < 65536) copy_entries(i);
      else th.emplace_back(copy_entries, i);
    }
    for (auto& t : th) t.join();
  }
  auto reloc = [&](Ref r, size_t i) -> Ref {
    if (r != 0 && ref_slot(r) == kSlotCombo) return make_ref(kSlotCombo, ref_off(r) + combo_base[i]);
    return r;
  };
  // Stage by stage: the parts' groups and terms are relocated into their final positions
  // by one thread per part.
  const size_t np = parts.size();
  for (size_t s = 0; s < ns; s++) {
    Stage st;
    st.name = parts[0].stages[s].name;
    std::vector<size_t> gbase(np + 1, 0), tbase(np + 1, 0);
    for (size_t i = 0; i < np; i++) {
      gbase[i + 1] = gbase[i] + parts[i].stages[s].groups.size();
      tbase[i + 1] = tbase[i] + parts[i].stages[s].terms.size();
      st.flops += parts[i].stages[s].flops;
      st.items += parts[i].stages[s].items;
    }
    if (tbase[np] > size_t(INT32_MAX)) throw std::length_error("merge_programs: too many terms in a stage");
    st.groups.resize(gbase[np]);
    st.terms.resize(tbase[np]);
    auto relocate = [&](size_t i) {
      Stage& ps = parts[i].stages[s];
      const int32_t toff = static_cast<int32_t>(tbase[i]);
      Group* gd = st.groups.data() + gbase[i];
      for (size_t k = 0; k < ps.groups.size(); k++) {
        Group g = ps.groups[k];
        g.out = reloc(g.out, i);
        g.t0 += toff;
        g.t1 += toff;
        gd[k] = g;
      }
      Term* td = st.terms.data() + tbase[i];
      const int32_t lbase = static_cast<int32_t>(entry_base[i]);
      for (size_t k = 0; k < ps.terms.size(); k++) {
        Term t = ps.terms[k];
        if (t.flags & kHasA) t.a = reloc(t.a, i);
        t.b = reloc(t.b, i);
        if (t.flags & kHasC) t.c = reloc(t.c, i);
        if (t.list >= 0) t.list += lbase;
        td[k] = t;
      }
      std::vector<Group>().swap(ps.groups);
      std::vector<Term>().swap(ps.terms);
    };
    if (tbase[np] < 65536 || np == 1) {
      for (size_t i = 0; i < np; i++) relocate(i);
    } else {
      std::vector<std::thread> th;
      th.reserve(np);
      for (size_t i = 0; i < np; i++) th.emplace_back(relocate, i);
      for (auto& t : th) t.join();
    }
    const bool once = (s == 0 && parts[0].first_repeat_stage == 1);
    if (st.groups.empty()) continue;
    if (once) out.first_repeat_stage = 1;
    out.stages.push_back(std::move(st));
  }
  return out;
}

namespace {
thread_local int t_compile_threads = 0;
thread_local bool t_shared = false;
std::atomic<int> g_sharing{0};  // threads currently sharing the cores
}  // namespace

void set_thread_compile_threads(int n) { t_compile_threads = std::max(0, std::min(n, 256)); }

void share_compile_threads(bool on) {
  if (on == t_shared) return;
  t_shared = on;
  g_sharing += on ? 1 : -1;
}

int compile_threads() {
  if (t_shared) {
    const int hw = static_cast<int>(std::max(1u, std::min(std::thread::hardware_concurrency(), 64u)));
    return std::max(1, hw / std::max(1, g_sharing.load()));
  }
  if (t_compile_threads > 0) return t_compile_threads;
  if (const char* e = std::getenv("C2G_COMPILE_THREADS")) {
    const int n = std::atoi(e);
    if (n > 0) return std::min(n, 256);
  }
  const unsigned h = std::thread::hardware_concurrency();
  return static_cast<int>(std::max(1u, std::min(h, 64u)));
}

}  // namespace c2g
