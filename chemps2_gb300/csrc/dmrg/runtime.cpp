#include "runtime.hpp"

#include <string>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <numeric>
#include <sstream>
#include <thread>
#include <tuple>

namespace c2g {

namespace {
std::atomic<int64_t> g_launches{0};
inline int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// A team-variant tile before its items are split.

// Scheduling weight of one item of a term on a rows x cols tile: its flops plus a fixed
// per-item cost (term lookup, batch entry, pointer setup).
int64_t item_cost(const Term& t, int rows, int cols) { return term_flops(t, rows, cols) + 64; }

// Slots (concurrently evaluated items) of a team-variant CTA of tile class `cls`.
int warp_slots(int cls) {
  static const int gr[kWarpRowClasses] = {1, 1, 2, 2, 4, 4};
  static const int gc[kWarpColClasses] = {1, 2, 4, 4, 8};
  return 4 * 32 / (gr[warp_row_class(cls)] * gc[cls % kWarpColClasses]);
}

// The team variant spreads a stage over at least this many CTA-sized pieces of work, and
// splits a tile over at most kWarpMaxSplit CTAs.
constexpr int64_t kWarpCtaTarget = 2048;
constexpr int kWarpMaxSplit = 64;
}  // namespace

int64_t kernel_launches() { return g_launches.load(); }
void count_launches(int64_t n) { g_launches += n; }

void cuda_check(cudaError_t e, const char* expr, const char* file, int line) {
  if (e == cudaSuccess) return;
  std::ostringstream os;
  os << "CUDA error " << cudaGetErrorName(e) << " (" << cudaGetErrorString(e) << ") at " << file << ":" << line
     << " in " << expr;
  throw CudaError(e, os.str());
}

DevProgram::~DevProgram() {
  if (rt) {
    rt->release_quiet(blob);
    rt->release_quiet(combo);
    rt->release_quiet(combo32);
  }
}

Runtime::Runtime(int L, int device) : L_(L) {
  if (num_slots(L) > kMaxSlots) throw std::invalid_argument("chain too long for the device slot table");
  int count = 0;
  C2G_CUDA(cudaGetDeviceCount(&count));
  if (count <= 0) throw std::runtime_error("no CUDA device available: the DMRG hot path runs only on the GPU");
  if (device < 0) C2G_CUDA(cudaGetDevice(&device));
  C2G_CUDA(cudaSetDevice(device));
  device_ = device;
  C2G_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  C2G_CUDA(cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking));
  for (int b = 0; b < 2; b++) C2G_CUDA(cudaEventCreateWithFlags(&stg_ev_[b], cudaEventDisableTiming));
  // Keep freed blocks in the stream-ordered pool instead of returning them to the driver.
  cudaMemPool_t pool;
  C2G_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t threshold = UINT64_MAX;
  C2G_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
  host_slots_.assign(kMaxSlots, nullptr);
  host_slots32_.assign(kMaxSlots, nullptr);
  C2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&dev_slots_), sizeof(double*) * kMaxSlots));
  C2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&dev_slots32_), sizeof(float*) * kMaxSlots));
  C2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&partial_), sizeof(double) * (kDotBlocks * 64 + 4096)));
  // tile-scheduler counters of the persistent tensor-core kernels (two per kernel)
  C2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&sched_), sizeof(unsigned int) * 4));
  C2G_CUDA(cudaMemset(sched_, 0, sizeof(unsigned int) * 4));
  C2G_CUDA(cudaMallocHost(reinterpret_cast<void**>(&pinned_), sizeof(double) * 8));
  // error word of the kernels with bounded waits, mapped so that the host reads it after
  // any synchronisation without a copy
  C2G_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&err_host_), sizeof(int), cudaHostAllocMapped));
  *err_host_ = 0;
  C2G_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&err_dev_), err_host_, 0));
}

Runtime::~Runtime() {
  if (stream_) cudaStreamSynchronize(stream_);
  if (ones_) cudaFreeAsync(ones_, stream_);
  if (x32_) cudaFreeAsync(x32_, stream_);
  if (stream_) cudaStreamSynchronize(stream_);
  cudaFree(dev_slots_);
  cudaFree(dev_slots32_);
  cudaFree(partial_);
  cudaFree(sched_);
  if (copy_) cudaStreamSynchronize(copy_);
  for (int b = 0; b < 2; b++) {
    if (stg_buf_[b]) cudaFreeHost(stg_buf_[b]);
    if (stg_ev_[b]) cudaEventDestroy(stg_ev_[b]);
  }
  if (copy_) cudaStreamDestroy(copy_);
  for (int k = 0; k < kTransientKinds; k++)
    if (transient_[k]) cudaFreeAsync(transient_[k], stream_);
  if (stream_) cudaStreamSynchronize(stream_);
  if (pinned_) cudaFreeHost(pinned_);
  if (err_host_) cudaFreeHost(err_host_);
  if (aux_) {
    cudaStreamSynchronize(aux_);
    cudaStreamDestroy(aux_);
  }
  if (fork_ev_) cudaEventDestroy(fork_ev_);
  if (ext_in_) cudaEventDestroy(ext_in_);
  if (ext_out_) cudaEventDestroy(ext_out_);
  if (join_ev_) cudaEventDestroy(join_ev_);
  if (stream_) cudaStreamDestroy(stream_);
}

double* Runtime::alloc(int64_t n) {
  void* p = nullptr;
  const size_t bytes = sizeof(double) * static_cast<size_t>(std::max<int64_t>(n, 1));
  C2G_CUDA(cudaMallocAsync(&p, bytes, stream_));
  return static_cast<double*>(p);
}

void Runtime::release(void* p) {
  if (p) C2G_CUDA(cudaFreeAsync(p, stream_));
}

void Runtime::release_quiet(void* p) noexcept {
  if (p && cudaFreeAsync(p, stream_) != cudaSuccess) cudaGetLastError();
}

void Runtime::zero(double* p, int64_t n) {
  if (n > 0) C2G_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * n, stream_));
}

void Runtime::set_slot(int slot, double* p) {
  if (slot < 0 || slot >= kMaxSlots) throw std::out_of_range("slot");
  if (host_slots_[slot] != p) {
    host_slots_[slot] = p;
    slots_dirty_ = true;
  }
}

void Runtime::set_slot32(int slot, float* p) {
  if (slot < 0 || slot >= kMaxSlots) throw std::out_of_range("slot");
  if (host_slots32_[slot] != p) {
    host_slots32_[slot] = p;
    slots_dirty_ = true;
  }
}

float* Runtime::alloc_f32(int64_t n) {
  void* p = nullptr;
  C2G_CUDA(cudaMallocAsync(&p, sizeof(float) * static_cast<size_t>(std::max<int64_t>(n, 1)), stream_));
  return static_cast<float*>(p);
}

void Runtime::flush_slots() {
  if (!slots_dirty_) return;
  C2G_CUDA(cudaMemcpyAsync(dev_slots_, host_slots_.data(), sizeof(double*) * kMaxSlots, cudaMemcpyHostToDevice,
                           stream_));
  C2G_CUDA(cudaMemcpyAsync(dev_slots32_, host_slots32_.data(), sizeof(float*) * kMaxSlots, cudaMemcpyHostToDevice,
                           stream_));
  // The host vector may change before the copy runs: wait for it.
  C2G_CUDA(cudaStreamSynchronize(stream_));
  slots_dirty_ = false;
}

const double* Runtime::ones(int64_t n) {
  if (n > ones_cap_) {
    if (ones_) release(ones_);
    ones_ = nullptr;
    ones_cap_ = 0;
    const int64_t cap = std::max<int64_t>(n, 1024);
    ones_ = alloc(cap);
    ones_cap_ = cap;
    C2G_CUDA(launch_fill(ones_, 1.0, ones_cap_, stream_));
    count_launches(1);
  }
  return ones_;
}

SlotPtrs Runtime::ptrs(double* x, double* y, double* combo) {
  flush_slots();
  SlotPtrs sp;
  sp.table = dev_slots_;
  sp.x = x;
  sp.y = y;
  sp.combo = combo;
  sp.ones = ones_;
  sp.table32 = dev_slots32_;
  sp.x32 = nullptr;
  sp.combo32 = nullptr;
  sp.ones32 = nullptr;
  sp.inter = nullptr;
  sp.inter32 = nullptr;
  return sp;
}

void Runtime::reserve_staging(int64_t bytes, int64_t keep) {
  if (bytes <= staging_cap_) return;
  const int64_t cap = std::max<int64_t>(bytes, staging_cap_ + staging_cap_ / 2);
  char* fresh = nullptr;
  C2G_CUDA(cudaMallocHost(reinterpret_cast<void**>(&fresh), static_cast<size_t>(cap)));
  if (staging_) {
    if (keep > 0) std::memcpy(fresh, staging_, static_cast<size_t>(keep));
    C2G_CUDA(cudaFreeHost(staging_));
  }
  staging_ = fresh;
  staging_cap_ = cap;
}

// Buffers that live only during one stage launch (intermediates of the two-pass path,
// partial tiles of split tiles, their arrival counters) are shared by all programs of
// the runtime: programs run one after another on its stream, so the largest need is
// enough. Growth is stream-ordered; new counters start at zero (a launch leaves its
// counters at zero again).
void* Runtime::transient(int kind, int64_t bytes, bool zero) {
  if (bytes <= transient_cap_[kind]) return transient_[kind];
  if (transient_[kind]) C2G_CUDA(cudaFreeAsync(transient_[kind], stream_));
  const int64_t cap = std::max<int64_t>(bytes, transient_cap_[kind] + transient_cap_[kind] / 2);
  C2G_CUDA(cudaMallocAsync(&transient_[kind], static_cast<size_t>(cap), stream_));
  if (zero) C2G_CUDA(cudaMemsetAsync(transient_[kind], 0, static_cast<size_t>(cap), stream_));
  transient_cap_[kind] = cap;
  return transient_[kind];
}

double* Runtime::transient_doubles(int kind, int64_t n) {
  if (n <= 0) return nullptr;
  return static_cast<double*>(transient(kind, 8 * n, false));
}

unsigned int* Runtime::transient_counters(int kind, int64_t n) {
  if (n <= 0) return nullptr;
  return static_cast<unsigned int*>(transient(kind, static_cast<int64_t>(sizeof(unsigned int)) * n, true));
}

std::unique_ptr<DevProgram> Runtime::upload(const Program& p) { return upload_parts(&p, 1); }

std::unique_ptr<DevProgram> Runtime::upload(const std::vector<Program>& parts) {
  if (parts.empty()) throw std::invalid_argument("upload: no program");
  return upload_parts(parts.data(), parts.size());
}

// Uploads the concatenation of programs compiled from disjoint output shards (the same
// stage lists; see merge_programs) without building the merged program on the host: each
// shard's groups, terms and batch lists go straight to their place in the staging buffer,
// with combination-scratch references and batch-list offsets relocated on the way.
std::unique_ptr<DevProgram> Runtime::upload_parts(const Program* parts, size_t np) {
  auto dp = std::make_unique<DevProgram>();
  dp->rt = this;
  const size_t nsrc = parts[0].stages.size();
  for (size_t i = 0; i < np; i++)
    if (parts[i].stages.size() != nsrc) throw std::logic_error("upload: shards with different stage lists");
  std::vector<int64_t> combo_base(np), entry_base(np);
  int64_t cb = 0, eb = 0;
  for (size_t i = 0; i < np; i++) {
    combo_base[i] = cb;
    entry_base[i] = eb;
    cb = (np == 1) ? parts[i].combo_size : ((cb + parts[i].combo_size + 3) & ~int64_t(3));
    eb += static_cast<int64_t>(parts[i].entries.size());
  }
  if (eb > INT32_MAX) throw std::length_error("upload: batch table too large");
  dp->combo_size = cb;
  // the staging buffer of this upload: the one whose previous copy is oldest
  const int sb = stg_next_;
  stg_next_ ^= 1;
  if (stg_used_[sb]) C2G_CUDA(cudaEventSynchronize(stg_ev_[sb]));
  staging_ = stg_buf_[sb];
  staging_cap_ = stg_cap_[sb];
  struct KeepStaging {  // the buffer (possibly grown) goes back to its ring slot
    Runtime* rt;
    int b;
    ~KeepStaging() {
      rt->stg_buf_[b] = rt->staging_;
      rt->stg_cap_[b] = rt->staging_cap_;
    }
  } keep_staging{this, sb};
  auto reloc = [&](Ref r, size_t i) -> Ref {
    if (r != 0 && ref_slot(r) == kSlotCombo) return make_ref(kSlotCombo, ref_off(r) + combo_base[i]);
    return r;
  };
  // The merged stages: groups relocated, each with its shard; empty stages dropped.
  struct MergedStage {
    std::string name;
    size_t src = 0;
    std::vector<Group> groups;
    std::vector<int32_t> part;     // shard of each group
    std::vector<int64_t> tbase;    // first merged term of each shard
    int64_t nterms = 0, flops = 0, items = 0;
  };
  std::vector<MergedStage> stages;
  for (size_t s = 0; s < nsrc; s++) {
    MergedStage m;
    m.name = parts[0].stages[s].name;
    m.src = s;
    m.tbase.resize(np);
    size_t ng = 0;
    for (size_t i = 0; i < np; i++) ng += parts[i].stages[s].groups.size();
    if (ng == 0) continue;
    m.groups.reserve(ng);
    m.part.reserve(ng);
    for (size_t i = 0; i < np; i++) {
      const Stage& ps = parts[i].stages[s];
      m.tbase[i] = m.nterms;
      for (const Group& g0 : ps.groups) {
        Group g = g0;
        g.out = reloc(g.out, i);
        g.t0 += static_cast<int32_t>(m.nterms);
        g.t1 += static_cast<int32_t>(m.nterms);
        m.groups.push_back(g);
        m.part.push_back(static_cast<int32_t>(i));
      }
      m.nterms += static_cast<int64_t>(ps.terms.size());
      m.flops += ps.flops;
      m.items += ps.items;
      if (m.nterms > INT32_MAX) throw std::length_error("upload: too many terms in a stage");
    }
    if (s == 0 && parts[0].first_repeat_stage == 1) dp->first_repeat = 1;
    stages.push_back(std::move(m));
  }
  // Tile lists, the groups with the most work first. Groups of at most kWarpTile x
  // kWarpTile, and larger groups with light items, go to the team variant in kWarpTile
  // tiles; larger groups with heavy items take the two-pass path (or, with
  // C2G_LARGE=tile, the one-pass cooperative variant in kTile tiles).
  // (C2G_SANDWICH=item routes the light groups to the item-parallel variant instead.)
  const char* env = std::getenv("C2G_SANDWICH");
  const bool use_item = env && std::string(env) == "item";
  const size_t ns = stages.size();
  std::vector<std::vector<TileDesc>> tiles(ns), tiles_large(ns);
  std::vector<std::vector<WarpTile>> tiles_warp(ns);
  int64_t part_doubles = 0, ncounters = 0;
  // Two-pass path of large groups (C2G_LARGE=tile keeps them on the one-pass cooperative
  // kernel instead).
  const char* lenv = std::getenv("C2G_LARGE");
  const bool one_pass_large = lenv && std::string(lenv) == "tile";
  struct TwoPass {
    std::vector<InterJob> jobs;
    std::vector<GemmTile> jtiles;
    std::vector<int32_t> small;  // jobs of at most kInterSmallElems elements
    std::vector<SumGroup> groups;
    std::vector<SumItem> items;
    std::vector<GemmTile> stiles;
    std::vector<int32_t> chunk_first;  // first group (index into groups) of each chunk
    std::vector<int64_t> jtile_first, small_first;  // per group, and the totals at the end
  };
  std::vector<TwoPass> twopass(ns);
  // Bytes of pass-1 intermediates one chunk may hold (C2G_INTER_BUDGET_KB overrides).
  int64_t inter_budget = int64_t(8) << 30;
  if (const char* e = std::getenv("C2G_INTER_BUDGET_KB")) {
    const long long v = std::atoll(e);
    if (v > 0) inter_budget = static_cast<int64_t>(v) << 10;
  }
  int64_t inter_doubles = 0, gemm_part_doubles = 0, gemm_counters = 0;
  std::vector<std::vector<DevStage::PassChunk>> chunk_ranges(ns);
  // Blob layout: the batch table, then per stage its groups and terms, then the tile lists
  // of every stage. It is assembled in the runtime's pinned staging buffer: the terms of
  // each group are copied there in shape order (flags, k1, k2), so that neighbouring items
  // of the team variant share their loop structure, by all host threads.
  int64_t head = align256(sizeof(BatchEntry) * eb);
  std::vector<int64_t> off_groups(ns), off_terms(ns);
  for (size_t s = 0; s < ns; s++) {
    off_groups[s] = head;
    head += align256(sizeof(Group) * stages[s].groups.size());
    off_terms[s] = head;
    head += align256(sizeof(Term) * stages[s].nterms);
  }
  reserve_staging(head, 0);
  std::vector<Term*> terms(ns);
  for (size_t s = 0; s < ns; s++) {
    const MergedStage& st = stages[s];
    std::memcpy(staging_ + off_groups[s], st.groups.data(), sizeof(Group) * st.groups.size());
    terms[s] = reinterpret_cast<Term*>(staging_ + off_terms[s]);
  }
  {
    // work items: the batch table of each shard, and (stage, first group, last group)
    // chunks of about equal term counts
    struct Chunk {
      size_t s;
      size_t g0, g1;
    };
    std::vector<Chunk> chunks;
    for (size_t i = 0; i < np; i++)
      if (!parts[i].entries.empty()) chunks.push_back(Chunk{SIZE_MAX, i, 0});
    const int nthreads = std::max(1, compile_threads());
    int64_t total_terms = 0;
    for (const MergedStage& st : stages) total_terms += st.nterms;
    const int64_t per = std::max<int64_t>(total_terms / (4 * nthreads), 4096);
    for (size_t s = 0; s < ns; s++) {
      const MergedStage& st = stages[s];
      size_t g0 = 0;
      int64_t acc = 0;
      for (size_t g = 0; g < st.groups.size(); g++) {
        acc += st.groups[g].t1 - st.groups[g].t0;
        if (acc >= per || g + 1 == st.groups.size()) {
          chunks.push_back(Chunk{s, g0, g + 1});
          g0 = g + 1;
          acc = 0;
        }
      }
    }
    std::atomic<size_t> next{0};
    std::atomic<bool> bad{false};
    auto work = [&] {
      for (size_t c = next++; c < chunks.size(); c = next++) {
        if (chunks[c].s == SIZE_MAX) {
          const Program& pp = parts[chunks[c].g0];
          std::memcpy(staging_ + sizeof(BatchEntry) * entry_base[chunks[c].g0], pp.entries.data(),
                      sizeof(BatchEntry) * pp.entries.size());
          continue;
        }
        const MergedStage& st = stages[chunks[c].s];
        Term* out = terms[chunks[c].s];
        for (size_t g = chunks[c].g0; g < chunks[c].g1; g++) {
          const Group& G = st.groups[g];
          const size_t i = static_cast<size_t>(st.part[g]);
          const Term* src = parts[i].stages[st.src].terms.data() + (G.t0 - st.tbase[i]);
          const int32_t lbase = static_cast<int32_t>(entry_base[i]);
          for (int32_t k = 0; k < G.t1 - G.t0; k++) {
            Term t = src[k];
            if (np > 1) {
              if (t.flags & kHasA) t.a = reloc(t.a, i);
              t.b = reloc(t.b, i);
              if (t.flags & kHasC) t.c = reloc(t.c, i);
              if (t.list >= 0) t.list += lbase;
            }
            out[G.t0 + k] = t;
          }
          std::stable_sort(out + G.t0, out + G.t1, [](const Term& x, const Term& y) {
            return std::make_tuple(x.flags, x.k1, x.k2) < std::make_tuple(y.flags, y.k1, y.k2);
          });
          int32_t item0 = 0;
          for (Term* it = out + G.t0; it != out + G.t1; ++it) {
            if (it->count < 1) bad = true;
            it->item0 = item0;
            item0 += it->count;
          }
        }
      }
    };
    std::vector<std::thread> pool;
    const int nt = static_cast<int>(std::min<size_t>(nthreads, chunks.size()));
    for (int i = 1; i < nt; i++) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    if (bad) throw std::invalid_argument("task term without items");
  }
  // Per group of a stage: its tile kind and, for the team variant, the work of a tile of
  // each of its (at most four) tile shapes. Tiles of one shape in one group have the same
  // work and the same splits, so both are computed once per shape. Programs can hold
  // hundreds of thousands of small groups: everything here is linear in groups and terms.
  struct GroupTiles {
    int32_t kind = 0;         // 0 none, 1 cooperative / item variant, 2 team variant
    int32_t large = 0;
    int32_t tm = 0, tn = 0;   // tile counts
    int32_t rows[2] = {0, 0}; // full and last tile rows (shape index bit 1)
    int32_t cols[2] = {0, 0}; // full and last tile columns (shape index bit 0)
    int64_t work[4] = {0, 0, 0, 0};
    int32_t nsplit[4] = {1, 1, 1, 1};
    int32_t bounds[4] = {-1, -1, -1, -1};  // first of nsplit + 1 item boundaries in `splits`
  };
  auto present = [](const GroupTiles& gi, int k) {
    // shapes with a full (not last) tile exist only with more than one tile
    return !((!(k >> 1) && gi.tm < 2) || (!(k & 1) && gi.tn < 2));
  };
  auto shape_of = [](const GroupTiles& gi, int i, int j) {
    return ((i == gi.tm - 1) ? 2 : 0) | ((j == gi.tn - 1) ? 1 : 0);
  };
  const int nthreads = std::max(1, compile_threads());
  auto parallel_groups = [&](size_t n, int64_t nterms, const std::function<void(size_t, size_t)>& f) {
    const int nt = (nterms < 200000) ? 1 : static_cast<int>(std::min<size_t>(nthreads, (n + 63) / 64));
    if (nt <= 1) {
      f(0, n);
      return;
    }
    std::vector<std::thread> pool;
    const size_t per = (n + nt - 1) / nt;
    for (int i = 1; i < nt; i++) pool.emplace_back(f, std::min(n, i * per), std::min(n, (i + 1) * per));
    f(0, std::min(n, per));
    for (auto& t : pool) t.join();
  };
  int64_t tile_bytes = 0;
  for (size_t s = 0; s < ns; s++) {
    const MergedStage& st = stages[s];
    const Term* tt = terms[s];
    const size_t ng = st.groups.size();
    std::vector<GroupTiles> info(ng);
    std::atomic<bool> too_large{false};
    parallel_groups(ng, st.nterms, [&](size_t g0, size_t g1) {
      for (size_t g = g0; g < g1; g++) {
        const Group& G = st.groups[g];
        GroupTiles& gi = info[g];
        if (G.m <= 0 || G.n <= 0) continue;
        if (G.m >= 32768 * kWarpTile || G.n >= 65536 * kWarpTile) {
          too_large = true;
          continue;
        }
        int64_t items = 0;
        for (int t = G.t0; t < G.t1; t++) items += tt[t].count;
        const bool small = G.m <= kWarpTile && G.n <= kWarpTile;
        gi.large = !small && std::min(G.m, kTile) * std::min(G.n, kTile) >= kLargeTileElems &&
                   G.work >= kLargeItemFlops * std::max<int64_t>(items, 1);
        if (gi.large || use_item) {
          gi.kind = 1;
          gi.tm = (G.m + kTile - 1) / kTile;
          gi.tn = (G.n + kTile - 1) / kTile;
          continue;
        }
        gi.kind = 2;
        gi.tm = (G.m + kWarpTile - 1) / kWarpTile;
        gi.tn = (G.n + kWarpTile - 1) / kWarpTile;
        gi.rows[0] = std::min(kWarpTile, G.m);
        gi.rows[1] = G.m - (gi.tm - 1) * kWarpTile;
        gi.cols[0] = std::min(kWarpTile, G.n);
        gi.cols[1] = G.n - (gi.tn - 1) * kWarpTile;
        for (int k = 0; k < 4; k++) {
          if (!present(gi, k)) continue;
          const int r = gi.rows[k >> 1], c = gi.cols[k & 1];
          for (int t = G.t0; t < G.t1; t++) gi.work[k] += tt[t].count * item_cost(tt[t], r, c);
        }
      }
    });
    if (too_large) throw std::invalid_argument("output block too large for the tile index");
    int64_t warp_work = 0;
    for (const GroupTiles& gi : info) {
      if (gi.kind != 2) continue;
      // tiles per shape: (tm - 1) full rows and 1 last row, likewise for columns
      const int64_t nr[2] = {gi.tm - 1, 1}, nc[2] = {gi.tn - 1, 1};
      for (int k = 0; k < 4; k++)
        if (present(gi, k)) warp_work += nr[k >> 1] * nc[k & 1] * gi.work[k];
    }
    // Team-variant tiles: heavy tiles have their items split over several CTAs so that the
    // stage's work is spread over at least kWarpCtaTarget CTA-sized pieces; the split
    // points are at equal shares of the tile's work (computed for split shapes only).
    const int64_t piece = std::max<int64_t>(warp_work / kWarpCtaTarget, 1);
    std::vector<int32_t> splits;
    for (size_t g = 0; g < ng; g++) {
      GroupTiles& gi = info[g];
      if (gi.kind != 2) continue;
      const Group& G = st.groups[g];
      const int total = G.t1 > G.t0 ? tt[G.t1 - 1].item0 + tt[G.t1 - 1].count : 0;
      for (int k = 0; k < 4; k++) {
        if (!present(gi, k)) continue;
        const int r = gi.rows[k >> 1], c = gi.cols[k & 1];
        const int64_t work = gi.work[k];
        const int min_items = 2 * warp_slots(warp_class_id(r, c));
        int nsplit = static_cast<int>(std::min<int64_t>((work + piece - 1) / piece, kWarpMaxSplit));
        nsplit = std::max(1, std::min(nsplit, total / std::max(min_items, 1)));
        gi.nsplit[k] = nsplit;
        if (nsplit == 1) continue;
        gi.bounds[k] = static_cast<int32_t>(splits.size());
        splits.push_back(0);
        int t = G.t0;
        int64_t before = 0;  // work of the items before term t
        for (int q = 0; q < nsplit; q++) {
          int stop = total;
          if (q + 1 < nsplit) {
            const int64_t target = work * (q + 1) / nsplit;
            while (t < G.t1 && before + tt[t].count * item_cost(tt[t], r, c) < target) {
              before += tt[t].count * item_cost(tt[t], r, c);
              t++;
            }
            if (t < G.t1) {
              const int64_t cst = item_cost(tt[t], r, c);
              const int64_t inside = (target - before + cst - 1) / cst;
              stop = tt[t].item0 + static_cast<int>(std::min<int64_t>(inside, tt[t].count));
            }
            stop = std::max(stop, splits.back());
          }
          splits.push_back(stop);
        }
      }
    }
    // Large groups: every (term, entry) item becomes a pass-2 product, after a pass-1
    // intermediate when the item has both outer operands. Tiles lie on a 64 x 64 grid,
    // each cut to its part of the block rounded up to 16; long item lists are split at
    // equal shares of the work.
    TwoPass& tp = twopass[s];
    int64_t inter_off = 0;
    auto ext16 = [](int x) { return std::max(1, std::min(4, (x + 15) / 16)); };  // extent in units of 16
    auto tile_shape = [&](int rows, int cols) { return (ext16(rows) - 1) | ((ext16(cols) - 1) << 2); };
    // Planning is two passes over the large groups, both parallel: count each group's
    // items, jobs, job tiles and intermediate size, then fill the arrays at the groups'
    // prefix offsets (groups in the tile order below).
    struct Cursor {
      int64_t item = 0, job = 0, small = 0, jtile = 0, inter = 0;
    };
    auto plan_group = [&](int g, Cursor& c, bool fill) {
      const Group& G = st.groups[g];
      const BatchEntry* ents = reinterpret_cast<const BatchEntry*>(staging_);
      for (int t = G.t0; t < G.t1; t++) {
        const Term& T = tt[t];
        const bool ha = T.flags & kHasA, hc = T.flags & kHasC;
        const GemmOperand B{T.b, T.ldb, (T.flags & kTransB) ? 1 : 0};
        for (int p = 0; p < T.count; p++) {
          if (!fill) {
            if (ha && hc) {
              const int jm = (T.flags & kLeftFirst) ? G.m : T.k1, jn = (T.flags & kLeftFirst) ? T.k2 : G.n;
              c.inter += (static_cast<int64_t>(jm) * jn + 3) & ~int64_t(3);
              if (static_cast<int64_t>(jm) * jn <= kInterSmallElems) c.small++;
              else c.jtile += static_cast<int64_t>((jm + 63) / 64) * ((jn + 63) / 64);
              c.job++;
            }
            c.item++;
            continue;
          }
          double alpha = T.alpha;
          int64_t da = 0, dc = 0;
          if (T.list >= 0) {
            const BatchEntry& e = ents[T.list + p];
            alpha *= e.ratio;
            da = e.da;
            dc = e.dc;
          }
          const GemmOperand A{ha ? T.a + static_cast<uint64_t>(da) : 0, T.lda, (T.flags & kTransA) ? 1 : 0};
          const GemmOperand C{hc ? T.c + static_cast<uint64_t>(dc) : 0, T.ldc, (T.flags & kTransC) ? 1 : 0};
          SumItem it{};
          it.alpha = alpha;
          if (ha && hc) {
            InterJob J{};
            J.off = c.inter;
            const Ref S = make_ref(kSlotInter, c.inter);
            if (T.flags & kLeftFirst) {  // S = op(A_p) op(B), m x k2; out += alpha S op(C_p)
              J.l = A;
              J.r = B;
              J.m = G.m;
              J.n = T.k2;
              J.k = T.k1;
              it.l = GemmOperand{S, G.m, 0};
              it.r = C;
              it.k = T.k2;
            } else {  // S = op(B) op(C_p), k1 x n; out += alpha op(A_p) S
              J.l = B;
              J.r = C;
              J.m = T.k1;
              J.n = G.n;
              J.k = T.k2;
              it.l = A;
              it.r = GemmOperand{S, T.k1, 0};
              it.k = T.k1;
            }
            c.inter += (static_cast<int64_t>(J.m) * J.n + 3) & ~int64_t(3);
            if (static_cast<int64_t>(J.m) * J.n <= kInterSmallElems) {
              tp.small[c.small++] = static_cast<int32_t>(c.job);
            } else {
              for (int i = 0; i < (J.m + 63) / 64; i++)
                for (int j = 0; j < (J.n + 63) / 64; j++) {
                  GemmTile gt{};
                  gt.idx = static_cast<int32_t>(c.job);
                  gt.pos = (i << 16) | j;
                  gt.shape = tile_shape(std::min(64, J.m - 64 * i), std::min(64, J.n - 64 * j));
                  tp.jtiles[c.jtile++] = gt;
                }
            }
            tp.jobs[c.job++] = J;
          } else if (ha) {
            it.l = A;
            it.r = B;
            it.k = T.k1;
          } else if (hc) {
            it.l = B;
            it.r = C;
            it.k = T.k2;
          } else {
            it.r = B;
            it.k = 0;
          }
          tp.items[c.item++] = it;
        }
      }
    };
    auto plan_large_groups = [&](const std::vector<int32_t>& lg) {
      const size_t nl = lg.size();
      if (nl == 0) return;
      int64_t lterms = 0;
      for (int g : lg) lterms += st.groups[g].t1 - st.groups[g].t0;
      std::vector<Cursor> cnt(nl), at(nl);
      parallel_groups(nl, 4 * lterms, [&](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; q++) plan_group(lg[q], cnt[q], false);
      });
      Cursor tot;
      for (size_t q = 0; q < nl; q++) {
        at[q] = tot;
        tot.item += cnt[q].item;
        tot.job += cnt[q].job;
        tot.small += cnt[q].small;
        tot.jtile += cnt[q].jtile;
        tot.inter += cnt[q].inter;
      }
      if (tot.item > INT32_MAX || tot.job > INT32_MAX || tot.jtile > INT32_MAX)
        throw std::length_error("upload: too many large-group items");
      tp.items.resize(static_cast<size_t>(tot.item));
      tp.jobs.resize(static_cast<size_t>(tot.job));
      tp.small.resize(static_cast<size_t>(tot.small));
      tp.jtiles.resize(static_cast<size_t>(tot.jtile));
      tp.groups.resize(nl);
      tp.jtile_first.resize(nl + 1);
      tp.small_first.resize(nl + 1);
      for (size_t q = 0; q < nl; q++) {
        tp.jtile_first[q] = at[q].jtile;
        tp.small_first[q] = at[q].small;
      }
      tp.jtile_first[nl] = tot.jtile;
      tp.small_first[nl] = tot.small;
      // chunks of whole groups whose intermediates fit the budget; a chunk's
      // intermediates start at offset 0 of the buffer
      std::vector<int64_t> inter_base(nl, 0);
      tp.chunk_first.assign(1, 0);
      inter_off = 0;
      {
        int64_t base = 0;
        for (size_t q = 0; q < nl; q++) {
          if (q > 0 && at[q].inter + cnt[q].inter - base > inter_budget / 8) {
            tp.chunk_first.push_back(static_cast<int32_t>(q));
            base = at[q].inter;
          }
          inter_base[q] = base;
          inter_off = std::max(inter_off, at[q].inter + cnt[q].inter - base);
        }
      }
      parallel_groups(nl, 4 * lterms, [&](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; q++) {
          Cursor c = at[q];
          c.inter -= inter_base[q];
          plan_group(lg[q], c, true);
          const Group& G = st.groups[lg[q]];
          SumGroup sg{};
          sg.out = G.out;
          sg.m = G.m;
          sg.n = G.n;
          sg.ldo = G.ldo;
          sg.flags = G.flags;
          sg.i0 = static_cast<int32_t>(at[q].item);
          sg.i1 = static_cast<int32_t>(at[q].item + cnt[q].item);
          tp.groups[q] = sg;
        }
      });
    };
    // Tile order: the groups with the most work first, row-major within a group.
    // Team-variant tiles are then grouped by row class (one kernel per class), keeping
    // that order within a class.
    std::vector<int32_t> order(ng);
    {
      // stable LSD radix sort on the complemented work (descending work, program order
      // among equal work), 8 bits a pass
      std::vector<uint64_t> key(ng);
      uint64_t all = 0;
      for (size_t g = 0; g < ng; g++) {
        key[g] = ~static_cast<uint64_t>(std::max<int64_t>(st.groups[g].work, 0));
        all |= ~key[g];
      }
      std::iota(order.begin(), order.end(), 0);
      std::vector<int32_t> tmp(ng);
      int passes = 0;
      while (passes < 8 && (all >> (8 * passes)) != 0) passes++;
      for (int pass = 0; pass < passes; pass++) {
        const int sh = 8 * pass;
        size_t cnt[257] = {0};
        for (size_t q = 0; q < ng; q++) cnt[((key[order[q]] >> sh) & 255) + 1]++;
        for (int b = 0; b < 256; b++) cnt[b + 1] += cnt[b];
        for (size_t q = 0; q < ng; q++) tmp[cnt[(key[order[q]] >> sh) & 255]++] = order[q];
        order.swap(tmp);
      }
    }
    int64_t per_class[kWarpRowClasses] = {0};
    for (size_t g = 0; g < ng; g++) {
      const GroupTiles& gi = info[g];
      if (gi.kind != 2) continue;
      for (int i = 0; i < gi.tm; i++)
        for (int j = 0; j < gi.tn; j++) {
          const int k = shape_of(gi, i, j);
          per_class[warp_row_class(warp_class_id(gi.rows[k >> 1], gi.cols[k & 1]))] += gi.nsplit[k];
        }
    }
    int64_t class_at[kWarpRowClasses];
    int64_t nwarp_tiles = 0;
    for (int c = 0; c < kWarpRowClasses; c++) {
      class_at[c] = nwarp_tiles;
      nwarp_tiles += per_class[c];
    }
    {
      std::vector<int32_t> lg;
      if (!one_pass_large)
        for (int g : order)
          if (info[g].kind == 1 && info[g].large) lg.push_back(g);
      plan_large_groups(lg);
    }
    tiles_warp[s].resize(static_cast<size_t>(nwarp_tiles));
    WarpTile* wout = tiles_warp[s].data();
    int64_t part_off = 0, counter = 0;
    for (int g : order) {
      const Group& G = st.groups[g];
      const GroupTiles& gi = info[g];
      if (gi.kind == 1 && gi.large && !one_pass_large) {
        continue;  // planned above
      } else if (gi.kind == 1) {
        for (int i = 0; i < gi.tm; i++)
          for (int j = 0; j < gi.tn; j++) {
            const int rows = std::min(kTile, G.m - i * kTile), cols = std::min(kTile, G.n - j * kTile);
            (gi.large ? tiles_large : tiles)[s].push_back(TileDesc{g, (i << 16) | j, sandwich_grid(rows, cols), 0});
          }
      } else if (gi.kind == 2) {
        const int total = G.t1 > G.t0 ? tt[G.t1 - 1].item0 + tt[G.t1 - 1].count : 0;
        for (int i = 0; i < gi.tm; i++)
          for (int j = 0; j < gi.tn; j++) {
            const int k = shape_of(gi, i, j);
            const int rows = gi.rows[k >> 1], cols = gi.cols[k & 1];
            WarpTile wt{};
            wt.group = g;
            wt.pos = (i << 16) | j;
            wt.cls = warp_class_id(rows, cols);
            wt.nsplit = gi.nsplit[k];
            if (wt.nsplit > 1) {
              wt.part = part_off;
              wt.counter = static_cast<int32_t>(counter++);
              part_off += static_cast<int64_t>(wt.nsplit) * rows * cols;
            }
            int64_t& at = class_at[warp_row_class(wt.cls)];
            for (int q = 0; q < wt.nsplit; q++) {
              wt.split = q;
              wt.item0 = (wt.nsplit == 1) ? 0 : splits[gi.bounds[k] + q];
              wt.item1 = (wt.nsplit == 1) ? total : splits[gi.bounds[k] + q + 1];
              wout[at++] = wt;
            }
          }
      }
    }
    if (!tp.groups.empty()) {
      auto item_cost = [](const SumItem& it, int tm_, int tn_) {
        return 2 * static_cast<int64_t>(tm_) * tn_ * std::max(it.k, 1) + 8192;
      };
      // work of an item on a full tile of the group (edge tiles are smaller)
      auto gm16 = [&](const SumGroup& sg) { return 16 * ext16(std::min(64, sg.m)); };
      auto gn16 = [&](const SumGroup& sg) { return 16 * ext16(std::min(64, sg.n)); };
      int64_t total = 0;
      for (const SumGroup& sg : tp.groups) {
        const int64_t ntile = static_cast<int64_t>((sg.m + 63) / 64) * ((sg.n + 63) / 64);
        for (int i = sg.i0; i < sg.i1; i++) total += ntile * item_cost(tp.items[i], gm16(sg), gn16(sg));
      }
      const int64_t gpiece = std::max<int64_t>(total / kGemmCtaTarget, 1);
      int64_t gpart = 0, gcount = 0;
      std::vector<int32_t> bnd;
      std::vector<int64_t> stile_of(tp.groups.size() + 1, 0);
      for (size_t q = 0; q < tp.groups.size(); q++) {
        stile_of[q] = static_cast<int64_t>(tp.stiles.size());
        const SumGroup& sg = tp.groups[q];
        const int gm = gm16(sg), gn = gn16(sg);
        int64_t work = 0;
        for (int i = sg.i0; i < sg.i1; i++) work += item_cost(tp.items[i], gm, gn);
        int nsplit = static_cast<int>(std::min<int64_t>((work + gpiece - 1) / gpiece, kGemmMaxSplit));
        nsplit = std::max(1, std::min(nsplit, sg.i1 - sg.i0));
        bnd.assign(1, sg.i0);
        int64_t before = 0;
        int i = sg.i0;
        for (int k = 1; k < nsplit; k++) {
          const int64_t target = work * k / nsplit;
          while (i < sg.i1 && before + item_cost(tp.items[i], gm, gn) <= target) before += item_cost(tp.items[i++], gm, gn);
          bnd.push_back(std::max(i, bnd.back()));
        }
        bnd.push_back(sg.i1);
        for (int r = 0; r < (sg.m + 63) / 64; r++)
          for (int c = 0; c < (sg.n + 63) / 64; c++) {
            const int rows = std::min(64, sg.m - 64 * r), cols = std::min(64, sg.n - 64 * c);
            GemmTile gt{};
            gt.idx = static_cast<int32_t>(q);
            gt.pos = (r << 16) | c;
            gt.shape = tile_shape(rows, cols);
            gt.nsplit = nsplit;
            if (nsplit > 1) {
              gt.counter = static_cast<int32_t>(gcount++);
              gt.part = gpart;
              gpart += static_cast<int64_t>(nsplit) * (16 * ext16(rows)) * (16 * ext16(cols));
            }
            for (int k = 0; k < nsplit; k++) {
              gt.split = k;
              gt.item0 = bnd[k];
              gt.item1 = bnd[k + 1];
              tp.stiles.push_back(gt);
            }
          }
      }
      stile_of[tp.groups.size()] = static_cast<int64_t>(tp.stiles.size());
      gemm_part_doubles = std::max(gemm_part_doubles, gpart);
      gemm_counters = std::max(gemm_counters, gcount);
      inter_doubles = std::max(inter_doubles, inter_off);
      // chunk ranges: the job tiles, small jobs and pass-2 tiles of a chunk's groups are
      // contiguous (all filled in group order)
      const size_t nch = tp.chunk_first.size();
      chunk_ranges[s].resize(nch);
      for (size_t c = 0; c < nch; c++) {
        const size_t q0 = tp.chunk_first[c], q1 = (c + 1 < nch) ? tp.chunk_first[c + 1] : tp.groups.size();
        chunk_ranges[s][c] = DevStage::PassChunk{
            static_cast<int>(tp.jtile_first[q0]), static_cast<int>(tp.jtile_first[q1] - tp.jtile_first[q0]),
            static_cast<int>(tp.small_first[q0]), static_cast<int>(tp.small_first[q1] - tp.small_first[q0]),
            static_cast<int>(stile_of[q0]), static_cast<int>(stile_of[q1] - stile_of[q0])};
      }
      if (tp.items.size() > size_t(INT32_MAX) || tp.jobs.size() > size_t(INT32_MAX))
        throw std::length_error("upload: too many large-group items");
    }
    part_doubles = std::max(part_doubles, part_off);
    ncounters = std::max(ncounters, counter);
    tile_bytes += align256(sizeof(int32_t) * tp.small.size());
    tile_bytes += align256(sizeof(InterJob) * tp.jobs.size()) + align256(sizeof(GemmTile) * tp.jtiles.size()) +
                  align256(sizeof(SumGroup) * tp.groups.size()) + align256(sizeof(SumItem) * tp.items.size()) +
                  align256(sizeof(GemmTile) * tp.stiles.size());
    tile_bytes += align256(sizeof(TileDesc) * tiles[s].size()) + align256(sizeof(TileDesc) * tiles_large[s].size()) +
                  align256(sizeof(WarpTile) * tiles_warp[s].size());
  }
  const int64_t bytes = head + tile_bytes;
  reserve_staging(bytes, head);  // keeps the part already assembled
  C2G_CUDA(cudaMallocAsync(&dp->blob, std::max<int64_t>(bytes, 256), copy_));
  char* dbase = static_cast<char*>(dp->blob);
  int64_t off = head;
  auto put = [&](const void* src, size_t n) -> const void* {
    if (n) std::memcpy(staging_ + off, src, n);
    const void* d = dbase + off;
    off += align256(static_cast<int64_t>(n));
    return d;
  };
  dp->entries = reinterpret_cast<const BatchEntry*>(dbase);
  dp->nentries = eb;
  for (size_t s = 0; s < ns; s++) {
    const MergedStage& st = stages[s];
    DevStage ds;
    ds.name = st.name;
    ds.ngroups = static_cast<int>(st.groups.size());
    ds.nterms = static_cast<int>(st.nterms);
    ds.ntiles = static_cast<int>(tiles[s].size());
    ds.flops = st.flops;
    ds.items = st.items;
    ds.groups = reinterpret_cast<const Group*>(dbase + off_groups[s]);
    ds.terms = reinterpret_cast<const Term*>(dbase + off_terms[s]);
    ds.tiles = static_cast<const TileDesc*>(put(tiles[s].data(), sizeof(TileDesc) * tiles[s].size()));
    ds.ntiles_large = static_cast<int>(tiles_large[s].size());
    ds.tiles_large =
        static_cast<const TileDesc*>(put(tiles_large[s].data(), sizeof(TileDesc) * tiles_large[s].size()));
    ds.ntiles_warp = static_cast<int>(tiles_warp[s].size());
    for (const WarpTile& wt : tiles_warp[s]) ds.nwarp[warp_row_class(wt.cls)]++;
    ds.tiles_warp =
        static_cast<const WarpTile*>(put(tiles_warp[s].data(), sizeof(WarpTile) * tiles_warp[s].size()));
    const TwoPass& tp = twopass[s];
    ds.jobs = static_cast<const InterJob*>(put(tp.jobs.data(), sizeof(InterJob) * tp.jobs.size()));
    ds.jtiles = static_cast<const GemmTile*>(put(tp.jtiles.data(), sizeof(GemmTile) * tp.jtiles.size()));
    ds.njtiles = static_cast<int>(tp.jtiles.size());
    ds.jsmall = static_cast<const int32_t*>(put(tp.small.data(), sizeof(int32_t) * tp.small.size()));
    ds.njsmall = static_cast<int>(tp.small.size());
    ds.sgroups = static_cast<const SumGroup*>(put(tp.groups.data(), sizeof(SumGroup) * tp.groups.size()));
    ds.sitems = static_cast<const SumItem*>(put(tp.items.data(), sizeof(SumItem) * tp.items.size()));
    ds.stiles = static_cast<const GemmTile*>(put(tp.stiles.data(), sizeof(GemmTile) * tp.stiles.size()));
    ds.nstiles = static_cast<int>(tp.stiles.size());
    ds.chunks = chunk_ranges[s];
    dp->nterms += ds.nterms;
    if (static_cast<int>(s) < dp->first_repeat) dp->flops_once += ds.flops;
    else dp->flops_repeat += ds.flops;
    dp->stages.push_back(ds);
  }
  dp->bytes = bytes;
  C2G_CUDA(cudaMemcpyAsync(dp->blob, staging_, bytes, cudaMemcpyHostToDevice, copy_));
  C2G_CUDA(cudaEventRecord(stg_ev_[sb], copy_));
  stg_used_[sb] = true;
  C2G_CUDA(cudaStreamWaitEvent(stream_, stg_ev_[sb], 0));  // every use of the program follows the copy
  if (dp->combo_size > 0) dp->combo = alloc(dp->combo_size);
  // transient buffers come from the runtime's shared ones at run time (sizes only here)
  dp->part_size = part_doubles;
  dp->inter_size = inter_doubles;
  dp->gemm_part_size = gemm_part_doubles;
  dp->gemm_counter_count = gemm_counters;
  dp->counter_count = ncounters;
  return dp;
}

void Runtime::prepare(DevProgram& p) {
  if (p.prepared) return;
  SlotPtrs sp = ptrs(nullptr, nullptr, p.combo);
  sp.inter = transient_doubles(kTransientInter, p.inter_size);
  for (int s = 0; s < p.first_repeat; s++) launch_stage(p, p.stages[s], sp, Precision::kFP64);
  p.prepared = true;
  p.combo32_ready = false;
}

void Runtime::run(DevProgram& p, double* x, double* y, Precision prec, int64_t xlen) {
  prepare(p);
  SlotPtrs sp = ptrs(x, y, p.combo);
  if (prec != Precision::kFP64) {
    if (p.combo_size > 0 && !p.combo32_ready) {
      if (!p.combo32) p.combo32 = alloc_f32(p.combo_size);
      C2G_CUDA(launch_to_f32(p.combo32, p.combo, p.combo_size, stream_));
      count_launches(1);
      p.combo32_ready = true;
    }
    sp.combo32 = p.combo32;
    if (x) {
      if (xlen <= 0) throw std::invalid_argument("Runtime::run: an FP32 run needs the length of X");
      if (xlen > x32_cap_) {
        if (x32_) release(x32_);
        x32_ = nullptr;
        x32_cap_ = 0;
        x32_ = alloc_f32(xlen);
        x32_cap_ = xlen;
      }
      C2G_CUDA(launch_to_f32(x32_, x, xlen, stream_));
      count_launches(1);
      sp.x32 = x32_;
    }
  }
  sp.inter = transient_doubles(kTransientInter, p.inter_size);
  sp.inter32 = reinterpret_cast<float*>(sp.inter);
  for (size_t s = p.first_repeat; s < p.stages.size(); s++) launch_stage(p, p.stages[s], sp, prec);
}

// One stage: the two passes of its large groups, then the one-pass variants (all write
// disjoint output blocks).
void Runtime::launch_stage(const DevProgram& p, const DevStage& ds, const SlotPtrs& sp, Precision prec_run) {
  const Precision prec = simt_precision(prec_run);
  double* gemm_partials = transient_doubles(kTransientGemmPartials, p.gemm_part_size);
  unsigned* gemm_counters = transient_counters(kTransientGemmCounters, p.gemm_counter_count);
  double* partials = transient_doubles(kTransientPartials, p.part_size);
  unsigned* counters = transient_counters(kTransientCounters, p.counter_count);
  int npass = 0;
  for (const DevStage::PassChunk& ch : ds.chunks) {
    const GemmTile* jt = ds.jtiles + ch.jtile0;
    if (prec_run == Precision::kTC)
      C2G_CUDA(launch_inter_tc(ds.jobs, jt, ch.njtiles, sp, sched_, err_dev_, stream_));
    else
      C2G_CUDA(launch_inter_gemm(ds.jobs, jt, ch.njtiles, sp, stream_, prec));
    C2G_CUDA(launch_inter_small(ds.jobs, ds.jsmall + ch.small0, ch.nsmall, sp, stream_, prec));
    const GemmTile* st = ds.stiles + ch.stile0;
    if (prec_run == Precision::kTC)
      C2G_CUDA(launch_sum_tc(ds.sgroups, ds.sitems, st, ch.nstiles, gemm_partials, gemm_counters, sp, sched_ + 2,
                             err_dev_, stream_));
    else
      C2G_CUDA(launch_sum_gemm(ds.sgroups, ds.sitems, st, ch.nstiles, gemm_partials, gemm_counters, sp, stream_,
                               prec));
    npass += (ch.njtiles > 0) + (ch.nsmall > 0) + (ch.nstiles > 0);
  }
  C2G_CUDA(launch_sandwich_tiles(ds.groups, ds.terms, p.entries, ds.tiles_large, ds.ntiles_large, sp, stream_, prec));
  int nw = 0;
  const WarpLaunch wl{ds.groups, ds.terms, p.entries, ds.tiles_warp, partials, counters};
  C2G_CUDA(launch_sandwich_warp(wl, ds.nwarp, sp, stream_, prec, &nw));
  C2G_CUDA(launch_sandwich(ds.groups, ds.terms, p.entries, ds.tiles, ds.ntiles, sp, stream_, prec));
  count_launches(npass + (ds.ntiles > 0) + (ds.ntiles_large > 0) + nw);
}

void Runtime::sync() {
  C2G_CUDA(cudaStreamSynchronize(stream_));
  if (aux_) C2G_CUDA(cudaStreamSynchronize(aux_));
  check_device_error();
}

void Runtime::check_device_error() {
  if (err_host_ && *err_host_ != 0) {
    const int e = *err_host_;
    *err_host_ = 0;
    throw std::runtime_error("a tensor-core kernel gave up a bounded wait (device error word " + std::to_string(e) +
                             "); its output tiles were not written");
  }
}

cudaStream_t Runtime::aux_stream() {
  if (!aux_) {
    C2G_CUDA(cudaStreamCreateWithFlags(&aux_, cudaStreamNonBlocking));
    C2G_CUDA(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
    C2G_CUDA(cudaEventCreateWithFlags(&join_ev_, cudaEventDisableTiming));
  }
  return aux_;
}

void Runtime::fork_aux() {
  cudaStream_t a = aux_stream();
  C2G_CUDA(cudaEventRecord(fork_ev_, stream_));
  C2G_CUDA(cudaStreamWaitEvent(a, fork_ev_, 0));
}

void Runtime::wait_for(cudaStream_t other) {
  if (!ext_in_) C2G_CUDA(cudaEventCreateWithFlags(&ext_in_, cudaEventDisableTiming));
  C2G_CUDA(cudaEventRecord(ext_in_, other));
  C2G_CUDA(cudaStreamWaitEvent(stream_, ext_in_, 0));
}

void Runtime::signal_to(cudaStream_t other) {
  if (!ext_out_) C2G_CUDA(cudaEventCreateWithFlags(&ext_out_, cudaEventDisableTiming));
  C2G_CUDA(cudaEventRecord(ext_out_, stream_));
  C2G_CUDA(cudaStreamWaitEvent(other, ext_out_, 0));
}

void Runtime::join_aux() {
  if (!aux_) return;
  C2G_CUDA(cudaEventRecord(join_ev_, aux_));
  C2G_CUDA(cudaStreamWaitEvent(stream_, join_ev_, 0));
}

}  // namespace c2g
