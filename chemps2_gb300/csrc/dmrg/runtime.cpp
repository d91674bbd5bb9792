#include "runtime.hpp"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <sstream>
#include <thread>
#include <tuple>

namespace c2g {

namespace {
std::atomic<int64_t> g_launches{0};
inline int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// A team-variant tile before its items are split.
struct PendingTile {
  int group, pos, rows, cols;
  int64_t work;
};

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
    if (blob) rt->release(blob);
    if (combo) rt->release(combo);
    if (combo32) rt->release(combo32);
    if (partials) rt->release(partials);
    if (counters) rt->release(counters);
  }
}

Runtime::Runtime(int L, int device) : L_(L) {
  if (num_slots(L) > kMaxSlots) throw std::invalid_argument("chain too long for the device slot table");
  int count = 0;
  C2G_CUDA(cudaGetDeviceCount(&count));
  if (count <= 0) throw std::runtime_error("no CUDA device available: the DMRG hot path runs only on the GPU");
  if (device < 0) C2G_CUDA(cudaGetDevice(&device));
  C2G_CUDA(cudaSetDevice(device));
  C2G_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
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
  C2G_CUDA(cudaMallocHost(reinterpret_cast<void**>(&pinned_), sizeof(double) * 8));
}

Runtime::~Runtime() {
  if (stream_) cudaStreamSynchronize(stream_);
  if (ones_) cudaFreeAsync(ones_, stream_);
  if (x32_) cudaFreeAsync(x32_, stream_);
  if (stream_) cudaStreamSynchronize(stream_);
  cudaFree(dev_slots_);
  cudaFree(dev_slots32_);
  cudaFree(partial_);
  if (staging_) cudaFreeHost(staging_);
  if (pinned_) cudaFreeHost(pinned_);
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
    ones_cap_ = std::max<int64_t>(n, 1024);
    ones_ = alloc(ones_cap_);
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

std::unique_ptr<DevProgram> Runtime::upload(const Program& p) {
  auto dp = std::make_unique<DevProgram>();
  dp->rt = this;
  dp->first_repeat = p.first_repeat_stage;
  dp->combo_size = p.combo_size;
  // Tile lists, the groups with the most work first. Groups of at most kWarpTile x
  // kWarpTile, and larger groups with light items, go to the team variant in kWarpTile
  // tiles; larger groups with heavy items go to the cooperative variant in kTile tiles.
  // (C2G_SANDWICH=item routes the light groups to the item-parallel variant instead.)
  const char* env = std::getenv("C2G_SANDWICH");
  const bool use_item = env && std::string(env) == "item";
  const size_t ns = p.stages.size();
  std::vector<std::vector<TileDesc>> tiles(ns), tiles_large(ns);
  std::vector<std::vector<WarpTile>> tiles_warp(ns);
  int64_t part_doubles = 0, ncounters = 0;
  // Blob layout: the batch table, then per stage its groups and terms, then the tile lists
  // of every stage. It is assembled in the runtime's pinned staging buffer: the terms of
  // each group are copied there in shape order (flags, k1, k2), so that neighbouring items
  // of the team variant share their loop structure, by all host threads.
  int64_t head = align256(sizeof(BatchEntry) * p.entries.size());
  std::vector<int64_t> off_groups(ns), off_terms(ns);
  for (size_t s = 0; s < ns; s++) {
    off_groups[s] = head;
    head += align256(sizeof(Group) * p.stages[s].groups.size());
    off_terms[s] = head;
    head += align256(sizeof(Term) * p.stages[s].terms.size());
  }
  reserve_staging(head, 0);
  if (!p.entries.empty()) std::memcpy(staging_, p.entries.data(), sizeof(BatchEntry) * p.entries.size());
  std::vector<Term*> terms(ns);
  for (size_t s = 0; s < ns; s++) {
    const Stage& st = p.stages[s];
    if (!st.groups.empty()) std::memcpy(staging_ + off_groups[s], st.groups.data(), sizeof(Group) * st.groups.size());
    terms[s] = reinterpret_cast<Term*>(staging_ + off_terms[s]);
  }
  {
    // (stage, first group, last group) chunks of about equal term counts
    struct Chunk {
      size_t s;
      size_t g0, g1;
    };
    std::vector<Chunk> chunks;
    const int nthreads = std::max(1, compile_threads());
    int64_t total_terms = 0;
    for (const Stage& st : p.stages) total_terms += static_cast<int64_t>(st.terms.size());
    const int64_t per = std::max<int64_t>(total_terms / (4 * nthreads), 4096);
    for (size_t s = 0; s < ns; s++) {
      const Stage& st = p.stages[s];
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
        const Stage& st = p.stages[chunks[c].s];
        Term* out = terms[chunks[c].s];
        for (size_t g = chunks[c].g0; g < chunks[c].g1; g++) {
          const Group& G = st.groups[g];
          std::memcpy(out + G.t0, st.terms.data() + G.t0, sizeof(Term) * (G.t1 - G.t0));
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
  int64_t tile_bytes = 0;
  for (size_t s = 0; s < ns; s++) {
    const Stage& st = p.stages[s];
    std::vector<PendingTile> pending;
    int64_t warp_work = 0;
    std::vector<int> order(st.groups.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return st.groups[a].work > st.groups[b].work; });
    for (int g : order) {
      const Group& G = st.groups[g];
      if (G.m <= 0 || G.n <= 0) continue;
      if (G.m >= 32768 * kWarpTile || G.n >= 65536 * kWarpTile)
        throw std::invalid_argument("output block too large for the tile index");
      int64_t items = 0;
      for (int t = G.t0; t < G.t1; t++) items += st.terms[t].count;
      const bool small = G.m <= kWarpTile && G.n <= kWarpTile;
      const bool large = !small && std::min(G.m, kTile) * std::min(G.n, kTile) >= kLargeTileElems &&
                         G.work >= kLargeItemFlops * std::max<int64_t>(items, 1);
      if (large || use_item) {
        const int tm = (G.m + kTile - 1) / kTile, tn = (G.n + kTile - 1) / kTile;
        for (int i = 0; i < tm; i++)
          for (int j = 0; j < tn; j++) {
            const int rows = std::min(kTile, G.m - i * kTile), cols = std::min(kTile, G.n - j * kTile);
            (large ? tiles_large : tiles)[s].push_back(TileDesc{g, (i << 16) | j, sandwich_grid(rows, cols), 0});
          }
      } else {
        const int tm = (G.m + kWarpTile - 1) / kWarpTile, tn = (G.n + kWarpTile - 1) / kWarpTile;
        for (int i = 0; i < tm; i++)
          for (int j = 0; j < tn; j++) {
            const int rows = std::min(kWarpTile, G.m - i * kWarpTile), cols = std::min(kWarpTile, G.n - j * kWarpTile);
            pending.push_back(PendingTile{g, (i << 16) | j, rows, cols, 0});
            for (int t = G.t0; t < G.t1; t++)
              pending.back().work += terms[s][t].count * item_cost(terms[s][t], rows, cols);
            warp_work += pending.back().work;
          }
      }
    }
    // Team-variant tiles: heavy tiles have their items split over several CTAs so that the
    // stage's work is spread over at least kWarpCtaTarget CTA-sized pieces.
    const int64_t piece = std::max<int64_t>(warp_work / kWarpCtaTarget, 1);
    int64_t part_off = 0, counter = 0;
    for (const PendingTile& pt : pending) {
      const Group& G = st.groups[pt.group];
      const int cls = warp_class_id(pt.rows, pt.cols);
      const int total = G.t1 > G.t0 ? terms[s][G.t1 - 1].item0 + terms[s][G.t1 - 1].count : 0;
      const int min_items = 2 * warp_slots(cls);
      int nsplit = static_cast<int>(std::min<int64_t>((pt.work + piece - 1) / piece, kWarpMaxSplit));
      nsplit = std::max(1, std::min(nsplit, total / std::max(min_items, 1)));
      WarpTile wt{};
      wt.group = pt.group;
      wt.pos = pt.pos;
      wt.cls = cls;
      wt.nsplit = nsplit;
      if (nsplit > 1) {
        wt.part = part_off;
        wt.counter = static_cast<int32_t>(counter++);
        part_off += static_cast<int64_t>(nsplit) * pt.rows * pt.cols;
      }
      // item boundaries at equal shares of the tile's work
      int t = G.t0;
      int64_t before = 0;  // work of the items before term t
      int start = 0;
      for (int k = 0; k < nsplit; k++) {
        int stop = total;
        if (k + 1 < nsplit) {
          const int64_t target = pt.work * (k + 1) / nsplit;
          while (t < G.t1 && before + terms[s][t].count * item_cost(terms[s][t], pt.rows, pt.cols) < target) {
            before += terms[s][t].count * item_cost(terms[s][t], pt.rows, pt.cols);
            t++;
          }
          stop = total;
          if (t < G.t1) {
            const int64_t c = item_cost(terms[s][t], pt.rows, pt.cols);
            const int64_t inside = (target - before + c - 1) / c;
            stop = terms[s][t].item0 + static_cast<int>(std::min<int64_t>(inside, terms[s][t].count));
          }
          stop = std::max(stop, start);
        }
        wt.split = k;
        wt.item0 = start;
        wt.item1 = stop;
        tiles_warp[s].push_back(wt);
        start = stop;
      }
    }
    part_doubles = std::max(part_doubles, part_off);
    ncounters = std::max(ncounters, counter);
    // team-variant tiles ordered by row class (one kernel per class), work order kept
    std::stable_sort(tiles_warp[s].begin(), tiles_warp[s].end(), [](const WarpTile& a, const WarpTile& b) {
      return warp_row_class(a.cls) < warp_row_class(b.cls);
    });
    tile_bytes += align256(sizeof(TileDesc) * tiles[s].size()) + align256(sizeof(TileDesc) * tiles_large[s].size()) +
                  align256(sizeof(WarpTile) * tiles_warp[s].size());
  }
  const int64_t bytes = head + tile_bytes;
  reserve_staging(bytes, head);  // keeps the part already assembled
  C2G_CUDA(cudaMallocAsync(&dp->blob, std::max<int64_t>(bytes, 256), stream_));
  char* dbase = static_cast<char*>(dp->blob);
  int64_t off = head;
  auto put = [&](const void* src, size_t n) -> const void* {
    if (n) std::memcpy(staging_ + off, src, n);
    const void* d = dbase + off;
    off += align256(static_cast<int64_t>(n));
    return d;
  };
  dp->entries = reinterpret_cast<const BatchEntry*>(dbase);
  dp->nentries = static_cast<int64_t>(p.entries.size());
  for (size_t s = 0; s < ns; s++) {
    const Stage& st = p.stages[s];
    DevStage ds;
    ds.name = st.name;
    ds.ngroups = static_cast<int>(st.groups.size());
    ds.nterms = static_cast<int>(st.terms.size());
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
    dp->nterms += ds.nterms;
    if (static_cast<int>(s) < dp->first_repeat) dp->flops_once += ds.flops;
    else dp->flops_repeat += ds.flops;
    dp->stages.push_back(ds);
  }
  dp->bytes = bytes;
  C2G_CUDA(cudaMemcpyAsync(dp->blob, staging_, bytes, cudaMemcpyHostToDevice, stream_));
  C2G_CUDA(cudaStreamSynchronize(stream_));  // the staging buffer is reused by the next upload
  if (dp->combo_size > 0) dp->combo = alloc(dp->combo_size);
  if (part_doubles > 0) dp->partials = alloc(part_doubles);
  if (ncounters > 0) {
    C2G_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dp->counters), sizeof(unsigned) * ncounters, stream_));
    C2G_CUDA(cudaMemsetAsync(dp->counters, 0, sizeof(unsigned) * ncounters, stream_));
  }
  return dp;
}

void Runtime::prepare(DevProgram& p) {
  if (p.prepared) return;
  const SlotPtrs sp = ptrs(nullptr, nullptr, p.combo);
  for (int s = 0; s < p.first_repeat; s++) {
    const DevStage& ds = p.stages[s];
    C2G_CUDA(launch_sandwich_tiles(ds.groups, ds.terms, p.entries, ds.tiles_large, ds.ntiles_large, sp, stream_));
    int nw = 0;
    const WarpLaunch wl{ds.groups, ds.terms, p.entries, ds.tiles_warp, p.partials, p.counters};
    C2G_CUDA(launch_sandwich_warp(wl, ds.nwarp, sp, stream_, Precision::kFP64, &nw));
    C2G_CUDA(launch_sandwich(ds.groups, ds.terms, p.entries, ds.tiles, ds.ntiles, sp, stream_));
    count_launches((ds.ntiles > 0) + (ds.ntiles_large > 0) + nw);
  }
  p.prepared = true;
  p.combo32_ready = false;
}

void Runtime::run(DevProgram& p, double* x, double* y, Precision prec, int64_t xlen) {
  prepare(p);
  SlotPtrs sp = ptrs(x, y, p.combo);
  if (prec == Precision::kFP32) {
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
        x32_cap_ = xlen;
        x32_ = alloc_f32(x32_cap_);
      }
      C2G_CUDA(launch_to_f32(x32_, x, xlen, stream_));
      count_launches(1);
      sp.x32 = x32_;
    }
  }
  for (size_t s = p.first_repeat; s < p.stages.size(); s++) {
    const DevStage& ds = p.stages[s];
    C2G_CUDA(
        launch_sandwich_tiles(ds.groups, ds.terms, p.entries, ds.tiles_large, ds.ntiles_large, sp, stream_, prec));
    int nw = 0;
    const WarpLaunch wl{ds.groups, ds.terms, p.entries, ds.tiles_warp, p.partials, p.counters};
    C2G_CUDA(launch_sandwich_warp(wl, ds.nwarp, sp, stream_, prec, &nw));
    C2G_CUDA(launch_sandwich(ds.groups, ds.terms, p.entries, ds.tiles, ds.ntiles, sp, stream_, prec));
    count_launches((ds.ntiles > 0) + (ds.ntiles_large > 0) + nw);
  }
}

void Runtime::sync() { C2G_CUDA(cudaStreamSynchronize(stream_)); }

}  // namespace c2g
