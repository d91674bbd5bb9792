// CheMPS2::DMRG on the GPU: sweep control on the host (CheMPS2/DMRG.cpp:268-452), every
// numerical step as device task programs or device kernels.
#include "chemps2/DMRG.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cusolverDn.h>
#include <string>
#include <unistd.h>
#include <unordered_map>

#include "static_scratch.hpp"

#include "davidson.hpp"
#include "correlations.hpp"
#include "excite.hpp"
#include "fcicoef.hpp"
#include "gauge.hpp"
#include "twodm.hpp"
#include "compile.hpp"
#include "heff.hpp"
#include "layout.hpp"
#include "operators.hpp"
#include "rng.hpp"
#include "runtime.hpp"
#include "sobject.hpp"
#include "symm.hpp"

namespace CheMPS2 {

using c2g::Blk;
using c2g::BoundaryOps;
using c2g::DevProgram;
using c2g::MpsLayout;
using c2g::MpsT;
using c2g::Program;
using c2g::TaskBuilder;
using c2g::TwoSiteLayout;

namespace {

// Davidson parameters of CheMPS2/include/chemps2/Options.h:70-72.
constexpr int kDavidsonNumVec = 32;
constexpr int kDavidsonNumVecKeep = 3;
constexpr double kDavidsonPrecondCutoff = 1e-12;

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

MpsT mps_tensor(const MpsLayout* lay, int site) {
  MpsT t;
  t.lay = lay;
  t.base = c2g::make_ref(c2g::kSlotMpsBase + site, 0);
  return t;
}

void check_solver(cusolverStatus_t s, const char* what) {
  if (s != CUSOLVER_STATUS_SUCCESS)
    throw std::runtime_error(std::string("cuSOLVER error ") + std::to_string(static_cast<int>(s)) + " in " + what);
}

}  // namespace

struct DMRG::ProgramCache {
  struct Entry {
    std::unique_ptr<DevProgram> dp;
    long long operand_bytes = 0;
    long long bytes = 0;  // device bytes counted against the limit
    unsigned long long last_use = 0;
  };
  std::unordered_map<std::string, Entry> map;
  long long bytes = 0;
  long long limit = 0;
  unsigned long long clock = 0;
  long long hits = 0, misses = 0;
};

std::string DMRG::dims_key(const char* kind, const int index, const int bmin, const int bmax, const int extra) const {
  std::string key(kind);
  key.push_back('|');
  const int hdr[2] = {index, extra};
  key.append(reinterpret_cast<const char*>(hdr), sizeof(hdr));
  for (int b = std::max(bmin, 0); b <= std::min(bmax, L); b++) {
    const int ns = denBK->num_sectors(b);
    key.push_back('/');
    for (int id = 0; id < ns; id++) {
      const int d = denBK->cur_dim_by_id(b, id);
      key.append(reinterpret_cast<const char*>(&d), sizeof(d));
    }
  }
  return key;
}

DevProgram& DMRG::program(const std::string& key, const std::function<c2g::Compiled()>& build,
                          long long* operand_bytes) {
  ProgramCache& pc = *pcache_;
  pc.clock++;
  auto it = pc.map.find(key);
  if (it != pc.map.end()) {
    pc.hits++;
    it->second.last_use = pc.clock;
    it->second.dp->prepared = false;  // its combination stage reads operator data: rerun
    if (operand_bytes) *operand_bytes = it->second.operand_bytes;
    return *it->second.dp;
  }
  pc.misses++;
  const double tc = now();
  c2g::Compiled c = build();
  stats_.t_compile += now() - tc;
  ProgramCache::Entry e;
  const double tu = now();
  e.dp = c.parts.empty() ? rt->upload(c.program) : rt->upload(c.parts);
  stats_.t_upload += now() - tu;
  e.operand_bytes = c.operand_bytes;
  e.last_use = pc.clock;
  // records and the FP64 combination buffer, plus its FP32 copy when matvecs run in FP32
  const long long size = e.dp->bytes + (precision_ != 0 ? 12 : 8) * e.dp->combo_size;
  e.bytes = size;
  // Least recently used programs leave first; the programs of the current step (the last
  // few requests) stay, since callers hold references to them.
  while (pc.bytes + size > pc.limit && !pc.map.empty()) {
    auto victim = pc.map.end();
    for (auto jt = pc.map.begin(); jt != pc.map.end(); ++jt)
      if (jt->second.last_use + 8 < pc.clock && (victim == pc.map.end() || jt->second.last_use < victim->second.last_use))
        victim = jt;
    if (victim == pc.map.end()) break;
    pc.bytes -= victim->second.bytes;
    pc.map.erase(victim);
  }
  pc.bytes += size;
  if (operand_bytes) *operand_bytes = e.operand_bytes;
  auto ins = pc.map.emplace(key, std::move(e));
  return *ins.first->second.dp;
}

struct DMRG::HeffCache {
  int index = -1;
  unsigned long long version = 0;
  std::unique_ptr<TwoSiteLayout> S;
  std::unique_ptr<DevProgram> program, diag;
  int64_t operand_bytes = 0;
  double* xbuf = nullptr;
  double* ybuf = nullptr;
  int64_t xbuf_len = 0;
};

// A stored (lower) state of the excited-state machinery: its bookkeeper and MPS, and its
// overlap tensors with the current MPS at every boundary.
struct DMRG::ExcState {
  std::unique_ptr<SyBookkeeper> bk;
  std::vector<std::unique_ptr<MpsLayout>> lay;
  std::vector<double*> mps;
  double eshift = 0.0;
  std::vector<std::unique_ptr<c2g::OverlapLayout>> olay;  // [reference index b]: boundary b + 1
  std::vector<double*> odev;
  std::vector<int> odir;  // 1 moving right, 2 moving left, 0 none
};

DMRG::DMRG(Problem* ProbIn, ConvergenceScheme* OptSchemeIn, const bool makechkpt, const std::string, int* occupancies)
    : Prob(ProbIn), OptScheme(OptSchemeIn), makecheckpoints_(makechkpt) {
  rng_ = std::make_unique<c2g::HostRand>();
  construct(occupancies);
}

DMRG::DMRG(Problem* ProbIn, ConvergenceScheme* OptSchemeIn, const DMRGOptions& options)
    : Prob(ProbIn), OptScheme(OptSchemeIn), makecheckpoints_(options.makechkpt) {
  rng_ = options.private_seed ? std::make_unique<c2g::HostRand>(options.seed) : std::make_unique<c2g::HostRand>();
  construct(options.occupancies);
}

void DMRG::construct(int* occupancies) {
  heff_cache_ = std::make_unique<HeffCache>();
  pcache_ = std::make_unique<ProgramCache>();
  pcache_->limit = 16LL << 30;
  if (const char* e = std::getenv("C2G_PROGRAM_CACHE_GB")) pcache_->limit = static_cast<long long>(std::atof(e) * (1LL << 30));
  if (!Prob->checkConsistency()) throw std::invalid_argument("DMRG: inconsistent Problem");
  if (OptScheme->get_number() < 1) throw std::invalid_argument("DMRG: empty ConvergenceScheme");
  L = Prob->gL();
  if (L < 2) throw std::invalid_argument("DMRG: at least two orbitals are required");
  Prob->construct_mxelem();
  rt = std::make_unique<c2g::Runtime>(L);
  mps_lay.resize(L);
  mps_dev.assign(L, nullptr);
  ops.resize(L - 1);
  ops_dev.assign(L - 1, nullptr);
  ops_dev32.assign(L - 1, nullptr);
  isAllocated.assign(L - 1, 0);
  setup_mps(occupancies);
  PreSolve();
}

DMRG::~DMRG() {
  if (rt) {
    try {
      rt->sync();
    } catch (...) {
    }
    if (solver_) cusolverDnDestroy(static_cast<cusolverDnHandle_t>(solver_));
    pcache_.reset();
    if (heff_cache_) {
      heff_cache_->program.reset();
      heff_cache_->diag.reset();
      rt->release_quiet(heff_cache_->xbuf);
      rt->release_quiet(heff_cache_->ybuf);
    }
    for (double* p : mps_dev) rt->release_quiet(p);
    for (auto& st : exc_) {
      for (double* p : st->odev) rt->release_quiet(p);
      for (double* p : st->mps) rt->release_quiet(p);
    }
    for (double* p : ops_dev) rt->release_quiet(p);
    for (float* p : ops_dev32) rt->release_quiet(p);
    try {
      rt->sync();
    } catch (...) {
    }
  }
}

// CheMPS2/DMRG.cpp:100-256 (setupBookkeeperAndMPS) with CheMPS2/TensorT.cpp:167-173.
namespace {
constexpr char kMpsMagic[8] = {'C', '2', 'G', 'M', 'P', 'S', '0', '1'};
}  // namespace

// CheMPS2/DMRGmpsio.cpp:27-94 (saveMPS): header, virtual dimensions of every boundary in
// bookkeeper order, converged flag, then the tensors of every site. The file is written
// under a temporary name, flushed to disk and then renamed over the previous checkpoint,
// so a process killed mid-write leaves the last complete checkpoint in place.
void DMRG::save_mps(bool converged) const {
  const std::string tmp_name = mps_storage_name_ + ".tmp";
  std::FILE* f = std::fopen(tmp_name.c_str(), "wb");
  if (!f) throw std::runtime_error("saveMPS: cannot open " + tmp_name);
  auto put = [&](const void* p, size_t n) {
    if (std::fwrite(p, 1, n, f) != n) {
      std::fclose(f);
      std::remove(tmp_name.c_str());
      throw std::runtime_error("saveMPS: write failed for " + tmp_name);
    }
  };
  const int32_t head[7] = {L, Prob->gN(), Prob->gTwoS(), Prob->gIrrep(), denBK->getNumberOfIrreps(),
                           converged ? 1 : 0, 0};
  put(kMpsMagic, 8);
  put(head, sizeof(head));
  const SyBookkeeper& bk = *denBK;
  for (int b = 0; b <= L; b++)
    for (int n = bk.gNmin(b); n <= bk.gNmax(b); n++)
      for (int s2 = bk.gTwoSmin(b, n); s2 <= bk.gTwoSmax(b, n); s2 += 2)
        for (int i = 0; i < bk.getNumberOfIrreps(); i++) {
          const int32_t d = bk.gCurrentDim(b, n, s2, i);
          put(&d, sizeof(d));
        }
  for (int site = 0; site < L; site++) {
    std::vector<double> data(static_cast<size_t>(mps_lay[site]->size()));
    if (!data.empty())
      C2G_CUDA(cudaMemcpyAsync(data.data(), mps_dev[site], sizeof(double) * data.size(), cudaMemcpyDeviceToHost,
                               rt->stream()));
    rt->sync();
    const int64_t n = static_cast<int64_t>(data.size());
    put(&n, sizeof(n));
    put(data.data(), sizeof(double) * data.size());
  }
  const bool flushed = std::fflush(f) == 0 && fsync(fileno(f)) == 0;
  if (std::fclose(f) != 0 || !flushed) {
    std::remove(tmp_name.c_str());
    throw std::runtime_error("saveMPS: could not flush " + tmp_name);
  }
  if (std::rename(tmp_name.c_str(), mps_storage_name_.c_str()) != 0) {
    std::remove(tmp_name.c_str());
    throw std::runtime_error("saveMPS: could not rename " + tmp_name + " to " + mps_storage_name_);
  }
}

// CheMPS2/DMRGmpsio.cpp:96-162 (loadDIM, loadMPS). False when the file does not exist.
bool DMRG::load_mps() {
  std::FILE* f = std::fopen(mps_storage_name_.c_str(), "rb");
  if (!f) return false;
  auto get = [&](void* p, size_t n) {
    if (std::fread(p, 1, n, f) != n) {
      std::fclose(f);
      throw std::runtime_error("loadMPS: " + mps_storage_name_ + " is truncated");
    }
  };
  char magic[8];
  get(magic, 8);
  int32_t head[7];
  get(head, sizeof(head));
  if (std::memcmp(magic, kMpsMagic, 8) != 0 || head[0] != L || head[1] != Prob->gN() || head[2] != Prob->gTwoS() ||
      head[3] != Prob->gIrrep() || head[4] != denBK->getNumberOfIrreps()) {
    std::fclose(f);
    throw std::runtime_error("loadMPS: " + mps_storage_name_ + " belongs to another problem");
  }
  SyBookkeeper& bk = *denBK;
  for (int b = 0; b <= L; b++)
    for (int n = bk.gNmin(b); n <= bk.gNmax(b); n++)
      for (int s2 = bk.gTwoSmin(b, n); s2 <= bk.gTwoSmax(b, n); s2 += 2)
        for (int i = 0; i < bk.getNumberOfIrreps(); i++) {
          int32_t d = 0;
          get(&d, sizeof(d));
          if (b > 0 && b < L) bk.SetDim(b, n, s2, i, d);
        }
  for (int site = 0; site < L; site++) {
    mps_lay[site] = std::make_unique<MpsLayout>();
    mps_lay[site]->build(bk, site);
    int64_t n = 0;
    get(&n, sizeof(n));
    if (n != mps_lay[site]->size()) {
      std::fclose(f);
      throw std::runtime_error("loadMPS: tensor sizes in " + mps_storage_name_ + " differ from its dimensions");
    }
    std::vector<double> data(static_cast<size_t>(n));
    get(data.data(), sizeof(double) * data.size());
    upload_mps(site, data);
  }
  std::fclose(f);
  return true;
}

// CheMPS2/DMRGmpsio.cpp:164-173
void DMRG::deleteStoredMPS() {
  for (int k = 0; k <= static_cast<int>(exc_.size()); k++) std::remove(("CheMPS2_MPS" + std::to_string(k) + ".c2g").c_str());
}

void DMRG::setup_mps(int* occupancies) {
  denBK = std::make_unique<SyBookkeeper>(Prob, OptScheme->get_D(0));
  if (!denBK->IsPossible()) throw std::invalid_argument("DMRG: the targeted symmetry sector is impossible");
  mps_storage_name_ = "CheMPS2_MPS" + std::to_string(exc_.size()) + ".c2g";
  loaded_mps_ = makecheckpoints_ && load_mps();
  if (loaded_mps_) return;
  std::vector<int> occ;
  if (occupancies) {
    occ.assign(occupancies, occupancies + L);
    if (Prob->gReorder()) {
      std::vector<int> tmp(occ);
      for (int c = 0; c < L; c++) occ[c] = tmp[Prob->gf2(c)];
      for (int c = 0; c < L; c++) occupancies[c] = occ[c];
    }
  }
  int left_n = 0, left_i = 0, left_2s = 0;
  for (int site = 0; site < L; site++) {
    mps_lay[site] = std::make_unique<MpsLayout>();
    mps_lay[site]->build(*denBK, site);
    const MpsLayout& lay = *mps_lay[site];
    std::vector<double> data(lay.size());
    for (auto& v : data) v = 2 * rng_->unit() - 1.0;
    if (occupancies) {
      const int right_n = left_n + occ[site];
      const int right_i = (occ[site] == 1) ? c2g::irrep_prod(left_i, Prob->gIrrep(site)) : left_i;
      const int right_2s = (occ[site] == 1) ? left_2s + 1 : left_2s;
      for (int NL = right_n - 2; NL <= right_n; NL++) {
        const int DS = (right_n == NL + 1) ? 1 : 0;
        const int IL = (right_n == NL + 1) ? c2g::irrep_prod(right_i, Prob->gIrrep(site)) : right_i;
        for (int TwoSL = right_2s - DS; TwoSL <= right_2s + DS; TwoSL += 2) {
          const int k = lay.kappa(NL, TwoSL, IL, right_n, right_2s, right_i);
          if (k < 0) continue;
          const int dimL2 = lay.rows[k];
          double* space = data.data() + lay.k2i[k];
          for (int row = 0; row < dimL2; row++) space[row] = 0.0;
          if (NL == left_n && TwoSL == left_2s && IL == left_i) space[0] = 42;
        }
      }
      left_n = right_n;
      left_i = right_i;
      left_2s = right_2s;
    }
    left_normalize_host(site, data);
    upload_mps(site, data);
  }
}

// CheMPS2/TensorT.cpp:188-289 (QR per right sector, Householder, Q kept) as used by
// DMRG::left_normalize(site, NULL). Initialisation.
void DMRG::left_normalize_host(int site, std::vector<double>& data) {
  c2g::left_normalize(*denBK, site, *mps_lay[site], data);
}

void DMRG::download_mps(int site, std::vector<double>& data) {
  data.resize(static_cast<size_t>(mps_lay[site]->size()));
  if (!data.empty())
    C2G_CUDA(cudaMemcpyAsync(data.data(), mps_dev[site], sizeof(double) * data.size(), cudaMemcpyDeviceToHost,
                             rt->stream()));
  rt->sync();
}

int DMRG::exc_slot(int state, bool overlap, int idx) const {
  return c2g::num_slots(L) + state * 2 * L + (overlap ? L : 0) + idx;
}

// CheMPS2/DMRG.cpp:464-473
void DMRG::activateExcitations(const int maxExcIn) {
  if (maxExcIn < 1) throw std::invalid_argument("activateExcitations: at least one state");
  if (c2g::num_slots(L) + maxExcIn * 2 * L > c2g::kMaxSlots)
    throw std::invalid_argument("activateExcitations: too many states for the device slot table");
  exc_active_ = true;
  max_exc_ = maxExcIn;
}

// CheMPS2/DMRG.cpp:475-505
void DMRG::newExcitation(const double EshiftIn) {
  if (!exc_active_) throw std::logic_error("newExcitation: excitations are not activated");
  if (static_cast<int>(exc_.size()) >= max_exc_) throw std::logic_error("newExcitation: maximum number of states");
  two_dm_.reset();
  corr_.reset();
  delete_all_ops();
  release_overlaps();
  auto st = std::make_unique<ExcState>();
  st->eshift = EshiftIn;
  st->bk = std::move(denBK);
  st->lay = std::move(mps_lay);
  st->mps = std::move(mps_dev);
  st->olay.resize(L - 1);
  st->odev.assign(L - 1, nullptr);
  st->odir.assign(L - 1, 0);
  const int k = static_cast<int>(exc_.size());
  for (int site = 0; site < L; site++) {
    rt->set_slot(exc_slot(k, false, site), st->mps[site]);
    rt->set_slot(c2g::kSlotMpsBase + site, nullptr);
  }
  exc_.push_back(std::move(st));
  mps_lay.clear();
  mps_lay.resize(L);
  mps_dev.assign(L, nullptr);
  setup_mps(nullptr);
  PreSolve();
}

void DMRG::release_overlaps() {
  for (size_t k = 0; k < exc_.size(); k++)
    for (int b = 0; b < L - 1; b++) {
      ExcState& st = *exc_[k];
      if (st.odev[b]) rt->release(st.odev[b]);
      st.odev[b] = nullptr;
      st.odir[b] = 0;
      st.olay[b].reset();
      rt->set_slot(exc_slot(static_cast<int>(k), true, b), nullptr);
    }
}

// The overlap tensors of boundary index + 1 with every stored state, after the operator
// update of that boundary (CheMPS2/DMRGoperators.cpp:556-566, :889-899).
void DMRG::update_overlaps(const int index, const bool moving_right) {
  for (size_t k = 0; k < exc_.size(); k++) {
    ExcState& st = *exc_[k];
    const int site = moving_right ? index : index + 1;
    const int pidx = moving_right ? index - 1 : index + 1;
    const bool edge = moving_right ? (index == 0) : (index == L - 2);
    if (!edge && st.odir[pidx] != (moving_right ? 1 : 2))
      throw std::logic_error("excited states: overlap tensors of the previous boundary missing");
    auto lay = std::make_unique<c2g::OverlapLayout>();
    lay->build(*denBK, *st.bk, index + 1);
    if (st.odev[index]) rt->release(st.odev[index]);
    st.odev[index] = nullptr;
    st.odev[index] = rt->alloc(std::max<int64_t>(lay->size(), 1));
    rt->zero(st.odev[index], lay->size());
    const int slot = exc_slot(static_cast<int>(k), true, index);
    rt->set_slot(slot, st.odev[index]);
    c2g::OverlapT out{lay.get(), c2g::make_ref(slot, 0)};
    c2g::OverlapT prev;
    if (!edge) prev = c2g::OverlapT{st.olay[pidx].get(), c2g::make_ref(exc_slot(static_cast<int>(k), true, pidx), 0)};
    const MpsT tdown{st.lay[site].get(), c2g::make_ref(exc_slot(static_cast<int>(k), false, site), 0)};
    TaskBuilder tb;
    c2g::compile_overlap_update(tb, *denBK, *st.bk, moving_right, index, edge ? nullptr : &prev, out,
                                mps_tensor(mps_lay[site].get(), site), tdown);
    auto dp = rt->upload(tb.finalize());
    rt->run(*dp, nullptr, nullptr);
    rt->sync();
    st.olay[index] = std::move(lay);
    st.odir[index] = moving_right ? 1 : 2;
  }
}

// CheMPS2/DMRGtechnics.cpp:276-298
void DMRG::gauge_left_normalize(int site, bool into_next) {
  std::vector<double> t, n;
  download_mps(site, t);
  if (into_next) {
    download_mps(site + 1, n);
    c2g::left_normalize(*denBK, site, *mps_lay[site], t, mps_lay[site + 1].get(), &n);
    upload_mps(site + 1, n);
  } else {
    c2g::left_normalize(*denBK, site, *mps_lay[site], t);
  }
  upload_mps(site, t);
  version_++;
}

// CheMPS2/DMRGtechnics.cpp:300-322: LQ of MPS[site], L into MPS[site - 1]
void DMRG::gauge_right_normalize(int site) {
  std::vector<double> t, p;
  download_mps(site, t);
  download_mps(site - 1, p);
  c2g::right_normalize(*denBK, site, *mps_lay[site], t, mps_lay[site - 1].get(), &p);
  upload_mps(site, t);
  upload_mps(site - 1, p);
  version_++;
}

// CheMPS2/TwoDM.cpp:445-628 for one site, as device task programs (chunked so that the
// products of one program fit a work budget).
void DMRG::fill_2dm_site(int site) {
  if (site > 0 && isAllocated[site - 1] != 1) throw std::logic_error("2-RDM: left operators missing");
  if (site < L - 1 && isAllocated[site] != 2) throw std::logic_error("2-RDM: right operators missing");
  c2g::TwoDMContext ctx;
  ctx.bk = denBK.get();
  ctx.L = L;
  ctx.site = site;
  ctx.T = mps_tensor(mps_lay[site].get(), site);
  ctx.left = (site > 0) ? ops[site - 1].get() : nullptr;
  ctx.right = (site < L - 1) ? ops[site].get() : nullptr;
  const std::vector<c2g::TwoDMInstance> inst = c2g::twodm_instances(ctx);
  const int nvalues = inst.back().value0 + c2g::twodm_num_values(inst.back().kind);
  std::vector<double> values(nvalues, 0.0);
  // doubles (256 MB) of products per program; C2G_TWODM_BUDGET overrides it (tests force
  // several programs per site with a small budget)
  static const int64_t kWorkBudget = [] {
    const char* e = std::getenv("C2G_TWODM_BUDGET");
    const long long v = e ? std::atoll(e) : 0;
    return v > 0 ? static_cast<int64_t>(v) : int64_t(1) << 25;
  }();
  size_t first = 0;
  while (first < inst.size()) {
    size_t last = first;
    int64_t work = 0;
    while (last < inst.size() && (last == first || work + inst[last].work <= kWorkBudget)) work += inst[last++].work;
    TaskBuilder tb;
    c2g::compile_twodm(tb, ctx, inst, first, last);
    auto dp = rt->upload(tb.finalize());
    const int v0 = inst[first].value0;
    const int nv = inst[last - 1].value0 + c2g::twodm_num_values(inst[last - 1].kind) - v0;
    double* dwork = rt->alloc(std::max<int64_t>(work, 1));
    double* dy = rt->alloc(nv);
    rt->zero(dy, nv);
    rt->set_slot(c2g::kSlotWork, dwork);
    rt->run(*dp, nullptr, dy);
    C2G_CUDA(cudaMemcpyAsync(values.data() + v0, dy, sizeof(double) * nv, cudaMemcpyDeviceToHost, rt->stream()));
    rt->sync();
    rt->set_slot(c2g::kSlotWork, nullptr);
    rt->release(dwork);
    rt->release(dy);
    first = last;
  }
  c2g::twodm_assemble(*two_dm_, site, inst, values);
}

// CheMPS2/DMRGtechnics.cpp:40-120 (the 2-RDM part of calc_rdms_and_correlations)
void DMRG::calc2DMandCorrelations() {
  if (L < 2) throw std::invalid_argument("calc2DMandCorrelations: at least two orbitals");
  // the whole MPS left-canonical, then the left operators of boundary L - 2
  gauge_left_normalize(L - 2, true);
  gauge_left_normalize(L - 1, false);
  update_moving_right(L - 2);
  two_dm_ = std::make_unique<TwoDM>(Prob, L);
  for (int site = L - 1; site >= 0; site--) {
    fill_2dm_site(site);
    if (site > 0) {
      gauge_right_normalize(site);
      update_moving_left(site - 1);
    }
  }
  two_dm_->correct_higher_multiplicities();
  // Correlation pass from the left (CheMPS2/DMRGtechnics.cpp:157-176), which also brings
  // the state back to that of a finished right sweep: MPS[0 .. L-2] left-normalised, the
  // left operators of boundaries 0 .. L-3.
  corr_ = std::make_unique<Correlations>(Prob, two_dm_.get());
  std::unique_ptr<c2g::CorrTensors> cprev;
  double* dprev = nullptr;
  for (int site = 0; site < L - 1; site++) {
    gauge_left_normalize(site, true);
    const int s = site + 1;  // the orthogonality centre
    auto cnext = std::make_unique<c2g::CorrTensors>();
    const int slot = (s % 2 == 0) ? c2g::kSlotCorr0 : c2g::kSlotCorr1;
    c2g::allocate_corr(*cnext, *denBK, s, slot);
    double* dnext = rt->alloc(std::max<int64_t>(cnext->size, 1));
    rt->zero(dnext, cnext->size);
    rt->set_slot(slot, dnext);
    {
      TaskBuilder tb;
      c2g::compile_corr_update(tb, *denBK, *Prob, L, s, cprev.get(), *cnext, mps_tensor(mps_lay[site].get(), site));
      auto dp = rt->upload(tb.finalize());
      rt->run(*dp, nullptr, nullptr);
    }
    {
      TaskBuilder tb;
      const int64_t work = c2g::compile_corr_fill(tb, *denBK, s, mps_tensor(mps_lay[s].get(), s), *cnext);
      auto dp = rt->upload(tb.finalize());
      const int nv = s * c2g::kCorrValues;
      double* dwork = rt->alloc(std::max<int64_t>(work, 1));
      double* dy = rt->alloc(nv);
      rt->zero(dy, nv);
      rt->set_slot(c2g::kSlotWork, dwork);
      rt->run(*dp, nullptr, dy);
      std::vector<double> values(nv);
      C2G_CUDA(cudaMemcpyAsync(values.data(), dy, sizeof(double) * nv, cudaMemcpyDeviceToHost, rt->stream()));
      rt->sync();
      rt->set_slot(c2g::kSlotWork, nullptr);
      rt->release(dwork);
      rt->release(dy);
      for (int p = 0; p < s; p++) corr_->fill_pair(p, s, values.data() + p * c2g::kCorrValues);
    }
    if (dprev) {
      rt->set_slot((s % 2 == 0) ? c2g::kSlotCorr1 : c2g::kSlotCorr0, nullptr);
      rt->release(dprev);
    }
    cprev = std::move(cnext);
    dprev = dnext;
    if (site <= L - 3) update_moving_right(site);
  }
  if (dprev) {
    rt->sync();
    rt->release(dprev);
  }
  rt->set_slot(c2g::kSlotCorr0, nullptr);
  rt->set_slot(c2g::kSlotCorr1, nullptr);
}

void DMRG::upload_mps(int site, const std::vector<double>& data) {
  if (mps_dev[site]) rt->release(mps_dev[site]);
  mps_dev[site] = nullptr;
  mps_dev[site] = rt->alloc(static_cast<int64_t>(data.size()));
  C2G_CUDA(cudaMemcpyAsync(mps_dev[site], data.data(), sizeof(double) * data.size(), cudaMemcpyHostToDevice,
                           rt->stream()));
  rt->sync();
  rt->set_slot(c2g::kSlotMpsBase + site, mps_dev[site]);
}

void DMRG::drop_f32(const int b) {
  if (ops_dev32[b]) rt->release(ops_dev32[b]);
  ops_dev32[b] = nullptr;
  rt->set_slot32(c2g::slot_ops(L, b), nullptr);
}

// FP32 copies exist only for the operators that the Heff of sites (index, index + 1)
// reads (boundaries index - 1 and index + 1); a conversion streams one boundary's
// operators once (FP64 read, FP32 write), small beside the matvecs of a step, and the
// copies of all other boundaries are released (at L = 40, D = 4000 they would hold half
// as many bytes again as the FP64 operators).
void DMRG::ensure_f32(const int index) {
  for (int b = 0; b < L - 1; b++) {
    const bool needed = (b == index - 1 || b == index + 1) && ops[b] && ops_dev[b];
    if (!needed) {
      if (ops_dev32[b]) drop_f32(b);
      continue;
    }
    if (ops_dev32[b]) continue;
    ops_dev32[b] = rt->alloc_f32(ops[b]->size);
    C2G_CUDA(c2g::launch_to_f32(ops_dev32[b], ops_dev[b], ops[b]->size, rt->stream()));
    c2g::count_launches(1);
    rt->set_slot32(c2g::slot_ops(L, b), ops_dev32[b]);
  }
}

namespace {
// matvec arithmetic codes of the C-ABI: 0 FP64, 1 FP32, 2 tensor cores (split BF16)
c2g::Precision matvec_precision(const int code) {
  switch (code) {
    case 0: return c2g::Precision::kFP64;
    case 1: return c2g::Precision::kFP32;
    case 2: return c2g::Precision::kTC;
    default: throw std::invalid_argument("matvec precision must be 0 (FP64), 1 (FP32) or 2 (tensor cores)");
  }
}
}  // namespace

void DMRG::set_precision(int mode, double mixed_tol) {
  if (mode < 0 || mode > 2) throw std::invalid_argument("precision mode must be 0, 1 or 2");
  precision_ = mode;
  mixed_tol_ = mixed_tol;
}

int DMRG::get_num_mps_var() const {
  int n = 0;
  for (int s = 0; s < L; s++) n += static_cast<int>(mps_lay[s]->size());
  return n;
}

void DMRG::delete_all_ops() {
  version_++;
  for (int b = 0; b < L - 1; b++) {
    if (ops_dev[b]) rt->release(ops_dev[b]);
    ops_dev[b] = nullptr;
    drop_f32(b);
    ops[b].reset();
    rt->set_slot(c2g::slot_ops(L, b), nullptr);
    isAllocated[b] = 0;
  }
}

void DMRG::PreSolve() {
  // The matrix elements may have changed (Problem::setMxElement): compiled programs carry
  // them in their coefficients, so none may be reused.
  if (pcache_) {
    pcache_->map.clear();
    pcache_->bytes = 0;
  }
  if (heff_cache_) {
    heff_cache_->program.reset();
    heff_cache_->diag.reset();
    heff_cache_->index = -1;
  }
  delete_all_ops();
  for (int cnt = 0; cnt < L - 2; cnt++) update_moving_right(cnt);
  TotalMinEnergy = 1e8;
  MaxDiscWeightLastSweep = 0.0;
}

// CheMPS2/DMRGoperators.cpp:243-575 via the task compiler: all operators of boundary
// index + 1, moving right, from those of boundary index and MPS[index].
void DMRG::update_moving_right(const int index) {
  const double t0 = now();
  if (ops_dev[index]) rt->release(ops_dev[index]);
  ops_dev[index] = nullptr;
  ops[index] = std::make_unique<BoundaryOps>();
  c2g::allocate_ops(*ops[index], *denBK, L, index, true, c2g::slot_ops(L, index));
  ops_dev[index] = rt->alloc(ops[index]->size);
  rt->set_slot(c2g::slot_ops(L, index), ops_dev[index]);
  isAllocated[index] = 1;
  version_++;
  c2g::UpdateContext ctx;
  ctx.bk = denBK.get();
  ctx.prob = Prob;
  ctx.L = L;
  ctx.index = index;
  ctx.moving_right = true;
  ctx.prev = (index > 0) ? ops[index - 1].get() : nullptr;
  if (index > 0 && isAllocated[index - 1] != 1) throw std::logic_error("update_moving_right: left operators missing");
  ctx.next = ops[index].get();
  ctx.mps = mps_tensor(mps_lay[index].get(), index);
  DevProgram& dp = program(dims_key("update", index, index, index + 2, ctx.moving_right ? 1 : 0),
                           [&] { return c2g::compile_update_program(ctx, false); });
  rt->zero(ops_dev[index], ops[index]->size);
  rt->run(dp, nullptr, nullptr);
  drop_f32(index);
  // no synchronisation: the host goes on compiling the next site's programs while the
  // update runs; everything that reads its results is ordered after it on the stream
  if (!exc_.empty()) update_overlaps(index, true);
  stats_.t_update += now() - t0;
}

// CheMPS2/DMRGoperators.cpp:577-908, mirrored.
void DMRG::update_moving_left(const int index) {
  const double t0 = now();
  if (ops_dev[index]) rt->release(ops_dev[index]);
  ops_dev[index] = nullptr;
  ops[index] = std::make_unique<BoundaryOps>();
  c2g::allocate_ops(*ops[index], *denBK, L, index, false, c2g::slot_ops(L, index));
  ops_dev[index] = rt->alloc(ops[index]->size);
  rt->set_slot(c2g::slot_ops(L, index), ops_dev[index]);
  isAllocated[index] = 2;
  version_++;
  c2g::UpdateContext ctx;
  ctx.bk = denBK.get();
  ctx.prob = Prob;
  ctx.L = L;
  ctx.index = index;
  ctx.moving_right = false;
  ctx.prev = (index + 1 < L - 1) ? ops[index + 1].get() : nullptr;
  if (index + 1 < L - 1 && isAllocated[index + 1] != 2)
    throw std::logic_error("update_moving_left: right operators missing");
  ctx.next = ops[index].get();
  ctx.mps = mps_tensor(mps_lay[index + 1].get(), index + 1);
  DevProgram& dp = program(dims_key("update", index, index, index + 2, ctx.moving_right ? 1 : 0),
                           [&] { return c2g::compile_update_program(ctx, false); });
  rt->zero(ops_dev[index], ops[index]->size);
  rt->run(dp, nullptr, nullptr);
  drop_f32(index);
  // no synchronisation (as in update_moving_right)
  if (!exc_.empty()) update_overlaps(index, false);
  stats_.t_update += now() - t0;
}

double DMRG::Solve() {
  bool change = (TotalMinEnergy < 1e8);
  double Energy = 0.0;
  for (int instruction = 0; instruction < OptScheme->get_number(); instruction++) {
    int nIterations = 0;
    double EnergyPrevious = Energy + 10 * OptScheme->get_energy_conv(instruction);
    while (std::fabs(Energy - EnergyPrevious) > OptScheme->get_energy_conv(instruction) &&
           nIterations < OptScheme->get_max_sweeps(instruction)) {
      EnergyPrevious = Energy;
      Energy = sweep(false, change, instruction);
      change = true;
      Energy = sweep(true, change, instruction);
      if (verbose)
        std::printf("instruction %d sweep %d: E = %.15f  max discarded weight = %.3e\n", instruction, nIterations,
                    Energy, MaxDiscWeightLastSweep);
      if (makecheckpoints_) save_mps(false);
      nIterations++;
    }
  }
  return TotalMinEnergy;
}

// CheMPS2/DMRG.cpp:335-402 (sweepleft / sweepright).
double DMRG::sweep(const bool moving_right, const bool change, const int instruction) {
  double Energy = 0.0;
  const double noise_level = std::fabs(OptScheme->get_noise_prefactor(instruction)) * MaxDiscWeightLastSweep;
  const double rtol = OptScheme->get_dvdson_rtol(instruction);
  const int D = OptScheme->get_D(instruction);
  MaxDiscWeightLastSweep = 0.0;
  LastMinEnergy = 1e8;
  if (moving_right) {
    for (int index = 0; index < L - 2; index++) {
      Energy = solve_site(index, rtol, noise_level, D, true, change);
      step_energies_.push_back(Energy);
      TotalMinEnergy = std::min(TotalMinEnergy, Energy);
      LastMinEnergy = std::min(LastMinEnergy, Energy);
      update_moving_right(index);
    }
  } else {
    for (int index = L - 2; index > 0; index--) {
      Energy = solve_site(index, rtol, noise_level, D, false, change);
      step_energies_.push_back(Energy);
      TotalMinEnergy = std::min(TotalMinEnergy, Energy);
      LastMinEnergy = std::min(LastMinEnergy, Energy);
      update_moving_left(index);
    }
  }
  return Energy;
}

// CheMPS2/DMRG.cpp:404-452 (solve_site) with Sobject::Join / Split and Heff::SolveDAVIDSON.
double DMRG::solve_site(const int index, const double dvdson_rtol, const double noise_level,
                        const int virtual_dimension, const bool moving_right, const bool change) {
  cudaStream_t s = rt->stream();
  // ---- Join
  double t0 = now();
  TwoSiteLayout S;
  S.build(*denBK, index);
  const int64_t veclen = S.size();
  double* svec = rt->alloc(veclen);
  {
    DevProgram& dp = program(dims_key("join", index, index, index + 2), [&] {
      c2g::Compiled c;
      TaskBuilder tb;
      c2g::compile_join(tb, *denBK, S, mps_tensor(mps_lay[index].get(), index),
                        mps_tensor(mps_lay[index + 1].get(), index + 1));
      c.program = tb.finalize();
      return c;
    });
    rt->run(dp, nullptr, svec);
    rt->sync();
  }
  stats_.t_join += now() - t0;

  // ---- Davidson
  t0 = now();
  c2g::HeffContext ctx;
  ctx.bk = denBK.get();
  ctx.prob = Prob;
  ctx.S = &S;
  ctx.left = (index > 0) ? ops[index - 1].get() : nullptr;
  ctx.right = (index + 1 < L - 1) ? ops[index + 1].get() : nullptr;
  if (index > 0 && isAllocated[index - 1] != 1) throw std::logic_error("solve_site: left operators missing");
  if (index + 1 < L - 1 && isAllocated[index + 1] != 2) throw std::logic_error("solve_site: right operators missing");
  int maxdim = 1;
  for (int k = 0; k < S.nkappa; k++) maxdim = std::max(maxdim, std::max(S.rows[k], S.cols[k]));
  rt->ones(maxdim);
  double* diag = rt->alloc(veclen);
  DevProgram& dpd = program(dims_key("diag", index, index, index + 2, 0),
                            [&] { return c2g::compile_heff_diag_program(ctx, false); });
  rt->run(dpd, nullptr, diag);
  long long heff_operand_bytes = 0;
  DevProgram& dph_ref = program(dims_key("heff", index, index, index + 2, 0),
                                [&] { return c2g::compile_heff_program(ctx, true, false); }, &heff_operand_bytes);
  DevProgram* dph = &dph_ref;
  rt->prepare(*dph);
  c2g::DeviceDavidson dav(*rt, veclen, kDavidsonNumVec, kDavidsonNumVecKeep, dvdson_rtol, kDavidsonPrecondCutoff);
  dav.set_rand(rng_.get());
  cudaEvent_t e0, e1;
  C2G_CUDA(cudaEventCreate(&e0));
  C2G_CUDA(cudaEventCreate(&e1));
  float mv_ms = 0.f;
  // Projection vectors of the stored lower states (CheMPS2/DMRGtechnics.cpp:509-620):
  // y += sum_s (V_s . x) V_s after every matvec (CheMPS2/HeffDiagrams1.cpp:65-86).
  const int nexc = static_cast<int>(exc_.size());
  double* vmat = nullptr;
  double* vcoef = nullptr;
  if (nexc > 0) {
    vmat = rt->alloc(veclen * nexc);
    vcoef = rt->alloc(std::max(nexc, 1));
    for (int k = 0; k < nexc; k++) {
      ExcState& st = *exc_[k];
      TwoSiteLayout Sk;
      Sk.build(*st.bk, index);
      double* sup = rt->alloc(std::max<int64_t>(Sk.size(), 1));
      {
        TaskBuilder tb;
        c2g::compile_join(tb, *st.bk, Sk, MpsT{st.lay[index].get(), c2g::make_ref(exc_slot(k, false, index), 0)},
                          MpsT{st.lay[index + 1].get(), c2g::make_ref(exc_slot(k, false, index + 1), 0)});
        auto dp = rt->upload(tb.finalize());
        rt->run(*dp, nullptr, sup);
      }
      {
        if (index > 0 && st.odir[index - 1] != 1) throw std::logic_error("excited states: left overlaps missing");
        if (index + 1 < L - 1 && st.odir[index + 1] != 2) throw std::logic_error("excited states: right overlaps missing");
        c2g::OverlapT ol, orr;
        if (index > 0) ol = c2g::OverlapT{st.olay[index - 1].get(), c2g::make_ref(exc_slot(k, true, index - 1), 0)};
        if (index + 1 < L - 1)
          orr = c2g::OverlapT{st.olay[index + 1].get(), c2g::make_ref(exc_slot(k, true, index + 1), 0)};
        TaskBuilder tb;
        c2g::compile_veff(tb, S, Sk, c2g::make_ref(c2g::kSlotX, 0), index > 0 ? &ol : nullptr,
                          index + 1 < L - 1 ? &orr : nullptr, std::sqrt(st.eshift) / (Prob->gTwoS() + 1.0),
                          c2g::make_ref(c2g::kSlotY, 0));
        auto dp = rt->upload(tb.finalize());
        rt->run(*dp, sup, vmat + static_cast<int64_t>(k) * veclen);
      }
      rt->sync();
      rt->release(sup);
    }
  }
  auto matvec = [&](const double* x, double* y, c2g::Precision prec) {
    C2G_CUDA(cudaEventRecord(e0, s));
    rt->run(*dph, const_cast<double*>(x), y, prec, veclen);
    if (nexc > 0) {
      C2G_CUDA(c2g::launch_multi_dot(vmat, veclen, nexc, x, veclen, rt->partial(), vcoef, s));
      C2G_CUDA(c2g::launch_combine(y, 1.0, vmat, veclen, vcoef, nexc, veclen, s));
      c2g::count_launches(3);
    }
    C2G_CUDA(cudaEventRecord(e1, s));
    C2G_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    C2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    mv_ms += ms;
  };
  if (precision_ != 0) ensure_f32(index);
  const c2g::DavidsonStats ds =
      dav.solve(svec, diag, matvec, precision_ != 0, mixed_tol_, matvec_precision(precision_ == 0 ? 1 : precision_));
  stats_.n_matvec_fp32 += ds.n_matvec_fp32;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  rt->release(diag);
  if (vmat) rt->release(vmat);
  if (vcoef) rt->release(vcoef);
  stats_.n_matvec += ds.n_matvec;
  stats_.n_davidson++;
  stats_.t_matvec += 1e-3 * mv_ms;
  stats_.matvec_flops += static_cast<double>(dph->flops_repeat) * ds.n_matvec;
  stats_.matvec_bytes += static_cast<double>(heff_operand_bytes + 16 * veclen) * ds.n_matvec;
  const double Energy = ds.energy + Prob->gEconst();
  stats_.last_energy = Energy;
  stats_.t_solve += now() - t0;
  if (verbose) {
    std::printf("Energy at sites (%d, %d) is %.15f  [%d matvecs]", index, index + 1, Energy, ds.n_matvec);
    if (precision_ != 0)
      std::printf("  reduced-precision phase %d matvecs to residual %.2e%s, exact residual %.2e, %d refinement cycles, "
                  "%d reduced in all",
                  ds.n_lo, ds.lo_rnorm, ds.lo_stalled ? (ds.fp64_fallback ? " (stalled: solved in FP64)" : " (stalled)") : "",
                  ds.r_exact0, ds.n_cycles, ds.n_matvec_fp32);
    std::printf("\n");
    std::fflush(stdout);
  }

  // ---- Split
  t0 = now();
  if (noise_level > 0.0) {
    // CheMPS2/Sobject.cpp:652-661: noise in program convention, i.e. scaled by
    // sqrt(2S_R + 1) in the symmetric convention kept here.
    std::vector<double> noise(veclen);
    for (int k = 0; k < S.nkappa; k++) {
      const double f = std::sqrt(S.TwoSR[k] + 1.0);
      for (int64_t c = S.k2i[k]; c < S.k2i[k + 1]; c++)
        noise[c] = f * noise_level * (rng_->unit() - 0.5);
    }
    double* dn = rt->alloc(veclen);
    C2G_CUDA(cudaMemcpyAsync(dn, noise.data(), sizeof(double) * veclen, cudaMemcpyHostToDevice, s));
    C2G_CUDA(c2g::launch_axpy(svec, 1.0, dn, veclen, s));
    c2g::count_launches(1);
    rt->sync();
    rt->release(dn);
  }
  const c2g::SplitPlan plan = c2g::plan_split(*denBK, index, moving_right);
  double* work = rt->alloc(std::max<int64_t>(plan.work_size, 1));
  rt->zero(work, plan.work_size);
  rt->set_slot(c2g::kSlotWork, work);
  {
    DevProgram& dp = program(dims_key("split_assemble", index, index, index + 2, moving_right ? 1 : 0), [&] {
      c2g::Compiled c;
      TaskBuilder tb;
      c2g::compile_split_assemble(tb, *denBK, S, plan);
      c.program = tb.finalize();
      return c;
    });
    rt->run(dp, svec, nullptr);
  }
  // Eigendecomposition of every Gram matrix (FP64): sectors up to kBatchedEigMax in one
  // batched Jacobi launch, those up to kBatchedEigLargeMax in a second one (all sectors
  // of a launch at once, one CTA each), larger ones with cuSOLVER syevd.
  std::vector<c2g::EigJob> jobs;
  int nsmall = 0, nmax_large = 0;
  for (const auto& c : plan.centers)
    if (c.cd > 0 && c.g <= c2g::kBatchedEigMax) jobs.push_back(c2g::EigJob{c.g, 0, c.offG, c.offE, c.offU});
  nsmall = static_cast<int>(jobs.size());
  for (const auto& c : plan.centers)
    if (c.cd > 0 && c.g > c2g::kBatchedEigMax && c.g <= c2g::kBatchedEigLargeMax) {
      jobs.push_back(c2g::EigJob{c.g, 0, c.offG, c.offE, c.offU});
      nmax_large = std::max(nmax_large, c.g);
    }
  // The batched kernels run on the auxiliary stream, overlapping the syevd calls below on
  // the main one; the main stream joins them before the eigenvalues are read. `jobs`
  // (pageable) stays alive until that final synchronisation.
  bool forked = false;
  if (!jobs.empty()) {
    rt->fork_aux();
    forked = true;
    cudaStream_t a = rt->aux_stream();
    c2g::EigJob* djobs = nullptr;
    C2G_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&djobs), sizeof(c2g::EigJob) * jobs.size(), a));
    C2G_CUDA(cudaMemcpyAsync(djobs, jobs.data(), sizeof(c2g::EigJob) * jobs.size(), cudaMemcpyHostToDevice, a));
    if (nsmall > 0) {
      C2G_CUDA(c2g::launch_batched_eig(djobs, nsmall, work, a));
      c2g::count_launches(1);
    }
    const int nlarge = static_cast<int>(jobs.size()) - nsmall;
    if (nlarge > 0) {
      C2G_CUDA(c2g::launch_batched_eig_large(djobs + nsmall, nlarge, nmax_large, work, a));
      c2g::count_launches(1);
    }
    C2G_CUDA(cudaFreeAsync(djobs, a));
  }
  if (!solver_) {
    cusolverDnHandle_t h = nullptr;
    check_solver(cusolverDnCreate(&h), "create");
    solver_ = h;
    check_solver(cusolverDnSetStream(h, s), "stream");
  }
  cusolverDnHandle_t sh = static_cast<cusolverDnHandle_t>(solver_);
  int gmax = 0;
  for (const auto& c : plan.centers) gmax = std::max(gmax, (c.cd > 0 && c.g > c2g::kBatchedEigLargeMax) ? c.g : 0);
  int lwork = 0;
  double* dwork = nullptr;
  int* dinfo = nullptr;
  C2G_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dinfo), sizeof(int) * std::max<size_t>(plan.centers.size(), 1), s));
  C2G_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int) * std::max<size_t>(plan.centers.size(), 1), s));
  if (gmax > 0) {
    check_solver(cusolverDnDsyevd_bufferSize(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, gmax, work, gmax,
                                             work, &lwork),
                 "bufferSize");
    dwork = rt->alloc(std::max(lwork, 1));
  }
  for (size_t ic = 0; ic < plan.centers.size(); ic++) {
    const auto& c = plan.centers[ic];
    if (c.cd <= 0 || c.g <= c2g::kBatchedEigLargeMax) continue;
    int lw = 0;
    check_solver(cusolverDnDsyevd_bufferSize(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, c.g, work + c.offG,
                                             c.g, work + c.offE, &lw),
                 "bufferSize");
    if (lw > lwork) {
      rt->release(dwork);
      lwork = lw;
      dwork = rt->alloc(lwork);
    }
    check_solver(cusolverDnDsyevd(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, c.g, work + c.offG, c.g,
                                  work + c.offE, dwork, lwork, dinfo + ic),
                 "syevd");
    // eigenvectors in descending order of the eigenvalue
    C2G_CUDA(c2g::launch_reverse_columns(work + c.offU, work + c.offG, c.g, c.g, s));
    c2g::count_launches(1);
  }
  if (forked) rt->join_aux();
  std::vector<double> evals(plan.work_size > 0 ? plan.work_size : 1);
  std::vector<int> info(std::max<size_t>(plan.centers.size(), 1));
  // only the eigenvalue segments are needed; copy each
  for (const auto& c : plan.centers)
    if (c.cd > 0)
      C2G_CUDA(cudaMemcpyAsync(evals.data() + c.offE, work + c.offE, sizeof(double) * c.g, cudaMemcpyDeviceToHost, s));
  C2G_CUDA(cudaMemcpyAsync(info.data(), dinfo, sizeof(int) * info.size(), cudaMemcpyDeviceToHost, s));
  rt->sync();
  for (size_t ic = 0; ic < plan.centers.size(); ic++)
    if (info[ic] != 0) throw std::runtime_error("Split: eigensolver failed for a center sector");
  if (dwork) rt->release(dwork);
  C2G_CUDA(cudaFreeAsync(dinfo, s));

  // Singular values per center sector, descending (CheMPS2/Sobject.cpp:418-420).
  const int nC = static_cast<int>(plan.centers.size());
  std::vector<std::vector<double>> lambdas(nC);
  for (int ic = 0; ic < nC; ic++) {
    const auto& c = plan.centers[ic];
    lambdas[ic].resize(c.cd);
    for (int i = 0; i < c.cd; i++) lambdas[ic][i] = std::sqrt(std::max(evals[c.offE + c.g - 1 - i], 0.0));
  }
  // CheMPS2/Sobject.cpp:431-519: new virtual dimensions and discarded weight.
  double discardedWeight = 0.0;
  bool updateSectors = false;
  std::vector<int> NewDims(nC);
  if (change) {
    int totalDimSVD = 0;
    for (int ic = 0; ic < nC; ic++) {
      NewDims[ic] = plan.centers[ic].cd;
      totalDimSVD += NewDims[ic];
    }
    if (totalDimSVD > virtual_dimension) {
      std::vector<double> values;
      values.reserve(totalDimSVD);
      for (int ic = 0; ic < nC; ic++)
        for (int i = 0; i < NewDims[ic]; i++) values.push_back(lambdas[ic][i]);
      std::sort(values.begin(), values.end(), std::greater<double>());
      const double lowerBound = values[virtual_dimension];
      for (int ic = 0; ic < nC; ic++)
        for (int cnt = 0; cnt < NewDims[ic]; cnt++)
          if (lambdas[ic][cnt] <= lowerBound) NewDims[ic] = cnt;
      double totalSum = 0.0, discardedSum = 0.0;
      for (int ic = 0; ic < nC; ic++)
        for (int i = 0; i < plan.centers[ic].cd; i++) {
          const double temp = (plan.centers[ic].TwoSM + 1) * lambdas[ic][i] * lambdas[ic][i];
          totalSum += temp;
          if (lambdas[ic][i] <= lowerBound) discardedSum += temp;
        }
      discardedWeight = discardedSum / totalSum;
    }
    for (int ic = 0; ic < nC; ic++) {
      const auto& c = plan.centers[ic];
      if (NewDims[ic] != denBK->gCurrentDim(index + 1, c.NM, c.TwoSM, c.IM)) updateSectors = true;
    }
  }
  if (updateSectors)
    for (int ic = 0; ic < nC; ic++) {
      const auto& c = plan.centers[ic];
      denBK->SetDim(index + 1, c.NM, c.TwoSM, c.IM, NewDims[ic]);
    }
  std::vector<int> dims_m(nC);
  for (int ic = 0; ic < nC; ic++) {
    const auto& c = plan.centers[ic];
    dims_m[ic] = denBK->gCurrentDim(index + 1, c.NM, c.TwoSM, c.IM);
  }
  // New MPS tensors for sites index and index + 1 (CheMPS2/Sobject.cpp:521-590).
  for (int site = index; site <= index + 1; site++) {
    mps_lay[site] = std::make_unique<MpsLayout>();
    mps_lay[site]->build(*denBK, site);
    double* old = mps_dev[site];
    mps_dev[site] = rt->alloc(mps_lay[site]->size());
    rt->zero(mps_dev[site], mps_lay[site]->size());
    rt->set_slot(c2g::kSlotMpsBase + site, mps_dev[site]);
    rt->release(old);
  }
  {
    // keyed on the new dimensions at index + 1 (and the unchanged ones at index, index + 2)
    DevProgram& dp = program(dims_key("split_copy", index, index, index + 2, moving_right ? 1 : 0), [&] {
      c2g::Compiled c;
      TaskBuilder tb;
      c2g::compile_split_copy(tb, plan, dims_m, mps_tensor(mps_lay[index].get(), index),
                              mps_tensor(mps_lay[index + 1].get(), index + 1));
      c.program = tb.finalize();
      return c;
    });
    rt->run(dp, nullptr, nullptr);
  }
  rt->sync();
  rt->set_slot(c2g::kSlotWork, nullptr);
  rt->release(work);
  rt->release(svec);
  version_++;
  MaxDiscWeightLastSweep = std::max(MaxDiscWeightLastSweep, discardedWeight);
  stats_.t_split += now() - t0;
  return Energy;
}

// The Heff program of sites (index, index + 1), compiled once per state of the MPS and
// operators (every update, split and PreSolve advances the state version).
DMRG::HeffCache& DMRG::heff_program(const int index, const bool with_diag) {
  if (index < 0 || index > L - 2) throw std::out_of_range("heff: index");
  if (index > 0 && isAllocated[index - 1] != 1) throw std::logic_error("heff: left operators missing");
  if (index + 1 < L - 1 && isAllocated[index + 1] != 2) throw std::logic_error("heff: right operators missing");
  HeffCache& c = *heff_cache_;
  if (!(c.index == index && c.version == version_ && c.program)) {
    c.program.reset();
    c.diag.reset();
    c.S = std::make_unique<TwoSiteLayout>();
    c.S->build(*denBK, index);
    c2g::HeffContext ctx;
    ctx.bk = denBK.get();
    ctx.prob = Prob;
    ctx.S = c.S.get();
    ctx.left = (index > 0) ? ops[index - 1].get() : nullptr;
    ctx.right = (index + 1 < L - 1) ? ops[index + 1].get() : nullptr;
    const double tc = now();
    c2g::Compiled ch = c2g::compile_heff_program(ctx, true, false);
    stats_.t_compile += now() - tc;
    const double tu = now();
    c.program = ch.parts.empty() ? rt->upload(ch.program) : rt->upload(ch.parts);
    stats_.t_upload += now() - tu;
    rt->prepare(*c.program);
    c.operand_bytes = ch.operand_bytes;
    c.index = index;
    c.version = version_;
  }
  if (with_diag && !c.diag) {
    c2g::HeffContext ctx;
    ctx.bk = denBK.get();
    ctx.prob = Prob;
    ctx.S = c.S.get();
    ctx.left = (index > 0) ? ops[index - 1].get() : nullptr;
    ctx.right = (index + 1 < L - 1) ? ops[index + 1].get() : nullptr;
    c2g::Compiled cd = c2g::compile_heff_diag_program(ctx, false);
    c.diag = cd.parts.empty() ? rt->upload(cd.program) : rt->upload(cd.parts);
  }
  return c;
}

double DMRG::bench_heff(const int index, const int warmup, const int steps, double* flops, double* bytes,
                        long long* launches, const long long flush_bytes, const int precision) {
  const c2g::Precision prec = matvec_precision(precision);
  cudaStream_t s = rt->stream();
  HeffCache& c = heff_program(index, false);
  const int64_t veclen = c.S->size();
  double* x = rt->alloc(veclen);
  double* y = rt->alloc(veclen);
  {
    TaskBuilder tb;
    c2g::compile_join(tb, *denBK, *c.S, mps_tensor(mps_lay[index].get(), index),
                      mps_tensor(mps_lay[index + 1].get(), index + 1));
    auto dp = rt->upload(tb.finalize());
    rt->run(*dp, nullptr, x);
  }
  double* flush = nullptr;
  const int64_t nflush = flush_bytes > 0 ? (flush_bytes + 7) / 8 : 0;
  if (nflush > 0) flush = rt->alloc(nflush);
  if (prec != c2g::Precision::kFP64) ensure_f32(index);
  for (int i = 0; i < warmup; i++) rt->run(*c.program, x, y, prec, veclen);
  rt->sync();
  const long long l0 = c2g::kernel_launches();
  cudaEvent_t e0, e1;
  C2G_CUDA(cudaEventCreate(&e0));
  C2G_CUDA(cudaEventCreate(&e1));
  double total_ms = 0.0;
  for (int i = 0; i < steps; i++) {
    if (flush) C2G_CUDA(cudaMemsetAsync(flush, i & 0xff, sizeof(double) * nflush, s));  // evicts L2
    C2G_CUDA(cudaEventRecord(e0, s));
    rt->run(*c.program, x, y, prec, veclen);
    C2G_CUDA(cudaEventRecord(e1, s));
    C2G_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    C2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    total_ms += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (launches) *launches = c2g::kernel_launches() - l0;
  if (flops) *flops = static_cast<double>(c.program->flops_repeat);
  if (bytes) *bytes = static_cast<double>(c.operand_bytes) + 16.0 * veclen;
  if (flush) rt->release(flush);
  rt->release(x);
  rt->release(y);
  rt->sync();
  return steps > 0 ? total_ms / steps : 0.0;
}

long long DMRG::mps_size(const int site) const {
  if (site < 0 || site >= L) throw std::out_of_range("mps_size: site");
  return mps_lay[site]->size();
}

void DMRG::get_mps(const int site, double* out, const long long n) const {
  if (site < 0 || site >= L) throw std::out_of_range("get_mps: site");
  if (n != mps_lay[site]->size()) throw std::invalid_argument("get_mps: length differs from the tensor size");
  if (n > 0) {
    if (!out) throw std::invalid_argument("get_mps: null buffer");
    C2G_CUDA(cudaMemcpyAsync(out, mps_dev[site], sizeof(double) * n, cudaMemcpyDeviceToHost, rt->stream()));
  }
  rt->sync();
}

// CheMPS2/DMRGtechnics.cpp:341-470 on the host, from the downloaded MPS tensors
double DMRG::getFCIcoefficient(int* alpha, int* beta) const {
  if (!alpha || !beta) throw std::invalid_argument("getFCIcoefficient: null occupation array");
  std::vector<std::vector<double>> data(L);
  std::vector<const c2g::MpsLayout*> lay(L);
  std::vector<const double*> T(L);
  for (int k = 0; k < L; k++) {
    const long long n = mps_size(k);
    data[k].resize(static_cast<size_t>(std::max<long long>(n, 1)));
    if (n > 0) get_mps(k, data[k].data(), n);
    lay[k] = mps_lay[k].get();
    T[k] = data[k].data();
  }
  return c2g::fci_coefficient(*denBK, *Prob, lay, T, alpha, beta);
}

// CheMPS2/DMRGtechnics.cpp:324-339
double DMRG::getSpecificCoefficient(int* coeff) const {
  if (!coeff) throw std::invalid_argument("getSpecificCoefficient: null occupation array");
  std::vector<int> a(L), b(L);
  for (int h = 0; h < L; h++) {
    if (coeff[h] < 0 || coeff[h] > 2) throw std::invalid_argument("getSpecificCoefficient: occupations must be 0, 1 or 2");
    a[h] = (coeff[h] >= 1) ? 1 : 0;
    b[h] = (coeff[h] == 2) ? 1 : 0;
  }
  return getFCIcoefficient(a.data(), b.data());
}

long long DMRG::sobject_size(const int index) const {
  if (index < 0 || index > L - 2) throw std::out_of_range("sobject_size: index");
  TwoSiteLayout S;
  S.build(*denBK, index);
  return S.size();
}

void DMRG::heff_apply_host(const int index, const bool join_into_x, double* x, double* y, double* diag,
                           const long long n, const int precision) {
  if (!x || !y) throw std::invalid_argument("heff_apply: null buffer");
  cudaStream_t s = rt->stream();
  HeffCache& c = heff_program(index, diag != nullptr);
  const int64_t veclen = c.S->size();
  if (n != veclen) throw std::invalid_argument("heff_apply: vector length differs from the two-site object size");
  if (c.xbuf_len < veclen) {
    rt->release(c.xbuf);
    rt->release(c.ybuf);
    c.xbuf = rt->alloc(veclen);
    c.ybuf = rt->alloc(veclen);
    c.xbuf_len = veclen;
  }
  if (join_into_x) {
    TaskBuilder tb;
    c2g::compile_join(tb, *denBK, *c.S, mps_tensor(mps_lay[index].get(), index),
                      mps_tensor(mps_lay[index + 1].get(), index + 1));
    auto dp = rt->upload(tb.finalize());
    rt->run(*dp, nullptr, c.xbuf);
    C2G_CUDA(cudaMemcpyAsync(x, c.xbuf, sizeof(double) * veclen, cudaMemcpyDeviceToHost, s));
  } else {
    C2G_CUDA(cudaMemcpyAsync(c.xbuf, x, sizeof(double) * veclen, cudaMemcpyHostToDevice, s));
  }
  const c2g::Precision prec = matvec_precision(precision);
  if (prec != c2g::Precision::kFP64) ensure_f32(index);
  rt->run(*c.program, c.xbuf, c.ybuf, prec, veclen);
  C2G_CUDA(cudaMemcpyAsync(y, c.ybuf, sizeof(double) * veclen, cudaMemcpyDeviceToHost, s));
  if (diag) {
    int maxdim = 1;
    for (int k = 0; k < c.S->nkappa; k++) maxdim = std::max(maxdim, std::max(c.S->rows[k], c.S->cols[k]));
    rt->ones(maxdim);
    rt->run(*c.diag, nullptr, c.ybuf);
    C2G_CUDA(cudaMemcpyAsync(diag, c.ybuf, sizeof(double) * veclen, cudaMemcpyDeviceToHost, s));
  }
  rt->sync();
}

void DMRG::heff_apply_device(const int index, const double* x_dev, double* y_dev, const long long n,
                             const int precision, void* stream) {
  if (!x_dev || !y_dev) throw std::invalid_argument("heff_apply_device: null buffer");
  if (index < 0 || index > L - 2) throw std::out_of_range("heff_apply_device: index");
  if (precision != 0 && precision != 1) throw std::invalid_argument("heff_apply_device: precision must be 0 or 1");
  HeffCache& c = heff_program(index, false);
  const int64_t veclen = c.S->size();
  if (n != veclen) throw std::invalid_argument("heff_apply_device: vector length differs from the two-site object size");
  cudaStream_t u = static_cast<cudaStream_t>(stream);
  if (u) rt->wait_for(u);  // x is ready once the caller's stream gets here
  const c2g::Precision prec = matvec_precision(precision);
  if (prec != c2g::Precision::kFP64) ensure_f32(index);
  rt->run(*c.program, const_cast<double*>(x_dev), y_dev, prec, veclen);
  if (u) rt->signal_to(u);  // the caller's stream waits for y
  else rt->sync();
}

void DMRG::heff_apply_noalloc(const int index, const double* x, double* y, const long long n) {
  if (!x || !y) throw std::invalid_argument("heff_apply_noalloc: null buffer");
  if (index < 0 || index > L - 2) throw std::out_of_range("heff_apply_noalloc: index");
  // the size limit is checked first, from the sector dimensions alone
  const int64_t veclen = sobject_size(index);
  if (n != veclen) throw std::invalid_argument("heff_apply_noalloc: vector length differs from the two-site object size");
  if (veclen > c2g::kStaticScratchMaxVector)
    throw std::invalid_argument("heff_apply_noalloc: two-site object of " + std::to_string(veclen) +
                                " doubles is too large for the static scratch (at most " +
                                std::to_string(c2g::kStaticScratchMaxVector) + ")");
  const int64_t ystart = (veclen + 31) / 32 * 32;  // y starts on a 256-byte boundary
  HeffCache& c = *heff_cache_;
  if (!(c.index == index && c.version == version_ && c.program))
    throw std::invalid_argument("heff_apply_noalloc: no Heff program for this index and state (call heff_apply first)");
  // the runtime's stream, memory and scratch belong to its device, whichever device the
  // calling thread has current; that device is made current for this call and restored
  int caller_dev = 0;
  C2G_CUDA(cudaGetDevice(&caller_dev));
  const int dev = rt->device();
  if (caller_dev != dev) C2G_CUDA(cudaSetDevice(dev));
  struct Restore {
    int from, to;
    ~Restore() {
      if (from != to) cudaSetDevice(to);
    }
  } restore{dev, caller_dev};
  double* base = nullptr;
  C2G_CUDA(c2g::static_scratch(dev, &base));
  double* dx = base;
  double* dy = base + ystart;
  cudaStream_t s = rt->stream();
  C2G_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * veclen, cudaMemcpyHostToDevice, s));
  // the program writes every output block; y is cleared so that no earlier caller's data
  // can survive in it
  C2G_CUDA(cudaMemsetAsync(dy, 0, sizeof(double) * veclen, s));
  rt->run(*c.program, dx, dy);
  C2G_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * veclen, cudaMemcpyDeviceToHost, s));
  rt->sync();  // the scratch is free for the next caller once this returns
}

}  // namespace CheMPS2
