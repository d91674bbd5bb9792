// extern "C" boundary: wraps the drop-in C++ classes into opaque handles with status codes.
#include "../../include/chemps2_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "device/kernels.cuh"
#include "dmrg/runtime.hpp"
#include "host/chemps2/Batch.h"
#include "host/chemps2/ConvergenceScheme.h"
#include "host/chemps2/DMRG.h"
#include "host/chemps2/Hamiltonian.h"
#include "host/chemps2/Problem.h"
#include "host/chemps2/SyBookkeeper.h"
#include "host/layout.hpp"
#include "host/rng.hpp"
#include "host/symm.hpp"

struct c2g_hamiltonian {
  std::unique_ptr<CheMPS2::Hamiltonian> h;
};
struct c2g_problem {
  std::unique_ptr<CheMPS2::Problem> p;
};
struct c2g_scheme {
  std::unique_ptr<CheMPS2::ConvergenceScheme> s;
};
struct c2g_dmrg {
  std::unique_ptr<CheMPS2::DMRG> d;
};

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

template <class F>
int guarded(F&& f) {
  try {
    f();
    g_error.clear();
    return C2G_OK;
  } catch (const c2g::CudaError& e) {
    if (e.code == cudaErrorNoDevice || e.code == cudaErrorInsufficientDriver) return fail(C2G_ERR_NO_DEVICE, e.what());
    return fail(C2G_ERR_CUDA, e.what());
  } catch (const std::invalid_argument& e) {
    return fail(C2G_ERR_INVALID, e.what());
  } catch (const std::out_of_range& e) {
    return fail(C2G_ERR_INVALID, e.what());
  } catch (const std::logic_error& e) {
    return fail(C2G_ERR_INTERNAL, e.what());
  } catch (const std::runtime_error& e) {
    const std::string w = e.what();
    if (w.find("no CUDA device") != std::string::npos) return fail(C2G_ERR_NO_DEVICE, w);
    return fail(C2G_ERR_OTHER, w);
  } catch (const std::exception& e) {
    return fail(C2G_ERR_OTHER, e.what());
  } catch (...) {
    return fail(C2G_ERR_OTHER, "unknown exception");
  }
}

// The C2G_NUM_STATS layout of c2g_dmrg_stats.
void fill_stats(const CheMPS2::DMRGStats& s, double* out, int n) {
  const double v[C2G_NUM_STATS] = {static_cast<double>(s.n_matvec), static_cast<double>(s.n_davidson),
                                   s.t_join, s.t_solve, s.t_split, s.t_update, s.t_matvec, s.t_compile,
                                   s.matvec_flops, s.matvec_bytes, s.last_energy,
                                   static_cast<double>(s.n_matvec_fp32), s.t_upload};
  for (int i = 0; i < n && i < C2G_NUM_STATS; i++) out[i] = v[i];
}

#define NEED(x)                                                        \
  do {                                                                 \
    if (!(x)) throw std::invalid_argument("null argument: " #x);       \
  } while (0)

}  // namespace

extern "C" {

const char* c2g_last_error(void) { return g_error.c_str(); }
int c2g_version(void) { return 100; }
int c2g_srand(unsigned int seed) {
  std::srand(seed);
  return C2G_OK;
}
int c2g_kernel_launches(long long* count) {
  return guarded([&] {
    NEED(count);
    *count = c2g::kernel_launches();
  });
}

// ---- Hamiltonian
int c2g_hamiltonian_create(int L, int group, const int* irreps, c2g_hamiltonian** out) {
  return guarded([&] {
    NEED(irreps);
    NEED(out);
    auto h = std::make_unique<c2g_hamiltonian>();
    h->h = std::make_unique<CheMPS2::Hamiltonian>(L, group, irreps);
    *out = h.release();
  });
}
int c2g_hamiltonian_create_fcidump(const char* path, int group, c2g_hamiltonian** out) {
  return guarded([&] {
    NEED(path);
    NEED(out);
    auto h = std::make_unique<c2g_hamiltonian>();
    h->h = std::make_unique<CheMPS2::Hamiltonian>(std::string(path), group);
    *out = h.release();
  });
}
int c2g_hamiltonian_destroy(c2g_hamiltonian* h) {
  delete h;
  return C2G_OK;
}
int c2g_hamiltonian_get_L(const c2g_hamiltonian* h, int* L) {
  return guarded([&] {
    NEED(h);
    NEED(L);
    *L = h->h->getL();
  });
}
int c2g_hamiltonian_get_group(const c2g_hamiltonian* h, int* group) {
  return guarded([&] {
    NEED(h);
    NEED(group);
    *group = h->h->getNGroup();
  });
}
int c2g_hamiltonian_get_irrep(const c2g_hamiltonian* h, int orb, int* irrep) {
  return guarded([&] {
    NEED(h);
    NEED(irrep);
    if (orb < 0 || orb >= h->h->getL()) throw std::invalid_argument("orbital index");
    *irrep = h->h->getOrbitalIrrep(orb);
  });
}
int c2g_hamiltonian_set_econst(c2g_hamiltonian* h, double v) {
  return guarded([&] {
    NEED(h);
    h->h->setEconst(v);
  });
}
int c2g_hamiltonian_get_econst(const c2g_hamiltonian* h, double* v) {
  return guarded([&] {
    NEED(h);
    NEED(v);
    *v = h->h->getEconst();
  });
}
static void check_orb(const CheMPS2::Hamiltonian& h, int i) {
  if (i < 0 || i >= h.getL()) throw std::invalid_argument("orbital index out of range");
}
int c2g_hamiltonian_set_tmat(c2g_hamiltonian* h, int i, int j, double v) {
  return guarded([&] {
    NEED(h);
    check_orb(*h->h, i);
    check_orb(*h->h, j);
    h->h->setTmat(i, j, v);
  });
}
int c2g_hamiltonian_get_tmat(const c2g_hamiltonian* h, int i, int j, double* v) {
  return guarded([&] {
    NEED(h);
    NEED(v);
    check_orb(*h->h, i);
    check_orb(*h->h, j);
    *v = h->h->getTmat(i, j);
  });
}
int c2g_hamiltonian_set_vmat(c2g_hamiltonian* h, int i, int j, int k, int l, double v) {
  return guarded([&] {
    NEED(h);
    for (int o : {i, j, k, l}) check_orb(*h->h, o);
    h->h->setVmat(i, j, k, l, v);
  });
}
int c2g_hamiltonian_get_vmat(const c2g_hamiltonian* h, int i, int j, int k, int l, double* v) {
  return guarded([&] {
    NEED(h);
    NEED(v);
    for (int o : {i, j, k, l}) check_orb(*h->h, o);
    *v = h->h->getVmat(i, j, k, l);
  });
}

// ---- Problem
int c2g_problem_create(const c2g_hamiltonian* h, int two_s, int n, int irrep, c2g_problem** out) {
  return guarded([&] {
    NEED(h);
    NEED(out);
    auto p = std::make_unique<c2g_problem>();
    p->p = std::make_unique<CheMPS2::Problem>(h->h.get(), two_s, n, irrep);
    *out = p.release();
  });
}
int c2g_problem_destroy(c2g_problem* p) {
  delete p;
  return C2G_OK;
}
int c2g_problem_setup_reorder_d2h(c2g_problem* p) {
  return guarded([&] {
    NEED(p);
    p->p->SetupReorderD2h();
  });
}
int c2g_problem_setup_reorder_c2v(c2g_problem* p) {
  return guarded([&] {
    NEED(p);
    p->p->SetupReorderC2v();
  });
}
int c2g_problem_setup_reorder_custom(c2g_problem* p, const int* dmrg2ham) {
  return guarded([&] {
    NEED(p);
    NEED(dmrg2ham);
    p->p->setup_reorder_custom(const_cast<int*>(dmrg2ham));
  });
}
int c2g_problem_construct_mxelem(c2g_problem* p) {
  return guarded([&] {
    NEED(p);
    p->p->construct_mxelem();
  });
}
static void check_mx(const CheMPS2::Problem& p, int a, int b, int c, int d) {
  for (int o : {a, b, c, d})
    if (o < 0 || o >= p.gL()) throw std::invalid_argument("orbital index out of range");
  if (!p.has_mxelem()) throw std::invalid_argument("matrix elements not constructed (construct_mxelem)");
}
int c2g_problem_set_mx_element(c2g_problem* p, int a, int b, int c, int d, double v) {
  return guarded([&] {
    NEED(p);
    check_mx(*p->p, a, b, c, d);
    p->p->setMxElement(a, b, c, d, v);
  });
}
int c2g_problem_get_mx_element(const c2g_problem* p, int a, int b, int c, int d, double* v) {
  return guarded([&] {
    NEED(p);
    NEED(v);
    check_mx(*p->p, a, b, c, d);
    *v = p->p->gMxElement(a, b, c, d);
  });
}
int c2g_problem_check_rohf_occ(const c2g_problem* p, const int* occupancies, int* ok) {
  return guarded([&] {
    NEED(p);
    NEED(occupancies);
    NEED(ok);
    *ok = p->p->check_rohf_occ(occupancies) ? 1 : 0;
  });
}

int c2g_hamiltonian_write_fcidump(const c2g_hamiltonian* h, const char* path, int nelec, int two_s, int irrep) {
  return guarded([&] {
    NEED(h);
    NEED(path);
    h->h->writeFCIDUMP(std::string(path), nelec, two_s, irrep);
  });
}

int c2g_problem_check_consistency(const c2g_problem* p, int* ok) {
  return guarded([&] {
    NEED(p);
    NEED(ok);
    *ok = p->p->checkConsistency() ? 1 : 0;
  });
}

// ---- ConvergenceScheme
int c2g_scheme_create(int n, c2g_scheme** out) {
  return guarded([&] {
    NEED(out);
    if (n < 1) throw std::invalid_argument("number of instructions must be positive");
    auto s = std::make_unique<c2g_scheme>();
    s->s = std::make_unique<CheMPS2::ConvergenceScheme>(n);
    *out = s.release();
  });
}
int c2g_scheme_destroy(c2g_scheme* s) {
  delete s;
  return C2G_OK;
}
int c2g_scheme_set_instruction(c2g_scheme* s, int i, int D, double econv, int max_sweeps, double noise,
                               double rtol) {
  return guarded([&] {
    NEED(s);
    s->s->set_instruction(i, D, econv, max_sweeps, noise, rtol);
  });
}

// ---- bookkeeping (no GPU)
int c2g_bookkeeper_sectors(const c2g_problem* p, int D, int boundary, int* out, int cap, int* count) {
  return guarded([&] {
    NEED(p);
    NEED(count);
    CheMPS2::SyBookkeeper bk(p->p.get(), D);
    if (boundary < 0 || boundary > bk.gL()) throw std::invalid_argument("boundary out of range");
    const int ns = bk.num_sectors(boundary);
    *count = ns;
    if (cap <= 0) return;
    NEED(out);
    for (int id = 0; id < ns && id < cap; id++) {
      int n, s, i;
      bk.sector_labels(boundary, id, &n, &s, &i);
      out[5 * id + 0] = n;
      out[5 * id + 1] = s;
      out[5 * id + 2] = i;
      out[5 * id + 3] = bk.fci_dim_by_id(boundary, id);
      out[5 * id + 4] = bk.cur_dim_by_id(boundary, id);
    }
  });
}

int c2g_sobject_layout(const c2g_problem* p, int D, int index, int* labels, int64_t* k2i, int* reorder, int cap,
                       int* nkappa) {
  return guarded([&] {
    NEED(p);
    NEED(nkappa);
    CheMPS2::SyBookkeeper bk(p->p.get(), D);
    if (index < 0 || index > bk.gL() - 2) throw std::invalid_argument("index out of range");
    c2g::TwoSiteLayout S;
    S.build(bk, index);
    *nkappa = S.nkappa;
    if (cap <= 0) return;
    if (cap < S.nkappa) throw std::invalid_argument("capacity too small");
    NEED(labels);
    NEED(k2i);
    NEED(reorder);
    for (int k = 0; k < S.nkappa; k++) {
      const int v[9] = {S.NL[k], S.TwoSL[k], S.IL[k], S.N1[k], S.N2[k], S.TwoJ[k], S.NR[k], S.TwoSR[k], S.IR[k]};
      for (int j = 0; j < 9; j++) labels[9 * k + j] = v[j];
      k2i[k] = S.k2i[k];
      reorder[k] = S.reorder[k];
    }
    k2i[S.nkappa] = S.k2i[S.nkappa];
  });
}

int c2g_wigner3j(int ja, int jb, int jc, int ma, int mb, int mc, double* v) {
  return guarded([&] {
    NEED(v);
    *v = c2g::wigner3j(ja, jb, jc, ma, mb, mc);
  });
}

int c2g_wigner6j(int a, int b, int c, int d, int e, int f, double* v) {
  return guarded([&] {
    NEED(v);
    *v = c2g::wigner6j(a, b, c, d, e, f);
  });
}
int c2g_wigner9j(int a, int b, int c, int d, int e, int f, int g, int h, int i, double* v) {
  return guarded([&] {
    NEED(v);
    *v = c2g::wigner9j(a, b, c, d, e, f, g, h, i);
  });
}

// ---- DMRG
int c2g_dmrg_create(c2g_problem* p, c2g_scheme* s, const int* occupancies, c2g_dmrg** out) {
  return guarded([&] {
    NEED(p);
    NEED(s);
    NEED(out);
    auto d = std::make_unique<c2g_dmrg>();
    d->d = std::make_unique<CheMPS2::DMRG>(p->p.get(), s->s.get(), false, "/tmp", const_cast<int*>(occupancies));
    *out = d.release();
  });
}
int c2g_dmrg_create_chkpt(c2g_problem* p, c2g_scheme* s, int makechkpt, const int* occupancies, c2g_dmrg** out) {
  return guarded([&] {
    NEED(p);
    NEED(s);
    NEED(out);
    auto d = std::make_unique<c2g_dmrg>();
    d->d = std::make_unique<CheMPS2::DMRG>(p->p.get(), s->s.get(), makechkpt != 0, "/tmp",
                                           const_cast<int*>(occupancies));
    *out = d.release();
  });
}
int c2g_dmrg_loaded_mps(const c2g_dmrg* d, int* loaded) {
  return guarded([&] {
    NEED(d);
    NEED(loaded);
    *loaded = d->d->loadedMPS() ? 1 : 0;
  });
}
int c2g_dmrg_delete_stored_mps(c2g_dmrg* d) {
  return guarded([&] {
    NEED(d);
    d->d->deleteStoredMPS();
  });
}
int c2g_dmrg_destroy(c2g_dmrg* d) {
  return guarded([&] { delete d; });
}
int c2g_dmrg_solve(c2g_dmrg* d, double* energy) {
  return guarded([&] {
    NEED(d);
    NEED(energy);
    *energy = d->d->Solve();
  });
}
int c2g_dmrg_presolve(c2g_dmrg* d) {
  return guarded([&] {
    NEED(d);
    d->d->PreSolve();
  });
}
int c2g_dmrg_set_precision(c2g_dmrg* d, int mode, double mixed_tol) {
  return guarded([&] {
    NEED(d);
    if (mode < 0 || mode > 2)
      throw std::invalid_argument("precision mode must be 0 (FP64), 1 (mixed, FP32) or 2 (mixed, tensor cores)");
    if (!(mixed_tol > 0.0)) throw std::invalid_argument("mixed tolerance must be positive");
    d->d->set_precision(mode, mixed_tol);
  });
}
int c2g_dmrg_set_verbose(c2g_dmrg* d, int v) {
  return guarded([&] {
    NEED(d);
    d->d->set_verbose(v != 0);
  });
}
int c2g_dmrg_num_mps_var(const c2g_dmrg* d, int* n) {
  return guarded([&] {
    NEED(d);
    NEED(n);
    *n = d->d->get_num_mps_var();
  });
}
int c2g_dmrg_max_discarded_weight(const c2g_dmrg* d, double* w) {
  return guarded([&] {
    NEED(d);
    NEED(w);
    *w = d->d->get_MaxDiscardedWeightLastSweep();
  });
}
int c2g_dmrg_solve_site(c2g_dmrg* d, int index, double rtol, double noise, int D, int moving_right, int change,
                        double* energy) {
  return guarded([&] {
    NEED(d);
    NEED(energy);
    *energy = d->d->solve_site(index, rtol, noise, D, moving_right != 0, change != 0);
  });
}
int c2g_dmrg_update(c2g_dmrg* d, int index, int moving_right) {
  return guarded([&] {
    NEED(d);
    if (moving_right)
      d->d->update_moving_right(index);
    else
      d->d->update_moving_left(index);
  });
}
int c2g_dmrg_stats(const c2g_dmrg* d, double* out, int n) {
  return guarded([&] {
    NEED(d);
    NEED(out);
    fill_stats(d->d->stats(), out, n);
  });
}
int c2g_dmrg_reset_stats(c2g_dmrg* d) {
  return guarded([&] {
    NEED(d);
    d->d->reset_stats();
  });
}
int c2g_dmrg_bench_heff(c2g_dmrg* d, int index, int warmup, int steps, long long flush_bytes, int precision,
                        double* ms, double* flops, double* bytes, long long* launches) {
  return guarded([&] {
    NEED(d);
    NEED(ms);
    *ms = d->d->bench_heff(index, warmup, steps, flops, bytes, launches, flush_bytes, precision);
  });
}

int c2g_dmrg_sobject_size(const c2g_dmrg* d, int index, int64_t* n) {
  return guarded([&] {
    NEED(d);
    NEED(n);
    *n = d->d->sobject_size(index);
  });
}
int c2g_dmrg_heff_apply(c2g_dmrg* d, int index, int join_into_x, double* x, double* y, double* diag, int64_t n) {
  return guarded([&] {
    NEED(d);
    d->d->heff_apply_host(index, join_into_x != 0, x, y, diag, n);
  });
}
int c2g_dmrg_heff_apply_fp32(c2g_dmrg* d, int index, double* x, double* y, int64_t n) {
  return guarded([&] {
    NEED(d);
    d->d->heff_apply_host(index, false, x, y, nullptr, n, 1);
  });
}
int c2g_dmrg_heff_apply_precision(c2g_dmrg* d, int index, double* x, double* y, int64_t n, int precision) {
  return guarded([&] {
    NEED(d);
    d->d->heff_apply_host(index, false, x, y, nullptr, n, precision);
  });
}
int c2g_dmrg_activate_excitations(c2g_dmrg* d, int max_exc) {
  return guarded([&] {
    NEED(d);
    d->d->activateExcitations(max_exc);
  });
}
int c2g_dmrg_new_excitation(c2g_dmrg* d, double eshift) {
  return guarded([&] {
    NEED(d);
    d->d->newExcitation(eshift);
  });
}
int c2g_dmrg_calc_2dm(c2g_dmrg* d) {
  return guarded([&] {
    NEED(d);
    d->d->calc2DMandCorrelations();
  });
}
int c2g_dmrg_get_2dm(const c2g_dmrg* d, int ham_order, double* A, double* B) {
  return guarded([&] {
    NEED(d);
    const CheMPS2::TwoDM* dm = d->d->get2DM();
    if (!dm) throw std::invalid_argument("get_2dm: no 2-RDM computed (call c2g_dmrg_calc_2dm)");
    const int L = dm->gL();
    for (int a = 0; a < L; a++)
      for (int b = 0; b < L; b++)
        for (int c = 0; c < L; c++)
          for (int e = 0; e < L; e++) {
            const size_t at = a + static_cast<size_t>(L) * (b + static_cast<size_t>(L) * (c + static_cast<size_t>(L) * e));
            if (A) A[at] = ham_order ? dm->getTwoDMA_HAM(a, b, c, e) : dm->getTwoDMA_DMRG(a, b, c, e);
            if (B) B[at] = ham_order ? dm->getTwoDMB_HAM(a, b, c, e) : dm->getTwoDMB_DMRG(a, b, c, e);
          }
  });
}
int c2g_dmrg_2dm_trace_energy(const c2g_dmrg* d, double* trace, double* energy) {
  return guarded([&] {
    NEED(d);
    const CheMPS2::TwoDM* dm = d->d->get2DM();
    if (!dm) throw std::invalid_argument("2dm_trace_energy: no 2-RDM computed (call c2g_dmrg_calc_2dm)");
    if (trace) *trace = dm->trace();
    if (energy) *energy = dm->energy();
  });
}
int c2g_dmrg_get_correlations(const c2g_dmrg* d, int ham_order, double* cspin, double* cdens, double* cspinflip,
                              double* cdirad, double* mutinfo, double* entropy) {
  return guarded([&] {
    NEED(d);
    const CheMPS2::Correlations* c = d->d->getCorrelations();
    if (!c) throw std::invalid_argument("get_correlations: none computed (call c2g_dmrg_calc_2dm)");
    const int L = c->gL();
    for (int r = 0; r < L; r++) {
      if (entropy) entropy[r] = ham_order ? c->SingleOrbitalEntropy_HAM(r) : c->SingleOrbitalEntropy_DMRG(r);
      for (int q = 0; q < L; q++) {
        const size_t at = r + static_cast<size_t>(L) * q;
        if (cspin) cspin[at] = ham_order ? c->getCspin_HAM(r, q) : c->getCspin_DMRG(r, q);
        if (cdens) cdens[at] = ham_order ? c->getCdens_HAM(r, q) : c->getCdens_DMRG(r, q);
        if (cspinflip) cspinflip[at] = ham_order ? c->getCspinflip_HAM(r, q) : c->getCspinflip_DMRG(r, q);
        if (cdirad) cdirad[at] = ham_order ? c->getCdirad_HAM(r, q) : c->getCdirad_DMRG(r, q);
        if (mutinfo) mutinfo[at] = ham_order ? c->getMutualInformation_HAM(r, q) : c->getMutualInformation_DMRG(r, q);
      }
    }
  });
}
int c2g_dmrg_heff_apply_device(c2g_dmrg* d, int index, const double* x_dev, double* y_dev, int64_t n, int precision,
                               void* stream) {
  return guarded([&] {
    NEED(d);
    d->d->heff_apply_device(index, x_dev, y_dev, n, precision, stream);
  });
}
int c2g_dmrg_sectors(const c2g_dmrg* d, int boundary, int* out, int cap, int* count) {
  return guarded([&] {
    NEED(d);
    NEED(count);
    const CheMPS2::SyBookkeeper& bk = *d->d->get_bookkeeper();
    if (boundary < 0 || boundary > bk.gL()) throw std::invalid_argument("boundary out of range");
    const int ns = bk.num_sectors(boundary);
    *count = ns;
    if (cap <= 0) return;
    NEED(out);
    for (int id = 0; id < ns && id < cap; id++) {
      int n, s, i;
      bk.sector_labels(boundary, id, &n, &s, &i);
      out[5 * id + 0] = n;
      out[5 * id + 1] = s;
      out[5 * id + 2] = i;
      out[5 * id + 3] = bk.fci_dim_by_id(boundary, id);
      out[5 * id + 4] = bk.cur_dim_by_id(boundary, id);
    }
  });
}
int c2g_dmrg_get_mps(const c2g_dmrg* d, int site, double* out, int64_t cap, int64_t* n) {
  return guarded([&] {
    NEED(d);
    NEED(n);
    *n = d->d->mps_size(site);
    if (cap <= 0) return;
    if (cap < *n) throw std::invalid_argument("c2g_dmrg_get_mps: buffer shorter than the tensor");
    d->d->get_mps(site, out, *n);
  });
}

int c2g_dmrg_fci_coefficient(const c2g_dmrg* d, const int* alpha, const int* beta, double* coeff) {
  return guarded([&] {
    NEED(d);
    NEED(alpha);
    NEED(beta);
    NEED(coeff);
    *coeff = d->d->getFCIcoefficient(const_cast<int*>(alpha), const_cast<int*>(beta));
  });
}
int c2g_dmrg_step_energies(const c2g_dmrg* d, double* out, int cap, int* count) {
  return guarded([&] {
    NEED(d);
    NEED(count);
    const std::vector<double>& e = d->d->step_energies();
    *count = static_cast<int>(e.size());
    if (out)
      for (int i = 0; i < std::min(cap, *count); i++) out[i] = e[i];
  });
}
int c2g_dmrg_heff_apply_noalloc(c2g_dmrg* d, int index, const double* x, double* y, int64_t n) {
  return guarded([&] {
    NEED(d);
    d->d->heff_apply_noalloc(index, x, y, n);
  });
}

int c2g_batch_solve(int n, c2g_problem* const* problems, c2g_scheme* const* schemes, const unsigned int* seeds,
                    int workers, double* energies, long long* matvecs, double* seconds, int* statuses,
                    double* stats) {
  std::vector<CheMPS2::BatchResult> res;
  const int rc = guarded([&] {
    if (n < 0) throw std::invalid_argument("c2g_batch_solve: negative problem count");
    if (n > 0) {
      NEED(problems);
      NEED(schemes);
      NEED(seeds);
    }
    std::vector<CheMPS2::Problem*> ps(n);
    std::vector<CheMPS2::ConvergenceScheme*> ss(n);
    for (int i = 0; i < n; i++) {
      NEED(problems[i]);
      NEED(schemes[i]);
      ps[i] = problems[i]->p.get();
      ss[i] = schemes[i]->s.get();
    }
    res = CheMPS2::SolveBatch(ps, ss, std::vector<unsigned>(seeds, seeds + n), workers);
  });
  if (rc != C2G_OK) return rc;
  int first = C2G_OK;
  std::string first_error;
  for (int i = 0; i < n; i++) {
    const auto& r = res[i];
    // the same codes the single-problem calls return for these failures
    static const int kCode[5] = {C2G_OK, C2G_ERR_INVALID, C2G_ERR_CUDA, C2G_ERR_NO_DEVICE, C2G_ERR_OTHER};
    const int code = (r.status >= 0 && r.status < 5) ? kCode[r.status] : C2G_ERR_OTHER;
    if (energies) energies[i] = r.energy;
    if (matvecs) matvecs[i] = r.n_matvec;
    if (seconds) seconds[i] = r.seconds;
    if (statuses) statuses[i] = code;
    if (stats) fill_stats(r.stats, stats + static_cast<size_t>(i) * C2G_NUM_STATS, C2G_NUM_STATS);
    if (code != C2G_OK && first == C2G_OK) {
      first = code;
      first_error = "problem " + std::to_string(i) + ": " + r.error;
    }
  }
  if (first != C2G_OK) return fail(first, first_error);
  return C2G_OK;
}

int c2g_truncation_eig(int count, const int* n, const double* mats, double* evals, double* evecs) {
  return guarded([&] {
    if (count < 0) throw std::invalid_argument("c2g_truncation_eig: negative count");
    if (count == 0) return;
    NEED(n);
    NEED(mats);
    NEED(evals);
    NEED(evecs);
    std::vector<c2g::EigJob> small, large;
    int64_t tot = 0, totn = 0;
    int nmax = 0;
    for (int i = 0; i < count; i++) {
      if (n[i] < 1 || n[i] > c2g::kBatchedEigLargeMax)
        throw std::invalid_argument("c2g_truncation_eig: matrix order outside 1..128");
      tot += static_cast<int64_t>(n[i]) * n[i];
      totn += n[i];
    }
    // device layout: all matrices (Gram slots), then the eigenvalues, then the eigenvectors
    int64_t og = 0, oe = tot, ou = tot + totn;
    for (int i = 0; i < count; i++) {
      const c2g::EigJob jb{n[i], 0, og, oe, ou};
      (n[i] <= c2g::kBatchedEigMax ? small : large).push_back(jb);
      if (n[i] > c2g::kBatchedEigMax) nmax = std::max(nmax, n[i]);
      og += static_cast<int64_t>(n[i]) * n[i];
      oe += n[i];
      ou += static_cast<int64_t>(n[i]) * n[i];
    }
    double* d = nullptr;
    c2g::EigJob* dj = nullptr;
    C2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&d), sizeof(double) * (2 * tot + totn)));
    C2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&dj), sizeof(c2g::EigJob) * count));
    std::vector<c2g::EigJob> all(small);
    all.insert(all.end(), large.begin(), large.end());
    C2G_CUDA(cudaMemcpy(d, mats, sizeof(double) * tot, cudaMemcpyHostToDevice));
    C2G_CUDA(cudaMemcpy(dj, all.data(), sizeof(c2g::EigJob) * count, cudaMemcpyHostToDevice));
    if (!small.empty()) C2G_CUDA(c2g::launch_batched_eig(dj, static_cast<int>(small.size()), d, nullptr));
    if (!large.empty())
      C2G_CUDA(c2g::launch_batched_eig_large(dj + small.size(), static_cast<int>(large.size()), nmax, d, nullptr));
    C2G_CUDA(cudaDeviceSynchronize());
    C2G_CUDA(cudaMemcpy(evals, d + tot, sizeof(double) * totn, cudaMemcpyDeviceToHost));
    C2G_CUDA(cudaMemcpy(evecs, d + tot + totn, sizeof(double) * tot, cudaMemcpyDeviceToHost));
    cudaFree(dj);
    cudaFree(d);
  });
}

int c2g_rayleigh_ritz_eig(int n, const double* mat, int warm, double* evals, double* evecs, int reps,
                          double* us_per_call) {
  return guarded([&] {
    if (n < 1 || n > 32) throw std::invalid_argument("c2g_rayleigh_ritz_eig: order outside 1..32");
    if (reps < 1) throw std::invalid_argument("c2g_rayleigh_ritz_eig: reps must be positive");
    NEED(mat);
    NEED(evals);
    NEED(evecs);
    constexpr int ld = 32;
    std::vector<double> hm(static_cast<size_t>(ld) * ld, 0.0), he(static_cast<size_t>(ld) * ld, 0.0);
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) hm[i + ld * j] = mat[i + static_cast<size_t>(n) * j];
    if (warm)
      for (int j = 0; j < n - 1; j++)
        for (int i = 0; i < n - 1; i++) he[i + ld * j] = evecs[i + static_cast<size_t>(n - 1) * j];
    double* d = nullptr;
    C2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&d), sizeof(double) * (2 * ld * ld + ld)));
    struct Free {
      double* p;
      ~Free() { cudaFree(p); }
    } guard_free{d};
    double* dm = d;
    double* de = d + ld * ld;
    double* dv = d + 2 * ld * ld;
    C2G_CUDA(cudaMemcpy(dm, hm.data(), sizeof(double) * ld * ld, cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    C2G_CUDA(cudaEventCreate(&e0));
    C2G_CUDA(cudaEventCreate(&e1));
    float total_ms = 0.f;
    for (int r = 0; r < reps; r++) {
      // every repetition starts from the same inputs (the kernel overwrites evecs)
      C2G_CUDA(cudaMemcpy(de, he.data(), sizeof(double) * ld * ld, cudaMemcpyHostToDevice));
      C2G_CUDA(cudaEventRecord(e0));
      C2G_CUDA(c2g::launch_small_eig(dm, n, ld, dv, de, nullptr, warm != 0));
      C2G_CUDA(cudaEventRecord(e1));
      C2G_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      C2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      total_ms += ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<double> hv(ld);
    C2G_CUDA(cudaMemcpy(hv.data(), dv, sizeof(double) * ld, cudaMemcpyDeviceToHost));
    C2G_CUDA(cudaMemcpy(he.data(), de, sizeof(double) * ld * ld, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++) evals[i] = hv[i];
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) evecs[i + static_cast<size_t>(n) * j] = he[i + ld * j];
    if (us_per_call) *us_per_call = 1e3 * total_ms / reps;
  });
}

int c2g_device_memory_info(int device, int64_t* free_bytes, int64_t* pool_used_bytes) {
  return guarded([&] {
    NEED(free_bytes);
    NEED(pool_used_bytes);
    int cur = 0;
    C2G_CUDA(cudaGetDevice(&cur));
    if (device < 0) device = cur;
    if (device != cur) C2G_CUDA(cudaSetDevice(device));
    size_t fr = 0, tot = 0;
    cudaError_t e = cudaMemGetInfo(&fr, &tot);
    cudaMemPool_t pool = nullptr;
    uint64_t used = 0;
    if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, device);
    if (e == cudaSuccess) e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    if (device != cur) cudaSetDevice(cur);
    C2G_CUDA(e);
    *free_bytes = static_cast<int64_t>(fr);
    *pool_used_bytes = static_cast<int64_t>(used);
  });
}

int c2g_host_rand_sample(unsigned int seed, int n, int* out) {
  return guarded([&] {
    if (n < 0) throw std::invalid_argument("c2g_host_rand_sample: negative count");
    if (n > 0) NEED(out);
    c2g::HostRand r(seed);
    for (int i = 0; i < n; i++) out[i] = r.next();
  });
}

}  // extern "C"
