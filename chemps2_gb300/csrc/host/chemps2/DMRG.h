// Drop-in replacement for CheMPS2::DMRG (CheMPS2/include/chemps2/DMRG.h:93-162), for the
// two-site ground-state sweep: DMRG(Problem*, ConvergenceScheme*, ...), Solve() and
// PreSolve(). The MPS, the renormalized operators of every boundary and the Davidson
// vectors live in GPU memory; the Heff matvec, its diagonal, Join, Split and the operator
// updates run as device task programs (the task compiler is in the host sources, the
// kernels in the device sources). There is no CPU execution path: without a CUDA device
// the constructor throws.
#pragma once

#include <functional>
#include <memory>
#include <string>
#include <stdexcept>
#include <vector>

#include "ConvergenceScheme.h"
#include "Problem.h"
#include "SyBookkeeper.h"
#include "Correlations.h"
#include "TwoDM.h"

namespace c2g {
class Runtime;
class HostRand;
struct BoundaryOps;
struct MpsLayout;
struct DevProgram;
struct Compiled;
}  // namespace c2g

namespace CheMPS2 {

struct DMRGStats {
  long long n_matvec = 0;         // Heff applications
  long long n_matvec_fp32 = 0;    // of which with FP32 arithmetic (mixed precision)
  long long n_davidson = 0;       // Davidson solves
  double t_join = 0, t_solve = 0, t_split = 0, t_update = 0;  // seconds, host wall clock
  double t_matvec = 0;            // seconds inside Heff applications (device time)
  double t_compile = 0;           // seconds in the host task compiler
  double t_upload = 0;            // seconds uploading compiled programs (host work and copy)
  double matvec_flops = 0;        // ledger flops of all Heff applications
  double matvec_bytes = 0;        // ledger bytes of all Heff applications
  double last_energy = 0;
};

// Extension: construction options for DMRG objects that run on concurrent host threads
// (the batch entry point). With `private_seed` set, the object's random draws (MPS start,
// noise, Davidson guess fallback) come from its own generator seeded with `seed`: the
// sequence srand(seed) and rand() give, without the shared state of rand().
struct DMRGOptions {
  bool private_seed = false;
  unsigned seed = 1;
  bool makechkpt = false;
  int* occupancies = nullptr;
};

class DMRG {
 public:
  DMRG(Problem* Prob, ConvergenceScheme* OptScheme, const bool makechkpt = false,
       const std::string tmpfolder = "/tmp", int* occupancies = nullptr);
  DMRG(Problem* Prob, ConvergenceScheme* OptScheme, const DMRGOptions& options);
  ~DMRG();
  DMRG(const DMRG&) = delete;
  DMRG& operator=(const DMRG&) = delete;

  // Sweeps according to the convergence scheme; returns the lowest energy encountered
  // (including the constant part of the Hamiltonian), as CheMPS2/DMRG.cpp:268-333.
  double Solve();
  // Rebuilds every renormalized operator from the current MPS (CheMPS2/DMRG.cpp:258-266);
  // required after Problem::setMxElement.
  void PreSolve();

  int get_num_mps_var() const;
  double get_MaxDiscardedWeightLastSweep() const { return MaxDiscWeightLastSweep; }
  double get_TotalMinEnergy() const { return TotalMinEnergy; }
  const SyBookkeeper* get_bookkeeper() const { return denBK.get(); }
  const DMRGStats& stats() const { return stats_; }
  // Extension: the energy of every two-site step Solve() has run, in order (the reference
  // prints them, CheMPS2/DMRG.cpp:335-402; here they are kept for comparison).
  const std::vector<double>& step_energies() const { return step_energies_; }
  // Extension for checking: the current MPS tensor of `site` as TensorT::gStorage holds it
  // (CheMPS2/include/chemps2/TensorT.h:50; blocks in TensorT's order, column-major),
  // copied to host memory, and its length.
  long long mps_size(const int site) const;
  void get_mps(const int site, double* out, const long long n) const;
  // The coefficient of the determinant with occupations alpha[h], beta[h] (0 or 1) of the
  // Hamiltonian orbitals h in the current MPS (CheMPS2/DMRGtechnics.cpp:341-470), and of
  // the one given by coeff[h] in {0 empty, 1 one up electron, 2 doubly occupied}
  // (:324-339). Zero when the determinant lies outside the targeted sector.
  double getFCIcoefficient(int* alpha, int* beta) const;
  double getSpecificCoefficient(int* coeff) const;
  void reset_stats() { stats_ = DMRGStats(); }
  void set_verbose(bool v) { verbose = v; }
  // 0: FP64 Heff matvecs (the reference's arithmetic). 1: mixed, the Davidson solver
  // expands its subspace with FP32-arithmetic matvecs down to residual `mixed_tol`, then
  // finishes with FP64 matvecs to the instruction's tolerance, so energies and
  // eigenvectors are FP64 results.
  void set_precision(int mode, double mixed_tol = 1e-5);
  int get_precision() const { return precision_; }

  // One two-site step at sites (index, index + 1): Join, Davidson, Split. Returns the
  // energy (with the constant part). Exposed for the benchmark and tests.
  double solve_site(const int index, const double dvdson_rtol, const double noise_level,
                    const int virtual_dimension, const bool moving_right, const bool change);
  void update_moving_right(const int index);
  void update_moving_left(const int index);

  // Benchmark support: build the two-site object at `index`, then time `steps` Heff
  // applications after `warmup` untimed ones. Returns milliseconds per application and
  // the ledger work of one application.
  // flush_bytes > 0: a buffer of that size is overwritten before every timed application
  // (outside the timed interval) so that the operators are read from HBM, not L2.
  double bench_heff(const int index, const int warmup, const int steps, double* flops, double* bytes,
                    long long* launches, const long long flush_bytes = 0, const int precision = 0);

  // Host-buffer access to the effective Hamiltonian at sites (index, index + 1), in the
  // symmetric convention: y = Heff x (and its diagonal when diag is non-null). With
  // join_into_x, x is first overwritten by the joined current two-site object.
  long long sobject_size(const int index) const;
  // precision 1: FP32 arithmetic for the matvec (the diagonal stays FP64).
  void heff_apply_host(const int index, const bool join_into_x, double* x, double* y, double* diag,
                       const long long n, const int precision = 0);
  // y = Heff x (FP64) with no device allocation: x and y are staged through a static
  // device array shared by the process (not safe for concurrent calls). The Heff program
  // at `index` must already exist for the current state (a heff_apply_host call there).
  void heff_apply_noalloc(const int index, const double* x, double* y, const long long n);
  // Extension: y_dev = Heff x_dev on the caller's device buffers (precision 0: FP64, 1:
  // FP32 arithmetic). With a CUDA stream the call is ordered after the work already on it
  // and that stream waits for the result (no host synchronisation); without one the call
  // returns when y_dev is written.
  void heff_apply_device(const int index, const double* x_dev, double* y_dev, const long long n,
                         const int precision, void* stream);

  // CheMPS2/DMRG.h calc2DMandCorrelations (CheMPS2/DMRGtechnics.cpp:40-262 without the
  // 3-RDM): the two-particle density matrix of the current state, one site at a time from
  // the right with the MPS brought into mixed-canonical form around it, then the
  // correlation functions and the two-orbital mutual information in a pass from the left
  // (which also restores a left-canonical MPS and the operators of a finished right sweep,
  // so Solve() can continue). get2DM() / getCorrelations() return them (null before).
  void calc2DMandCorrelations();
  // CheMPS2/include/chemps2/DMRG.h:111: the 2-RDM and correlations; the 3-RDM is not
  // built in this implementation, so do_3rdm must be false.
  void calc_rdms_and_correlations(const bool do_3rdm, const bool disk_3rdm = false) {
    (void)disk_3rdm;
    if (do_3rdm) throw std::invalid_argument("calc_rdms_and_correlations: the 3-RDM is not available");
    calc2DMandCorrelations();
  }
  // CheMPS2/include/chemps2/DMRG.h:148: the renormalized operators live in device memory,
  // never on disk, so there is nothing to delete.
  void deleteStoredOperators() {}
  const TwoDM* get2DM() const { return two_dm_.get(); }
  const Correlations* getCorrelations() const { return corr_.get(); }

  // CheMPS2/DMRG.h activateExcitations / newExcitation (CheMPS2/DMRG.cpp:464-505): after
  // newExcitation(E_shift) the current state is stored and Solve() targets the next one,
  // every stored state s adding E_shift_s |V_s><V_s| to the effective Hamiltonian
  // (CheMPS2/HeffDiagrams1.cpp:65-86); at most maxExcIn stored states.
  void activateExcitations(const int maxExcIn);
  void newExcitation(const double EshiftIn);

  // MPS checkpoints (CheMPS2/DMRGmpsio.cpp:27-173, CheMPS2/DMRG.cpp:106-158,334): with
  // makechkpt, the MPS of the current state is written to CheMPS2_MPS<state>.c2g in the
  // working directory after every left+right sweep, and a DMRG constructed (or a new
  // excitation set up) while that file exists starts from it. The file holds the same
  // content as the reference's HDF5 file (virtual dimensions, MPS tensors, a converged flag)
  // in a flat binary layout. deleteStoredMPS removes the files.
  void deleteStoredMPS();
  bool loadedMPS() const { return loaded_mps_; }

 private:
  struct HeffCache;
  HeffCache& heff_program(const int index, const bool with_diag);
  std::unique_ptr<HeffCache> heff_cache_;
  unsigned long long version_ = 0;  // advanced by every change of the MPS or the operators

  // Compiled device programs, keyed by their kind, site and the sector dimensions they
  // depend on: once the virtual dimensions settle, later sweeps reuse the programs and
  // only their combination stages (which read operator data) run again.
  struct ProgramCache;
  std::unique_ptr<ProgramCache> pcache_;
  c2g::DevProgram& program(const std::string& key, const std::function<c2g::Compiled()>& build,
                           long long* operand_bytes = nullptr);
  std::string dims_key(const char* kind, const int index, const int bmin, const int bmax, const int extra = 0) const;

  bool makecheckpoints_ = false;
  bool loaded_mps_ = false;
  std::string mps_storage_name_;
  void save_mps(bool converged) const;
  bool load_mps();

  struct ExcState;
  std::vector<std::unique_ptr<ExcState>> exc_;
  bool exc_active_ = false;
  int max_exc_ = 0;
  int exc_slot(int state, bool overlap, int idx) const;
  void update_overlaps(int index, bool moving_right);
  void release_overlaps();

  std::unique_ptr<TwoDM> two_dm_;
  std::unique_ptr<Correlations> corr_;
  void download_mps(int site, std::vector<double>& data);
  void gauge_left_normalize(int site, bool into_next);
  void gauge_right_normalize(int site);
  void fill_2dm_site(int site);

  std::unique_ptr<c2g::HostRand> rng_;
  void construct(int* occupancies);
  void setup_mps(int* occupancies);
  void left_normalize_host(int site, std::vector<double>& data);
  void upload_mps(int site, const std::vector<double>& data);
  void delete_all_ops();
  double sweep(const bool moving_right, const bool change, const int instruction);

  Problem* Prob;
  ConvergenceScheme* OptScheme;
  int L;
  bool verbose = false;
  int precision_ = 0;
  double mixed_tol_ = 1e-5;
  std::unique_ptr<SyBookkeeper> denBK;
  std::unique_ptr<c2g::Runtime> rt;
  void* solver_ = nullptr;  // cuSOLVER handle of the truncation step (created on first use)
  std::vector<std::unique_ptr<c2g::MpsLayout>> mps_lay;
  std::vector<double*> mps_dev;
  std::vector<std::unique_ptr<c2g::BoundaryOps>> ops;
  std::vector<double*> ops_dev;
  std::vector<float*> ops_dev32;  // FP32 copies of the operators the current FP32 matvec reads
  void drop_f32(const int boundary);
  void ensure_f32(const int index);
  std::vector<int> isAllocated;  // 0 none, 1 moving right, 2 moving left
  double TotalMinEnergy = 1e8;
  double LastMinEnergy = 1e8;
  double MaxDiscWeightLastSweep = 0.0;
  DMRGStats stats_;
  std::vector<double> step_energies_;
};

}  // namespace CheMPS2
