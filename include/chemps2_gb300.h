/* C-ABI of the GB300 implementation of CheMPS2's two-site DMRG sweep.
 *
 * Every entry point returns an int status: C2G_OK (0) or a negative error code; the
 * message of the last error on the calling thread is returned by c2g_last_error(). No
 * C++ exception crosses this boundary. Objects are opaque handles owned by the caller,
 * with the reference's ownership rules: a Hamiltonian must outlive the Problems built on
 * it, and a Problem and a ConvergenceScheme must outlive the DMRG built on them
 * (CheMPS2/include/chemps2/DMRG.h, private-member comments).
 *
 * Each function names the reference interface it replaces (path:line inside the CheMPS2
 * project), or says that it has no counterpart there.
 */
#ifndef CHEMPS2_GB300_H
#define CHEMPS2_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  C2G_OK = 0,
  C2G_ERR_INVALID = -1,   /* invalid argument (the reference asserts)            */
  C2G_ERR_CUDA = -2,      /* a CUDA call failed                                   */
  C2G_ERR_NO_DEVICE = -3, /* no CUDA device: there is no CPU execution path       */
  C2G_ERR_INTERNAL = -4,  /* internal consistency check failed                    */
  C2G_ERR_OTHER = -5
};

typedef struct c2g_hamiltonian c2g_hamiltonian;
typedef struct c2g_problem c2g_problem;
typedef struct c2g_scheme c2g_scheme;
typedef struct c2g_dmrg c2g_dmrg;

/* Library */
const char* c2g_last_error(void);
int c2g_version(void);
/* Seeds the C library generator used for the random initial MPS, the Davidson fallback
 * guess and the noise, as the reference's callers do with srand (CheMPS2/Initialize.cpp:29). */
int c2g_srand(unsigned int seed);
/* Number of kernels this library launched in this process. */
int c2g_kernel_launches(long long* count);

/* CheMPS2::Hamiltonian (CheMPS2/Hamiltonian.cpp:33-64, :66-102 FCIDUMP, :104-145 setters) */
int c2g_hamiltonian_create(int L, int group, const int* irreps, c2g_hamiltonian** out);
int c2g_hamiltonian_create_fcidump(const char* path, int group, c2g_hamiltonian** out);
int c2g_hamiltonian_destroy(c2g_hamiltonian* h);
int c2g_hamiltonian_get_L(const c2g_hamiltonian* h, int* L);
int c2g_hamiltonian_get_group(const c2g_hamiltonian* h, int* group);
int c2g_hamiltonian_get_irrep(const c2g_hamiltonian* h, int orb, int* irrep);
int c2g_hamiltonian_set_econst(c2g_hamiltonian* h, double value);
int c2g_hamiltonian_get_econst(const c2g_hamiltonian* h, double* value);
int c2g_hamiltonian_set_tmat(c2g_hamiltonian* h, int i, int j, double value);
int c2g_hamiltonian_get_tmat(const c2g_hamiltonian* h, int i, int j, double* value);
int c2g_hamiltonian_set_vmat(c2g_hamiltonian* h, int i, int j, int k, int l, double value);
int c2g_hamiltonian_get_vmat(const c2g_hamiltonian* h, int i, int j, int k, int l, double* value);

/* CheMPS2::Problem (CheMPS2/Problem.cpp:33-56 ctor, :57-335 reorderings, :351-384 matrix elements) */
int c2g_problem_create(const c2g_hamiltonian* h, int two_s, int n, int irrep, c2g_problem** out);
int c2g_problem_destroy(c2g_problem* p);
int c2g_problem_setup_reorder_d2h(c2g_problem* p);
int c2g_problem_setup_reorder_c2v(c2g_problem* p);
int c2g_problem_setup_reorder_custom(c2g_problem* p, const int* dmrg2ham);
int c2g_problem_construct_mxelem(c2g_problem* p);
int c2g_problem_set_mx_element(c2g_problem* p, int a, int b, int c, int d, double value);
int c2g_problem_get_mx_element(const c2g_problem* p, int a, int b, int c, int d, double* value);
int c2g_problem_check_consistency(const c2g_problem* p, int* ok);
/* Problem::check_rohf_occ (CheMPS2/Problem.cpp:422-451): whether occupations 0, 1, 2 of
 * the L DMRG sites give the targeted (N, 2S, irrep) with the open shells high-spin. */
int c2g_problem_check_rohf_occ(const c2g_problem* p, const int* occupancies, int* ok);
/* Hamiltonian::writeFCIDUMP (CheMPS2/Hamiltonian.cpp:539-582): the Hamiltonian as an
 * FCIDUMP file with NELEC, MS2 and ISYM as given. */
int c2g_hamiltonian_write_fcidump(const c2g_hamiltonian* h, const char* path, int nelec, int two_s, int irrep);

/* CheMPS2::ConvergenceScheme (CheMPS2/ConvergenceScheme.cpp:29-76) */
int c2g_scheme_create(int n_instructions, c2g_scheme** out);
int c2g_scheme_destroy(c2g_scheme* s);
int c2g_scheme_set_instruction(c2g_scheme* s, int instruction, int D, double energy_conv, int max_sweeps,
                               double noise_prefactor, double dvdson_rtol);

/* CheMPS2::SyBookkeeper (CheMPS2/SyBookkeeper.cpp:29-323): sector dimensions at boundary b
 * for a bookkeeper built with virtual dimension D. Writes up to `cap` rows of
 * (N, 2S, I, FCI dim, current dim) into `out` (5 ints per row) and their count into
 * `count`; call with cap = 0 to query the count. Needs no GPU. */
int c2g_bookkeeper_sectors(const c2g_problem* p, int D, int boundary, int* out, int cap, int* count);

/* CheMPS2::Sobject block table (CheMPS2/Sobject.cpp:36-145) of sites (index, index + 1)
 * for a bookkeeper with virtual dimension D: per block the 9 labels
 * (NL, 2SL, IL, N1, N2, 2J, NR, 2SR, IR), kappa2index (nkappa + 1 entries) and the
 * size-sorted visiting order. Query sizes with cap = 0. Needs no GPU. */
int c2g_sobject_layout(const c2g_problem* p, int D, int index, int* labels, int64_t* kappa2index, int* reorder,
                       int cap, int* nkappa);

/* Wigner symbols (CheMPS2/Wigner.cpp:243-370), arguments are twice the spins (and, for
 * the 3j symbol, twice the projections). */
int c2g_wigner3j(int ja, int jb, int jc, int ma, int mb, int mc, double* value);
int c2g_wigner6j(int a, int b, int c, int d, int e, int f, double* value);
int c2g_wigner9j(int a, int b, int c, int d, int e, int f, int g, int h, int i, double* value);

/* CheMPS2::DMRG (CheMPS2/include/chemps2/DMRG.h:93-162, CheMPS2/DMRG.cpp:36-452). The
 * constructor builds the random initial MPS and all renormalized operators on the GPU. */
int c2g_dmrg_create(c2g_problem* p, c2g_scheme* s, const int* occupancies, c2g_dmrg** out);
/* DMRG(Prob, OptScheme, makechkpt, tmpfolder, occupancies) (CheMPS2/DMRG.cpp:37-158) with
 * checkpoints: makechkpt != 0 loads CheMPS2_MPS<state>.c2g from the working directory when
 * it exists and writes it after every sweep (CheMPS2/DMRGmpsio.cpp). */
int c2g_dmrg_create_chkpt(c2g_problem* p, c2g_scheme* s, int makechkpt, const int* occupancies, c2g_dmrg** out);
/* 1 when the MPS was loaded from a checkpoint file (the reference's loadedMPS). */
int c2g_dmrg_loaded_mps(const c2g_dmrg* d, int* loaded);
/* DMRG::deleteStoredMPS (CheMPS2/DMRGmpsio.cpp:164-173): removes the checkpoint files. */
int c2g_dmrg_delete_stored_mps(c2g_dmrg* d);
int c2g_dmrg_destroy(c2g_dmrg* d);
int c2g_dmrg_solve(c2g_dmrg* d, double* energy);            /* DMRG::Solve    */
int c2g_dmrg_presolve(c2g_dmrg* d);                         /* DMRG::PreSolve */
int c2g_dmrg_set_verbose(c2g_dmrg* d, int verbose);
/* Arithmetic of the Heff matvecs: 0 FP64 (default, the reference's); 1 mixed (FP32
 * matvecs inside Davidson down to residual mixed_tol, then FP64 refinement to the
 * instruction's tolerance); 2 mixed as 1 with the reduced-precision matvecs' large blocks
 * on the tensor cores (split-BF16 three-term products, FP32 accumulation). No counterpart
 * in the reference. The `precision` argument of the matvec entry points below takes the
 * matching codes for one matvec: 0 FP64, 1 FP32, 2 tensor cores. */
int c2g_dmrg_set_precision(c2g_dmrg* d, int mode, double mixed_tol);
int c2g_dmrg_num_mps_var(const c2g_dmrg* d, int* n);        /* DMRG::get_num_mps_var */
int c2g_dmrg_max_discarded_weight(const c2g_dmrg* d, double* w);
/* One two-site step (DMRG::solve_site, CheMPS2/DMRG.cpp:404-452) and one operator update
 * (DMRG::updateMovingRight / updateMovingLeft, CheMPS2/DMRGoperators.cpp:243-908). */
int c2g_dmrg_solve_site(c2g_dmrg* d, int index, double dvdson_rtol, double noise_level, int D, int moving_right,
                        int change, double* energy);
int c2g_dmrg_update(c2g_dmrg* d, int index, int moving_right);
/* Statistics, in this order: n_matvec, n_davidson, t_join, t_solve, t_split, t_update,
 * t_matvec, t_compile, matvec_flops, matvec_bytes, last_energy, n_matvec_fp32, t_upload
 * (seconds, flops, bytes). */
#define C2G_NUM_STATS 13
int c2g_dmrg_stats(const c2g_dmrg* d, double* out, int n);
int c2g_dmrg_reset_stats(c2g_dmrg* d);
/* Heff applications at sites (index, index + 1) on the current MPS (CheMPS2/Heff.cpp:43-248):
 * `steps` timed applications after `warmup` untimed ones, CUDA-event timed on the DMRG's
 * stream. With flush_bytes > 0 a buffer of that size is overwritten before each timed
 * application, outside the timed interval, so that the operators come from HBM. Returns
 * milliseconds per application, the ledger flops and bytes of one application and the
 * number of kernels launched in the timed region. No counterpart in the reference. */
int c2g_dmrg_bench_heff(c2g_dmrg* d, int index, int warmup, int steps, long long flush_bytes, int precision,
                        double* ms_per_matvec, double* flops, double* bytes, long long* launches);

/* Effective Hamiltonian on host buffers (the path of CheMPS2/Heff.cpp:43-315 with the
 * copies in and out included): n must equal the size of the two-site object at sites
 * (index, index + 1) (c2g_dmrg_sobject_size). y = Heff x in the symmetric convention
 * (CheMPS2/Sobject.cpp:624-650); diag (nullable) receives the diagonal of Heff. With
 * join_into_x != 0, x is first overwritten by the joined current two-site object. */
int c2g_dmrg_sobject_size(const c2g_dmrg* d, int index, int64_t* n);
int c2g_dmrg_heff_apply(c2g_dmrg* d, int index, int join_into_x, double* x, double* y, double* diag, int64_t n);
/* As c2g_dmrg_heff_apply with the matvec in FP32 arithmetic (operands converted on load,
 * lane sums in FP32, the output in FP64). No counterpart in the reference. */
int c2g_dmrg_heff_apply_fp32(c2g_dmrg* d, int index, double* x, double* y, int64_t n);
/* As c2g_dmrg_heff_apply (no join, no diagonal) with the matvec arithmetic chosen by
 * `precision`: 0 FP64, 1 FP32, 2 the large blocks on the tensor cores (split-BF16
 * three-term products, FP32 accumulation) and the rest in FP32. No counterpart in the
 * reference. */
int c2g_dmrg_heff_apply_precision(c2g_dmrg* d, int index, double* x, double* y, int64_t n, int precision);
/* DMRG::activateExcitations (CheMPS2/DMRG.cpp:464-473): allow up to max_exc stored states. */
int c2g_dmrg_activate_excitations(c2g_dmrg* d, int max_exc);
/* DMRG::newExcitation (CheMPS2/DMRG.cpp:475-505): store the current state; the next
 * c2g_dmrg_solve targets the next state with the stored ones shifted up by eshift. */
int c2g_dmrg_new_excitation(c2g_dmrg* d, double eshift);
/* DMRG::calc2DMandCorrelations (CheMPS2/DMRGtechnics.cpp:40-120; the 2-RDM part): the
 * spin-summed two-particle density matrices A and B of the current state
 * (CheMPS2/TwoDM.cpp:445-640). The state and the operators afterwards are those of a
 * finished right sweep, so c2g_dmrg_solve may continue. */
int c2g_dmrg_calc_2dm(c2g_dmrg* d);
/* The 2-RDMs as L^4 arrays, element (a,b,c,d) at a + L*(b + L*(c + L*d)); ham_order != 0:
 * Hamiltonian orbital order (TwoDM::getTwoDMA_HAM), else DMRG order (getTwoDMA_DMRG).
 * A or B may be NULL. */
int c2g_dmrg_get_2dm(const c2g_dmrg* d, int ham_order, double* A, double* B);
/* TwoDM::trace (= N(N-1)) and TwoDM::energy (Econst + 1/2 sum A h). */
int c2g_dmrg_2dm_trace_energy(const c2g_dmrg* d, double* trace, double* energy);
/* DMRG::getCorrelations (CheMPS2/Correlations.cpp), filled by c2g_dmrg_calc_2dm: L x L
 * tables (row + L*col) Cspin, Cdens, Cspinflip, Cdirad and the two-orbital mutual
 * information, and the L single-orbital entropies; ham_order as c2g_dmrg_get_2dm. Any
 * pointer may be NULL. */
int c2g_dmrg_get_correlations(const c2g_dmrg* d, int ham_order, double* cspin, double* cdens, double* cspinflip,
                              double* cdirad, double* mutinfo, double* entropy);
/* The DMRG object's own SyBookkeeper (current virtual dimensions after the sweeps so far,
 * SyBookkeeper::gCurrentDim, CheMPS2/SyBookkeeper.cpp:165,271-280) at boundary b, in the
 * row format of c2g_bookkeeper_sectors. */
int c2g_dmrg_sectors(const c2g_dmrg* d, int boundary, int* out, int cap, int* count);
/* TensorT::gStorage of the current MPS tensor of `site` (CheMPS2/include/chemps2/TensorT.h:50,
 * block order of CheMPS2/TensorT.cpp:38-110, each block column-major), copied to `out`;
 * *n receives its length (query with cap = 0). */
int c2g_dmrg_get_mps(const c2g_dmrg* d, int site, double* out, int64_t cap, int64_t* n);
/* The coefficient of one determinant in the current MPS (DMRG::getFCIcoefficient,
 * CheMPS2/DMRGtechnics.cpp:341-470): alpha[h] and beta[h] in {0, 1} are the occupations
 * of the L Hamiltonian orbitals; *coeff is 0 when the determinant lies outside the
 * targeted (N, 2S, irrep) sector. */
int c2g_dmrg_fci_coefficient(const c2g_dmrg* d, const int* alpha, const int* beta, double* coeff);
/* The energy of every two-site step the sweeps of c2g_dmrg_solve have run, in order (the
 * reference prints them in DMRG::sweepleft / sweepright, CheMPS2/DMRG.cpp:335-402, and
 * keeps only their minimum). *count receives the number of steps; up to cap of them are
 * written to out (which may be NULL). */
int c2g_dmrg_step_energies(const c2g_dmrg* d, double* out, int cap, int* count);
/* No counterpart in the reference. For callers that cannot allocate device memory while
 * they run: a host program whose device memory is all handed out by its own allocator
 * (a fixed budget reserved at start-up), or one that must not call cudaMalloc / cudaFree
 * because those calls can synchronise the device and stall the work of other streams.
 * As c2g_dmrg_heff_apply (FP64, no join, no diagonal) with no allocation at all: x and y
 * are staged through one file-scope device array of 2 M doubles (16 MiB, held by every
 * GPU that loads the library until the process exits), so n may be at most 1 048 544.
 * The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture. y's half of
 * the array is cleared on every call. The Heff program at `index` must already exist for
 * the current state (a c2g_dmrg_heff_apply call there); otherwise, or when n differs from
 * the two-site object's size or exceeds the limit, C2G_ERR_INVALID. Every call shares
 * the array: calls that overlap on the GPU (several threads or DMRG objects at once)
 * race; each call synchronises before it returns, so calls made one after another are
 * safe. */
int c2g_dmrg_heff_apply_noalloc(c2g_dmrg* d, int index, const double* x, double* y, int64_t n);
/* No counterpart in the reference (its Heff::makeHeff, CheMPS2/Heff.cpp:43-248, works on
 * host arrays): y_dev = Heff x_dev at sites (index, index + 1) on the caller's device
 * buffers of n doubles, FP64 (precision 0) or FP32 arithmetic (precision 1), for the
 * current MPS and operators. `stream` (a cudaStream_t, or NULL): the call is ordered after
 * the work already issued on it and that stream waits for y_dev, without a host
 * synchronisation; with NULL the call returns when y_dev is written. */
int c2g_dmrg_heff_apply_device(c2g_dmrg* d, int index, const double* x_dev, double* y_dev, int64_t n, int precision,
                               void* stream);

/* ---- Batches of independent problems (no counterpart in the reference, whose callers
 * loop over problems with one CheMPS2::DMRG each, e.g. CheMPS2/CASSCFnewtonraphson.cpp:
 * 242-245) */
/* CheMPS2::SolveBatch: solves problems[i] with schemes[i], i < n, each with its own DMRG
 * object, CUDA stream and random start (the one srand(seeds[i]) gives). At most `workers`
 * problems run at once on host threads sharing the current device (workers <= 1: one after
 * another). Every problem is attempted; per-problem outputs (any may be NULL): energies
 * (Solve()), matvecs (Heff applications), seconds (wall clock of construction and Solve),
 * statuses (C2G_OK or the error code of that problem), stats (n x C2G_NUM_STATS, the
 * layout of c2g_dmrg_stats). Returns C2G_OK when all were solved, else the first failed
 * problem's code (c2g_last_error names it). */
int c2g_batch_solve(int n, c2g_problem* const* problems, c2g_scheme* const* schemes, const unsigned int* seeds,
                    int workers, double* energies, long long* matvecs, double* seconds, int* statuses,
                    double* stats);
/* The FP64 eigensolver of the truncation step (CheMPS2/Sobject.cpp:418, where the
 * reference calls dgesdd on the sector matrices; here the Gram matrices are diagonalised)
 * for matrices of order 1..128, exposed for testing: `count` symmetric matrices of orders
 * n[i], column-major and concatenated in `mats`; evals receives each matrix's eigenvalues
 * in ascending order (concatenated), evecs its eigenvectors in descending order of the
 * eigenvalue, each column signed so that its largest-magnitude entry is positive. */
int c2g_truncation_eig(int count, const int* n, const double* mats, double* evals, double* evecs);
/* The Rayleigh-Ritz eigensolver of the Davidson solver (CheMPS2/Davidson.cpp:242-276,
 * where the reference calls dsyev), exposed for testing: the symmetric n x n matrix `mat`
 * (column-major, n <= 32) on the device, `reps` times, CUDA-event timed (*us_per_call,
 * nullable). Eigenvalues ascending in evals, eigenvectors in the columns of evecs (n x n).
 * warm != 0: on entry evecs holds ((n-1) x (n-1), column-major) the eigenvectors of the
 * leading (n-1) x (n-1) block, as in a Davidson expansion step. */
int c2g_rayleigh_ritz_eig(int n, const double* mat, int warm, double* evals, double* evecs, int reps,
                          double* us_per_call);
/* No counterpart in the reference (a diagnostic): the free memory of `device` (< 0: the
 * calling thread's current device; cudaMemGetInfo) and the bytes in use from that
 * device's default stream-ordered pool (cudaMemPoolAttrUsedMemCurrent), where this
 * library's stream-ordered allocations live. */
int c2g_device_memory_info(int device, int64_t* free_bytes, int64_t* pool_used_bytes);
/* The first n draws of the private random generator a batch member seeded with `seed`
 * uses (equal to srand(seed); rand() of the GNU C library). No GPU needed. */
int c2g_host_rand_sample(unsigned int seed, int n, int* out);

#ifdef __cplusplus
}
#endif

#endif /* CHEMPS2_GB300_H */
