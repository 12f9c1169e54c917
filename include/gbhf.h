/* libgbhf -- GB300-native restricted Hartree-Fock hot path, C ABI.
 *
 * Drop-in replacement for the numerical core of felipeZ/Haskell-abinitio's
 * Science.QuantumChemistry modules.  Every entry point below names the
 * reference function it replaces (paths relative to the reference checkout).
 *
 * Conventions (identical to the reference's Repa `U` arrays):
 *   - all arrays are host memory, contiguous float64, owned by the caller;
 *     the library copies in and out and keeps no pointer after a call;
 *   - a "flat" symmetric matrix is its row-major upper triangle, element
 *     (i,j), i<=j, at index i*N - i*(i-1)/2 + (j-i)   (indexDIM2toFlat,
 *     NumericalTools/LinearAlgebra.hs:250-253); length N(N+1)/2;
 *   - a square matrix is N*N row-major (DIM2); eigenvectors are columns,
 *     eigenvalues ascending (eigenSolve, NumericalTools/EigenValues.hs:29-31);
 *   - coordinates are in bohr.
 * Every call returns a gbhf_status; gbhf_last_error() gives the message.
 * One context per host thread; calls on a context are serialised.  The
 * context owns its device memory and one CUDA stream on the chosen device.
 * There is no CPU fallback: without a usable GPU gbhf_create fails.
 */
#ifndef GBHF_H
#define GBHF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbhf_ctx gbhf_ctx;

typedef enum {
  GBHF_OK = 0,
  GBHF_ERR_BAD_INPUT = 1,      /* mirrors HSFOCKException (Error.hs:19-24) */
  GBHF_ERR_NOT_CONVERGED = 2,  /* mirrors error "SCF maxium steps exceeded" (HartreeFock.hs:123) */
  GBHF_ERR_SINGULAR = 3,       /* DIIS system singular after dropping every vector (DIIS.hs:79) */
  GBHF_ERR_CUDA = 4,           /* a CUDA runtime call failed */
  GBHF_ERR_DEVICE_TIMEOUT = 5, /* a bounded device loop gave up (Jacobi sweeps, grid barrier) */
  GBHF_ERR_NO_DEVICE = 6,      /* no usable GPU */
  GBHF_ERR_UNSUPPORTED = 7,    /* input outside what the kernels implement (e.g. f functions, incomplete shells) */
  GBHF_ERR_INDEX = 8           /* the reference's bounds-checked lookup would fail (Harris guess, HartreeFock.hs:143-146) */
} gbhf_status;

/* Numerics / driver presets. */
typedef enum {
  GBHF_MODE_REFERENCE = 0, /* the reference's numerics: tabulated Boys grid + Taylor (TableBoys.hs:45-69),
                              primitive screening at 1e-8 (IntegralsEvaluation.hs:308-315),
                              S_ii = 1 (IntegralsEvaluation.hs:183-184), stored canonical ERIs */
  GBHF_MODE_EXACT = 1      /* exact Boys function, contracted Schwarz screening, direct J/K */
} gbhf_mode;

typedef enum {
  GBHF_PREC_FP64 = 0,  /* every ERI in FP64 */
  GBHF_PREC_MIXED = 1  /* ERIs with Schwarz bound below mixed_cutoff in FP32; Fock accumulation,
                          DIIS and the eigen-solve always FP64 */
} gbhf_precision;

/* GBHF_GUESS_SAD (superposition of atomic densities: block-diagonal densities of
 * spherically averaged free atoms) has no counterpart in the reference, which
 * offers the Harris functional and the core Hamiltonian
 * (HartreeFock/HartreeFock.hs:128-149).  GBHF_GUESS_DENSITY restarts from the
 * density given to gbhf_set_guess_density (a checkpoint of an earlier SCF). */
typedef enum { GBHF_GUESS_HARRIS = 0, GBHF_GUESS_CORE = 1, GBHF_GUESS_SAD = 2, GBHF_GUESS_DENSITY = 3 } gbhf_guess;

/* SCF options.  gbhf_scf_opts_reference() fills the reference's constants
 * (HartreeFock.hs:78,81,87,113; DIIS.hs:58). */
typedef struct {
  int mode;              /* gbhf_mode */
  int precision;         /* gbhf_precision (direct J/K only) */
  int guess;             /* gbhf_guess */
  int diis_size;         /* vectors in one extrapolation, current included (reference: 5) */
  int max_iter;          /* reference: 30 */
  int incremental;       /* 1: rebuild only G(D_n - D_(n-1)) between full builds */
  int full_rebuild_every;/* incremental mode: full rebuild period (0 = never) */
  int final_fp64;        /* mixed mode: once converged in mixed precision, continue with full FP64
                            builds until converged again */
  int ref_stop_rule;     /* 1: stop when step>0 and max|e| < conv_error, E from F_DIIS and the new D
                                (HartreeFock.hs:112-114); 0: stop on |dE| and RMS(dD) */
  double conv_error;     /* reference: 1e-7 */
  double conv_energy;    /* |dE| threshold (baseline 1e-10) */
  double conv_density;   /* RMS(dD) threshold (baseline 1e-8) */
  double diis_start;     /* DIIS switches on once max|e| < diis_start (reference 0.1) */
  double schwarz_cutoff; /* contracted Schwarz screening (baseline 1e-12) */
  double mixed_cutoff;   /* FP32 for quartets with bound below this (baseline 1e-4) */
  double charge;         /* total charge; n_occ = floor((sum Z - charge)/2) (HartreeFock.hs:75-76) */
  double grad_mixed_cutoff; /* gbhf_scf_batch gradients, mixed precision: FP32 derivative integrals for
                               quartets with bound Q_ab Q_cd max(w)^2 below this (0: mixed_cutoff) */
  int autotune;          /* 1: unless this context already holds tuned task budgets, run gbhf_autotune
                            on the call's basis before the first step (J/K, with the starting density)
                            and, in gbhf_scf_batch, before the gradients (with their density) */
} gbhf_scf_opts;

/* Result buffers are caller-owned; any pointer may be NULL.  Sizes:
 * fock_flat/density_flat N(N+1)/2, coeff N*N, orb_energies N. */
typedef struct {
  double energy;
  int iterations;
  int converged;
  int n_occupied;
  double nuclear_repulsion;
  double* fock_flat;
  double* coeff;
  double* density_flat;
  double* orb_energies;
  /* statistics of the last call */
  double eri_quartets;       /* contracted shell quartets computed, summed over builds */
  double eri_fn_quartets;    /* contracted basis-function quartets computed, summed over builds */
  double eri_prim_quartets;  /* primitive quartets computed, summed over builds */
  double eri_fp32_fraction;  /* share of primitive quartets evaluated in FP32 */
  double fock_builds;
} gbhf_result;

/* ----------------------------------------------------------- context ---- */
gbhf_status gbhf_create(gbhf_ctx** ctx, int device);
gbhf_status gbhf_destroy(gbhf_ctx* ctx);
const char* gbhf_last_error(gbhf_ctx* ctx);
int gbhf_version(void);

/* [AtomData] flattened to structure-of-arrays (GlobalTypes.hs:92-105,
 * replaces the atom/basis half of initializeAtoms, HsFock/Initialize.hs:30-41):
 * n_cgf contracted Gaussians, CGF k on atom cgf_atom[k] with Cartesian
 * exponents cgf_lxyz[3k..3k+2] and cgf_nprim[k] primitives whose
 * (coefficient, exponent) follow in prim_coef/prim_exp (coefficients already
 * carry normCoeff, NormalizeBasis.hs:52-59).  s, p and d functions; the direct
 * J/K and gradient kernels group them into shells (components in createCGF
 * order x,y,z and xx,xy,xz,yy,yz,zz, shared exponents, proportional
 * coefficients) and return GBHF_ERR_UNSUPPORTED for CGFs that form no shell. */
gbhf_status gbhf_set_basis(gbhf_ctx* ctx, int n_atoms, const double* xyz_bohr, const double* charges,
                           int n_cgf, const int* cgf_atom, const int* cgf_lxyz, const int* cgf_nprim,
                           const double* prim_coef, const double* prim_exp);

/* generateGridBoys 0.1 (NumericalTools/TableBoys.hs:58-63): the caller's
 * 15 x 1001 grid, grid[m*1001+i] = boysF m (0.1 i).  Used by GBHF_MODE_REFERENCE;
 * without it that mode fails with GBHF_ERR_BAD_INPUT. */
gbhf_status gbhf_set_boys_grid(gbhf_ctx* ctx, const double* grid);

/* generateGridBoys 0.1 computed on the device (boysF, Boys.hs:54-66: erf for
 * m = 0, Kummer's integral by 256-point Gauss-Legendre for m >= 1) and made
 * the context's reference grid; grid_out (15 x 1001, may be NULL) receives it. */
gbhf_status gbhf_generate_boys_grid(gbhf_ctx* ctx, double* grid_out);

/* Boys values F_m(x), m = 0..m_max, for n points: mode EXACT uses the device
 * table, mode REFERENCE boysTaylor on the uploaded grid.  out[i*(m_max+1)+m]. */
gbhf_status gbhf_boys(gbhf_ctx* ctx, int mode, int m_max, int n, const double* x, double* out);

/* mtxOverlap (Integrals/IntegralsEvaluation.hs:169-177). */
gbhf_status gbhf_overlap(gbhf_ctx* ctx, int mode, double* s_flat);
/* hcore (Integrals/IntegralsEvaluation.hs:227-240). */
gbhf_status gbhf_hcore(gbhf_ctx* ctx, int mode, double* h_flat);

/* calcIntegrals (HartreeFock/HartreeFock.hs:166-181): every unique contracted
 * ERI in the reference's canonical key order; length (P(P+1)/2), P = N(N+1)/2. */
int64_t gbhf_eri_canonical_length(int n_basis);
gbhf_status gbhf_eri_canonical(gbhf_ctx* ctx, int mode, double* eri, int64_t length);

/* fock (HartreeFock/HartreeFock.hs:213-241): F = H + G(D).  Mode REFERENCE
 * contracts the stored canonical ERIs (calcGmatrix); mode EXACT runs the
 * direct J/K kernels at the given precision with Schwarz screening. */
gbhf_status gbhf_fock(gbhf_ctx* ctx, int mode, int precision, double schwarz_cutoff, double mixed_cutoff,
                      const double* h_flat, const double* d_flat, double* f_flat);

/* symmOrtho (HartreeFock/BasisOrthogonalization.hs:26-34): X = U s^-1/2 U^T of
 * the square overlap matrix. */
gbhf_status gbhf_symm_ortho(gbhf_ctx* ctx, int n, const double* s_square, double* x_square);

/* eigenSolve (NumericalTools/EigenValues.hs:29-31): symmetric eigenpairs,
 * ascending, eigenvectors as columns of the N*N row-major output. */
gbhf_status gbhf_eigen_solve(gbhf_ctx* ctx, int n, const double* a_square, double* evals, double* evecs);

/* Eigen-solve that allocates nothing.  No counterpart in the reference: it
 * exists for callers that must not allocate device memory during the call,
 * e.g. code running inside another framework's custom-call hook, where that
 * framework owns every buffer.  d_a (n x n, row-major, symmetric), d_evals (n)
 * and d_evecs (n x n, eigenvectors as columns, eigenvalues ascending) are
 * device pointers owned by the caller; `stream` is a cudaStream_t (NULL =
 * the default stream) and the call returns after that stream has finished the
 * work.  The solver's working memory is one static device array sized for
 * n <= GBHF_NOALLOC_EIGEN_MAX_N (about 1.5 MiB, held by every GPU that loads
 * the library until the process exits); larger n returns GBHF_ERR_BAD_INPUT.
 * The first call on a device resolves that array's device address (in the
 * CUDA context current then) and the launch geometry; make that first call
 * before any stream capture.  After a cudaDeviceReset of that device the
 * resolved address is stale: do not call this entry point on it again.  All
 * calls share the array, so calls that overlap on the GPU (other host threads
 * or streams) race: serialise them. */
#define GBHF_NOALLOC_EIGEN_MAX_N 256
gbhf_status gbhf_eigen_solve_noalloc(int n, const double* d_a, double* d_evals, double* d_evecs, void* stream);

/* Superposition-of-atomic-densities starting density of the context's basis
 * (flat upper triangle, N(N+1)/2).  No counterpart in the reference (its guesses
 * are harrisFunctional and the core Hamiltonian, HartreeFock/HartreeFock.hs:
 * 128-149); it is the starting density of gbhf_scf with GBHF_GUESS_SAD. */
gbhf_status gbhf_sad_density(gbhf_ctx* ctx, double* density_flat);

/* Checkpoint / restart and structured logging of the SCF (the reference prints
 * `show` dumps of its matrices every step, HartreeFock.hs:116-117, and has no
 * restart).  gbhf_set_guess_density stores a starting density (flat upper
 * triangle of the current basis, e.g. density_flat of an earlier gbhf_scf) for
 * the next gbhf_scf with guess = GBHF_GUESS_DENSITY; a new basis clears it.
 * gbhf_scf_trace copies the per-step records of the last gbhf_scf,
 * GBHF_SCF_TRACE_FIELDS doubles each: step, energy, energy change, RMS density
 * change, max |DIIS error|, stored DIIS vectors, phase (0 FP64, 1 mixed, 2 the
 * FP64 phase after a mixed one), milliseconds of the step (device time between
 * stream events at its start and end); *n_records = steps. */
#define GBHF_SCF_TRACE_FIELDS 8

/* Open-shell (unrestricted) SCF for multiplicity 2S+1: the reference parses a
 * multiplicity (--multi, Main.hs:55; OptsCheck.hs:31) but always runs the
 * closed-shell scfHF.  n_alpha - n_beta = multiplicity - 1 electrons of the
 * molecule (charge from opts); exact mode (direct J/K), FP64 or mixed builds,
 * core or SAD start; DIIS on both spins with one set of coefficients.  s2 is
 * <S^2> of the UHF determinant.  Output arrays may be NULL. */
typedef struct {
  double energy;
  int iterations;
  int converged;
  int n_alpha, n_beta;
  double s2;
  double* density_alpha_flat;   /* N(N+1)/2: D_a = C_a,occ C_a,occ^T */
  double* density_beta_flat;
  double* orb_energies_alpha;   /* N */
  double* orb_energies_beta;
} gbhf_uhf_result;
gbhf_status gbhf_scf_uhf(gbhf_ctx* ctx, const gbhf_scf_opts* opts, int multiplicity, gbhf_uhf_result* result);
gbhf_status gbhf_set_guess_density(gbhf_ctx* ctx, const double* density_flat);
gbhf_status gbhf_scf_trace(gbhf_ctx* ctx, double* out, int max_records, int* n_records);

/* diagonalHF (HartreeFock/HartreeFock.hs:263-273): X^T F X, eigen-solve,
 * C = X C', density P = 2 C_occ C_occ^T (calcDensity, :195-208). */
gbhf_status gbhf_diagonal_hf(gbhf_ctx* ctx, int n, const double* f_flat, const double* x_square, int n_occupied,
                             double* coeff, double* density_flat, double* orb_energies);

/* calcErrorMtx (HartreeFock/DIIS.hs:119-132): e = X^T (F D S - S D F) X. */
gbhf_status gbhf_diis_error(gbhf_ctx* ctx, int n, const double* f_flat, const double* s_flat, const double* d_flat,
                            const double* x_square, double* e_square);

/* diis (HartreeFock/DIIS.hs:70-88): extrapolated Fock from the current pair
 * (e, F) followed by n_hist stored pairs, newest first.  On a singular system
 * the oldest stored pair is dropped and the solve retried; *n_used returns how
 * many stored pairs remained. */
gbhf_status gbhf_diis_extrapolate(gbhf_ctx* ctx, int n, int n_hist, const double* errors_square,
                                  const double* focks_flat, double* f_out_flat, int* n_used);

/* gaussElem (NumericalTools/GaussElimination.hs:42-98): unpivoted Gauss
 * elimination of an m x m system; returns GBHF_ERR_SINGULAR where the
 * reference returns Nothing. */
gbhf_status gbhf_gauss_elem(gbhf_ctx* ctx, int m, const double* a, const double* b, double* x);

/* scfHF (HartreeFock/HartreeFock.hs:70-123) on the current basis. */
void gbhf_scf_opts_reference(gbhf_scf_opts* opts);
void gbhf_scf_opts_baseline(gbhf_scf_opts* opts);
gbhf_status gbhf_scf(gbhf_ctx* ctx, const gbhf_scf_opts* opts, gbhf_result* result);

/* Analytic RHF nuclear gradient (energyGradient, HartreeFock/Derivatives.hs:40-48,
 * which is dead code in the reference): dE/dR for density D and energy-weighted
 * density W (both flat), grad[3*atom + axis] in hartree/bohr.  With D and W
 * NULL the last SCF of this basis is used.  Two-electron terms are screened at
 * Q_ab Q_cd max(w)^2 < schwarz_cutoff (w: shell-block maxima of |D|); with
 * GBHF_PREC_MIXED the quartets whose bound is below 1e-4 use FP32 derivative
 * integrals. */
gbhf_status gbhf_gradient(gbhf_ctx* ctx, int precision, double schwarz_cutoff, const double* d_flat,
                          const double* w_flat, double* grad);

/* Analytic unrestricted (open-shell) gradient, the backward call of
 * gbhf_scf_uhf; no counterpart in the reference, which has neither an
 * open-shell driver (--multi is parsed and ignored, Main.hs:55) nor a working
 * gradient (Derivatives.hs:40-48).  da_flat, db_flat: alpha and beta densities
 * D_s = C_s,occ C_s,occ^T; w_flat: W = sum_s C_s,occ eps_s C_s,occ^T (all flat,
 * N(N+1)/2); all three NULL: the last converged gbhf_scf_uhf of this basis.
 * grad[3*atom + axis] in hartree/bohr; screening and precision as gbhf_gradient. */
gbhf_status gbhf_gradient_uhf(gbhf_ctx* ctx, int precision, double schwarz_cutoff, const double* da_flat,
                              const double* db_flat, const double* w_flat, double* grad);

/* Many molecules in one call (batched SCF, no counterpart in the reference,
 * whose scfHF takes one molecule): molecule k owns atoms
 * [atom_off[k], atom_off[k+1]) and CGFs [cgf_off[k], cgf_off[k+1]) of the
 * concatenated arrays.  energies[k] and converged[k] are written; grads (3 x
 * total atoms, may be NULL) receives analytic gradients. */
gbhf_status gbhf_scf_batch(gbhf_ctx* ctx, int n_mol, const int* atom_off, const int* cgf_off,
                           const double* xyz_bohr, const double* charges, const int* cgf_atom,
                           const int* cgf_lxyz, const int* cgf_nprim, const double* prim_coef,
                           const double* prim_exp, const gbhf_scf_opts* opts, double* energies,
                           int* iterations, int* converged, double* grads);

/* Task budgets of the direct builds (no counterpart in the reference).  A
 * class's task list splits its work into tasks of (bra pair, up to
 * kets_per_task kets, a range of bra primitives) with at most
 * prim_quartets_per_lane primitive quartets per lane and task.  which = 0:
 * J/K, 21 quartet classes in the order of gbhf_profile_classes; which = 1:
 * gradient, 36 (bra class, ket class) pairs, pair classes ss, ps, pp, ds, dp,
 * dd, bra-major.  budgets[2k] = prim_quartets_per_lane (1..65535),
 * budgets[2k+1] = kets_per_task (1..32; the lane-per-ket classes take 32);
 * n >= 2 x classes.  gbhf_set_task_budgets with budgets == NULL restores the
 * defaults. */
gbhf_status gbhf_get_task_budgets(gbhf_ctx* ctx, int which, int* budgets, int n);
gbhf_status gbhf_set_task_budgets(gbhf_ctx* ctx, int which, const int* budgets, int n);
/* Autotuner: times every class's launch of the J/K (which 0) or two-electron
 * gradient (which 1) build on the current basis under candidate budgets
 * (primitive quartets per lane x 1/4 .. 4, then kets per task 1, 2, 4, 8 for
 * the warp-per-quartet d classes), each candidate the minimum of `repeats`
 * builds with the density density_flat (N(N+1)/2; NULL: the SAD guess), and
 * keeps per class the fastest when it beats the current budget by more than
 * 3%.  class_ms (may be NULL; 2 x classes) receives per class the
 * milliseconds before and after. */
gbhf_status gbhf_autotune(gbhf_ctx* ctx, int which, int precision, double schwarz_cutoff, double mixed_cutoff,
                          const double* density_flat, int repeats, double* class_ms);

/* Measurement hooks: device-time of the J/K kernels since the last reset
 * (CUDA events on the context stream), launches issued by the library, and
 * per-kernel-class statistics.  stats[0..19]: J/K milliseconds FP64, FP32,
 * primitive quartets FP64, FP32, shell quartets, function quartets,
 * total library kernel launches, dense linear-algebra milliseconds, then
 * host wall milliseconds of the SCF phases (setup, Fock, DIIS,
 * diagonalisation, other), Jacobi sweeps and Jacobi calls, milliseconds of
 * the batched gradients, steps of the last batched SCF, purification steps
 * and calls (single-molecule density builds), host milliseconds of the
 * shell-pair setup. */
gbhf_status gbhf_profile_reset(gbhf_ctx* ctx, int enable_events);
gbhf_status gbhf_profile_read(gbhf_ctx* ctx, double* stats, int n_stats);
/* Per ERI class and precision (FP64, FP32) since the last reset:
 * out[(class*2+prec)*4 + k], k = shell quartets, function quartets, primitive
 * quartets, kernel milliseconds; 21 classes (168 values): (ss|ss) (ps|ss)
 * (ps|ps) (pp|ss) (pp|ps) (pp|pp), then (ds|ss) (ds|ps) (ds|pp) (ds|ds)
 * (dp|ss) (dp|ps) (dp|pp) (dp|ds) (dp|dp) (dd|ss) (dd|ps) (dd|pp) (dd|ds)
 * (dd|dp) (dd|dd). */
gbhf_status gbhf_profile_classes(gbhf_ctx* ctx, double* out168);
/* CUDA events on the context stream (slots 0..7) and the time between two. */
gbhf_status gbhf_event_record(gbhf_ctx* ctx, int slot);
gbhf_status gbhf_event_elapsed(gbhf_ctx* ctx, int slot_start, int slot_end, double* ms);
/* Overwrite a device buffer larger than L2 (256 MiB) on the context stream. */
gbhf_status gbhf_flush_l2(gbhf_ctx* ctx);
/* Measured FMA throughput of this GPU's CUDA cores (TFLOP/s, 2 flops per
 * FMA) for precision GBHF_PREC_FP64 or GBHF_PREC_MIXED (= FP32). */
gbhf_status gbhf_peak_flops(gbhf_ctx* ctx, int precision, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* GBHF_H */
