/*
 * hpgpu.h - C ABI of the GB300 partitioning library (libhpgpu.so).
 *
 * The library runs horton-part's iterative stockholder loop on one GPU:
 * pro-atom evaluation on the Becke-weighted molecular grid, promolecule and
 * at_weights ratio, weighted per-atom/per-shell moment integrals and the
 * per-atom (MBIS, GISA, aLISA) or global (gLISA) parameter update, until the
 * outer change drops below the threshold.
 *
 * Reference entry points this ABI replaces (paths inside horton-part's
 * src/horton_part):
 *   hp_job_create   <- WPart/AbstractISAWPart/GaussianISAWPart/LinearISAWPart/
 *                      GlobalLinearISAWPart constructors: core/base.py:416-488,
 *                      core/iterstock.py:64-114, gisa.py:114-160,
 *                      alisa.py:1205-1256, glisa.py:58-117
 *   hp_job_run      <- do_partitioning: core/iterstock.py:159-193 (MBIS, GISA,
 *                      aLISA), glisa.py:248-281 (gLISA)
 *   hp_step         <- one pass of the outer loop body: core/iterstock.py:172-188
 *                      (_update_propars + _update_entropy + compute_change);
 *                      for gLISA one solver iteration, glisa.py:748-798
 *   hp_job_info_get / hp_job_results_get
 *                   <- part.cache["niter"/"change"/"charges"/"propars"/
 *                      "history_*"/"promoldens"/"at_weights_{i}"],
 *                      core/iterstock.py:48-58, mbis.py:347-362
 *
 * Conventions
 *   - All pointers in descriptors and result structs are HOST pointers; the
 *     library copies inputs to the device in hp_job_create and copies results
 *     into caller-owned buffers in hp_job_results_get.
 *   - Every call returns an hp_status (0 = HP_OK). No C++ exception crosses
 *     the ABI. hp_last_error() returns a message for the calling thread.
 *   - A context is used by one host thread at a time. Jobs belong to the
 *     context that created them.
 *   - No CPU fallback: when no usable sm_103 device is present,
 *     hp_ctx_create fails with HP_ERR_CUDA.
 */
#ifndef HPGPU_H
#define HPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HPGPU_ABI_VERSION 4

typedef enum {
  HP_OK = 0,
  HP_ERR_INVALID = 1,       /* bad argument (reference: ValueError/TypeError) */
  HP_ERR_NO_MEMORY = 2,     /* device allocation failed or HBM budget exceeded */
  HP_ERR_NOT_CONVERGED = 3, /* reference: RuntimeError("Not converged!") */
  HP_ERR_NUMERIC = 4,       /* negative pro-atom density, singular Hessian,
                               failed line search (reference: RuntimeError) */
  HP_ERR_TIMEOUT = 5,       /* a bounded device wait ran out */
  HP_ERR_CUDA = 6,          /* CUDA runtime error or no usable device */
  HP_ERR_UNSUPPORTED = 7,   /* option not implemented on this path */
  HP_ERR_STATE = 8          /* call made in the wrong state */
} hp_status;

typedef enum {
  HP_SCHEME_MBIS = 0,  /* mbis.py  MBISWPart */
  HP_SCHEME_GISA = 1,  /* gisa.py  GaussianISAWPart */
  HP_SCHEME_LISA = 2,  /* alisa.py LinearISAWPart (aLISA) */
  HP_SCHEME_GLISA = 3, /* glisa.py GlobalLinearISAWPart (gLISA) */
  HP_SCHEME_NLIS = 4   /* nlis.py NLISWPart and gmbis.py GMBISWPart: shells
                          N n S^(3/n) exp(-S r^n) / (4 pi Gamma(3/n)), three
                          parameters (N, S, n) per shell in initial_propars,
                          n fixed (nlis.py:99-195); FP64 only */
} hp_scheme;

typedef enum {
  HP_SOLVER_DEFAULT = 0, /* MBIS fixed point; GISA QP; aLISA sc; gLISA newton */
  HP_SOLVER_SC = 1,      /* alisa.py:193-291, glisa.py:805-848 */
  HP_SOLVER_NEWTON = 2,  /* alisa.py:543-602, glisa.py:573-575 (exact Newton) */
  HP_SOLVER_M_NEWTON = 3,/* alisa.py:605-664, glisa.py:577-591 (line search) */
  HP_SOLVER_QP = 4,      /* gisa.py:348-421 (quadratic program) */
  HP_SOLVER_PNEWTON = 5, /* gLISA with non-negative populations: projected Newton on
                            the extended KL objective; reaches the optimum of the
                            reference's cvxopt solver (glisa.py:488-571), whose
                            package is not available */
  HP_SOLVER_QUASI_NEWTON = 6 /* aLISA: BFGS on the inverse Hessian with the
                            positivity line search (alisa.py:683-750 through
                            _solver_general_newton, mode "bfgs", :753-938) */
} hp_solver;

typedef enum {
  HP_PRECISION_FP64 = 0,  /* every step in FP64 */
  HP_PRECISION_MIXED = 1, /* MBIS, GISA, aLISA sc: FP32 evaluation, compensated
                             sums, FP64 updates and change test (optional
                             finish, see polish: float-float for MBIS, FP64 for
                             the basis schemes). gLISA Newton solvers:
                             float-float evaluation, Hessian on the tensor
                             cores (TF32) with an FP32 factor; with polish,
                             the step is refined against the exact product
                             in the finish. */
  HP_PRECISION_FF = 2     /* MBIS: every evaluation in float-float arithmetic
                             (about 48 significant bits) on the FP32 pipes,
                             FP64 updates and tests: FP64-class results */
} hp_precision;

/* Warning bits reported in hp_job_info.warnings (the reference logs these). */
#define HP_WARN_INNER_NOT_CONVERGED 1u /* mbis.py:162, alisa.py:289 */
#define HP_WARN_POPULATION 2u          /* utils.py:418-456 */
#define HP_WARN_NEGATIVE_PARS 4u       /* utils.py:459-488 */
#define HP_WARN_NOISE_FLOOR 8u         /* mixed precision stopped at its noise floor */

typedef struct hp_ctx hp_ctx;
typedef struct hp_job hp_job;

typedef struct {
  int32_t scheme;    /* hp_scheme */
  int32_t solver;    /* hp_solver */
  int32_t precision; /* hp_precision */
  int32_t grid_type; /* 2 or 3 (molecular grid); 1 (atom grids: MBIS, NLIS,
                        GISA, aLISA sc, gLISA) */
  int64_t natom;
  int64_t npoint;
  const double* coordinates;    /* natom x 3, bohr */
  const double* pseudo_numbers; /* natom */
  const double* points;         /* npoint x 3, row-major */
  const double* weights;        /* npoint */
  const double* density;        /* npoint */
  /* Shells. shell_offsets[natom+1] delimits each atom's shells.
   * MBIS: each shell has the parameter pair (N_k, S_k); shell_orders and
   *       shell_exponents are ignored.
   * NLIS: each shell has the triple (N_k, S_k, n_k), n_k fixed; shell_orders
   *       and shell_exponents are ignored.
   * Basis schemes: shell k has fixed order n_k and exponent alpha_k and one
   *       parameter (its population c_k). */
  const int32_t* shell_offsets;
  const double* shell_orders;
  const double* shell_exponents;
  /* Initial parameters: MBIS 2 per shell (N, S); NLIS 3 (N, S, n); basis
   * schemes 1 per shell.
   * For the basis schemes the library rescales them so that their sum is
   * the integrated density (gisa.py:85-86). */
  const double* initial_propars;
  double threshold;
  double inner_threshold; /* used as min(inner_threshold, threshold) */
  double density_cutoff;
  double negative_cutoff;
  double population_cutoff;
  double tau;             /* line-search start (m-newton) */
  int32_t maxiter;        /* outer iterations (gLISA: solver iterations) */
  int32_t inner_maxiter;  /* MBIS 2000, aLISA sc 100000, aLISA newton 10000 */
  int32_t linspace_size;  /* line-search trial count (m-newton) */
  int32_t polish;         /* mixed precision: 1 = finish in float-float (MBIS)
                             or FP64 (basis schemes) once the FP32-evaluated
                             outer change is within 100 x the threshold or has
                             stopped decreasing (its noise floor); 0 = stay in
                             FP32 to the threshold and stop with
                             HP_WARN_NOISE_FLOOR only at the floor. gLISA
                             with the tensor-core Hessian: 1 = refine the
                             Newton step once against the exact product H d
                             while the last outer change is within 100 x the
                             threshold; 0 = never */
  int32_t nrad;           /* grid_type 1: radial nodes over all atom grids */
  /* grid_type 1 (atom grids, the reference's default; base.py:619-628,
   * mbis.py:174-187): atom a owns the radial shells [radial_offsets[a],
   * radial_offsets[a+1]) of the concatenated radial grids (nodes
   * radial_points, weights radial_weights), and shell s owns the consecutive
   * grid points [shell_point_offsets[s], shell_point_offsets[s+1]) with
   * angular weights point_sphere_weights (Lebedev weight / 4 pi, summing to
   * 1 over a shell). NULL for grid_type 2/3. */
  const int32_t* radial_offsets;      /* natom + 1 */
  const int64_t* shell_point_offsets; /* nrad + 1 */
  const double* point_sphere_weights; /* npoint */
  const double* radial_points;        /* nrad */
  const double* radial_weights;       /* nrad */
} hp_job_desc;

typedef struct {
  int64_t natom;
  int64_t npoint;
  int64_t nparam;
  int64_t niter;        /* outer iterations done */
  int64_t inner_iterations; /* sum of inner iterations over atoms and outer iterations */
  double change;        /* last outer change */
  int32_t done;         /* 1 when converged, hit maxiter or failed */
  int32_t status;       /* hp_status of the job (HP_OK unless it failed) */
  uint32_t warnings;    /* HP_WARN_* bits */
  int32_t converged;    /* 1 when the change fell below the threshold */
  int64_t device_bytes; /* device memory held by the job */
  double point_atom_evals; /* pro-atom evaluations done so far (sum over passes) */
  int32_t polish_iterations; /* mixed precision: FP64 outer iterations after a stall */
  int32_t f64_factors; /* gLISA with the tensor-core Hessian: Newton steps whose
                          FP32 factor met a non-positive pivot (or whose free set
                          exceeded 224 shells) and were factored in FP64 */
  int64_t g_active_values; /* gLISA fused passes: values of G in the rows that are
                              not identically zero on their point tile (the
                              values those passes read), summed over tiles;
                              0 when the job has no such index */
  double point_atom_evals_skipped; /* MBIS on the molecular grid: evaluations of
                                      point_atom_evals (which counts every atom at
                                      every point, the reference's convention)
                                      that the per-atom cutoff skipped */
} hp_job_info;

typedef struct {
  double* charges;           /* natom */
  double* propars;           /* nparam */
  double* history_propars;   /* niter x nparam */
  double* history_charges;   /* niter x natom (empty for gLISA) */
  double* history_entropies; /* niter */
  double* history_changes;   /* niter */
  double* promoldens;        /* npoint */
  double* at_weights;        /* natom x npoint */
} hp_job_results;

/* Library */
int32_t hp_abi_version(void);
const char* hp_last_error(void);

/* Context: one device, one stream, an HBM budget in bytes (0 = 90 % of free
 * memory). `stream` may be NULL (the library creates one) or a cudaStream_t
 * owned by the caller. */
int32_t hp_ctx_create(int32_t device, size_t hbm_budget, void* stream, hp_ctx** out);
int32_t hp_ctx_destroy(hp_ctx* ctx);
int32_t hp_ctx_synchronize(hp_ctx* ctx);
/* Bytes reserved by live jobs and the budget. */
int32_t hp_ctx_memory(hp_ctx* ctx, size_t* used, size_t* budget);

/* Jobs */
int32_t hp_job_create(hp_ctx* ctx, const hp_job_desc* desc, hp_job** out);
int32_t hp_job_destroy(hp_job* job);
/* Advance every live job in `jobs` by one outer iteration. Kernels of all
 * jobs go to the context stream; the host waits once at the end. `n_live`
 * receives the number of jobs still running. */
int32_t hp_step(hp_ctx* ctx, hp_job* const* jobs, int32_t njobs, int32_t* n_live);
/* Advance every live job by up to max_iterations (1..64) outer iterations in
 * one host round trip. gLISA (newton, projected Newton, sc): the iterations
 * are queued back to back and the device stops a job at the iteration that
 * converges, fails or reaches maxiter (the results equal one iteration per
 * hp_step); other schemes and gLISA m-newton advance one iteration per call.
 * (No reference counterpart: several passes of the loop body of
 * glisa.py:748-798 without returning to Python.) */
int32_t hp_step_n(hp_ctx* ctx, hp_job* const* jobs, int32_t njobs, int32_t max_iterations,
                  int32_t* n_live);
/* Run one job to completion (the whole do_partitioning); gLISA jobs queue
 * two to four solver iterations per host round trip. */
int32_t hp_job_run(hp_ctx* ctx, hp_job* job);
int32_t hp_job_info_get(hp_job* job, hp_job_info* out);
int32_t hp_job_results_get(hp_job* job, const hp_job_results* out);
/* Restart a job from its initial parameters; inputs stay on the device.
 * (No reference counterpart: re-running do_partitioning after part.clear(),
 * core/base.py:164-167, without re-uploading the grid.) */
int32_t hp_job_reset(hp_job* job);

/* Evaluation service of the gLISA solvers whose iterations run on the host
 * (DIIS, CDIIS, trust-region, quasi-Newton: glisa.py:595-615, 883-1028, with
 * algo/diis.py, algo/cdiis.py, algo/quasi_newton.py): the host keeps the
 * solver state (a few vectors of nparam values), the device does every pass
 * over the grid. FP64 gLISA jobs on the molecular grid only
 * (HP_ERR_UNSUPPORTED otherwise); x, y, delta, keep, grad, hess and x_out
 * are HOST arrays of nparam (hess: nparam x nparam) values.
 *
 * hp_glisa_evaluate <- GlobalLinearISAWPart._working_matrix (glisa.py:411-479)
 *   with calc_promol_dens (glisa.py:346-348): at populations x, f =
 *   int rho ln(rho/rho0), grad_i = -int rho g_i/rho0 (nderiv >= 1), hess_ij =
 *   int rho g_i g_j/rho0^2 (nderiv = 2), pro_pop = int rho0. */
int32_t hp_glisa_evaluate(hp_job* job, const double* x, int32_t nderiv, double* f, double* grad,
                          double* hess, double* pro_pop);
/* kind 0: sqrt(int (rho0(x) - rho0(y))^2), the promolecule change of the
 *   DIIS and trust-region convergence tests (glisa.py:886-893, 958-962);
 * kind 1: the outer change of compute_change (core/iterstock.py:32-45). */
int32_t hp_glisa_change(hp_job* job, const double* x, const double* y, int32_t kind,
                        double* change);
/* The valid-promolecule line search of _solver_general_newton
 * (glisa.py:675-743): the first t of linspace(tau, 0, linspace_size) (the
 * job's tau and linspace_size) with every pro-atom of x + keep * t * delta
 * at or above negative_cutoff on the grid; *step = t and x_out = that point,
 * or *step = -1 when no trial is valid. */
int32_t hp_glisa_line_search(hp_job* job, const double* x, const double* delta, const double* keep,
                             double* step, double* x_out);
/* End a host-driven job at populations x after niter iterations: the checks,
 * at_weights and charges of glisa.py:268-278 (check_pro_atom_parameters,
 * utils.py:255-398); the job is done afterwards and hp_job_results_get
 * returns its charges and parameters (the histories stay with the host). */
int32_t hp_glisa_finish(hp_job* job, const double* x, int32_t niter);

/* ------------------------------------------------------------------------
 * Density generator: the electron density of a contracted-Gaussian
 * wavefunction on grid points (scripts/generate_density.py:119-204, with
 * rho = einsum("ab,bp,ap->p", D, phi, phi) at :186-188), in FP64.
 *
 * Shells follow Gaussian's fchk conventions (0 <= l <= 3; Cartesian
 * components in file order; pure functions m = 0, +1, -1, ... given by the
 * caller's Cartesian-to-pure matrices). coeffs already include the
 * primitive normalisation (2a/pi)^(3/4) (4a)^(l/2) / sqrt((2l-1)!!).
 * ------------------------------------------------------------------------ */
typedef struct {
  int32_t nshell;
  const double* centers;      /* [nshell][3], bohr */
  const int32_t* shell_info;  /* [nshell][5]: l, pure, nprim, first primitive, first function */
  int32_t nprim;
  const double* exponents;    /* [nprim] */
  const double* coeffs;       /* [nprim] */
  int32_t nbasis;
  int32_t nmat;               /* density matrices (total, spin, ...) */
  const double* mats;         /* [nmat][nbasis][nbasis], symmetric */
  const double* pure2;        /* [5][6] row-major, or NULL when no pure d shell */
  const double* pure3;        /* [7][10] row-major, or NULL when no pure f shell */
} hp_density_desc;

typedef struct hp_density_plan hp_density_plan;

/* Copy the basis and the matrices to the device. */
int32_t hp_density_plan_create(hp_ctx* ctx, const hp_density_desc* desc, hp_density_plan** out);
/* out[m * npoint + p] = sum_ab mats[m]_ab phi_a(points[p]) phi_b(points[p]).
 * device_ptrs = 0: points and out are host arrays (copied in and out);
 * 1: device arrays of the plan's context, used in place (asynchronous on
 * the context stream). */
int32_t hp_density_plan_eval(hp_density_plan* plan, int64_t npoint, const double* points,
                             double* out, int32_t device_ptrs);
/* Work performed since the plan was created: [0] shell-tile pairs kept by
 * the screening, [1] basis values evaluated, [2] FMA per matrix in the
 * contraction (synchronises the context stream). */
int32_t hp_density_plan_stats(hp_density_plan* plan, uint64_t* stats);
int32_t hp_density_plan_destroy(hp_density_plan* plan);

/* Kernel timing with CUDA events on the context stream, per kernel family
 * (hp_kernel_family). Enabling clears the accumulators. */
typedef enum {
  HP_KERNEL_PROMOL = 0,     /* pro-atoms, promolecule, at_weights */
  HP_KERNEL_INNER = 1,      /* MBIS / aLISA inner solver passes, GISA moments */
  HP_KERNEL_CHANGE = 2,     /* outer change pass */
  HP_KERNEL_GLISA_PRO = 3,  /* gLISA promolecule, ratios, entropy (fused jobs: also
                               the gradient, the outer change and the tensor-core
                               Hessian, all in one pass over G) */
  HP_KERNEL_GLISA_GRAD = 4, /* gLISA gradient */
  HP_KERNEL_GLISA_HESS = 5, /* gLISA Hessian G^T diag(w rho/rho0^2) G */
  HP_KERNEL_GLISA_SOLVE = 6,/* gLISA Newton solve (reduction of the partial sums,
                               factor, step, refinement) */
  HP_KERNEL_OTHER = 7,
  HP_KERNEL_GLISA_TRIALS = 8,/* gLISA step-length search: trial objectives and the
                               pick (projected Newton), line search (m-newton),
                               the update (newton, sc) */
  HP_KERNEL_COUNT = 9
} hp_kernel_family;
int32_t hp_ctx_profile(hp_ctx* ctx, int32_t enable);
int32_t hp_ctx_profile_get(hp_ctx* ctx, int32_t family, double* ms, int64_t* launches);

/* MBIS inner fixed point for ONE atom that allocates no memory. It has no
 * counterpart in the reference; it computes what the reference's per-atom
 * solver opt_mbis_propars does for one atom on the molecular grid.
 *
 * For callers that cannot call cudaMalloc: code running inside a host
 * application's own device-memory pool, plug-in hosts that forbid allocation
 * after start-up, and loops where an allocation would synchronise the device.
 *
 * All array arguments are DEVICE pointers owned by the caller: rho_a, weights
 * and radial_dist hold npoint values (the atom's AIM density w_a * rho, the
 * grid weights and |r - R_a|); propars holds the 2*nshell (N, S) pairs on
 * input and the solution on output. niter and converged are optional HOST
 * outputs. Runs on `stream` (NULL = default stream) and returns after it;
 * it blocks the host on that stream every 4 inner iterations (8 for the first
 * chunk) to read its done flag, so it is synchronous, not asynchronous.
 * Limits: 1 <= nshell <= 7 and npoint <= 2,097,152 (HP_ERR_INVALID beyond).
 * The scratch is one 492 KB static device array per GPU, shared by all calls:
 * calls that overlap on the GPU (other streams or threads) race on it. The
 * first call on a device looks up that array's address; make that first call
 * before any stream capture. The address is kept for the life of the process:
 * calls after cudaDeviceReset are unsupported. A CUDA error already pending
 * when the call starts is returned as HP_ERR_CUDA without clearing it. */
int32_t hp_mbis_inner_noalloc(const double* rho_a, const double* weights,
                              const double* radial_dist, int64_t npoint, int32_t nshell,
                              double* propars, double threshold, double density_cutoff,
                              int32_t maxiter, int32_t* niter, int32_t* converged, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HPGPU_H */
