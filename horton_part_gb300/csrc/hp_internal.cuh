// Internal declarations shared by the partitioning kernels and the runtime.
//
// Data layout in HBM (per job):
//   grid       px, py, pz, w, rho          FP64 SoA, npoint each
//              pxh/pxl ... (float hi/lo)   mixed precision only
//   atoms      ax, ay, az                  FP64, natom
//   shells     shell_off[natom+1], per-shell (order, alpha, prefactor)
//   params     propars / propars_old / cur / prev      FP64, nparam
//   per point  promol                      FP64, npoint
//   per pair   rhoa[natom][npoint]         FP64 (the AIM density w_a * rho)
//   partials   apart[natom][QA][ntile]     FP64 per (atom, point-tile) sums
//              jpart[QJ][ntile]            FP64 per point-tile sums
//
// Work is cut into point tiles of kTilePoints consecutive grid points. Every
// kernel is launched over a *batch* of jobs: block b finds its job by a
// binary search in a prefix array of per-job block counts, so one launch
// serves many molecules of uneven size. All reductions are deterministic:
// fixed per-thread point order, fixed warp-shuffle trees, per-tile partials
// written without atomics and summed over tiles in a fixed order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hp {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxShells = 16;  // per atom
// A point tile is kThreads * ppt consecutive points; ppt is fixed per job
// (it depends only on that job's npoint, so a job's reductions are the same
// alone and inside a batch).

// Per-atom partial quantities (index q in apart[atom][q][tile]).
// Layout depends on the kernel family; QA is the per-atom stride.
enum AtomQ {
  QA_POP = 0,      // sum w * rho_a (from the at_weights pass)
  QA_CHANGE = 1,   // sum w * (pro_new - pro_old)^2 (outer change)
  QA_INNER = 2     // first slot of the inner-solver quantities
};

// Per-job partial quantities (index q in jpart[q][tile]).
enum JobQ {
  QJ_ENTROPY = 0,  // sum w rho ln(rho/promol)
  QJ_NELEC = 1,    // sum w rho
  QJ_NEG = 2,      // count of points with promolecule < negative_cutoff
  QJ_ENT_PREV = 3, // fused gLISA jobs: QJ_ENTROPY / QJ_NEG of the parameters at the
  QJ_NEG_PREV = 4, // start of the iteration (the pass that forms them runs one step early)
  QJ_COUNT = 5
};

// Device-side scalars of a job, mirrored to pinned host memory after each
// step (one contiguous array of Mailbox for all job slots of a context).
enum MailD {
  MD_CHANGE = 0,      // last outer change
  MD_ENTROPY = 1,     // last entropy
  MD_NELEC = 2,       // integrated density
  MD_INNER_TOTAL = 3, // inner iterations summed over atoms (exact in FP64)
  MD_LS_X = 4,        // accepted line-search step (gLISA m-newton)
  MD_SKIPPED = 5,     // point-atom evaluations skipped by the per-atom cutoff (summed)
  MD_EVAL_A = 6,      // host-driven gLISA solvers: objective or change of the last evaluation
  MD_EVAL_B = 7,      // host-driven gLISA solvers: int rho0 of the last evaluation
  MD_COUNT = 8
};
enum MailI {
  MI_ITER = 0,        // outer iterations done (history rows written)
  MI_NACTIVE = 1,     // atoms whose inner solver is still running
  MI_ERR = 2,         // ErrFlag bits
  MI_WARN = 3,        // warning bits (HP_WARN_*)
  MI_CONVERGED = 4,   // gLISA solver converged flag
  MI_F64_FACTORS = 5, // gLISA Newton steps of a tensor-core job factored in FP64
  MI_DONE = 6,        // gLISA: finished (converged, failed or out of iterations)
  MI_R0T = 7,         // fused gLISA: 1 + the accepted trial whose densities (r0t) are the next
                      // pass's rho0, 0 when that pass forms rho0 = G^T c itself
  MI_COUNT = 8
};
struct Mailbox {
  double d[MD_COUNT];
  int i[MI_COUNT];
};

enum ErrFlag {
  E_NEG_DENSITY = 1,   // pro-atom / promolecule density below negative_cutoff
  E_SINGULAR = 2,      // Hessian not positive definite
  E_LINESEARCH = 4,    // no valid trial step
  E_INNER_NOT_CONV = 8,// Newton inner loop hit its iteration limit
  E_QP = 16,           // QP active-set did not finish
  E_TIMEOUT = 32       // a bounded mbarrier wait ran out (tensor-core Hessian)
};

enum WarnFlag { W_INNER = 1, W_POPULATION = 2, W_NEG_PARS = 4 };

enum Scheme { SCHEME_MBIS = 0, SCHEME_GISA = 1, SCHEME_LISA = 2, SCHEME_GLISA = 3, SCHEME_NLIS = 4 };
enum Solver { SOLVER_DEFAULT = 0, SOLVER_SC = 1, SOLVER_NEWTON = 2, SOLVER_M_NEWTON = 3,
              SOLVER_QP = 4, SOLVER_PNEWTON = 5, SOLVER_BFGS = 6 };
constexpr int kTrials = 8;  // projected-Newton step lengths 2^-t evaluated per pass
enum Model { MODEL_MBIS = 0, MODEL_BASIS = 1, MODEL_NLIS = 2 };
// Evaluation phase of a job (JobDev::mixed): FP64, FP32 with compensated sums,
// or float-float (MBIS).
enum Phase { PH_FP64 = 0, PH_FP32 = 1, PH_FF = 2 };

struct JobDev {
  // grid
  const double* px;
  const double* py;
  const double* pz;
  const double* w;
  const double* rho;
  const float* pxh; const float* pxl;
  const float* pyh; const float* pyl;
  const float* pzh; const float* pzl;
  const float* wf;
  const float* rhof;
  const float* wl;        // mixed / ff: low parts of w and rho (w = wf + wl)
  const float* rhol;
  const float* shf;       // mixed: per shell (order, alpha, prefactor) as FP32
  const float* atf;       // mixed: atom coordinates as FP32 hi/lo [natom][6]
  const double* qp_p;     // GISA: per-atom QP matrix P (K_a x K_a, FP64), at shell_off^2 offsets
  const int* qp_off;      // GISA: offset of atom a's P block (natom + 1)
  float* fpar;            // mixed: FP32 pro-atom coefficients of propars (2 per shell);
                          // ff: (A hi, A lo, S hi, S lo) per shell
  float* fco;             // mixed: per-shell FP32 coefficients [nshell][8] of a (new, old)
                          // parameter pair: MBIS (A_new, S_new, A_old, S_old, g, dS),
                          // basis (c_new, c_old - c_new); A = N S^3/(8 pi), g = A_old/A_new - 1;
                          // MBIS slots 6, 7: low parts of A_new, S_new (ff)
  float* promolf;         // mixed: FP32 promolecule
  // atoms and shells
  const double* ax;
  const double* ay;
  const double* az;
  const double* zpseudo;
  const int* shell_off;   // natom + 1
  const int* par_off;     // natom + 1
  const double* sh_order;
  const double* sh_alpha;
  const double* sh_pref;
  // parameters and solver state
  double* propars;
  double* propars_init;   // initial parameters (hp_job_reset)
  double* propars_old;
  double* cur;
  double* prev;
  double* delta;          // Newton steps (nparam)
  double* hinv;           // aLISA quasi-Newton: inverse-Hessian estimate per atom [natom][kMaxShells^2]
  double* olddf;          // aLISA quasi-Newton: gradient of the previous inner iteration (nparam)
  double* step;           // aLISA quasi-Newton: step taken by the previous inner iteration (nparam)
  double* keep;           // gLISA line-search mask (nparam)
  // buffers
  double* promol;
  double* invpro;         // FP64 jobs: 1 / promol (one division per point, not per pair)
  double* rhoa;
  double* apart;
  double* jpart;
  double* atom_out;       // [natom][AO_COUNT]
  int* active;            // natom
  int* inner_it;          // natom
  int* ls_fail;           // per (atom, tile) line-search failure bitmask
  double* gmat;           // gLISA: basis values [nshell][npoint]
  double* gpart;          // gLISA: gradient partials [nshell][ntile]
  double* hpart;          // gLISA: Hessian partials [nsplit][nshell][nshell]
  double* hess;           // gLISA: Hessian [nshell][nshell]
  double* chol;           // gLISA: Cholesky factor work space [nshell][nshell]
  double* grad;           // gLISA: gradient [nshell]
  double* dvec1;          // gLISA: w rho / rho0 (0 where sick), npoint
  double* dvec2;          // gLISA: w rho / rho0^2 (0 where sick), npoint
  double* ctrial;         // gLISA projected Newton: trial populations [kTrials][nshell]
  double* tpart;          // gLISA projected Newton: trial objective partials [kTrials][ntile], then
                          // the magnitudes of their FP32 terms [kTrials][ntile]
  int* freeidx;           // gLISA Newton: free-variable list [nshell], count at [nshell]
  float* gmat32;          // gLISA tensor-core Hessian: FP32 copy of gmat [nshell][npoint]
                          // (with gff: the high part of G = gmat32 + gmat_lo)
  float* gmat_lo;         // gLISA, gff: low part of G [nshell][npoint] (gmat is not stored)
  float* clipf;           // gLISA, gff: clipped shells' (c hi, c lo, delta hi, delta lo) [nshell]
  float2* rdist;          // mixed / ff (MBIS, GISA, aLISA): point-atom distances as float pairs [natom][npoint]
  float4* wrf;            // fused gLISA: (w rho hi, lo, rho hi, lo) per point (constant)
  float2* r0f;            // fused gLISA: rho0 as float pairs [npoint]
  float2* r0t;            // fused gLISA: the trial pass's rho0 of each trial as float pairs [kTrials][npoint]
  float2* d2f;            // fused gLISA: w rho / rho0^2 as float pairs [npoint]
  double* hsum;           // gLISA tensor-core Hessian: refinement product H delta [nshell]
  int* gact;              // fused gLISA: per point tile the shells nonzero on it [ntile][nshell + 1]
  float* gpack;           // fused gLISA: the tiles' active rows of G packed per 32-point sub-tile
                          // ([sub-tile][active row][32 points], high plane then low plane)
  int64_t* gtile_off;     // fused gLISA: start of tile t's sub-tiles in a plane of gpack (floats)
  int64_t gpack_plane;    // fused gLISA: floats per plane of gpack
  int nact_max;           // fused gLISA: most active rows of a tile
  int* fsched;            // fused gLISA: tile schedule. [0, nb]: block b's entries [fsched[b],
                          // fsched[b + 1]) of the list at fsched + nb + 1 (ntile tiles, ascending
                          // within a block); then the ntile tiles heaviest first (trial pass);
                          // nb = min(ntile, kFuseCtas)
  double* wgram;          // fused gLISA on the molecular grid: per atom the lower triangle of its
                          // weighted Gram block W_a[i][j] = sum_p w_p g_i(p) g_j(p) (the outer change)
  int* wgoff;             // atom a's triangle starts at wgoff[a] [natom + 1]
  int wgn;                // entries of wgram (wgoff[natom])
  float2* d1f;            // gLISA, gff: w rho / rho0 as float pairs, npoint
  float2* hvf;            // gLISA, gff: the refinement's hvec as float pairs, npoint
  float* hess_s;          // gLISA tensor-core Hessian: sqrt(w rho / rho0^2) as FP32, npoint
  double* hvec;           // gLISA refinement: w rho / rho0^2 * (G^T delta)(p), npoint
  double* rho0;           // gLISA: promolecule of the current populations, npoint
  int* clip;              // gLISA projected Newton: shells clipped at the full step [nshell],
                          // count at [nshell], their trial counts t_m at [nshell + 1 ...]
  // grid_type 1 (atom grids, MBIS): atom a owns radial shells [rad_off[a],
  // rad_off[a+1]); shell s owns the grid points [shell_pt[s], shell_pt[s+1])
  // with angular weights wsph (Lebedev weight / 4 pi)
  const int* rad_off;     // natom + 1
  const long long* shell_pt;  // nrad + 1
  const double* wsph;     // npoint
  const double* rad_r;    // nrad: radial nodes
  const double* rad_w;    // nrad: radial weights
  double* radrho;         // nrad: spherical average of w_a rho
  double* hist_propars;   // [maxiter][nparam]
  double* hist_charges;   // [maxiter][natom]
  double* hist_ent;       // [maxiter]
  double* hist_chg;       // [maxiter]
  double* charges;        // natom
  // per-atom cutoff (MBIS on the molecular grid): per point tile its bounding
  // sphere and weight sum [ntile][5] = (cx, cy, cz, R, sum w), and per (atom,
  // tile) the largest AIM density rho_a on the tile from the last at_weights
  // pass [natom][ntile]; null when the job has no cutoff
  const double* tgeo;
  float* amax;
  Mailbox* mail;
  int natom, npoint, ntile, nparam, nshell, qa;
  int scheme, solver, mixed, maxiter;
  int inner_maxiter, linspace_size, nsplit, ppt;  // ppt: points per thread per tile
  int local, nrad;                               // local: grid_type 1 (atom grids)
  int tile_points, htiles, tc, gff;              // htiles: 64-wide Hessian tiles per side;
                                                 // tc: gLISA Hessian on the tensor cores;
                                                 // gff: gLISA G passes in float-float
  int fuse;                                      // gff with nshell <= kFuseMaxShells: fused passes
  int refine;                                    // tc with polish: refine the Newton step in the finish
  double threshold, inner_threshold, density_cutoff, negative_cutoff, population_cutoff, tau;
};

// gLISA with the tensor-core Hessian: the Newton direction from the FP32
// factor carries ~1e-6 relative error, which the outer iteration does not
// notice (same iteration counts, same optimum: the gradient and objective are
// exact). With polish, the iterations of the finish (last outer change within
// 100 x the threshold) refine it once against the exact product H delta.
// Read from the job's mailbox, which only the end of a step writes, so every
// kernel of a step sees the same answer.
__device__ __forceinline__ bool glisa_idle(const JobDev& J);
__device__ __forceinline__ bool glisa_refine_now(const JobDev& J) {
  return J.refine && J.mail->i[MI_ITER] > 0 && J.mail->d[MD_CHANGE] < 100.0 * J.threshold;
}

// Per-atom cutoff of the MBIS inner solve and outer change. The reference
// sums every grid point for every atom. A point contributes nothing to
// atom a's inner moments where rho_a < density_cutoff (the sick mask of
// mbis.py:126-133); a (atom, tile) pair whose largest rho_a on the tile is
// below the cutoff therefore adds exact zeros to the moments, and only the
// change term sum_p w (pro_old - pro_new)^2 remains, which is bounded by
// W_t (pro_old + pro_new)(r_min)^2: W_t the tile's weight sum and r_min the
// distance from the atom to the tile's bounding sphere (a sum of Slater
// shells with non-negative populations decreases with r). Such a pair is
// skipped when that bound is below kSkipRel x threshold^2, 1e-16 of the
// squared change at which the loop stops: below the rounding of the sums
// themselves. The outer change (core/iterstock.py:32-45) skips a pair on
// the same bound with the outer threshold.
constexpr double kSkipRel = 1e-16;

// Largest v over the block (valid in thread 0); red: kWarps floats.
__device__ __forceinline__ float block_max_f(float v, float* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) red[warp] = v;
  __syncthreads();
  float m = red[0];
  for (int k = 1; k < (int)(blockDim.x >> 5); ++k) m = fmaxf(m, red[k]);
  return m;
}

__device__ __forceinline__ double tile_rmin(const JobDev& J, int a, int t) {
  const double* g = J.tgeo + 5 * (size_t)t;
  const double dx = J.ax[a] - g[0], dy = J.ay[a] - g[1], dz = J.az[a] - g[2];
  return fmax(0.0, sqrt(dx * dx + dy * dy + dz * dz) - g[3]);
}

__device__ __forceinline__ double tile_weight(const JobDev& J, int t) {
  return J.tgeo[5 * (size_t)t + 4];
}

// Upper bound of an MBIS pro-atom (pairs (N_k, S_k), N_k >= 0) at distance
// r >= 0 from its atom: sum |N_k| S_k^3 / (8 pi) exp(-S_k r).
__device__ __forceinline__ double mbis_bound(const double* par, int nsh, double r) {
  double b = 0.0;
  for (int k = 0; k < nsh; ++k) {
    const double n = fabs(par[2 * k]), x = par[2 * k + 1];
    b += n * x * x * x * (0.125 / M_PI) * exp(-x * r);
  }
  return b;
}

// Upper bound of sum_k |a_k - b_k| g_k(r) for an atom's basis shells s0 ..
// s0 + nsh - 1 (unit-population shells N(alpha, n) exp(-alpha r^n), which
// decrease with r); b null: sum_k |a_k| g_k(r).
__device__ __forceinline__ double basis_bound(const JobDev& J, int s0, int nsh, const double* a,
                                              const double* b, double r) {
  double s = 0.0;
  for (int k = 0; k < nsh; ++k) {
    const double c = b ? a[k] - b[k] : a[k];
    const int m = s0 + k;
    s += fabs(c) * J.sh_pref[m] * exp(-J.sh_alpha[m] * pow(r, J.sh_order[m]));
  }
  return s;
}

// The same bound from the FP32 shell coefficient table of the mixed and
// float-float kernels (fco: per shell 8 floats; A = N S^3 / (8 pi) at column
// ca, S at column ca + 1).
__device__ __forceinline__ float mbis_bound_f(const float* co, int nsh, int ca, float r) {
  float b = 0.0f;
  for (int k = 0; k < nsh; ++k) b += fabsf(co[8 * k + ca]) * expf(-co[8 * k + ca + 1] * r);
  return b;
}

// Records a skipped pair: its points count as skipped evaluations (`passes`
// pro-atom evaluations per point).
__device__ __forceinline__ void count_skipped(const JobDev& J, int t, double passes) {
  const int n = min(J.tile_points, J.npoint - t * J.tile_points);
  atomicAdd(&J.mail->d[MD_SKIPPED], passes * (double)n);
}

// gLISA jobs advance several solver iterations per host round trip:
// k_outer_finish marks a job finished (converged, failed or out of
// iterations) in MI_DONE, and every kernel of a gLISA step returns at once
// for such a job, so the iterations queued after its last one do nothing.
__device__ __forceinline__ bool glisa_idle(const JobDev& J) {
  return J.scheme == SCHEME_GLISA && J.mail->i[MI_DONE] != 0;
}


enum AtomOut {
  AO_POP = 0,
  AO_CHANGE = 1,
  AO_INNER_CHANGE = 2,
  AO_LS_X = 3,
  AO_COUNT = 4
};

// A batch of jobs for one launch: block b belongs to the job j with
// prefix[j] <= b < prefix[j + 1].
struct Batch {
  const JobDev* jobs;
  const int* prefix;
  int njobs;
};

__device__ __forceinline__ int find_job(const Batch& bt, int b) {
  int lo = 0, hi = bt.njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (bt.prefix[mid] <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Deterministic block sum of Q per-thread values. Result valid in out[0..Q)
// (shared memory) after the call, for all threads.
template <int Q>
__device__ __forceinline__ void block_sum(double (&acc)[Q], double* red /* [kWarps][Q] */,
                                          double* out /* [Q] */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    double v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp * Q + q] = v;
  }
  __syncthreads();
  if (threadIdx.x < Q) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kWarps; ++k) s += red[k * Q + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

__device__ __forceinline__ double block_sum1(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kWarps; ++k) s += red[k];
  __syncthreads();
  return s;
}

// Per-tile partial sums of mixed-precision jobs are float-float pairs stored
// in the FP64 slot (bit pattern of a float2); FP64 jobs store doubles.
__device__ __forceinline__ double partial_value(const JobDev& J, const double* slot) {
  if (!J.mixed) return *slot;
  const float2 v = *reinterpret_cast<const float2*>(slot);
  return (double)v.x + (double)v.y;
}

__device__ __forceinline__ void store_partial(const JobDev& J, double* slot, double v) {
  if (!J.mixed) {
    *slot = v;
    return;
  }
  const float hi = (float)v;
  *reinterpret_cast<float2*>(slot) = make_float2(hi, (float)(v - (double)hi));
}

// Fixed-order sum of n values with stride (one thread).
__device__ __forceinline__ double serial_sum(const double* p, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += p[i];
  return s;
}

constexpr double kInv8PiD = 0.039788735772973836;  // 1 / (8 pi)

// FP32 coefficients of shell s for a (new, old) parameter pair, formed in
// FP64 (mixed precision only): MBIS (A_new, S_new, A_old, S_old, g, dS) with
// A = N S^3 / (8 pi), g = A_old / A_new - 1, dS = S_new - S_old; basis
// schemes (c_new, c_old - c_new).
__device__ __forceinline__ void fill_fco(const JobDev& J, int s, const double* pnew,
                                         const double* pold) {
  float* c = J.fco + 8 * s;
  if (J.scheme == SCHEME_MBIS) {
    const double n1 = pnew[2 * s], s1 = pnew[2 * s + 1];
    const double n0 = pold[2 * s], s0 = pold[2 * s + 1];
    const double a1 = n1 * s1 * s1 * s1 * kInv8PiD, a0 = n0 * s0 * s0 * s0 * kInv8PiD;
    c[0] = (float)a1;
    c[1] = (float)s1;
    c[2] = (float)a0;
    c[3] = (float)s0;
    c[4] = a1 != 0.0 ? (float)(a0 / a1 - 1.0) : 0.0f;
    c[5] = (float)(s1 - s0);
    c[6] = (float)(a1 - (double)c[0]);
    c[7] = (float)(s1 - (double)c[1]);
  } else {
    c[0] = (float)pnew[s];
    c[1] = (float)(pold[s] - pnew[s]);
  }
}

// Distance from grid point p to atom a.
template <typename T>
struct Dist;

template <>
struct Dist<double> {
  __device__ __forceinline__ static double r(const JobDev& J, int p, int a) {
    const double dx = J.px[p] - J.ax[a];
    const double dy = J.py[p] - J.ay[a];
    const double dz = J.pz[p] - J.az[a];
    return sqrt(dx * dx + dy * dy + dz * dz);
  }
};

// Mixed precision: coordinates as float hi + lo pairs; the difference is
// formed as (xh - axh) + (xl - axl), which keeps ~1e-7 relative accuracy
// in the distance without FP64 arithmetic.
template <>
struct Dist<float> {
  __device__ __forceinline__ static float r(const JobDev& J, int p, int a) {
    if (J.rdist) return J.rdist[(size_t)a * J.npoint + p].x;  // stored float-float distance
    const float* c = J.atf + 6 * a;  // xh, xl, yh, yl, zh, zl (no FP64 work per point)
    const float dx = (J.pxh[p] - c[0]) + (J.pxl[p] - c[1]);
    const float dy = (J.pyh[p] - c[2]) + (J.pyl[p] - c[3]);
    const float dz = (J.pzh[p] - c[4]) + (J.pzl[p] - c[5]);
    return sqrtf(dx * dx + dy * dy + dz * dz);
  }
};

__device__ __forceinline__ double dexp(double x) { return exp(x); }
__device__ __forceinline__ float dexp(float x) { return expf(x); }

constexpr double kInv8Pi = 0.039788735772973836;  // 1 / (8 pi)

// MBIS Slater shell N S^3 exp(-S r) / (8 pi)  (mbis.py:128, mbis.py:258)
template <typename T>
__device__ __forceinline__ T slater_shell(T n, T s, T r) {
  return n * (s * s * s) * dexp(-s * r) * (T)kInv8Pi;
}

// Basis shell N(alpha, n) exp(-alpha r^n), unit population (core/basis.py:161-163)
template <typename T>
__device__ __forceinline__ T basis_shell(T order, T alpha, T pref, T r) {
  T rn;
  if (order == (T)2) rn = r * r;
  else if (order == (T)1) rn = r;
  else rn = pow(r, order);
  return pref * dexp(-alpha * rn);
}

// NLIS / GMBIS shell with population N: N n S^(3/n) exp(-S r^n) / (4 pi
// Gamma(3/n)) (nlis.py:148, 298); n = 1 is MBIS's Slater shell.
__device__ __forceinline__ double nlis_shell(double N, double S, double n, double r) {
  const double rn = n == 1.0 ? r : n == 2.0 ? r * r : pow(r, n);
  return N * n * pow(S, 3.0 / n) * exp(-S * rn) / (4.0 * M_PI * tgamma(3.0 / n));
}

// r^n for an NLIS shell order.
__device__ __forceinline__ double nlis_rn(double n, double r) {
  return n == 1.0 ? r : n == 2.0 ? r * r : pow(r, n);
}

}  // namespace hp

namespace hp {

// Launch kinds: blocks per job for each kind of work.
enum Kind {
  K_POINT = 0,      // one block per point tile
  K_POINT1 = 6,     // one block per kThreads points (kernels without per-tile sums)
  K_ATOM_TILE = 1,  // one block per (atom, point tile)
  K_ATOM = 2,       // one 32-thread block per atom
  K_JOB = 3,        // one block per job
  K_HESS = 4,       // gLISA Hessian: (tile pair, point split)
  K_SQUARE = 5,     // gLISA reduce: ceil(nshell^2 / kThreads)
  K_FUSE = 7,       // fused gLISA pass: min(ntile, kFuseCtas) persistent blocks per job
  K_NKIND = 8
};

// Persistent blocks of the fused gLISA pass per job (two per SM): each
// accumulates the Hessian of its point tiles in tensor memory and writes one
// partial, so a fused job has nsplit = min(ntile, kFuseCtas) partials.
constexpr int kFuseCtas = 2 * 152;

struct HostBatch {
  Batch b[K_NKIND];
  int blocks[K_NKIND];
  int nact_max = 0;  // fused gLISA: most active rows of a tile over the batch's jobs
};

void launch_nelec(const HostBatch& hb, cudaStream_t st);
void launch_copy_old(const HostBatch& hb, cudaStream_t st);
void launch_promol(const HostBatch& hb, cudaStream_t st, int mixed, int model);
void launch_final_atweights(const HostBatch& hb, cudaStream_t st, int mixed, int model, int use_old);
void launch_change(const HostBatch& hb, cudaStream_t st, int mixed, int model);
void launch_outer_finish(const HostBatch& hb, cudaStream_t st, int with_charges);
void launch_charges(const HostBatch& hb, cudaStream_t st);
void launch_inner_init(const HostBatch& hb, cudaStream_t st);
void launch_count_active(const HostBatch& hb, cudaStream_t st);
void launch_mbis_inner(const HostBatch& hb, cudaStream_t st, int mixed);
void launch_nlis_inner(const HostBatch& hb, cudaStream_t st);  // NLIS / GMBIS, FP64
void launch_nlis_local(const HostBatch& hb, cudaStream_t st);  // spherical averages + radial solve
void launch_gisa(const HostBatch& hb, cudaStream_t st, int mixed);
void launch_lisa_sc_inner(const HostBatch& hb, cudaStream_t st, int mixed);
void launch_lisa_newton_inner(const HostBatch& hb, cudaStream_t st, int mixed, int modified);
void launch_glisa_basis(const HostBatch& hb, cudaStream_t st);
void launch_glisa_pro(const HostBatch& hb, cudaStream_t st);
void launch_glisa_grad(const HostBatch& hb, cudaStream_t st);
void launch_glisa_hess(const HostBatch& hb, cudaStream_t st);
void launch_glisa_reduce(const HostBatch& hb, cudaStream_t st);
void launch_glisa_solve(const HostBatch& hb, cudaStream_t st, int projected, int max_shells, int tc);
void launch_glisa_apply(const HostBatch& hb, cudaStream_t st, int mode);
void launch_glisa_keep(const HostBatch& hb, cudaStream_t st);
void launch_glisa_ls(const HostBatch& hb, cudaStream_t st, int first, int count);
void launch_glisa_change(const HostBatch& hb, cudaStream_t st);
void launch_glisa_check(const HostBatch& hb, cudaStream_t st);
// evaluation service of the host-driven gLISA solvers (FP64 jobs):
// what 0: objective (entropy) and int rho0 after k_glisa_pro;
// what 1: sqrt(int (sum_m delta_m g_m)^2), the promolecule change for delta;
// what 2: sqrt(sum over atoms of the QA_CHANGE partials) after k_glisa_change
void launch_glisa_eval(const HostBatch& hb, cudaStream_t st, int what);
// trials + Armijo pick; fuse_shells > 0: the fused trial pass (batch of fused jobs)
void launch_glisa_pnewton(const HostBatch& hb, cudaStream_t st, int gff, int fuse_shells);
// fuse_shells: largest shell count of the batch's fused jobs (0: none);
// unfused: some job of the batch takes the separate passes
void launch_glisa_refine(const HostBatch& hb, cudaStream_t st, int gff, int fuse_shells, int unfused);

// gLISA passes over G in float-float (hp_glisa_ff.cu); shells per job at most
// kGffMaxShells (their coefficients are staged in shared memory)
constexpr int kGffMaxShells = 2048;
// fused passes (one read of G for a product and the row sums that follow it):
// two shared-memory stages of [S][64] float pairs
constexpr int kFuseMaxShells = 192;
// mode 1 with point_pass: k_glisa_point_ff after the pass (else the caller
// launches it, launch_glisa_point_ff)
void launch_glisa_fused_ff(const HostBatch& hb, cudaStream_t st, int mode, int max_shells,
                           bool point_pass = true);
void launch_glisa_point_ff(const HostBatch& hb, cudaStream_t st);
void launch_glisa_basis_ff(const HostBatch& hb, cudaStream_t st);
void launch_rdist_ff(const HostBatch& hb, cudaStream_t st);  // rdist of the batch's jobs
void launch_glisa_pro_ff(const HostBatch& hb, cudaStream_t st);
void launch_glisa_grad_ff(const HostBatch& hb, cudaStream_t st);
void launch_glisa_hv_ff(const HostBatch& hb, cudaStream_t st);  // hvec and G hvec
void launch_glisa_trials_ff(const HostBatch& hb, cudaStream_t st);
void launch_glisa_final_ff(const HostBatch& hb, cudaStream_t st);   // final promolecule, then at_weights
void launch_glisa_active(const HostBatch& hb, cudaStream_t st);    // per-tile active shells
void launch_glisa_pack(const HostBatch& hb, cudaStream_t st);      // active rows packed per sub-tile

// job creation: the points' SoA and float-pair forms, w and rho pairs
struct StageArgs {
  const double* pts;       // (n, 3) as the caller passed them (device copy)
  int n;
  double* xyz[3];          // px, py, pz
  float* hi[3];            // pxh, pyh, pzh (null: no float pairs)
  float* lo[3];            // pxl, pyl, pzl
  const double* w;         // weights and density (device)
  const double* rho;
  float* wf; float* wl;    // null: no w / rho pairs
  float* rf; float* rl;
};
void launch_stage_points(const StageArgs& a, cudaStream_t st);
void launch_glisa_wgram(const HostBatch& hb, cudaStream_t st);     // per-atom Gram blocks (outer change)
void launch_glisa_trials_fused(const HostBatch& hb, cudaStream_t st, int max_shells);
void launch_atweights(const HostBatch& hb, cudaStream_t st);        // k_atweights alone
void launch_glisa_change_ff(const HostBatch& hb, cudaStream_t st);

// tensor-core Hessian (hp_tcgen05.cu)
int tc_hess_blocks(const JobDev& J);
// Jobs with at most kTcSinglePassShells shells take the single-pass kernel,
// whose per-split partials are FP32 packed lower triangles (M (M + 1) / 2
// floats per split, row-major: entry (i, j <= i) at i (i + 1) / 2 + j);
// the tiled kernel writes full FP64 M x M partials.
constexpr int kTcSinglePassShells = 256;
// max_shells / min_shells: largest and smallest shell count among the batch's jobs
void launch_glisa_hess_tc(const HostBatch& hb, cudaStream_t st, int max_shells, int min_shells);
void launch_glisa_gram_tc(const HostBatch& hb, cudaStream_t st);  // G diag(w) G^T of fused jobs into hpart

// mixed precision (hp_mixed.cu)
void launch_promol_mx(const HostBatch& hb, cudaStream_t st, int model);
void launch_change_mx(const HostBatch& hb, cudaStream_t st, int model);
void launch_mbis_inner_mx(const HostBatch& hb, cudaStream_t st);
void launch_basis_qvec_mx(const HostBatch& hb, cudaStream_t st);
void launch_lisa_sc_inner_mx(const HostBatch& hb, cudaStream_t st);
void launch_final_atweights_mx(const HostBatch& hb, cudaStream_t st, int model, int use_old);

// MBIS on atom grids (hp_local.cu)
void launch_mbis_local(const HostBatch& hb, cudaStream_t st);  // spherical averages + radial inner solve
void launch_change_radial(const HostBatch& hb, cudaStream_t st);
void launch_gisa_local(const HostBatch& hb, cudaStream_t st);     // spherical averages + radial moments
void launch_lisa_sc_local(const HostBatch& hb, cudaStream_t st);  // spherical averages + radial sc solve
void launch_gisa_qp(const HostBatch& hb, cudaStream_t st);        // k_gisa_qp alone

// float-float MBIS (hp_ff.cu)
void launch_promol_ff(const HostBatch& hb, cudaStream_t st);
void launch_mbis_inner_ff(const HostBatch& hb, cudaStream_t st);
void launch_final_atweights_ff(const HostBatch& hb, cudaStream_t st, int use_old);

extern long long g_launch_count;
// Density of contracted Gaussians on points (hp_density.cu).
struct DensityArgs {
  const double* points;  // [npoint][3]
  int64_t npoint;
  int nshell, nbasis, nmat, tile;
  const double* centers;  // [nshell][3]
  const int* info;        // [nshell][5]: l, pure, nprim, first primitive, first function
  const double* amin;     // [nshell] smallest exponent of the shell
  const double* exps;     // [nprim]
  const double* coefs;    // [nprim] contraction coefficient x primitive normalisation
  const double* mats;     // [nmat][nbasis][nbasis]
  double* out;            // [nmat][npoint]
  unsigned long long* stats;  // [3]: shell-tile pairs, function-point pairs, FMA per matrix; or null
};
constexpr size_t kDensSmemMax = 200 * 1024;
size_t density_smem_bytes(int nbasis, int nshell, int tile);
int density_tile(int nbasis, int nshell);
int set_pure_tables(const double* pure2, const double* pure3);
void launch_density(const DensityArgs& a, cudaStream_t st);

// Message returned by hp_last_error() for the calling thread (hp_runtime.cu).
void set_error_text(const char* msg);

constexpr int kHessTile = 64;
constexpr int kNewtonQ(int k) { return k + k * (k + 1) / 2 + 2; }

}  // namespace hp
