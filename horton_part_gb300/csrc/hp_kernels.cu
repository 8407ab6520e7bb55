// Partitioning kernels for sm_103a.
//
// One kernel family per hot-path step of horton-part's stockholder loop
// (file:line are in the reference package src/horton_part):
//   k_promol          pro-atoms on the molecular grid + promolecule
//                     (core/stockholder.py:153-175, 352-367; mbis.py:263-289;
//                      gisa.py:202-220)
//   k_atweights       at_weights = clip(pro_a / promol, 0, 1), rho_a = w_a rho,
//                     per-atom populations, entropy integral
//                     (core/stockholder.py:369-377, 145-151; mbis.py:200-203)
//   k_change          sum_a int (rho_a0(new) - rho_a0(old))^2
//                     (core/iterstock.py:32-45)
//   k_mbis_*          MBIS inner fixed point (mbis.py:81-163)
//   k_basis_qvec, k_gisa_qp   GISA quadratic program (gisa.py:348-421)
//   k_lisa_sc_*       aLISA self-consistent solver (alisa.py:193-291)
//   k_lisa_newton_*   aLISA (modified) Newton solver (alisa.py:753-938)
//   k_glisa_*         gLISA global Newton / SC (glisa.py:335-479, 617-879)
// Every kernel runs over a batch of jobs (see hp_internal.cuh).
#include <math.h>

#include "hp_internal.cuh"

namespace hp {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

struct AtomTile {
  int job, atom, tile;
};

__device__ __forceinline__ const JobDev& decode_local(const Batch& bt, int& local) {
  const int b = blockIdx.x;
  const int j = find_job(bt, b);
  local = b - bt.prefix[j];
  return bt.jobs[j];
}

__device__ __forceinline__ AtomTile decode_atom_tile(const Batch& bt, const JobDev*& Jp) {
  const int b = blockIdx.x;
  const int j = find_job(bt, b);
  Jp = &bt.jobs[j];
  const int local = b - bt.prefix[j];
  AtomTile t;
  t.job = j;
  t.atom = local / Jp->ntile;
  t.tile = local - t.atom * Jp->ntile;
  return t;
}

__device__ __forceinline__ int point_of(const JobDev& J, int tile, int i) {
  return tile * J.tile_points + i * kThreads + threadIdx.x;
}

// Warp sum over tiles with a fixed lane order (deterministic): four
// independent chains per lane (tiles t, t + 32, t + 64, t + 96 of every 128)
// so that their loads are in flight together, added in a fixed order.
__device__ __forceinline__ double warp_tile_sum(const JobDev& J, const double* p, int ntile) {
  const int lane = threadIdx.x & 31;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int t = lane;
  for (; t + 96 < ntile; t += 128) {
    s0 += partial_value(J, p + t);
    s1 += partial_value(J, p + t + 32);
    s2 += partial_value(J, p + t + 64);
    s3 += partial_value(J, p + t + 96);
  }
  for (; t < ntile; t += 32) s0 += partial_value(J, p + t);
  double s = (s0 + s1) + (s2 + s3);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

__device__ __forceinline__ double* apart_ptr(const JobDev& J, int a, int q) {
  return J.apart + ((size_t)a * J.qa + q) * J.ntile;
}

template <typename T>
__device__ __forceinline__ T shell_value(const JobDev& J, int s, T r) {
  return basis_shell<T>((T)J.sh_order[s], (T)J.sh_alpha[s], (T)J.sh_pref[s], r);
}

// Unit-population shell s at grid point p: read from the stored basis matrix
// when the job keeps one (basis schemes, FP64), else evaluated at distance r.
template <typename T>
__device__ __forceinline__ T basis_val(const JobDev& J, int s, int p, T r) {
  if (J.gmat) return (T)J.gmat[(size_t)s * J.npoint + p];
  if (J.gmat_lo)  // float-float planes of G (gLISA with the tensor-core Hessian)
    return (T)((double)J.gmat32[(size_t)s * J.npoint + p] + (double)J.gmat_lo[(size_t)s * J.npoint + p]);
  return shell_value<T>(J, s, r);
}

// Distance to atom a, skipped when a stored basis matrix makes it unused.
template <typename T, int MODEL>
__device__ __forceinline__ T dist_for(const JobDev& J, int p, int a) {
  if (MODEL == MODEL_BASIS && J.gmat) return (T)0;
  return Dist<T>::r(J, p, a);
}

// Pro-atom of atom a at grid point p (distance r) with parameters par.
template <typename T, int MODEL>
__device__ __forceinline__ T proatom(const JobDev& J, int a, const double* par, T r, int p) {
  const int s0 = J.shell_off[a], s1 = J.shell_off[a + 1];
  const double* pa = par + J.par_off[a];
  T y = (T)0;
  if (MODEL == MODEL_MBIS) {
    for (int k = 0; k < s1 - s0; ++k) y += slater_shell<T>((T)pa[2 * k], (T)pa[2 * k + 1], r);
  } else if (MODEL == MODEL_NLIS) {
    for (int k = 0; k < s1 - s0; ++k)
      y += (T)nlis_shell(pa[3 * k], pa[3 * k + 1], pa[3 * k + 2], (double)r);
  } else {
    for (int k = 0; k < s1 - s0; ++k) y += (T)pa[k] * basis_val<T>(J, s0 + k, p, r);
  }
  return y;
}

// numpy.linspace(start, stop, num, endpoint): i * step + start, last element
// forced to stop when endpoint is true.
__device__ __forceinline__ double linspace_at(double start, double stop, int num, bool endpoint,
                                              int i) {
  const int div = endpoint ? num - 1 : num;
  if (endpoint && i == num - 1) return stop;
  const double step = (stop - start) / (double)div;
  return (double)i * step + start;
}

// In-place Cholesky solve of a small SPD system (n <= 16), one thread.
// Returns false when a pivot is not positive.
__device__ bool small_chol_solve(double* A /* n*n */, double* b, int n) {
  for (int k = 0; k < n; ++k) {
    double d = A[k * n + k];
    for (int j = 0; j < k; ++j) d -= A[k * n + j] * A[k * n + j];
    if (!(d > 0.0)) return false;
    d = sqrt(d);
    A[k * n + k] = d;
    for (int i = k + 1; i < n; ++i) {
      double v = A[i * n + k];
      for (int j = 0; j < k; ++j) v -= A[i * n + j] * A[k * n + j];
      A[i * n + k] = v / d;
    }
  }
  for (int i = 0; i < n; ++i) {
    double v = b[i];
    for (int j = 0; j < i; ++j) v -= A[i * n + j] * b[j];
    b[i] = v / A[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double v = b[i];
    for (int j = i + 1; j < n; ++j) v -= A[j * n + i] * b[j];
    b[i] = v / A[i * n + i];
  }
  return true;
}

// ---------------------------------------------------------------------------
// job set-up
// ---------------------------------------------------------------------------

// Job creation: the caller's (N, 3) points (copied to the device as they
// are) into SoA FP64 coordinates and, for the float paths, their float pairs
// (hi = the rounded value, lo = the rounded remainder, as the host would form
// them); for mixed jobs also w and rho as float pairs. One thread per point.
__global__ void __launch_bounds__(kThreads) k_stage_points(StageArgs a) {
  const int p = blockIdx.x * kThreads + threadIdx.x;
  if (p >= a.n) return;
  const double v[3] = {a.pts[3 * (size_t)p], a.pts[3 * (size_t)p + 1], a.pts[3 * (size_t)p + 2]};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a.xyz[c][p] = v[c];
    if (a.hi[c]) {
      const float h = (float)v[c];
      a.hi[c][p] = h;
      a.lo[c][p] = (float)(v[c] - (double)h);
    }
  }
  if (a.wf) {
    const double w = a.w[p], r = a.rho[p];
    const float wh = (float)w, rh = (float)r;
    a.wf[p] = wh;
    a.wl[p] = (float)(w - (double)wh);
    a.rf[p] = rh;
    a.rl[p] = (float)(r - (double)rh);
  }
}

void launch_stage_points(const StageArgs& a, cudaStream_t st) {
  if (a.n <= 0) return;
  k_stage_points<<<(a.n + kThreads - 1) / kThreads, kThreads, 0, st>>>(a);
  ++g_launch_count;
}

__global__ void __launch_bounds__(kThreads) k_nelec(Batch bt) {
  __shared__ double red[kWarps];
  int tile;
  const JobDev& J = decode_local(bt, tile);
  double acc = 0.0;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, tile, i);
    if (p < J.npoint) acc += J.w[p] * J.rho[p];
  }
  const double s = block_sum1(acc, red);
  if (threadIdx.x == 0) store_partial(J, J.jpart + (size_t)QJ_NELEC * J.ntile + tile, s);
}

// Integrated density; basis schemes rescale the initial populations to it
// (gisa.py:85-86).
__global__ void k_init_params(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  const double nelec = warp_tile_sum(J, J.jpart + (size_t)QJ_NELEC * J.ntile, J.ntile);
  const int lane = threadIdx.x & 31;
  if (lane == 0) J.mail->d[MD_NELEC] = nelec;
  if (J.scheme != SCHEME_MBIS && J.scheme != SCHEME_NLIS) {  // basis schemes: populations only
    double s = 0.0;  // lanes over the parameters, then a fixed-order shuffle sum
    for (int i = lane; i < J.nparam; i += 32) s += J.propars[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    for (int i = lane; i < J.nparam; i += 32) J.propars[i] = J.propars[i] / s * nelec;
  }
}

__global__ void k_copy_old(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  for (int i = threadIdx.x; i < J.nparam; i += blockDim.x) J.propars_old[i] = J.propars[i];
  if (J.fuse)  // entropy and negativity partials of the parameters the step starts from
    for (int t = threadIdx.x; t < J.ntile; t += blockDim.x) {
      J.jpart[(size_t)QJ_ENT_PREV * J.ntile + t] = J.jpart[(size_t)QJ_ENTROPY * J.ntile + t];
      J.jpart[(size_t)QJ_NEG_PREV * J.ntile + t] = J.jpart[(size_t)QJ_NEG * J.ntile + t];
    }
}

// ---------------------------------------------------------------------------
// stockholder weights
// ---------------------------------------------------------------------------

// One block per kThreads points (launch kind K_POINT1).
template <typename T, int MODEL>
__global__ void __launch_bounds__(kThreads) k_promol(Batch bt) {
  int blk;
  const JobDev& J = decode_local(bt, blk);
  const int p = blk * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  double promol = 0.0;
  for (int a = 0; a < J.natom; ++a) {
    const T r = dist_for<T, MODEL>(J, p, a);
    const double pro = (double)proatom<T, MODEL>(J, a, J.propars, r, p);
    J.rhoa[(size_t)a * J.npoint + p] = pro;
    promol += pro;
    promol += 1e-100;
  }
  J.promol[p] = promol;
  J.invpro[p] = 1.0 / promol;
}

__global__ void __launch_bounds__(kThreads) k_atweights(Batch bt) {
  __shared__ double red[kWarps * 2];
  __shared__ double out[2];
  __shared__ float redm[kWarps];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  double acc[2] = {0.0, 0.0};
  float vmax = 0.0f;  // largest rho_a on the tile (per-atom cutoff)
  double* ra = J.rhoa + (size_t)at.atom * J.npoint;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const double promol = J.promol[p];
    const double rho = J.rho[p];
    const double aw = fmin(fmax(ra[p] * J.invpro[p], 0.0), 1.0);
    const double v = aw * rho;
    ra[p] = v;
    vmax = fmaxf(vmax, v > 3e38 ? 3e38f : (float)v);
    acc[0] += J.w[p] * v;
    if (at.atom == 0) {
      const bool sick = (promol < J.density_cutoff) || (rho < J.density_cutoff);
      if (!sick) acc[1] += J.w[p] * rho * log(rho / promol);
    }
  }
  block_sum<2>(acc, red, out);
  if (J.amax) {
    const float m = block_max_f(vmax, redm);
    if (threadIdx.x == 0) J.amax[(size_t)at.atom * J.ntile + at.tile] = m;
  }
  if (threadIdx.x == 0) {
    apart_ptr(J, at.atom, QA_POP)[at.tile] = out[0];
    if (at.atom == 0) J.jpart[(size_t)QJ_ENTROPY * J.ntile + at.tile] = out[1];
  }
}

// at_weights output: clip(pro_a / promol, 0, 1) into rhoa (use_old: the
// parameters at the start of the last outer iteration).
template <typename T, int MODEL>
__global__ void __launch_bounds__(kThreads) k_final_atweights(Batch bt, int use_old) {
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  const double* par = use_old ? J.propars_old : J.propars;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const T r = dist_for<T, MODEL>(J, p, at.atom);
    const double pro = (double)proatom<T, MODEL>(J, at.atom, par, r, p);
    J.rhoa[(size_t)at.atom * J.npoint + p] = fmin(fmax(pro / J.promol[p], 0.0), 1.0);
  }
}

// ---------------------------------------------------------------------------
// outer change and end of an outer iteration
// ---------------------------------------------------------------------------

template <typename T, int MODEL>
__global__ void __launch_bounds__(kThreads) k_change(Batch bt) {
  __shared__ double red[kWarps];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  if (MODEL != MODEL_NLIS && J.tgeo) {  // per-atom cutoff: bound of the pair's change term
    const double r = tile_rmin(J, at.atom, at.tile);
    const int s0 = J.shell_off[at.atom], nsh = J.shell_off[at.atom + 1] - s0;
    const double* pn = J.propars + J.par_off[at.atom];
    const double* po = J.propars_old + J.par_off[at.atom];
    const double b = MODEL == MODEL_MBIS ? mbis_bound(pn, nsh, r) + mbis_bound(po, nsh, r)
                                         : basis_bound(J, s0, nsh, pn, po, r);
    if (tile_weight(J, at.tile) * b * b < kSkipRel * J.threshold * J.threshold) {
      if (threadIdx.x == 0) {
        apart_ptr(J, at.atom, QA_CHANGE)[at.tile] = 0.0;
        count_skipped(J, at.tile, 2.0);
      }
      return;
    }
  }
  double acc = 0.0;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const T r = dist_for<T, MODEL>(J, p, at.atom);
    double d;
    if (MODEL == MODEL_BASIS && J.gmat) {
      // stored basis: one sum over exact FP64 coefficient differences
      d = 0.0;
      const int s0 = J.shell_off[at.atom], s1 = J.shell_off[at.atom + 1];
      for (int s = s0; s < s1; ++s)
        d += (J.propars[s] - J.propars_old[s]) * J.gmat[(size_t)s * J.npoint + p];
    } else {
      d = (double)proatom<T, MODEL>(J, at.atom, J.propars, r, p) -
          (double)proatom<T, MODEL>(J, at.atom, J.propars_old, r, p);
    }
    acc += J.w[p] * d * d;
  }
  const double s = block_sum1(acc, red);
  if (threadIdx.x == 0) apart_ptr(J, at.atom, QA_CHANGE)[at.tile] = s;
}

// sum_{i, j in a} dc_i W_a[i][j] dc_j (dc = propars - propars_old) from the
// lower triangle of atom a's Gram block (k_glisa_wgram): one warp, lanes over
// the triangle's entries, summed in a fixed order. The int w (sum_{i in a}
// dc_i g_i)^2 of compute_change (glisa.py:776) for fused gLISA jobs on the
// molecular grid.
__device__ double gram_change(const JobDev& J, int a) {
  const int lane = threadIdx.x & 31;
  const int s0 = J.shell_off[a];
  const int k = J.shell_off[a + 1] - s0;
  const double* W = J.wgram + J.wgoff[a];
  double v = 0.0;
  for (int e = lane; e < k * (k + 1) / 2; e += 32) {
    int i = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
    while (i * (i + 1) / 2 > e) --i;
    while ((i + 1) * (i + 2) / 2 <= e) ++i;
    const int j = e - i * (i + 1) / 2;
    const double di = J.propars[s0 + i] - J.propars_old[s0 + i];
    const double dj = J.propars[s0 + j] - J.propars_old[s0 + j];
    v += (i == j ? 1.0 : 2.0) * W[e] * di * dj;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One block per job: change, entropy, charges (with_charges) and the
// history row (core/iterstock.py:172-188). Warps sum atoms' tiles in
// parallel; thread 0 adds the atoms in order (deterministic).
// One block of kFinishThreads per job: each warp sums whole rows of tile
// partials, so 32 warps take the atoms' sums (and, on the last warp, the
// entropy) in one round instead of several.
constexpr int kFinishThreads = 1024;
__global__ void __launch_bounds__(kFinishThreads) k_outer_finish(Batch bt, int with_charges) {
  __shared__ double ent_s;
  __shared__ double change_s;
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int it = J.mail->i[MI_ITER];
  for (int a = warp; a < J.natom; a += nw) {
    const double s = J.wgram ? gram_change(J, a) : warp_tile_sum(J, apart_ptr(J, a, QA_CHANGE), J.ntile);
    const double pop = with_charges ? warp_tile_sum(J, apart_ptr(J, a, QA_POP), J.ntile) : 0.0;
    if (lane == 0) {
      J.atom_out[a * AO_COUNT + AO_CHANGE] = s;
      if (with_charges) J.charges[a] = J.zpseudo[a] - pop;
    }
  }
  if (warp == nw - 1) {
    const int q = J.fuse ? QJ_ENT_PREV : QJ_ENTROPY;
    const double ent = warp_tile_sum(J, J.jpart + (size_t)q * J.ntile, J.ntile);
    if (lane == 0) ent_s = ent;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double msd = 0.0;
    for (int a = 0; a < J.natom; ++a) msd += J.atom_out[a * AO_COUNT + AO_CHANGE];
    change_s = sqrt(msd);
  }
  __syncthreads();
  if (it < J.maxiter) {
    for (int i = threadIdx.x; i < J.nparam; i += blockDim.x)
      J.hist_propars[(size_t)it * J.nparam + i] = J.propars[i];
    if (with_charges)
      for (int a = threadIdx.x; a < J.natom; a += blockDim.x)
        J.hist_charges[(size_t)it * J.natom + a] = J.charges[a];
  }
  if (threadIdx.x == 0) {
    J.mail->d[MD_CHANGE] = change_s;
    J.mail->d[MD_ENTROPY] = ent_s;
    if (it < J.maxiter) {
      J.hist_ent[it] = ent_s;
      J.hist_chg[it] = change_s;
    }
    J.mail->i[MI_ITER] = it + 1;
    // gLISA: the host's end-of-step tests (error, converged, out of
    // iterations), made here so that queued iterations skip a finished job
    if (J.scheme == SCHEME_GLISA &&
        (J.mail->i[MI_ERR] != 0 || change_s < J.threshold || it + 1 >= J.maxiter))
      J.mail->i[MI_DONE] = 1;
  }
}

// Charges from QA_POP (gLISA end, glisa.py:269-278): one warp per atom.
constexpr int kChargesThreads = 512;
__global__ void __launch_bounds__(kChargesThreads) k_charges(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  const int warp = threadIdx.x >> 5;
  for (int a = warp; a < J.natom; a += kChargesThreads / 32) {
    const double pop = warp_tile_sum(J, apart_ptr(J, a, QA_POP), J.ntile);
    if ((threadIdx.x & 31) == 0) J.charges[a] = J.zpseudo[a] - pop;
  }
}

// Mixed precision only: the inner change of FP32-evaluated pro-atoms has a
// noise floor (about 1e-9 of the pro-atom's L2 norm), so the FP32 inner solve
// stops at 1000 x the inner threshold; the exact convergence to the
// threshold happens in the FP64 outer iterations that finish a mixed job.
__device__ __forceinline__ bool mixed_stalled(const JobDev& J, int a, double change) {
  (void)a;
  return J.mixed == PH_FP32 && change < 1e3 * J.inner_threshold;
}

__global__ void k_count_active(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  const int lane = threadIdx.x & 31;
  int c = 0;
  for (int a = lane; a < J.natom; a += 32) c += J.active[a];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0) J.mail->i[MI_NACTIVE] = c;
}

__global__ void k_inner_init(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  for (int i = threadIdx.x; i < J.nparam; i += blockDim.x) {
    J.cur[i] = J.propars[i];
    J.prev[i] = J.propars[i];
  }
  for (int a = threadIdx.x; a < J.natom; a += blockDim.x) {
    J.active[a] = 1;
    J.inner_it[a] = 0;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = 1e300;
  }
  if (J.mixed)
    for (int s = threadIdx.x; s < J.nshell; s += blockDim.x) fill_fco(J, s, J.propars, J.propars);
  if (threadIdx.x == 0) {
    J.mail->i[MI_NACTIVE] = J.natom;
    J.mail->d[MD_INNER_TOTAL] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// MBIS inner fixed point (mbis.py:81-163)
// ---------------------------------------------------------------------------

constexpr int kMbisMaxShell = 7;            // get_nshell() <= 7 (mbis.py:36-46)
constexpr int kMbisQ = 2 * kMbisMaxShell + 1;

template <typename T>
__global__ void __launch_bounds__(kThreads) k_mbis_inner(Batch bt) {
  __shared__ double red[kWarps * kMbisQ];
  __shared__ double out[kMbisQ];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  if (!J.active[at.atom]) return;
  const int nsh = J.shell_off[at.atom + 1] - J.shell_off[at.atom];
  const double* pc = J.cur + J.par_off[at.atom];
  const double* pp = J.prev + J.par_off[at.atom];
  const bool first = J.inner_it[at.atom] == 0;
  if (J.tgeo && J.amax[(size_t)at.atom * J.ntile + at.tile] < (float)J.density_cutoff) {
    // per-atom cutoff: rho_a below the cutoff on the whole tile (the moments
    // are exact zeros); skip if the change term is negligible too
    const double r = tile_rmin(J, at.atom, at.tile);
    const double b = mbis_bound(pc, nsh, r) + (first ? 0.0 : mbis_bound(pp, nsh, r));
    if (tile_weight(J, at.tile) * b * b < kSkipRel * J.inner_threshold * J.inner_threshold) {
      if (threadIdx.x < 2 * nsh) apart_ptr(J, at.atom, QA_INNER + threadIdx.x)[at.tile] = 0.0;
      if (threadIdx.x == 0) {
        apart_ptr(J, at.atom, QA_INNER + kMbisQ - 1)[at.tile] = 0.0;
        count_skipped(J, at.tile, 1.0);
      }
      return;
    }
  }
  T cn[kMbisMaxShell], cs[kMbisMaxShell], pn[kMbisMaxShell], ps[kMbisMaxShell];
#pragma unroll
  for (int k = 0; k < kMbisMaxShell; ++k) {
    const bool on = k < nsh;
    cn[k] = on ? (T)pc[2 * k] : (T)0;
    cs[k] = on ? (T)pc[2 * k + 1] : (T)0;
    pn[k] = on ? (T)pp[2 * k] : (T)0;
    ps[k] = on ? (T)pp[2 * k + 1] : (T)0;
  }
  double acc[kMbisQ];
#pragma unroll
  for (int q = 0; q < kMbisQ; ++q) acc[q] = 0.0;
  const double* ra = J.rhoa + (size_t)at.atom * J.npoint;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const T r = Dist<T>::r(J, p, at.atom);
    T t[kMbisMaxShell];
    T pro = (T)0, oldpro = (T)0;
#pragma unroll
    for (int k = 0; k < kMbisMaxShell; ++k) {
      t[k] = (T)0;
      if (k < nsh) {
        t[k] = slater_shell<T>(cn[k], cs[k], r);
        pro += t[k];
        if (!first) oldpro += slater_shell<T>(pn[k], ps[k], r);
      }
    }
    const double rho = ra[p];
    const double w = J.w[p];
    const bool sick = (rho < J.density_cutoff) || ((double)pro < J.density_cutoff);
    const double ratio = sick ? 0.0 : rho / (double)pro;
#pragma unroll
    for (int k = 0; k < kMbisMaxShell; ++k) {
      const double m0 = w * ((double)t[k] * ratio);
      acc[2 * k] += m0;
      acc[2 * k + 1] += m0 * (double)r;
    }
    const double e = (double)oldpro - (double)pro;
    acc[kMbisQ - 1] += w * e * e;
  }
  block_sum<kMbisQ>(acc, red, out);
  if (threadIdx.x < 2 * nsh) apart_ptr(J, at.atom, QA_INNER + threadIdx.x)[at.tile] = out[threadIdx.x];
  if (threadIdx.x == 0) apart_ptr(J, at.atom, QA_INNER + kMbisQ - 1)[at.tile] = out[kMbisQ - 1];
}

// One warp per atom: N_k <- m0_k, S_k <- 3 m0_k / m1_k, convergence test.
// NLIS / GMBIS inner iteration (nlis.py:99-195), per (atom, tile): with the
// unit shells u_k = n S^(3/n) exp(-S r^n) / (4 pi Gamma(3/n)) (prefactors
// formed once per block) and t_k = N_k u_k: m0_k = int w t_k rho_a / pro,
// m1_k = int w u_k (rho_a / pro) r^n_k (the reference's m1, without N_k), and
// int w (oldpro - pro)^2 for the inner change. FP64.
__global__ void __launch_bounds__(kThreads) k_nlis_inner(Batch bt) {
  __shared__ double red[kWarps * kMbisQ];
  __shared__ double out[kMbisQ];
  __shared__ double pu[2][kMbisMaxShell];  // unit-shell prefactors of cur, prev
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  if (!J.active[at.atom]) return;
  const int nsh = J.shell_off[at.atom + 1] - J.shell_off[at.atom];
  const double* pc = J.cur + J.par_off[at.atom];
  const double* pp = J.prev + J.par_off[at.atom];
  const bool first = J.inner_it[at.atom] == 0;
  if (threadIdx.x < 2 * nsh) {
    const int k = threadIdx.x % nsh;
    const double* q = threadIdx.x < nsh ? pc : pp;
    const double n = q[3 * k + 2];
    pu[threadIdx.x / nsh][k] = n * pow(q[3 * k + 1], 3.0 / n) / (4.0 * M_PI * tgamma(3.0 / n));
  }
  __syncthreads();
  double acc[kMbisQ];
#pragma unroll
  for (int q = 0; q < kMbisQ; ++q) acc[q] = 0.0;
  const double* ra = J.rhoa + (size_t)at.atom * J.npoint;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const double r = Dist<double>::r(J, p, at.atom);
    double u[kMbisMaxShell], rn[kMbisMaxShell];
    double pro = 0.0, oldpro = 0.0;
#pragma unroll
    for (int k = 0; k < kMbisMaxShell; ++k) {
      u[k] = 0.0;
      rn[k] = 0.0;
      if (k < nsh) {
        rn[k] = nlis_rn(pc[3 * k + 2], r);
        u[k] = pu[0][k] * exp(-pc[3 * k + 1] * rn[k]);
        pro += pc[3 * k] * u[k];
        if (!first) oldpro += pp[3 * k] * pu[1][k] * exp(-pp[3 * k + 1] * nlis_rn(pp[3 * k + 2], r));
      }
    }
    const double rho = ra[p];
    const double w = J.w[p];
    const bool sick = (rho < J.density_cutoff) || (pro < J.density_cutoff);
    const double ratio = sick ? 0.0 : rho / pro;
#pragma unroll
    for (int k = 0; k < kMbisMaxShell; ++k) {
      if (k < nsh) {
        const double wu = w * u[k] * ratio;
        acc[2 * k] += wu * pc[3 * k];
        acc[2 * k + 1] += wu * rn[k];
      }
    }
    const double e = oldpro - pro;
    acc[kMbisQ - 1] += w * e * e;
  }
  block_sum<kMbisQ>(acc, red, out);
  if (threadIdx.x < 2 * nsh) apart_ptr(J, at.atom, QA_INNER + threadIdx.x)[at.tile] = out[threadIdx.x];
  if (threadIdx.x == 0) apart_ptr(J, at.atom, QA_INNER + kMbisQ - 1)[at.tile] = out[kMbisQ - 1];
}

// NLIS update per atom: N_k <- m0_k, S_k <- 3 / (n_k m1_k) (1e-5 where m1_k is
// within 1e-8 of zero, numpy.isclose), n_k fixed; convergence as MBIS.
__global__ void k_nlis_update(Batch bt) {
  int a;
  const JobDev& J = decode_local(bt, a);
  if (!J.active[a]) return;
  const int lane = threadIdx.x & 31;
  const int nsh = J.shell_off[a + 1] - J.shell_off[a];
  double m[2 * kMbisMaxShell];
  for (int q = 0; q < 2 * nsh; ++q) m[q] = warp_tile_sum(J, apart_ptr(J, a, QA_INNER + q), J.ntile);
  const double chg2 = warp_tile_sum(J, apart_ptr(J, a, QA_INNER + kMbisQ - 1), J.ntile);
  if (lane != 0) return;
  const int it = J.inner_it[a];
  const double change = (it == 0) ? 1e100 : sqrt(chg2);
  double* pc = J.cur + J.par_off[a];
  double* pp = J.prev + J.par_off[a];
  double* pr = J.propars + J.par_off[a];
  double nw[3 * kMbisMaxShell];
  for (int k = 0; k < nsh; ++k) {
    const double n = pc[3 * k + 2], m1 = m[2 * k + 1];
    nw[3 * k] = m[2 * k];
    nw[3 * k + 1] = fabs(m1) <= 1e-8 ? 1e-5 : 3.0 / (m1 * n);
    nw[3 * k + 2] = n;
  }
  const bool conv = change < J.inner_threshold;
  if (conv || it + 1 >= J.inner_maxiter) {
    for (int q = 0; q < 3 * nsh; ++q) pr[q] = nw[q];
    J.active[a] = 0;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = change;
    atomicAdd(&J.mail->d[MD_INNER_TOTAL], (double)(it + 1));
    if (!conv) atomicOr(&J.mail->i[MI_WARN], W_INNER);
  } else {
    for (int q = 0; q < 3 * nsh; ++q) {
      pp[q] = pc[q];
      pc[q] = nw[q];
    }
    J.inner_it[a] = it + 1;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = change;
  }
}

__global__ void k_mbis_update(Batch bt) {
  int a;
  const JobDev& J = decode_local(bt, a);
  if (!J.active[a]) return;
  const int lane = threadIdx.x & 31;
  const int nsh = J.shell_off[a + 1] - J.shell_off[a];
  double m[2 * kMbisMaxShell];
  for (int q = 0; q < 2 * nsh; ++q) m[q] = warp_tile_sum(J, apart_ptr(J, a, QA_INNER + q), J.ntile);
  const double chg2 = warp_tile_sum(J, apart_ptr(J, a, QA_INNER + kMbisQ - 1), J.ntile);
  if (lane != 0) return;
  const int it = J.inner_it[a];
  const double change = (it == 0) ? 1e100 : sqrt(chg2);
  double* pc = J.cur + J.par_off[a];
  double* pp = J.prev + J.par_off[a];
  double* pr = J.propars + J.par_off[a];
  double nw[2 * kMbisMaxShell];
  for (int k = 0; k < nsh; ++k) {
    nw[2 * k] = m[2 * k];
    nw[2 * k + 1] = 3.0 * m[2 * k] / m[2 * k + 1];
  }
  const bool conv = change < J.inner_threshold || mixed_stalled(J, a, change);
  if (conv || it + 1 >= J.inner_maxiter) {
    for (int q = 0; q < 2 * nsh; ++q) pr[q] = nw[q];
    J.active[a] = 0;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = change;
    atomicAdd(&J.mail->d[MD_INNER_TOTAL], (double)(it + 1));
    if (!conv) atomicOr(&J.mail->i[MI_WARN], W_INNER);
  } else {
    for (int q = 0; q < 2 * nsh; ++q) {
      pp[q] = pc[q];
      pc[q] = nw[q];
    }
    J.inner_it[a] = it + 1;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = change;
    if (J.mixed)
      for (int s = J.shell_off[a]; s < J.shell_off[a + 1]; ++s) fill_fco(J, s, J.cur, J.prev);
  }
}

// ---------------------------------------------------------------------------
// GISA (gisa.py:257-279, 348-421)
// ---------------------------------------------------------------------------


// q-vector moments sum_p w g_k rho_a (unit-population shells).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_basis_qvec(Batch bt) {
  __shared__ double red[kWarps * kMaxShells];
  __shared__ double out[kMaxShells];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  const int s0 = J.shell_off[at.atom];
  const int nsh = J.shell_off[at.atom + 1] - s0;
  double acc[kMaxShells];
#pragma unroll
  for (int q = 0; q < kMaxShells; ++q) acc[q] = 0.0;
  const double* ra = J.rhoa + (size_t)at.atom * J.npoint;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const T r = dist_for<T, MODEL_BASIS>(J, p, at.atom);
    const double wr = J.w[p] * ra[p];
#pragma unroll
    for (int k = 0; k < kMaxShells; ++k)
      if (k < nsh) acc[k] += wr * (double)basis_val<T>(J, s0 + k, p, r);
  }
  block_sum<kMaxShells>(acc, red, out);
  if (threadIdx.x < nsh) apart_ptr(J, at.atom, QA_INNER + threadIdx.x)[at.tile] = out[threadIdx.x];
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Warp minimum with the lowest lane as tie-break; returns the winning lane.
__device__ __forceinline__ int warp_argmin_d(double v, double& vmin) {
  int idx = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov < v || (ov == v && oi < idx)) {
      v = ov;
      idx = oi;
    }
  }
  vmin = v;
  return idx;
}

// One warp per atom: the GISA quadratic program (gisa.py:348-421)
//   min 1/2 x^T P x + q^T x,  x >= 0,  sum x = int w rho_a,
// P precomputed per atom (twice the Gaussian overlap), q_k = -2 int w g_k rho_a.
// Exact primal active-set method (Nocedal & Wright, Algorithm 16.3) started at
// x = total/K, the same iteration as the oracle's qp_simplex_nonneg. Lane k
// owns variable k; the equality-constrained step on the free set solves
// P_FF u = -g_F and P_FF v = 1 with one Cholesky factor, lambda = sum u / sum v,
// p = u - lambda v.
__global__ void k_gisa_qp(Batch bt) {
  __shared__ double Ps[kMaxShells][kMaxShells + 1];
  __shared__ double M[kMaxShells][kMaxShells + 1];
  __shared__ double rhs[2][kMaxShells];
  __shared__ int bad;
  int a;
  const JobDev& J = decode_local(bt, a);
  const int lane = threadIdx.x & 31;
  const int s0 = J.shell_off[a];
  const int n = J.shell_off[a + 1] - s0;
  double qi = 0.0;
  for (int k = 0; k < n; ++k) {
    const double v = -2.0 * warp_tile_sum(J, apart_ptr(J, a, QA_INNER + k), J.ntile);
    if (lane == k) qi = v;
  }
  const double pop = warp_tile_sum(J, apart_ptr(J, a, QA_POP), J.ntile);
  const double* P = J.qp_p + J.qp_off[a];
  for (int e = lane; e < n * n; e += 32) Ps[e / n][e % n] = P[e];
  if (lane == 0) bad = 0;
  __syncwarp();
  const bool mine = lane < n;
  // Warm start: the previous outer iteration's solution rescaled to the new
  // population, with its zero populations in the working set. The QP is
  // strictly convex, so the optimum does not depend on the start; the active
  // set rarely changes between outer iterations, so one or two steps finish.
  const double prev = mine ? J.propars[J.par_off[a] + lane] : 0.0;
  const double psum = warp_sum_d((mine && prev > 0.0) ? prev : 0.0);
  double x;
  bool work;
  if (psum > 0.0) {
    x = (mine && prev > 0.0) ? prev * (pop / psum) : 0.0;
    work = mine && !(prev > 0.0);
  } else {
    x = mine ? pop / n : 0.0;
    work = false;
  }
  bool done = false;
  bool at_min = false;  // x minimises the objective on the current free set
  for (int iter = 0; iter < 200 && !done; ++iter) {
    double g = 0.0;
    if (mine) {
      g = qi;
      for (int j = 0; j < n; ++j) g += Ps[lane][j] * __shfl_sync(0xffffffffu, x, j);
    } else {
      for (int j = 0; j < n; ++j) (void)__shfl_sync(0xffffffffu, x, j);
    }
    const unsigned fmask = __ballot_sync(0xffffffffu, mine && !work);
    const int nf = __popc(fmask);
    const bool fr = (fmask >> lane) & 1u;
    const int rank = __popc(fmask & ((1u << lane) - 1u));
    if (at_min) {
      // After a full (unblocked) step x is the subspace minimiser: the
      // multiplier of sum x = total is lambda = -mean(g_F); release the
      // most negative bound multiplier g_i + lambda, or stop. (Testing the
      // next step for zero instead would sit below the rounding noise of
      // the Cholesky solve when P is ill-conditioned.)
      const double lam0 = -warp_sum_d(fr ? g : 0.0) / (double)(nf > 0 ? nf : 1);
      const double gmax = warp_max_d(mine ? fabs(g) : 0.0);
      double mumin;
      const int jmin = warp_argmin_d((mine && work) ? g + lam0 : 1e300, mumin);
      if (!(mumin < -1e-12 * fmax(1.0, gmax))) {
        done = true;
      } else {
        if (lane == jmin) work = false;
        at_min = false;
      }
      continue;
    }
    if (fr)
      for (int j = 0; j < n; ++j)
        if ((fmask >> j) & 1u) M[rank][__popc(fmask & ((1u << j) - 1u))] = Ps[lane][j];
    __syncwarp();
    for (int k = 0; k < nf; ++k) {  // right-looking Cholesky, lane r owns row r
      if (lane == k) {
        const double d = M[k][k];
        if (!(d > 0.0)) bad = 1;
        M[k][k] = sqrt(fmax(d, 1e-300));
      }
      __syncwarp();
      if (lane > k && lane < nf) M[lane][k] /= M[k][k];
      __syncwarp();
      if (lane > k && lane < nf)
        for (int j = k + 1; j <= lane; ++j) M[lane][j] -= M[lane][k] * M[j][k];
      __syncwarp();
    }
    if (fr) {
      rhs[0][rank] = -g;
      rhs[1][rank] = 1.0;
    }
    __syncwarp();
    if (lane < 2) {  // two triangular solves, one per lane
      double* b = rhs[lane];
      for (int i = 0; i < nf; ++i) {
        double v = b[i];
        for (int j = 0; j < i; ++j) v -= M[i][j] * b[j];
        b[i] = v / M[i][i];
      }
      for (int i = nf - 1; i >= 0; --i) {
        double v = b[i];
        for (int j = i + 1; j < nf; ++j) v -= M[j][i] * b[j];
        b[i] = v / M[i][i];
      }
    }
    __syncwarp();
    const double u = fr ? rhs[0][rank] : 0.0;
    const double v = fr ? rhs[1][rank] : 0.0;
    const double lam = warp_sum_d(u) / warp_sum_d(v);
    const double p = fr ? u - lam * v : 0.0;
    const double pmax = warp_max_d(fabs(p));
    const double xmax = warp_max_d(mine ? fmax(1.0, fabs(x)) : 1.0);
    if (pmax <= 1e-14 * xmax) {
      at_min = true;
      continue;
    }
    double amin;
    const int blk = warp_argmin_d((fr && p < 0.0) ? -x / p : 1e300, amin);
    const double alpha = amin < 1.0 ? amin : 1.0;
    x += alpha * p;
    if (amin < 1.0) {
      if (lane == blk) {
        x = 0.0;
        work = true;
      }
    } else {
      at_min = true;
    }
  }
  if (!done || bad) {
    if (lane == 0) atomicOr(&J.mail->i[MI_ERR], E_QP);
  }
  if (mine) J.propars[J.par_off[a] + lane] = x;
  const double s = warp_sum_d(mine ? x : 0.0);
  const unsigned neg = __ballot_sync(0xffffffffu, mine && x < J.negative_cutoff);
  if (lane == 0) {
    if (fabs(s - pop) > J.population_cutoff) atomicOr(&J.mail->i[MI_WARN], W_POPULATION);
    if (neg) atomicOr(&J.mail->i[MI_WARN], W_NEG_PARS);
  }
}

// ---------------------------------------------------------------------------
// aLISA self-consistent solver (alisa.py:193-291)
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(kThreads) k_lisa_sc_inner(Batch bt) {
  constexpr int Q = kMaxShells + 1;
  __shared__ double red[kWarps * Q];
  __shared__ double out[Q];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  if (!J.active[at.atom]) return;
  const int s0 = J.shell_off[at.atom];
  const int nsh = J.shell_off[at.atom + 1] - s0;
  const double* pc = J.cur + J.par_off[at.atom];
  const double* pp = J.prev + J.par_off[at.atom];
  const bool first = J.inner_it[at.atom] == 0;
  if (J.tgeo && J.amax[(size_t)at.atom * J.ntile + at.tile] < (float)J.density_cutoff) {
    // per-atom cutoff (kSkipRel): zero moments, negligible change term
    const double b = first ? 0.0 : basis_bound(J, s0, nsh, pc, pp, tile_rmin(J, at.atom, at.tile));
    if (tile_weight(J, at.tile) * b * b < kSkipRel * J.inner_threshold * J.inner_threshold) {
      if (threadIdx.x < nsh) apart_ptr(J, at.atom, QA_INNER + threadIdx.x)[at.tile] = 0.0;
      if (threadIdx.x == 0) {
        apart_ptr(J, at.atom, QA_INNER + Q - 1)[at.tile] = 0.0;
        count_skipped(J, at.tile, 1.0);
      }
      return;
    }
  }
  double acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0;
  const double* ra = J.rhoa + (size_t)at.atom * J.npoint;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const T r = dist_for<T, MODEL_BASIS>(J, p, at.atom);
    T g[kMaxShells];
    T pro = (T)0, oldpro = (T)0;
#pragma unroll
    for (int k = 0; k < kMaxShells; ++k) {
      g[k] = (T)0;
      if (k < nsh) {
        g[k] = basis_val<T>(J, s0 + k, p, r);
        pro += g[k] * (T)pc[k];
        if (!first) oldpro += g[k] * (T)pp[k];
      }
    }
    const double rho = ra[p];
    const double w = J.w[p];
    const bool sick = (rho < J.density_cutoff) || ((double)pro < J.density_cutoff);
    const double ratio = sick ? 0.0 : rho / (double)pro;
#pragma unroll
    for (int k = 0; k < kMaxShells; ++k)
      if (k < nsh) acc[k] += w * ((double)g[k] * pc[k] * ratio);
    const double e = (double)oldpro - (double)pro;
    acc[Q - 1] += w * e * e;
  }
  block_sum<Q>(acc, red, out);
  if (threadIdx.x < nsh) apart_ptr(J, at.atom, QA_INNER + threadIdx.x)[at.tile] = out[threadIdx.x];
  if (threadIdx.x == 0) apart_ptr(J, at.atom, QA_INNER + Q - 1)[at.tile] = out[Q - 1];
}

__global__ void k_lisa_sc_update(Batch bt) {
  constexpr int Q = kMaxShells + 1;
  int a;
  const JobDev& J = decode_local(bt, a);
  if (!J.active[a]) return;
  const int lane = threadIdx.x & 31;
  const int nsh = J.shell_off[a + 1] - J.shell_off[a];
  double m[kMaxShells];
  for (int k = 0; k < nsh; ++k) m[k] = warp_tile_sum(J, apart_ptr(J, a, QA_INNER + k), J.ntile);
  const double chg2 = warp_tile_sum(J, apart_ptr(J, a, QA_INNER + Q - 1), J.ntile);
  const double pop = warp_tile_sum(J, apart_ptr(J, a, QA_POP), J.ntile);
  if (lane != 0) return;
  const int it = J.inner_it[a];
  const double change = (it == 0) ? 1e100 : sqrt(chg2);
  double* pc = J.cur + J.par_off[a];
  double* pp = J.prev + J.par_off[a];
  double* pr = J.propars + J.par_off[a];
  const bool conv = change < J.inner_threshold || mixed_stalled(J, a, change);
  if (conv || it + 1 >= J.inner_maxiter) {
    double s = 0.0;
    for (int k = 0; k < nsh; ++k) {
      pr[k] = m[k];
      s += m[k];
    }
    J.active[a] = 0;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = change;
    atomicAdd(&J.mail->d[MD_INNER_TOTAL], (double)(it + 1));
    if (!conv) atomicOr(&J.mail->i[MI_WARN], W_INNER);
    else if (fabs(s - pop) > J.population_cutoff) atomicOr(&J.mail->i[MI_WARN], W_POPULATION);
  } else {
    for (int k = 0; k < nsh; ++k) {
      pp[k] = pc[k];
      pc[k] = m[k];
    }
    J.inner_it[a] = it + 1;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = change;
    if (J.mixed)
      for (int s = J.shell_off[a]; s < J.shell_off[a + 1]; ++s) fill_fco(J, s, J.cur, J.prev);
  }
}

// ---------------------------------------------------------------------------
// aLISA Newton / modified Newton (alisa.py:753-938)
// ---------------------------------------------------------------------------

constexpr int kNtQ = kMaxShells + kMaxShells * (kMaxShells + 1) / 2 + 2;  // grad, hess, chg, neg
constexpr int kStage = 256;  // points staged in shared memory per round

// Partial gradient, Hessian, change and negativity count per (atom, tile).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_lisa_newton_inner(Batch bt) {
  __shared__ double gs[kMaxShells][kStage + 1];
  __shared__ double f1[kStage], f2[kStage], fe[kStage], fn[kStage];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  if (!J.active[at.atom]) return;
  const int s0 = J.shell_off[at.atom];
  const int nsh = J.shell_off[at.atom + 1] - s0;
  const int nq = nsh + nsh * (nsh + 1) / 2;
  const double* pc = J.cur + J.par_off[at.atom];
  const double* pp = J.prev + J.par_off[at.atom];
  const bool first = J.inner_it[at.atom] == 0;
  const double* ra = J.rhoa + (size_t)at.atom * J.npoint;
  // Output q owned by thread q: q < nsh -> grad_k; else Hessian entry (k,l), l <= k.
  int qk = 0, ql = 0;
  const int q = threadIdx.x;
  if (q >= nsh && q < nq) {
    int e = q - nsh, k = 0;
    while (e > k) {
      e -= k + 1;
      ++k;
    }
    qk = k;
    ql = e;
  }
  double acc = 0.0, acc_e = 0.0, acc_n = 0.0;
  const int npts = J.tile_points;
  for (int base = 0; base < npts; base += kStage) {
    // stage kStage points: thread t handles point base + t
    {
      const int t = threadIdx.x;
      const int p = at.tile * J.tile_points + base + t;
      double v1 = 0.0, v2 = 0.0, ve = 0.0, vn = 0.0;
      if (t < kStage && base + t < npts && p < J.npoint) {
        const T r = dist_for<T, MODEL_BASIS>(J, p, at.atom);
        T pro = (T)0, oldpro = (T)0;
        for (int k = 0; k < nsh; ++k) {
          const T g = basis_val<T>(J, s0 + k, p, r);
          gs[k][t] = (double)g;
          pro += g * (T)pc[k];
          if (!first) oldpro += g * (T)pp[k];
        }
        const double rho = ra[p];
        const double w = J.w[p];
        const bool sick = (rho < J.density_cutoff) || ((double)pro < J.density_cutoff);
        const double ratio = sick ? 0.0 : rho / (double)pro;
        v1 = w * ratio;
        v2 = sick ? 0.0 : w * (ratio / (double)pro);
        const double e = (double)oldpro - (double)pro;
        ve = w * e * e;
        vn = ((double)pro < J.negative_cutoff) ? 1.0 : 0.0;
      } else if (t < kStage) {
        for (int k = 0; k < nsh; ++k) gs[k][t] = 0.0;
      }
      if (t < kStage) {
        f1[t] = v1;
        f2[t] = v2;
        fe[t] = ve;
        fn[t] = vn;
      }
    }
    __syncthreads();
    if (q < nsh) {
      for (int t = 0; t < kStage; ++t) acc += gs[q][t] * f1[t];
    } else if (q < nq) {
      for (int t = 0; t < kStage; ++t) acc += gs[qk][t] * gs[ql][t] * f2[t];
    } else if (q == nq) {
      for (int t = 0; t < kStage; ++t) acc_e += fe[t];
    } else if (q == nq + 1) {
      for (int t = 0; t < kStage; ++t) acc_n += fn[t];
    }
    __syncthreads();
  }
  if (q < nq) apart_ptr(J, at.atom, QA_INNER + q)[at.tile] = acc;
  else if (q == nq) apart_ptr(J, at.atom, QA_INNER + nq)[at.tile] = acc_e;
  else if (q == nq + 1) apart_ptr(J, at.atom, QA_INNER + nq + 1)[at.tile] = acc_n;
}

// One warp per atom: convergence test, Newton step (exact mode applies it).
__global__ void k_lisa_newton_update(Batch bt) {
  int a;
  const JobDev& J = decode_local(bt, a);
  if (!J.active[a]) return;
  const int lane = threadIdx.x & 31;
  const int nsh = J.shell_off[a + 1] - J.shell_off[a];
  const int nq = nsh + nsh * (nsh + 1) / 2;
  double v[kNtQ];
  for (int q = 0; q < nq + 2; ++q) v[q] = warp_tile_sum(J, apart_ptr(J, a, QA_INNER + q), J.ntile);
  const double pop = warp_tile_sum(J, apart_ptr(J, a, QA_POP), J.ntile);
  if (lane != 0) return;
  const int it = J.inner_it[a];
  const double change = (it == 0) ? 1e100 : sqrt(v[nq]);
  double* pc = J.cur + J.par_off[a];
  double* pp = J.prev + J.par_off[a];
  double* pr = J.propars + J.par_off[a];
  double* dl = J.delta + J.par_off[a];
  if (change < J.inner_threshold) {
    // converged on the current parameters (alisa.py:881-892)
    double s = 0.0;
    for (int k = 0; k < nsh; ++k) {
      pr[k] = pc[k];
      s += pc[k];
    }
    J.active[a] = 0;
    J.atom_out[a * AO_COUNT + AO_INNER_CHANGE] = change;
    atomicAdd(&J.mail->d[MD_INNER_TOTAL], (double)(it + 1));
    if (v[nq + 1] > 0.0) atomicOr(&J.mail->i[MI_ERR], E_NEG_DENSITY);
    if (fabs(s - pop) > J.population_cutoff) atomicOr(&J.mail->i[MI_WARN], W_POPULATION);
    return;
  }
  if (it + 1 >= J.inner_maxiter) {
    J.active[a] = 0;
    atomicOr(&J.mail->i[MI_ERR], E_INNER_NOT_CONV);
    return;
  }
  double H[kMaxShells * kMaxShells], b[kMaxShells];
  for (int k = 0; k < nsh; ++k) b[k] = -1.0 + v[k];  // -1 - df, df = -sum w g ratio
  if (J.solver == SOLVER_BFGS) {
    // quasi-Newton (alisa.py:896-905, algo/quasi_newton.py:24-49): the
    // inverse-Hessian estimate starts at the identity at the first inner
    // iteration and takes the BFGS update
    //   H += (s.y + y H y) s s^T / (s.y)^2 - (H y s^T + s y^T H) / s.y,
    //   y = df - df_old, s the step of the previous line search;
    // the step is H (-1 - df), applied by the positivity line search
    double* hv = J.hinv + (size_t)a * kMaxShells * kMaxShells;
    double* od = J.olddf + J.par_off[a];
    const double* sp = J.step + J.par_off[a];
    if (it == 0) {
      for (int k = 0; k < nsh; ++k)
        for (int l = 0; l < nsh; ++l) hv[k * nsh + l] = k == l ? 1.0 : 0.0;
    } else {
      double y[kMaxShells], hy[kMaxShells], yh[kMaxShells];
      double sy = 0.0;
      for (int k = 0; k < nsh; ++k) {
        y[k] = -v[k] - od[k];
        sy += sp[k] * y[k];
      }
      double yhy = 0.0;
      for (int k = 0; k < nsh; ++k) {
        double a1 = 0.0, a2 = 0.0;
        for (int l = 0; l < nsh; ++l) {
          a1 += hv[k * nsh + l] * y[l];  // (H y)_k
          a2 += y[l] * hv[l * nsh + k];  // (y^T H)_k
        }
        hy[k] = a1;
        yh[k] = a2;
      }
      for (int k = 0; k < nsh; ++k) yhy += y[k] * hy[k];
      const double c1 = (sy + yhy) / (sy * sy);
      for (int k = 0; k < nsh; ++k)
        for (int l = 0; l < nsh; ++l)
          hv[k * nsh + l] += c1 * sp[k] * sp[l] - (hy[k] * sp[l] + sp[k] * yh[l]) / sy;
    }
    for (int k = 0; k < nsh; ++k) {
      double d = 0.0;
      for (int l = 0; l < nsh; ++l) d += hv[k * nsh + l] * b[l];
      dl[k] = d;
      od[k] = -v[k];
    }
    return;
  }
  int e = nsh;
  for (int k = 0; k < nsh; ++k)
    for (int l = 0; l <= k; ++l) {
      H[k * nsh + l] = v[e];
      H[l * nsh + k] = v[e];
      ++e;
    }
  if (!small_chol_solve(H, b, nsh)) {
    J.active[a] = 0;
    atomicOr(&J.mail->i[MI_ERR], E_SINGULAR);
    return;
  }
  if (J.solver == SOLVER_NEWTON) {
    for (int k = 0; k < nsh; ++k) {
      pp[k] = pc[k];
      pc[k] = pc[k] + b[k];
    }
    J.inner_it[a] = it + 1;
  } else {
    for (int k = 0; k < nsh; ++k) dl[k] = b[k];
  }
}

// Line search (modified Newton): bit i set if trial x_i = linspace(tau, 0,
// L)[i] gives a pro-atom <= negative_cutoff somewhere in the tile
// (alisa.py:841-877).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_lisa_ls(Batch bt) {
  __shared__ int red[kWarps];
  __shared__ double trial[32][kMaxShells];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  if (!J.active[at.atom]) return;
  const int s0 = J.shell_off[at.atom];
  const int nsh = J.shell_off[at.atom + 1] - s0;
  const int L = J.linspace_size < 32 ? J.linspace_size : 32;
  const double* pc = J.cur + J.par_off[at.atom];
  const double* dl = J.delta + J.par_off[at.atom];
  for (int e = threadIdx.x; e < L * nsh; e += blockDim.x) {
    const int i = e / nsh, k = e - i * nsh;
    const double x = linspace_at(J.tau, 0.0, L, true, i);
    trial[i][k] = pc[k] + x * dl[k];
  }
  __syncthreads();
  int fail = 0;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    const T r = dist_for<T, MODEL_BASIS>(J, p, at.atom);
    double g[kMaxShells];
    for (int k = 0; k < nsh; ++k) g[k] = (double)basis_val<T>(J, s0 + k, p, r);
    for (int tr = 0; tr < L; ++tr) {
      double v = 0.0;
      for (int k = 0; k < nsh; ++k) v += g[k] * trial[tr][k];
      if (!(v > J.negative_cutoff)) fail |= 1 << tr;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) fail |= __shfl_xor_sync(0xffffffffu, fail, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = fail;
  __syncthreads();
  if (threadIdx.x == 0) {
    int f = 0;
    for (int k = 0; k < kWarps; ++k) f |= red[k];
    J.ls_fail[(size_t)at.atom * J.ntile + at.tile] = f;
  }
}

__global__ void k_lisa_ls_pick(Batch bt) {
  int a;
  const JobDev& J = decode_local(bt, a);
  if (!J.active[a]) return;
  const int lane = threadIdx.x & 31;
  int f = 0;
  for (int t = lane; t < J.ntile; t += 32) f |= J.ls_fail[(size_t)a * J.ntile + t];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) f |= __shfl_xor_sync(0xffffffffu, f, o);
  if (lane != 0) return;
  const int L = J.linspace_size < 32 ? J.linspace_size : 32;
  int pick = -1;
  for (int i = 0; i < L; ++i)
    if (!(f & (1 << i))) {
      pick = i;
      break;
    }
  const int nsh = J.shell_off[a + 1] - J.shell_off[a];
  double* pc = J.cur + J.par_off[a];
  double* pp = J.prev + J.par_off[a];
  const double* dl = J.delta + J.par_off[a];
  if (pick < 0) {
    J.active[a] = 0;
    atomicOr(&J.mail->i[MI_ERR], E_LINESEARCH);
    return;
  }
  const double x = linspace_at(J.tau, 0.0, L, true, pick);
  double* st = J.step ? J.step + J.par_off[a] : nullptr;  // quasi-Newton: the step taken
  for (int k = 0; k < nsh; ++k) {
    pp[k] = pc[k];
    const double sk = x * dl[k];
    pc[k] = pc[k] + sk;
    if (st) st[k] = sk;
  }
  J.inner_it[a] += 1;
}

// ---------------------------------------------------------------------------
// gLISA (glisa.py)
// ---------------------------------------------------------------------------

// G[m][p] = unit-population basis function m at point p (gisa.py:91-106 with
// force_on_molgrid=True).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_glisa_basis(Batch bt) {
  int tile;
  const JobDev& J = decode_local(bt, tile);
  // jobs that recompute their shells keep no basis matrix; float-float planes
  // without an FP64 copy are written by k_glisa_basis_ff
  if (!J.gmat) return;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, tile, i);
    if (p >= J.npoint) continue;
    for (int a = 0; a < J.natom; ++a) {
      const T r = Dist<T>::r(J, p, a);
      for (int s = J.shell_off[a]; s < J.shell_off[a + 1]; ++s) {
        const double g = (double)shell_value<T>(J, s, r);
        const size_t e = (size_t)s * J.npoint + p;
        if (J.gmat) J.gmat[e] = g;
        if (J.gmat32) {
          const float hi = (float)g;
          J.gmat32[e] = hi;
        }
      }
    }
  }
}

// rho0 = G^T c (glisa.py:346-348); d1 = w rho/rho0, d2 = w rho/rho0^2 (0 where
// sick); entropy and negativity partials (glisa.py:441-450, 784).
__global__ void __launch_bounds__(kThreads) k_glisa_pro(Batch bt) {
  __shared__ double red[kWarps * 2];
  __shared__ double out[2];
  int tile;
  const JobDev& J = decode_local(bt, tile);
  if (glisa_idle(J)) return;
  double acc[2] = {0.0, 0.0};
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, tile, i);
    if (p >= J.npoint) continue;
    double rho0 = 0.0;
#pragma unroll 8
    for (int m = 0; m < J.nshell; ++m) rho0 += J.gmat[(size_t)m * J.npoint + p] * J.propars[m];
    const double rho = J.rho[p];
    const double w = J.w[p];
    const bool sick = (rho < J.density_cutoff) || (rho0 < J.density_cutoff);
    const double inv = sick ? 0.0 : 1.0 / rho0;
    const double ratio = rho * inv;
    const double d2 = w * ratio * inv;
    J.dvec1[p] = w * ratio;
    J.dvec2[p] = d2;
    J.rho0[p] = rho0;
    if (J.hess_s) J.hess_s[p] = sqrtf((float)d2);
    if (!sick) acc[0] += w * rho * log(ratio);
    if (rho0 < J.negative_cutoff) acc[1] += 1.0;
  }
  block_sum<2>(acc, red, out);
  if (threadIdx.x == 0) {
    J.jpart[(size_t)QJ_ENTROPY * J.ntile + tile] = out[0];
    J.jpart[(size_t)QJ_NEG * J.ntile + tile] = out[1];
  }
}

// gpart[m][tile] = sum_p G[m][p] v[p] with v = d1 (gradient) or v = hvec
// (Hessian-vector product of the refinement); one warp per row m.
__global__ void __launch_bounds__(kThreads) k_glisa_grad(Batch bt, int use_hvec) {
  int tile;
  const JobDev& J = decode_local(bt, tile);
  if (glisa_idle(J)) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p0 = tile * J.tile_points;
  const int p1 = min(p0 + J.tile_points, J.npoint);
  const double* v = use_hvec ? J.hvec : J.dvec1;
  for (int m = warp; m < J.nshell; m += kWarps) {
    const double* g = J.gmat + (size_t)m * J.npoint;
    double s = 0.0;
#pragma unroll 8
    for (int p = p0 + lane; p < p1; p += 32) s += g[p] * v[p];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) J.gpart[(size_t)m * J.ntile + tile] = s;
  }
}

// Hessian partials: 64x64 tile (ti, tj), ti >= tj, over one point split.
constexpr int kHT = 64;
constexpr int kHK = 16;

__global__ void __launch_bounds__(kThreads) k_glisa_hess(Batch bt) {
  __shared__ double As[kHK][kHT + 1];
  __shared__ double Bs[kHK][kHT + 1];
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  const int npair = J.htiles * (J.htiles + 1) / 2;
  const int split = local / npair;
  int pr = local - split * npair;
  int ti = 0;
  while (pr > ti) {
    pr -= ti + 1;
    ++ti;
  }
  const int tj = pr;
  const int i0 = ti * kHT, j0 = tj * kHT;
  const int chunk = (J.npoint + J.nsplit - 1) / J.nsplit;
  const int pbeg = split * chunk;
  const int pend = min(pbeg + chunk, J.npoint);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
  for (int k0 = pbeg; k0 < pend; k0 += kHK) {
    // load 64 rows x 16 points of each operand; thread -> (row, point) pairs
    for (int e = threadIdx.x; e < kHT * kHK; e += kThreads) {
      const int row = e / kHK, kk = e - row * kHK;
      const int p = k0 + kk;
      const int ia = i0 + row, jb = j0 + row;
      double va = 0.0, vb = 0.0;
      if (p < pend) {
        if (ia < J.nshell) va = J.gmat[(size_t)ia * J.npoint + p] * J.dvec2[p];
        if (jb < J.nshell) vb = J.gmat[(size_t)jb * J.npoint + p];
      }
      As[kk][row] = va;
      Bs[kk][row] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kHK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = As[kk][ty * 4 + u];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = Bs[kk][tx * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += a[u] * b[v];
    }
    __syncthreads();
  }
  const int M = J.nshell;
  double* out = J.hpart + (size_t)split * M * M;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
      if (i < M && j < M && i >= j) out[(size_t)i * M + j] = acc[u][v];
    }
}

// Sum Hessian partials over splits (fixed order) into the lower triangle and
// mirror; gradient rows from gpart.
// kReduceThreads per block: enough warps per SM to keep the partials' loads
// in flight (the job has only nshell^2 / kThreads blocks).
constexpr int kReduceThreads = 1024;
constexpr int kReduceWarps = kReduceThreads / 32;
__global__ void __launch_bounds__(kReduceThreads) k_glisa_reduce(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  const int M = J.nshell;
  const int e = local * kReduceThreads + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (M * M + kThreads - 1) / kThreads;  // this job's K_SQUARE blocks
  if (J.tc && M <= kTcSinglePassShells) {
    // FP32 packed lower triangles of the single-pass tensor-core kernels.
    // The triangle's E elements form chunks of 32 (lane = element); the block
    // takes G = ceil(chunks / nblk) chunks at once, W = warps / G warps per
    // chunk, warp sub of a chunk summing the splits sub, sub + W, ... (16
    // loads in flight per lane, compensated FP32 sums in split order); the
    // W partials of a chunk are combined in FP64 in warp order. G and W
    // depend only on the shell count, so the order is fixed per job.
    __shared__ double wsum[kReduceWarps][32];
    const int E = M * (M + 1) / 2;
    const int chunks = (E + 31) / 32;
    const int G = min((chunks + nblk - 1) / nblk, kReduceWarps);
    const int W = kReduceWarps / G;
    const float* hp = reinterpret_cast<const float*>(J.hpart);
    for (int c0 = local * G; c0 < chunks; c0 += nblk * G) {
      const int g = warp / W, sub = warp - g * W;
      const int c = c0 + g;
      const int ec = c * 32 + lane;
      float s = 0.0f, cc = 0.0f;
      if (g < G && c < chunks && ec < E) {
        constexpr int kU = 16;
        int sp = sub;
        for (; sp + (kU - 1) * W < J.nsplit; sp += kU * W) {
          float x[kU];
#pragma unroll
          for (int u = 0; u < kU; ++u) x[u] = hp[(size_t)(sp + u * W) * E + ec];
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const float t = s + x[u];
            const float bb = t - s;
            cc += (s - (t - bb)) + (x[u] - bb);
            s = t;
          }
        }
        for (; sp < J.nsplit; sp += W) {
          const float x = hp[(size_t)sp * E + ec];
          const float t = s + x;
          const float bb = t - s;
          cc += (s - (t - bb)) + (x - bb);
          s = t;
        }
      }
      wsum[warp][lane] = (double)s + (double)cc;
      __syncthreads();
      if (warp < G) {
        const int cw = c0 + warp;
        const int ew = cw * 32 + lane;
        if (cw < chunks && ew < E) {
          double v = 0.0;
          for (int q = 0; q < W; ++q) v += wsum[warp * W + q][lane];
          int i = (int)((sqrtf(8.0f * (float)ew + 1.0f) - 1.0f) * 0.5f);
          while (i * (i + 1) / 2 > ew) --i;
          while ((i + 1) * (i + 2) / 2 <= ew) ++i;
          const int j = ew - i * (i + 1) / 2;
          J.hess[(size_t)i * M + j] = v;
          J.hess[(size_t)j * M + i] = v;
        }
      }
      __syncthreads();
    }
  } else if (e < M * M) {
    const int i = e / M, j = e - i * M;
    if (i >= j) {
      double s = 0.0;
      for (int sp = 0; sp < J.nsplit; ++sp) s += J.hpart[(size_t)sp * M * M + e];
      J.hess[(size_t)i * M + j] = s;
      J.hess[(size_t)j * M + i] = s;
    }
  }
  // gradient rows: one warp per row, lanes over tiles (four chains, fixed order)
  for (int m = local * kReduceWarps + warp; m < M; m += nblk * kReduceWarps) {
    const double* gp = J.gpart + (size_t)m * J.ntile;
    double h0 = 0.0, h1 = 0.0, h2 = 0.0, h3 = 0.0;
    int t = lane;
    for (; t + 96 < J.ntile; t += 128) {
      h0 += gp[t];
      h1 += gp[t + 32];
      h2 += gp[t + 64];
      h3 += gp[t + 96];
    }
    for (; t < J.ntile; t += 32) h0 += gp[t];
    double h = (h0 + h1) + (h2 + h3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if (lane == 0) J.grad[m] = -h;  // df_i = -int rho g_i / rho0 (glisa.py:452-455)
  }
}

// In-place Cholesky factor of the n x n matrix L (row stride n) by all
// threads of the block (right-looking, one barrier per column); sets *bad on
// a non-positive pivot. At step k warp w updates the rows i > k with
// i = w (mod warps), lanes over the columns k < j <= i, using a copy of the
// unscaled column k (colbuf[0..n)); the lane that updates entry (i, k+1)
// copies it into the next column buffer (colbuf[n..2n)), and the lane that
// updates the next diagonal entry forms the next pivot's square root and
// reciprocal (one FP64 sqrt and division per column, not per thread).
// On return L holds the factor in its lower triangle and its transpose in
// the upper triangle (row-contiguous backward substitution), and dinv[k] =
// 1 / L[k][k]. colbuf: 2n doubles.
__device__ void chol_factor(double* L, int n, int* bad, double* colbuf, double* dinv) {
  __shared__ double piv_s[2], rinv_s[2];  // sqrt(a_kk), 1 / a_kk of the next two steps
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  double* col = colbuf;
  double* nxt = colbuf + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) col[i] = L[(size_t)i * n];
  if (threadIdx.x == 0 && n > 0) {
    const double a = L[0];
    if (!(a > 0.0)) *bad = 1;
    piv_s[0] = sqrt(fmax(a, 1e-300));
    rinv_s[0] = 1.0 / fmax(a, 1e-300);
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const double piv = piv_s[k & 1], rinv = rinv_s[k & 1];
    const double ipiv = piv * rinv;  // 1 / sqrt(a_kk)
    if (threadIdx.x == 0) {
      L[(size_t)k * n + k] = piv;
      dinv[k] = ipiv;
    }
    for (int i = k + 1 + warp; i < n; i += nwarp) {
      const double ci = col[i];
      const double li = ci * rinv;
      double* row = L + (size_t)i * n;
      for (int j = k + 1 + lane; j <= i; j += 32) {
        const double v = row[j] - li * col[j];
        row[j] = v;
        if (j == k + 1) {
          nxt[i] = v;
          if (i == k + 1) {  // the next pivot
            if (!(v > 0.0)) *bad = 1;
            piv_s[(k + 1) & 1] = sqrt(fmax(v, 1e-300));
            rinv_s[(k + 1) & 1] = 1.0 / fmax(v, 1e-300);
          }
        }
      }
      if (lane == 0) {
        const double lik = ci * ipiv;
        row[k] = lik;
        L[(size_t)k * n + i] = lik;
      }
    }
    __syncthreads();
    double* t = col;
    col = nxt;
    nxt = t;
  }
}

constexpr int kSolveSmem = 1024;  // vector length solved in shared memory

// y <- (L L^T)^-1 y by all threads of the block, column by column (one
// barrier per column): forward, z_j = y_j / L_jj and y_i -= L_ij z_j for
// i > j; backward with the rows of L, x_j = z_j / L_jj and z_i -= L_ji x_j
// for i < j. Works in shared memory when n <= kSolveSmem (else in place in y).
__device__ void chol_solve_block(const double* L, const double* dinv, int n, double* y) {
  __shared__ double yb[kSolveSmem], zb[kSolveSmem];
  const bool sm = n <= kSolveSmem;
  double* a = sm ? yb : y;
  double* z = sm ? zb : y;  // in place: z_j overwrites y_j once y_j is no longer read
  if (sm)
    for (int i = threadIdx.x; i < n; i += blockDim.x) yb[i] = y[i];
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const double zj = a[j] * dinv[j];
    const double* col = L + j;  // L[i][j] = col[i n]
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) a[i] -= col[(size_t)i * n] * zj;
    __syncthreads();
    if (threadIdx.x == 0) z[j] = zj;
  }
  __syncthreads();
  for (int j = n - 1; j >= 0; --j) {
    const double xj = z[j] * dinv[j];
    const double* row = L + (size_t)j * n;  // L[j][i], i < j
    for (int i = threadIdx.x; i < j; i += blockDim.x) z[i] -= row[i] * xj;
    __syncthreads();
    if (threadIdx.x == 0) z[j] = xj;
  }
  __syncthreads();
  if (sm)
    for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = zb[i];
  __syncthreads();
}

// Largest free set whose FP32 factor, 1 / diagonal and right-hand side fit
// the Newton step's 200 KB of dynamic shared memory.
constexpr int kNewtonF32Max = 224;

// chol_factor in FP32, for the factor of the tensor-core Hessian: that
// matrix carries ~1e-7 relative error already, so an FP32 factor is as good a
// preconditioner for the FP64-residual refinement as an FP64 one (same
// direction error after each refinement step), at 1/64 of the FP64 cost per
// operation on GB300. Same layout: factor in the lower triangle, its
// transpose in the upper, dinv[k] = 1 / L[k][k].
//
// Right-looking in panels of 8 columns, two block barriers per panel:
//  (1) warp 0 factors the panel's 8 x 8 diagonal block (lane t holds row t;
//      pivots and multipliers travel by shuffles) into pl / pr;
//  (2) one thread per trailing row i forms its 8 panel entries (a triangular
//      solve against pl) and stores them in the upper copy, row k + s;
//  (3) the rank-8 update of the trailing lower triangle in 4 x 4 register
//      tiles by warps 1.., while warp 0 updates the next diagonal block
//      itself and goes straight on to (1) for the next panel.
// The upper copy (rows of finished panels) is never read as part of the
// trailing matrix; one pass at the end mirrors it into the lower triangle.
// Every element's updates are applied panel by panel, columns in order, so
// the factor does not depend on the thread count.
constexpr int kCholPanel = 8;

// (1): the diagonal block at rows / columns kk.. of L, on warp 0
__device__ __forceinline__ void chol_diag_f(float* L, int n, int kk, float (*pl)[kCholPanel],
                                            float* pr, float* dinv, int* bad) {
  const int t = threadIdx.x & 31;
  const int nb = min(kCholPanel, n - kk);
  const float tiny = 1e-37f;
  float a[kCholPanel], lrow[kCholPanel];
#pragma unroll
  for (int u = 0; u < kCholPanel; ++u) {
    a[u] = (t < nb && u <= t) ? L[(size_t)(kk + t) * n + kk + u] : (u == t ? 1.0f : 0.0f);
    lrow[u] = 0.0f;
  }
  bool neg = false;
  float mypiv = 1.0f, myr = 1.0f;
#pragma unroll
  for (int s = 0; s < kCholPanel; ++s) {
    const float d = __shfl_sync(0xffffffffu, a[s], s);
    const float dd = fmaxf(d, tiny);
    const float piv = sqrtf(dd);
    const float r = piv / dd;  // 1 / sqrt(d)
    if (s < nb && !(d > 0.0f)) neg = true;
    if (t == s) {
      mypiv = piv;
      myr = r;
    }
    const float lts = t > s ? a[s] * r : 0.0f;
    lrow[s] = lts;
#pragma unroll
    for (int u = s + 1; u < kCholPanel; ++u) {
      const float lus = __shfl_sync(0xffffffffu, lts, u);
      if (t >= u) a[u] = fmaf(-lts, lus, a[u]);
    }
  }
  if (t < nb) {
    dinv[kk + t] = myr;
    pr[t] = myr;
    L[(size_t)(kk + t) * n + kk + t] = mypiv;
#pragma unroll
    for (int s = 0; s < kCholPanel; ++s) {
      pl[t][s] = lrow[s];
      if (s < t) L[(size_t)(kk + s) * n + kk + t] = lrow[s];  // upper copy
    }
  }
  if (neg && t == 0) *bad = 1;
}

__device__ void chol_factor_f(float* L, int n, int* bad, float* dinv) {
  __shared__ float pl[kCholPanel][kCholPanel];
  __shared__ float pr[kCholPanel];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0 && n > 0) chol_diag_f(L, n, 0, pl, pr, dinv, bad);
  __syncthreads();
  for (int k = 0; k + kCholPanel < n; k += kCholPanel) {
    const int k8 = k + kCholPanel;
    // (2) panel entries of the trailing rows
    for (int i = k8 + threadIdx.x; i < n; i += blockDim.x) {
      const float* row = L + (size_t)i * n + k;
      float x[kCholPanel];
#pragma unroll
      for (int s = 0; s < kCholPanel; ++s) {
        float v = row[s];
#pragma unroll
        for (int u = 0; u < s; ++u) v = fmaf(-x[u], pl[s][u], v);
        x[s] = v * pr[s];
        L[(size_t)(k + s) * n + i] = x[s];
      }
    }
    __syncthreads();
    const float* P = L + (size_t)k * n;  // panel entry s of row i at P[s n + i]
    if (warp == 0) {
      // (3) on the next diagonal block (rows / columns k8 .. k8 + 7), then (1)
      const int nb = min(kCholPanel, n - k8);
      for (int e = lane; e < kCholPanel * (kCholPanel + 1) / 2; e += 32) {
        int a = 0;
        while ((a + 1) * (a + 2) / 2 <= e) ++a;
        const int c = e - a * (a + 1) / 2;
        if (a < nb) {
          const int i = k8 + a, j = k8 + c;
          float v = L[(size_t)i * n + j];
#pragma unroll
          for (int s = 0; s < kCholPanel; ++s) v = fmaf(-P[(size_t)s * n + i], P[(size_t)s * n + j], v);
          L[(size_t)i * n + j] = v;
        }
      }
      __syncwarp();
      chol_diag_f(L, n, k8, pl, pr, dinv, bad);
    } else {
      // (3) on the 4 x 4 tiles below the next diagonal block
      const int m = n - k8;
      const int T = (m + 3) / 4;
      const int ntile = T * (T + 1) / 2 - 3;  // tile rows 0 and 1 lie in the diagonal block
      for (int tt = threadIdx.x - 32; tt < ntile; tt += blockDim.x - 32) {
        const int lin = tt + 3;
        int ti = (int)((sqrtf(8.0f * (float)lin + 1.0f) - 1.0f) * 0.5f);
        while (ti * (ti + 1) / 2 > lin) --ti;
        while ((ti + 1) * (ti + 2) / 2 <= lin) ++ti;
        const int tj = lin - ti * (ti + 1) / 2;
        const int i0 = k8 + 4 * ti, j0 = k8 + 4 * tj;
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + a, j = j0 + c;
            acc[a][c] = (i < n && j <= i) ? L[(size_t)i * n + j] : 0.0f;
          }
#pragma unroll
        for (int s = 0; s < kCholPanel; ++s) {
          float xa[4], yc[4];
#pragma unroll
          for (int a = 0; a < 4; ++a) xa[a] = i0 + a < n ? P[(size_t)s * n + i0 + a] : 0.0f;
#pragma unroll
          for (int c = 0; c < 4; ++c) yc[c] = j0 + c < n ? P[(size_t)s * n + j0 + c] : 0.0f;
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][c] = fmaf(-xa[a], yc[c], acc[a][c]);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + a, j = j0 + c;
            if (i < n && j <= i) L[(size_t)i * n + j] = acc[a][c];
          }
      }
    }
    __syncthreads();
  }
  // lower triangle from the upper copy
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, jj = e - i * n;
    if (jj < i) L[e] = L[(size_t)jj * n + i];
  }
  __syncthreads();
}

// y <- (L L^T)^-1 y by the whole block (L as left by chol_factor_f, y in
// shared memory), in blocks of 32 rows: one warp solves the diagonal block
// (element i in lane i - j0, each column's value broadcast by a shuffle),
// then every thread updates one of the remaining rows with the block's 32
// columns. Forward with the columns of L (the upper copy: conflict-free
// across rows), backward with its rows. Each element receives its updates in
// column order, forward ascending and backward descending, as in a plain
// column-by-column substitution.
__device__ void chol_solve_f(const float* L, const float* dinv, int n, float* y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = (n + 31) / 32;
  for (int jb = 0; jb < nb; ++jb) {
    const int j0 = jb * 32, j1 = min(j0 + 32, n);
    if (warp == 0) {
      const int i = j0 + lane;
      float b = i < n ? y[i] : 0.0f;
      for (int j = j0; j < j1; ++j) {
        const float zj = __shfl_sync(0xffffffffu, b, j - j0) * dinv[j];
        if (i > j && i < n) b = fmaf(-L[(size_t)j * n + i], zj, b);
        else if (i == j) b = zj;
      }
      if (i < n) y[i] = b;
    }
    __syncthreads();
    for (int i = j1 + threadIdx.x; i < n; i += blockDim.x) {
      float b = y[i];
      for (int j = j0; j < j1; ++j) b = fmaf(-L[(size_t)j * n + i], y[j], b);
      y[i] = b;
    }
    __syncthreads();
  }
  for (int jb = nb - 1; jb >= 0; --jb) {
    const int j0 = jb * 32, j1 = min(j0 + 32, n);
    if (warp == 0) {
      const int i = j0 + lane;
      float b = i < n ? y[i] : 0.0f;
      for (int j = j1 - 1; j >= j0; --j) {
        const float xj = __shfl_sync(0xffffffffu, b, j - j0) * dinv[j];
        if (i < j) b = fmaf(-L[(size_t)j * n + i], xj, b);
        else if (i == j) b = xj;
      }
      if (i < n) y[i] = b;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < j0; i += blockDim.x) {
      float b = y[i];
      for (int j = j1 - 1; j >= j0; --j) b = fmaf(-L[(size_t)j * n + i], y[j], b);
      y[i] = b;
    }
    __syncthreads();
  }
}

// Shared memory of the Newton step: the factor (dynamic, when |F|^2 doubles
// fit in kNewtonSmemL) and the two column buffers (when |F| <= kNewtonColMax).
constexpr int kNewtonSmemL = 200 * 1024;
constexpr int kNewtonColMax = 256;
// FP32 factor in shared memory (factor, 1 / diagonal and the right-hand side)
// the step runs on one SM; 16 warps (the panel factor needs no more, and keeps
// its 4 x 4 update tiles in registers at this size)
constexpr int kNewtonThreads = 512;
constexpr int kNewtonWarps = kNewtonThreads / 32;
static_assert(4 * (kNewtonF32Max * kNewtonF32Max + 2 * kNewtonF32Max) <= kNewtonSmemL, "FP32 factor");

__global__ void __launch_bounds__(kNewtonThreads) k_glisa_newton_step(Batch bt, int projected,
                                                                       int fp64_only) {
  extern __shared__ double l_smem[];
  __shared__ double col_smem[2 * kNewtonColMax];
  __shared__ int bad;
  __shared__ int wcount[kNewtonWarps];
  __shared__ int fid[kNewtonF32Max];
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  const int M = J.nshell;
  // fp64_only: the relaunch for jobs whose multi-block FP32 factor failed
  if (fp64_only && J.freeidx[M + 1] != 3) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();  // every thread has read the mark before thread 0 rewrites freeidx
  // free set in shell order: per-warp ballots and a prefix over the warps
  int nf = 0;
  for (int base = 0; base < M; base += kNewtonThreads) {
    const int m = base + threadIdx.x;
    bool f = false;
    if (m < M) f = !projected || J.propars[m] > 0.0 || 1.0 + J.grad[m] < 0.0;
    const unsigned b = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wcount[warp] = __popc(b);
    __syncthreads();
    int off = nf, total = nf;
    for (int w = 0; w < kNewtonWarps; ++w) {
      if (w < warp) off += wcount[w];
      total += wcount[w];
    }
    if (f) {
      const int pos = off + __popc(b & ((1u << lane) - 1u));
      J.freeidx[pos] = m;
      if (pos < kNewtonF32Max) fid[pos] = m;
    }
    __syncthreads();
    nf = total;
  }
  if (threadIdx.x == 0) {
    J.freeidx[M] = nf;
    bad = 0;
  }
  __syncthreads();
  if (J.tc && nf > kNewtonF32Max && !fp64_only) {
    // tensor-core Hessian with a free set above the shared-memory factor:
    // the free block's lower triangle in FP32 into chol, factored and solved
    // by k_glisa_chol_panel / k_glisa_chol_update / k_glisa_chol_solve;
    // freeidx[nshell + 1] = 2 marks the form
    float* Lg = reinterpret_cast<float*>(J.chol);
    for (int e = threadIdx.x; e < nf * nf; e += kNewtonThreads) {
      const int i = e / nf, j = e - i * nf;
      Lg[e] = j <= i ? (float)J.hess[(size_t)J.freeidx[i] * M + J.freeidx[j]] : 0.0f;
    }
    for (int m = threadIdx.x; m < M; m += kNewtonThreads) J.delta[m] = 0.0;
    if (threadIdx.x == 0) J.freeidx[M + 1] = 2;
    return;
  }
  if (J.tc && nf <= kNewtonF32Max && !fp64_only) {
    // tensor-core Hessian: FP32 factor and solve in shared memory; the factor
    // (with 1 / diagonal after it) is kept in chol for the refinement steps,
    // freeidx[nshell + 1] = 1 marks it as FP32
    float* Lf = reinterpret_cast<float*>(l_smem);
    float* dv = Lf + nf * nf;
    float* yv = dv + nf;
    {  // lower triangle (all the factor reads), eight loads in flight per thread
      const double* __restrict__ hs = J.hess;
      const int ne = nf * (nf + 1) / 2;
      constexpr int kBatch = 8;
      for (int e0 = threadIdx.x; e0 < ne; e0 += kBatch * kNewtonThreads) {
        double v[kBatch];
        int dst[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
          const int e = e0 + u * kNewtonThreads;
          dst[u] = -1;
          v[u] = 0.0;
          if (e < ne) {
            int i = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
            while (i * (i + 1) / 2 > e) --i;
            while ((i + 1) * (i + 2) / 2 <= e) ++i;
            const int j = e - i * (i + 1) / 2;
            dst[u] = i * nf + j;
            v[u] = hs[(size_t)fid[i] * M + fid[j]];
          }
        }
#pragma unroll
        for (int u = 0; u < kBatch; ++u)
          if (dst[u] >= 0) Lf[dst[u]] = (float)v[u];
      }
    }
    for (int m = threadIdx.x; m < M; m += kNewtonThreads) J.delta[m] = 0.0;
    __syncthreads();
    chol_factor_f(Lf, nf, &bad, dv);
    if (!bad) {
      for (int i = threadIdx.x; i < nf; i += kNewtonThreads) yv[i] = (float)(-(1.0 + J.grad[fid[i]]));
      __syncthreads();
      chol_solve_f(Lf, dv, nf, yv);
      for (int i = threadIdx.x; i < nf; i += kNewtonThreads) J.delta[fid[i]] = (double)yv[i];
      float* keep = reinterpret_cast<float*>(J.chol);
      for (int e = threadIdx.x; e < nf * nf + nf; e += kNewtonThreads) keep[e] = Lf[e];
      if (threadIdx.x == 0) J.freeidx[M + 1] = 1;
      return;
    }
    // not positive definite in FP32: the FP64 factor below decides
    __syncthreads();
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
  }
  if (J.tc && threadIdx.x == 0) atomicAdd(&J.mail->i[MI_F64_FACTORS], 1);
  if (threadIdx.x == 0) J.freeidx[M + 1] = 0;
  const bool l_in_smem = (size_t)nf * nf * sizeof(double) <= (size_t)kNewtonSmemL;
  double* L = l_in_smem ? l_smem : J.chol;
  for (int e = threadIdx.x; e < nf * nf; e += kNewtonThreads) {
    const int i = e / nf, j = e % nf;
    L[e] = J.hess[(size_t)J.freeidx[i] * M + J.freeidx[j]];
  }
  for (int m = threadIdx.x; m < M; m += kNewtonThreads) J.delta[m] = 0.0;
  __syncthreads();
  // column buffers in shared memory when they fit, else in ctrial (kTrials x
  // nshell, free until the trial set); 1 / diag(L) at ctrial[2 nshell, 3 nshell)
  // (kept for the refinement)
  double* colbuf = nf <= kNewtonColMax ? col_smem : J.ctrial;
  chol_factor(L, nf, &bad, colbuf, J.ctrial + 2 * M);
  double* y = J.keep;  // scratch (the m-newton mask is formed after the step)
  for (int i = threadIdx.x; i < nf; i += kNewtonThreads) y[i] = -(1.0 + J.grad[J.freeidx[i]]);
  __syncthreads();
  chol_solve_block(L, J.ctrial + 2 * M, nf, y);
  for (int i = threadIdx.x; i < nf; i += kNewtonThreads) J.delta[J.freeidx[i]] = y[i];
  if (threadIdx.x == 0 && bad) atomicOr(&J.mail->i[MI_ERR], E_SINGULAR);
  if (l_in_smem)  // the refinement steps read the factor from chol
    for (int e = threadIdx.x; e < nf * nf; e += kNewtonThreads) J.chol[e] = L[e];
}

// FP32 Cholesky of a large free block (freeidx[nshell + 1] = 2, set by
// k_glisa_newton_step), right-looking in panels of kCholBP columns over the
// factor in global memory (nf x nf floats in chol, 1 / diag after them, the
// layout of the shared-memory form: lower triangle and its upper copy), so
// that the trailing updates spread over many blocks:
//   k_glisa_chol_panel(p)   one block per job: the panel's diagonal block
//                           factored by one warp (lane = row), then every
//                           trailing row's panel entries by a triangular
//                           solve (one thread per row), each written with its
//                           upper copy;
//   k_glisa_chol_update(p)  the rank-kCholBP update of the trailing lower
//                           triangle in 64 x 64 tiles (4 x 4 per thread), the
//                           blocks of launch kind K_SQUARE mapped onto the
//                           tiles, the rest return;
//   k_glisa_chol_solve      one block per job: the two triangular solves
//                           (chol_solve_f on the global factor) into delta.
// A non-positive pivot marks the job (freeidx[nshell + 1] = 3) for the FP64
// factor of k_glisa_newton_step (fp64_only). Every element receives its
// updates panel by panel in column order, independent of the block count.
constexpr int kCholBP = 32;
constexpr int kCholTile = 64;

__device__ __forceinline__ bool chol_big(const JobDev& J) {
  return !glisa_idle(J) && J.tc && J.freeidx[J.nshell + 1] == 2;
}

__global__ void __launch_bounds__(kThreads) k_glisa_chol_panel(Batch bt, int panel) {
  __shared__ float D[kCholBP][kCholBP + 1];
  __shared__ float Xs[kThreads][kCholBP + 1];  // trailing rows' panel columns
  __shared__ float Rp[kCholBP];                // 1 / the panel's pivots
  int local;
  const JobDev& J = decode_local(bt, local);
  if (!chol_big(J)) return;
  const int n = J.freeidx[J.nshell];
  const int k = panel * kCholBP;
  if (k >= n) return;
  const int nb = min(kCholBP, n - k);
  float* L = reinterpret_cast<float*>(J.chol);
  float* dinv = L + (size_t)n * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < kCholBP * kCholBP; e += kThreads) {
    const int i = e / kCholBP, j = e - i * kCholBP;
    D[i][j] = (i < nb && j <= i) ? L[(size_t)(k + i) * n + k + j] : 0.0f;
  }
  __syncthreads();
  if (warp == 0) {  // lane t holds row t in registers; pivots and multipliers by shuffles
    float a[kCholBP];
#pragma unroll
    for (int u = 0; u < kCholBP; ++u)
      a[u] = (lane < nb && u <= lane) ? D[lane][u] : (u == lane ? 1.0f : 0.0f);
    bool neg = false;
    float mypiv = 1.0f, myr = 1.0f;
#pragma unroll
    for (int s2 = 0; s2 < kCholBP; ++s2) {
      const float d = __shfl_sync(0xffffffffu, a[s2], s2);
      const float piv = sqrtf(fmaxf(d, 1e-37f));
      const float r = 1.0f / piv;
      if (s2 < nb && !(d > 0.0f)) neg = true;
      if (lane == s2) {
        mypiv = piv;
        myr = r;
      }
      const float lts = lane > s2 ? a[s2] * r : 0.0f;  // L[lane][s2]
      if (lane > s2) a[s2] = lts;
#pragma unroll
      for (int u = s2 + 1; u < kCholBP; ++u) {
        const float lus = __shfl_sync(0xffffffffu, lts, u);
        if (lane >= u) a[u] = fmaf(-lts, lus, a[u]);
      }
    }
    if (lane < nb) {
#pragma unroll
      for (int u = 0; u < kCholBP; ++u)
        if (u < lane) D[lane][u] = a[u];
      D[lane][lane] = mypiv;
      dinv[k + lane] = myr;
      Rp[lane] = myr;
    }
    // not positive definite in FP32: the FP64 factor decides (k_glisa_newton_step
    // relaunched with fp64_only); the later panels see the mark and return
    if (neg && lane == 0) J.freeidx[J.nshell + 1] = 3;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nb * nb; e += kThreads) {  // the diagonal block and its upper copy
    const int i = e / nb, j = e - i * nb;
    if (j <= i) {
      L[(size_t)(k + i) * n + k + j] = D[i][j];
      L[(size_t)(k + j) * n + k + i] = D[i][j];
    }
  }
  // the trailing rows' panel entries, kThreads rows at a time: the rows'
  // panel columns staged in shared memory by coalesced loads (a warp per
  // row), solved one thread per row, written back the same way, with the
  // upper copy written by columns (coalesced across the rows)
  for (int rb = k + nb; rb < n; rb += kThreads) {
    const int nr = min(kThreads, n - rb);
    __syncthreads();  // Xs free
    for (int e = threadIdx.x; e < nr * kCholBP; e += kThreads) {
      const int a = e / kCholBP, c = e - a * kCholBP;
      Xs[a][c] = c < nb ? L[(size_t)(rb + a) * n + k + c] : 0.0f;
    }
    __syncthreads();
    if (threadIdx.x < nr) {  // column by column: the later entries' updates are independent
      const int a = threadIdx.x;
      float v[kCholBP];
#pragma unroll
      for (int c = 0; c < kCholBP; ++c) v[c] = Xs[a][c];
#pragma unroll
      for (int s2 = 0; s2 < kCholBP; ++s2) {
        if (s2 < nb) {
          const float x = v[s2] * Rp[s2];
          v[s2] = x;
#pragma unroll
          for (int u = s2 + 1; u < kCholBP; ++u) v[u] = fmaf(-x, D[u][s2], v[u]);
        }
      }
#pragma unroll
      for (int c = 0; c < kCholBP; ++c) Xs[a][c] = v[c];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nr * kCholBP; e += kThreads) {
      const int a = e / kCholBP, c = e - a * kCholBP;
      if (c < nb) L[(size_t)(rb + a) * n + k + c] = Xs[a][c];
    }
    for (int e = threadIdx.x; e < nb * nr; e += kThreads) {
      const int c = e / nr, a = e - c * nr;
      L[(size_t)(k + c) * n + rb + a] = Xs[a][c];
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_glisa_chol_update(Batch bt, int panel) {
  __shared__ float Pi[kCholTile][kCholBP + 1], Pj[kCholTile][kCholBP + 1];
  int local;
  const JobDev& J = decode_local(bt, local);
  if (!chol_big(J)) return;
  const int n = J.freeidx[J.nshell];
  const int k = panel * kCholBP;
  const int r0 = k + kCholBP;  // the trailing matrix starts here
  if (r0 >= n) return;
  const int T = (n - r0 + kCholTile - 1) / kCholTile;
  if (local >= T * (T + 1) / 2) return;
  int bi = (int)((sqrtf(8.0f * (float)local + 1.0f) - 1.0f) * 0.5f);
  while (bi * (bi + 1) / 2 > local) --bi;
  while ((bi + 1) * (bi + 2) / 2 <= local) ++bi;
  const int bj = local - bi * (bi + 1) / 2;
  const int i0 = r0 + kCholTile * bi, j0 = r0 + kCholTile * bj;
  const float* L = reinterpret_cast<const float*>(J.chol);
  for (int e = threadIdx.x; e < kCholTile * kCholBP; e += kThreads) {
    const int a = e / kCholBP, c = e - a * kCholBP;
    Pi[a][c] = i0 + a < n ? L[(size_t)(i0 + a) * n + k + c] : 0.0f;
    Pj[a][c] = j0 + a < n ? L[(size_t)(j0 + a) * n + k + c] : 0.0f;
  }
  __syncthreads();
  float* Lw = reinterpret_cast<float*>(J.chol);
  const int ti = (threadIdx.x >> 4) * 4, tj = (threadIdx.x & 15) * 4;  // 4 x 4 elements per thread
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = 0.0f;
#pragma unroll 8
  for (int s2 = 0; s2 < kCholBP; ++s2) {
    float xa[4], yc[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) xa[a] = Pi[ti + a][s2];
#pragma unroll
    for (int c = 0; c < 4; ++c) yc[c] = Pj[tj + c][s2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][c] = fmaf(xa[a], yc[c], acc[a][c]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ti + a, j = j0 + tj + c;
      if (i < n && j <= i) Lw[(size_t)i * n + j] -= acc[a][c];
    }
}

// y <- (L L^T)^-1 y with L in global memory (the multi-block factor): as
// chol_solve_f, with each 32 x 32 diagonal block staged in shared memory
// first, so that the sequential part on warp 0 reads shared memory; the
// off-diagonal updates read rows of L (coalesced across the threads).
__device__ void chol_solve_global(const float* L, const float* dinv, int n, float* y) {
  __shared__ float B[32][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = (n + 31) / 32;
  for (int jb = 0; jb < nb; ++jb) {
    const int j0 = jb * 32, j1 = min(j0 + 32, n), w = j1 - j0;
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {  // B[c][r] = L[j0 + c][j0 + r] (upper copy: L_rc)
      const int c = e >> 5, r = e & 31;
      B[c][r] = (c < w && r < w) ? L[(size_t)(j0 + c) * n + j0 + r] : 0.0f;
    }
    __syncthreads();
    if (warp == 0) {
      const int i = j0 + lane;
      float b = i < n ? y[i] : 0.0f;
      for (int j = 0; j < w; ++j) {
        const float zj = __shfl_sync(0xffffffffu, b, j) * dinv[j0 + j];
        if (lane > j && lane < w) b = fmaf(-B[j][lane], zj, b);
        else if (lane == j) b = zj;
      }
      if (i < n) y[i] = b;
    }
    __syncthreads();
    for (int i = j1 + threadIdx.x; i < n; i += blockDim.x) {
      float b = y[i];
      for (int j = j0; j < j1; ++j) b = fmaf(-L[(size_t)j * n + i], y[j], b);
      y[i] = b;
    }
  }
  for (int jb = nb - 1; jb >= 0; --jb) {
    const int j0 = jb * 32, j1 = min(j0 + 32, n), w = j1 - j0;
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {  // B[c][r] = L[j0 + c][j0 + r] (lower: L_cr)
      const int c = e >> 5, r = e & 31;
      B[c][r] = (c < w && r < w) ? L[(size_t)(j0 + c) * n + j0 + r] : 0.0f;
    }
    __syncthreads();
    if (warp == 0) {
      const int i = j0 + lane;
      float b = i < n ? y[i] : 0.0f;
      for (int j = w - 1; j >= 0; --j) {
        const float xj = __shfl_sync(0xffffffffu, b, j) * dinv[j0 + j];
        if (lane < j) b = fmaf(-B[j][lane], xj, b);
        else if (lane == j) b = xj;
      }
      if (i < n) y[i] = b;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < j0; i += blockDim.x) {
      float b = y[i];
      for (int j = j1 - 1; j >= j0; --j) b = fmaf(-L[(size_t)j * n + i], y[j], b);
      y[i] = b;
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kNewtonThreads) k_glisa_chol_solve(Batch bt) {
  extern __shared__ float ysm[];
  int local;
  const JobDev& J = decode_local(bt, local);
  if (!chol_big(J)) return;
  const int M = J.nshell;
  const int n = J.freeidx[M];
  const float* L = reinterpret_cast<const float*>(J.chol);
  for (int i = threadIdx.x; i < n; i += kNewtonThreads) ysm[i] = (float)(-(1.0 + J.grad[J.freeidx[i]]));
  __syncthreads();
  chol_solve_global(L, L + (size_t)n * n, n, ysm);
  for (int i = threadIdx.x; i < n; i += kNewtonThreads) J.delta[J.freeidx[i]] = (double)ysm[i];
}

// Hessian-vector product with the exact FP64 Hessian, first half:
// hvec[p] = (w rho / rho0^2)(p) * sum_m G[m][p] delta[m]. The second half is
// k_glisa_grad(use_hvec = 1): gpart[m][tile] = sum_p G[m][p] hvec[p].
__global__ void __launch_bounds__(kThreads) k_glisa_hv(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  const int p = local * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  double u = 0.0;
#pragma unroll 8
  for (int m = 0; m < J.nshell; ++m) u += J.gmat[(size_t)m * J.npoint + p] * J.delta[m];
  J.hvec[p] = J.dvec2[p] * u;
}

// Row sums of the per-tile partials: hsum[m] = sum over tiles of gpart[m]
// (the exact product H delta of the refinement), one warp per row, lanes over
// tiles in four chains combined in a fixed order; many blocks, so the sums
// leave the one-block refinement kernel.
__global__ void __launch_bounds__(kThreads) k_glisa_gsum(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  if (!glisa_refine_now(J)) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (J.nshell * J.nshell + kThreads - 1) / kThreads;  // this job's K_SQUARE blocks
  for (int m = local * kWarps + warp; m < J.nshell; m += nblk * kWarps) {
    const double* gp = J.gpart + (size_t)m * J.ntile;
    double h0 = 0.0, h1 = 0.0, h2 = 0.0, h3 = 0.0;
    int t = lane;
    for (; t + 96 < J.ntile; t += 128) {
      h0 += gp[t];
      h1 += gp[t + 32];
      h2 += gp[t + 64];
      h3 += gp[t + 96];
    }
    for (; t < J.ntile; t += 32) h0 += gp[t];
    double h = (h0 + h1) + (h2 + h3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if (lane == 0) J.hsum[m] = h;
  }
}

// One step of iterative refinement of the Newton system on the free set:
// r = (-1 - df)_F - (H delta)_F with the exact FP64 product, then
// delta_F += (L L^T)^-1 r with the factor of the (tensor-core) Hessian.
__global__ void __launch_bounds__(kThreads) k_glisa_refine(Batch bt) {
  extern __shared__ double l_smem[];
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  if (!glisa_refine_now(J)) return;
  const int M = J.nshell;
  const int nf = J.freeidx[M];
  const bool f32 = J.freeidx[M + 1] != 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double* r = J.keep;
  (void)lane;
  (void)warp;
  for (int i = threadIdx.x; i < nf; i += kThreads) {  // H delta rows from k_glisa_gsum
    const int m = J.freeidx[i];
    r[i] = -(1.0 + J.grad[m]) - J.hsum[m];
  }
  __syncthreads();
  if (f32 && nf > kNewtonF32Max) {  // the multi-block FP32 factor: solved in place
    float* yv = reinterpret_cast<float*>(l_smem);
    for (int i = threadIdx.x; i < nf; i += kThreads) yv[i] = (float)r[i];
    __syncthreads();
    const float* keep = reinterpret_cast<const float*>(J.chol);
    chol_solve_global(keep, keep + (size_t)nf * nf, nf, yv);
    for (int i = threadIdx.x; i < nf; i += kThreads) J.delta[J.freeidx[i]] += (double)yv[i];
    return;
  }
  if (f32) {  // FP32 factor of k_glisa_newton_step: copy it in, the block solves
    float* Lf = reinterpret_cast<float*>(l_smem);
    float* yv = Lf + nf * nf + nf;
    const float* keep = reinterpret_cast<const float*>(J.chol);
    const int ne = nf * nf + nf;
    for (int e = threadIdx.x; e < ne / 4; e += kThreads)  // chol and the dynamic shared base are 16-byte aligned
      reinterpret_cast<float4*>(Lf)[e] = reinterpret_cast<const float4*>(keep)[e];
    for (int e = ne / 4 * 4 + threadIdx.x; e < ne; e += kThreads) Lf[e] = keep[e];
    for (int i = threadIdx.x; i < nf; i += kThreads) yv[i] = (float)r[i];
    __syncthreads();
    chol_solve_f(Lf, Lf + nf * nf, nf, yv);
    for (int i = threadIdx.x; i < nf; i += kThreads) J.delta[J.freeidx[i]] += (double)yv[i];
    return;
  }
  chol_solve_block(J.chol, J.ctrial + 2 * M, nf, r);
  for (int i = threadIdx.x; i < nf; i += kThreads) J.delta[J.freeidx[i]] += r[i];
}

// Projected-Newton trial points c_t = max(c + 2^-t delta, 0), t < kTrials,
// and the list of shells the projection clips at the full step (the clipped
// set of every shorter step is a subset of it). A block of NT threads (tms:
// kTrialSetSmem ints of shared memory, wcount: NT / 32).
constexpr int kTrialSetSmem = 2048;  // shells whose clip steps are sorted in shared memory

template <int NT>
__device__ void trial_set_body(const JobDev& J, int* tms, int* wcount) {
  const int M = J.nshell;
  for (int e = threadIdx.x; e < kTrials * M; e += NT) {
    const int t = e / M, m = e - t * M;
    const double a = ldexp(1.0, -t);
    J.ctrial[e] = fmax(J.propars[m] + a * J.delta[m], 0.0);
  }
  // clipped shells with the number of trials t_m at which they are clipped
  // (c + 2^-t delta < 0 for t < t_m), sorted by t_m, largest first, shells
  // of equal t_m in index order
  int* tm = J.clip + M + 1;
  if (M <= kTrialSetSmem) {  // all threads: t_m per shell, then one ballot compaction per t
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int m = threadIdx.x; m < M; m += NT) {
      int t = 0;
      if (J.propars[m] + J.delta[m] < 0.0) {
        t = 1;
        while (t < kTrials && J.propars[m] + ldexp(1.0, -t) * J.delta[m] < 0.0) ++t;
      }
      tms[m] = t;
    }
    __syncthreads();
    int n = 0;
    for (int t = kTrials; t >= 1; --t) {
      for (int base = 0; base < M; base += NT) {
        const int m = base + threadIdx.x;
        const bool f = m < M && tms[m] == t;
        const unsigned b = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wcount[warp] = __popc(b);
        __syncthreads();
        int off = n, total = n;
        for (int w = 0; w < NT / 32; ++w) {
          if (w < warp) off += wcount[w];
          total += wcount[w];
        }
        if (f) {
          const int k = off + __popc(b & ((1u << lane) - 1u));
          J.clip[k] = m;
          tm[k] = t;
        }
        __syncthreads();
        n = total;
      }
    }
    if (threadIdx.x == 0) J.clip[M] = n;
  } else if (threadIdx.x == 0) {
    int n = 0;
    for (int m = 0; m < M; ++m) {
      if (!(J.propars[m] + J.delta[m] < 0.0)) continue;
      int t = 1;
      while (t < kTrials && J.propars[m] + ldexp(1.0, -t) * J.delta[m] < 0.0) ++t;
      int k = n++;
      while (k > 0 && tm[k - 1] < t) {
        J.clip[k] = J.clip[k - 1];
        tm[k] = tm[k - 1];
        --k;
      }
      J.clip[k] = m;
      tm[k] = t;
    }
    J.clip[M] = n;
  }
  if (J.clipf) {  // float pairs (c hi, c lo, delta hi, delta lo) of the clipped shells
    __syncthreads();
    const int n = J.clip[M];
    for (int k = threadIdx.x; k < n; k += NT) {
      const int m = J.clip[k];
      const double c = J.propars[m], d = J.delta[m];
      const float ch = (float)c, dh = (float)d;
      J.clipf[4 * k] = ch;
      J.clipf[4 * k + 1] = (float)(c - (double)ch);
      J.clipf[4 * k + 2] = dh;
      J.clipf[4 * k + 3] = (float)(d - (double)dh);
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_glisa_trial_set(Batch bt) {
  __shared__ int tms[kTrialSetSmem];
  __shared__ int wcount[kWarps];
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  trial_set_body<kThreads>(J, tms, wcount);
}

// Line-search mask (glisa.py:688-699 with utils.py:556-577): per atom, the
// most diffuse shells with |c| < 1e-4 and a negative step stay fixed.
__global__ void k_glisa_keep(Batch bt) {
  int a;
  const JobDev& J = decode_local(bt, a);
  if ((threadIdx.x & 31) != 0) return;
  const int s0 = J.shell_off[a];
  const int n = J.shell_off[a + 1] - s0;
  int order[kMaxShells];
  for (int k = 0; k < n; ++k) order[k] = k;
  // stable insertion sort by exponent (numpy argsort default is not stable,
  // but exponents within an atom are distinct)
  for (int k = 1; k < n; ++k) {
    const int v = order[k];
    int j = k - 1;
    while (j >= 0 && J.sh_alpha[s0 + order[j]] > J.sh_alpha[s0 + v]) {
      order[j + 1] = order[j];
      --j;
    }
    order[j + 1] = v;
  }
  for (int k = 0; k < n; ++k) J.keep[s0 + k] = 1.0;
  for (int k = 0; k < n; ++k) {
    const int m = s0 + order[k];
    if (fabs(J.propars[m]) < 1e-4 && J.delta[m] < 0.0) J.keep[m] = 0.0;
    else break;
  }
}

// Validity of trial steps x_i = linspace(tau, 0, L, endpoint=False)[first + i]
// for i < count (<= 64): bit set if some pro-atom of this atom is below
// negative_cutoff in the tile (glisa.py:283-307).
__global__ void __launch_bounds__(kThreads) k_glisa_ls(Batch bt, int first, int count) {
  __shared__ unsigned long long red[kWarps];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  const int s0 = J.shell_off[at.atom];
  const int nsh = J.shell_off[at.atom + 1] - s0;
  unsigned long long fail = 0ull;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    for (int tr = 0; tr < count; ++tr) {
      const double x = linspace_at(J.tau, 0.0, J.linspace_size, false, first + tr);
      double v = 0.0;
      for (int k = 0; k < nsh; ++k) {
        const int m = s0 + k;
        const double c = J.propars[m] + J.keep[m] * (x * J.delta[m]);
        v += c * J.gmat[(size_t)m * J.npoint + p];
      }
      if (v < J.negative_cutoff) fail |= 1ull << tr;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) fail |= __shfl_xor_sync(0xffffffffu, fail, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = fail;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long f = 0ull;
    for (int k = 0; k < kWarps; ++k) f |= red[k];
    reinterpret_cast<unsigned long long*>(J.ls_fail)[(size_t)at.atom * J.ntile + at.tile] = f;
  }
}

// Pick the first valid trial among [first, first+count) and apply it; sets
// MD_LS_X = -1 if none is valid.
__global__ void k_glisa_ls_pick(Batch bt, int first, int count) {
  int local;
  const JobDev& J = decode_local(bt, local);
  const int lane = threadIdx.x & 31;
  const unsigned long long* lf = reinterpret_cast<const unsigned long long*>(J.ls_fail);
  unsigned long long f = 0ull;
  for (int e = lane; e < J.natom * J.ntile; e += 32) f |= lf[e];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) f |= __shfl_xor_sync(0xffffffffu, f, o);
  __shared__ int pick;
  if (lane == 0) {
    pick = -1;
    for (int i = 0; i < count; ++i)
      if (!(f & (1ull << i))) {
        pick = first + i;
        break;
      }
  }
  __syncwarp();
  if (pick < 0) {
    if (lane == 0) J.mail->d[MD_LS_X] = -1.0;
    return;
  }
  const double x = linspace_at(J.tau, 0.0, J.linspace_size, false, pick);
  for (int m = lane; m < J.nshell; m += 32) J.propars[m] = J.propars[m] + J.keep[m] * (x * J.delta[m]);
  if (lane == 0) J.mail->d[MD_LS_X] = x;
}

// Exact Newton: propars += delta. SC: c_m <- c_m int rho g_m / rho0.
__global__ void k_glisa_apply(Batch bt, int mode) {
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  for (int m = threadIdx.x; m < J.nshell; m += blockDim.x) {
    if (mode == 0) J.propars[m] = J.propars[m] + J.delta[m];
    else J.propars[m] = J.propars[m] * (-J.grad[m]);
  }
}

// Change from stored basis values (glisa.py:776 via compute_change).
__global__ void __launch_bounds__(kThreads) k_glisa_change(Batch bt) {
  __shared__ double red[kWarps];
  const JobDev* Jp;
  const AtomTile at = decode_atom_tile(bt, Jp);
  const JobDev& J = *Jp;
  if (glisa_idle(J)) return;
  const int s0 = J.shell_off[at.atom], s1 = J.shell_off[at.atom + 1];
  double acc = 0.0;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, at.tile, i);
    if (p >= J.npoint) continue;
    double r1 = 0.0, r2 = 0.0;
    for (int m = s0; m < s1; ++m) {
      const double g = J.gmat[(size_t)m * J.npoint + p];
      r1 += J.propars[m] * g;
      r2 += J.propars_old[m] * g;
    }
    const double d = r1 - r2;
    acc += J.w[p] * d * d;
  }
  const double s = block_sum1(acc, red);
  if (threadIdx.x == 0) apart_ptr(J, at.atom, QA_CHANGE)[at.tile] = s;
}

// gLISA convergence bookkeeping: negativity of the promolecule used in the
// last iteration and the population check (glisa.py:786-798).
__global__ void k_glisa_check(Batch bt) {
  int local;
  const JobDev& J = decode_local(bt, local);
  const int q = J.fuse ? QJ_NEG_PREV : QJ_NEG;  // the promolecule of the last step's start
  const double neg = warp_tile_sum(J, J.jpart + (size_t)q * J.ntile, J.ntile);
  if ((threadIdx.x & 31) != 0) return;
  if (neg > 0.0) atomicOr(&J.mail->i[MI_ERR], E_NEG_DENSITY);
  double s = 0.0;
  for (int m = 0; m < J.nshell; ++m) s += J.propars[m];
  if (fabs(s - J.mail->d[MD_NELEC]) > J.population_cutoff) atomicOr(&J.mail->i[MI_WARN], W_POPULATION);
}

// ---------------------------------------------------------------------------
// Evaluation service of the host-driven gLISA solvers (DIIS, CDIIS,
// trust-region, quasi-Newton; glisa.py:595-615, 883-1028). The host holds
// the solver state (a few vectors of nshell values); the device does the grid
// work of function_g, _working_matrix, calc_promol_dens and compute_change
// for the populations the host uploads.
// ---------------------------------------------------------------------------

// Per point tile into atom 0's QA_POP slot: what 0: sum w rho0 (rho0 from
// k_glisa_pro); what 1: sum w (sum_m delta_m G_m)^2.
__global__ void __launch_bounds__(kThreads) k_glisa_eval_tiles(Batch bt, int what) {
  __shared__ double red[kWarps];
  int tile;
  const JobDev& J = decode_local(bt, tile);
  double acc = 0.0;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, tile, i);
    if (p >= J.npoint) continue;
    if (what == 0) {
      acc += J.w[p] * J.rho0[p];
    } else {
      double d = 0.0;
#pragma unroll 8
      for (int m = 0; m < J.nshell; ++m) d += J.delta[m] * J.gmat[(size_t)m * J.npoint + p];
      acc += J.w[p] * d * d;
    }
  }
  const double s = block_sum1(acc, red);
  if (threadIdx.x == 0) apart_ptr(J, 0, QA_POP)[tile] = s;
}

// One warp: the totals into the mailbox (fixed summation order).
__global__ void k_glisa_eval_sum(Batch bt, int what) {
  int local;
  const JobDev& J = decode_local(bt, local);
  if (what == 0) {
    const double e = warp_tile_sum(J, J.jpart + (size_t)QJ_ENTROPY * J.ntile, J.ntile);
    const double p = warp_tile_sum(J, apart_ptr(J, 0, QA_POP), J.ntile);
    if ((threadIdx.x & 31) == 0) {
      J.mail->d[MD_EVAL_A] = e;
      J.mail->d[MD_EVAL_B] = p;
    }
  } else if (what == 1) {
    const double s = warp_tile_sum(J, apart_ptr(J, 0, QA_POP), J.ntile);
    if ((threadIdx.x & 31) == 0) J.mail->d[MD_EVAL_A] = sqrt(s);
  } else {
    double msd = 0.0;
    for (int a = 0; a < J.natom; ++a) msd += warp_tile_sum(J, apart_ptr(J, a, QA_CHANGE), J.ntile);
    if ((threadIdx.x & 31) == 0) J.mail->d[MD_EVAL_A] = sqrt(msd);
  }
}

// ---------------------------------------------------------------------------
// gLISA with non-negative populations: projected Newton (the optimum of the
// reference's cvxopt solver, glisa.py:488-571)
//
// F(c) = int rho ln(rho / rho0) + sum c is the extended KL objective whose
// Newton step the reference's newton solver takes (H delta = -1 - df,
// glisa.py:763-769); minimising it over c >= 0 gives the cvxopt optimum
// (sum c = int rho holds there automatically). Per iteration: variables at 0
// whose gradient dF_k = 1 + df_k is non-negative stay fixed (Bertsekas'
// projected Newton), the Newton system is solved on the free set, and the
// step lengths 2^-t (t < kTrials) are tried on the projection
// max(c + 2^-t delta, 0) with the Armijo rule in one pass over the grid.
// ---------------------------------------------------------------------------

// The free-set step is k_glisa_newton_step(projected = 1); the trial points
// come from k_glisa_trial_set after the optional refinement.

// Trial objective differences: tpart[t][tile] = this tile's part of
// f(c_t) - f(c), f(c) = sum over healthy points of w rho ln(rho / rho0(c)).
//   rho0_t = sum_m max(c_m + a_t delta_m, 0) g_m
//          = rho0 + a_t (G^T delta) + sum_{m clipped at t} -(c_m + a_t delta_m) g_m,
// one pass over G plus the few clipped shells. Where a point is healthy for
// both, its term is -w rho log1p((rho0_t - rho0) / rho0): the relative change
// is formed in FP64 and goes through the FP32 log1pf, which keeps each term
// (and the difference the Armijo test compares) accurate to ~1e-7 of itself
// without an FP64 log per trial; the few points whose sick status differs
// between rho0 and rho0_t take FP64 logs. Sums in float-float per thread.
__global__ void __launch_bounds__(kThreads) k_glisa_trials(Batch bt) {
  __shared__ double red[kWarps * 2 * kTrials];
  __shared__ double out[2 * kTrials];
  int tile;
  const JobDev& J = decode_local(bt, tile);
  if (glisa_idle(J)) return;
  float ah[kTrials], al[kTrials], an[kTrials];
#pragma unroll
  for (int t = 0; t < kTrials; ++t) ah[t] = al[t] = an[t] = 0.0f;
  const int nclip = J.clip[J.nshell];
  const double cut = J.density_cutoff;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_of(J, tile, i);
    if (p >= J.npoint) continue;
    double u = 0.0;
#pragma unroll 8
    for (int m = 0; m < J.nshell; ++m) u += J.gmat[(size_t)m * J.npoint + p] * J.delta[m];
    // corr_t = -sum_{m clipped at t} (c_m + 2^-t delta_m) g_m: the clipped
    // sets shrink as t grows, so walk the list (sorted by t_m, largest first)
    // once, keeping the running sums of c g and delta g
    double corr[kTrials];
    {
      double sc = 0.0, sd = 0.0;
      int k = 0;
#pragma unroll
      for (int t = kTrials - 1; t >= 0; --t) {
        for (; k < nclip && J.clip[J.nshell + 1 + k] > t; ++k) {
          const int m = J.clip[k];
          const double g = J.gmat[(size_t)m * J.npoint + p];
          sc += J.propars[m] * g;
          sd += J.delta[m] * g;
        }
        corr[t] = -(sc + ldexp(1.0, -t) * sd);
      }
    }
    const double rho = J.rho[p], w = J.w[p], r0 = J.rho0[p];
    const bool h0 = !(rho < cut || r0 < cut);
    const double inv = h0 ? 1.0 / r0 : 0.0;
    const float wr = (float)(w * rho);
#pragma unroll
    for (int t = 0; t < kTrials; ++t) {
      const double dr = ldexp(1.0, -t) * u + corr[t];
      const double rt = r0 + dr;
      const bool ht = !(rho < cut || rt < cut);
      double big = 0.0;
      float term = 0.0f;
      if (h0 && ht) {
        term = -wr * log1pf((float)(dr * inv));
        an[t] += fabsf(term);
      } else if (ht) big = w * rho * log(rho / rt);
      else if (h0) big = -(w * rho * log(rho / r0));
      if (big != 0.0) {
        const float bh = (float)big;
        term = bh;
        al[t] += (float)(big - (double)bh);
      }
      const float s = ah[t] + term;  // TwoSum into (ah, al)
      const float bb = s - ah[t];
      al[t] += (ah[t] - (s - bb)) + (term - bb);
      ah[t] = s;
    }
  }
  double acc[2 * kTrials];
#pragma unroll
  for (int t = 0; t < kTrials; ++t) {
    acc[t] = (double)ah[t] + (double)al[t];
    acc[kTrials + t] = (double)an[t];
  }
  block_sum<2 * kTrials>(acc, red, out);
  if (threadIdx.x < 2 * kTrials) J.tpart[(size_t)threadIdx.x * J.ntile + tile] = out[threadIdx.x];
}

// One warp per job: Armijo choice among the trials, apply the step.
// One warp per trial (kTrials warps): warp t forms F(c_t) - F(c) and the
// Armijo bound of trial t; the first trial (in step order) that passes is
// taken, the shortest step if none does. The trial passes form most terms
// of f(c_t) - f(c) with the FP32 log1pf (a few ulp of each term: the ratio,
// log1pf and the product), and return the sum of those terms' magnitudes
// beside the difference (tpart rows kTrials + t). A trial passes when its
// difference is within kArmijoUlps ulp of that sum of the Armijo bound:
// near the optimum the predicted decrease falls below the resolution of the
// FP32 terms, the test can no longer tell the steps apart, and the full
// Newton step is the one to take (a shortened step there moves the
// parameters by a fraction of the remaining error and ends the loop on a
// change that is small only because the step was).
constexpr double kArmijoUlps = 8.0;
// The trial pass forms each trial's rho0 as rho0 + 2^-t G^T delta plus the
// clipped shells' corrections (float-float); the fused pass that follows
// takes the accepted trial's values as its rho0 while the last change is at
// least kR0HandoffChange times the threshold. Each hand-off adds the
// rounding of one float-float update (a few 1e-15 of rho0 + |G^T delta|),
// which only steers the early iterations; from four orders of magnitude
// above the threshold on, every pass forms rho0 = G^T c itself, so the
// converged parameters are those of the direct evaluation.
constexpr double kR0HandoffChange = 1e4;

__global__ void __launch_bounds__(32 * kTrials) k_glisa_trial_pick(Batch bt) {
  __shared__ int pass[kTrials];
  __shared__ int pick_s;
  int local;
  const JobDev& J = decode_local(bt, local);
  if (glisa_idle(J)) return;
  const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
  const int M = J.nshell;
  // sum (c_t - c) over the step the trial pass evaluated, 2^-t delta_m on
  // the shells the projection keeps and -c_m on those it clips: near the
  // optimum the whole change of F is ~1e-16, below the rounding of either
  // the difference of the two sums (each ~ the electron count) or of c_t
  // itself (c_t - c differs from 2^-t delta by the rounding of c + 2^-t
  // delta, ~1e-16 c per shell, which rho0_t does not contain)
  const double a = ldexp(1.0, -t);
  double ds = 0.0, dec = 0.0;
  for (int m = lane; m < M; m += 32) {
    const double c = J.propars[m], x = c + a * J.delta[m];
    const double d = x < 0.0 ? -c : a * J.delta[m];
    ds += d;
    dec += (1.0 + J.grad[m]) * d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ds += __shfl_xor_sync(0xffffffffu, ds, o);
    dec += __shfl_xor_sync(0xffffffffu, dec, o);
  }
  double df = 0.0, dn = 0.0;  // f(c_t) - f(c), and the magnitude of its FP32 terms
  for (int q = lane; q < J.ntile; q += 32) {
    df += J.tpart[(size_t)t * J.ntile + q];
    dn += J.tpart[(size_t)(kTrials + t) * J.ntile + q];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    df += __shfl_xor_sync(0xffffffffu, df, o);
    dn += __shfl_xor_sync(0xffffffffu, dn, o);
  }
  // Armijo on F = f + sum c: F(c_t) <= F(c) + 1e-4 dF.(c_t - c), up to the
  // rounding of the FP32 terms
  if (lane == 0) pass[t] = df + ds <= 1e-4 * dec + kArmijoUlps * 0x1p-24 * dn;
  __syncthreads();
  if (threadIdx.x == 0) {
    int pick = kTrials - 1;
    for (int k = 0; k < kTrials; ++k)
      if (pass[k]) {
        pick = k;
        break;
      }
    pick_s = pick;
    J.mail->d[MD_LS_X] = ldexp(1.0, -pick);
    // fused jobs away from convergence: the next pass takes rho0 of the
    // accepted trial from the trial pass (r0t) instead of forming G^T c
    J.mail->i[MI_R0T] = J.r0t && J.mail->d[MD_CHANGE] >= kR0HandoffChange * J.threshold ? pick + 1 : 0;
  }
  __syncthreads();
  const int pick = pick_s;
  // the step's start (k_copy_old's work, which projected-Newton steps leave
  // to this kernel): the parameters, and for fused jobs the entropy and
  // negativity partials of the pass at them
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    J.propars_old[m] = J.propars[m];
    J.propars[m] = J.ctrial[pick * M + m];
  }
  if (J.fuse)
    for (int q = threadIdx.x; q < J.ntile; q += blockDim.x) {
      J.jpart[(size_t)QJ_ENT_PREV * J.ntile + q] = J.jpart[(size_t)QJ_ENTROPY * J.ntile + q];
      J.jpart[(size_t)QJ_NEG_PREV * J.ntile + q] = J.jpart[(size_t)QJ_NEG * J.ntile + q];
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

long long g_launch_count = 0;  // kernel launches issued by this library (host counter)

#define HP_LAUNCH(kernel, kind, threads, ...)                                          \
  do {                                                                                 \
    if (hb.blocks[kind] > 0) {                                                         \
      kernel<<<hb.blocks[kind], threads, 0, st>>>(hb.b[kind], ##__VA_ARGS__);          \
      ++g_launch_count;                                                                \
    }                                                                                  \
  } while (0)

void launch_nelec(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_nelec, K_POINT, kThreads);
  HP_LAUNCH(k_init_params, K_JOB, 32);
}

void launch_copy_old(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_copy_old, K_JOB, 128); }

// FP32 variants live in hp_mixed.cu, float-float (MBIS) in hp_ff.cu; `mixed`
// is the job group's evaluation phase (Phase).
void launch_promol(const HostBatch& hb, cudaStream_t st, int mixed, int model) {
  if (mixed == PH_FF && model == MODEL_MBIS) return launch_promol_ff(hb, st);
  if (mixed) return launch_promol_mx(hb, st, model);
  if (model == MODEL_MBIS) HP_LAUNCH((k_promol<double, MODEL_MBIS>), K_POINT1, kThreads);
  else if (model == MODEL_NLIS) HP_LAUNCH((k_promol<double, MODEL_NLIS>), K_POINT1, kThreads);
  else HP_LAUNCH((k_promol<double, MODEL_BASIS>), K_POINT1, kThreads);
  HP_LAUNCH(k_atweights, K_ATOM_TILE, kThreads);
}

void launch_gisa_qp(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_gisa_qp, K_ATOM, 32); }

void launch_atweights(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_atweights, K_ATOM_TILE, kThreads);
}

void launch_final_atweights(const HostBatch& hb, cudaStream_t st, int mixed, int model,
                            int use_old) {
  if (mixed == PH_FF && model == MODEL_MBIS) return launch_final_atweights_ff(hb, st, use_old);
  if (mixed) return launch_final_atweights_mx(hb, st, model, use_old);
  if (model == MODEL_MBIS) HP_LAUNCH((k_final_atweights<double, MODEL_MBIS>), K_ATOM_TILE, kThreads, use_old);
  else if (model == MODEL_NLIS)
    HP_LAUNCH((k_final_atweights<double, MODEL_NLIS>), K_ATOM_TILE, kThreads, use_old);
  else HP_LAUNCH((k_final_atweights<double, MODEL_BASIS>), K_ATOM_TILE, kThreads, use_old);
}

void launch_change(const HostBatch& hb, cudaStream_t st, int mixed, int model) {
  if (mixed) return launch_change_mx(hb, st, model);
  if (model == MODEL_MBIS) HP_LAUNCH((k_change<double, MODEL_MBIS>), K_ATOM_TILE, kThreads);
  else if (model == MODEL_NLIS) HP_LAUNCH((k_change<double, MODEL_NLIS>), K_ATOM_TILE, kThreads);
  else HP_LAUNCH((k_change<double, MODEL_BASIS>), K_ATOM_TILE, kThreads);
}

void launch_outer_finish(const HostBatch& hb, cudaStream_t st, int with_charges) {
  HP_LAUNCH(k_outer_finish, K_JOB, kFinishThreads, with_charges);
}

void launch_charges(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_charges, K_JOB, kChargesThreads); }

void launch_inner_init(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_inner_init, K_JOB, 128); }

void launch_count_active(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_count_active, K_JOB, 32);
}

void launch_mbis_inner(const HostBatch& hb, cudaStream_t st, int mixed) {
  if (mixed == PH_FF) launch_mbis_inner_ff(hb, st);
  else if (mixed) launch_mbis_inner_mx(hb, st);
  else HP_LAUNCH(k_mbis_inner<double>, K_ATOM_TILE, kThreads);
  HP_LAUNCH(k_mbis_update, K_ATOM, 32);
}

void launch_nlis_inner(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_nlis_inner, K_ATOM_TILE, kThreads);
  HP_LAUNCH(k_nlis_update, K_ATOM, 32);
}

void launch_gisa(const HostBatch& hb, cudaStream_t st, int mixed) {
  if (mixed) launch_basis_qvec_mx(hb, st);
  else HP_LAUNCH(k_basis_qvec<double>, K_ATOM_TILE, kThreads);
  HP_LAUNCH(k_gisa_qp, K_ATOM, 32);
}

void launch_lisa_sc_inner(const HostBatch& hb, cudaStream_t st, int mixed) {
  if (mixed) launch_lisa_sc_inner_mx(hb, st);
  else HP_LAUNCH(k_lisa_sc_inner<double>, K_ATOM_TILE, kThreads);
  HP_LAUNCH(k_lisa_sc_update, K_ATOM, 32);
}

// Newton keeps FP64 evaluation (its Hessian needs it); mixed jobs are
// rejected for this solver at job creation.
void launch_lisa_newton_inner(const HostBatch& hb, cudaStream_t st, int mixed, int modified) {
  (void)mixed;
  HP_LAUNCH(k_lisa_newton_inner<double>, K_ATOM_TILE, kThreads);
  HP_LAUNCH(k_lisa_newton_update, K_ATOM, 32);
  if (modified) {
    HP_LAUNCH(k_lisa_ls<double>, K_ATOM_TILE, kThreads);
    HP_LAUNCH(k_lisa_ls_pick, K_ATOM, 32);
  }
}

void launch_glisa_basis(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_glisa_basis<double>, K_POINT, kThreads);
}

void launch_glisa_pro(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_glisa_pro, K_POINT, kThreads); }
void launch_glisa_grad(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_glisa_grad, K_POINT, kThreads, 0);
}
void launch_glisa_hess(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_glisa_hess, K_HESS, kThreads); }
void launch_glisa_reduce(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_glisa_reduce, K_SQUARE, kReduceThreads);
}

void launch_glisa_solve(const HostBatch& hb, cudaStream_t st, int projected, int max_shells, int tc) {
  static int configured_device = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured_device != dev) {
    cudaFuncSetAttribute(k_glisa_newton_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kNewtonSmemL);
    cudaFuncSetAttribute(k_glisa_refine, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kNewtonSmemL);
    cudaFuncSetAttribute(k_glisa_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kNewtonSmemL);
    configured_device = dev;
  }
  if (hb.blocks[K_JOB] > 0) {
    k_glisa_newton_step<<<hb.blocks[K_JOB], kNewtonThreads, kNewtonSmemL, st>>>(hb.b[K_JOB], projected, 0);
    ++g_launch_count;
  }
  // free sets above the shared-memory factor (tensor-core Hessian): the
  // multi-block FP32 factor; the kernels return for the other jobs
  if (tc && max_shells > kNewtonF32Max && hb.blocks[K_JOB] > 0) {
    const int npanel = (max_shells + kCholBP - 1) / kCholBP;
    for (int p = 0; p < npanel; ++p) {
      HP_LAUNCH(k_glisa_chol_panel, K_JOB, kThreads, p);
      HP_LAUNCH(k_glisa_chol_update, K_SQUARE, kThreads, p);
    }
    k_glisa_chol_solve<<<hb.blocks[K_JOB], kNewtonThreads, 4 * (size_t)max_shells, st>>>(hb.b[K_JOB]);
    k_glisa_newton_step<<<hb.blocks[K_JOB], kNewtonThreads, kNewtonSmemL, st>>>(hb.b[K_JOB], projected, 1);
    g_launch_count += 2;
  }
}

void launch_glisa_refine(const HostBatch& hb, cudaStream_t st, int gff, int fuse_shells, int unfused) {
  if (gff) {
    if (fuse_shells > 0) launch_glisa_fused_ff(hb, st, 0, fuse_shells);
    if (unfused) launch_glisa_hv_ff(hb, st);
  } else {
    HP_LAUNCH(k_glisa_hv, K_POINT1, kThreads);
    HP_LAUNCH(k_glisa_grad, K_POINT, kThreads, 1);
  }
  HP_LAUNCH(k_glisa_gsum, K_SQUARE, kThreads);  // K_SQUARE: ceil(M^2 / 256) >= ceil(M / 8) blocks
  if (hb.blocks[K_JOB] > 0) {  // dynamic shared memory: the FP32 factor (set up by launch_glisa_solve)
    k_glisa_refine<<<hb.blocks[K_JOB], kThreads, kNewtonSmemL, st>>>(hb.b[K_JOB]);
    ++g_launch_count;
  }
}

void launch_glisa_apply(const HostBatch& hb, cudaStream_t st, int mode) {
  HP_LAUNCH(k_glisa_apply, K_JOB, 128, mode);
}

void launch_glisa_keep(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_glisa_keep, K_ATOM, 32); }

void launch_glisa_ls(const HostBatch& hb, cudaStream_t st, int first, int count) {
  HP_LAUNCH(k_glisa_ls, K_ATOM_TILE, kThreads, first, count);
  HP_LAUNCH(k_glisa_ls_pick, K_JOB, 32, first, count);
}

void launch_glisa_change(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH(k_glisa_change, K_ATOM_TILE, kThreads);
}

void launch_glisa_check(const HostBatch& hb, cudaStream_t st) { HP_LAUNCH(k_glisa_check, K_JOB, 32); }

void launch_glisa_eval(const HostBatch& hb, cudaStream_t st, int what) {
  if (what != 2) HP_LAUNCH(k_glisa_eval_tiles, K_POINT, kThreads, what);
  HP_LAUNCH(k_glisa_eval_sum, K_JOB, 32, what);
}

void launch_glisa_pnewton(const HostBatch& hb, cudaStream_t st, int gff, int fuse_shells) {
  HP_LAUNCH(k_glisa_trial_set, K_JOB, kThreads);
  if (fuse_shells > 0) launch_glisa_trials_fused(hb, st, fuse_shells);
  else if (gff) launch_glisa_trials_ff(hb, st);
  else HP_LAUNCH(k_glisa_trials, K_POINT, kThreads);
  HP_LAUNCH(k_glisa_trial_pick, K_JOB, 32 * kTrials);
}

}  // namespace hp
