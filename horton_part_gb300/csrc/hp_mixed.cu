// Mixed-precision kernels: FP32 evaluation, compensated (float-float) sums,
// FP64 parameter updates.
//
// GB300 issues an FP64 warp instruction at a small fraction of the FP32 rate
// (each one occupies the FP64 pipe for tens of cycles even with one active
// lane), so these kernels execute no FP64 instruction per point, per thread
// or per block:
//   * shells, distances and ratios in FP32 (expf; distances from hi/lo float
//     coordinates);
//   * per-thread, per-warp and per-block sums in float-float (TwoSum); the
//     per-tile partial is stored as a float pair in the FP64 slot and turned
//     into FP64 by the per-atom update kernels (partial_value);
//   * every per-shell coefficient (N S^3 / 8 pi, the change coefficients) is
//     formed in FP64 once per iteration by a tiny kernel or by the update
//     kernels and read here as FP32 (JobDev::fpar, JobDev::fco);
//   * every change integrand pro(new) - pro(old) is formed from FP64
//     parameter differences, so it keeps its relative accuracy:
//       MBIS   t_old - t_new = t_new [g + (1 + g) expm1((S_new - S_old) r)],
//              g = A_old / A_new - 1,  A = N S^3 / (8 pi)
//       basis  sum_k (c_old - c_new)_k g_k
// Same steps and reference citations as hp_kernels.cu.
#include <math.h>

#include "hp_internal.cuh"

namespace hp {

namespace {

struct ff {
  float hi, lo;
};

// TwoSum (Knuth): s + e == a + b exactly.
__device__ __forceinline__ ff ff_add(ff a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b - bb);
  return {s, a.lo + e};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
  const float hi = s + e;
  return {hi, e - (hi - s)};
}

// Block sum of Q float-float accumulators (fixed order); out[q] valid for all
// threads afterwards.
template <int Q>
__device__ __forceinline__ void block_sum_ff(ff (&acc)[Q], float2* red, float2* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    ff v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ff w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
      v = ff_add(v, w);
    }
    if (lane == 0) red[warp * Q + q] = make_float2(v.hi, v.lo);
  }
  __syncthreads();
  if (threadIdx.x < Q) {
    ff s{0.f, 0.f};
#pragma unroll
    for (int k = 0; k < kWarps; ++k) {
      const float2 r = red[k * Q + threadIdx.x];
      s = ff_add(s, ff{r.x, r.y});
    }
    out[threadIdx.x] = make_float2(s.hi, s.lo);
  }
  __syncthreads();
}

__device__ __forceinline__ const JobDev& decode_local_mx(const Batch& bt, int& local) {
  const int j = find_job(bt, blockIdx.x);
  local = blockIdx.x - bt.prefix[j];
  return bt.jobs[j];
}

__device__ __forceinline__ const JobDev& decode_at_mx(const Batch& bt, int& atom, int& tile) {
  const int j = find_job(bt, blockIdx.x);
  const JobDev& J = bt.jobs[j];
  const int local = blockIdx.x - bt.prefix[j];
  atom = local / J.ntile;
  tile = local - atom * J.ntile;
  return J;
}

__device__ __forceinline__ void put_partial(const JobDev& J, int a, int q, int tile, float2 v) {
  *reinterpret_cast<float2*>(J.apart + ((size_t)a * J.qa + q) * J.ntile + tile) = v;
}

__device__ __forceinline__ float* rhoa_f(const JobDev& J, int a) {
  return reinterpret_cast<float*>(J.rhoa) + (size_t)a * J.npoint;
}

// Unit-population basis shell from the FP32 shell table.
__device__ __forceinline__ float shell_value_f(const JobDev& J, int s, float r) {
  return basis_shell<float>(J.shf[3 * s], J.shf[3 * s + 1], J.shf[3 * s + 2], r);
}

// t_old - t_new of one MBIS shell from its fco coefficients.
__device__ __forceinline__ float mbis_shell_delta(float t_new, const float* c, float r) {
  const float g = c[4], dS = c[5];
  const float x = dS * r;
  if (fabsf(x) < 16.0f) return t_new * (g + (1.0f + g) * expm1f(x));
  return c[2] * expf(-c[3] * r) - t_new;
}

}  // namespace

// FP64 -> FP32 coefficient tables (one block per job, threads over shells).
// which = 0: fpar from propars (promolecule pass);
// which = 1: fco from (propars, propars_old) (outer change pass).
__global__ void k_prep_mx(Batch bt, int which) {
  int local;
  const JobDev& J = decode_local_mx(bt, local);
  for (int s = threadIdx.x; s < J.nshell; s += blockDim.x) {
    if (which == 1) {
      fill_fco(J, s, J.propars, J.propars_old);
    } else if (J.scheme == SCHEME_MBIS) {
      const double n = J.propars[2 * s], x = J.propars[2 * s + 1];
      J.fpar[2 * s] = (float)(n * x * x * x * kInv8Pi);
      J.fpar[2 * s + 1] = (float)x;
    } else {
      J.fpar[s] = (float)J.propars[s];
    }
  }
}

// ---------------------------------------------------------------------------
// promolecule and at_weights (core/stockholder.py:153-175, 352-384)
// ---------------------------------------------------------------------------

// One block per kThreads points.
template <int MODEL>
__global__ void __launch_bounds__(kThreads) k_promol_mx(Batch bt) {
  int blk;
  const JobDev& J = decode_local_mx(bt, blk);
  const int p = blk * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  ff promol{0.f, 0.f};
  for (int a = 0; a < J.natom; ++a) {
    const float r = Dist<float>::r(J, p, a);
    float pro = 0.f;
    const int s0 = J.shell_off[a], s1 = J.shell_off[a + 1];
    if (MODEL == MODEL_MBIS) {
      for (int s = s0; s < s1; ++s) pro += J.fpar[2 * s] * expf(-J.fpar[2 * s + 1] * r);
    } else {
      for (int s = s0; s < s1; ++s) pro += J.fpar[s] * shell_value_f(J, s, r);
    }
    rhoa_f(J, a)[p] = pro;
    promol = ff_add(promol, pro);
  }
  // the promolecule is kept as a float pair (hi, lo) in the FP64 buffer; the
  // host forms the double (plus 1e-100 per atom) when results are read
  reinterpret_cast<float2*>(J.promol)[p] = make_float2(promol.hi, promol.lo);
  J.promolf[p] = promol.hi + promol.lo;
}

__global__ void __launch_bounds__(kThreads) k_atweights_mx(Batch bt) {
  __shared__ float2 red[kWarps * 2];
  __shared__ float2 out[2];
  int a, tile;
  const JobDev& J = decode_at_mx(bt, a, tile);
  ff acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
  float* ra = rhoa_f(J, a);
  const float cut = (float)J.density_cutoff;
  float vmax = 0.0f;  // largest rho_a on the tile (per-atom cutoff)
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const float promol = J.promolf[p];
    const float rho = J.rhof[p];
    const float aw = promol > 0.f ? fminf(fmaxf(ra[p] / promol, 0.f), 1.f) : 0.f;
    const float v = aw * rho;
    ra[p] = v;
    vmax = fmaxf(vmax, v);
    acc[0] = ff_add(acc[0], J.wf[p] * v);
    if (a == 0 && !(promol < cut || rho < cut)) acc[1] = ff_add(acc[1], J.wf[p] * rho * logf(rho / promol));
  }
  block_sum_ff<2>(acc, red, out);
  if (J.amax) {
    __shared__ float redm[kWarps];
    const float m = block_max_f(vmax, redm);
    if (threadIdx.x == 0) J.amax[(size_t)a * J.ntile + tile] = m;
  }
  if (threadIdx.x == 0) {
    put_partial(J, a, QA_POP, tile, out[0]);
    if (a == 0) *reinterpret_cast<float2*>(J.jpart + (size_t)QJ_ENTROPY * J.ntile + tile) = out[1];
  }
}

// ---------------------------------------------------------------------------
// outer change (core/iterstock.py:32-45), coefficients in fco (k_prep_mx 1)
// ---------------------------------------------------------------------------

template <int MODEL>
__global__ void __launch_bounds__(kThreads) k_change_mx(Batch bt) {
  __shared__ float2 red[kWarps];
  __shared__ float2 out[1];
  int a, tile;
  const JobDev& J = decode_at_mx(bt, a, tile);
  const int s0 = J.shell_off[a], n = J.shell_off[a + 1] - s0;
  const float* co = J.fco + 8 * s0;
  if (J.tgeo) {  // per-atom cutoff: bound of the pair's change term
    const float r = (float)tile_rmin(J, a, tile);
    double b = 0.0;
    if (MODEL == MODEL_MBIS) {
      b = (double)mbis_bound_f(co, n, 0, r) + (double)mbis_bound_f(co, n, 2, r);
    } else {  // sum_k |c_old - c_new|_k g_k(r)
      for (int k = 0; k < n; ++k) b += (double)(fabsf(co[8 * k + 1]) * shell_value_f(J, s0 + k, r));
    }
    if (tile_weight(J, tile) * b * b < kSkipRel * J.threshold * J.threshold) {
      if (threadIdx.x == 0) {
        put_partial(J, a, QA_CHANGE, tile, make_float2(0.f, 0.f));
        count_skipped(J, tile, 2.0);
      }
      return;
    }
  }
  ff acc[1] = {{0.f, 0.f}};
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const float r = Dist<float>::r(J, p, a);
    float delta = 0.f;
    if (MODEL == MODEL_MBIS) {
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        if (k < n) {
          const float* c = co + 8 * k;
          delta += mbis_shell_delta(c[0] * expf(-c[1] * r), c, r);
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kMaxShells; ++k)
        if (k < n) delta += co[8 * k + 1] * shell_value_f(J, s0 + k, r);
    }
    acc[0] = ff_add(acc[0], J.wf[p] * delta * delta);
  }
  block_sum_ff<1>(acc, red, out);
  if (threadIdx.x == 0) put_partial(J, a, QA_CHANGE, tile, out[0]);
}

// ---------------------------------------------------------------------------
// MBIS inner fixed point (mbis.py:81-163); coefficients of (cur, prev) in fco,
// written by k_inner_init / k_mbis_update
// ---------------------------------------------------------------------------

constexpr int kMxMbisQ = 2 * 7 + 1;

// At most 64 registers: four blocks (32 warps) per SM to hide the latency of
// the rho_a and coordinate loads.
__global__ void __launch_bounds__(kThreads, 4) k_mbis_inner_mx(Batch bt) {
  __shared__ float2 red[kWarps * kMxMbisQ];
  __shared__ float2 out[kMxMbisQ];
  int a, tile;
  const JobDev& J = decode_at_mx(bt, a, tile);
  if (!J.active[a]) return;
  const bool first = J.inner_it[a] == 0;
  const int s0 = J.shell_off[a], n = J.shell_off[a + 1] - s0;
  const float* co = J.fco + 8 * s0;
  if (J.tgeo && J.amax[(size_t)a * J.ntile + tile] < (float)J.density_cutoff) {
    // per-atom cutoff (see kSkipRel): zero moments, negligible change term
    const float r = (float)tile_rmin(J, a, tile);
    const double b = (double)mbis_bound_f(co, n, 0, r) + (first ? 0.0 : (double)mbis_bound_f(co, n, 2, r));
    if (tile_weight(J, tile) * b * b < kSkipRel * J.inner_threshold * J.inner_threshold) {
      if (threadIdx.x < 2 * n) put_partial(J, a, QA_INNER + threadIdx.x, tile, make_float2(0.f, 0.f));
      if (threadIdx.x == 0) {
        put_partial(J, a, QA_INNER + kMxMbisQ - 1, tile, make_float2(0.f, 0.f));
        count_skipped(J, tile, 1.0);
      }
      return;
    }
  }
  ff acc[kMxMbisQ];
#pragma unroll
  for (int q = 0; q < kMxMbisQ; ++q) acc[q] = {0.f, 0.f};
  const float* ra = rhoa_f(J, a);
  const float cut = (float)J.density_cutoff;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const float r = Dist<float>::r(J, p, a);
    float t[7];
    float pro = 0.f, delta = 0.f;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      t[k] = 0.f;
      if (k < n) {
        const float* c = co + 8 * k;
        t[k] = c[0] * expf(-c[1] * r);
        pro += t[k];
        if (!first) delta += mbis_shell_delta(t[k], c, r);
      }
    }
    const float rho = ra[p];
    const float w = J.wf[p];
    const bool sick = (rho < cut) || (pro < cut);
    const float wr = sick ? 0.f : w * (rho / pro);
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      if (k < n) {
        const float m0 = wr * t[k];
        acc[2 * k] = ff_add(acc[2 * k], m0);
        acc[2 * k + 1] = ff_add(acc[2 * k + 1], m0 * r);
      }
    }
    acc[kMxMbisQ - 1] = ff_add(acc[kMxMbisQ - 1], w * delta * delta);
  }
  block_sum_ff<kMxMbisQ>(acc, red, out);
  if (threadIdx.x < 2 * n) put_partial(J, a, QA_INNER + threadIdx.x, tile, out[threadIdx.x]);
  if (threadIdx.x == 0) put_partial(J, a, QA_INNER + kMxMbisQ - 1, tile, out[kMxMbisQ - 1]);
}

// ---------------------------------------------------------------------------
// GISA moments and aLISA self-consistent inner step
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kThreads) k_basis_qvec_mx(Batch bt) {
  __shared__ float2 red[kWarps * kMaxShells];
  __shared__ float2 out[kMaxShells];
  int a, tile;
  const JobDev& J = decode_at_mx(bt, a, tile);
  const int s0 = J.shell_off[a], n = J.shell_off[a + 1] - s0;
  ff acc[kMaxShells];
#pragma unroll
  for (int q = 0; q < kMaxShells; ++q) acc[q] = {0.f, 0.f};
  const float* ra = rhoa_f(J, a);
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const float r = Dist<float>::r(J, p, a);
    const float wr = J.wf[p] * ra[p];
#pragma unroll
    for (int k = 0; k < kMaxShells; ++k)
      if (k < n) acc[k] = ff_add(acc[k], wr * shell_value_f(J, s0 + k, r));
  }
  block_sum_ff<kMaxShells>(acc, red, out);
  if (threadIdx.x < n) put_partial(J, a, QA_INNER + threadIdx.x, tile, out[threadIdx.x]);
}

__global__ void __launch_bounds__(kThreads) k_lisa_sc_inner_mx(Batch bt) {
  constexpr int Q = kMaxShells + 1;
  __shared__ float2 red[kWarps * Q];
  __shared__ float2 out[Q];
  int a, tile;
  const JobDev& J = decode_at_mx(bt, a, tile);
  if (!J.active[a]) return;
  const int s0 = J.shell_off[a], n = J.shell_off[a + 1] - s0;
  const bool first = J.inner_it[a] == 0;
  const float* co = J.fco + 8 * s0;
  if (J.tgeo && J.amax[(size_t)a * J.ntile + tile] < (float)J.density_cutoff) {
    // per-atom cutoff (kSkipRel): zero moments, negligible change term
    double b = 0.0;
    if (!first) {
      const float r = (float)tile_rmin(J, a, tile);
      for (int k = 0; k < n; ++k) b += (double)(fabsf(co[8 * k + 1]) * shell_value_f(J, s0 + k, r));
    }
    if (tile_weight(J, tile) * b * b < kSkipRel * J.inner_threshold * J.inner_threshold) {
      if (threadIdx.x < n) put_partial(J, a, QA_INNER + threadIdx.x, tile, make_float2(0.f, 0.f));
      if (threadIdx.x == 0) {
        put_partial(J, a, QA_INNER + Q - 1, tile, make_float2(0.f, 0.f));
        count_skipped(J, tile, 1.0);
      }
      return;
    }
  }
  ff acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = {0.f, 0.f};
  const float* ra = rhoa_f(J, a);
  const float cut = (float)J.density_cutoff;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const float r = Dist<float>::r(J, p, a);
    float g[kMaxShells];
    float pro = 0.f, delta = 0.f;
#pragma unroll
    for (int k = 0; k < kMaxShells; ++k) {
      g[k] = 0.f;
      if (k < n) {
        g[k] = shell_value_f(J, s0 + k, r);
        pro += co[8 * k] * g[k];
        delta += co[8 * k + 1] * g[k];
      }
    }
    if (first) delta = 0.f;
    const float rho = ra[p];
    const float w = J.wf[p];
    const bool sick = (rho < cut) || (pro < cut);
    const float wr = sick ? 0.f : w * (rho / pro);
#pragma unroll
    for (int k = 0; k < kMaxShells; ++k)
      if (k < n) acc[k] = ff_add(acc[k], wr * (co[8 * k] * g[k]));
    acc[Q - 1] = ff_add(acc[Q - 1], w * delta * delta);
  }
  block_sum_ff<Q>(acc, red, out);
  if (threadIdx.x < n) put_partial(J, a, QA_INNER + threadIdx.x, tile, out[threadIdx.x]);
  if (threadIdx.x == 0) put_partial(J, a, QA_INNER + Q - 1, tile, out[Q - 1]);
}

// at_weights output (FP64 values written over the float rho_a buffer; runs
// once per job).
template <int MODEL>
__global__ void __launch_bounds__(kThreads) k_final_atweights_mx(Batch bt, int use_old) {
  int a, tile;
  const JobDev& J = decode_at_mx(bt, a, tile);
  const double* par = use_old ? J.propars_old : J.propars;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const float r = Dist<float>::r(J, p, a);
    const int s0 = J.shell_off[a], n = J.shell_off[a + 1] - s0;
    const double* pa = par + J.par_off[a];
    float pro = 0.f;
    if (MODEL == MODEL_MBIS) {
      for (int k = 0; k < n; ++k) {
        const double nn = pa[2 * k], s = pa[2 * k + 1];
        pro += (float)(nn * s * s * s * kInv8Pi) * expf(-(float)s * r);
      }
    } else {
      for (int k = 0; k < n; ++k) pro += (float)pa[k] * shell_value_f(J, s0 + k, r);
    }
    const float2 pm = reinterpret_cast<const float2*>(J.promol)[p];
    const double promol = (double)pm.x + (double)pm.y + 1e-100 * (double)J.natom;
    J.rhoa[(size_t)a * J.npoint + p] = fmin(fmax((double)pro / promol, 0.0), 1.0);
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

#define HP_LAUNCH_MX(kernel, kind, threads, ...)                                       \
  do {                                                                                 \
    if (hb.blocks[kind] > 0) {                                                         \
      kernel<<<hb.blocks[kind], threads, 0, st>>>(hb.b[kind], ##__VA_ARGS__);          \
      ++g_launch_count;                                                                \
    }                                                                                  \
  } while (0)

void launch_promol_mx(const HostBatch& hb, cudaStream_t st, int model) {
  HP_LAUNCH_MX(k_prep_mx, K_JOB, 128, 0);
  if (model == MODEL_MBIS) HP_LAUNCH_MX(k_promol_mx<MODEL_MBIS>, K_POINT1, kThreads);
  else HP_LAUNCH_MX(k_promol_mx<MODEL_BASIS>, K_POINT1, kThreads);
  HP_LAUNCH_MX(k_atweights_mx, K_ATOM_TILE, kThreads);
}

void launch_change_mx(const HostBatch& hb, cudaStream_t st, int model) {
  HP_LAUNCH_MX(k_prep_mx, K_JOB, 128, 1);
  if (model == MODEL_MBIS) HP_LAUNCH_MX(k_change_mx<MODEL_MBIS>, K_ATOM_TILE, kThreads);
  else HP_LAUNCH_MX(k_change_mx<MODEL_BASIS>, K_ATOM_TILE, kThreads);
}

void launch_mbis_inner_mx(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_MX(k_mbis_inner_mx, K_ATOM_TILE, kThreads);
}

void launch_basis_qvec_mx(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_MX(k_basis_qvec_mx, K_ATOM_TILE, kThreads);
}

void launch_lisa_sc_inner_mx(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_MX(k_lisa_sc_inner_mx, K_ATOM_TILE, kThreads);
}

void launch_final_atweights_mx(const HostBatch& hb, cudaStream_t st, int model, int use_old) {
  if (model == MODEL_MBIS) HP_LAUNCH_MX(k_final_atweights_mx<MODEL_MBIS>, K_ATOM_TILE, kThreads, use_old);
  else HP_LAUNCH_MX(k_final_atweights_mx<MODEL_BASIS>, K_ATOM_TILE, kThreads, use_old);
}

}  // namespace hp
