// MBIS kernels in float-float arithmetic: FP64-class results (~1e-13
// relative per pro-atom value) from the FP32 pipes.
//
// Used for the precision "ff" (every outer iteration) and for the finish of
// a mixed-precision MBIS job (the outer iterations after the FP32 phase).
// What is FF: distances (from hi/lo float coordinates), shell exponentials
// (Tang's table-driven exp, hp_ff.cuh), pro-atoms, promolecule, at_weights,
// the ratio rho_a / pro and the per-shell moments with their sums. What stays
// FP32: the change integrands pro(old) - pro(new), formed from exact FP64
// parameter differences (t_new [g + (1 + g) expm1(dS r)]), whose FP32 value
// is accurate relative to the change itself. What is FP64: the per-point
// entropy term (one log per point, not per pair), the parameter updates and
// the convergence tests. Same steps and reference citations as the FP64
// kernels (mbis.py:81-163, core/stockholder.py:153-175, 352-384).
#include <math.h>

#include "hp_ff.cuh"
#include "hp_internal.cuh"

namespace hp {

namespace ffa {

// 2^(i/64), i = 0..63, as (hi, lo) float pairs; copied into shared memory by
// each block (the index differs between lanes).
__constant__ float2 c_exp2_table[64];

// Block-local copy of the table (call with all threads, before any exp_ff).
__device__ __forceinline__ void load_exp_table(float2* tab) {
  if (threadIdx.x < 64) tab[threadIdx.x] = c_exp2_table[threadIdx.x];
  __syncthreads();
}

}  // namespace ffa

namespace {

using ffa::f2;

__device__ __forceinline__ const JobDev& decode_local_ff(const Batch& bt, int& local) {
  const int j = find_job(bt, blockIdx.x);
  local = blockIdx.x - bt.prefix[j];
  return bt.jobs[j];
}

__device__ __forceinline__ const JobDev& decode_at_ff(const Batch& bt, int& atom, int& tile) {
  const int j = find_job(bt, blockIdx.x);
  const JobDev& J = bt.jobs[j];
  const int local = blockIdx.x - bt.prefix[j];
  atom = local / J.ntile;
  tile = local - atom * J.ntile;
  return J;
}

__device__ __forceinline__ float2* rhoa_ff(const JobDev& J, int a) {
  return reinterpret_cast<float2*>(J.rhoa) + (size_t)a * J.npoint;
}

__device__ __forceinline__ f2 load2(const float2* p) {
  const float2 v = *p;
  return {v.x, v.y};
}

// Squared distance from grid point p to atom a; coordinates as float hi/lo pairs.
__device__ __forceinline__ f2 dist2_ff(const JobDev& J, int p, int a) {
  const float* c = J.atf + 6 * a;  // xh, xl, yh, yl, zh, zl
  const f2 dx = ffa::add(ffa::two_sum(J.pxh[p], -c[0]), J.pxl[p] - c[1]);
  const f2 dy = ffa::add(ffa::two_sum(J.pyh[p], -c[2]), J.pyl[p] - c[3]);
  const f2 dz = ffa::add(ffa::two_sum(J.pzh[p], -c[4]), J.pzl[p] - c[5]);
  return ffa::add_pos(ffa::add_pos(ffa::sqr(dx), ffa::sqr(dy)), ffa::sqr(dz));
}

// Distance from grid point p to atom a (the stored pair when the job keeps
// one: the same value, computed once at job start by k_rdist_ff).
__device__ __forceinline__ f2 dist_ff(const JobDev& J, int p, int a) {
  if (J.rdist) return load2(&J.rdist[(size_t)a * J.npoint + p]);
  return ffa::sqrt_ff(dist2_ff(J, p, a));
}

// Slater shell A exp(-S r), A = N S^3 / (8 pi), from FF coefficients.
__device__ __forceinline__ f2 slater_ff(f2 A, f2 S, f2 r, const float2* tab) {
  return ffa::mul(A, ffa::exp_ff(ffa::neg(ffa::mul(S, r)), tab));
}

// t_old - t_new of one MBIS shell (FP32) from the fco coefficients.
__device__ __forceinline__ float shell_delta_f(float t_new, const float* c, float r) {
  const float g = c[4], dS = c[5];
  const float x = dS * r;
  if (fabsf(x) < 16.0f) return t_new * (g + (1.0f + g) * expm1f(x));
  return c[2] * expf(-c[3] * r) - t_new;
}

// Deterministic block sum of Q FF accumulators; out[q] valid for all threads.
template <int Q>
__device__ __forceinline__ void block_sum_f2(f2 (&acc)[Q], float2* red, float2* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    f2 v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const f2 w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
      v = ffa::add(v, w);
    }
    if (lane == 0) red[warp * Q + q] = make_float2(v.hi, v.lo);
  }
  __syncthreads();
  if (threadIdx.x < Q) {
    f2 s{0.f, 0.f};
#pragma unroll
    for (int k = 0; k < kWarps; ++k) s = ffa::add(s, load2(&red[k * Q + threadIdx.x]));
    out[threadIdx.x] = make_float2(s.hi, s.lo);
  }
  __syncthreads();
}

__device__ __forceinline__ void put_partial_ff(const JobDev& J, int a, int q, int tile, float2 v) {
  *reinterpret_cast<float2*>(J.apart + ((size_t)a * J.qa + q) * J.ntile + tile) = v;
}

__device__ __forceinline__ void split(double v, float* hi, float* lo) {
  *hi = (float)v;
  *lo = (float)(v - (double)*hi);
}

}  // namespace

// FF coefficients of the current parameters: fpar[4 s ..] = (A hi, A lo, S hi, S lo).
__global__ void k_prep_ff(Batch bt) {
  int local;
  const JobDev& J = decode_local_ff(bt, local);
  for (int s = threadIdx.x; s < J.nshell; s += blockDim.x) {
    const double n = J.propars[2 * s], x = J.propars[2 * s + 1];
    split(n * x * x * x * kInv8Pi, &J.fpar[4 * s], &J.fpar[4 * s + 1]);
    split(x, &J.fpar[4 * s + 2], &J.fpar[4 * s + 3]);
  }
}

// Promolecule and pro-atoms (FF); one thread per point, all atoms.
__global__ void __launch_bounds__(kThreads) k_promol_ff(Batch bt) {
  __shared__ float2 tab[64];
  ffa::load_exp_table(tab);
  int blk;
  const JobDev& J = decode_local_ff(bt, blk);
  const int p = blk * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  f2 promol{0.f, 0.f};
  for (int a = 0; a < J.natom; ++a) {
    const f2 r = dist_ff(J, p, a);
    f2 pro{0.f, 0.f};
    for (int s = J.shell_off[a]; s < J.shell_off[a + 1]; ++s) {
      const float* c = J.fpar + 4 * s;
      pro = ffa::add_pos(pro, slater_ff(f2{c[0], c[1]}, f2{c[2], c[3]}, r, tab));
    }
    rhoa_ff(J, a)[p] = make_float2(pro.hi, pro.lo);
    promol = ffa::add_pos(promol, pro);
  }
  reinterpret_cast<float2*>(J.promol)[p] = make_float2(promol.hi, promol.lo);
  J.promolf[p] = promol.hi + promol.lo;
}

// at_weights w_a = clip(pro_a / promol, 0, 1), rho_a = w_a rho (FF), atom
// populations (FF partials) and the entropy (FP64 per point, atom 0's blocks).
__global__ void __launch_bounds__(kThreads) k_atweights_ff(Batch bt) {
  __shared__ float2 red[kWarps];
  __shared__ float2 out[1];
  __shared__ double redd[kWarps];
  int a, tile;
  const JobDev& J = decode_at_ff(bt, a, tile);
  f2 acc[1] = {{0.f, 0.f}};
  double ent = 0.0;
  float vmax = 0.0f;  // largest rho_a on the tile (per-atom cutoff)
  float2* ra = rhoa_ff(J, a);
  const float2* pm = reinterpret_cast<const float2*>(J.promol);
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const f2 promol = load2(&pm[p]);
    const f2 rho{J.rhof[p], J.rhol[p]};
    f2 aw{0.f, 0.f};
    if (promol.hi > 0.f) {
      aw = ffa::div(load2(&ra[p]), promol);
      if (aw.hi < 0.f) aw = {0.f, 0.f};
      if (aw.hi > 1.f || (aw.hi == 1.f && aw.lo > 0.f)) aw = {1.f, 0.f};
    }
    const f2 v = ffa::mul(aw, rho);
    ra[p] = make_float2(v.hi, v.lo);
    vmax = fmaxf(vmax, v.hi);
    acc[0] = ffa::add_pos(acc[0], ffa::mul(f2{J.wf[p], J.wl[p]}, v));
    if (a == 0) {
      const double r = J.rho[p], pr = ffa::to_double(promol);
      if (!(r < J.density_cutoff || pr < J.density_cutoff)) ent += J.w[p] * r * log(r / pr);
    }
  }
  block_sum_f2<1>(acc, red, out);
  if (J.amax) {
    __shared__ float redm[kWarps];
    const float m = block_max_f(vmax, redm);
    if (threadIdx.x == 0) J.amax[(size_t)a * J.ntile + tile] = m;
  }
  if (threadIdx.x == 0) put_partial_ff(J, a, QA_POP, tile, out[0]);
  if (a == 0) {
    const double s = block_sum1(ent, redd);
    if (threadIdx.x == 0) store_partial(J, J.jpart + (size_t)QJ_ENTROPY * J.ntile + tile, s);
  }
}

// MBIS inner fixed point (mbis.py:81-163): per-shell moments in FF; the inner
// change from the FP32 difference formula. fco per shell: (A_new hi, S_new hi,
// A_old, S_old, g, dS, A_new lo, S_new lo).
constexpr int kFfMbisQ = 2 * 7 + 1;

__global__ void __launch_bounds__(kThreads, 4) k_mbis_inner_ff(Batch bt) {
  __shared__ float2 tab[64];
  __shared__ float2 red[kWarps * kFfMbisQ];
  __shared__ float2 out[kFfMbisQ];
  ffa::load_exp_table(tab);
  int a, tile;
  const JobDev& J = decode_at_ff(bt, a, tile);
  if (!J.active[a]) return;
  const bool first = J.inner_it[a] == 0;
  const int s0 = J.shell_off[a], n = J.shell_off[a + 1] - s0;
  const float* co = J.fco + 8 * s0;
  if (J.tgeo && J.amax[(size_t)a * J.ntile + tile] < (float)J.density_cutoff) {
    // per-atom cutoff (see kSkipRel): zero moments, negligible change term
    const float r = (float)tile_rmin(J, a, tile);
    const double b = (double)mbis_bound_f(co, n, 0, r) + (first ? 0.0 : (double)mbis_bound_f(co, n, 2, r));
    if (tile_weight(J, tile) * b * b < kSkipRel * J.inner_threshold * J.inner_threshold) {
      if (threadIdx.x < 2 * n) put_partial_ff(J, a, QA_INNER + threadIdx.x, tile, make_float2(0.f, 0.f));
      if (threadIdx.x == 0) {
        put_partial_ff(J, a, QA_INNER + kFfMbisQ - 1, tile, make_float2(0.f, 0.f));
        count_skipped(J, tile, 1.0);
      }
      return;
    }
  }
  f2 acc[kFfMbisQ];
#pragma unroll
  for (int q = 0; q < kFfMbisQ; ++q) acc[q] = {0.f, 0.f};
  const float2* ra = rhoa_ff(J, a);
  const float cut = (float)J.density_cutoff;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const f2 r = dist_ff(J, p, a);
    f2 t[7];
    f2 pro{0.f, 0.f};
    float delta = 0.f;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      t[k] = {0.f, 0.f};
      if (k < n) {
        const float* c = co + 8 * k;
        t[k] = slater_ff(f2{c[0], c[6]}, f2{c[1], c[7]}, r, tab);
        pro = ffa::add_pos(pro, t[k]);
        if (!first) delta += shell_delta_f(t[k].hi, c, r.hi);
      }
    }
    const f2 rho = load2(&ra[p]);
    const f2 w{J.wf[p], J.wl[p]};
    const bool sick = (rho.hi < cut) || (pro.hi < cut);
    const f2 wr = sick ? f2{0.f, 0.f} : ffa::mul(w, ffa::div(rho, pro));
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      if (k < n) {
        const f2 m0 = ffa::mul(wr, t[k]);
        acc[2 * k] = ffa::add_pos(acc[2 * k], m0);
        acc[2 * k + 1] = ffa::add_pos(acc[2 * k + 1], ffa::mul(m0, r));
      }
    }
    acc[kFfMbisQ - 1] = ffa::add(acc[kFfMbisQ - 1], w.hi * delta * delta);
  }
  block_sum_f2<kFfMbisQ>(acc, red, out);
  if (threadIdx.x < 2 * n) put_partial_ff(J, a, QA_INNER + threadIdx.x, tile, out[threadIdx.x]);
  if (threadIdx.x == 0) put_partial_ff(J, a, QA_INNER + kFfMbisQ - 1, tile, out[kFfMbisQ - 1]);
}

// at_weights output (FP64 values written over the rho_a buffer; once per job).
__global__ void __launch_bounds__(kThreads) k_final_atweights_ff(Batch bt, int use_old) {
  __shared__ float2 tab[64];
  __shared__ float2 coef[2 * 7];
  ffa::load_exp_table(tab);
  int a, tile;
  const JobDev& J = decode_at_ff(bt, a, tile);
  const int n = J.shell_off[a + 1] - J.shell_off[a];
  const double* pa = (use_old ? J.propars_old : J.propars) + J.par_off[a];
  if (threadIdx.x < n) {
    const double nn = pa[2 * threadIdx.x], s = pa[2 * threadIdx.x + 1];
    float h, l;
    split(nn * s * s * s * kInv8Pi, &h, &l);
    coef[2 * threadIdx.x] = make_float2(h, l);
    split(s, &h, &l);
    coef[2 * threadIdx.x + 1] = make_float2(h, l);
  }
  __syncthreads();
  const float2* pm = reinterpret_cast<const float2*>(J.promol);
  for (int i = 0; i < J.ppt; ++i) {
    const int p = tile * J.tile_points + i * kThreads + threadIdx.x;
    if (p >= J.npoint) continue;
    const f2 r = dist_ff(J, p, a);
    f2 pro{0.f, 0.f};
    for (int k = 0; k < n; ++k) pro = ffa::add_pos(pro, slater_ff(load2(&coef[2 * k]), load2(&coef[2 * k + 1]), r, tab));
    const double promol = ffa::to_double(load2(&pm[p])) + 1e-100 * (double)J.natom;
    J.rhoa[(size_t)a * J.npoint + p] = fmin(fmax(ffa::to_double(pro) / promol, 0.0), 1.0);
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

namespace {

// 2^(i/64) as float pairs, from the host's double-precision exp2; once per device.
void ensure_exp_table() {
  static int done_mask = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 31 && (done_mask >> dev) & 1) return;
  float2 t[64];
  for (int i = 0; i < 64; ++i) {
    const double v = exp2((double)i / 64.0);
    const float hi = (float)v;
    t[i] = make_float2(hi, (float)(v - (double)hi));
  }
  cudaMemcpyToSymbol(ffa::c_exp2_table, t, sizeof(t));
  if (dev < 31) done_mask |= 1 << dev;
}

}  // namespace

// Point-atom distances of a mixed / ff job as float pairs (once per job):
// every later kernel reads them instead of re-forming the distance.
__global__ void __launch_bounds__(kThreads) k_rdist_ff(Batch bt) {
  int blk;
  const JobDev& J = decode_local_ff(bt, blk);
  if (!J.rdist) return;
  const int p = blk * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  for (int a = 0; a < J.natom; ++a) {
    const f2 d2 = dist2_ff(J, p, a);
    const f2 r = d2.hi > 0.0f ? ffa::sqrt_ff(d2) : f2{0.0f, 0.0f};
    J.rdist[(size_t)a * J.npoint + p] = make_float2(r.hi, r.lo);
  }
}

// Basis matrix of a gLISA job as float-float planes (gmat32 = hi, gmat_lo =
// lo): G[s][p] = pref_s exp(-alpha_s r^order_s), the unit-population shells
// of gisa.py:91-106 (force_on_molgrid=True) with the normalisation of
// core/basis.py:161. Orders 2 (from the squared distance) and 1 are evaluated
// in FF, any other order in FP64. fpar[4 s ..] = (pref hi, pref lo, alpha hi,
// alpha lo). One thread per grid point, all shells. The shells' orders are
// classified once per block into shared memory (an FP64 comparison per shell
// and point would run on the FP64 pipe, 1/64 of the FP32 rate).
__global__ void __launch_bounds__(kThreads) k_glisa_basis_ff(Batch bt) {
  __shared__ float2 tab[64];
  __shared__ int ord[kGffMaxShells];  // 2, 1 (FF paths) or 0 (FP64)
  ffa::load_exp_table(tab);
  int blk;
  const JobDev& J = decode_local_ff(bt, blk);
  for (int s = threadIdx.x; s < J.nshell; s += kThreads) {
    const double o = J.sh_order[s];
    ord[s] = o == 2.0 ? 2 : o == 1.0 ? 1 : 0;
  }
  __syncthreads();
  const int p = blk * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  if (J.wrf) {  // w rho and rho as float pairs for the fused passes
    const double rho = J.rho[p], wr = J.w[p] * rho;
    float4 q;
    split(wr, &q.x, &q.y);
    split(rho, &q.z, &q.w);
    J.wrf[p] = q;
  }
  if (J.wgram) J.hess_s[p] = sqrtf((float)J.w[p]);  // scale of the weighted Gram matrix
  for (int a = 0; a < J.natom; ++a) {
    const f2 d2 = dist2_ff(J, p, a);
    const f2 r = d2.hi > 0.0f ? ffa::sqrt_ff(d2) : f2{0.0f, 0.0f};
    for (int s = J.shell_off[a]; s < J.shell_off[a + 1]; ++s) {
      const int order = ord[s];
      f2 g;
      if (order != 0) {
        const float* c = J.fpar + 4 * s;
        const f2 x = ffa::mul(f2{c[2], c[3]}, order == 2 ? d2 : r);
        g = ffa::mul(f2{c[0], c[1]}, ffa::exp_ff(ffa::neg(x), tab));
      } else {
        const double v = basis_shell<double>(J.sh_order[s], J.sh_alpha[s], J.sh_pref[s],
                                             Dist<double>::r(J, p, a));
        split(v, &g.hi, &g.lo);
      }
      const size_t e = (size_t)s * J.npoint + p;
      J.gmat32[e] = g.hi;
      J.gmat_lo[e] = g.lo;
    }
  }
}

#define HP_LAUNCH_FF(kernel, kind, threads, ...)                                       \
  do {                                                                                 \
    if (hb.blocks[kind] > 0) {                                                         \
      kernel<<<hb.blocks[kind], threads, 0, st>>>(hb.b[kind], ##__VA_ARGS__);          \
      ++g_launch_count;                                                                \
    }                                                                                  \
  } while (0)

void launch_promol_ff(const HostBatch& hb, cudaStream_t st) {
  ensure_exp_table();
  HP_LAUNCH_FF(k_prep_ff, K_JOB, 128);
  HP_LAUNCH_FF(k_promol_ff, K_POINT1, kThreads);
  HP_LAUNCH_FF(k_atweights_ff, K_ATOM_TILE, kThreads);
}

void launch_mbis_inner_ff(const HostBatch& hb, cudaStream_t st) {
  ensure_exp_table();
  HP_LAUNCH_FF(k_mbis_inner_ff, K_ATOM_TILE, kThreads);
}

void launch_rdist_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_FF(k_rdist_ff, K_POINT1, kThreads);
}

void launch_glisa_basis_ff(const HostBatch& hb, cudaStream_t st) {
  ensure_exp_table();
  HP_LAUNCH_FF(k_glisa_basis_ff, K_POINT1, kThreads);
}

void launch_final_atweights_ff(const HostBatch& hb, cudaStream_t st, int use_old) {
  ensure_exp_table();
  HP_LAUNCH_FF(k_final_atweights_ff, K_ATOM_TILE, kThreads, use_old);
}

}  // namespace hp
