// gLISA passes over the basis matrix G in float-float arithmetic (the
// tensor-core Hessian form of the Newton solvers).
//
// G is stored as two float planes, G = G_hi + G_lo (about 48 significant
// bits; G_hi is the operand of the tensor-core Hessian), and every product
// sum over G - the promolecule rho0 = G^T c, the gradient rows G d1, the
// Hessian-vector products of the refinement, the trial promolecules and the
// change - is a compensated dot product (Dot2 of Ogita, Rump and Oishi, SIAM
// J. Sci. Comput. 26(6), 2005: TwoProd by FMA and TwoSum, the error terms
// summed in a second float) on the FP32 pipes instead of FP64 FMAs, which
// GB300 issues at 1/64 of the FP32 rate. Per-point scalars (ratios, logs,
// the sick masks) stay FP64. The result of a sum over n terms is accurate to
// ~n eps_f^2 of the sum of |terms| (eps_f = 2^-24), far below the solver's
// thresholds; the gLISA steps are otherwise those of hp_kernels.cu
// (glisa.py:346-348, 411-479, 748-798).
#include <math.h>

#include "hp_ff.cuh"
#include "hp_internal.cuh"

namespace hp {

namespace {

struct Dot2 {
  float s, c;  // running sum and the sum of its rounding errors
};

__device__ __forceinline__ void dot2_add(Dot2& a, float xh, float xl, float yh, float yl) {
  const float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  const float s = a.s + p;
  const float bb = s - a.s;
  a.c += ((a.s - (s - bb)) + (p - bb)) + e;
  a.s = s;
}

__device__ __forceinline__ void dot2_merge(Dot2& a, const Dot2& b) {
  const float s = a.s + b.s;
  const float bb = s - a.s;
  a.c += ((a.s - (s - bb)) + (b.s - bb)) + b.c;
  a.s = s;
}

__device__ __forceinline__ double dot2_value(const Dot2& a) { return (double)a.s + (double)a.c; }

__device__ __forceinline__ float2 split2(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

__device__ __forceinline__ const JobDev& decode_local_gf(const Batch& bt, int& local) {
  const int j = find_job(bt, blockIdx.x);
  local = blockIdx.x - bt.prefix[j];
  return bt.jobs[j];
}

__device__ __forceinline__ int point_in_tile(const JobDev& J, int tile, int i) {
  return tile * J.tile_points + i * kThreads + threadIdx.x;
}

// FP64 vector -> float pairs in shared memory (all threads; ends with a barrier).
__device__ __forceinline__ void load_pairs(const double* v, int n, float2* out) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = split2(v[i]);
  __syncthreads();
}

// sum_m G[m][p] x[m] for one point: four independent compensated sums
// (shells m = 0, 1, 2, 3 mod 4) merged in a fixed order, so the dependency
// chains overlap.
__device__ __forceinline__ double g_dot(const JobDev& J, int p, const float2* x) {
  Dot2 d0{0.f, 0.f}, d1{0.f, 0.f}, d2{0.f, 0.f}, d3{0.f, 0.f};
  const size_t N = J.npoint;
  const int M = J.nshell;
  int m = 0;
  for (; m + 3 < M; m += 4) {
    dot2_add(d0, J.gmat32[m * N + p], J.gmat_lo[m * N + p], x[m].x, x[m].y);
    dot2_add(d1, J.gmat32[(m + 1) * N + p], J.gmat_lo[(m + 1) * N + p], x[m + 1].x, x[m + 1].y);
    dot2_add(d2, J.gmat32[(m + 2) * N + p], J.gmat_lo[(m + 2) * N + p], x[m + 2].x, x[m + 2].y);
    dot2_add(d3, J.gmat32[(m + 3) * N + p], J.gmat_lo[(m + 3) * N + p], x[m + 3].x, x[m + 3].y);
  }
  for (; m < M; ++m) dot2_add(d0, J.gmat32[m * N + p], J.gmat_lo[m * N + p], x[m].x, x[m].y);
  dot2_merge(d0, d1);
  dot2_merge(d2, d3);
  dot2_merge(d0, d2);
  return dot2_value(d0);
}

}  // namespace

// rho0 = G^T c (glisa.py:346-348); d1 = w rho/rho0 (also as a float pair),
// d2 = w rho/rho0^2 (0 where sick); entropy and negativity partials.
__global__ void __launch_bounds__(kThreads) k_glisa_pro_ff(Batch bt) {
  __shared__ float2 cf[kGffMaxShells];
  __shared__ double red[kWarps * 2];
  __shared__ double out[2];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  load_pairs(J.propars, J.nshell, cf);
  double acc[2] = {0.0, 0.0};
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_in_tile(J, tile, i);
    if (p >= J.npoint) continue;
    const double rho0 = g_dot(J, p, cf);
    const double rho = J.rho[p];
    const double w = J.w[p];
    const bool sick = (rho < J.density_cutoff) || (rho0 < J.density_cutoff);
    const double inv = sick ? 0.0 : 1.0 / rho0;
    const double ratio = rho * inv;
    const double d2 = w * ratio * inv;
    J.dvec1[p] = w * ratio;
    J.d1f[p] = split2(w * ratio);
    J.dvec2[p] = d2;
    J.rho0[p] = rho0;
    J.hess_s[p] = sqrtf((float)d2);
    if (!sick) acc[0] += w * rho * log(ratio);
    if (rho0 < J.negative_cutoff) acc[1] += 1.0;
  }
  block_sum<2>(acc, red, out);
  if (threadIdx.x == 0) {
    J.jpart[(size_t)QJ_ENTROPY * J.ntile + tile] = out[0];
    J.jpart[(size_t)QJ_NEG * J.ntile + tile] = out[1];
  }
}

// gpart[m][tile] = sum_p G[m][p] v[p] with v = d1 (gradient) or the
// refinement's hvec; one warp per row m, lanes over the tile's points.
__global__ void __launch_bounds__(kThreads) k_glisa_grad_ff(Batch bt, int use_hvec) {
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p0 = tile * J.tile_points;
  const int p1 = min(p0 + J.tile_points, J.npoint);
  const float2* v = use_hvec ? J.hvf : J.d1f;
  const size_t N = J.npoint;
  for (int m = warp; m < J.nshell; m += kWarps) {
    const float* gh = J.gmat32 + m * N;
    const float* gl = J.gmat_lo + m * N;
    // four independent compensated sums over the lane's points
    Dot2 d{0.f, 0.f}, e{0.f, 0.f}, f{0.f, 0.f}, g{0.f, 0.f};
    int p = p0 + lane;
    for (; p + 96 < p1; p += 128) {
      const float2 x0 = v[p], x1 = v[p + 32], x2 = v[p + 64], x3 = v[p + 96];
      dot2_add(d, gh[p], gl[p], x0.x, x0.y);
      dot2_add(e, gh[p + 32], gl[p + 32], x1.x, x1.y);
      dot2_add(f, gh[p + 64], gl[p + 64], x2.x, x2.y);
      dot2_add(g, gh[p + 96], gl[p + 96], x3.x, x3.y);
    }
    for (; p < p1; p += 32) {
      const float2 x = v[p];
      dot2_add(d, gh[p], gl[p], x.x, x.y);
    }
    dot2_merge(d, e);
    dot2_merge(f, g);
    dot2_merge(d, f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const Dot2 b{__shfl_xor_sync(0xffffffffu, d.s, o), __shfl_xor_sync(0xffffffffu, d.c, o)};
      dot2_merge(d, b);
    }
    if (lane == 0) J.gpart[(size_t)m * J.ntile + tile] = dot2_value(d);
  }
}

// Refinement, first half: hvec[p] = (w rho / rho0^2)(p) * sum_m G[m][p] delta[m].
__global__ void __launch_bounds__(kThreads) k_glisa_hv_ff(Batch bt) {
  __shared__ float2 df[kGffMaxShells];
  int local;
  const JobDev& J = decode_local_gf(bt, local);
  load_pairs(J.delta, J.nshell, df);
  const int p = local * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  J.hvf[p] = split2(J.dvec2[p] * g_dot(J, p, df));
}

// Trial objective differences of the projected Newton step, as
// k_glisa_trials with G^T delta as a compensated dot product.
__global__ void __launch_bounds__(kThreads) k_glisa_trials_ff(Batch bt) {
  __shared__ float2 df[kGffMaxShells];
  __shared__ double red[kWarps * kTrials];
  __shared__ double out[kTrials];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  load_pairs(J.delta, J.nshell, df);
  float ah[kTrials], al[kTrials];
#pragma unroll
  for (int t = 0; t < kTrials; ++t) ah[t] = al[t] = 0.0f;
  const int nclip = J.clip[J.nshell];
  const double cut = J.density_cutoff;
  const size_t N = J.npoint;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_in_tile(J, tile, i);
    if (p >= J.npoint) continue;
    const double u = g_dot(J, p, df);
    double corr[kTrials];
    {
      double sc = 0.0, sd = 0.0;
      int k = 0;
#pragma unroll
      for (int t = kTrials - 1; t >= 0; --t) {
        for (; k < nclip && J.clip[J.nshell + 1 + k] > t; ++k) {
          const int m = J.clip[k];
          const double g = (double)J.gmat32[m * N + p] + (double)J.gmat_lo[m * N + p];
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
      if (h0 && ht) term = -wr * log1pf((float)(dr * inv));
      else if (ht) big = w * rho * log(rho / rt);
      else if (h0) big = -(w * rho * log(rho / r0));
      if (big != 0.0) {
        const float bh = (float)big;
        term = bh;
        al[t] += (float)(big - (double)bh);
      }
      const float s = ah[t] + term;
      const float bb = s - ah[t];
      al[t] += (ah[t] - (s - bb)) + (term - bb);
      ah[t] = s;
    }
  }
  double acc[kTrials];
#pragma unroll
  for (int t = 0; t < kTrials; ++t) acc[t] = (double)ah[t] + (double)al[t];
  block_sum<kTrials>(acc, red, out);
  if (threadIdx.x < kTrials) J.tpart[(size_t)threadIdx.x * J.ntile + tile] = out[threadIdx.x];
}

// Outer change per (atom, tile): sum_p w (sum_{m in atom} (c - c_old)_m g_m)^2
// (glisa.py:776 via compute_change), the differences formed in FP64.
__global__ void __launch_bounds__(kThreads) k_glisa_change_ff(Batch bt) {
  __shared__ float2 dc[kMaxShells];
  __shared__ double red[kWarps];
  const int jb = find_job(bt, blockIdx.x);
  const JobDev& J = bt.jobs[jb];
  const int local = blockIdx.x - bt.prefix[jb];
  const int atom = local / J.ntile, tile = local - atom * J.ntile;
  const int s0 = J.shell_off[atom], n = J.shell_off[atom + 1] - s0;
  if (threadIdx.x < n) dc[threadIdx.x] = split2(J.propars[s0 + threadIdx.x] - J.propars_old[s0 + threadIdx.x]);
  __syncthreads();
  const size_t N = J.npoint;
  double acc = 0.0;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_in_tile(J, tile, i);
    if (p >= J.npoint) continue;
    Dot2 d{0.f, 0.f};
    for (int k = 0; k < n; ++k)
      dot2_add(d, J.gmat32[(s0 + k) * N + p], J.gmat_lo[(s0 + k) * N + p], dc[k].x, dc[k].y);
    const double v = dot2_value(d);
    acc += J.w[p] * v * v;
  }
  const double s = block_sum1(acc, red);
  if (threadIdx.x == 0) J.apart[((size_t)atom * J.qa + QA_CHANGE) * J.ntile + tile] = s;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

#define HP_LAUNCH_GF(kernel, kind, threads, ...)                                       \
  do {                                                                                 \
    if (hb.blocks[kind] > 0) {                                                         \
      kernel<<<hb.blocks[kind], threads, 0, st>>>(hb.b[kind], ##__VA_ARGS__);          \
      ++g_launch_count;                                                                \
    }                                                                                  \
  } while (0)

void launch_glisa_pro_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_pro_ff, K_POINT, kThreads);
}

void launch_glisa_grad_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_grad_ff, K_POINT, kThreads, 0);
}

void launch_glisa_hv_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_hv_ff, K_POINT1, kThreads);
  HP_LAUNCH_GF(k_glisa_grad_ff, K_POINT, kThreads, 1);
}

void launch_glisa_trials_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_trials_ff, K_POINT, kThreads);
}

void launch_glisa_change_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_change_ff, K_ATOM_TILE, kThreads);
}

}  // namespace hp
