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
#include "hp_umma.cuh"

namespace hp {

namespace {

using ffa::f2;

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

// a < c for a normalised float pair a and the float pair c of a double
// (lexicographic: the double comparison except within ~1e-14 of c).
__device__ __forceinline__ bool below(ffa::f2 a, float2 c) {
  return a.hi < c.x || (a.hi == c.x && a.lo < c.y);
}

// The compensated sum as a normalised float pair.
__device__ __forceinline__ ffa::f2 dot2_ff(const Dot2& a) { return ffa::two_sum(a.s, a.c); }

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

// 2^(i/64) as float pairs for ffa::exp_ff (this translation unit's copy).
__constant__ float2 c_exp2_gl[64];

// FP64 vector -> float pairs in shared memory (all threads; ends with a barrier).
__device__ __forceinline__ void load_pairs(const double* v, int n, float2* out) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = split2(v[i]);
  __syncthreads();
}

// sum_m G[m][p] x[m] for one point: four independent compensated sums
// (shells m = 0, 1, 2, 3 mod 4) merged in a fixed order, so the dependency
// chains overlap.
__device__ __forceinline__ Dot2 g_dot2(const JobDev& J, int p, const float2* x) {
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
  return d0;
}

__device__ __forceinline__ double g_dot(const JobDev& J, int p, const float2* x) {
  return dot2_value(g_dot2(J, p, x));
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
  if (glisa_idle(J)) return;
  if (J.fuse) return;  // k_glisa_fused_ff<1>
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
  if (glisa_idle(J)) return;
  if (J.fuse) return;  // k_glisa_fused_ff
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
  if (glisa_idle(J)) return;
  if (J.fuse) return;  // k_glisa_fused_ff<0>
  load_pairs(J.delta, J.nshell, df);
  const int p = local * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  J.hvf[p] = split2(J.dvec2[p] * g_dot(J, p, df));
}

// u = G^T delta per point as a normalised float pair (in hvf, free after the
// refinement), for the trial promolecules; a light kernel at full occupancy
// so that this pass over G streams at the memory rate.
__global__ void __launch_bounds__(kThreads) k_glisa_u_ff(Batch bt) {
  __shared__ float2 df[kGffMaxShells];
  int local;
  const JobDev& J = decode_local_gf(bt, local);
  if (glisa_idle(J)) return;
  load_pairs(J.delta, J.nshell, df);
  const int p = local * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  const f2 u = dot2_ff(g_dot2(J, p, df));
  J.hvf[p] = make_float2(u.hi, u.lo);
}

// Trial objective differences of the projected Newton step (the steps of
// k_glisa_trials) on the FP32 pipes: u = G^T delta (k_glisa_u_ff) and the clipped-shell
// corrections are compensated dot products (the clipped shells' c and delta
// as float pairs from k_glisa_trial_set), rho0_t - rho0 = 2^-t u + corr_t is
// a float-float sum, and the sick tests compare float-float values with the
// cutoff's float pair. The relative change (rho0_t - rho0) / rho0 goes to
// log1pf as before; only the points whose sick status differs take FP64 logs.
__global__ void __launch_bounds__(kThreads) k_glisa_trials_ff(Batch bt) {
  __shared__ double red[kWarps * 2 * kTrials];
  __shared__ double out[2 * kTrials];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  if (glisa_idle(J)) return;
  float ah[kTrials], al[kTrials], an[kTrials];
#pragma unroll
  for (int t = 0; t < kTrials; ++t) ah[t] = al[t] = an[t] = 0.0f;
  const int nclip = J.clip[J.nshell];
  const int* tm = J.clip + J.nshell + 1;
  const float4* cd = reinterpret_cast<const float4*>(J.clipf);
  const double cut = J.density_cutoff;
  const float2 cutp = split2(cut);
  const size_t N = J.npoint;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_in_tile(J, tile, i);
    if (p >= J.npoint) continue;
    const float2 up = J.hvf[p];
    const f2 u{up.x, up.y};
    // corr_t = -sum_{m clipped at t} (c_m + 2^-t delta_m) g_m, running sums
    // over the list sorted by t_m (largest first)
    f2 corr[kTrials];
    {
      Dot2 sc{0.f, 0.f}, sd{0.f, 0.f};
      int k = 0;
#pragma unroll
      for (int t = kTrials - 1; t >= 0; --t) {
        for (; k < nclip && tm[k] > t; ++k) {
          const int m = J.clip[k];
          const float gh = J.gmat32[m * N + p], gl = J.gmat_lo[m * N + p];
          const float4 v = cd[k];
          dot2_add(sc, gh, gl, v.x, v.y);
          dot2_add(sd, gh, gl, v.z, v.w);
        }
        const f2 d = dot2_ff(sd);
        const float a = ldexpf(1.0f, -t);
        corr[t] = ffa::neg(ffa::add(dot2_ff(sc), f2{a * d.hi, a * d.lo}));
      }
    }
    const double rho = J.rho[p], w = J.w[p], r0 = J.rho0[p];
    const bool rs = rho < cut;
    const bool h0 = !(rs || r0 < cut);
    const float2 r0p = split2(r0);
    const float inv = h0 ? 1.0f / r0p.x : 0.0f;
    const float wr = (float)(w * rho);
#pragma unroll
    for (int t = 0; t < kTrials; ++t) {
      const float a = ldexpf(1.0f, -t);
      const f2 dr = ffa::add(f2{a * u.hi, a * u.lo}, corr[t]);
      const f2 rt = ffa::add(dr, f2{r0p.x, r0p.y});
      const bool below = rt.hi < cutp.x || (rt.hi == cutp.x && rt.lo < cutp.y);
      const bool ht = !(rs || below);
      double big = 0.0;
      float term = 0.0f;
      if (h0 && ht) {
        term = -wr * log1pf(dr.hi * inv);
        an[t] += fabsf(term);
      } else if (ht) big = w * rho * log(rho / ffa::to_double(rt));
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
  double acc[2 * kTrials];
#pragma unroll
  for (int t = 0; t < kTrials; ++t) {
    acc[t] = (double)ah[t] + (double)al[t];
    acc[kTrials + t] = (double)an[t];
  }
  block_sum<2 * kTrials>(acc, red, out);
  if (threadIdx.x < 2 * kTrials) J.tpart[(size_t)threadIdx.x * J.ntile + tile] = out[threadIdx.x];
}

// ---------------------------------------------------------------------------
// Fused passes: one read of G for a product G^T x and the row sums G v that
// depend on it. A block (256 threads, two per SM) streams its point tiles
// through shared memory in sub-tiles of kFuseSP = 32 points (both planes of
// the tile's active rows from the packed layout, TMA bulk copies into a ring
// of staging slots, so that the next sub-tiles load while one is
// processed). Warp w owns the active rows
// i = w, w + 8, ... of the tile (lane = point); per sub-tile
//   A  the warp sums G[m][p] x[m] over its rows in two compensated chains,
//      merged into the warp's partial sum of u(p);
//   A' warp 0 merges the eight partials in warp order and forms v(p) (and
//      for MODE 1 s(p), writing rho0(p)) for the sub-tile's points, published
//      in shared memory;
//   B  every warp adds G[m][p] v(p) of its rows to compensated accumulators
//      kept in registers across the tile (reduced once at its end) and, MODE
//      1, writes its rows of X = G_hi diag(s) for the tensor-core Hessian.
// The staged values are read again in B rather than kept in registers from
// A: the block runs at two per SM with at most 128 registers a thread, and
// holding them across the barriers costs more issue slots than the second
// shared-memory read (measured: 195 against 135 million warp instructions
// per pass on the benchmark molecule).
// No FP64 arithmetic per point: w rho and rho come as float pairs (wrf, set
// once per job), the outputs are float pairs.
// MODE 0 (refinement product): x = delta, v = (w rho / rho0^2) u.
// MODE 1 (promolecule + gradient): x = c, u = rho0 (r0f) and v = w rho /
//   rho0, quotients in float-float (the entropy, w rho / rho0^2 and the
//   negativity count follow in k_glisa_point_ff). The outer change of the
//   step that produced c needs no pass over the grid: k_outer_finish forms
//   it from the per-atom Gram blocks of k_glisa_wgram.
// Jobs with more than kFuseMaxShells shells use k_glisa_pro_ff /
// k_glisa_hv_ff with k_glisa_grad_ff.
// ---------------------------------------------------------------------------

constexpr int kFuseThreads = 256;
constexpr int kFuseWarps = kFuseThreads / 32;
constexpr int kFuseSP = 32;                             // points per sub-tile (one per lane)
// B keeps the gradient sums of a warp's first kFuseRows rows (tile rows below
// kFuseWarps kFuseRows = 96) in registers across the tile; the rows past
// them (tiles with more active shells) are reduced across the lanes per
// sub-tile and summed per row in shared memory.
constexpr int kFuseRows = 12;
constexpr int kFuseRegRowsTotal = kFuseWarps * kFuseRows;
// Shared memory of one block at most (two blocks per SM share 228 KB).
constexpr size_t kFuseSmemMax = 112 * 1024;

// The packed sub-tiles of G (gpack: per sub-tile nact rows x 32 points, one
// contiguous block per plane) reach shared memory by TMA bulk copies into a
// ring of slots of 2 nact x 128 bytes: as many slots (at most kRingSlots,
// one mbarrier each) as the ring holds for the tile's nact, so that the
// copies of the next sub-tiles are in flight while one is processed.
constexpr int kRingSlots = 6;

// Shared memory of a fused pass for S shells without its staging ring (bytes).
__host__ __device__ constexpr size_t fuse_fixed_bytes(int S) {
  return 8 * (size_t)S                     // per active row: x as a float pair
         + 8 * (size_t)kFuseWarps * kFuseSP  // partial sums
         + 32 * (size_t)kFuseSP              // per point: (v, s)
         + 8 * (size_t)(kFuseMaxShells - kFuseRegRowsTotal)  // gradient sums of the rows past them
         + 8 * (2 * kFuseWarps + 2)          // block sums
         + 12 * (size_t)S                    // active shells, positions, X keys
         + 16 + 8 * kRingSlots;              // the ring's mbarriers (16-byte aligned)
}

// The tile's active-shell list into shared memory: act[0..nact) ascending and
// pos[m] = its index (-1 for a shell that is zero on the whole tile).
__device__ __forceinline__ int load_active(const JobDev& J, int tile, int* act, int* pos) {
  const int S = J.nshell;
  const int* g = J.gact + (size_t)tile * (S + 1);
  const int nact = g[S];
  for (int m = threadIdx.x; m < S; m += kFuseThreads) pos[m] = -1;
  __syncthreads();
  for (int i = threadIdx.x; i < nact; i += kFuseThreads) {
    act[i] = g[i];
    pos[g[i]] = i;
  }
  return nact;
}

// Zero partial row sums of the shells that are inactive on this tile.
__device__ __forceinline__ void zero_inactive(const JobDev& J, int tile, const int* pos) {
  for (int m = threadIdx.x; m < J.nshell; m += kFuseThreads)
    if (pos[m] < 0) J.gpart[(size_t)m * J.ntile + tile] = 0.0;
}

// Shared memory of the promolecule + gradient pass (MODE 1), which also
// stages the sub-tile's X = G_hi diag(s) for the tensor-core Hessian: the
// fused layout plus the X tile (fuse_x_rows(S) rows of 128 bytes, 1024-byte
// aligned), an mbarrier and the tensor-memory slot. At least kFuseSmemFloor
// bytes, so that at most two blocks share an SM (two 256-column tensor-memory
// allocations fill its 512 columns).
__host__ __device__ constexpr int fuse_x_rows(int S) {
  return (S + 15) / 16 * 16 > umma::kTcM ? (S + 15) / 16 * 16 : umma::kTcM;
}
constexpr size_t kFuseSmemFloor = 78 * 1024;
__host__ __device__ constexpr size_t fuse_fixed_bytes(int S, int mode) {
  return mode ? fuse_fixed_bytes(S) + 128 * (size_t)fuse_x_rows(S) + 1024 + 64 : fuse_fixed_bytes(S);
}
constexpr int kFuseTmemCols = 256;
constexpr int kMmaThread = kFuseThreads - 32;  // lane 0 of the last warp issues the MMAs

// The staging ring of a fused pass over jobs of at most S shells (floats):
// the rest of kFuseSmemMax (at least kFuseSmemFloor in all), in 128-byte
// units. It must hold one sub-tile of the job's largest tile.
__host__ __device__ constexpr int fuse_ring_floats(int S, int mode) {
  return (int)((kFuseSmemMax - fuse_fixed_bytes(S, mode)) / 128 * 32);
}
static_assert(fuse_ring_floats(kFuseMaxShells, 1) >= 2 * kFuseMaxShells * kFuseSP,
              "fused pass shared memory: one sub-tile of the largest tile");
static_assert(fuse_fixed_bytes(kFuseMaxShells, 1) + 4 * (size_t)fuse_ring_floats(kFuseMaxShells, 1) >=
                  kFuseSmemFloor, "at most two blocks per SM");

// Persistent blocks (launch kind K_FUSE): block b of a job takes the point
// tiles the job's schedule gives it (fsched: longest processing time first
// over the tiles' active-row work, ascending within a block; nb =
// min(ntile, kFuseCtas)). The per-tile outputs (gradient rows, change) stay
// per tile.
//
// MODE 1 also accumulates the Hessian H = X X^T of its tiles on the tensor
// cores (glisa.py:457-470): in B every warp writes its rows of X (X[m][p] =
// G_hi[m][p] s(p), s(p) = sqrt(w rho) / rho0, 0 where sick, rounded to TF32
// to nearest) into the 128B-swizzled K-major tile in shared memory (the
// tile's inactive rows stay zero); at the next block barrier thread 0 issues
// tcgen05.mma.kind::tf32 (M = 128, K = 8, four per sub-tile) for
//   D1 (tensor-memory columns 0..n1-1):  A = X rows 0..127,        B = rows 0..n1-1,
//   D2 (columns c2..c2+n1-129):          A = X rows n1-128..n1-1, B = rows 128..n1-1,
// n1 = S rounded up to 16, c2 = n1 rounded up to 32 (D2 only when S > 128),
// and commits to an mbarrier that the writers of the next sub-tile wait on.
// D1 holds H[i][j] for i < 128 (its columns j >= 128 are H[j][i]); the rows
// 256 - n1 .. 127 of D2 hold H[i][j] for i, j >= 128. At the end the block
// writes its packed FP32 lower triangle to hpart[block] (k_glisa_reduce sums
// the nsplit partials in FP64 in a fixed order). The accumulation order is
// fixed (one issuing thread, tiles and sub-tiles in order), so a job's H is
// the same alone and in a batch. Relative accuracy of H: a few 1e-4 (TF32
// operands, FP32 accumulation of non-negative terms); the Newton direction
// is refined against the exact product in the finish (polish), and the
// gradient and objective stay compensated.
//
// Per tile the active rows' values that every sub-tile needs are compacted
// once: x[act[i]] (xa) and the X-tile word of row act[i] for lane 0 (xkey;
// the 128B swizzle makes lane l's word xkey ^ l), so that the row loops read
// them at fixed offsets.
// MODE 1 writes rho0 (r0f); the entropy, the negativity count and w rho /
// rho0^2 (d2f) follow in k_glisa_point_ff.
template <int MODE>
__global__ void __launch_bounds__(kFuseThreads, 2) k_glisa_fused_ff(Batch bt, int ring_floats) {
  extern __shared__ float4 fsm[];
  int local;
  const JobDev& J = decode_local_gf(bt, local);
  if (glisa_idle(J)) return;
  if (!J.fuse) return;
  if (MODE == 0 && !glisa_refine_now(J)) return;
  const int jb = find_job(bt, blockIdx.x);
  const int nblk_job = bt.prefix[jb + 1] - bt.prefix[jb];
  const int S = J.nshell;
  const bool hess = MODE == 1;
  // MODE 1: the X tile first (1024-byte aligned), then the fused layout
  const uint32_t raw = umma::smem_u32(fsm);
  const uint32_t xoff = hess ? ((1024u - (raw & 1023u)) & 1023u) : 0u;
  const int xrows = fuse_x_rows(S);
  uint32_t* xt = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(fsm) + xoff);
  float* ring = hess ? reinterpret_cast<float*>(xt + 32 * xrows) : reinterpret_cast<float*>(fsm);
  float2* xa = reinterpret_cast<float2*>(ring + ring_floats);  // x of active row i
  Dot2* part = reinterpret_cast<Dot2*>(xa + S);
  float4* pvs = reinterpret_cast<float4*>(part + kFuseWarps * kFuseSP);  // (v hi, v lo, s, -)
  Dot2* ovf = reinterpret_cast<Dot2*>(pvs + 2 * kFuseSP);  // rows i >= kFuseRegRowsTotal
  double* red = reinterpret_cast<double*>(ovf + (kFuseMaxShells - kFuseRegRowsTotal));
  int* act = reinterpret_cast<int*>(red + 2 * kFuseWarps + 2);
  int* pos = act + S;
  int* xkey = pos + S;
  uint64_t* rbar = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(xkey + S) + 15) & ~uintptr_t(15));
  uint64_t* mbar = rbar + kRingSlots;  // the MMAs' commits (MODE 1)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);
  __shared__ volatile int timed_out;
  const float2 cutp = split2(J.density_cutoff);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float4* __restrict__ wrfp = J.wrf;
  const float2* __restrict__ d2in = J.d2f;
  float2* r0fo = J.r0f;
  const int n1 = (S + 15) / 16 * 16;
  const int c2 = (n1 + 31) / 32 * 32;
  const bool has_d2 = n1 > umma::kTcM;
  const uint32_t bar = umma::smem_u32(mbar);
  const uint32_t rbar0 = umma::smem_u32(rbar);
  if (threadIdx.x == 0) {
    for (int b = 0; b < kRingSlots; ++b) umma::mbar_init(rbar0 + 8 * b, 1);
    timed_out = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  uint32_t ring_phase = 0;  // bit b: parity of the next completion of slot b
  uint32_t tmem = 0;
  int nmma = 0;  // sub-tiles whose MMAs have been issued (= commits on bar)
  if (hess) {
    if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       umma::smem_u32(tmem_slot)),
                   "r"(kFuseTmemCols));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
      umma::mbar_init(bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    tmem = *tmem_slot;
  }
  // The MMAs of the X tile as it stands (thread 0; after a block barrier
  // that follows the writers' proxy fences).
  // descriptors of the X tile's operands at K offset 0; K step kk adds 32
  // bytes to the start address (2 in the descriptor's 16-byte units)
  const uint32_t xs = umma::smem_u32(xt);
  const uint64_t da1 = umma::umma_desc(xs);
  const uint64_t da2 = umma::umma_desc(xs + (n1 - umma::kTcM) * 128);
  const uint64_t db2 = umma::umma_desc(xs + umma::kTcM * 128);
  const uint32_t id1 = umma::idesc_tf32(n1);
  const uint32_t id2 = umma::idesc_tf32(has_d2 ? n1 - umma::kTcM : 16);
  auto issue_mma = [&]() {
    asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
    for (int kk = 0; kk < kFuseSP / 8; ++kk) {
      const uint32_t acc = (nmma > 0 || kk > 0) ? 1u : 0u;
      umma::umma_tf32(tmem, da1 + 2 * kk, da1 + 2 * kk, id1, acc);
      if (has_d2) umma::umma_tf32(tmem + (uint32_t)c2, da2 + 2 * kk, db2 + 2 * kk, id2, acc);
    }
    umma::umma_commit(bar);
  };
  // Every thread: the MMAs of the last issued sub-tile have read the X tile.
  auto wait_mma = [&]() {
    if (nmma > 0 && !timed_out && !umma::mbar_wait_sleep(bar, (uint32_t)((nmma - 1) & 1))) timed_out = 1;
  };
  const double* x = MODE ? J.propars : J.delta;
  // MODE 1 after an accepted projected-Newton trial (away from convergence):
  // rho0 of this pass is the trial pass's density of that trial (r0t), and
  // the pass skips A and A' (one block barrier per sub-tile instead of three)
  const int r0sel = MODE == 1 ? J.mail->i[MI_R0T] : 0;
  const float2* __restrict__ r0in = r0sel > 0 ? J.r0t + (size_t)(r0sel - 1) * J.npoint : nullptr;

  const int* __restrict__ tiles = J.fsched + nblk_job + 1;
  for (int k = J.fsched[local]; k < J.fsched[local + 1]; ++k) {
    const int tile = tiles[k];
    const int p0 = tile * J.tile_points;
    const int p1 = min(p0 + J.tile_points, J.npoint);
    const int nsub = (p1 - p0 + kFuseSP - 1) / kFuseSP;
    if (hess) {
      wait_mma();  // the previous tile's last MMAs have read the X tile
      for (int e = threadIdx.x; e < 32 * xrows; e += kFuseThreads) xt[e] = 0u;  // inactive rows
    }
    __syncthreads();  // shared state of the previous tile no longer in use
    const int nact = load_active(J, tile, act, pos);
    __syncthreads();
    // staging ring for this tile: nslot slots of slotf floats (high plane,
    // then low plane, nact rows of 32 points each); thread 0 keeps the
    // copies of nslot - 1 sub-tiles ahead in flight
    const int slotf = 2 * nact * kFuseSP;
    const int nslot = nact > 0 ? min(kRingSlots, max(1, ring_floats / slotf)) : 1;
    const float* src = J.gpack + J.gtile_off[tile];
    auto issue = [&](int k) {
      const int b = k % nslot;
      const uint32_t bytes = (uint32_t)nact * kFuseSP * 4;
      umma::mbar_expect_tx(rbar0 + 8 * b, 2 * bytes);
      if (bytes) {
        const uint32_t dst = umma::smem_u32(ring + (size_t)b * slotf);
        umma::bulk_g2s(dst, src + (size_t)k * nact * kFuseSP, bytes, rbar0 + 8 * b);
        umma::bulk_g2s(dst + bytes, src + J.gpack_plane + (size_t)k * nact * kFuseSP, bytes, rbar0 + 8 * b);
      }
    };
    if (threadIdx.x == 0)
      for (int k2 = 0; k2 < nslot - 1 && k2 < nsub; ++k2) issue(k2);
    for (int i = threadIdx.x; i < nact; i += kFuseThreads) {
      const int m = act[i];
      xa[i] = split2(x[m]);
      xkey[i] = m * 32 + ((m & 7) << 2);
      if (i >= kFuseRegRowsTotal) ovf[i - kFuseRegRowsTotal] = Dot2{0.f, 0.f};
    }
    // this warp's rows i = warp + 8 r, r < nr
    const int nr = nact > warp ? (nact - warp + kFuseWarps - 1) / kFuseWarps : 0;
    Dot2 acc[kFuseRows];
#pragma unroll
    for (int r = 0; r < kFuseRows; ++r) acc[r] = Dot2{0.f, 0.f};
    // rho0 given: the per-point pairs of the next sub-tile are loaded one
    // sub-tile ahead, so that their latency overlaps the current one
    float4 qn = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 rn = make_float2(0.f, 0.f);
    if (r0in && p0 + lane < p1) {
      qn = wrfp[p0 + lane];
      rn = r0in[p0 + lane];
    }
    for (int sub = 0; sub < nsub; ++sub) {
      const int slot = sub % nslot;
      const float* gh = ring + (size_t)slot * slotf;
      const float* gl = gh + nact * kFuseSP;
      const int q0 = p0 + sub * kFuseSP;
      __syncthreads();  // every thread is done with sub - 1 (its slot is free)
      if (threadIdx.x == 0 && sub + nslot - 1 < nsub) issue(sub + nslot - 1);
      // X of sub - 1 is complete: its MMAs (issued by the last warp; warp 0
      // has the per-point step of this sub-tile ahead)
      if (hess && sub > 0 && threadIdx.x == kMmaThread && !timed_out) issue_mma();
      if (hess && sub > 0) ++nmma;
      const int pq = q0 + lane;
      const float* ghw = gh + warp * kFuseSP + lane;
      const float* glw = gl + warp * kFuseSP + lane;
      f2 v{0.f, 0.f};
      float sx = 0.0f;
      if (r0in) {
        // rho0 given: every warp forms v and s of its lane's point (warp 0
        // also stores rho0) from the pairs loaded one sub-tile earlier
        const float4 q = qn;
        const float2 r0s = rn;
        if (pq + kFuseSP < p1) {
          qn = wrfp[pq + kFuseSP];
          rn = r0in[pq + kFuseSP];
        }
        if (!timed_out && !umma::mbar_wait_sleep(rbar0 + 8 * slot, (ring_phase >> slot) & 1u))
          timed_out = 1;
        ring_phase ^= 1u << slot;  // sub-tile sub is in the slot
        if (pq < p1) {
          const f2 r0{r0s.x, r0s.y};
          if (warp == 0) r0fo[pq] = r0s;
          if (!(below(f2{q.z, q.w}, cutp) || below(r0, cutp))) {
            v = ffa::div(f2{q.x, q.y}, r0);
            sx = sqrtf(q.x) / r0.hi;
          }
        }
      } else {
        // per-point inputs of warp 0, loaded before phase A so that their
        // latency overlaps it: (w rho, rho) pairs (MODE 1) or the d2 pair (MODE 0)
        float4 qpre = make_float4(0.f, 0.f, 0.f, 0.f);
        if (pq < p1 && warp == 0) {
          if (MODE == 1) qpre = wrfp[pq];
          else {
            const float2 d2 = d2in[pq];
            qpre = make_float4(d2.x, d2.y, 0.f, 0.f);
          }
        }
        if (!timed_out && !umma::mbar_wait_sleep(rbar0 + 8 * slot, (ring_phase >> slot) & 1u))
          timed_out = 1;
        ring_phase ^= 1u << slot;  // sub-tile sub is in the slot
        {  // A: rows r even in chain d, odd in chain e
          Dot2 d{0.f, 0.f}, e{0.f, 0.f};
          int r = 0;
          for (; r + 1 < nr; r += 2) {
            const float2 x1 = xa[warp + kFuseWarps * r], x2 = xa[warp + kFuseWarps * (r + 1)];
            dot2_add(d, ghw[r * kFuseWarps * kFuseSP], glw[r * kFuseWarps * kFuseSP], x1.x, x1.y);
            dot2_add(e, ghw[(r + 1) * kFuseWarps * kFuseSP], glw[(r + 1) * kFuseWarps * kFuseSP], x2.x,
                     x2.y);
          }
          if (r < nr) {
            const float2 x1 = xa[warp + kFuseWarps * r];
            dot2_add(d, ghw[r * kFuseWarps * kFuseSP], glw[r * kFuseWarps * kFuseSP], x1.x, x1.y);
          }
          dot2_merge(d, e);
          part[warp * kFuseSP + lane] = d;
        }
        __syncthreads();  // partial sums visible
        if (warp == 0) {
          // A': the eight partial sums merged in warp order; v (and s, rho0)
          Dot2 du = part[lane];
#pragma unroll
          for (int q = 1; q < kFuseWarps; ++q) dot2_merge(du, part[q * kFuseSP + lane]);
          f2 vw{0.f, 0.f};
          float sw = 0.0f;
          if (pq < p1) {
            if (MODE == 0) {
              vw = ffa::mul(dot2_ff(du), f2{qpre.x, qpre.y});
            } else {
              const f2 r0 = dot2_ff(du);
              r0fo[pq] = make_float2(r0.hi, r0.lo);
              const bool sick = below(f2{qpre.z, qpre.w}, cutp) || below(r0, cutp);
              if (!sick) {
                vw = ffa::div(f2{qpre.x, qpre.y}, r0);
                sw = sqrtf(qpre.x) / r0.hi;
              }
            }
          }
          pvs[lane] = make_float4(vw.hi, vw.lo, sw, 0.f);
        }
        __syncthreads();  // v and s of the sub-tile visible
        const float4 pv = pvs[lane];
        v = f2{pv.x, pv.y};
        sx = pv.z;
      }
      if (hess) wait_mma();  // the MMAs of sub - 1 have read the X tile
      // B (and the rows of X)
#pragma unroll
      for (int r = 0; r < kFuseRows; ++r) {
        if (r < nr) {
          const float g1 = ghw[r * kFuseWarps * kFuseSP], g2 = glw[r * kFuseWarps * kFuseSP];
          if (hess) xt[xkey[warp + kFuseWarps * r] ^ lane] = umma::to_tf32_rn(g1 * sx);
          dot2_add(acc[r], g1, g2, v.hi, v.lo);
        }
      }
      for (int r = kFuseRows; r < nr; ++r) {  // rows past the register sums: lane sum per sub-tile
        const int i = warp + kFuseWarps * r;
        const float g1 = ghw[r * kFuseWarps * kFuseSP], g2 = glw[r * kFuseWarps * kFuseSP];
        if (hess) xt[xkey[i] ^ lane] = umma::to_tf32_rn(g1 * sx);
        Dot2 t{0.f, 0.f};
        dot2_add(t, g1, g2, v.hi, v.lo);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const Dot2 b{__shfl_xor_sync(0xffffffffu, t.s, o), __shfl_xor_sync(0xffffffffu, t.c, o)};
          dot2_merge(t, b);
        }
        if (lane == 0) dot2_merge(ovf[i - kFuseRegRowsTotal], t);
      }
      if (hess) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (hess) {  // the tile's last sub-tile
      __syncthreads();
      if (threadIdx.x == kMmaThread && !timed_out) issue_mma();
      ++nmma;
    }
#pragma unroll
    for (int r = 0; r < kFuseRows; ++r) {
      const int i = warp + kFuseWarps * r;
      if (i < nact) {  // warp-uniform
        Dot2 d = acc[r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const Dot2 b{__shfl_xor_sync(0xffffffffu, d.s, o), __shfl_xor_sync(0xffffffffu, d.c, o)};
          dot2_merge(d, b);
        }
        if (lane == 0) J.gpart[(size_t)act[i] * J.ntile + tile] = dot2_value(d);
      }
    }
    for (int r = kFuseRows; r < nr; ++r)
      if (lane == 0) {
        const int i = warp + kFuseWarps * r;
        J.gpart[(size_t)act[i] * J.ntile + tile] = dot2_value(ovf[i - kFuseRegRowsTotal]);
      }
    zero_inactive(J, tile, pos);
  }
  if (!hess) return;
  // Epilogue: the block's Hessian partial from tensor memory. Warp w reads
  // lanes 32 (w % 4) .. + 31; warps w and w + 4 take alternate 8-column chunks.
  wait_mma();  // the last commit covers every MMA of the block
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();
  const bool ok = nmma > 0 && !timed_out;
  float* out = reinterpret_cast<float*>(J.hpart) + (size_t)local * (S * (S + 1) / 2);
  const int quad = warp & 3;
  for (int part2 = 0; part2 < (has_d2 ? 2 : 1); ++part2) {
    const int ncols = part2 == 0 ? n1 : n1 - umma::kTcM;
    const int col0 = part2 == 0 ? 0 : c2;
    const int row = part2 == 0 ? quad * 32 + lane : n1 - umma::kTcM + quad * 32 + lane;  // row of H
    for (int c = 8 * (warp >> 2); c < ncols; c += 16) {
      uint32_t vv[8];
      if (ok) {
        const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(col0 + c);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
            : "=r"(vv[0]), "=r"(vv[1]), "=r"(vv[2]), "=r"(vv[3]), "=r"(vv[4]), "=r"(vv[5]),
              "=r"(vv[6]), "=r"(vv[7])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) vv[q] = 0u;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float h = __uint_as_float(vv[q]);
        if (part2 == 0) {
          const int i = row, j = c + q;  // D1: H[i][j], i < 128
          if (i < S && j < S) {
            if (j <= i) out[i * (i + 1) / 2 + j] = h;
            else if (j >= umma::kTcM) out[j * (j + 1) / 2 + i] = h;  // H[j][i], j below row 128
          }
        } else {
          const int i = row, j = umma::kTcM + c + q;  // D2: H[i][j], i, j >= 128
          if (i >= umma::kTcM && i < S && j <= i) out[i * (i + 1) / 2 + j] = h;
        }
      }
    }
  }
  if (timed_out && threadIdx.x == 0) atomicOr(&J.mail->i[MI_ERR], E_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kFuseTmemCols));
  }
}

// Per-point outputs of the promolecule pass of a fused job, one block per
// point tile (after k_glisa_fused_ff<1>, which wrote rho0 as float pairs):
// w rho / rho0^2 (d2f, 0 where sick), the entropy terms w rho ln(rho / rho0)
// (ln from logf plus one Newton step on exp_ff, error ~ the square of
// logf's) and the count of points below negative_cutoff, per tile in
// jpart (QJ_ENTROPY, QJ_NEG).
__global__ void __launch_bounds__(kThreads) k_glisa_point_ff(Batch bt) {
  __shared__ float2 tab[64];
  __shared__ double red[2 * kWarps];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  if (glisa_idle(J)) return;
  if (!J.fuse) return;
  if (threadIdx.x < 64) tab[threadIdx.x] = c_exp2_gl[threadIdx.x];
  __syncthreads();
  const float2 cutp = split2(J.density_cutoff), negp = split2(J.negative_cutoff);
  const int p0 = tile * J.tile_points;
  const int p1 = min(p0 + J.tile_points, J.npoint);
  f2 ent{0.f, 0.f};
  float nneg = 0.0f;
  for (int p = p0 + threadIdx.x; p < p1; p += kThreads) {
    const float4 q = J.wrf[p];  // (w rho) and rho as float pairs
    const float2 r0s = J.r0f[p];
    const f2 r0{r0s.x, r0s.y};
    const bool sick = below(f2{q.z, q.w}, cutp) || below(r0, cutp);
    f2 dd{0.f, 0.f};
    if (!sick) {
      const f2 v = ffa::div(f2{q.x, q.y}, r0);
      dd = ffa::div(v, r0);
      const f2 ratio = ffa::div(f2{q.z, q.w}, r0);
      const float l0 = logf(ratio.hi);
      const f2 e = ffa::exp_ff(f2{-l0, 0.f}, tab);
      const f2 l = ffa::add(ffa::add(ffa::mul(ratio, e), -1.0f), l0);
      ent = ffa::add(ent, ffa::mul(f2{q.x, q.y}, l));
    }
    J.d2f[p] = make_float2(dd.hi, dd.lo);
    if (below(r0, negp)) nneg += 1.0f;
  }
  double e = ffa::to_double(ent), n = (double)nneg;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, o);
    n += __shfl_xor_sync(0xffffffffu, n, o);
  }
  if (lane == 0) {
    red[2 * warp] = e;
    red[2 * warp + 1] = n;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double se = 0.0, sn = 0.0;
    for (int k = 0; k < kWarps; ++k) {
      se += red[2 * k];
      sn += red[2 * k + 1];
    }
    J.jpart[(size_t)QJ_ENTROPY * J.ntile + tile] = se;
    J.jpart[(size_t)QJ_NEG * J.ntile + tile] = sn;
  }
}

// Trial objective differences for fused jobs: k_glisa_u_ff and
// k_glisa_trials_ff in one pass over staged sub-tiles (as k_glisa_fused_ff:
// the packed sub-tiles by TMA bulk copies into a staging ring). Per sub-tile: A forms the eight warps' partial sums
// of u = G^T delta and C the clipped-shell group sums (warp g: group g);
// then warp 0 merges the partials (warp order) into u and the groups into
// their suffix sums (group kTrials - 1 first), so that trial t reads the sum
// of the groups t..kTrials-1 at once; T: warp t evaluates trial t for the 32
// points (lane = point) and keeps its sum in registers; the tile's eight sums
// go to tpart at its end.
static_assert(kTrials == kFuseWarps, "one warp per trial step");

// Shared memory of the trial pass for S shells without its staging ring (bytes).
__host__ __device__ constexpr size_t trials_fixed_bytes(int S) {
  return 16 * (size_t)kTrials * kFuseSP           // group sums, then their suffix sums
         + 8 * (size_t)kFuseWarps * kFuseSP         // partial sums of u
         + 8 * (size_t)kFuseSP                      // u per point
         + 512                                      // exp table
         + 8 * (size_t)S                            // delta as float pairs
         + 12 * (size_t)S + 16                      // act, pos, clipped shells' rows
         + 16 + 8 * kRingSlots;                     // the ring's mbarriers
}
__host__ __device__ constexpr int trials_ring_floats(int S) {
  return (int)((kFuseSmemMax - trials_fixed_bytes(S)) / 128 * 32);
}
static_assert(trials_ring_floats(kFuseMaxShells) >= 2 * kFuseMaxShells * kFuseSP, "trial pass shared memory");

__global__ void __launch_bounds__(kFuseThreads, 2) k_glisa_trials_fused(Batch bt, int ring_floats) {
  extern __shared__ float4 fsm[];
  int local;
  const JobDev& J = decode_local_gf(bt, local);
  if (glisa_idle(J)) return;
  if (!J.fuse) return;
  // heaviest tiles first (the block scheduler starts the blocks in order)
  const int tile = J.fsched[min(J.ntile, kFuseCtas) + 1 + J.ntile + local];
  const int S = J.nshell;
  float* ring = reinterpret_cast<float*>(fsm);
  float4* grp = reinterpret_cast<float4*>(ring + ring_floats);  // [kTrials][kFuseSP]
  Dot2* part = reinterpret_cast<Dot2*>(grp + kTrials * kFuseSP);
  float2* uv = reinterpret_cast<float2*>(part + kFuseWarps * kFuseSP);
  float2* tab = uv + kFuseSP;  // exp table
  float2* xv = tab + 64;
  int* act = reinterpret_cast<int*>(xv + S);
  int* pos = act + S;
  int* cpos = pos + S;  // per clipped shell its active row on this tile (-1: zero here)
  uint64_t* rbar = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(cpos + S) + 15) & ~uintptr_t(15));
  const uint32_t rbar0 = umma::smem_u32(rbar);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p0 = tile * J.tile_points;
  const int p1 = min(p0 + J.tile_points, J.npoint);
  const int nsub = (p1 - p0 + kFuseSP - 1) / kFuseSP;
  const float2* __restrict__ r0in = J.r0f;
  const float4* __restrict__ wrfp = J.wrf;
  if (threadIdx.x == 0) {
    for (int b = 0; b < kRingSlots; ++b) umma::mbar_init(rbar0 + 8 * b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  const int nact = load_active(J, tile, act, pos);
  __syncthreads();
  // staging ring (as k_glisa_fused_ff)
  const int slotf = 2 * nact * kFuseSP;
  const int nslot = nact > 0 ? min(kRingSlots, max(1, ring_floats / slotf)) : 1;
  const float* src = J.gpack + J.gtile_off[tile];
  uint32_t ring_phase = 0;
  int timed_out = 0;
  auto issue = [&](int k) {
    const int b = k % nslot;
    const uint32_t bytes = (uint32_t)nact * kFuseSP * 4;
    umma::mbar_expect_tx(rbar0 + 8 * b, 2 * bytes);
    if (bytes) {
      const uint32_t dst = umma::smem_u32(ring + (size_t)b * slotf);
      umma::bulk_g2s(dst, src + (size_t)k * nact * kFuseSP, bytes, rbar0 + 8 * b);
      umma::bulk_g2s(dst + bytes, src + J.gpack_plane + (size_t)k * nact * kFuseSP, bytes, rbar0 + 8 * b);
    }
  };
  if (threadIdx.x == 0)
    for (int k2 = 0; k2 < nslot - 1 && k2 < nsub; ++k2) issue(k2);
  for (int i = threadIdx.x; i < nact; i += kFuseThreads) xv[i] = split2(J.delta[act[i]]);  // by active row
  const int t = warp;  // this warp's trial: step 2^-t
  const float at = ldexpf(1.0f, -t);
  const int nclip = J.clip[S];
  const int* tm = J.clip + S + 1;
  // clipped shells with t_m > t: a prefix of the list (sorted, largest
  // first) of length ktab[t]; group g = the shells with min(t_m, kTrials) =
  // g + 1, the list segment [ktab[g + 1], ktab[g]) (group kTrials - 1 from
  // 0), is clipped in the trials t <= g
  __shared__ int ktab[kTrials];
  if (threadIdx.x < kTrials) {
    int k = 0;
    while (k < nclip && tm[k] > (int)threadIdx.x) ++k;
    ktab[threadIdx.x] = k;
  }
  for (int k = threadIdx.x; k < nclip; k += kFuseThreads) cpos[k] = pos[J.clip[k]];
  const float4* cd = reinterpret_cast<const float4*>(J.clipf);
  const float2 cutp = split2(J.density_cutoff);
  if (threadIdx.x < 64) tab[threadIdx.x] = c_exp2_gl[threadIdx.x];
  float ah = 0.0f, al = 0.0f, an = 0.0f;
  for (int sub = 0; sub < nsub; ++sub) {
    const int slot = sub % nslot;
    const float* gh = ring + (size_t)slot * slotf;
    const float* gl = gh + nact * kFuseSP;
    __syncthreads();  // every thread is done with sub - 1 (its slot is free)
    if (threadIdx.x == 0 && sub + nslot - 1 < nsub) issue(sub + nslot - 1);
    const int pq = p0 + sub * kFuseSP + lane;  // this lane's point: inputs loaded before A
    float2 r0pre = make_float2(0.f, 0.f);
    float4 qpre = make_float4(0.f, 0.f, 0.f, 0.f);
    if (pq < p1) {
      r0pre = r0in[pq];
      qpre = wrfp[pq];
    }
    if (!timed_out && !umma::mbar_wait_sleep(rbar0 + 8 * slot, (ring_phase >> slot) & 1u))
      timed_out = 1;
    ring_phase ^= 1u << slot;
    {  // A (active rows i = warp mod 8; delta compacted by active row)
      Dot2 d{0.f, 0.f}, e{0.f, 0.f};
      int i = warp;
      const float* ghl = gh + lane;
      const float* gll = gl + lane;
      for (; i + kFuseWarps < nact; i += 2 * kFuseWarps) {
        const float2 x1 = xv[i], x2 = xv[i + kFuseWarps];
        dot2_add(d, ghl[i * kFuseSP], gll[i * kFuseSP], x1.x, x1.y);
        const int i2 = i + kFuseWarps;
        dot2_add(e, ghl[i2 * kFuseSP], gll[i2 * kFuseSP], x2.x, x2.y);
      }
      if (i < nact) {
        const float2 x1 = xv[i];
        dot2_add(d, ghl[i * kFuseSP], gll[i * kFuseSP], x1.x, x1.y);
      }
      dot2_merge(d, e);
      part[warp * kFuseSP + lane] = d;
    }
    {  // C: warp g sums the clipped shells of group g for the 32 points, once
      const int g = warp;
      const int k1 = ktab[g], k0 = g + 1 < kTrials ? ktab[g + 1] : 0;
      Dot2 sc{0.f, 0.f}, sd{0.f, 0.f};
      for (int k = k0; k < k1; ++k) {
        const int i = cpos[k];
        if (i < 0) continue;  // the shell is zero on this tile
        const float4 v = cd[k];
        const float g1 = gh[i * kFuseSP + lane], g2 = gl[i * kFuseSP + lane];
        dot2_add(sc, g1, g2, v.x, v.y);
        dot2_add(sd, g1, g2, v.z, v.w);
      }
      grp[g * kFuseSP + lane] = make_float4(sc.s, sc.c, sd.s, sd.c);
    }
    __syncthreads();
    if (warp == 0) {  // u (warp 0) and the groups' suffix sums (warp 1)
      Dot2 du = part[lane];
#pragma unroll
      for (int q = 1; q < kFuseWarps; ++q) dot2_merge(du, part[q * kFuseSP + lane]);
      const f2 u = dot2_ff(du);
      uv[lane] = make_float2(u.hi, u.lo);
    } else if (warp == 1) {
      float4 v = grp[(kTrials - 1) * kFuseSP + lane];
      Dot2 sc{v.x, v.y}, sd{v.z, v.w};
#pragma unroll
      for (int g = kTrials - 2; g >= 0; --g) {
        v = grp[g * kFuseSP + lane];
        dot2_merge(sc, Dot2{v.x, v.y});
        dot2_merge(sd, Dot2{v.z, v.w});
        grp[g * kFuseSP + lane] = make_float4(sc.s, sc.c, sd.s, sd.c);
      }
    }
    __syncthreads();
    const int p = pq;
    if (p < p1) {  // T
      const float2 uu = uv[lane];
      const f2 u{uu.x, uu.y};
      const float4 gs = grp[t * kFuseSP + lane];  // groups t .. kTrials - 1
      const f2 dsd = dot2_ff(Dot2{gs.z, gs.w});
      const f2 corr = ffa::neg(ffa::add(dot2_ff(Dot2{gs.x, gs.y}), f2{at * dsd.hi, at * dsd.lo}));
      const float2 r0p = r0pre;
      const float4 q = qpre;  // (w rho) and rho as float pairs
      const bool rs = below(f2{q.z, q.w}, cutp);
      const bool h0 = !(rs || below(f2{r0p.x, r0p.y}, cutp));
      const f2 dr = ffa::add(f2{at * u.hi, at * u.lo}, corr);
      const f2 rt = ffa::add(dr, f2{r0p.x, r0p.y});
      J.r0t[(size_t)t * J.npoint + p] = make_float2(rt.hi, rt.lo);  // rho0 of the trial (next pass)
      const bool ht = !(rs || below(rt, cutp));
      float term = 0.0f;
      if (h0 && ht) {
        term = -q.x * log1pf(dr.hi / r0p.x);
        an += fabsf(term);
      } else if (ht || h0) {
        // the sick status changes: +-(w rho) ln(rho / rho0) in float-float
        // (logf, then one Newton step on the float-float exponential)
        const f2 ratio = ffa::div(f2{q.z, q.w}, ht ? rt : f2{r0p.x, r0p.y});
        const float l0 = logf(ratio.hi);
        const f2 e = ffa::exp_ff(f2{-l0, 0.f}, tab);
        const f2 l = ffa::add(ffa::add(ffa::mul(ratio, e), -1.0f), l0);
        const f2 big = ffa::mul(f2{q.x, q.y}, ht ? l : ffa::neg(l));
        term = big.hi;
        al += big.lo;
      }
      const float s2 = ah + term;
      const float bb = s2 - ah;
      al += (ah - (s2 - bb)) + (term - bb);
      ah = s2;
    }
  }
  double v = (double)ah + (double)al, vn = (double)an;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_xor_sync(0xffffffffu, v, o);
    vn += __shfl_xor_sync(0xffffffffu, vn, o);
  }
  if (lane == 0) {
    J.tpart[(size_t)t * J.ntile + tile] = v;
    J.tpart[(size_t)(kTrials + t) * J.ntile + tile] = vn;
  }
  if (timed_out && lane == 0) atomicOr(&J.mail->i[MI_ERR], E_TIMEOUT);
}

// Outer change (glisa.py:776 via compute_change): sum over atoms of
// int w (sum_{m in atom} (c - c_old)_m g_m)^2, one block per point tile, all
// atoms per point (one read of G). The differences are formed in FP64 and
// each atom's sum over its shells is a compensated dot product; its square
// and the weight are FP32 (the change is compared with the threshold, where
// 1e-7 relative is ample), summed per thread as a float pair. The tile's
// total goes to atom 0's slot (the other atoms' slots get 0).
__global__ void __launch_bounds__(kThreads) k_glisa_change_ff(Batch bt) {
  __shared__ float2 dc[kGffMaxShells];
  __shared__ double red[kWarps];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  if (glisa_idle(J)) return;
  for (int i = threadIdx.x; i < J.nshell; i += kThreads) dc[i] = split2(J.propars[i] - J.propars_old[i]);
  __syncthreads();
  const size_t N = J.npoint;
  float ah = 0.0f, al = 0.0f;
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_in_tile(J, tile, i);
    if (p >= J.npoint) continue;
    const float wf = (float)J.w[p];
    int m = J.shell_off[0];
    for (int a = 0; a < J.natom; ++a) {
      const int m1 = J.shell_off[a + 1];
      Dot2 d{0.f, 0.f};
      for (; m < m1; ++m) dot2_add(d, J.gmat32[m * N + p], J.gmat_lo[m * N + p], dc[m].x, dc[m].y);
      const float v = d.s + d.c;
      const float term = wf * v * v;
      const float t = ah + term;
      const float bb = t - ah;
      al += (ah - (t - bb)) + (term - bb);
      ah = t;
    }
  }
  const double sum = block_sum1((double)ah + (double)al, red);
  for (int a = threadIdx.x; a < J.natom; a += kThreads)
    J.apart[((size_t)a * J.qa + QA_CHANGE) * J.ntile + tile] = a == 0 ? sum : 0.0;
}

// Active shells of every point tile of a fused job (once per job, after the
// basis): gact[tile][0..n) the shells with a nonzero value on the tile, in
// order, n at gact[tile][S]. A float-float value is zero exactly when its
// high part is, so the passes that skip the other rows add exact zeros less.
__global__ void __launch_bounds__(kThreads) k_glisa_active(Batch bt) {
  __shared__ int flag[kFuseMaxShells];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  if (!J.fuse) return;
  const int S = J.nshell;
  const size_t N = J.npoint;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p0 = tile * J.tile_points;
  const int p1 = min(p0 + J.tile_points, J.npoint);
  for (int m = warp; m < S; m += kWarps) {
    bool nz = false;
    for (int p = p0 + lane; p < p1; p += 32) nz |= J.gmat32[m * N + p] != 0.0f;
    nz = __any_sync(0xffffffffu, nz);
    if (lane == 0) flag[m] = nz ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int* g = J.gact + (size_t)tile * (S + 1);
    int n = 0;
    for (int m = 0; m < S; ++m)
      if (flag[m]) g[n++] = m;
    g[S] = n;
  }
}

// The active rows of every point tile of a fused job packed per 32-point
// sub-tile (after k_glisa_active): sub-tile s of tile t holds its nact rows
// of 32 points contiguously, gpack[gtile_off[t] + (s nact + i) 32 + l] =
// G[act[i]][p0 + 32 s + l] (0 past the job's last point), the low plane
// gpack_plane floats after the high one. One block per tile.
__global__ void __launch_bounds__(kThreads) k_glisa_pack(Batch bt) {
  __shared__ int act[kFuseMaxShells];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  if (!J.fuse || !J.gpack) return;
  const int S = J.nshell;
  const int* g = J.gact + (size_t)tile * (S + 1);
  const int nact = g[S];
  for (int i = threadIdx.x; i < nact; i += kThreads) act[i] = g[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p0 = tile * J.tile_points;
  const int p1 = min(p0 + J.tile_points, J.npoint);
  const int nsub = (p1 - p0 + 31) / 32;
  const size_t N = J.npoint;
  float* hi = J.gpack + J.gtile_off[tile];
  float* lo = hi + J.gpack_plane;
  // warp per active row, streaming along the row's points (coalesced
  // reads); sub-tile s of row i goes to ((s nact + i) 32 + lane)
  for (int i = warp; i < nact; i += kWarps) {
    const float* rh = J.gmat32 + (size_t)act[i] * N;
    const float* rl = J.gmat_lo + (size_t)act[i] * N;
    for (int sb = 0; sb < nsub; sb += 4) {
      float vh[4], vl[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int p = p0 + 32 * (sb + u) + lane;
        const bool in = sb + u < nsub && p < p1;
        vh[u] = in ? rh[p] : 0.0f;
        vl[u] = in ? rl[p] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (sb + u < nsub) {
          const size_t dst = ((size_t)(sb + u) * nact + i) * 32 + lane;
          hi[dst] = vh[u];
          lo[dst] = vl[u];
        }
    }
  }
}

// Per-atom weighted Gram blocks of G, for the outer change of fused jobs on
// the molecular grid (glisa.py:776 via compute_change). The change of a step
// is sum_a int w (sum_{i in a} dc_i g_i)^2 = sum_a dc_a^T W_a dc_a with
// W_a[i][j] = sum_p w_p g_i(p) g_j(p) over the shells i, j of atom a: the
// same quadrature sum regrouped, so no pass over the grid is needed per
// iteration (k_outer_finish forms the quadratic forms in FP64). W depends on
// G and the weights only and is formed at each job initialisation, after
// the basis: the tensor cores form the whole weighted Gram matrix
// G diag(w) G^T (k_glisa_hess_tc1 with the scale sqrt(w): X = G_hi sqrt(w)
// split into TF32 high and low parts, three MMAs per product, ~1e-6
// relative) as one FP32 triangle per point range in hpart, and
// k_glisa_wgram sums the ranges' values of the atoms' diagonal blocks in
// FP64 in range order, one warp per entry.
__global__ void __launch_bounds__(kThreads) k_glisa_wgram(Batch bt) {
  int local;
  const JobDev& J = decode_local_gf(bt, local);
  if (!J.fuse || !J.wgram) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int M = J.nshell;
  const size_t tri = (size_t)M * (M + 1) / 2;
  const float* hp = reinterpret_cast<const float*>(J.hpart);
  const int nblk = (M * M + kThreads - 1) / kThreads;  // this job's K_SQUARE blocks
  for (int e = local * kWarps + warp; e < J.wgn; e += nblk * kWarps) {
    int lo = 0, hi = J.natom;  // the atom a with wgoff[a] <= e < wgoff[a + 1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (J.wgoff[mid] <= e) lo = mid;
      else hi = mid;
    }
    const int q = e - J.wgoff[lo];  // local triangle entry (i, j), i >= j
    int i = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
    while (i * (i + 1) / 2 > q) --i;
    while ((i + 1) * (i + 2) / 2 <= q) ++i;
    const int j = q - i * (i + 1) / 2;
    const int gi = J.shell_off[lo] + i, gj = J.shell_off[lo] + j;
    const size_t t = (size_t)gi * (gi + 1) / 2 + gj;
    double h0 = 0.0, h1 = 0.0, h2 = 0.0, h3 = 0.0;
    int sp = lane;
    for (; sp + 96 < J.nsplit; sp += 128) {
      h0 += hp[(size_t)sp * tri + t];
      h1 += hp[(size_t)(sp + 32) * tri + t];
      h2 += hp[(size_t)(sp + 64) * tri + t];
      h3 += hp[(size_t)(sp + 96) * tri + t];
    }
    for (; sp < J.nsplit; sp += 32) h0 += hp[(size_t)sp * tri + t];
    double h = (h0 + h1) + (h2 + h3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if (lane == 0) J.wgram[e] = h;
  }
}

// Final promolecule of a float-float gLISA job (glisa.py:268-278 through
// core/stockholder.py:153-175): per point, each atom's pro-atom
// sum_m c_m g_m as a compensated dot product; rho_a, the promolecule (+1e-100
// per atom, as k_promol) and its reciprocal in FP64 for k_glisa_atweights_ff.
__global__ void __launch_bounds__(kThreads) k_glisa_promol_ff(Batch bt) {
  __shared__ float2 cf[kGffMaxShells];
  int blk;
  const JobDev& J = decode_local_gf(bt, blk);
  load_pairs(J.propars, J.nshell, cf);
  const int p = blk * kThreads + threadIdx.x;
  if (p >= J.npoint) return;
  const size_t N = J.npoint;
  double promol = 0.0;
  int m = J.shell_off[0];
  for (int a = 0; a < J.natom; ++a) {
    const int m1 = J.shell_off[a + 1];
    Dot2 d{0.f, 0.f};
    for (; m < m1; ++m) dot2_add(d, J.gmat32[m * N + p], J.gmat_lo[m * N + p], cf[m].x, cf[m].y);
    const double pro = dot2_value(d);
    J.rhoa[(size_t)a * N + p] = pro;
    promol += pro;
    promol += 1e-100;
  }
  J.promol[p] = promol;
  J.invpro[p] = 1.0 / promol;
}

// at_weights of a float-float gLISA job from the final promolecule, one block
// per point tile for all atoms (k_atweights takes a block per atom and tile
// and re-reads the per-point arrays for each atom): per atom
// rho_a = clip(pro_a / promol, 0, 1) rho, the tile's sum of w rho_a (QA_POP)
// and largest rho_a, and the tile's entropy sum of w rho ln(rho / promol)
// over the points above the cutoff. Each thread takes its points in the same
// order and the block sums are the same as in k_atweights.
__global__ void __launch_bounds__(kThreads) k_glisa_atweights_ff(Batch bt) {
  __shared__ double red[kWarps];
  __shared__ double out[1];
  __shared__ float redm[kWarps];
  int tile;
  const JobDev& J = decode_local_gf(bt, tile);
  const size_t N = J.npoint;
  double acc[1] = {0.0};
  for (int i = 0; i < J.ppt; ++i) {
    const int p = point_in_tile(J, tile, i);
    if (p >= J.npoint) continue;
    const double promol = J.promol[p], rho = J.rho[p];
    const bool sick = (promol < J.density_cutoff) || (rho < J.density_cutoff);
    if (!sick) acc[0] += J.w[p] * rho * log(rho / promol);
  }
  block_sum<1>(acc, red, out);
  if (threadIdx.x == 0) J.jpart[(size_t)QJ_ENTROPY * J.ntile + tile] = out[0];
  // the largest rho_a per tile only where a per-atom cutoff keeps it (its
  // comparison and conversion are FP64 operations, like the sums)
  const bool want_max = J.amax != nullptr;
  for (int a = 0; a < J.natom; ++a) {
    double pop[1] = {0.0};
    float vmax = 0.0f;
    double* ra = J.rhoa + (size_t)a * N;
#pragma unroll 4
    for (int i = 0; i < J.ppt; ++i) {
      const int p = point_in_tile(J, tile, i);
      if (p >= J.npoint) continue;
      const double v = fmin(fmax(ra[p] * J.invpro[p], 0.0), 1.0) * J.rho[p];
      ra[p] = v;
      if (want_max) vmax = fmaxf(vmax, v > 3e38 ? 3e38f : (float)v);
      pop[0] += J.w[p] * v;
    }
    block_sum<1>(pop, red, out);
    if (want_max) {
      const float mx = block_max_f(vmax, redm);
      if (threadIdx.x == 0) J.amax[(size_t)a * J.ntile + tile] = mx;
    }
    if (threadIdx.x == 0) J.apart[((size_t)a * J.qa + QA_POP) * J.ntile + tile] = out[0];
  }
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

namespace {

// 2^(i/64) as float pairs, from the host's double-precision exp2; once per device.
void ensure_exp_table_gl() {
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
  cudaMemcpyToSymbol(c_exp2_gl, t, sizeof(t));
  cudaFuncSetAttribute(k_glisa_fused_ff<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kFuseSmemMax);
  cudaFuncSetAttribute(k_glisa_fused_ff<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kFuseSmemMax);
  cudaFuncSetAttribute(k_glisa_trials_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kFuseSmemMax);
  if (dev < 31) done_mask |= 1 << dev;
}

}  // namespace

void launch_glisa_point_ff(const HostBatch& hb, cudaStream_t st) {
  if (hb.blocks[K_POINT] > 0) {
    ensure_exp_table_gl();
    k_glisa_point_ff<<<hb.blocks[K_POINT], kThreads, 0, st>>>(hb.b[K_POINT]);
    ++g_launch_count;
  }
}

void launch_glisa_fused_ff(const HostBatch& hb, cudaStream_t st, int mode, int max_shells,
                           bool point_pass) {
  if (hb.blocks[K_FUSE] <= 0) return;
  ensure_exp_table_gl();
  const int ring = fuse_ring_floats(max_shells, mode);
  const size_t smem = fuse_fixed_bytes(max_shells, mode) + 4 * (size_t)ring;
  if (mode) {
    k_glisa_fused_ff<1><<<hb.blocks[K_FUSE], kFuseThreads, smem, st>>>(hb.b[K_FUSE], ring);
    ++g_launch_count;
    if (point_pass && hb.blocks[K_POINT] > 0) {
      k_glisa_point_ff<<<hb.blocks[K_POINT], kThreads, 0, st>>>(hb.b[K_POINT]);
      ++g_launch_count;
    }
  } else {
    k_glisa_fused_ff<0><<<hb.blocks[K_FUSE], kFuseThreads, smem, st>>>(hb.b[K_FUSE], ring);
    ++g_launch_count;
  }
}

void launch_glisa_trials_fused(const HostBatch& hb, cudaStream_t st, int max_shells) {
  if (hb.blocks[K_POINT] <= 0) return;
  ensure_exp_table_gl();
  const int ring = trials_ring_floats(max_shells);
  k_glisa_trials_fused<<<hb.blocks[K_POINT], kFuseThreads,
                         trials_fixed_bytes(max_shells) + 4 * (size_t)ring, st>>>(hb.b[K_POINT], ring);
  ++g_launch_count;
}

void launch_glisa_active(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_active, K_POINT, kThreads);
}

void launch_glisa_pack(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_pack, K_POINT, kThreads);
}

void launch_glisa_wgram(const HostBatch& hb, cudaStream_t st) {
  launch_glisa_gram_tc(hb, st);
  HP_LAUNCH_GF(k_glisa_wgram, K_SQUARE, kThreads);
}

void launch_glisa_final_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_promol_ff, K_POINT1, kThreads);
  HP_LAUNCH_GF(k_glisa_atweights_ff, K_POINT, kThreads);
}

void launch_glisa_trials_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_u_ff, K_POINT1, kThreads);
  HP_LAUNCH_GF(k_glisa_trials_ff, K_POINT, kThreads);
}

void launch_glisa_change_ff(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_GF(k_glisa_change_ff, K_POINT, kThreads);
}

}  // namespace hp
