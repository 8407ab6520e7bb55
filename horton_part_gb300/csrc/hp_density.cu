// Density of contracted Gaussians on grid points (horton-part's density
// generator, scripts/generate_density.py:119-204: the basis functions on the
// points, then rho = einsum("ab,bp,ap->p", D, phi, phi) at :186-188), in
// FP64 on the GPU.
//
// One block per tile of T consecutive points (T chosen by the host so that
// the tile's basis values fit in shared memory, at most kDensTile):
//  1. the tile's bounding box; a shell is skipped for the whole tile when
//     a_min d_min^2 > kDensExpCut (a_min its smallest exponent, d_min the
//     distance from its centre to the box), i.e. every primitive is below
//     exp(-kDensExpCut) ~ 1e-26 of its peak there; the significant shells
//     are compacted in shell order (block prefix sum);
//  2. phi[f][p] for the significant functions: one thread per (shell, point)
//     forms the contracted radial factor sum_k c_k exp(-a_k r^2) and the
//     shell's Cartesian components (file order), combined into pure
//     functions with the shell's (2l+1) x ncart matrix (constant memory);
//  3. rho(p) = sum_a phi_a (D_aa phi_a + 2 sum_{b<a} D_ab phi_b) for every
//     density matrix (total, spin, ...): the block's threads split as
//     (point, a-slice), rows a = slice, slice + S, ... in order, and the
//     slices' sums are added in slice order.
// The arithmetic is FP64 throughout (exp, products and sums); the cost is
// the FP64 issue rate of phase 3 (n_sig^2 / 2 FMA per point and matrix).
#include <math.h>

#include "hp_internal.cuh"

namespace hp {

namespace {

constexpr int kDensThreads = 256;
constexpr int kDensTile = 64;
constexpr double kDensExpCut = 60.0;

// (2l+1) x ncart matrices of the pure functions of l = 2, 3 (row-major, rows
// m = 0, +1, -1, ...), set from the host tables.
__constant__ double c_pure2[5 * 6];
__constant__ double c_pure3[7 * 10];

// Cartesian components of one point for angular momentum l in file order
// (s; x y z; xx yy zz xy xz yz; xxx yyy zzz xyy xxy xxz xzz yzz yyz xyz).
__device__ __forceinline__ int cart_values(int l, double x, double y, double z, double* c) {
  switch (l) {
    case 0:
      c[0] = 1.0;
      return 1;
    case 1:
      c[0] = x;
      c[1] = y;
      c[2] = z;
      return 3;
    case 2:
      c[0] = x * x;
      c[1] = y * y;
      c[2] = z * z;
      c[3] = x * y;
      c[4] = x * z;
      c[5] = y * z;
      return 6;
    default:
      c[0] = x * x * x;
      c[1] = y * y * y;
      c[2] = z * z * z;
      c[3] = x * y * y;
      c[4] = x * x * y;
      c[5] = x * x * z;
      c[6] = x * z * z;
      c[7] = y * z * z;
      c[8] = y * y * z;
      c[9] = x * y * z;
      return 10;
  }
}

__device__ __forceinline__ double block_min_max(double v, bool is_max, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, u) : fmin(v, u);
  }
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = red[0];
  for (int w = 1; w < kDensThreads / 32; ++w) r = is_max ? fmax(r, red[w]) : fmin(r, red[w]);
  return r;
}

// Basis values of significant shell j of the tile at its point i (phase 2).
__device__ __forceinline__ void shell_values(const DensityArgs& a, int s, int64_t p, double* out,
                                             int T) {
  const int l = a.info[5 * s], pure = a.info[5 * s + 1];
  const double x = a.points[p * 3] - a.centers[3 * s];
  const double y = a.points[p * 3 + 1] - a.centers[3 * s + 1];
  const double z = a.points[p * 3 + 2] - a.centers[3 * s + 2];
  const double r2 = x * x + y * y + z * z;
  const int nprim = a.info[5 * s + 2], k0 = a.info[5 * s + 3];
  double rad = 0.0;
  for (int k = 0; k < nprim; ++k) rad += a.coefs[k0 + k] * exp(-a.exps[k0 + k] * r2);
  double c[10];
  const int nc = cart_values(l, x, y, z, c);
  if (!pure) {
    for (int q = 0; q < nc; ++q) out[(size_t)q * T] = rad * c[q];
  } else {
    const double* tm = l == 2 ? c_pure2 : c_pure3;
    for (int m = 0; m < 2 * l + 1; ++m) {
      double v = 0.0;
      for (int q = 0; q < nc; ++q) v += tm[m * nc + q] * c[q];
      out[(size_t)m * T] = rad * v;
    }
  }
}

// Shared memory: phi [nbasis][T] doubles, the slice sums (kDensThreads
// doubles), then the significant functions' basis indices (nbasis ints),
// the significant shells (nshell ints) and their first local function
// (nshell + 1 ints).
__global__ void __launch_bounds__(kDensThreads) k_density(DensityArgs a) {
  extern __shared__ double dsm[];
  __shared__ double red[kDensThreads / 32];
  __shared__ int wcnt[kDensThreads / 32], wfun[kDensThreads / 32];
  const int T = a.tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double* phi = dsm;
  double* slice = phi + (size_t)a.nbasis * T;
  int* fidx = reinterpret_cast<int*>(slice + kDensThreads);
  int* sidx = fidx + a.nbasis;
  int* soff = sidx + a.nshell;
  const int64_t p0 = (int64_t)blockIdx.x * T;
  const int np = (int)min((int64_t)T, a.npoint - p0);
  // 1. bounding box of the tile and the significant shells (in shell order)
  double lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    double vmin = INFINITY, vmax = -INFINITY;
    for (int i = threadIdx.x; i < np; i += kDensThreads) {
      const double v = a.points[(p0 + i) * 3 + k];
      vmin = fmin(vmin, v);
      vmax = fmax(vmax, v);
    }
    lo[k] = block_min_max(vmin, false, red);
    hi[k] = block_min_max(vmax, true, red);
  }
  int ns = 0, nf = 0;
  for (int base = 0; base < a.nshell; base += kDensThreads) {
    const int s = base + threadIdx.x;
    bool sig = false;
    int nfs = 0;
    if (s < a.nshell) {
      double d2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double c = a.centers[3 * s + k];
        const double d = c < lo[k] ? lo[k] - c : (c > hi[k] ? c - hi[k] : 0.0);
        d2 += d * d;
      }
      sig = a.amin[s] * d2 <= kDensExpCut;
      const int l = a.info[5 * s], pure = a.info[5 * s + 1];
      nfs = sig ? (pure ? 2 * l + 1 : (l + 1) * (l + 2) / 2) : 0;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, sig);
    int fpre = nfs;  // inclusive prefix of the function counts within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, fpre, o);
      if (lane >= o) fpre += u;
    }
    if (lane == 31) {
      wcnt[warp] = __popc(bal);
      wfun[warp] = fpre;
    }
    __syncthreads();
    int so = ns, fo = nf, st = ns, ft = nf;
    for (int w = 0; w < kDensThreads / 32; ++w) {
      if (w < warp) {
        so += wcnt[w];
        fo += wfun[w];
      }
      st += wcnt[w];
      ft += wfun[w];
    }
    if (sig) {
      const int j = so + __popc(bal & ((1u << lane) - 1u));
      sidx[j] = s;
      soff[j] = fo + fpre - nfs;
    }
    __syncthreads();
    ns = st;
    nf = ft;
  }
  if (threadIdx.x == 0) soff[ns] = nf;
  __syncthreads();
  for (int j = threadIdx.x; j < ns; j += kDensThreads) {
    const int f0 = a.info[5 * sidx[j] + 4];
    for (int q = soff[j]; q < soff[j + 1]; ++q) fidx[q] = f0 + (q - soff[j]);
  }
  if (a.stats && threadIdx.x == 0) {
    const unsigned long long nn = (unsigned long long)np;
    atomicAdd(&a.stats[0], (unsigned long long)ns);
    atomicAdd(&a.stats[1], (unsigned long long)nf * nn);
    atomicAdd(&a.stats[2], (unsigned long long)nf * (unsigned long long)(nf + 1) / 2ull * nn);
  }
  // 2. basis values of the significant shells (zero past the last point)
  for (int e = threadIdx.x; e < ns * T; e += kDensThreads) {
    const int j = e / T, i = e - j * T;
    double* out = phi + (size_t)soff[j] * T + i;
    if (i < np) {
      shell_values(a, sidx[j], p0 + i, out, T);
    } else {
      for (int q = 0; q < soff[j + 1] - soff[j]; ++q) out[(size_t)q * T] = 0.0;
    }
  }
  __syncthreads();
  // 3. rho for every matrix: thread (point i, slice q); rows a = q, q + S, ...
  const int S = kDensThreads / T;  // T divides kDensThreads
  const int i = threadIdx.x % T, q = threadIdx.x / T;
  for (int mat = 0; mat < a.nmat; ++mat) {
    const double* D = a.mats + (size_t)mat * a.nbasis * a.nbasis;
    double acc = 0.0;
    for (int ra = q; ra < nf; ra += S) {
      const double* Drow = D + (size_t)fidx[ra] * a.nbasis;
      const double pa = phi[(size_t)ra * T + i];
      double y = 0.0;
      for (int rb = 0; rb < ra; ++rb) y += Drow[fidx[rb]] * phi[(size_t)rb * T + i];
      acc += pa * (Drow[fidx[ra]] * pa + 2.0 * y);
    }
    slice[threadIdx.x] = acc;
    __syncthreads();
    if (q == 0 && i < np) {
      double r = 0.0;
      for (int k = 0; k < S; ++k) r += slice[k * T + i];
      a.out[(size_t)mat * a.npoint + p0 + i] = r;
    }
    __syncthreads();
  }
}

}  // namespace

size_t density_smem_bytes(int nbasis, int nshell, int tile) {
  return ((size_t)nbasis * tile + kDensThreads) * sizeof(double) +
         sizeof(int) * ((size_t)nbasis + 2 * (size_t)nshell + 1);
}

int density_tile(int nbasis, int nshell) {
  for (int t = kDensTile; t >= 8; t /= 2)
    if (density_smem_bytes(nbasis, nshell, t) <= kDensSmemMax) return t;
  return 0;
}

int set_pure_tables(const double* pure2, const double* pure3) {
  if (cudaMemcpyToSymbol(c_pure2, pure2, sizeof(double) * 5 * 6) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_pure3, pure3, sizeof(double) * 7 * 10) != cudaSuccess) return 1;
  return 0;
}

void launch_density(const DensityArgs& a, cudaStream_t st) {
  static int configured = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured != dev) {
    cudaFuncSetAttribute(k_density, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDensSmemMax);
    configured = dev;
  }
  const int64_t nblk = (a.npoint + a.tile - 1) / a.tile;
  if (nblk <= 0) return;
  k_density<<<(unsigned)nblk, kDensThreads, density_smem_bytes(a.nbasis, a.nshell, a.tile), st>>>(a);
  ++g_launch_count;
}

}  // namespace hp
