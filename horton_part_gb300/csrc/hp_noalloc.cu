// MBIS inner fixed point for one atom, allocating no memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a host
// application's own device-memory pool or arena (where a stray allocation
// breaks the pool's accounting or fragments it), plug-in hosts that forbid
// allocation after start-up, and latency-critical loops where an allocation
// would synchronise the device. hp_mbis_inner_noalloc serves them: the caller
// passes device pointers for every input and output, and the kernel's
// scratch (per-tile partial sums and the solver state) lives in the
// file-scope array below, which every GPU that loads this library holds until
// the process exits. Nothing here calls cudaMalloc, cudaFree or an
// allocating library routine.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "hp_internal.cuh"
#include "hpgpu.h"

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaPpt = 2;
constexpr int kNaTile = kNaThreads * kNaPpt;   // 512 points per block
constexpr int kNaMaxTiles = 4096;              // => at most 2,097,152 points
constexpr int kNaMaxShell = 7;                 // MBIS shells per atom (mbis.py:36-46)
constexpr int kNaQ = 2 * kNaMaxShell + 1;      // m0_k, m1_k, change
constexpr int kNaState = 64;                   // solver state, after the partials
// state layout (doubles): [0,14) current (N,S), [14,28) previous, 28 iteration,
// 29 done flag, 30 converged flag, 31 last change
constexpr int kSCur = 0, kSPrev = 14, kSIt = 28, kSDone = 29, kSConv = 30, kSChange = 31;

}  // namespace

// Scratch of hp_mbis_inner_noalloc: kNaQ x kNaMaxTiles partial sums plus the
// solver state, 61,504 doubles (492 KB) per device. Shared by every call on
// the device; the contents stay from the last call.
static __device__ __align__(256) double hp_noalloc_scratch[kNaQ * kNaMaxTiles + kNaState];

namespace {

__global__ void k_na_init(const double* __restrict__ propars, int nshell, double* scratch) {
  double* st = scratch + kNaQ * kNaMaxTiles;
  const int t = threadIdx.x;
  if (t < kNaState) st[t] = 0.0;  // clear the state left by the previous call
  __syncthreads();
  if (t < 2 * nshell) {
    st[kSCur + t] = propars[t];
    st[kSPrev + t] = propars[t];
  }
}

// Same arithmetic as the job kernel k_mbis_inner<double> (one atom).
__global__ void __launch_bounds__(kNaThreads)
    k_na_mbis_inner(const double* __restrict__ rho, const double* __restrict__ w,
                    const double* __restrict__ r, int npoint, int nshell, double density_cutoff,
                    double* scratch) {
  __shared__ double red[hp::kWarps * kNaQ];
  __shared__ double out[kNaQ];
  const double* st = scratch + kNaQ * kNaMaxTiles;
  if (st[kSDone] != 0.0) return;
  const bool first = st[kSIt] == 0.0;
  double cn[kNaMaxShell], cs[kNaMaxShell], pn[kNaMaxShell], ps[kNaMaxShell];
#pragma unroll
  for (int k = 0; k < kNaMaxShell; ++k) {
    const bool on = k < nshell;
    cn[k] = on ? st[kSCur + 2 * k] : 0.0;
    cs[k] = on ? st[kSCur + 2 * k + 1] : 0.0;
    pn[k] = on ? st[kSPrev + 2 * k] : 0.0;
    ps[k] = on ? st[kSPrev + 2 * k + 1] : 0.0;
  }
  double acc[kNaQ];
#pragma unroll
  for (int q = 0; q < kNaQ; ++q) acc[q] = 0.0;
  for (int i = 0; i < kNaPpt; ++i) {
    const int p = blockIdx.x * kNaTile + i * kNaThreads + threadIdx.x;
    if (p >= npoint) continue;
    const double rr = r[p];
    double t[kNaMaxShell];
    double pro = 0.0, oldpro = 0.0;
#pragma unroll
    for (int k = 0; k < kNaMaxShell; ++k) {
      t[k] = 0.0;
      if (k < nshell) {
        t[k] = hp::slater_shell<double>(cn[k], cs[k], rr);
        pro += t[k];
        if (!first) oldpro += hp::slater_shell<double>(pn[k], ps[k], rr);
      }
    }
    const double rh = rho[p];
    const double wp = w[p];
    const bool sick = (rh < density_cutoff) || (pro < density_cutoff);
    const double ratio = sick ? 0.0 : rh / pro;
#pragma unroll
    for (int k = 0; k < kNaMaxShell; ++k) {
      const double m0 = wp * (t[k] * ratio);
      acc[2 * k] += m0;
      acc[2 * k + 1] += m0 * rr;
    }
    const double e = oldpro - pro;
    acc[kNaQ - 1] += wp * e * e;
  }
  hp::block_sum<kNaQ>(acc, red, out);
  if (threadIdx.x < kNaQ) scratch[threadIdx.x * kNaMaxTiles + blockIdx.x] = out[threadIdx.x];
}

// One warp: fixed-order sums over tiles, parameter update, convergence test.
__global__ void k_na_mbis_update(int ntile, int nshell, double threshold, int maxiter,
                                 double* __restrict__ propars, double* scratch) {
  double* st = scratch + kNaQ * kNaMaxTiles;
  if (st[kSDone] != 0.0) return;
  const int lane = threadIdx.x & 31;
  double m[kNaQ];
  for (int q = 0; q < kNaQ; ++q) {
    double s = 0.0;
    if (q < 2 * nshell || q == kNaQ - 1)
      for (int t = lane; t < ntile; t += 32) s += scratch[q * kNaMaxTiles + t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    m[q] = s;
  }
  if (lane != 0) return;
  const int it = (int)st[kSIt];
  const double change = it == 0 ? 1e100 : sqrt(m[kNaQ - 1]);
  double nw[2 * kNaMaxShell];
  for (int k = 0; k < nshell; ++k) {
    nw[2 * k] = m[2 * k];
    nw[2 * k + 1] = 3.0 * m[2 * k] / m[2 * k + 1];
  }
  const bool conv = change < threshold;
  if (conv || it + 1 >= maxiter) {
    for (int q = 0; q < 2 * nshell; ++q) propars[q] = nw[q];
    st[kSDone] = 1.0;
    st[kSConv] = conv ? 1.0 : 0.0;
    st[kSChange] = change;
    st[kSIt] = (double)(it + 1);
  } else {
    for (int q = 0; q < 2 * nshell; ++q) {
      st[kSPrev + q] = st[kSCur + q];
      st[kSCur + q] = nw[q];
    }
    st[kSIt] = (double)(it + 1);
  }
}

std::mutex g_na_mutex;
// Per-device address of hp_noalloc_scratch, looked up once per process.
// cudaDeviceReset unloads the module: calls after a reset are unsupported.
double* g_na_ptr[64] = {};

// Status with its message for hp_last_error() (every error path sets one).
int na_fail(int code, const char* what, cudaError_t e = cudaSuccess) {
  std::string msg = std::string("hp_mbis_inner_noalloc: ") + what;
  if (e != cudaSuccess) msg += std::string(": ") + cudaGetErrorString(e);
  hp::set_error_text(msg.c_str());
  return code;
}

}  // namespace

extern "C" int32_t hp_mbis_inner_noalloc(const double* rho_a, const double* weights,
                                         const double* radial_dist, int64_t npoint,
                                         int32_t nshell, double* propars, double threshold,
                                         double density_cutoff, int32_t maxiter, int32_t* niter,
                                         int32_t* converged, void* stream) {
  if (!rho_a || !weights || !radial_dist || !propars)
    return na_fail(HP_ERR_INVALID, "null device pointer");
  if (nshell < 1 || nshell > kNaMaxShell) return na_fail(HP_ERR_INVALID, "nshell must be 1..7");
  if (maxiter < 1) return na_fail(HP_ERR_INVALID, "maxiter must be positive");
  if (npoint < 1 || npoint > (int64_t)kNaTile * kNaMaxTiles)
    return na_fail(HP_ERR_INVALID, "npoint must be 1..2,097,152 (size of the static scratch)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(HP_ERR_CUDA, "cudaGetDevice", e);
  if (dev < 0 || dev >= 64) return na_fail(HP_ERR_CUDA, "device index above 63");
  // An error left pending by the caller's own work is reported, not cleared:
  // it is theirs, and the launches below would otherwise be blamed for it.
  e = cudaPeekAtLastError();
  if (e != cudaSuccess) return na_fail(HP_ERR_CUDA, "a CUDA error was pending before the call", e);
  double* scratch = nullptr;
  {
    // Set-up, once per device, with that device current: the host-side name
    // hp_noalloc_scratch is not a device address; ask the runtime for it.
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, hp_noalloc_scratch);
      if (e != cudaSuccess || !p) return na_fail(HP_ERR_CUDA, "cudaGetSymbolAddress", e);
      g_na_ptr[dev] = (double*)p;
    }
    scratch = g_na_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int ntile = (int)((npoint + kNaTile - 1) / kNaTile);
  k_na_init<<<1, kNaState, 0, st>>>(propars, nshell, scratch);
  double state[kNaState];
  int launched = 0;
  while (launched < maxiter) {
    const int chunk = launched == 0 ? 8 : 4;
    for (int c = 0; c < chunk && launched < maxiter; ++c, ++launched) {
      k_na_mbis_inner<<<ntile, kNaThreads, 0, st>>>(rho_a, weights, radial_dist, (int)npoint, nshell,
                                                    density_cutoff, scratch);
      k_na_mbis_update<<<1, 32, 0, st>>>(ntile, nshell, threshold, maxiter, propars, scratch);
    }
    e = cudaGetLastError();  // nothing was pending above: these are our launches
    if (e != cudaSuccess) return na_fail(HP_ERR_CUDA, "kernel launch", e);
    e = cudaMemcpyAsync(state, scratch + kNaQ * kNaMaxTiles, sizeof(state), cudaMemcpyDeviceToHost,
                        st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return na_fail(HP_ERR_CUDA, "reading the solver state", e);
    if (state[kSDone] != 0.0) break;
  }
  if (niter) *niter = (int32_t)state[kSIt];
  if (converged) *converged = state[kSConv] != 0.0 ? 1 : 0;
  return HP_OK;
}
