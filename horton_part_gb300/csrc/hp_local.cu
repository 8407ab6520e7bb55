// Atom grids (grid_type 1): the reference's class default. MBIS, GISA and
// aLISA (sc) update each atom on its radial grid; gLISA only measures its
// change there.
//
// The promolecule and the at_weights are formed on the molecular grid as for
// grid_type 2/3 (core/stockholder.py:352-384). Each atom then works on its
// own atom grid: the AIM density w_a rho is spherically averaged over each
// radial shell of the atom's grid (the node values of the spline that
// qc-grid's AtomGrid.spherical_average returns, mbis.py:174-187), the inner
// MBIS fixed point runs on the atom's radial grid with the weights
// 4 pi r^2 w_r (mbis.py:81-163, all inner iterations of all atoms in one
// launch: one block per atom), the atom's population is the radial integral
// of the average, and the outer change is the radial integral of the
// squared pro-atom difference (core/iterstock.py:43-44). All FP64: the
// radial grids have ~10^2 nodes per atom.
//
// Layout: atom a owns radial shells [rad_off[a], rad_off[a+1]); shell s owns
// the consecutive grid points [shell_pt[s], shell_pt[s+1]) with angular
// weights wsph (Lebedev weight / 4 pi, summing to 1 over a shell).
#include <math.h>

#include "hp_internal.cuh"

namespace hp {

namespace {

__device__ __forceinline__ const JobDev& decode_atom_lc(const Batch& bt, int& atom) {
  const int j = find_job(bt, blockIdx.x);
  atom = blockIdx.x - bt.prefix[j];
  return bt.jobs[j];
}

// rho_a at point p in the storage format of the job's evaluation phase.
__device__ __forceinline__ double rhoa_value(const JobDev& J, int a, int p) {
  const size_t e = (size_t)a * J.npoint + p;
  if (J.mixed == PH_FP32) return (double)reinterpret_cast<const float*>(J.rhoa)[e];
  if (J.mixed == PH_FF) {
    const float2 v = reinterpret_cast<const float2*>(J.rhoa)[e];
    return (double)v.x + (double)v.y;
  }
  return J.rhoa[e];
}

// Per-atom value into tile 0 of a partial array, zeros in the other tiles
// (the outer kernels sum partials over tiles).
__device__ __forceinline__ void put_atom_partial(const JobDev& J, int a, int q, double v) {
  double* slot = J.apart + ((size_t)a * J.qa + q) * J.ntile;
  for (int t = threadIdx.x; t < J.ntile; t += blockDim.x) store_partial(J, slot + t, t == 0 ? v : 0.0);
}

// Unit-population shell s of a basis scheme at distance r (core/basis.py:161).
__device__ __forceinline__ double radial_shell(const JobDev& J, int s, double r) {
  return basis_shell<double>(J.sh_order[s], J.sh_alpha[s], J.sh_pref[s], r);
}

constexpr int kLocalMaxRad = 1024;  // radial nodes per atom
constexpr int kLocalQ = 2 * 7 + 1;  // MBIS moments (2 per shell) + inner change

}  // namespace

// Spherical averages: one block per atom, warps over its radial shells,
// lanes over a shell's points (fixed xor tree).
__global__ void __launch_bounds__(kThreads) k_sph_avg(Batch bt) {
  int a;
  const JobDev& J = decode_atom_lc(bt, a);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = J.rad_off[a] + warp; s < J.rad_off[a + 1]; s += kWarps) {
    double v = 0.0;
    for (long long p = J.shell_pt[s] + lane; p < J.shell_pt[s + 1]; p += 32)
      v += J.wsph[p] * rhoa_value(J, a, (int)p);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) J.radrho[s] = v;
  }
}

// Inner MBIS fixed point of every atom on its radial grid (one block per
// atom, every inner iteration in this launch), population and charge input.
__global__ void __launch_bounds__(kThreads) k_mbis_radial(Batch bt) {
  __shared__ double red[kWarps * kLocalQ];
  __shared__ double out[kLocalQ];
  __shared__ double par[14];
  __shared__ int done_s;
  int a;
  const JobDev& J = decode_atom_lc(bt, a);
  const int r0 = J.rad_off[a], nrad = J.rad_off[a + 1] - r0;
  const int nsh = J.shell_off[a + 1] - J.shell_off[a];
  double* pa = J.propars + J.par_off[a];
  if (threadIdx.x < 2 * nsh) par[threadIdx.x] = pa[threadIdx.x];
  if (threadIdx.x == 0) done_s = 0;
  // this thread's radial nodes (nrad <= kLocalMaxRad = 4 x kThreads)
  constexpr int kPer = kLocalMaxRad / kThreads;
  double rr[kPer], ww[kPer], rh[kPer], oldpro[kPer];
  double pop = 0.0;
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int i = threadIdx.x + q * kThreads;
    const bool in = i < nrad;
    rr[q] = in ? J.rad_r[r0 + i] : 1.0;
    ww[q] = in ? 4.0 * M_PI * rr[q] * rr[q] * J.rad_w[r0 + i] : 0.0;
    rh[q] = in ? J.radrho[r0 + i] : 0.0;
    oldpro[q] = 0.0;
    pop += ww[q] * rh[q];
  }
  {
    double acc1[1] = {pop};
    block_sum<1>(acc1, red, out);
    put_atom_partial(J, a, QA_POP, out[0]);
  }
  __syncthreads();
  int it = 0;
  double change = 1e100;
  for (; it < J.inner_maxiter; ++it) {
    double acc[kLocalQ];
#pragma unroll
    for (int q = 0; q < kLocalQ; ++q) acc[q] = 0.0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      double t[7];
      double pro = 0.0;
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        t[k] = 0.0;
        if (k < nsh) {
          const double n = par[2 * k], s = par[2 * k + 1];
          t[k] = n * s * s * s * exp(-s * rr[q]) * kInv8Pi;
          pro += t[k];
        }
      }
      const bool sick = (rh[q] < J.density_cutoff) || (pro < J.density_cutoff);
      const double ratio = sick ? 0.0 : rh[q] / pro;
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        if (k < nsh) {
          const double m0 = ww[q] * t[k] * ratio;
          acc[2 * k] += m0;
          acc[2 * k + 1] += m0 * rr[q];
        }
      }
      const double e = oldpro[q] - pro;
      acc[kLocalQ - 1] += ww[q] * e * e;
      oldpro[q] = pro;
    }
    block_sum<kLocalQ>(acc, red, out);
    if (threadIdx.x == 0) {
      for (int k = 0; k < nsh; ++k) {
        par[2 * k] = out[2 * k];
        par[2 * k + 1] = 3.0 * out[2 * k] / out[2 * k + 1];
      }
      change = it == 0 ? 1e100 : sqrt(out[kLocalQ - 1]);
      done_s = change < J.inner_threshold;
    }
    __syncthreads();
    if (done_s) break;
  }
  if (threadIdx.x < 2 * nsh) pa[threadIdx.x] = par[threadIdx.x];
  if (threadIdx.x == 0) {
    const bool conv = it < J.inner_maxiter;
    atomicAdd(&J.mail->d[MD_INNER_TOTAL], (double)(conv ? it + 1 : J.inner_maxiter));
    if (!conv) atomicOr(&J.mail->i[MI_WARN], W_INNER);
  }
}

// NLIS / GMBIS inner fixed point of every atom on its radial grid
// (nlis.py:99-195 on the spherical average; one block per atom, every inner
// iteration in this launch), population for the charges. FP64.
__global__ void __launch_bounds__(kThreads) k_nlis_radial(Batch bt) {
  __shared__ double red[kWarps * kLocalQ];
  __shared__ double out[kLocalQ];
  __shared__ double par[21];
  __shared__ double pu[7];
  __shared__ int done_s;
  int a;
  const JobDev& J = decode_atom_lc(bt, a);
  const int r0 = J.rad_off[a], nrad = J.rad_off[a + 1] - r0;
  const int nsh = J.shell_off[a + 1] - J.shell_off[a];
  double* pa = J.propars + J.par_off[a];
  if (threadIdx.x < 3 * nsh) par[threadIdx.x] = pa[threadIdx.x];
  if (threadIdx.x == 0) done_s = 0;
  constexpr int kPer = kLocalMaxRad / kThreads;
  double rr[kPer], ww[kPer], rh[kPer], oldpro[kPer];
  double pop = 0.0;
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int i = threadIdx.x + q * kThreads;
    const bool in = i < nrad;
    rr[q] = in ? J.rad_r[r0 + i] : 1.0;
    ww[q] = in ? 4.0 * M_PI * rr[q] * rr[q] * J.rad_w[r0 + i] : 0.0;
    rh[q] = in ? J.radrho[r0 + i] : 0.0;
    oldpro[q] = 0.0;
    pop += ww[q] * rh[q];
  }
  {
    double acc1[1] = {pop};
    block_sum<1>(acc1, red, out);
    put_atom_partial(J, a, QA_POP, out[0]);
  }
  __syncthreads();
  int it = 0;
  for (; it < J.inner_maxiter; ++it) {
    if (threadIdx.x < nsh) {  // unit-shell prefactors n S^(3/n) / (4 pi Gamma(3/n))
      const double n = par[3 * threadIdx.x + 2];
      pu[threadIdx.x] = n * pow(par[3 * threadIdx.x + 1], 3.0 / n) / (4.0 * M_PI * tgamma(3.0 / n));
    }
    __syncthreads();
    double acc[kLocalQ];
#pragma unroll
    for (int q = 0; q < kLocalQ; ++q) acc[q] = 0.0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      double u[7], rn[7];
      double pro = 0.0;
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        u[k] = 0.0;
        rn[k] = 0.0;
        if (k < nsh) {
          rn[k] = nlis_rn(par[3 * k + 2], rr[q]);
          u[k] = pu[k] * exp(-par[3 * k + 1] * rn[k]);
          pro += par[3 * k] * u[k];
        }
      }
      const bool sick = (rh[q] < J.density_cutoff) || (pro < J.density_cutoff);
      const double ratio = sick ? 0.0 : rh[q] / pro;
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        if (k < nsh) {
          const double wu = ww[q] * u[k] * ratio;
          acc[2 * k] += wu * par[3 * k];
          acc[2 * k + 1] += wu * rn[k];
        }
      }
      const double e = oldpro[q] - pro;
      acc[kLocalQ - 1] += ww[q] * e * e;
      oldpro[q] = pro;
    }
    block_sum<kLocalQ>(acc, red, out);
    if (threadIdx.x == 0) {
      for (int k = 0; k < nsh; ++k) {
        const double n = par[3 * k + 2], m1 = out[2 * k + 1];
        par[3 * k] = out[2 * k];
        par[3 * k + 1] = fabs(m1) <= 1e-8 ? 1e-5 : 3.0 / (m1 * n);
      }
      const double change = it == 0 ? 1e100 : sqrt(out[kLocalQ - 1]);
      done_s = change < J.inner_threshold;
    }
    __syncthreads();
    if (done_s) break;
  }
  if (threadIdx.x < 3 * nsh) pa[threadIdx.x] = par[threadIdx.x];
  if (threadIdx.x == 0) {
    const bool conv = it < J.inner_maxiter;
    atomicAdd(&J.mail->d[MD_INNER_TOTAL], (double)(conv ? it + 1 : J.inner_maxiter));
    if (!conv) atomicOr(&J.mail->i[MI_WARN], W_INNER);
  }
}

// Outer change on the radial grids: sum_i 4 pi r_i^2 w_i (pro_new - pro_old)^2
// (MBIS: Slater shells of both parameter sets; basis schemes: the parameter
// differences times the unit-population shells at the nodes).
__global__ void __launch_bounds__(kThreads) k_change_radial(Batch bt) {
  __shared__ double red[kWarps];
  int a;
  const JobDev& J = decode_atom_lc(bt, a);
  if (glisa_idle(J)) return;
  const int r0 = J.rad_off[a], nrad = J.rad_off[a + 1] - r0;
  const int s0 = J.shell_off[a], nsh = J.shell_off[a + 1] - s0;
  const double* pn = J.propars + J.par_off[a];
  const double* po = J.propars_old + J.par_off[a];
  const bool mbis = J.scheme == SCHEME_MBIS;
  const bool nlis = J.scheme == SCHEME_NLIS;
  double acc = 0.0;
  for (int i = threadIdx.x; i < nrad; i += kThreads) {
    const double r = J.rad_r[r0 + i];
    double d = 0.0;
    for (int k = 0; k < nsh; ++k) {
      if (nlis) {
        d += nlis_shell(pn[3 * k], pn[3 * k + 1], pn[3 * k + 2], r);
        d -= nlis_shell(po[3 * k], po[3 * k + 1], po[3 * k + 2], r);
      } else if (mbis) {
        d += pn[2 * k] * pn[2 * k + 1] * pn[2 * k + 1] * pn[2 * k + 1] * exp(-pn[2 * k + 1] * r) * kInv8Pi;
        d -= po[2 * k] * po[2 * k + 1] * po[2 * k + 1] * po[2 * k + 1] * exp(-po[2 * k + 1] * r) * kInv8Pi;
      } else {
        d += (pn[k] - po[k]) * radial_shell(J, s0 + k, r);
      }
    }
    acc += 4.0 * M_PI * r * r * J.rad_w[r0 + i] * d * d;
  }
  const double s = block_sum1(acc, red);
  put_atom_partial(J, a, QA_CHANGE, s);
}

// GISA on atom grids (gisa.py:281-318): the quadratic program's moments
// q_k = sum_i 4 pi r_i^2 w_i g_k(r_i) rho_sph(r_i) and the population from
// the spherical average on the atom's radial grid, into tile 0 of the
// partials k_gisa_qp reads (one block per atom).
__global__ void __launch_bounds__(kThreads) k_basis_radial_qvec(Batch bt) {
  __shared__ double red[kWarps * (kMaxShells + 1)];
  __shared__ double out[kMaxShells + 1];
  int a;
  const JobDev& J = decode_atom_lc(bt, a);
  const int r0 = J.rad_off[a], nrad = J.rad_off[a + 1] - r0;
  const int s0 = J.shell_off[a], nsh = J.shell_off[a + 1] - s0;
  double acc[kMaxShells + 1];
#pragma unroll
  for (int q = 0; q <= kMaxShells; ++q) acc[q] = 0.0;
  for (int i = threadIdx.x; i < nrad; i += kThreads) {
    const double r = J.rad_r[r0 + i];
    const double wr = 4.0 * M_PI * r * r * J.rad_w[r0 + i] * J.radrho[r0 + i];
#pragma unroll
    for (int k = 0; k < kMaxShells; ++k)
      if (k < nsh) acc[k] += wr * radial_shell(J, s0 + k, r);
    acc[kMaxShells] += wr;
  }
  block_sum<kMaxShells + 1>(acc, red, out);
  for (int k = 0; k < nsh; ++k) put_atom_partial(J, a, QA_INNER + k, out[k]);
  put_atom_partial(J, a, QA_POP, out[kMaxShells]);
}

// aLISA self-consistent solver on atom grids (alisa.py:193-291 on the
// spherical average, gisa.py:281-318): every inner iteration of one atom in
// one block, c_k <- sum_i 4 pi r_i^2 w_i c_k g_k(r_i) rho_sph / pro until the
// radial change of the pro-atom is below the inner threshold; population
// for the charges.
__global__ void __launch_bounds__(kThreads) k_lisa_sc_radial(Batch bt) {
  __shared__ double red[kWarps * (kMaxShells + 1)];
  __shared__ double out[kMaxShells + 1];
  __shared__ double par[kMaxShells];
  __shared__ int done_s;
  int a;
  const JobDev& J = decode_atom_lc(bt, a);
  const int r0 = J.rad_off[a], nrad = J.rad_off[a + 1] - r0;
  const int s0 = J.shell_off[a], nsh = J.shell_off[a + 1] - s0;
  double* pa = J.propars + J.par_off[a];
  if (threadIdx.x < nsh) par[threadIdx.x] = pa[threadIdx.x];
  if (threadIdx.x == 0) done_s = 0;
  constexpr int kPer = kLocalMaxRad / kThreads;
  double rr[kPer], ww[kPer], rh[kPer], oldpro[kPer];
  double pop = 0.0;
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int i = threadIdx.x + q * kThreads;
    const bool in = i < nrad;
    rr[q] = in ? J.rad_r[r0 + i] : 1.0;
    ww[q] = in ? 4.0 * M_PI * rr[q] * rr[q] * J.rad_w[r0 + i] : 0.0;
    rh[q] = in ? J.radrho[r0 + i] : 0.0;
    oldpro[q] = 0.0;
    pop += ww[q] * rh[q];
  }
  {
    double acc1[1] = {pop};
    block_sum<1>(acc1, red, out);
    put_atom_partial(J, a, QA_POP, out[0]);
  }
  __syncthreads();
  int it = 0;
  for (; it < J.inner_maxiter; ++it) {
    double acc[kMaxShells + 1];
#pragma unroll
    for (int q = 0; q <= kMaxShells; ++q) acc[q] = 0.0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      double pro = 0.0;
      for (int k = 0; k < nsh; ++k) pro += par[k] * radial_shell(J, s0 + k, rr[q]);
      const bool sick = (rh[q] < J.density_cutoff) || (pro < J.density_cutoff);
      const double ratio = sick ? 0.0 : rh[q] / pro;
      const double wr = ww[q] * ratio;
#pragma unroll
      for (int k = 0; k < kMaxShells; ++k)
        if (k < nsh) acc[k] += wr * par[k] * radial_shell(J, s0 + k, rr[q]);
      const double e = oldpro[q] - pro;
      acc[kMaxShells] += ww[q] * e * e;
      oldpro[q] = pro;
    }
    block_sum<kMaxShells + 1>(acc, red, out);
    if (threadIdx.x == 0) {
      for (int k = 0; k < nsh; ++k) par[k] = out[k];
      const double change = it == 0 ? 1e100 : sqrt(out[kMaxShells]);
      done_s = change < J.inner_threshold;
    }
    __syncthreads();
    if (done_s) break;
  }
  if (threadIdx.x < nsh) pa[threadIdx.x] = par[threadIdx.x];
  if (threadIdx.x == 0) {
    const bool conv = it < J.inner_maxiter;
    atomicAdd(&J.mail->d[MD_INNER_TOTAL], (double)(conv ? it + 1 : J.inner_maxiter));
    if (!conv) atomicOr(&J.mail->i[MI_WARN], W_INNER);
  }
}

#define HP_LAUNCH_LC(kernel, kind, threads, ...)                                       \
  do {                                                                                 \
    if (hb.blocks[kind] > 0) {                                                         \
      kernel<<<hb.blocks[kind], threads, 0, st>>>(hb.b[kind], ##__VA_ARGS__);          \
      ++g_launch_count;                                                                \
    }                                                                                  \
  } while (0)

void launch_mbis_local(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_LC(k_sph_avg, K_ATOM, kThreads);
  HP_LAUNCH_LC(k_mbis_radial, K_ATOM, kThreads);
}

void launch_change_radial(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_LC(k_change_radial, K_ATOM, kThreads);
}

void launch_nlis_local(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_LC(k_sph_avg, K_ATOM, kThreads);
  HP_LAUNCH_LC(k_nlis_radial, K_ATOM, kThreads);
}

void launch_gisa_local(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_LC(k_sph_avg, K_ATOM, kThreads);
  HP_LAUNCH_LC(k_basis_radial_qvec, K_ATOM, kThreads);
}

void launch_lisa_sc_local(const HostBatch& hb, cudaStream_t st) {
  HP_LAUNCH_LC(k_sph_avg, K_ATOM, kThreads);
  HP_LAUNCH_LC(k_lisa_sc_radial, K_ATOM, kThreads);
}

}  // namespace hp
