// gLISA Hessian on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   H = G diag(w rho / rho0^2) G^T = X X^T,   X[m][p] = G[m][p] s(p),
//   s(p) = sqrt(w rho / rho0^2) (0 where sick)          (glisa.py:457-470)
//
// Output tiles cover the lower triangle of H: row block i0 (128 rows, the
// UMMA M) against column block j0 (N columns, a multiple of 16 up to 256,
// ending at the tile's last row). One CTA (512 threads, one per SM: two
// 97 KB stages of shared memory) computes one tile over one range of grid
// points. Per block
// of 32 points the threads form X from G (FP32 copy) and s, split it into two
// TF32 parts X = X_hi + X_lo (X_hi: X with its low 13 mantissa bits cleared;
// X_lo = X - X_hi, exact, whose low bits the MMA ignores) and write A
// (128 x 32) and B (N x 32; on a diagonal tile B is A itself) K-major into
// one of two shared-memory stages in the
// 128-byte-swizzled layout; one thread issues tcgen05.mma.kind::tf32
// (M = 128, K = 8) for X_hi X_hi^T, X_hi X_lo^T and X_lo X_hi^T into one FP32
// accumulator in tensor memory and commits to the stage's mbarrier. Each
// thread keeps the operands of the next two blocks in registers (loads two
// blocks ahead), so HBM latency overlaps the staging of block k+1 and the
// MMAs of block k. The accumulator is
// read back with tcgen05.ld and written as the CTA's partial; partials over point ranges are summed in FP64
// in a fixed order (k_glisa_reduce). Relative accuracy of H is about 1e-7
// (the dropped X_lo X_lo^T term and FP32 accumulation); the Newton step is
// refined against the exact FP64 product H delta (k_glisa_refine), so the
// solver converges as with the FP64 Hessian.
//
// Every mbarrier wait is bounded: on time-out the kernel sets E_TIMEOUT,
// frees its tensor memory and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include "hp_internal.cuh"
#include "hp_umma.cuh"

namespace hp {

using namespace umma;

namespace {

constexpr int kTcNMax = 256;    // largest UMMA N
constexpr int kTcK = 32;        // points per block: 32 x 4 B = one 128-byte swizzle row
constexpr int kTcThreads = 512; // four warpgroups (each covers tensor-memory lanes 0..127)
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kRowsA = kTcM / kTcWarps;     // A rows staged per warp
constexpr int kRowsB = kTcNMax / kTcWarps;  // B rows staged per warp (at most)
constexpr int kTcCols = 256;    // tensor-memory columns (FP32 accumulator, N <= 256)
constexpr int kT1Rows = kTcSinglePassShells;  // single-pass form (k_glisa_hess_tc1)

// shared-memory layout (offsets from a 1024-byte-aligned base): two stages
// of (A_hi, A_lo, B_hi, B_lo), then the stages' mbarriers and the TMEM slot
constexpr int kOffAhi = 0;
constexpr int kOffAlo = kOffAhi + kTcM * kTcK * 4;     // 16 KB
constexpr int kOffBhi = kOffAlo + kTcM * kTcK * 4;     // 32 KB
constexpr int kOffBlo = kOffBhi + kTcNMax * kTcK * 4;  // 64 KB
constexpr int kStageBytes = kOffBlo + kTcNMax * kTcK * 4;  // 96 KB
constexpr int kOffBar = 2 * kStageBytes;               // 192 KB
constexpr int kSmemBytes = kOffBar + 64 + 1024;        // + alignment slack

// Lower-triangular tile list of an M x M Hessian: row block r0 (128 rows)
// pairs with column blocks of up to 256 columns that start before the
// block's end row. Returns the number of tiles; for idx in range also the
// tile's (i0, j0, n), n a multiple of 16.
__host__ __device__ inline int tc_tiles(int M, int idx, int* i0, int* j0, int* n) {
  int t = 0;
  for (int r0 = 0; r0 < M; r0 += kTcM) {
    const int rend = r0 + kTcM < M ? r0 + kTcM : M;  // columns j < rend are needed
    for (int c0 = 0; c0 < rend; c0 += kTcNMax) {
      if (t == idx) {
        int w = rend - c0;
        if (w > kTcNMax) w = kTcNMax;
        *i0 = r0;
        *j0 = c0;
        *n = (w + 15) / 16 * 16;
      }
      ++t;
    }
  }
  return t;
}

}  // namespace

__global__ void __launch_bounds__(kTcThreads) k_glisa_hess_tc(Batch bt) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* sm = smem_raw + (base - raw);
  const uint32_t bar0 = base + kOffBar;  // stage s: bar0 + 8 s
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kOffBar + 16);
  __shared__ int timed_out;

  const int jb = find_job(bt, blockIdx.x);
  const JobDev& J = bt.jobs[jb];
  if (glisa_idle(J)) return;
  const int local = blockIdx.x - bt.prefix[jb];
  const int M = J.nshell, N = J.npoint;
  if (M <= kT1Rows) return;  // k_glisa_hess_tc1
  const int ntiles = tc_tiles(M, -1, nullptr, nullptr, nullptr);
  const int split = local / ntiles;
  int i0 = 0, j0 = 0, ncol = 16;
  tc_tiles(M, local - split * ntiles, &i0, &j0, &ncol);
  const int chunk = ((N + J.nsplit - 1) / J.nsplit + kTcK - 1) / kTcK * kTcK;
  const int pbeg = split * chunk;
  const int pend = min(pbeg + chunk, N);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t idesc = idesc_tf32(ncol);
  // diagonal tile (B rows = the first ncol rows of A): the MMAs read A for B
  const bool diag = (j0 == i0) && (ncol <= kTcM);
  // 128B-swizzle layout of a K-major tile of 32-bit elements with 128-byte
  // rows: element (row, k) sits at word row * 32 + ((k / 4) ^ (row mod 8)) * 4
  // + k mod 4 (16-byte chunk c of row r at chunk c ^ (r mod 8); 8-row groups
  // 1024 bytes apart). This thread's rows all have row mod 8 = warp mod 8 and
  // its k is its lane, so the in-row word offset is one constant.
  const uint32_t swz_col = (uint32_t)((((lane >> 2) ^ (warp & 7)) << 2) | (lane & 3));

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTcCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    timed_out = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  // rows of this thread: A rows warp + 16 r (r < 8), B rows warp + 16 r
  // (row < ncol); operands of two blocks in flight (slots 0 and 1)
  float va0[kRowsA], vb0[kRowsB], s0 = 0.0f;
  float va1[kRowsA], vb1[kRowsB], s1 = 0.0f;
  auto load_block = [&](float (&va)[kRowsA], float (&vb)[kRowsB], float& s, int kb) {
    const int p = kb + lane;
    const bool inr = p < pend;
    s = inr ? J.hess_s[p] : 0.0f;
#pragma unroll
    for (int r = 0; r < kRowsA; ++r) {
      const int m = i0 + warp + kTcWarps * r;
      va[r] = (inr && m < M) ? J.gmat32[(size_t)m * N + p] : 0.0f;
    }
#pragma unroll
    for (int r = 0; r < kRowsB; ++r) {
      const int row = warp + kTcWarps * r;
      const int m = j0 + row;
      vb[r] = (!diag && inr && row < ncol && m < M) ? J.gmat32[(size_t)m * N + p] : 0.0f;
    }
  };

  int nblocks = 0;
  // one block: wait for its stage, stage it from registers, issue its MMAs,
  // refill the registers with the block two ahead; false when a wait timed out
  auto do_block = [&](float (&va)[kRowsA], float (&vb)[kRowsB], float& s, int kb) -> bool {
    const int st = nblocks & 1;
    uint8_t* stage = sm + st * kStageBytes;
    uint32_t* a_hi = reinterpret_cast<uint32_t*>(stage + kOffAhi);
    uint32_t* a_lo = reinterpret_cast<uint32_t*>(stage + kOffAlo);
    uint32_t* b_hi = reinterpret_cast<uint32_t*>(stage + kOffBhi);
    uint32_t* b_lo = reinterpret_cast<uint32_t*>(stage + kOffBlo);
    if (nblocks >= 2) {
      // the MMAs of block nblocks - 2 (the stage's previous commit, number
      // (nblocks >> 1) - 1 on this barrier) must have read the stage
      if (!mbar_wait_sleep(bar0 + 8 * st, (uint32_t)(((nblocks >> 1) - 1) & 1))) timed_out = 1;
    }
#pragma unroll
    for (int r = 0; r < kRowsA; ++r) {
      const float x = va[r] * s;
      const uint32_t hi = __float_as_uint(x) & kTf32Mask;
      const uint32_t off = (uint32_t)((warp + kTcWarps * r) * 32) + swz_col;
      a_hi[off] = hi;
      a_lo[off] = __float_as_uint(x - __uint_as_float(hi));
    }
    if (!diag) {
#pragma unroll
      for (int r = 0; r < kRowsB; ++r) {
        const int row = warp + kTcWarps * r;
        if (row < ncol) {
          const float x = vb[r] * s;
          const uint32_t hi = __float_as_uint(x) & kTf32Mask;
          const uint32_t off = (uint32_t)(row * 32) + swz_col;
          b_hi[off] = hi;
          b_lo[off] = __float_as_uint(x - __uint_as_float(hi));
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (timed_out) return false;
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ahi = smem_u32(a_hi), alo = smem_u32(a_lo);
      const uint32_t bhi = diag ? ahi : smem_u32(b_hi), blo = diag ? alo : smem_u32(b_lo);
#pragma unroll
      for (int k = 0; k < kTcK / 8; ++k) {  // K = 8 TF32 = 32 bytes per MMA
        const uint32_t acc = (nblocks > 0 || k > 0) ? 1u : 0u;
        umma_tf32(tmem, umma_desc(ahi + 32 * k), umma_desc(bhi + 32 * k), idesc, acc);
        umma_tf32(tmem, umma_desc(ahi + 32 * k), umma_desc(blo + 32 * k), idesc, 1u);
        umma_tf32(tmem, umma_desc(alo + 32 * k), umma_desc(bhi + 32 * k), idesc, 1u);
      }
      umma_commit(bar0 + 8 * st);
    }
    ++nblocks;
    if (kb + 2 * kTcK < pend) load_block(va, vb, s, kb + 2 * kTcK);
    return true;
  };

  if (pbeg < pend) load_block(va0, vb0, s0, pbeg);
  if (pbeg + kTcK < pend) load_block(va1, vb1, s1, pbeg + kTcK);
  for (int kb = pbeg; kb < pend; kb += 2 * kTcK) {
    if (!do_block(va0, vb0, s0, kb)) break;
    if (kb + kTcK < pend && !do_block(va1, vb1, s1, kb + kTcK)) break;
  }
  if (nblocks > 0 && !timed_out) {
    // the last commit covers every MMA issued before it
    const int last = nblocks - 1;
    if (!mbar_wait_sleep(bar0 + 8 * (last & 1), (uint32_t)((last >> 1) & 1))) timed_out = 1;
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();

  // epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. + 31 (rows of the
  // tile); the four warps of a lane quarter take every fourth 8-column chunk
  double* out = J.hpart + (size_t)split * M * M;
  const int quad = warp & 3;
  const int i = i0 + quad * 32 + lane;
  const bool ok = nblocks > 0 && !timed_out;
  for (int c = 8 * (warp >> 2); c < ncol; c += 32) {
    uint32_t v[8];
    if (ok) {
      const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = 0u;
    }
    if (i < M) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int j = j0 + c + q;
        if (j < M && j <= i) out[(size_t)i * M + j] = (double)__uint_as_float(v[q]);
      }
    }
  }
  if (timed_out && threadIdx.x == 0) atomicOr(&J.mail->i[MI_ERR], E_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols));
  }
}

// ---------------------------------------------------------------------------
// Single-pass form for S <= 256 shells: one CTA per point range computes the
// whole lower triangle from one staging of X. Per block of 32 points the
// CTA stages rows 0..S-1 of X (hi and lo planes, 128B-swizzled K-major, rows
// S..255 zero, written once) and issues two accumulations:
//   D1 (TMEM columns 0..N1-1):    A = rows 0..127,   B = rows 0..N1-1,
//                                  N1 = S rounded up to 16;
//   D2 (TMEM columns 256..+N2-1): A = rows 128..255, B = rows 128..N1-1,
//                                  N2 = N1 - 128 (only when S > 128).
// D1 holds H[i][j] for i < 128 (its columns j >= 128 are the entries H[j][i]
// of the rows below 128), D2 the block i, j >= 128. Every X row is staged
// once per block (the tiled form stages up to three 128-row operands per
// block) and the MMA area per block is 128 x (N1 + N2).
// ---------------------------------------------------------------------------
constexpr int kT1Plane = kT1Rows * kTcK * 4;      // 32 KB
constexpr int kT1Stage = 2 * kT1Plane;             // hi + lo
constexpr int kT1Stages = 3;                       // shared-memory stages
constexpr int kT1OffBar = kT1Stages * kT1Stage;    // 192 KB
constexpr int kT1Smem = kT1OffBar + 64 + 1024;     // + barriers, TMEM slot, alignment slack
constexpr int kT1Cols = 512;                       // D1 at 0, D2 at 256
constexpr int kT1StageWarps = 16;                  // producers: rows warp + 16 r
constexpr int kT1Items = kT1Rows * (kTcK / 4) / (kT1StageWarps * 32);  // 16-byte chunks per producer
constexpr int kT1Threads = (kT1StageWarps + 1) * 32;  // + one warp that issues the MMAs

// Warp-specialised: warps 0..15 stage blocks into a ring of three shared-
// memory stages and arrive on the stage's "full" barrier (one arrival per
// warp); warp 16's elected lane waits for it, issues the block's MMAs and
// commits them to the stage's "empty" barrier, which the producers wait on
// before refilling the stage. No block-wide barrier per block: staging of
// the next blocks overlaps the MMAs of the previous ones.
__global__ void __launch_bounds__(kT1Threads) k_glisa_hess_tc1(Batch bt) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* sm = smem_raw + (base - raw);
  const uint32_t bar0 = base + kT1OffBar;  // full[s] at bar0 + 8 s, empty[s] at bar0 + 8 (3 + s)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kT1OffBar + 8 * 2 * kT1Stages);
  __shared__ volatile int timed_out;

  const int jb = find_job(bt, blockIdx.x);
  const JobDev& J = bt.jobs[jb];
  if (glisa_idle(J)) return;
  const int M = J.nshell, N = J.npoint;
  if (M > kT1Rows) return;  // the tiled kernel (k_glisa_hess_tc) takes this job
  const int split = blockIdx.x - bt.prefix[jb];
  const int chunk = ((N + J.nsplit - 1) / J.nsplit + kTcK - 1) / kTcK * kTcK;
  const int pbeg = split * chunk;
  const int pend = min(pbeg + chunk, N);
  const int nblk = pend > pbeg ? (pend - pbeg + kTcK - 1) / kTcK : 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n1 = (M + 15) / 16 * 16;
  const int n2 = n1 > kTcM ? n1 - kTcM : 0;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kT1Cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  // rows M..255 of both planes of every stage stay zero
  for (int e = threadIdx.x; e < kT1Stages * 2 * (kT1Rows - M) * kTcK; e += kT1Threads) {
    const int k = e % kTcK;
    const int rr = e / kTcK;
    const int row = M + rr % (kT1Rows - M);
    const int plane = rr / (kT1Rows - M);  // stage * 2 + (lo ? 1 : 0)
    reinterpret_cast<uint32_t*>(sm + plane * kT1Plane)[row * kTcK + k] = 0u;
  }
  if (threadIdx.x == 0) {
    for (int st = 0; st < kT1Stages; ++st) {
      mbar_init(bar0 + 8 * st, kT1StageWarps);
      mbar_init(bar0 + 8 * (kT1Stages + st), 1);
    }
    timed_out = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp < kT1StageWarps) {
    // producers: thread t stages the 16-byte chunk c = t mod 8 (points 4c ..
    // 4c + 3 of the block) of rows t / 8 + 64 j (< M): one 16-byte load of G,
    // the four scales, and one 16-byte store per plane into the chunk's
    // swizzled position (c ^ (row mod 8)). Operands of two blocks in registers.
    // The job's pointers live in registers: the asm statements below clobber
    // memory, which would otherwise reload them from the job table each block.
    const float* __restrict__ g32 = J.gmat32;
    const float* __restrict__ hsv = J.hess_s;
    const int tid = threadIdx.x;
    const int c = tid & 7;
    const int r0 = tid >> 3;
    const bool vec = (N & 3) == 0;  // 16-byte aligned rows; else element loads
    float4 v0[kT1Items], v1[kT1Items], s0 = make_float4(0.f, 0.f, 0.f, 0.f), s1 = s0;
    auto load_block = [&](float4 (&v)[kT1Items], float4& s, int k) {
      const int p = pbeg + k * kTcK + 4 * c;
      if (vec) {
        const bool inr = p < pend;  // pend is a multiple of 4 when N is
        s = inr ? *reinterpret_cast<const float4*>(hsv + p) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < kT1Items; ++j) {
          const int row = r0 + 64 * j;
          v[j] = (inr && row < M) ? *reinterpret_cast<const float4*>(g32 + (size_t)row * N + p)
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
        }
      } else {
        float sv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) sv[q] = p + q < pend ? hsv[p + q] : 0.0f;
        s = make_float4(sv[0], sv[1], sv[2], sv[3]);
#pragma unroll
        for (int j = 0; j < kT1Items; ++j) {
          const int row = r0 + 64 * j;
          float e[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) e[q] = (row < M && p + q < pend) ? g32[(size_t)row * N + p + q] : 0.0f;
          v[j] = make_float4(e[0], e[1], e[2], e[3]);
        }
      }
    };
    auto split_store = [&](uint8_t* hi_row, uint8_t* lo_row, float4 x) {
      const uint4 h = make_uint4(__float_as_uint(x.x) & kTf32Mask, __float_as_uint(x.y) & kTf32Mask,
                                 __float_as_uint(x.z) & kTf32Mask, __float_as_uint(x.w) & kTf32Mask);
      const uint4 l = make_uint4(__float_as_uint(x.x - __uint_as_float(h.x)),
                                 __float_as_uint(x.y - __uint_as_float(h.y)),
                                 __float_as_uint(x.z - __uint_as_float(h.z)),
                                 __float_as_uint(x.w - __uint_as_float(h.w)));
      *reinterpret_cast<uint4*>(hi_row) = h;
      *reinterpret_cast<uint4*>(lo_row) = l;
    };
    auto stage_block = [&](float4 (&v)[kT1Items], float4& s, int k) -> bool {
      const int st = k % kT1Stages;
      if (k >= kT1Stages &&
          !mbar_wait_sleep(bar0 + 8 * (kT1Stages + st), (uint32_t)((k / kT1Stages - 1) & 1))) {
        timed_out = 1;
        return false;
      }
      uint8_t* stage = sm + st * kT1Stage;
#pragma unroll
      for (int j = 0; j < kT1Items; ++j) {
        const int row = r0 + 64 * j;
        if (row < M) {
          const float4 x = make_float4(v[j].x * s.x, v[j].y * s.y, v[j].z * s.z, v[j].w * s.w);
          const int off = row * (kTcK * 4) + ((c ^ (row & 7)) << 4);
          split_store(stage + off, stage + kT1Plane + off, x);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(bar0 + 8 * st);
      if (k + 2 < nblk) load_block(v, s, k + 2);
      return true;
    };
    if (nblk > 0) load_block(v0, s0, 0);
    if (nblk > 1) load_block(v1, s1, 1);
    for (int k = 0; k < nblk; k += 2) {
      if (timed_out || !stage_block(v0, s0, k)) break;
      if (k + 1 < nblk && (timed_out || !stage_block(v1, s1, k + 1))) break;
    }
  } else if (lane == 0) {
    // the MMA issuer
    const uint32_t idesc1 = idesc_tf32(n1);
    const uint32_t idesc2 = idesc_tf32(n2 > 0 ? n2 : 16);
    for (int k = 0; k < nblk; ++k) {
      const int st = k % kT1Stages;
      if (timed_out || !mbar_wait_sleep(bar0 + 8 * st, (uint32_t)((k / kT1Stages) & 1))) {
        timed_out = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t hi = base + st * kT1Stage, lo = hi + kT1Plane;
      const uint32_t hi2 = hi + kTcM * kTcK * 4, lo2 = lo + kTcM * kTcK * 4;  // row 128
#pragma unroll
      for (int kk = 0; kk < kTcK / 8; ++kk) {
        const uint32_t acc = (k > 0 || kk > 0) ? 1u : 0u;
        umma_tf32(tmem, umma_desc(hi + 32 * kk), umma_desc(hi + 32 * kk), idesc1, acc);
        umma_tf32(tmem, umma_desc(hi + 32 * kk), umma_desc(lo + 32 * kk), idesc1, 1u);
        umma_tf32(tmem, umma_desc(lo + 32 * kk), umma_desc(hi + 32 * kk), idesc1, 1u);
        if (n2 > 0) {
          const uint32_t t2 = tmem + 256u;
          umma_tf32(t2, umma_desc(hi2 + 32 * kk), umma_desc(hi2 + 32 * kk), idesc2, acc);
          umma_tf32(t2, umma_desc(hi2 + 32 * kk), umma_desc(lo2 + 32 * kk), idesc2, 1u);
          umma_tf32(t2, umma_desc(lo2 + 32 * kk), umma_desc(hi2 + 32 * kk), idesc2, 1u);
        }
      }
      umma_commit(bar0 + 8 * (kT1Stages + st));
    }
    if (nblk > 0 && !timed_out) {  // the last commit covers every MMA
      const int last = nblk - 1;
      if (!mbar_wait_sleep(bar0 + 8 * (kT1Stages + last % kT1Stages), (uint32_t)((last / kT1Stages) & 1)))
        timed_out = 1;
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();

  // epilogue (producer warps): warp w reads tensor-memory lanes 32 (w % 4) ..
  // + 31; the four warps of a lane quarter take every fourth 8-column chunk;
  // the split's partial is the packed lower triangle in FP32
  float* out = reinterpret_cast<float*>(J.hpart) + (size_t)split * (M * (M + 1) / 2);
  const bool ok = nblk > 0 && !timed_out;
  if (warp < kT1StageWarps) {
    const int quad = warp & 3;
    for (int part = 0; part < 2; ++part) {
      const int ncols = part == 0 ? n1 : n2;
      const int i = part * kTcM + quad * 32 + lane;  // row of H
      for (int c = 8 * (warp >> 2); c < ncols; c += 32) {
        uint32_t v[8];
        if (ok) {
          const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(part * 256 + c);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                "=r"(v[7])
              : "r"(taddr));
          asm volatile("tcgen05.wait::ld.sync.aligned;");
        } else {
#pragma unroll
          for (int q = 0; q < 8; ++q) v[q] = 0u;
        }
        if (i < M) {
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int j = part * kTcM + c + q;
            if (j >= M) continue;
            const float h = __uint_as_float(v[q]);
            if (j <= i) out[i * (i + 1) / 2 + j] = h;
            else if (part == 0 && j >= kTcM) out[j * (j + 1) / 2 + i] = h;  // H[j][i], j below row 128
          }
        }
      }
    }
  }
  if (timed_out && threadIdx.x == 0) atomicOr(&J.mail->i[MI_ERR], E_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kT1Cols));
  }
}

// The weighted Gram matrix G diag(w) G^T of a fused job on the molecular
// grid (its per-atom diagonal blocks give the outer change): the same
// single-pass kernel with the scale sqrt(w) (hess_s, set by
// k_glisa_basis_ff), one CTA per point range over the fused pass's nsplit
// ranges (launch kind K_FUSE: min(ntile, kFuseCtas) blocks per job), into
// hpart, which the job's first fused pass overwrites.
void launch_glisa_gram_tc(const HostBatch& hb, cudaStream_t st) {
  static int configured_device = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured_device != dev) {
    cudaFuncSetAttribute(k_glisa_hess_tc1, cudaFuncAttributeMaxDynamicSharedMemorySize, kT1Smem);
    configured_device = dev;
  }
  if (hb.blocks[K_FUSE] <= 0) return;
  k_glisa_hess_tc1<<<hb.blocks[K_FUSE], kT1Threads, kT1Smem, st>>>(hb.b[K_FUSE]);
  ++g_launch_count;
}

int tc_hess_blocks(const JobDev& J) {
  if (J.nshell <= kT1Rows) return J.nsplit;  // k_glisa_hess_tc1: one CTA per point range
  return tc_tiles(J.nshell, -1, nullptr, nullptr, nullptr) * J.nsplit;
}

void launch_glisa_hess_tc(const HostBatch& hb, cudaStream_t st, int max_shells, int min_shells) {
  static int configured_device = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured_device != dev) {
    cudaFuncSetAttribute(k_glisa_hess_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    cudaFuncSetAttribute(k_glisa_hess_tc1, cudaFuncAttributeMaxDynamicSharedMemorySize, kT1Smem);
    configured_device = dev;
  }
  if (hb.blocks[K_HESS] <= 0) return;
  if (min_shells <= kT1Rows) {
    k_glisa_hess_tc1<<<hb.blocks[K_HESS], kT1Threads, kT1Smem, st>>>(hb.b[K_HESS]);
    ++g_launch_count;
  }
  if (max_shells > kT1Rows) {
    k_glisa_hess_tc<<<hb.blocks[K_HESS], kTcThreads, kSmemBytes, st>>>(hb.b[K_HESS]);
    ++g_launch_count;
  }
}

}  // namespace hp
