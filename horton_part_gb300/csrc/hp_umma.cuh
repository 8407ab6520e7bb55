// tcgen05 (5th-generation tensor core) and mbarrier helpers in inline PTX,
// shared by the tensor-core Hessian kernels (hp_tcgen05.cu) and the fused
// gLISA pass that forms the Hessian on the fly (hp_glisa_ff.cu).
//
// Operands are K-major tiles of 32-bit elements in shared memory with
// 128-byte rows in the 128-byte swizzle layout: element (row, k) at word
// row * 32 + ((k / 4) ^ (row mod 8)) * 4 + k mod 4, 8-row groups 1024 bytes
// apart, the tile 1024-byte aligned. Every mbarrier wait is bounded.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hp {
namespace umma {

constexpr int kTcM = 128;  // UMMA M (rows of A, tensor-memory lanes)
constexpr long long kWaitLimit = 1ll << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}


// UMMA shared-memory descriptor: start address, leading byte offset (unused
// for swizzled K-major; 16 B), stride byte offset 1024 B (between 8-row
// groups), descriptor version 1, 128B swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor, kind::tf32: D = F32 (bits 4-5), A = B = TF32
// (bits 7-9, 10-12), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__device__ __forceinline__ uint32_t idesc_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kTcM >> 4) << 24);
}

// High TF32 part of a float: sign, exponent and the top 10 mantissa bits.
constexpr uint32_t kTf32Mask = 0xFFFFE000u;

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; returns false on time-out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// try_wait that may suspend the thread for up to `ns` nanoseconds (woken
// when the phase completes), so that waiting warps issue few instructions.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint32_t bar, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}

// Bounded wait with suspension: at most kSleepWaitLimit tries of up to 1 us.
constexpr int kSleepWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait_sleep(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < kSleepWaitLimit; ++i)
    if (mbar_try_wait_sleep(bar, parity, 1000u)) return true;
  return false;
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

// One arrival that also adds `bytes` to the transaction count of the
// current phase (the producer of TMA bulk copies, mbarrier count 1).
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// Bulk copy (TMA, untiled) of `bytes` from global to this CTA's shared
// memory, completing on the mbarrier: both addresses 16-byte aligned, bytes
// a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// float -> TF32 with round-to-nearest (ties away), as a 32-bit pattern
// whose low 13 bits are zero.
__device__ __forceinline__ uint32_t to_tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

}  // namespace umma
}  // namespace hp
