// Float-float ("double-single") arithmetic on the FP32 pipes.
//
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits (relative accuracy ~1e-14). GB300 executes FP64
// at 1/64 of the FP32 rate (2 DFMA vs 128 FFMA per clock per SM), so the
// pro-atom evaluations that must be FP64-accurate are done in this format:
// an FF multiply-add costs ~6 FP32 instructions, an FF exponential ~60.
//
// Building blocks (Dekker 1971, Knuth TAOCP vol. 2 4.2.2; the FF layer as
// in Hida, Li and Bailey's double-double library, restated for floats):
//   two_sum       s + e = a + b exactly (6 flops)
//   fast_two_sum  same for |a| >= |b| (3 flops)
//   two_prod      p + e = a * b exactly (FMA)
// Exponential: Tang's table-driven method (ACM TOMS 15(2), 1989) with
// 64 table entries 2^(i/64) held as FF pairs (written once per device from
// the host's double-precision exp2).
#pragma once

#include <cuda_runtime.h>

namespace hp {
namespace ffa {

struct f2 {
  float hi, lo;
};

__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ f2 two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ f2 from_float(float a) { return {a, 0.0f}; }

__device__ __forceinline__ f2 add(f2 a, f2 b) {
  f2 s = two_sum(a.hi, b.hi);
  const f2 t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ f2 add(f2 a, float b) {
  f2 s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}

// a + b when no cancellation occurs (|a + b| not much below |a| + |b|, e.g.
// operands of the same sign): cheaper, same accuracy.
__device__ __forceinline__ f2 add_pos(f2 a, f2 b) {
  f2 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ f2 sqr(f2 a) {
  f2 p = two_prod(a.hi, a.hi);
  p.lo = fmaf(2.0f * a.hi, a.lo, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ f2 neg(f2 a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ f2 sub(f2 a, f2 b) { return add(a, neg(b)); }

__device__ __forceinline__ f2 mul(f2 a, f2 b) {
  f2 p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, p.lo);
  p.lo = fmaf(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ f2 mul(f2 a, float b) {
  f2 p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

// a / b: one correction of the float quotient (error ~ eps^2).
__device__ __forceinline__ f2 div(f2 a, f2 b) {
  const float inv = __frcp_rn(b.hi);
  const float q1 = a.hi * inv;
  const f2 r = sub(a, mul(b, q1));
  return fast_two_sum(q1, r.hi * inv);
}

// sqrt(a), a > 0: one Newton correction of the float root.
__device__ __forceinline__ f2 sqrt_ff(f2 a) {
  const float y = sqrtf(a.hi);
  const f2 d = sub(a, two_prod(y, y));
  return fast_two_sum(y, d.hi * (0.5f / y));
}

__device__ __forceinline__ double to_double(f2 a) { return (double)a.hi + (double)a.lo; }

// exp(x) for an FF argument x <= 88 (returns 0 below the FP32 normal range,
// x < -87). x = (64 m + i) ln2/64 + r, |r| <= ln2/128, with ln2/64 split into
// three floats (the first with 9 significant bits, so n times it is exact);
// exp(r) = 1 + r + r^2/2 + r^3 (1/6 + r/24 + r^2/120) (truncation < 4e-17).
__device__ __forceinline__ f2 exp_ff(f2 x, const float2* tab) {
  if (x.hi < -87.0f) return {0.0f, 0.0f};
  const float kL1 = 0x1.63p-7f, kL2 = -0x1.bd0106p-19f, kL3 = 0x1.cf79acp-46f;
  const float nf = rintf(x.hi * 92.3324813842773f);  // 64 / ln2
  const int n = (int)nf;
  // r = x - n (L1 + L2 + L3): x.hi - n L1 is exact (n L1 fits a float and the
  // difference is exact by Sterbenz), n L2 is formed exactly by two_prod
  const f2 p2 = two_prod(nf, kL2);
  f2 r = two_sum(x.hi - nf * kL1, x.lo);
  r = add(r, -p2.hi);
  r = add(r, -(p2.lo + nf * kL3));
  // 1 + r + r^2/2 + c
  f2 sq = two_prod(r.hi, r.hi);
  sq.lo = fmaf(2.0f * r.hi, r.lo, sq.lo);
  const f2 half = {0.5f * sq.hi, 0.5f * sq.lo};
  const float c =
      r.hi * sq.hi * fmaf(r.hi, fmaf(r.hi, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f);
  // |r^2/2| << |r| and |c| << |r|: no cancellation, so the cheaper sums
  // (two_sum of the high parts) keep the full accuracy
  f2 e = add_pos(r, half);
  e = add(e, c);
  e = add(e, 1.0f);
  const int m = n >> 6;  // floor(n / 64)
  const int i = n - (m << 6);
  const float2 t = tab[i];
  f2 v = mul(f2{t.x, t.y}, e);
  const float scale = __int_as_float((min(max(m, -126), 127) + 127) << 23);  // 2^m
  return {v.hi * scale, v.lo * scale};
}

}  // namespace ffa
}  // namespace hp
