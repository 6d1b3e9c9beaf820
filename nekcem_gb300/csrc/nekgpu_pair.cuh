// Float-pair helpers shared by the mixed-precision kernels: FP64 <-> FP32
// pieces by integer operations (no FP64 or conversion-pipe instructions), the
// Knuth two-sum, and a non-overlapping float pair joined into one FP64 value.
#pragma once

#include <cuda_runtime.h>

namespace nekgpu {
namespace {

// ---------------------------------------------------------------------------
// integer-only FP64 -> FP32 pieces
// ---------------------------------------------------------------------------
// top 24 bits of the mantissa (truncation); |d| < 2^-126 -> signed zero
__device__ __forceinline__ float d2f_hi(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  unsigned m = __funnelshift_l(lo, hi, 3) - 0xC0000000u;
  m = (m & 0x7FFFFFFFu) | (hi & 0x80000000u);
  return __uint_as_float((hi & 0x7FF00000u) >= 0x38100000u ? m : (hi & 0x80000000u));
}
// d - d2f_hi(d): the low 29 mantissa bits as a float (same sign as d);
// zero when |d| < 2^-74 (where it is below 2^-97 in magnitude)
__device__ __forceinline__ float d2f_lo(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned L = lo & 0x1FFFFFFFu;
  const int ex = (int)((hi >> 20) & 0x7FFu);  // biased exponent
  const float scale = __int_as_float((ex - 948) << 23);  // 2^(ex-1075)
  float f = __uint2float_rn(L) * scale;
  f = (ex >= 949) ? f : 0.0f;
  return __uint_as_float(__float_as_uint(f) | (hi & 0x80000000u));
}
// exact FP32 -> FP64 for normal floats and zeros (FP32 subnormals, below
// 2^-126, come out as 2^-127 (1.m): their absolute error is below 2^-126).
// The FP64 exponent is the FP32 one rebiased by 1023 - 127 = 896; it stays
// below 2048, so the add never carries into the sign bit.
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned mag = b & 0x7FFFFFFFu;
  const unsigned hi = ((mag >> 3) + 0x38000000u) | (b & 0x80000000u);
  return __hiloint2double((int)(mag ? hi : b), (int)(b << 29));
}

// s + t as an FP64 value for a non-overlapping float pair (|t| <= ulp(s)/2, a
// two-sum output), by integer operations: t, in units of the FP64 ulp of s,
// is below 2^29 and lands in the 29 low mantissa bits that s leaves zero
// (added, or subtracted with a borrow from s's last float bit; in units of
// the lower binade when s is a power of two and t takes it below).  Exact
// whenever s + t fits in 53 bits, else t's bits below them are truncated
// (under one FP64 ulp).  Zero or subnormal t, or subnormal s: f2d(s).
__device__ __forceinline__ double pair_to_double(float s, float t) {
  const unsigned bs = __float_as_uint(s), bt = __float_as_uint(t);
  const int es = (int)((bs >> 23) & 0xFFu), et = (int)((bt >> 23) & 0xFFu);
  const unsigned opp = (bs ^ bt) >> 31;
  const int sh = et - es + 29 + (int)(opp & ((bs & 0x7FFFFFu) == 0u ? 1u : 0u));
  unsigned mt = (bt & 0x7FFFFFu) | 0x800000u;
  mt = (et != 0 && es != 0) ? mt : 0u;
  const unsigned x = sh >= 0 ? (mt << sh) : (mt >> min(-sh, 31));
  const long long xs = opp ? -(long long)x : (long long)x;
  return __longlong_as_double(__double_as_longlong(f2d(s)) + xs);
}

// Knuth two-sum: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

}  // namespace
}  // namespace nekgpu
