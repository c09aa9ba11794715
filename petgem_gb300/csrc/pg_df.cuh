// Double-float arithmetic: a value is an unevaluated sum hi + lo of two
// FP32 numbers (~48-bit mantissa).  Products are made error-free with FMA and
// sums are compensated (two-sum), so results carry ~2^-48 relative error while
// running on the FP32 pipes (on GB300 ~57x the FP64 rate).  Every operation
// is a round-to-nearest intrinsic, so the compiler neither contracts a
// multiply into a following add nor reassociates: the transformations stay
// error-free and every kernel that uses them rounds identically.
#pragma once
#include <cuda_runtime.h>

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (sh, sl) += (ah, al) * (bh, bl); the accumulator stays unnormalised
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float ph = __fmul_rn(ah, bh);
  float pl = __fmaf_rn(ah, bh, -ph);
  pl = __fmaf_rn(ah, bl, pl);
  pl = __fmaf_rn(al, bh, pl);
  float t, e;
  two_sum(sh, ph, t, e);
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(e, pl));
}

// (sh, sl) += (bh, bl)
__device__ __forceinline__ void df_add(float& sh, float& sl, float bh, float bl) {
  float t, e;
  two_sum(sh, bh, t, e);
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(e, bl));
}


// float -> double by moving the IEEE fields with integer instructions: exact
// (like a conversion instruction) for every input, but off the FP64 pipe,
// which on GB300 runs ~2 operations per clock per SM.
__device__ __forceinline__ double f32_to_f64_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t ex = (u >> 23) & 0xffu;
  const uint32_t sign = u & 0x80000000u;
  const uint32_t m = u & 0x7fffffu;
  if (ex == 0u) {
    if (m == 0u) return __hiloint2double((int)sign, 0);
    // subnormal: m * 2^-149 with the leading bit of m at position k
    const int k = 31 - __clz(m);
    const unsigned long long frac = ((unsigned long long)m << (52 - k)) & 0xfffffffffffffull;
    const unsigned long long bits =
        ((unsigned long long)sign << 32) | ((unsigned long long)(k + 874) << 52) | frac;
    return __longlong_as_double((long long)bits);
  }
  uint32_t hi = sign | (((ex == 255u) ? 0x7ffu : ex + 896u) << 20) | (m >> 3);
  if (ex == 255u && m != 0u) hi |= 0x80000u;   // NaN stays NaN
  return __hiloint2double((int)hi, (int)(u << 29));
}

// hi + lo rounded once to double (one FP64 add)
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  return __dadd_rn(f32_to_f64_exact(hi), f32_to_f64_exact(lo));
}
