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

// ---- double-float values as a pair ------------------------------------------
struct dfv {
  float h, l;
};

// (a + b) renormalised, assuming |a| >= |b| (fast two-sum)
__device__ __forceinline__ dfv df_quick(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfv{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfv df_mul(dfv a, dfv b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_quick(p, e);
}

__device__ __forceinline__ dfv df_sum(dfv a, dfv b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return df_quick(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ dfv df_neg(dfv a) { return dfv{-a.h, -a.l}; }

// 1 / a: FP32 reciprocal refined by one double-float Newton step
__device__ __forceinline__ dfv df_rcp(dfv a) {
  const float r0 = __frcp_rn(a.h);
  const dfv ar = df_mul(a, dfv{r0, 0.f});
  const dfv e = df_sum(dfv{1.f, 0.f}, df_neg(ar));          // 1 - a r0, small
  return df_sum(dfv{r0, 0.f}, df_mul(dfv{r0, 0.f}, e));
}

// double -> double-float with integer instructions: hi = the leading 24
// significant bits of v (truncated), lo = the next 24 bits of the remainder
// (truncated), so hi + lo = v within 2^-48 |v|.  Magnitudes outside
// [2^-70, 2^100] (including 0, inf, nan) take a conversion instruction.
__device__ __forceinline__ dfv df_from_double(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const uint32_t hi32 = (uint32_t)(u >> 32), lo32 = (uint32_t)u;
  const int e = (int)((hi32 >> 20) & 0x7ffu) - 1023;
  if (e < -70 || e > 100) return dfv{__double2float_rn(v), 0.f};
  const uint32_t sign = hi32 & 0x80000000u;
  const uint32_t m23 = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
  const float h = __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | m23);
  const uint32_t r = lo32 & 0x1fffffffu;   // remainder r * 2^(e - 52)
  float l = 0.f;
  if (r != 0u) {
    const int k = 31 - __clz(r);            // leading bit of r, 0..28
    const uint32_t mant = k >= 23 ? (r >> (k - 23)) : (r << (23 - k));
    l = __uint_as_float(sign | ((uint32_t)(e - 52 + k + 127) << 23) | (mant & 0x7fffffu));
  }
  return dfv{h, l};
}
