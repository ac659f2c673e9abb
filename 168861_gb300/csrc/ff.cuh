// Double-float ("ff") arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers with |lo| <= ulp(hi), about 46 significant bits.  The mixed-precision implicit
// step uses it for what must be more precise than FP32 -- its refinement residual
// b - A x, formed from the step's FP64 potentials -- because the GB300 executes FP64
// arithmetic and FP64 <-> FP32 conversions at about 1/70 of its FP32 rate, while an FP32
// pair operation costs 5-10 FP32 instructions.
//
// Methods: Dekker's and Knuth's error-free transformations (two_sum, quick_two_sum; the
// product's rounding error from one fused multiply-add), as in Shewchuk, "Adaptive
// precision floating-point arithmetic", and Hida, Li and Bailey's double-double library
// (the "sloppy" addition: one error-free sum of the high parts, the low parts added
// plainly).  Conversions between a double and a pair, and from a float to a double, are
// done on the bit patterns with integer instructions (no FP64 conversion instruction).
//
// Everything here is __host__ __device__ so that a CPU test can check it (tests/test_ff.py).
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define NRT_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define NRT_HD inline
#endif

namespace nrt {

struct ff {
  float hi, lo;
};

NRT_HD uint64_t bits_of(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  memcpy(&b, &d, 8);
  return b;
#endif
}
NRT_HD double double_of_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}
NRT_HD uint32_t bits_of(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
#endif
}
NRT_HD float float_of_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}
NRT_HD int clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz(x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

// IEEE operations, kept from being contracted into fused multiply-adds or reordered.
NRT_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  volatile float s = a + b;
  return s;
#endif
}
NRT_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  volatile float s = a - b;
  return s;
#endif
}
NRT_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  volatile float s = a * b;
  return s;
#endif
}
NRT_HD float ffma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

// a + b = s + e exactly (Knuth), any magnitudes.
NRT_HD ff two_sum(float a, float b) {
  const float s = fadd(a, b);
  const float bb = fsub(s, a);
  const float e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
  return ff{s, e};
}
// a + b = s + e exactly when |a| >= |b| or a == 0 (Dekker).
NRT_HD ff quick_two_sum(float a, float b) {
  const float s = fadd(a, b);
  return ff{s, fsub(b, fsub(s, a))};
}

NRT_HD ff ff_from(float a) { return ff{a, 0.0f}; }
NRT_HD ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
NRT_HD ff ff_scale2(ff a) { return ff{a.hi * 2.0f, a.lo * 2.0f}; }  // exact

NRT_HD ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, fadd(s.lo, fadd(a.lo, b.lo)));
}
NRT_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
NRT_HD ff ff_add_f(ff a, float b) {
  const ff s = two_sum(a.hi, b);
  return quick_two_sum(s.hi, fadd(s.lo, a.lo));
}
NRT_HD ff ff_mul_f(ff a, float b) {
  const float p = fmul(a.hi, b);
  float e = ffma(a.hi, b, -p);
  e = ffma(a.lo, b, e);
  return quick_two_sum(p, e);
}
NRT_HD ff ff_mul(ff a, ff b) {
  const float p = fmul(a.hi, b.hi);
  float e = ffma(a.hi, b.hi, -p);
  e = ffma(a.hi, b.lo, e);
  e = ffma(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}

// A double as a pair, by its bit pattern: hi holds the top 24 significant bits (so
// d - hi is exact), lo the next 24 of the remaining 29 (truncated), a relative error below
// 2^-46 for 2^-76 <= |d| < 2^100.  Between 2^-100 and 2^-76 lo would be an FP32 subnormal
// and is dropped (relative error below 2^-23; absolute below 2^-99); smaller values and
// zero give (0, 0).  Huge, infinite and NaN values keep their FP32 rounding in hi (through
// the FP64 conversion instruction), so that a non-finite state stays non-finite.
NRT_HD ff ff_of(double d) {
  const uint64_t b = bits_of(d);
  const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
  const int e = (int)((hw >> 20) & 0x7ffu);
  const uint32_t sign = hw & 0x80000000u;
  if (e < 1023 - 100) return ff{0.0f, 0.0f};
  if (e >= 1023 + 100) return ff{(float)d, 0.0f};
  const uint32_t hi = sign | ((uint32_t)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
  const uint32_t r = lw & 0x1fffffffu;  // the 29 bits below hi, weight 2^(e - 1023 - 52)
  uint32_t lo = 0;
  if (r) {
    const int p = 31 - clz32(r);          // leading bit, 0 .. 28
    const int ex = e - 948 + p;           // biased FP32 exponent of that bit
    if (ex >= 1) {
      const uint32_t m = p >= 23 ? (r >> (p - 23)) : (r << (23 - p));
      lo = sign | ((uint32_t)ex << 23) | (m & 0x7fffffu);
    }
  }
  return ff{float_of_bits(hi), float_of_bits(lo)};
}

// A float as a double, by its bit pattern (exact; FP32 subnormals become 0, Inf and NaN
// go through the conversion instruction).
NRT_HD double double_of(float f) {
  const uint32_t u = bits_of(f);
  const uint32_t ex = (u >> 23) & 0xffu;
  if (ex == 0) return 0.0;
  if (ex == 0xffu) return (double)f;
  return double_of_bits(((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(ex + 896u) << 52) |
                        ((uint64_t)(u & 0x7fffffu) << 29));
}

// v + (hi + lo) in FP64: the one form in which the mixed implicit step moves its FP64
// potentials (two FP64 additions).
NRT_HD double add_ff(double v, ff a) { return v + (double_of(a.hi) + double_of(a.lo)); }

}  // namespace nrt
