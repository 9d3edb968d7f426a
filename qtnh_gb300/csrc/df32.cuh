// Compensated FP32 arithmetic for complex128 data ("float-float", error-free
// transformations).
//
// GB300 executes FP64 at 1.2 TFLOP/s but FP32 at 70 TFLOP/s (measured), so a complex128
// gate (16 FP64 FMAs per amplitude) is FP64-bound at 18 % of the HBM roofline. The
// kernels that use this header keep complex128 in HBM, but compute on the FP32 pipe:
//
//   * a double x is split, with integer instructions only, into floats hi + lo where
//     hi is x truncated to 24 significant bits and lo the next 24 bits rounded to
//     nearest, so |x - (hi + lo)| <= 2^-48 |x|;
//   * a product a*b of two split numbers is p + e with p = fl(ah*bh) and
//     e = (ah*bh - p) + ah*bl + al*bh + al*bl, the first term exact by FMA
//     (Dekker's TwoProduct with a fused multiply-add);
//   * sums of the high parts use Knuth's TwoSum (exact: s + err = a + b), the
//     low-order terms are summed in plain FP32;
//   * the result pair is renormalised and turned back into a double with integer
//     instructions plus one FP64 add.
//
// For the magnitudes allowed by in_range() (state elements 0 or 2^-90..2^90, gate
// elements 0 or 2^-30..2^30) every intermediate is a normal float and the relative
// error of a complex multiply-accumulate chain of length 4 is ~2^-46 or better; the
// kernels fall back to native FP64 for a group that has anything outside that range.
// (References: T. J. Dekker, "A floating-point technique for extending the available
// precision", 1971; D. E. Knuth, TAOCP vol. 2, 4.2.2; Ogita, Rump, Oishi, "Accurate
// sum and dot product", 2005.)
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace qtnh_impl {
namespace df {

DF_HD uint64_t d2u(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
DF_HD double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}
DF_HD uint32_t f2u(float x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
DF_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

// Correctly rounded single operations that the compiler may not fuse.
DF_HD float add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  volatile float r = a + b;
  return r;
#endif
}
DF_HD float sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}
DF_HD float mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  volatile float r = a * b;
  return r;
#endif
}
DF_HD float fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}

struct f2 {
  float h, l;  // value h + l
};

// A double as its two 32-bit words (hi: sign, 11-bit exponent, top 20 mantissa bits).
// The fast paths test and split doubles through these words only, so no comparison
// or select on a double value reaches the FP64 pipe.
struct dwords {
  uint32_t hi, lo;
};

DF_HD dwords words(double x) {
  uint64_t u = d2u(x);
  return {(uint32_t)(u >> 32), (uint32_t)u};
}

// In range: zero, or biased exponent in [1023 - 90, 1023 + 90] (|x| in [2^-90, 2^91)).
DF_HD bool in_range_state(dwords w) {
  uint32_t e = (w.hi >> 20) & 0x7FFu;
  return (e - 933u) <= 180u || ((w.hi << 1) | w.lo) == 0u;
}
// Gate elements: zero or |x| in [2^-30, 2^31).
DF_HD bool in_range_gate(dwords w) {
  uint32_t e = (w.hi >> 20) & 0x7FFu;
  return (e - 993u) <= 60u || ((w.hi << 1) | w.lo) == 0u;
}
DF_HD bool in_range_state(double x) { return in_range_state(words(x)); }
DF_HD bool in_range_gate(double x) { return in_range_gate(words(x)); }

DF_HD uint32_t funnel_left3(uint32_t lo, uint32_t hi) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, 3);
#else
  return (hi << 3) | (lo >> 29);
#endif
}

// x -> hi + lo for an in-range x (see in_range_*). hi is x truncated to 24 significant
// bits: the funnel shift lines up the low 8 exponent bits and 23 mantissa bits, and
// for biased exponents e in [897, 1150] the float exponent e - 896 equals those 8 bits
// with the top bit flipped. lo is the remaining 29 mantissa bits r (weight 2^(E-52),
// E = e - 1023) rounded to 24 bits: r = r1 * 2^6 + r0 is turned into two exact floats
// by the magic-number trick, 2^(E-23) + r1 * 2^(E-46) - 2^(E-23) and
// 2^(E-29) + r0 * 2^(E-52) - 2^(E-29), whose sum is rounded once.
DF_HD f2 split(dwords w) {
  if (((w.hi << 1) | w.lo) == 0u) return {0.0f, 0.0f};
  const uint32_t sgn = w.hi & 0x80000000u;
  const uint32_t hi = (((funnel_left3(w.lo, w.hi) & 0x7FFFFFFFu) ^ 0x40000000u)) | sgn;
  const uint32_t e = (w.hi >> 20) & 0x7FFu;
  const uint32_t c1 = (e - 919u) << 23;           // 2^(E-23)
  const uint32_t c0 = c1 - (6u << 23);            // 2^(E-29)
  const float lo_hi = sub(u2f(c1 | ((w.lo >> 6) & 0x7FFFFFu)), u2f(c1));
  const float lo_lo = sub(u2f(c0 | (w.lo & 63u)), u2f(c0));
  const float lo = add(lo_hi, lo_lo);
  return {u2f(hi), u2f(f2u(lo) | sgn)};
}
DF_HD f2 split(double x) { return split(words(x)); }

// TwoSum (Knuth): s + err == a + b exactly.
DF_HD void two_sum(float a, float b, float& s, float& err) {
  s = add(a, b);
  float bb = sub(s, a);
  err = add(sub(a, sub(s, bb)), sub(b, bb));
}

// Product of two split reals: p + e ~ a*b with p = fl(ah*bh).
DF_HD void two_prod(f2 a, f2 b, float& p, float& e) {
  p = mul(a.h, b.h);
  e = fma(a.h, b.h, -p);
  e = fma(a.h, b.l, e);
  e = fma(a.l, b.h, e);
  e = fma(a.l, b.l, e);
}

// Accumulator for a real sum of products: value s + c.
struct acc {
  float s, c;
};

DF_HD acc acc_first(f2 a, f2 b) {
  acc r;
  two_prod(a, b, r.s, r.c);
  return r;
}

DF_HD void acc_mac(acc& r, f2 a, f2 b) {
  float p, e, s, err;
  two_prod(a, b, p, e);
  two_sum(r.s, p, s, err);
  r.s = s;
  r.c = add(r.c, add(err, e));
}

// Exact float -> double through the bit pattern (normal floats); zero and subnormal
// floats (rounding residue far below the result) give +-0.
DF_HD double exact_double(float f) {
  const uint32_t u = f2u(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t sgn = u & 0x80000000u;
  const uint32_t hi = e ? (sgn | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3)) : sgn;
  const uint32_t lo = e ? (u << 29) : 0u;
  return u2d(((uint64_t)hi << 32) | lo);
}

// s + c rounded once to double: both parts convert exactly, and the one FP64 add
// (two per complex element) uses the FP64 pipe that the rest of the path leaves idle.
DF_HD double to_double(acc r) { return exact_double(r.s) + exact_double(r.c); }

DF_HD f2 renorm(acc r) {
  f2 v;
  two_sum(r.s, r.c, v.h, v.l);
  return v;
}

// Complex value as four floats.
struct cf2 {
  f2 re, im;
};

DF_HD cf2 csplit(double re, double im) { return {split(re), split(im)}; }

DF_HD f2 neg(f2 a) { return {-a.h, -a.l}; }

// Complex product of split numbers: (a * b) as two accumulators.
DF_HD void cmul_acc(cf2 a, cf2 b, acc& re, acc& im) {
  re = acc_first(a.re, b.re);
  acc_mac(re, a.im, neg(b.im));
  im = acc_first(a.re, b.im);
  acc_mac(im, a.im, b.re);
}

}  // namespace df
}  // namespace qtnh_impl
