// Error-free slicing of complex128 operands for bf16 tensor-core products (the Ozaki
// scheme: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59, 2012).
//
// A real x of a group whose largest biased exponent is E is written as
//     x ~= sign(x) * sum_{j<6} X_j * 2^(-8 j) * 2^(E - 1030),   X_j in [0, 255],
// i.e. its 53-bit significand is aligned to the group's scale and cut into six 8-bit
// slices (48 bits; the bits below 2^(E-1070) are dropped). Every slice is an integer of
// at most 8 significant bits, so it is exact in bf16, and a product of two slices is
// exact in FP32. With K = 32 terms, sum_k A_i[k] X_j[k] < 2^21, and one level l = i + j
// gathers at most 6 such sums (< 2^23.6): the tensor core's FP32 accumulator holds every
// level sum exactly. The levels are then combined with compensated additions into a
// float pair carrying ~48 bits, and turned into a double with integer instructions and
// one FP64 add (df32.cuh).
#pragma once

#include "df32.cuh"

namespace qtnh_impl {
namespace oz {

constexpr int NS = 6;  // slices per operand
constexpr int NL = 7;  // levels kept: pairs (i, j) with i + j <= 6 (26 slice products)

// Biased double exponent (0 for zero and subnormals).
DF_HD uint32_t exponent(df::dwords w) { return (w.hi >> 20) & 0x7FFu; }

// The six 8-bit slices of x aligned to group exponent E (E >= exponent(x)), as bf16 bit
// patterns carrying the sign of x. x == 0 (or a subnormal) gives zeros.
DF_HD void slice(df::dwords w, uint32_t E, uint16_t out[NS]) {
  const uint32_t e = exponent(w);
  const uint32_t sgn16 = (w.hi >> 16) & 0x8000u;
  uint32_t s = E - e + 5;  // right shift that aligns the 53-bit significand to 48 bits at E
  uint32_t hi = (w.hi & 0xFFFFFu) | 0x100000u, lo = w.lo;  // 21 + 32 bits
  if (e == 0 || s >= 53) hi = lo = 0, s = 0;
  // 53-bit significand shifted right by s (5 <= s < 53) and rounded to nearest
  // (truncation would bias every product of a dot product the same way): M48 = h16:l32,
  // at most 2^48 (then c0 = 256, still exact in bf16).
  uint32_t l32, h16;
  if (s == 0) {
    l32 = h16 = 0;
  } else if (s < 32) {
    const uint32_t r = (lo >> (s - 1)) & 1u;  // first dropped bit
    l32 = (lo >> s) | (hi << (32 - s));
    h16 = hi >> s;
    const uint32_t l2 = l32 + r;
    h16 += (l2 < l32);
    l32 = l2;
  } else {
    const uint32_t r = (s == 32) ? (lo >> 31) : ((hi >> (s - 33)) & 1u);
    l32 = (hi >> (s - 32)) + r;
    h16 = 0;
  }
  const uint32_t c[NS] = {h16 >> 8, h16 & 0xFFu, l32 >> 24, (l32 >> 16) & 0xFFu, (l32 >> 8) & 0xFFu, l32 & 0xFFu};
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    // integer c (0..255) -> float exactly (magic number) -> bf16 by truncation (exact:
    // at most 8 significant bits), sign of x
    const float f = df::sub(df::u2f(0x4B000000u | c[j]), 8388608.0f);
    out[j] = (uint16_t)((df::f2u(f) >> 16) | sgn16);
  }
}

// Level sums C[l] (exact floats) -> the double 2^(Esum - 2060) * sum_l C[l] 2^(-8 l),
// where Esum is the sum of the two operands' group exponents. Level 6 is kept because
// its cross products of a high and a low slice (e.g. A_1 X_5) are 2^-47 of a typical
// product, not of the largest one; levels >= 7 are below 2^-55.
DF_HD double combine(const float C[NL], int32_t Esum) {
  // small levels first, plain adds (their rounding is below 2^-48 of the result)
  float t = df::fma(C[6], 0.00390625f /* 2^-8 */, C[5]);  // C5 + C6 2^-8, in units of 2^-40
  t = df::fma(t, 0.00390625f, C[4]);                          // C4 + ..., in units of 2^-32
  t = df::fma(t, 0.00390625f, C[3]);                          // C3 + ..., in units of 2^-24
  t = df::mul(t, 5.9604644775390625e-08f /* 2^-24 */);        // in units of 1
  // compensated: C[2] 2^-16 + C[1] 2^-8 + C[0]
  float s, e, s2, e2;
  df::two_sum(df::mul(C[2], 1.52587890625e-05f /* 2^-16 */), t, s, e);
  df::two_sum(df::mul(C[1], 0.00390625f), s, s2, e2);
  e = df::add(e, e2);
  df::two_sum(C[0], s2, s, e2);
  e = df::add(e, e2);
  // s + e, scaled by 2^(Esum - 2060) through the exponent field, one FP64 add
  const double hs = df::exact_double(s), he = df::exact_double(e);
  const int64_t shift = (int64_t)(Esum - 2060) << 52;
  const uint64_t us = df::d2u(hs), ue = df::d2u(he);
  const double ds = (us << 1) ? df::u2d(us + (uint64_t)shift) : hs;
  const double de = (ue << 1) ? df::u2d(ue + (uint64_t)shift) : he;
  return ds + de;
}

}  // namespace oz
}  // namespace qtnh_impl
