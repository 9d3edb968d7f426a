// Error-free slicing of complex128 operands for bf16 tensor-core products (the Ozaki
// scheme: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59, 2012).
//
// A real x of a group whose largest biased exponent is E is written with six balanced
// base-256 digits:
//     x ~= sum_{j<6} d_j * 2^(-8 j) * 2^(E - 1030),   |d_j| <= 128 (|d_0| <= 256),
// i.e. its 53-bit significand is aligned to the group's scale, rounded to 48 bits, and
// cut into digits. Every digit is an integer of at most 8 significant bits, so it is
// exact in bf16, and a product of two digits is exact in FP32. With K = 32 terms a level
// l = i + j (at most 6 digit pairs) sums to at most 2^22 in magnitude: the tensor core's
// FP32 accumulator holds every level sum exactly. The levels are then combined with
// compensated additions into a float pair carrying ~48 bits, and turned into a double
// with integer instructions and one FP64 add.
//
// The digit extraction runs on the FP32 pipe: the aligned significand is split into
// three 16-bit pieces (exact floats through the 2^23 magic number), and each piece into
// two balanced digits by rounding to a multiple of 256 (magic number 1.5 * 2^23), the
// carries rippling from the low piece upwards.
#pragma once

#include "df32.cuh"

namespace qtnh_impl {
namespace oz {

constexpr int NS = 6;  // digits per operand
constexpr int NL = 6;  // levels kept: pairs (i, j) with i + j <= 5 (21 digit products)

constexpr float RM = 12582912.0f;  // 1.5 * 2^23: x + RM - RM rounds |x| < 2^22 to an integer

// Biased double exponent (0 for zero and subnormals).
DF_HD uint32_t exponent(df::dwords w) { return (w.hi >> 20) & 0x7FFu; }

DF_HD uint32_t byte_perm(uint32_t a, uint32_t b, uint32_t sel) {
#ifdef __CUDA_ARCH__
  return __byte_perm(a, b, sel);
#else
  const uint64_t v = ((uint64_t)b << 32) | a;
  uint32_t r = 0;
  for (int i = 0; i < 4; ++i) r |= (uint32_t)((v >> (8 * ((sel >> (4 * i)) & 7u))) & 0xFFu) << (8 * i);
  return r;
#endif
}

// round(v / 256) for |v| < 2^30, exactly (one rounding of an exact quotient).
DF_HD float rdiv256(float v) { return df::sub(df::fma(v, 0.00390625f, RM), RM); }

// The six balanced digits of x at group exponent E (E >= exponent(x)), as floats
// (exact integers). x == 0 or a subnormal x gives zeros.
DF_HD void digits(df::dwords w, uint32_t E, float d[NS]) {
  const uint32_t e = exponent(w);
  const uint32_t s = E + 5u - e;  // right shift aligning the 53-bit significand to 48 bits at E
  const uint64_t mant = ((uint64_t)((w.hi & 0xFFFFFu) | 0x100000u) << 32) | w.lo;
  // rounded to nearest (a truncation would bias every product of a dot product the same
  // way); at most 2^48
  const uint64_t m48 = (e != 0u && s <= 53u) ? ((mant + (1ull << (s - 1u))) >> s) : 0ull;
  const uint32_t h = (uint32_t)(m48 >> 32), l = (uint32_t)m48;
  // signed pieces: (2^23 + P) * sg - 2^23 * sg is exactly sg * P
  const float sg = df::u2f((w.hi & 0x80000000u) | 0x3F800000u);
  const float msg = -8388608.0f * sg;
  float p0 = df::fma(df::u2f(0x4B000000u | h), sg, msg);
  float p1 = df::fma(df::u2f(byte_perm(l, 0x4B000000u, 0x7632u)), sg, msg);
  const float p2 = df::fma(df::u2f(byte_perm(l, 0x4B000000u, 0x7610u)), sg, msg);
  const float q2 = rdiv256(p2);
  d[5] = df::fma(q2, -256.0f, p2);
  const float c2 = rdiv256(q2);
  d[4] = df::fma(c2, -256.0f, q2);
  p1 = df::add(p1, c2);
  const float q1 = rdiv256(p1);
  d[3] = df::fma(q1, -256.0f, p1);
  const float c1 = rdiv256(q1);
  d[2] = df::fma(c1, -256.0f, q1);
  p0 = df::add(p0, c1);
  const float q0 = rdiv256(p0);
  d[1] = df::fma(q0, -256.0f, p0);
  d[0] = q0;
}

// Two digits as one bf16x2 register (lo in the low half). Exact: a digit has at most 8
// significant bits, so its float's low 16 bits are zero.
DF_HD uint32_t pack(float lo, float hi) { return byte_perm(df::f2u(lo), df::f2u(hi), 0x7632u); }

// f * 2^(Esum - 2060) as a double through the bit pattern: K20 = (Esum - 1164) << 20 is
// added to the exponent field (f is zero or a normal float; the group ranges keep the
// result a normal double).
DF_HD double scaled_double(float f, uint32_t K20) {
  const uint32_t u = df::f2u(f);
  const uint32_t a = u << 1;
  const uint32_t hi = a ? (((a >> 4) + K20) | (u & 0x80000000u)) : 0u;
  return df::u2d(((uint64_t)hi << 32) | (u << 29));
}

DF_HD uint32_t scale_bits(int32_t Esum) { return (uint32_t)(Esum - 1164) << 20; }

// Level sums C[l] (exact floats) -> the double 2^(Esum - 2060) * sum_{l<L} C[l] 2^(-8 l),
// K20 = scale_bits(Esum). With balanced digits (|d| <= 128) the dropped levels >= 6 add
// a relative error of ~1e-14 per 16x16 block (measured: rms 1e-14, worst 2e-14; keeping
// level 6 halves it).
template <int L = NL>
DF_HD double combine(const float* C, uint32_t K20) {
  // small levels first, plain roundings (below 2^-48 of the result)
  float t = C[L - 1];
  for (int l = L - 2; l >= 3; --l) t = df::fma(t, 0.00390625f /* 2^-8 */, C[l]);
  t = df::mul(t, 5.9604644775390625e-08f /* 2^-24 */);  // in units of 1
  // compensated: C[2] 2^-16 + C[1] 2^-8 + C[0]
  float s, e, s2, e2;
  df::two_sum(df::mul(C[2], 1.52587890625e-05f /* 2^-16 */), t, s, e);
  df::two_sum(df::mul(C[1], 0.00390625f), s, s2, e2);
  e = df::add(e, e2);
  df::two_sum(C[0], s2, s, e2);
  e = df::add(e, e2);
  return scaled_double(s, K20) + scaled_double(e, K20);
}

}  // namespace oz
}  // namespace qtnh_impl
