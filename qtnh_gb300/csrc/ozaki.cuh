// Error-free slicing of complex128 operands for bf16 tensor-core products (the Ozaki
// scheme: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59, 2012).
//
// A real x of a group whose largest biased exponent is E is written with six balanced
// base-256 digits:
//     x ~= sum_{j<6} d_j * 2^(-8 j) * 2^(E - 1030),   |d_j| <= 128 (|d_0| <= 256),
// i.e. its 53-bit significand is aligned to the group's scale and rounded to 48 bits
// (M48 = round(|x| 2^(1070 - E)) <= 2^48), and cut into digits. Every digit is an integer
// of at most 8 significant bits, so it is exact in bf16, and a product of two digits is
// exact in FP32. With K = 32 terms a level l = i + j (at most 6 digit pairs) sums to at
// most 2 * 32 * 256 * 128 + 4 * 32 * 128 * 128 = 2^22 in magnitude: the tensor core's
// FP32 accumulator holds every level sum exactly. The levels are then combined with compensated additions into a
// float pair carrying ~48 bits, and turned into a double with integer instructions and
// one FP64 add.
//
// Digit extraction: M48 + B, B = 0x808080808080, has bytes b_j (b_0 = bits 40..49, up
// to 384) with M48 = sum (b_j - 128) 256^(5-j) (the carries of the addition do the
// balancing); b_j - 128 comes out of one byte permute (the byte under the 2^23 magic
// exponent) and one FMA that also applies the sign. The rounding rides on the same
// addition: (floor(m / 2^(s-1)) + 2B + 1) >> 1 = round(m / 2^s) + B.
#pragma once

#include <math.h>

#include "df32.cuh"

namespace qtnh_impl {
namespace oz {

constexpr int NS = 6;  // digits per operand
constexpr int NL = 6;  // levels kept: pairs (i, j) with i + j <= 5 (21 digit products)

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

// Largest biased exponent of a set of doubles, from max(hi << 1) (the sign shifted out,
// the exponent on top): group_key() per element, then key_exponent() of the maximum.
DF_HD uint32_t group_key(df::dwords w) { return w.hi << 1; }
DF_HD uint32_t key_exponent(uint32_t key) { return key >> 21; }

// Group scale for digits(): E, or (for an all-zero group, E == 0) a scale at which every
// element's digits are 0.
DF_HD uint32_t digit_scale(uint32_t E) { return E ? E : 0x7FFu; }

// The six balanced digits of x at group scale Es = digit_scale(E) (E >= exponent(x),
// Es >= 58), as floats (exact integers, |d_0| <= 256, |d_j| <= 128). Zeros and
// subnormals give zeros (their alignment shift is clamped to 63 bits).
DF_HD void digits(df::dwords w, uint32_t Es, float d[NS]) {
  const uint32_t e = exponent(w);
  // right shift aligning the 53-bit significand to 48 bits at Es, clamped: zeros and
  // subnormals (e = 0) and elements below 2^-49 of the group fall to 0
  uint32_t s = Es + 5u - e;
  s = s < 63u ? s : 63u;
  const uint64_t mant = ((uint64_t)((w.hi & 0xFFFFFu) | 0x100000u) << 32) | w.lo;
  const uint64_t mb = ((mant >> (s - 1u)) + 0x1010101010101ull) >> 1;  // M48 + B
  const uint32_t h = (uint32_t)(mb >> 32), l = (uint32_t)mb;
  // (2^23 + b) * sg - (2^23 + 128) * sg = sg * (b - 128)
  const float sg = df::u2f((w.hi & 0x80000000u) | 0x3F800000u);
  const float off = -8388736.0f * sg;
  d[0] = df::fma(df::u2f(byte_perm(h, 0x4B000000u, 0x7621u)), sg, off);  // bits 40..49
  d[1] = df::fma(df::u2f(byte_perm(h, 0x4B000000u, 0x7650u)), sg, off);
  d[2] = df::fma(df::u2f(byte_perm(l, 0x4B000000u, 0x7653u)), sg, off);
  d[3] = df::fma(df::u2f(byte_perm(l, 0x4B000000u, 0x7652u)), sg, off);
  d[4] = df::fma(df::u2f(byte_perm(l, 0x4B000000u, 0x7651u)), sg, off);
  d[5] = df::fma(df::u2f(byte_perm(l, 0x4B000000u, 0x7650u)), sg, off);
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

// ---- fixed point between the passes of a gate layer (gate_umma.cu) ----
//
// Inside one gate layer the state passes from one fused pass to the next as signed 64-bit
// fixed point at a common scale, y = Y 2^-F (each pass records F and max |Y|). Those
// passes cut the state at ONE scale for all of it, 2^(E - 1030) with E the input's
// equivalent exponent, into six balanced digits (48 bits of the largest magnitude):
// m48 = sum_j d_j 2^(40 - 8j), |m48| <= 2^47:
//   * fixed point: m48 = round(Y 2^-sh), sh = bits(max |Y|) - 47 (a left shift when not
//     positive: every pass cuts the largest magnitude just below 2^47, so the scale cannot
//     drift down from pass to pass), E = 1070 + sh - F;
//   * doubles (the pass after the first, whose largest exponent was recorded): oz::digits
//     at E.
// The gate keeps six digits per row; state digit j meets gate digits 0 .. NL - 1 - j, NL = 6
// or 7 levels kept (for 7, a zero seventh gate digit block lets the first MMA write level
// 6 too): the level sums C_0 .. C_(NL-1) are exact in FP32 (|C_l| <= 2^22). T = sum_{l<6}
// C_l 2^(40 - 8l) (+ round(C_6 2^-8) for NL = 7) is an exact 64-bit integer up to that
// rounding (|T| < 2^63), the value is T 2^(erow + E - 2100), and the output at scale
// F_out = 2100 - E - max_o erow[o] is Y_o = round(T 2^(erow[o] - max erow)): a right shift,
// |Y_o| <= |T|.

// The six balanced digits of the fixed-point value x at shift sh (-32 < sh < 64; a left
// shift when sh <= 0), |round(x 2^-sh)| <= 2^47.
DF_HD int64_t fixed_round(int64_t x, int32_t sh) {
  return sh >= 1 ? (((x >> (sh - 1)) + 1) >> 1) : (int64_t)((uint64_t)x << (uint32_t)(-sh));
}

DF_HD void digits_fixed(int64_t x, int32_t sh, float d[NS]) {
  const int64_t m = fixed_round(x, sh);
  const uint64_t mb = (uint64_t)m + 0x808080808080ull;  // round(x 2^-sh) + B: bytes - 128 are the digits
  const uint32_t h = (uint32_t)(mb >> 32), l = (uint32_t)mb;
  const float off = -8388736.0f;  // -(2^23 + 128)
  d[0] = df::add(df::u2f(byte_perm(h, 0x4B000000u, 0x7621u)), off);  // bits 40..55 (at most 256)
  d[1] = df::add(df::u2f(byte_perm(h, 0x4B000000u, 0x7650u)), off);
  d[2] = df::add(df::u2f(byte_perm(l, 0x4B000000u, 0x7653u)), off);
  d[3] = df::add(df::u2f(byte_perm(l, 0x4B000000u, 0x7652u)), off);
  d[4] = df::add(df::u2f(byte_perm(l, 0x4B000000u, 0x7651u)), off);
  d[5] = df::add(df::u2f(byte_perm(l, 0x4B000000u, 0x7650u)), off);
}

// round(x 2^-sh) + 0x808080808080 (the biased value whose bytes minus 128 are the six
// balanced digits) with the rounding half and the bias folded into one 64-bit addend
// c = fixed_addend(sh): ((x + c) >> sh) for 1 <= sh <= 15 (x + c then lies in (0, 2^64)
// while |round(x 2^-sh)| <= 2^47), (x << -sh) + c for sh <= 0.
DF_HD uint64_t fixed_addend(int32_t sh) {
  const uint64_t B = 0x808080808080ull;
  return sh >= 1 ? ((uint64_t)1 << (sh - 1)) + (B << sh) : B;
}
DF_HD uint64_t fixed_biased(int64_t x, int32_t sh, uint64_t c) {
  return sh >= 1 ? ((uint64_t)x + c) >> sh : ((uint64_t)x << (uint32_t)(-sh)) + c;
}

// The six digits of two K-adjacent values as fp16x2 words still carrying the fp16 offset,
// from their biased values m0, m1 (fixed_biased): half j of word w[j] is 0x6400 | b_j, the
// fp16 of 1024 + b_j, where b_j is digit j's byte of m (b_0: bits 40..48, at most 256) --
// the first value in the low half, the second in the high half. Subtracting 1152 (0x6480)
// from both halves (one packed fp16 subtraction, exact) gives the balanced digits
// b_j - 128 of digits_fixed. Byte permutes only: one to pair the two values' bytes, one per
// word to put them under the exponent byte 0x64.
DF_HD void digit_words_biased(uint64_t m0, uint64_t m1, uint32_t w[NS]) {
  const uint32_t l0 = (uint32_t)m0, l1 = (uint32_t)m1, h0 = (uint32_t)(m0 >> 32), h1 = (uint32_t)(m1 >> 32);
  const uint32_t E = 0x64646464u;
  const uint32_t pa = byte_perm(l0, l1, 0x5140u);  // bytes 0 and 1 of both: digits 5 and 4
  const uint32_t pb = byte_perm(l0, l1, 0x7362u);  // bytes 2 and 3: digits 3 and 2
  const uint32_t pc = byte_perm(h0, h1, 0x5140u);  // bytes 4 and 5: digits 1 and 0 (its low 8 bits)
  w[5] = byte_perm(pa, E, 0x4140u);
  w[4] = byte_perm(pa, E, 0x4342u);
  w[3] = byte_perm(pb, E, 0x4140u);
  w[2] = byte_perm(pb, E, 0x4342u);
  w[1] = byte_perm(pc, E, 0x4140u);
  w[0] = byte_perm(pc, E, 0x4342u) | ((h0 >> 8) & 0x100u) | ((h1 << 8) & 0x1000000u);  // + bit 48 of each
}

// The same from two fixed-point values x0, x1 at shift sh (1 <= sh <= 15 or sh <= 0).
DF_HD void digit_words_fixed(int64_t x0, int64_t x1, int32_t sh, uint32_t w[NS]) {
  const uint64_t c = fixed_addend(sh);
  digit_words_biased(fixed_biased(x0, sh, c), fixed_biased(x1, sh, c), w);
}

// The shift that puts the largest |Y| of a fixed-point input just below 2^47 (right when
// positive, left when not), from maxhi, a value with the bit length of the largest |hi
// word| (fixed_hi_mag): the magnitude bound is taken as 2^(32 + bit length of maxhi).
DF_HD int32_t fixed_shift(uint32_t maxhi) {
  int32_t len = 0;
  while (len < 32 && (maxhi >> len)) ++len;
  return 32 + len - 47;
}

// The input's equivalent exponent E for shift sh and scale F.
DF_HD int fixed_exponent(int32_t sh, int32_t F) { return 1070 + sh - F; }

// |hi word| of a 64-bit value (one's complement for negatives: an upper bound of |x| >> 32).
DF_HD uint32_t fixed_hi_mag(int64_t x) {
  const int32_t hi = (int32_t)(x >> 32);
  return (uint32_t)(hi ^ (hi >> 31));
}

// A level sum (an exact integer of at most 2^22 in magnitude, held in a float) as an
// integer, read through the 1.5 2^23 bias: the float's bits minus 0x4B400000.
DF_HD int32_t level_int(float c) { return (int32_t)(df::f2u(df::add(c, 12582912.0f)) - 0x4B400000u); }

// The biased bits of a level sum c (|c| < 2^22): c + 1.5 2^23 is exact and its bits are
// 0x4B400000 + c.
DF_HD uint32_t level_bits(float c) { return df::f2u(df::add(c, 12582912.0f)); }

// T = sum_{l<6} C_l 2^(40 - 8l) (+ round(C_6 2^-8) for NL = 7 levels), exact up to that
// rounding, from the biased bits B_l = 0x4B400000 + C_l of the level sums (|C_l| < 2^22).
// A pair of levels is one multiply-add of the biased bits: B_{2i} 256 + B_{2i+1} =
// 256 C_{2i} + C_{2i+1} + 0x8B400000 (mod 2^32), which lies in (0, 2^32) for |C| < 2^22,
// so the three pairs enter the 64-bit sum as unsigned words and one constant,
// 0x8B400000 (2^32 + 2^16 + 1), removes their biases.
template <int NL>
DF_HD int64_t fixed_levels_bits(const uint32_t B[NL]) {
  static_assert(NL == 6 || NL == 7, "six or seven levels");
  const uint32_t X = B[0] * 256u + B[1];
  const uint32_t Y = B[2] * 256u + B[3];
  const uint32_t Z = B[4] * 256u + B[5];
  const uint64_t W = NL == 7 ? (uint64_t)(int64_t)((int32_t)(B[NL - 1] - 0x4B3FFF80u) >> 8) : 0;  // round(C_6 / 256)
  const uint64_t KB = 0x8B400000ull * 0x100010001ull;  // mod 2^64
  return (int64_t)(((uint64_t)X << 32) + ((uint64_t)Y << 16) + (uint64_t)Z + W - KB);
}

template <int NL>
DF_HD int64_t fixed_levels(const float C[NL]) {
  uint32_t B[NL];
  for (int l = 0; l < NL; ++l) B[l] = level_bits(C[l]);
  return fixed_levels_bits<NL>(B);
}

// A chain pass cuts the gate's digits at one scale for all rows (that of its largest row)
// when the rows' largest exponents differ by at most CHAIN_COMMON_SPAN: the outputs then
// come out at the common scale without a per-row shift, and a row keeps at least
// 48 - CHAIN_COMMON_SPAN bits of its own largest entry. Otherwise each row has its own
// scale and its outputs are shifted (rounded) to the common one.
constexpr int CHAIN_COMMON_SPAN = 2;

// Seven level sums with level 6 folded into level 5 in FP32 before the conversion:
// fma(C_6, 2^-8, C_5) rounded to an integer by the bias addition (|C_5 + C_6 2^-8| < 2^22):
// T = sum_{l<6} C_l 2^(40 - 8l) + C_6 2^-8 to within one unit of level 5 (2^-40 of level
// 0; the unmerged form rounds only C_6 2^-8), with six level conversions instead of seven.
DF_HD int64_t fixed_levels_merged(const float C[7]) {
  uint32_t B[6];
  for (int l = 0; l < 5; ++l) B[l] = level_bits(C[l]);
  B[5] = level_bits(df::fma(C[6], 0.00390625f, C[5]));
  return fixed_levels_bits<6>(B);
}

// round(T 2^-k) for 0 <= k <= 62 (ties up).
DF_HD int64_t fixed_round_shift(int64_t T, uint32_t k) {
  return k ? ((T + ((int64_t)1 << (k - 1))) >> k) : T;
}

// T 2^(e - 40) as a double (e = erow + E - 2060): one rounding, then an exact scaling
// while the result stays a normal double (else scalbn).
DF_HD double fixed_to_double(int64_t T, int e) {
  const double v = (double)T;
  if (v == 0.0) return 0.0;
  const uint64_t b = df::d2u(v);
  const int s = e - 40;
  const int en = (int)((b >> 52) & 0x7FFull) + s;
  if (en >= 1 && en <= 2046) return df::u2d(b + ((uint64_t)(int64_t)s << 52));
  return scalbn(v, s);
}

// ---- the dense GEMM form (gemm_oz.cu): digits per row of A and per column of B ----
//
// C^[r][n] = 2^(ea + eb - 2060) sum_l 2^(-8l) S_l with S_l the level sums of the digit
// products. A chunk's level sums are exact integers of at most 2^24 in magnitude; they are
// accumulated as T += S_0 2^24 + S_1 2^16 + S_2 2^8 + S_3 (exact 64-bit integer) and
// F += S_4 + 2^-8 S_5 (FP32, below 2^-32 of T's units), and C^ = 2^(ea + eb - 2084) (T +
// 2^-8 F).

// Adds one chunk's six level sums (exact integers held in floats) to (T, F).
DF_HD void gemm_accumulate(const float lv[NL], long long& T, float& F) {
  const long long s0 = (long long)(int)lv[0], s1 = (long long)(int)lv[1];
  const long long s2 = (long long)(int)lv[2], s3 = (long long)(int)lv[3];
  T += (s0 << 24) + (s1 << 16) + (s2 << 8) + s3;
  F = df::add(F, df::fma(lv[5], 0.00390625f, lv[4]));
}

// Exponent e of C^'s scale 2^e for row exponent ea and column exponent eb.
DF_HD int gemm_scale(uint32_t ea, uint32_t eb) { return (int)digit_scale(ea) + (int)digit_scale(eb) - 2084; }

// 2^e (T + 2^-8 F) as a double: one rounding of T + 2^-8 F, then an exact scaling while
// the result stays a normal double (else scalbn: overflow to infinity, gradual underflow).
DF_HD double gemm_finish(long long T, float F, int e) {
  const double v = fma((double)F, 0.00390625, (double)T);
  if (v == 0.0) return 0.0;
  const uint64_t b = df::d2u(v);
  const int en = (int)((b >> 52) & 0x7FFull) + e;
  if (en >= 1 && en <= 2046) return df::u2d(b + ((uint64_t)(int64_t)e << 52));
  return scalbn(v, e);
}

}  // namespace oz
}  // namespace qtnh_impl
