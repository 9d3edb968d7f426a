// Host-side check of the bf16-digit tensor-core scheme (qtnh_gb300/csrc/ozaki.cuh) used by
// the fused two-gate kernel: digits are exact bf16 values (the bf16x2 packing loses
// nothing) that reconstruct the 48-bit rounded operand, every level sum stays below 2^24
// (exact in FP32, accumulated here in the MMA's K order), and the recombined result of a
// 16x16 unitary applied to a group of 16 amplitudes is within ~1e-14 relative L2 of long
// double, also along a chain of 300 blocks. Prints "ok" on success.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <random>

#include "ozaki.cuh"

using namespace qtnh_impl;
typedef long double ld;
typedef std::complex<double> cd;

static int fails = 0;

static float bf16_lo(uint32_t p) { return df::u2f(p << 16); }
static float bf16_hi(uint32_t p) { return df::u2f(p & 0xFFFF0000u); }

static void unitary(std::mt19937_64& rng, int d, cd* u) {  // Gram-Schmidt on complex Gaussian rows
  std::normal_distribution<double> nd(0, 1);
  for (int i = 0; i < d * d; ++i) u[i] = {nd(rng), nd(rng)};
  for (int a = 0; a < d; ++a) {
    for (int b = 0; b < a; ++b) {
      cd dot = 0;
      for (int k = 0; k < d; ++k) dot += std::conj(u[b * d + k]) * u[a * d + k];
      for (int k = 0; k < d; ++k) u[a * d + k] -= dot * u[b * d + k];
    }
    double n = 0;
    for (int k = 0; k < d; ++k) n += std::norm(u[a * d + k]);
    for (int k = 0; k < d; ++k) u[a * d + k] /= std::sqrt(n);
  }
}

static void real_form(const cd* U, double R[32][32]) {
  for (int o = 0; o < 16; ++o)
    for (int i = 0; i < 16; ++i) {
      R[o][i] = U[o * 16 + i].real();
      R[o][16 + i] = -U[o * 16 + i].imag();
      R[16 + o][i] = U[o * 16 + i].imag();
      R[16 + o][16 + i] = U[o * 16 + i].real();
    }
}

// digits of v at group exponent E, checked: packing exact, digits in range,
// reconstruction within half a unit of 2^(E - 1070)
static void checked_digits(double v, uint32_t E, float d[oz::NS]) {
  oz::digits(df::words(v), oz::digit_scale(E), d);
  ld rec = 0;
  for (int j = 0; j < oz::NS; ++j) {
    const uint32_t p = oz::pack(d[j], -d[j]);
    if (bf16_lo(p) != d[j] || bf16_hi(p) != -d[j] || std::fabs(d[j]) > (j ? 128.0f : 256.0f)) {
      std::printf("digit %d of %a not exact in bf16 or out of range: %g\n", j, v, (double)d[j]);
      ++fails;
    }
    rec += std::ldexp((ld)d[j], 40 - 8 * j);
  }
  if (oz::exponent(df::words(v)) == 0) {
    if (rec != 0) std::printf("zero/subnormal %a gives nonzero digits\n", v), ++fails;
    return;
  }
  const ld want = std::ldexp((ld)v, 1070 - (int)E);  // v in units of 2^(E - 1070)
  if (std::fabs(rec - want) > 0.5L + 1e-9L) {
    std::printf("digits of %a do not reconstruct it: %Lg vs %Lg\n", v, rec, want);
    ++fails;
  }
}

static float max_level = 0;

// y = R x for one group through digits, level sums in the MMA's accumulation order
// (per k-tile of 16, per digit pair), recombined with L levels
template <int L>
static void apply(const double R[32][32], const double X[32], double out[32]) {
  uint32_t key = 0, Ex, Er[32] = {0};
  for (int k = 0; k < 32; ++k) key = std::max(key, oz::group_key(df::words(X[k])));
  Ex = oz::key_exponent(key);
  for (int r = 0; r < 32; ++r)
    for (int k = 0; k < 32; ++k) Er[r] = std::max(Er[r], oz::exponent(df::words(R[r][k])));
  static float B[32][oz::NS], A[32][32][oz::NS];
  for (int k = 0; k < 32; ++k) checked_digits(X[k], Ex, B[k]);
  for (int r = 0; r < 32; ++r)
    for (int k = 0; k < 32; ++k) checked_digits(R[r][k], Er[r], A[r][k]);
  for (int r = 0; r < 32; ++r) {
    float C[8] = {0};
    double exact[8] = {0};
    for (int i = 0; i < oz::NS; ++i)
      for (int kt = 0; kt < 2; ++kt)
        for (int j = 0; j < oz::NS && i + j < L; ++j)
          for (int k = 16 * kt; k < 16 * kt + 16; ++k) {
            C[i + j] += A[r][k][i] * B[k][j];
            exact[i + j] += (double)A[r][k][i] * (double)B[k][j];
          }
    for (int l = 0; l < L; ++l) {
      if ((double)C[l] != exact[l] || std::fabs(exact[l]) >= 16777216.0) {
        std::printf("level sum not exact: %g vs %g\n", exact[l], (double)C[l]);
        ++fails;
      }
      max_level = std::max(max_level, std::fabs(C[l]));
    }
    out[r] = oz::combine<L>(C, oz::scale_bits((int32_t)(Ex + Er[r])));
  }
}

template <int L>
static void accuracy(const char* name, double max_worst, double max_rms, double max_chain) {
  std::mt19937_64 rng(7);
  std::normal_distribution<double> nd(0, 1);
  std::uniform_int_distribution<int> sc(-60, 60);
  double worst = 0, sumsq = 0;
  const int trials = 4000;
  for (int t = 0; t < trials; ++t) {
    cd U[256];
    unitary(rng, 16, U);
    double R[32][32], X[32], y[32];
    real_form(U, R);
    const int s = sc(rng);
    for (int k = 0; k < 32; ++k) X[k] = std::ldexp(nd(rng), s);
    if (t % 7 == 0) X[t % 32] = 0.0, X[(t + 16) % 32] = 0.0;  // zeros in a group
    if (t % 11 == 0) X[(t + 3) % 32] *= 1e-9;                 // a small element
    apply<L>(R, X, y);
    ld num = 0, den = 0;
    for (int r = 0; r < 32; ++r) {
      ld ref = 0;
      for (int k = 0; k < 32; ++k) ref += (ld)R[r][k] * (ld)X[k];
      num += (y[r] - ref) * (y[r] - ref);
      den += ref * ref;
    }
    const double rel = (double)std::sqrt(num / den);
    worst = std::max(worst, rel);
    sumsq += rel * rel;
  }
  // chain of 300 fused blocks on one group (a 560-gate circuit is 280 blocks per group)
  double worst_chain = 0;
  for (int trial = 0; trial < 6; ++trial) {
    std::complex<ld> ref[16];
    double X[32];
    for (int i = 0; i < 16; ++i) X[i] = nd(rng), X[16 + i] = nd(rng), ref[i] = {(ld)X[i], (ld)X[16 + i]};
    for (int step = 0; step < 300; ++step) {
      cd U[256];
      unitary(rng, 16, U);
      double R[32][32], y[32];
      real_form(U, R);
      apply<L>(R, X, y);
      std::complex<ld> nref[16];
      for (int o = 0; o < 16; ++o) {
        nref[o] = 0;
        for (int i = 0; i < 16; ++i) nref[o] += std::complex<ld>(U[o * 16 + i].real(), U[o * 16 + i].imag()) * ref[i];
      }
      for (int o = 0; o < 16; ++o) ref[o] = nref[o];
      std::copy(y, y + 32, X);
    }
    ld num = 0, den = 0;
    for (int i = 0; i < 16; ++i) num += std::norm(std::complex<ld>(X[i], X[16 + i]) - ref[i]), den += std::norm(ref[i]);
    worst_chain = std::max(worst_chain, (double)std::sqrt(num / den));
  }
  const double rms = std::sqrt(sumsq / trials);
  std::printf("%s: 16x16 unitary on 16 amplitudes: worst %.3e rms %.3e; chain of 300 blocks: worst %.3e\n", name, worst,
              rms, worst_chain);
  if (worst > max_worst || rms > max_rms || worst_chain > max_chain) {
    std::printf("%s: accuracy outside bounds\n", name);
    ++fails;
  }
}

int main() {
  // edge values: powers of two, all-ones significands (rounding carries into 2^48),
  // negative zero, elements far below the group scale
  const double edge[] = {1.0, -1.0, 0.5, 1.0 - std::ldexp(1.0, -53), -std::ldexp(1.0, 1) + std::ldexp(1.0, -51), -0.0,
                         std::ldexp(1.0, -44), std::ldexp(1.0, -49), 3.0 / 7.0, -std::ldexp(1.0, -40) * 255.5};
  float d[oz::NS];
  for (double v : edge) checked_digits(v, oz::exponent(df::words(1.0)), d);
  checked_digits(1.0 - std::ldexp(1.0, -53), oz::exponent(df::words(0.75)), d);
  checked_digits(0.0, 0, d);                      // all-zero group (E = 0)
  checked_digits(4.9e-324, oz::exponent(df::words(1e-50)), d);  // subnormal in a group of the digit path
  for (int k = 0; k < 200000; ++k) {              // random values and group scales
    std::mt19937_64 r2(k);
    const double v = std::ldexp(std::uniform_real_distribution<double>(-1, 1)(r2), (int)(r2() % 120) - 60);
    const uint32_t e = oz::exponent(df::words(v));
    checked_digits(v, e + (uint32_t)(r2() % 60), d);
    checked_digits(v, e + 40 + (uint32_t)(r2() % 30), d);  // elements near or below 2^-48 of the group
  }
  accuracy<oz::NL>("kernel's levels", 5e-14, 2e-14, 2e-12);
  accuracy<7>("7 levels (information)", 1.0, 1.0, 1.0);
  std::printf("largest level sum %.0f (< 2^24)\n", max_level);
  if (fails) {
    std::printf("FAILED\n");
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
