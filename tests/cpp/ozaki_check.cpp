// Host-side check of the bf16-slice tensor-core scheme (qtnh_gb300/csrc/ozaki.cuh) used by
// the fused two-gate kernel: slices are exact bf16 values, every level sum stays below
// 2^24 (exact in FP32), and the recombined result of a 16x16 unitary applied to a group
// of 16 amplitudes is within ~1e-14 relative L2 of long double. Prints "ok" on success.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <random>

#include "ozaki.cuh"

using namespace qtnh_impl;
typedef long double ld;
typedef std::complex<double> cd;

static float bf16_to_float(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

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

int main() {
  std::mt19937_64 rng(7);
  std::normal_distribution<double> nd(0, 1);
  std::uniform_int_distribution<int> sc(-60, 60);
  int fails = 0;
  double worst = 0, sumsq = 0;
  int trials = 20000;
  float max_level = 0;
  for (int t = 0; t < trials; ++t) {
    cd U[256];
    unitary(rng, 16, U);
    // real matrix R (32x32): [[Re U, -Im U], [Im U, Re U]]
    double R[32][32];
    for (int o = 0; o < 16; ++o)
      for (int i = 0; i < 16; ++i) {
        R[o][i] = U[o * 16 + i].real();
        R[o][16 + i] = -U[o * 16 + i].imag();
        R[16 + o][i] = U[o * 16 + i].imag();
        R[16 + o][16 + i] = U[o * 16 + i].real();
      }
    uint32_t Er[32] = {0};  // per-row exponents of the gate matrix
    for (int r = 0; r < 32; ++r)
      for (double v : R[r]) Er[r] = std::max(Er[r], oz::exponent(df::words(v)));
    cd x[16];
    int s = sc(rng);
    for (auto& v : x) v = {std::ldexp(nd(rng), s), std::ldexp(nd(rng), s)};
    if (t % 7 == 0) x[t % 16] = 0.0;                        // zeros in a group
    if (t % 11 == 0) x[(t + 3) % 16] *= 1e-9;               // a small element
    double X[32];
    for (int i = 0; i < 16; ++i) X[i] = x[i].real(), X[16 + i] = x[i].imag();
    uint32_t Ex = 0;
    for (double v : X) Ex = std::max(Ex, oz::exponent(df::words(v)));
    uint16_t A[32][32][oz::NS], B[32][oz::NS];
    for (int r = 0; r < 32; ++r)
      for (int k = 0; k < 32; ++k) oz::slice(df::words(R[r][k]), Er[r], A[r][k]);
    for (int k = 0; k < 32; ++k) oz::slice(df::words(X[k]), Ex, B[k]);
    ld num = 0, den = 0;
    for (int r = 0; r < 32; ++r) {
      float C[oz::NL];
      for (int l = 0; l < oz::NL; ++l) {
        double acc = 0;  // exact: all partial sums are integers below 2^24
        float accf = 0;
        for (int i = 0; i <= l; ++i)
          for (int k = 0; k < 32 && (l - i) < oz::NS && i < oz::NS; ++k) {
            double p = (double)bf16_to_float(A[r][k][i]) * (double)bf16_to_float(B[k][l - i]);
            acc += p;
            accf += (float)p;
          }
        if (acc != (double)accf || std::fabs(acc) >= 16777216.0) {
          std::printf("level sum not exact: %g vs %g\n", acc, (double)accf);
          ++fails;
        }
        C[l] = accf;
        max_level = std::max(max_level, std::fabs(accf));
      }
      double y = oz::combine(C, (int32_t)(Ex + Er[r]));
      ld ref = 0;
      for (int k = 0; k < 32; ++k) ref += (ld)R[r][k] * (ld)X[k];
      num += (y - ref) * (y - ref);
      den += ref * ref;
    }
    double rel = (double)std::sqrt(num / den);
    worst = std::max(worst, rel);
    sumsq += rel * rel;
  }
  // chain of 300 fused blocks on one group (a 560-gate circuit is 280 blocks per group)
  double worst_chain = 0;
  for (int trial = 0; trial < 10; ++trial) {
    std::complex<ld> ref[16];
    cd cur[16];
    for (int i = 0; i < 16; ++i) cur[i] = {nd(rng), nd(rng)}, ref[i] = {(ld)cur[i].real(), (ld)cur[i].imag()};
    for (int step = 0; step < 300; ++step) {
      cd U[256];
      unitary(rng, 16, U);
      double R[32][32], X[32];
      for (int o = 0; o < 16; ++o)
        for (int i = 0; i < 16; ++i) {
          R[o][i] = U[o * 16 + i].real(), R[o][16 + i] = -U[o * 16 + i].imag();
          R[16 + o][i] = U[o * 16 + i].imag(), R[16 + o][16 + i] = U[o * 16 + i].real();
        }
      for (int i = 0; i < 16; ++i) X[i] = cur[i].real(), X[16 + i] = cur[i].imag();
      uint32_t Ex = 0, Er[32] = {0};
      for (double v : X) Ex = std::max(Ex, oz::exponent(df::words(v)));
      for (int r = 0; r < 32; ++r)
        for (double v : R[r]) Er[r] = std::max(Er[r], oz::exponent(df::words(v)));
      uint16_t B[32][oz::NS], A[oz::NS];
      for (int k = 0; k < 32; ++k) oz::slice(df::words(X[k]), Ex, B[k]);
      double out[32];
      for (int r = 0; r < 32; ++r) {
        float C[oz::NL] = {0};
        for (int k = 0; k < 32; ++k) {
          oz::slice(df::words(R[r][k]), Er[r], A);
          for (int i = 0; i < oz::NS; ++i)
            for (int j = 0; j < oz::NS && i + j < oz::NL; ++j)
              C[i + j] += bf16_to_float(A[i]) * bf16_to_float(B[k][j]);
        }
        out[r] = oz::combine(C, (int32_t)(Ex + Er[r]));
      }
      std::complex<ld> nref[16];
      for (int o = 0; o < 16; ++o) {
        nref[o] = 0;
        for (int i = 0; i < 16; ++i) nref[o] += std::complex<ld>(U[o * 16 + i].real(), U[o * 16 + i].imag()) * ref[i];
      }
      for (int o = 0; o < 16; ++o) ref[o] = nref[o], cur[o] = {out[o], out[16 + o]};
    }
    ld num = 0, den = 0;
    for (int i = 0; i < 16; ++i) num += std::norm(std::complex<ld>(cur[i].real(), cur[i].imag()) - ref[i]), den += std::norm(ref[i]);
    worst_chain = std::max(worst_chain, (double)std::sqrt(num / den));
  }
  std::printf("chain of 300 fused blocks: worst %.3e\n", worst_chain);
  if (worst_chain > 2e-12) ++fails;
  double rms = std::sqrt(sumsq / trials);
  std::printf("16x16 unitary on 16 amplitudes: worst %.3e rms %.3e, largest level sum %.0f (< 2^24)\n", worst, rms, max_level);
  if (worst > 1e-13 || rms > 2e-14) ++fails;
  if (fails) {
    std::printf("FAILED\n");
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
