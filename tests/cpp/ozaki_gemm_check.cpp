// Host-side check of the arithmetic of the FP64-accurate digit GEMM (qtnh_gb300/csrc/
// gemm_oz.cu; shared pieces in ozaki.cuh): the complex GEMM in real form, every real of a
// row of A cut into six balanced 8-bit digits at the row's largest exponent and every real
// of a column of B at the column's; per chunk of 128 reals of K every level sum is formed
// exactly (here in 64-bit integers, checked to stay within 2^24 so that the tensor core's
// FP32 accumulators hold it exactly), chunks accumulated as the kernel does
// (oz::gemm_accumulate), and the result finished by oz::gemm_finish. Compared with a
// long-double reference: relative L2 and the worst element error relative to the largest
// product magnitude of its row and column, on shapes with K from 1 to 1000 (several chunks
// and a padded tail), rows and columns of very different scale, zero rows and columns,
// and results near the bottom of the double range. Prints "ok" on success.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "ozaki.cuh"

using namespace qtnh_impl;
typedef long double ld;
typedef std::complex<double> cd;

static int fails = 0;

static uint32_t row_exponent(const cd* x, size_t n) {
  uint32_t key = 0;
  for (size_t k = 0; k < n; ++k)
    key = std::max(key, std::max(oz::group_key(df::words(x[k].real())), oz::group_key(df::words(x[k].imag()))));
  return oz::key_exponent(key);
}

// One GEMM C (M x N) = A (M x K) B'' ^T, B'' (N x K), the digit way; returns the worst
// element error relative to the largest |a||b| product sum of its row and column.
static void check(int M, int N, int K, std::mt19937_64& rng, double row_spread, double col_spread, double base,
                  const char* what) {
  std::normal_distribution<double> nd(0, 1);
  std::uniform_real_distribution<double> ud(-1, 1);
  std::vector<cd> A((size_t)M * K), B((size_t)N * K);
  for (int m = 0; m < M; ++m) {
    const double s = base * std::pow(2.0, std::round(ud(rng) * row_spread));
    for (int k = 0; k < K; ++k) A[(size_t)m * K + k] = cd(nd(rng), nd(rng)) * s;
  }
  for (int n = 0; n < N; ++n) {
    const double s = std::pow(2.0, std::round(ud(rng) * col_spread));
    for (int k = 0; k < K; ++k) B[(size_t)n * K + k] = cd(nd(rng), nd(rng)) * s;
  }
  if (M > 2) std::fill(A.begin() + K, A.begin() + 2 * K, cd(0, 0));  // a zero row
  if (N > 3) std::fill(B.begin() + 3 * K, B.begin() + 4 * K, cd(0, 0));  // a zero column
  const int Kr = 2 * K, Kpad = (Kr + 15) / 16 * 16;
  // digits: A^ rows (2m: Re, -Im; 2m+1: Im, Re), B^ rows (Re, Im), K-padded with zeros
  std::vector<float> dA((size_t)2 * M * Kpad * oz::NS, 0.0f), dB((size_t)N * Kpad * oz::NS, 0.0f);
  std::vector<uint32_t> ea(M), eb(N);
  for (int m = 0; m < M; ++m) {
    ea[m] = row_exponent(&A[(size_t)m * K], K);
    const uint32_t es = oz::digit_scale(ea[m]);
    for (int k = 0; k < K; ++k) {
      float dr[oz::NS], di[oz::NS];
      oz::digits(df::words(A[(size_t)m * K + k].real()), es, dr);
      oz::digits(df::words(A[(size_t)m * K + k].imag()), es, di);
      for (int j = 0; j < oz::NS; ++j) {
        dA[((size_t)(2 * m) * Kpad + 2 * k) * oz::NS + j] = dr[j];
        dA[((size_t)(2 * m) * Kpad + 2 * k + 1) * oz::NS + j] = -di[j];
        dA[((size_t)(2 * m + 1) * Kpad + 2 * k) * oz::NS + j] = di[j];
        dA[((size_t)(2 * m + 1) * Kpad + 2 * k + 1) * oz::NS + j] = dr[j];
      }
    }
  }
  for (int n = 0; n < N; ++n) {
    eb[n] = row_exponent(&B[(size_t)n * K], K);
    const uint32_t es = oz::digit_scale(eb[n]);
    for (int k = 0; k < K; ++k) {
      float dr[oz::NS], di[oz::NS];
      oz::digits(df::words(B[(size_t)n * K + k].real()), es, dr);
      oz::digits(df::words(B[(size_t)n * K + k].imag()), es, di);
      for (int j = 0; j < oz::NS; ++j) {
        dB[((size_t)n * Kpad + 2 * k) * oz::NS + j] = dr[j];
        dB[((size_t)n * Kpad + 2 * k + 1) * oz::NS + j] = di[j];
      }
    }
  }
  ld num = 0, den = 0;
  double worst = 0;
  for (int r = 0; r < 2 * M; ++r) {
    const int m = r / 2;
    for (int n = 0; n < N; ++n) {
      long long T = 0;
      float F = 0.0f;
      for (int c0 = 0; c0 < Kpad; c0 += 128) {
        long long S[oz::NL] = {0, 0, 0, 0, 0, 0};
        for (int k = c0; k < std::min(Kpad, c0 + 128); ++k)
          for (int i = 0; i < oz::NS; ++i)
            for (int j = 0; i + j < oz::NL; ++j)
              S[i + j] += (long long)dA[((size_t)r * Kpad + k) * oz::NS + i] * (long long)dB[((size_t)n * Kpad + k) * oz::NS + j];
        float lv[oz::NL];
        for (int l = 0; l < oz::NL; ++l) {
          if (std::llabs(S[l]) > (1ll << 24)) {
            std::printf("%s: level %d sum %lld exceeds 2^24\n", what, l, S[l]);
            ++fails;
          }
          lv[l] = (float)S[l];
        }
        oz::gemm_accumulate(lv, T, F);
      }
      const double got = oz::gemm_finish(T, F, oz::gemm_scale(ea[m], eb[n]));
      ld ref = 0, mag = 0;
      for (int k = 0; k < K; ++k) {
        const cd a = A[(size_t)m * K + k], b = B[(size_t)n * K + k];
        const ld re = (ld)a.real() * b.real() - (ld)a.imag() * b.imag();
        const ld im = (ld)a.real() * b.imag() + (ld)a.imag() * b.real();
        ref += (r & 1) ? im : re;
        mag += std::abs((ld)a.real()) * std::abs((ld)b.real()) + std::abs((ld)a.imag()) * std::abs((ld)b.imag()) +
               std::abs((ld)a.real()) * std::abs((ld)b.imag()) + std::abs((ld)a.imag()) * std::abs((ld)b.real());
      }
      num += (got - ref) * (got - ref);
      den += ref * ref;
      if (mag > 0) worst = std::max(worst, (double)(std::abs(got - ref) / mag));
      else if (got != 0) {
        std::printf("%s: zero row/column gives %g\n", what, got);
        ++fails;
      }
    }
  }
  const double rel = den > 0 ? (double)std::sqrt(num / den) : 0.0;
  std::printf("%-34s M=%4d N=%4d K=%4d  rel L2 %.2e  worst/|a||b| %.2e\n", what, M, N, K, rel, worst);
  if (!(rel < 1e-13) || !(worst < 1e-14)) {
    std::printf("%s: error too large\n", what);
    ++fails;
  }
}

int main() {
  std::mt19937_64 rng(20261204);
  check(5, 7, 1, rng, 0, 0, 1.0, "K = 1");
  check(9, 13, 64, rng, 0, 0, 1.0, "one chunk exactly");
  check(17, 11, 300, rng, 0, 0, 1.0, "several chunks, padded tail");
  check(12, 10, 1000, rng, 0, 0, 1.0, "K = 1000");
  check(16, 16, 257, rng, 60, 60, 1.0, "rows/columns spread over 2^+-60");
  check(8, 8, 200, rng, 0, 0, 1e-290, "results near the double range's bottom");
  check(8, 8, 200, rng, 0, 0, 1e150, "large magnitudes");
  if (fails) {
    std::printf("%d failures\n", fails);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
