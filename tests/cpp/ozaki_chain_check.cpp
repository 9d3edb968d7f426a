// Host-side check of the fixed-point chain of a gate layer (ozaki.cuh, as gate_umma.cu
// uses it): consecutive fused two-gate passes on one state, the first reading doubles at
// each group's own exponent and writing doubles (recording the largest exponent), the
// second reading doubles at that global exponent and writing 64-bit fixed point, the
// middle ones fixed point to fixed point, the last fixed point to doubles, with seven (the
// default) or six digit-product levels kept. Every level is summed exactly (here in 64-bit
// integers), as the tensor cores' FP32 accumulators do for K = 32. Compared with long
// double after every chain, on random states and unitaries, chains of up to 64 passes
// (the scale must not drift from pass to pass), states with a spread of magnitudes, and
// non-unitary layers. Prints "ok" on success.
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
typedef std::complex<ld> cld;

static int fails = 0;

struct State {
  bool fixed = false;
  std::vector<cd> d;           // double form
  std::vector<int64_t> y;      // fixed form: re, im interleaved
  int F = 0;
  uint32_t maxhi = 0, maxkey = 0;
};

static void unitary(std::mt19937_64& rng, int dim, std::vector<cd>& u, double scale) {
  std::normal_distribution<double> nd(0, 1);
  u.assign(dim * dim, 0);
  for (auto& x : u) x = {nd(rng), nd(rng)};
  for (int a = 0; a < dim; ++a) {
    for (int b = 0; b < a; ++b) {
      cd dot = 0;
      for (int k = 0; k < dim; ++k) dot += std::conj(u[b * dim + k]) * u[a * dim + k];
      for (int k = 0; k < dim; ++k) u[a * dim + k] -= dot * u[b * dim + k];
    }
    double nn = 0;
    for (int k = 0; k < dim; ++k) nn += std::norm(u[a * dim + k]);
    for (int k = 0; k < dim; ++k) u[a * dim + k] *= scale / std::sqrt(nn);
  }
}

// One fused pass of U16 = Ua (x) Ub on targets t[0..3] (t[0], t[1] for gate a), U[o][i].
// in_mode: 0 = doubles at each group's exponent, 1 = doubles at the recorded global exponent,
// 2 = fixed point; out_fixed: write fixed point (else doubles). NL: levels (6 or 7) kept by the chain passes (in_mode 1 and 2).
template <int NL>
static State pass(const State& in, int n, const int t[4], const std::vector<cd>& Ua, const std::vector<cd>& Ub,
                  int in_mode, bool out_fixed) {
  const std::size_t N = (std::size_t)1 << n;
  cd U[16][16];
  for (int o = 0; o < 16; ++o)
    for (int i = 0; i < 16; ++i) U[o][i] = Ua[(o >> 2) * 4 + (i >> 2)] * Ub[(o & 3) * 4 + (i & 3)];
  double R[32][32];
  for (int o = 0; o < 16; ++o)
    for (int i = 0; i < 16; ++i) {
      R[o][i] = U[o][i].real();
      R[o][16 + i] = -U[o][i].imag();
      R[16 + o][i] = U[o][i].imag();
      R[16 + o][16 + i] = U[o][i].real();
    }
  int erow[16], max_erow = 0;
  float rd[32][32][oz::NS];
  for (int o = 0; o < 16; ++o) {
    uint32_t e = 0;
    for (int i = 0; i < 16; ++i)
      e = std::max(e, std::max(oz::exponent(df::words(U[o][i].real())), oz::exponent(df::words(U[o][i].imag()))));
    erow[o] = (int)e;
    max_erow = std::max(max_erow, (int)e);
  }
  int min_erow = max_erow;
  for (int o = 0; o < 16; ++o) min_erow = std::min(min_erow, erow[o]);
  // chain passes: one digit scale for all rows when their exponents are within the span
  const bool common = in_mode != 0 && max_erow - min_erow <= oz::CHAIN_COMMON_SPAN;
  for (int r = 0; r < 32; ++r)
    for (int k = 0; k < 32; ++k)
      oz::digits(df::words(R[r][k]), oz::digit_scale((uint32_t)(common ? max_erow : erow[r & 15])), rd[r][k]);
  int32_t sh = 0;
  int Ein = 0;
  if (in_mode == 2) {
    sh = oz::fixed_shift(in.maxhi);
    Ein = oz::fixed_exponent(sh, in.F);
  } else if (in_mode == 1) {
    Ein = (int)oz::digit_scale(oz::key_exponent(in.maxkey));
  }
  State out;
  out.fixed = out_fixed;
  out.d.assign(N, 0);
  out.y.assign(2 * N, 0);
  out.F = 2100 - Ein - max_erow;
  const int p[4] = {n - 1 - t[0], n - 1 - t[1], n - 1 - t[2], n - 1 - t[3]};  // bit of target j
  for (std::size_t base = 0; base < N; ++base) {
    bool is_base = true;
    for (int j = 0; j < 4; ++j) is_base = is_base && !((base >> p[j]) & 1);
    if (!is_base) continue;
    std::size_t idx[16];
    for (int c = 0; c < 16; ++c) {
      idx[c] = base;
      for (int j = 0; j < 4; ++j)
        if ((c >> (3 - j)) & 1) idx[c] |= (std::size_t)1 << p[j];
    }
    float xd[32][7];
    int Eg = Ein;
    if (in_mode == 0) {
      uint32_t key = 0;
      for (int c = 0; c < 16; ++c)
        key = std::max(key, std::max(oz::group_key(df::words(in.d[idx[c]].real())), oz::group_key(df::words(in.d[idx[c]].imag()))));
      Eg = (int)oz::key_exponent(key);
    }
    for (int c = 0; c < 16; ++c) {
      xd[c][6] = xd[16 + c][6] = 0.0f;
      if (in_mode == 2) {
        oz::digits_fixed(in.y[2 * idx[c]], sh, xd[c]);
        oz::digits_fixed(in.y[2 * idx[c] + 1], sh, xd[16 + c]);
      } else if (in_mode == 1) {
        oz::digits(df::words(in.d[idx[c]].real()), (uint32_t)Eg, xd[c]);
        oz::digits(df::words(in.d[idx[c]].imag()), (uint32_t)Eg, xd[16 + c]);
      } else {
        const uint32_t es = oz::digit_scale((uint32_t)Eg);
        oz::digits(df::words(in.d[idx[c]].real()), es, xd[c]);
        oz::digits(df::words(in.d[idx[c]].imag()), es, xd[16 + c]);
        xd[c][6] = xd[16 + c][6] = 0.0f;
      }
    }
    // levels: 0..5 for the first pass, 0..NL-1 for the chain passes
    const int L = in_mode == 0 ? oz::NL : NL;
    for (int r = 0; r < 32; ++r) {
      long long S[7] = {0, 0, 0, 0, 0, 0, 0};
      for (int k = 0; k < 32; ++k)
        for (int i = 0; i < oz::NS; ++i)
          for (int j = 0; j < oz::NS && i + j < L; ++j) S[i + j] += (long long)rd[r][k][i] * (long long)xd[k][j];
      float C[7];
      for (int l = 0; l < 7; ++l) {
        if (std::llabs(S[l]) > (1ll << 22)) {
          std::printf("level sum %lld exceeds 2^22\n", S[l]);
          ++fails;
        }
        C[l] = (float)S[l];
      }
      const int o = r & 15;
      double v;
      if (in_mode == 0) {
        v = oz::combine(C, oz::scale_bits(erow[o] + Eg));
      } else {
        const int64_t T = NL == 7 ? oz::fixed_levels_merged(C) : oz::fixed_levels<NL>(C);
        if (out_fixed) {
          const int64_t Y = common ? T : oz::fixed_round_shift(T, (uint32_t)(max_erow - erow[o]));
          out.y[2 * idx[o] + (r >= 16)] = Y;
          out.maxhi = std::max(out.maxhi, oz::fixed_hi_mag(Y));
          continue;
        }
        v = oz::fixed_to_double(T, (common ? max_erow : erow[o]) + Ein - 2060);
      }
      if (r < 16) out.d[idx[o]].real(v);
      else out.d[idx[o]].imag(v);
    }
  }
  if (!out_fixed)
    for (auto& x : out.d)
      out.maxkey = std::max(out.maxkey, std::max(oz::group_key(df::words(x.real())), oz::group_key(df::words(x.imag()))));
  return out;
}

// R passes of a layer as the chain does it; returns the relative L2 error against long double.
template <int NL>
static double chain(std::mt19937_64& rng, int n, int R, double spread, double gscale) {
  const std::size_t N = (std::size_t)1 << n;
  std::normal_distribution<double> nd(0, 1);
  std::uniform_real_distribution<double> ud(-1, 1);
  State st;
  st.d.resize(N);
  for (auto& x : st.d) x = cd(nd(rng), nd(rng)) * std::pow(2.0, std::round(ud(rng) * spread));
  std::vector<cld> ref(st.d.begin(), st.d.end());
  for (int pss = 0; pss < R; ++pss) {
    std::vector<int> qs(n);
    for (int q = 0; q < n; ++q) qs[q] = q;
    std::shuffle(qs.begin(), qs.end(), rng);
    const int t[4] = {qs[0], qs[1], qs[2], qs[3]};
    std::vector<cd> Ua, Ub;
    unitary(rng, 4, Ua, gscale);
    unitary(rng, 4, Ub, 1.0);
    const int in_mode = pss == 0 ? 0 : (pss == 1 ? 1 : 2);
    const bool out_fixed = pss > 0 && pss < R - 1;
    st = pass<NL>(st, n, t, Ua, Ub, in_mode, out_fixed);
    // long double reference of the same pair
    std::vector<cld> nx(N, 0);
    const int p[4] = {n - 1 - t[0], n - 1 - t[1], n - 1 - t[2], n - 1 - t[3]};
    for (std::size_t x = 0; x < N; ++x) {
      int o = 0;
      for (int j = 0; j < 4; ++j) o = o * 2 + (int)((x >> p[j]) & 1);
      for (int i = 0; i < 16; ++i) {
        std::size_t y = x;
        for (int j = 0; j < 4; ++j) {
          const std::size_t m = (std::size_t)1 << p[j];
          y = ((i >> (3 - j)) & 1) ? (y | m) : (y & ~m);
        }
        const cld u = cld(Ua[(o >> 2) * 4 + (i >> 2)]) * cld(Ub[(o & 3) * 4 + (i & 3)]);
        nx[x] += u * ref[y];
      }
    }
    ref.swap(nx);
  }
  ld num = 0, den = 0;
  for (std::size_t x = 0; x < N; ++x) {
    num += std::norm(cld(st.d[x]) - ref[x]);
    den += std::norm(ref[x]);
  }
  return (double)std::sqrt(num / den);
}

// fixed_levels (biased bits, one constant) against the direct integer formula
// sum_{l<6} C_l 2^(40 - 8l) + floor((C_6 + 128) / 256) over random and extreme level sums
template <int NL>
static void check_levels(std::mt19937_64& rng) {
  const int64_t lim = (1 << 22) - 1;
  std::uniform_int_distribution<int64_t> U(-lim, lim);
  for (int it = 0; it < 200000; ++it) {
    int64_t C[NL];
    float F[NL];
    for (int l = 0; l < NL; ++l) {
      const int kind = (int)(rng() % 8);
      C[l] = kind == 0 ? lim : kind == 1 ? -lim : kind == 2 ? 0 : U(rng);
      F[l] = (float)C[l];
    }
    int64_t want = 0;
    for (int l = 0; l < 6; ++l) want += C[l] * ((int64_t)1 << (40 - 8 * l));
    if (NL == 7) want += (C[NL - 1] + 128) >> 8;
    const int64_t got = oz::fixed_levels<NL>(F);
    if (got != want) {
      if (fails < 5) std::printf("fixed_levels<%d>: %lld != %lld\n", NL, (long long)got, (long long)want);
      ++fails;
    }
  }
}

// digit_words_fixed (fp16 words of two values, before the packed subtraction of 1152)
// against digits_fixed: every half must be the fp16 of 1024 + (digit + 128)
static void check_digit_words(std::mt19937_64& rng) {
  for (int it = 0; it < 200000; ++it) {
    const int32_t sh = (int32_t)(rng() % 24) - 8;
    const int64_t lim = (int64_t)1 << 47;  // |round(x 2^-sh)| <= 2^47
    int64_t x[2];
    for (int k = 0; k < 2; ++k) {
      const int kind = (int)(rng() % 6);
      int64_t m = kind == 0 ? lim : kind == 1 ? -lim : kind == 2 ? lim - 1 : (int64_t)(rng() % (2 * (uint64_t)lim)) - lim;
      if (sh <= 0) m >>= -sh;  // a left shift must not overflow: x 2^-sh = m
      x[k] = sh >= 1 ? (int64_t)((uint64_t)m << sh) + (int64_t)(rng() % ((uint64_t)1 << sh)) - ((int64_t)1 << (sh - 1))
                     : m;
      if (std::llabs(oz::fixed_round(x[k], sh)) > lim) x[k] = 0;
    }
    if (sh > 15) continue;
    for (int k = 0; k < 2; ++k) {
      const uint64_t want = (uint64_t)oz::fixed_round(x[k], sh) + 0x808080808080ull;
      if (oz::fixed_biased(x[k], sh, oz::fixed_addend(sh)) != want) {
        if (fails < 5) std::printf("fixed_biased: x=%lld sh=%d\n", (long long)x[k], sh);
        ++fails;
      }
    }
    uint32_t w[oz::NS];
    oz::digit_words_fixed(x[0], x[1], sh, w);
    for (int k = 0; k < 2; ++k) {
      float d[oz::NS];
      oz::digits_fixed(x[k], sh, d);
      for (int j = 0; j < oz::NS; ++j) {
        const uint32_t hbits = (w[j] >> (16 * k)) & 0xFFFFu;
        const bool ok = (hbits & 0xFC00u) == 0x6400u && (double)(1024 + (int)(hbits & 0x3FFu)) - 1152.0 == (double)d[j];
        if (!ok) {
          if (fails < 5) std::printf("digit_words_fixed: x=%lld sh=%d digit %d half %04x vs %g\n", (long long)x[k], sh, j, hbits, d[j]);
          ++fails;
        }
      }
    }
  }
}

int main() {
  {
    std::mt19937_64 lr(99);
    check_levels<7>(lr);
    check_levels<6>(lr);
    check_digit_words(lr);
  }
  std::mt19937_64 rng(4242);
  struct Case {
    const char* what;
    int n, R;
    double spread, gscale, bar;
  } cases[] = {{"7 passes, unitary, Gaussian state", 10, 7, 0, 1.0, 1e-13},
               {"28 passes (four layers of a 28-qubit circuit)", 11, 28, 0, 1.0, 1e-13},
               {"64 passes", 10, 64, 0, 1.0, 2e-13},
               {"state magnitudes spread over 2^+-6, 28 passes", 11, 28, 6, 1.0, 2e-13},
               {"2 passes (no fixed-point pass)", 9, 2, 0, 1.0, 1e-13},
               {"3 passes", 9, 3, 0, 1.0, 1e-13},
               {"state magnitudes spread over 2^+-20", 10, 6, 20, 1.0, 2e-12},
               {"non-unitary: gate a scaled by 2^12", 9, 5, 0, 4096.0, 1e-13},
               {"non-unitary: gate a scaled by 2^-30", 9, 5, 0, std::pow(2.0, -30), 1e-13}};
  for (int nl : {7, 6})
    for (auto& c : cases) {
      const double e = nl == 7 ? chain<7>(rng, c.n, c.R, c.spread, c.gscale) : chain<6>(rng, c.n, c.R, c.spread, c.gscale);
      const double bar = nl == 7 ? c.bar : 3 * c.bar;  // six levels: ~2.5x the error
      std::printf("%d levels  %-46s n=%2d passes=%2d  rel L2 %.2e\n", nl, c.what, c.n, c.R, e);
      if (!(e < bar)) {
        std::printf("%s: error above %.0e\n", c.what, bar);
        ++fails;
      }
    }
  if (fails) {
    std::printf("%d failures\n", fails);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
