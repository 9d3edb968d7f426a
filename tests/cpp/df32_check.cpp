// Host-side check of the compensated FP32 arithmetic used by the complex128 kernels
// (qtnh_gb300/csrc/df32.cuh): split exactness, complex gate application error against
// long double, and the in-range classification. Prints "ok" and exits 0 on success.
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>

#include "df32.cuh"

using namespace qtnh_impl::df;
typedef long double ld;

static int fails = 0;
#define CHECK(c, ...) do { if (!(c)) { std::printf(__VA_ARGS__); std::printf("\n"); ++fails; } } while (0)

int main() {
  std::mt19937_64 rng(42);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_int_distribution<int> ed(-88, 88);

  // 1. split: |x - (hi + lo)| <= 2^-47 |x| over the whole range
  double worst_split = 0;
  for (int t = 0; t < 2000000; ++t) {
    double x = std::ldexp(nd(rng), ed(rng));
    if (!in_range_state(x)) continue;  // the kernels split only in-range values
    f2 s = split(x);
    ld err = std::fabs((ld)x - ((ld)s.h + (ld)s.l)) / std::fabs((ld)x);
    if ((double)err > worst_split) worst_split = (double)err;
  }
  CHECK(worst_split <= std::ldexp(1.0, -47), "split error %g", worst_split);
  CHECK(split(0.0).h == 0.0f && split(-0.0).l == 0.0f, "zero split");

  // 2. two-qubit complex gate, D = 4: y_o = sum_i g[i][o] x_i, relative L2 error vs long double
  double worst_gate = 0, sum_sq_err = 0, sum_sq = 0;
  for (int t = 0; t < 200000; ++t) {
    std::complex<double> g[16], x[4];
    for (auto& v : g) v = {nd(rng) * 0.5, nd(rng) * 0.5};
    int scale = ed(rng) / 2;
    for (auto& v : x) v = {std::ldexp(nd(rng), scale), std::ldexp(nd(rng), scale)};
    cf2 gs[16], xs[4];
    for (int i = 0; i < 16; ++i) gs[i] = csplit(g[i].real(), g[i].imag());
    for (int i = 0; i < 4; ++i) xs[i] = csplit(x[i].real(), x[i].imag());
    ld num = 0, den = 0;
    for (int o = 0; o < 4; ++o) {
      acc re, im;
      cmul_acc(gs[0 * 4 + o], xs[0], re, im);
      for (int i = 1; i < 4; ++i) {
        acc_mac(re, gs[i * 4 + o].re, xs[i].re);
        acc_mac(re, neg(gs[i * 4 + o].im), xs[i].im);
        acc_mac(im, gs[i * 4 + o].re, xs[i].im);
        acc_mac(im, gs[i * 4 + o].im, xs[i].re);
      }
      double yr = to_double(re), yi = to_double(im);
      ld rr = 0, ri = 0;
      for (int i = 0; i < 4; ++i) {
        rr += (ld)g[i * 4 + o].real() * x[i].real() - (ld)g[i * 4 + o].imag() * x[i].imag();
        ri += (ld)g[i * 4 + o].real() * x[i].imag() + (ld)g[i * 4 + o].imag() * x[i].real();
      }
      num += (yr - rr) * (yr - rr) + (yi - ri) * (yi - ri);
      den += rr * rr + ri * ri;
    }
    double rel = (double)std::sqrt(num / den);
    if (rel > worst_gate) worst_gate = rel;
    sum_sq_err += (double)(num / den);
    sum_sq += 1;
  }
  double rms_gate = std::sqrt(sum_sq_err / sum_sq);
  CHECK(worst_gate < 1e-13, "gate worst rel err %g", worst_gate);
  CHECK(rms_gate < 1.2e-14, "gate rms rel err %g", rms_gate);

  // 2b. error growth over a chain of 600 unitary two-qubit gates on one 4-amplitude
  // group (the circuit applies 560): must stay well inside the 1e-12 relative L2 bar.
  double worst_chain = 0;
  for (int trial = 0; trial < 20; ++trial) {
    std::complex<ld> ref[4];
    std::complex<double> cur[4];
    for (int i = 0; i < 4; ++i) cur[i] = {nd(rng), nd(rng)}, ref[i] = {(ld)cur[i].real(), (ld)cur[i].imag()};
    for (int step = 0; step < 600; ++step) {
      // random unitary 4x4 by Gram-Schmidt on a complex Gaussian matrix (long double)
      std::complex<ld> u[4][4];
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) u[a][b] = {(ld)nd(rng), (ld)nd(rng)};
      for (int a = 0; a < 4; ++a) {
        for (int b = 0; b < a; ++b) {
          std::complex<ld> d = 0;
          for (int k = 0; k < 4; ++k) d += std::conj(u[b][k]) * u[a][k];
          for (int k = 0; k < 4; ++k) u[a][k] -= d * u[b][k];
        }
        ld nrm = 0;
        for (int k = 0; k < 4; ++k) nrm += std::norm(u[a][k]);
        for (int k = 0; k < 4; ++k) u[a][k] /= std::sqrt(nrm);
      }
      // gate in SymmTensor layout g[in*4 + out] = U[out][in], rounded to double
      cf2 gs[16], xs[4];
      std::complex<double> gd[16];
      for (int i = 0; i < 4; ++i)
        for (int o = 0; o < 4; ++o) gd[i * 4 + o] = {(double)u[o][i].real(), (double)u[o][i].imag()};
      for (int i = 0; i < 16; ++i) gs[i] = csplit(gd[i].real(), gd[i].imag());
      for (int i = 0; i < 4; ++i) xs[i] = csplit(cur[i].real(), cur[i].imag());
      std::complex<ld> nref[4];
      for (int o = 0; o < 4; ++o) {
        acc re, im;
        cmul_acc(gs[o], xs[0], re, im);
        for (int i = 1; i < 4; ++i) {
          acc_mac(re, gs[i * 4 + o].re, xs[i].re);
          acc_mac(re, neg(gs[i * 4 + o].im), xs[i].im);
          acc_mac(im, gs[i * 4 + o].re, xs[i].im);
          acc_mac(im, gs[i * 4 + o].im, xs[i].re);
        }
        nref[o] = 0;
        for (int i = 0; i < 4; ++i) nref[o] += std::complex<ld>(gd[i * 4 + o].real(), gd[i * 4 + o].imag()) * ref[i];
        cur[o] = {to_double(re), to_double(im)};
      }
      for (int o = 0; o < 4; ++o) ref[o] = nref[o];
    }
    ld num = 0, den = 0;
    for (int i = 0; i < 4; ++i) num += std::norm(std::complex<ld>(cur[i].real(), cur[i].imag()) - ref[i]), den += std::norm(ref[i]);
    double rel = (double)std::sqrt(num / den);
    if (rel > worst_chain) worst_chain = rel;
  }
  CHECK(worst_chain < 2e-12, "600-gate chain rel err %g", worst_chain);

  // 3. range classification
  CHECK(in_range_state(0.0) && in_range_state(-0.0) && in_range_state(1.0) && in_range_state(std::ldexp(1.0, -90)) &&
            !in_range_state(std::ldexp(1.0, -91)) && !in_range_state(std::ldexp(1.0, 91)) &&
            !in_range_state(INFINITY) && !in_range_state(NAN) && !in_range_state(5e-324),
        "state range classification");
  CHECK(in_range_gate(1.0) && !in_range_gate(std::ldexp(1.0, 31)) && !in_range_gate(std::ldexp(1.0, -31)), "gate range");

  std::printf("split worst %.3e  gate worst %.3e  gate rms %.3e  600-gate chain worst %.3e\n", worst_split, worst_gate,
              rms_gate, worst_chain);
  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
