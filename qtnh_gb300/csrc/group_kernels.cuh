// Grouped kernels over many independent states: one launch applies an operation to a
// list of tasks (state, operands), each split into chunks; a persistent grid walks the
// (task, chunk) work items and finds a work item's task by binary search over the tasks'
// first chunk indices. Templated on the amplitude type: complex64 (float2, FP32 math; a
// gate is held as U_hi + U_lo in complex64) or complex128 (double2, FP64 math).
// Used by the batched executor (batch.cu) and the grouped layer step of the serving loop
// (group.cu).
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>

#include "cuda_common.cuh"
#include "df32.cuh"

namespace qtnh_impl {
namespace grp {

struct GateTask {
  void* psi;        // the state (2^n amplitudes)
  uint32_t n;       // qubits
  uint32_t ba, bb;  // bit positions of gate inputs 0 and 1
  uint32_t gate;    // index into the gate table
};
// Two disjoint two-qubit gates applied in one pass: gate ga on bits (a0, a1), gate gb on
// bits (b0, b1) (input 0, input 1 of each gate).
struct PairTask {
  void* psi;
  uint32_t n;
  uint32_t a0, a1, b0, b1;
  uint32_t ga, gb;
};
struct PhaseTask {
  void* psi;
  uint64_t table;  // offset of the lo table (2^split entries); the hi table follows (2^(n - split))
  uint32_t n, split;
};
struct SwapTask {
  void* psi;
  uint32_t n, ba, bb;
};
struct NormTask {
  void* psi;
  uint32_t n, slot;  // slot into the norm array
};

enum Kind { GATE = 0, PHASE = 1, SWAP = 2, NORM = 3, SCALE = 4, PAIR = 5 };

template <typename T>
struct Cx;
template <>
struct Cx<float2> {
  using R = float;
  static constexpr int GATE_WORDS = 32;  // U_hi[16], U_lo[16]
  __device__ static float2 make(float a, float b) { return make_float2(a, b); }
};
template <>
struct Cx<double2> {
  using R = double;
  static constexpr int GATE_WORDS = 16;  // U[16]
  __device__ static double2 make(double a, double b) { return make_double2(a, b); }
};

__device__ __forceinline__ uint32_t find_task(const uint64_t* __restrict__ cbeg, uint32_t ntasks, uint64_t w) {
  uint32_t lo = 0, hi = ntasks;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (cbeg[mid] <= w)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint64_t insert_zero(uint64_t x, uint32_t bit) {
  return ((x >> bit) << (bit + 1)) | (x & ((1ull << bit) - 1));
}

template <typename T, typename R>
__device__ __forceinline__ void cmac(T u, T x, R& re, R& im) {
  re = fma(u.x, x.x, re);
  re = fma(-u.y, x.y, re);
  im = fma(u.x, x.y, im);
  im = fma(u.y, x.x, im);
}

// One two-qubit gate per task: U[out * 4 + in], input index (input 0, input 1).
template <typename T, int THREADS>
__global__ void __launch_bounds__(THREADS) gate_kernel(const GateTask* __restrict__ tasks,
                                                       const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                                                       uint64_t total, const T* __restrict__ gates,
                                                       uint64_t chunk_groups) {
  using R = typename Cx<T>::R;
  constexpr int GW = Cx<T>::GATE_WORDS;
  __shared__ T g[GW];
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const GateTask t = tasks[s_task];
    if (threadIdx.x < GW) g[threadIdx.x] = gates[(uint64_t)t.gate * GW + threadIdx.x];
    __syncthreads();
    T* psi = static_cast<T*>(t.psi);
    const uint64_t ngroups = 1ull << (t.n - 2);
    const uint64_t g0 = (w - cbeg[s_task]) * chunk_groups;
    const uint64_t g1 = min(g0 + chunk_groups, ngroups);
    const uint32_t lo = min(t.ba, t.bb), hi = max(t.ba, t.bb);
    const uint64_t sa = 1ull << t.ba, sb = 1ull << t.bb;
    for (uint64_t grp = g0 + threadIdx.x; grp < g1; grp += THREADS) {
      const uint64_t x0 = insert_zero(insert_zero(grp, lo), hi);
      const uint64_t off[4] = {0, sb, sa, sa + sb};  // (input 0, input 1) = (0,0), (0,1), (1,0), (1,1)
      T x[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) x[i] = psi[x0 + off[i]];
#pragma unroll
      for (int o = 0; o < 4; ++o) {
        R re = 0, im = 0;
        if (GW == 32) {
#pragma unroll
          for (int i = 0; i < 4; ++i) cmac(g[16 + o * 4 + i], x[i], re, im);  // U_lo first (smaller terms)
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) cmac(g[o * 4 + i], x[i], re, im);
        psi[x0 + off[o]] = Cx<T>::make(re, im);
      }
    }
    __syncthreads();
  }
}

// One gate's table entries (GW amplitude-type words, 256 bytes) from shared memory into
// registers with 128-bit loads that the compiler keeps where they are: each gate is held
// in registers only while it is applied, so the pair kernel needs one gate's registers.
template <typename T, int GW>
union GateRegs {
  uint4 v[16];
  T u[GW];
};
template <typename T, int GW>
__device__ __forceinline__ void load_gate(const T* g, GateRegs<T, GW>& r) {
  static_assert(GW * sizeof(T) == 256, "a gate table entry is 256 bytes");
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(g);
#pragma unroll
  for (int k = 0; k < 16; ++k)
    asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.v[k].x), "=r"(r.v[k].y), "=r"(r.v[k].z), "=r"(r.v[k].w)
                 : "r"(a + 16u * k));
}

// Two disjoint gates per task on groups of 16 amplitudes (index (ia, ib), ia the input pair
// of gate a, ib that of gate b): gate b is applied to the 4 amplitudes of each ia, then
// gate a to the 4 of each ib, both in registers, so the state is read and written once
// for the two gates. Same arithmetic per gate as gate_kernel.
template <typename T, int THREADS>
__global__ void __launch_bounds__(THREADS) pair_kernel(const PairTask* __restrict__ tasks,
                                                       const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                                                       uint64_t total, const T* __restrict__ gates,
                                                       uint64_t chunk_groups) {
  using R = typename Cx<T>::R;
  constexpr int GW = Cx<T>::GATE_WORDS;
  __shared__ __align__(16) T g[2][GW];
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const PairTask t = tasks[s_task];
    if (threadIdx.x < 2 * GW) {
      const int k = threadIdx.x / GW, j = threadIdx.x % GW;
      g[k][j] = gates[(uint64_t)(k ? t.gb : t.ga) * GW + j];
    }
    __syncthreads();
    T* psi = static_cast<T*>(t.psi);
    const uint64_t ngroups = 1ull << (t.n - 4);
    const uint64_t g0 = (w - cbeg[s_task]) * chunk_groups;
    const uint64_t g1 = min(g0 + chunk_groups, ngroups);
    // zero bits inserted in increasing position order
    uint32_t pos[4] = {t.a0, t.a1, t.b0, t.b1};
#pragma unroll
    for (int i = 1; i < 4; ++i)
#pragma unroll
      for (int j = 3; j >= i; --j)
        if (pos[j - 1] > pos[j]) {
          const uint32_t tmp = pos[j - 1];
          pos[j - 1] = pos[j];
          pos[j] = tmp;
        }
    uint64_t offa[4], offb[4];  // (input 0, input 1) = (0,0), (0,1), (1,0), (1,1)
    offa[0] = 0, offa[1] = 1ull << t.a1, offa[2] = 1ull << t.a0, offa[3] = offa[1] + offa[2];
    offb[0] = 0, offb[1] = 1ull << t.b1, offb[2] = 1ull << t.b0, offb[3] = offb[1] + offb[2];
    for (uint64_t grp = g0 + threadIdx.x; grp < g1; grp += THREADS) {
      uint64_t x0 = grp;
#pragma unroll
      for (int i = 0; i < 4; ++i) x0 = insert_zero(x0, pos[i]);
      T x[16];
#pragma unroll
      for (int ia = 0; ia < 4; ++ia)
#pragma unroll
        for (int ib = 0; ib < 4; ++ib) x[ia * 4 + ib] = psi[x0 + offa[ia] + offb[ib]];
      GateRegs<T, GW> u;
      // gate b on each quadruple of fixed ia
      load_gate<T, GW>(g[1], u);
#pragma unroll
      for (int ia = 0; ia < 4; ++ia) {
        T y[4];
#pragma unroll
        for (int o = 0; o < 4; ++o) {
          R re = 0, im = 0;
          if (GW == 32) {
#pragma unroll
            for (int i = 0; i < 4; ++i) cmac(u.u[16 + o * 4 + i], x[ia * 4 + i], re, im);
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) cmac(u.u[o * 4 + i], x[ia * 4 + i], re, im);
          y[o] = Cx<T>::make(re, im);
        }
#pragma unroll
        for (int o = 0; o < 4; ++o) x[ia * 4 + o] = y[o];
      }
      // gate a on each quadruple of fixed ib, stored
      load_gate<T, GW>(g[0], u);
#pragma unroll
      for (int ib = 0; ib < 4; ++ib) {
#pragma unroll
        for (int o = 0; o < 4; ++o) {
          R re = 0, im = 0;
          if (GW == 32) {
#pragma unroll
            for (int i = 0; i < 4; ++i) cmac(u.u[16 + o * 4 + i], x[i * 4 + ib], re, im);
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) cmac(u.u[o * 4 + i], x[i * 4 + ib], re, im);
          psi[x0 + offa[o] + offb[ib]] = Cx<T>::make(re, im);
        }
      }
    }
    __syncthreads();
  }
}

// ---- exact fixed-point gates for complex64 states ----------------------------------
//
// Each group of amplitudes is scaled to integers at its largest exponent E:
// x_int = round(x * 2^(155 - E)) (|x_int| < 2^29); a gate is held as integers
// u_int = round(u * 2^s) (|u_int| < 2^30, s from the gate's largest entry). Products
// accumulate exactly in 64-bit integers (IMAD.WIDE), so an output carries one rounding:
// its conversion to float. Between the two gates of a pair the sums are brought back to
// 32 bits (right shift by the gate's `shift`, |y| < 2^29 by the row bound of the gate).
// Error per pass: the final rounding to complex64, plus 2^-28 of the group's largest
// amplitude from the integer scaling.
struct FxGate {
  int2 u[16];      // (Re, Im) of U[out * 4 + in] as integers at scale 2^s
  int32_t s;       // u = u_int * 2^-s
  int32_t shift;   // requantisation of a first-stage sum: y32 = round(y64 / 2^shift)
  int32_t pad[2];
};
static_assert(sizeof(FxGate) == 144, "FxGate layout");

// Host: the fixed-point form of U[out * 4 + in] (complex128).
inline FxGate make_fx_gate(const std::complex<double>* U) {
  FxGate g{};
  double mx = 0;
  for (int k = 0; k < 16; ++k) mx = std::max(mx, std::max(std::fabs(U[k].real()), std::fabs(U[k].imag())));
  const int eu = mx > 0 ? std::ilogb(mx) : 0;  // mx in [2^eu, 2^(eu + 1))
  g.s = 29 - eu;                                // |u_int| <= 2^30
  long long bound = 0;
  for (int o = 0; o < 4; ++o) {
    long long b = 0;
    for (int i = 0; i < 4; ++i) {
      const long long ur = std::llrint(std::ldexp(U[o * 4 + i].real(), g.s));
      const long long ui = std::llrint(std::ldexp(U[o * 4 + i].imag(), g.s));
      g.u[o * 4 + i] = make_int2((int)ur, (int)ui);
      b += std::llabs(ur) + std::llabs(ui);
    }
    bound = std::max(bound, b);
  }
  // |x_int| <= 2^29, so |y64| <= bound 2^29; shift so that |y32| <= 2^29 (+ rounding)
  int shift = 1;
  while (shift < 62 && (1ll << shift) < bound) ++shift;
  g.shift = shift;
  return g;
}

// float bits of 2^k for k in [-126, 127]
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// Scale exponent of a group whose largest |component| has float bits `m` (sign cleared):
// x * 2^se puts the largest below 2^29 (and at or above 2^28 unless the group is tiny).
__device__ __forceinline__ int fx_scale_exp(uint32_t m) {
  const int E = (int)(m >> 23);
  return max(-99, min(126, 155 - E));
}

__device__ __forceinline__ float fx_to_float(long long v, int k) { return ldexpf(__ll2float_rn(v), k); }

// One complex output o of gate g over 4 integer inputs (re, im): 64-bit exact sums.
__device__ __forceinline__ void fx_row(const FxGate& g, int o, const int (&xr)[4], const int (&xi)[4], long long& re,
                                       long long& im) {
  re = 0;
  im = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int2 u = g.u[o * 4 + i];
    re += (long long)u.x * xr[i] - (long long)u.y * xi[i];
    im += (long long)u.x * xi[i] + (long long)u.y * xr[i];
  }
}

// The 16 integer entries of a gate from shared memory into registers with loads the
// compiler keeps in place (one gate in registers at a time in the pair kernel).
struct FxRegs {
  int2 u[16];
};
__device__ __forceinline__ void fx_load(const FxGate& g, FxRegs& r) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(&g.u[0]);
#pragma unroll
  for (int k = 0; k < 8; ++k)
    asm volatile("ld.shared.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.u[2 * k].x), "=r"(r.u[2 * k].y), "=r"(r.u[2 * k + 1].x), "=r"(r.u[2 * k + 1].y)
                 : "r"(a + 16u * k));
}

// fx_row over register-held entries
__device__ __forceinline__ void fx_row_r(const FxRegs& g, int o, const int (&xr)[4], const int (&xi)[4],
                                         long long& re, long long& im) {
  re = 0;
  im = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int2 u = g.u[o * 4 + i];
    re += (long long)u.x * xr[i] - (long long)u.y * xi[i];
    im += (long long)u.x * xi[i] + (long long)u.y * xr[i];
  }
}

__device__ __forceinline__ int fx_requant(long long y, int shift) {
  return (int)((y + (1ll << (shift - 1))) >> shift);
}

// Single two-qubit gate per task, groups of 4 amplitudes (complex64).
// ---- complex128 states in float-float arithmetic (df32.cuh) ---------------------------
//
// The plain method's values (complex128 in and out, ~48-bit products and sums, one FP64
// add per output component) at FP32 speed: gate entries and amplitudes are split into
// float pairs, products are exact TwoProducts, sums compensated. A gate with entries
// outside the split range makes its whole task FP64; a group with amplitudes outside it
// is computed in FP64 (warp-divergent, rare for normalised states).

struct FfGate {
  df::cf2 u[16];   // U[out * 4 + in], split
  double2 d[16];   // the same in FP64
  int ok;
};

__device__ __forceinline__ void ff_load_gate(const double2* __restrict__ gates, uint32_t gi, FfGate& g, int j) {
  const double2 v = gates[(uint64_t)gi * 16 + j];
  g.d[j] = v;
  const bool ok = df::in_range_gate(v.x) && df::in_range_gate(v.y);
  g.u[j] = ok ? df::csplit(v.x, v.y) : df::cf2{{0.f, 0.f}, {0.f, 0.f}};
  if (!ok) g.ok = 0;
}

// out = sum_i U[o][i] x[i] over four split inputs, as two accumulators.
__device__ __forceinline__ void ff_row(const df::cf2* u, const df::cf2 (&x)[4], int o, df::acc& re, df::acc& im) {
  df::cmul_acc(u[o * 4], x[0], re, im);
#pragma unroll
  for (int i = 1; i < 4; ++i) {
    const df::cf2 g = u[o * 4 + i];
    df::acc_mac(re, g.re, x[i].re);
    df::acc_mac(re, df::neg(g.im), x[i].im);
    df::acc_mac(im, g.re, x[i].im);
    df::acc_mac(im, g.im, x[i].re);
  }
}

__device__ __forceinline__ bool ff_in_range(double2 v) {
  return df::in_range_state(v.x) && df::in_range_state(v.y);
}

// One two-qubit gate per task (as gate_kernel) in float-float.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) ff_gate_kernel(const GateTask* __restrict__ tasks,
                                                          const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                                                          uint64_t total, const double2* __restrict__ gates,
                                                          uint64_t chunk_groups) {
  __shared__ FfGate g;
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) {
      s_task = find_task(cbeg, ntasks, w);
      g.ok = 1;
    }
    __syncthreads();
    const GateTask t = tasks[s_task];
    if (threadIdx.x < 16) ff_load_gate(gates, t.gate, g, threadIdx.x);
    __syncthreads();
    double2* psi = static_cast<double2*>(t.psi);
    const uint64_t ngroups = 1ull << (t.n - 2);
    const uint64_t g0 = (w - cbeg[s_task]) * chunk_groups;
    const uint64_t g1 = min(g0 + chunk_groups, ngroups);
    const uint32_t lo = min(t.ba, t.bb), hi = max(t.ba, t.bb);
    const uint64_t sa = 1ull << t.ba, sb = 1ull << t.bb;
    const uint64_t off[4] = {0, sb, sa, sa + sb};
    for (uint64_t grp = g0 + threadIdx.x; grp < g1; grp += THREADS) {
      const uint64_t x0 = insert_zero(insert_zero(grp, lo), hi);
      double2 x[4];
      bool ok = g.ok != 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        x[i] = psi[x0 + off[i]];
        ok = ok && ff_in_range(x[i]);
      }
      if (ok) {
        df::cf2 xs[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) xs[i] = df::csplit(x[i].x, x[i].y);
#pragma unroll
        for (int o = 0; o < 4; ++o) {
          df::acc re, im;
          ff_row(g.u, xs, o, re, im);
          psi[x0 + off[o]] = make_double2(df::to_double(re), df::to_double(im));
        }
      } else {
#pragma unroll
        for (int o = 0; o < 4; ++o) {
          double re = 0, im = 0;
#pragma unroll
          for (int i = 0; i < 4; ++i) cmac(g.d[o * 4 + i], x[i], re, im);
          psi[x0 + off[o]] = make_double2(re, im);
        }
      }
    }
    __syncthreads();
  }
}

// Two disjoint gates per task (as pair_kernel) in float-float: gate b on the quadruple of
// each ia, its outputs kept as split pairs, then gate a on each ib, stored as doubles.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) ff_pair_kernel(const PairTask* __restrict__ tasks,
                                                          const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                                                          uint64_t total, const double2* __restrict__ gates,
                                                          uint64_t chunk_groups) {
  __shared__ FfGate g[2];
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) {
      s_task = find_task(cbeg, ntasks, w);
      g[0].ok = g[1].ok = 1;
    }
    __syncthreads();
    const PairTask t = tasks[s_task];
    if (threadIdx.x < 32) ff_load_gate(gates, threadIdx.x < 16 ? t.ga : t.gb, g[threadIdx.x >> 4], threadIdx.x & 15);
    __syncthreads();
    double2* psi = static_cast<double2*>(t.psi);
    const uint64_t ngroups = 1ull << (t.n - 4);
    const uint64_t g0 = (w - cbeg[s_task]) * chunk_groups;
    const uint64_t g1 = min(g0 + chunk_groups, ngroups);
    uint32_t pos[4] = {t.a0, t.a1, t.b0, t.b1};
#pragma unroll
    for (int i = 1; i < 4; ++i)
#pragma unroll
      for (int j = 3; j >= i; --j)
        if (pos[j - 1] > pos[j]) {
          const uint32_t tmp = pos[j - 1];
          pos[j - 1] = pos[j];
          pos[j] = tmp;
        }
    uint64_t offa[4], offb[4];
    offa[0] = 0, offa[1] = 1ull << t.a1, offa[2] = 1ull << t.a0, offa[3] = offa[1] + offa[2];
    offb[0] = 0, offb[1] = 1ull << t.b1, offb[2] = 1ull << t.b0, offb[3] = offb[1] + offb[2];
    const bool gok = g[0].ok != 0 && g[1].ok != 0;
    for (uint64_t grp = g0 + threadIdx.x; grp < g1; grp += THREADS) {
      uint64_t x0 = grp;
#pragma unroll
      for (int i = 0; i < 4; ++i) x0 = insert_zero(x0, pos[i]);
      double2 x[16];
      bool ok = gok;
#pragma unroll
      for (int ia = 0; ia < 4; ++ia)
#pragma unroll
        for (int ib = 0; ib < 4; ++ib) {
          x[ia * 4 + ib] = psi[x0 + offa[ia] + offb[ib]];
          ok = ok && ff_in_range(x[ia * 4 + ib]);
        }
      if (ok) {
        df::cf2 xs[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) xs[i] = df::csplit(x[i].x, x[i].y);
#pragma unroll
        for (int ia = 0; ia < 4; ++ia) {
          const df::cf2 in[4] = {xs[ia * 4], xs[ia * 4 + 1], xs[ia * 4 + 2], xs[ia * 4 + 3]};
#pragma unroll
          for (int o = 0; o < 4; ++o) {
            df::acc re, im;
            ff_row(g[1].u, in, o, re, im);
            xs[ia * 4 + o] = df::cf2{df::renorm(re), df::renorm(im)};
          }
        }
#pragma unroll
        for (int ib = 0; ib < 4; ++ib) {
          const df::cf2 in[4] = {xs[ib], xs[4 + ib], xs[8 + ib], xs[12 + ib]};
#pragma unroll
          for (int o = 0; o < 4; ++o) {
            df::acc re, im;
            ff_row(g[0].u, in, o, re, im);
            psi[x0 + offa[o] + offb[ib]] = make_double2(df::to_double(re), df::to_double(im));
          }
        }
      } else {
        // FP64, as pair_kernel<double2>
#pragma unroll
        for (int ia = 0; ia < 4; ++ia) {
          double2 y[4];
#pragma unroll
          for (int o = 0; o < 4; ++o) {
            double re = 0, im = 0;
#pragma unroll
            for (int i = 0; i < 4; ++i) cmac(g[1].d[o * 4 + i], x[ia * 4 + i], re, im);
            y[o] = make_double2(re, im);
          }
#pragma unroll
          for (int o = 0; o < 4; ++o) x[ia * 4 + o] = y[o];
        }
#pragma unroll
        for (int ib = 0; ib < 4; ++ib)
#pragma unroll
          for (int o = 0; o < 4; ++o) {
            double re = 0, im = 0;
#pragma unroll
            for (int i = 0; i < 4; ++i) cmac(g[0].d[o * 4 + i], x[i * 4 + ib], re, im);
            psi[x0 + offa[o] + offb[ib]] = make_double2(re, im);
          }
      }
    }
    __syncthreads();
  }
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) fx_gate_kernel(const GateTask* __restrict__ tasks,
                                                          const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                                                          uint64_t total, const FxGate* __restrict__ gates,
                                                          uint64_t chunk_groups) {
  __shared__ __align__(16) FxGate g;
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const GateTask t = tasks[s_task];
    if (threadIdx.x < 36) reinterpret_cast<int*>(&g)[threadIdx.x] = reinterpret_cast<const int*>(gates + t.gate)[threadIdx.x];
    __syncthreads();
    float2* psi = static_cast<float2*>(t.psi);
    const uint64_t ngroups = 1ull << (t.n - 2);
    const uint64_t g0 = (w - cbeg[s_task]) * chunk_groups;
    const uint64_t g1 = min(g0 + chunk_groups, ngroups);
    const uint32_t lo = min(t.ba, t.bb), hi = max(t.ba, t.bb);
    const uint64_t off[4] = {0, 1ull << t.bb, 1ull << t.ba, (1ull << t.ba) + (1ull << t.bb)};
    for (uint64_t grp = g0 + threadIdx.x; grp < g1; grp += THREADS) {
      const uint64_t x0 = insert_zero(insert_zero(grp, lo), hi);
      float2 x[4];
      uint32_t m = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        x[i] = psi[x0 + off[i]];
        m = max(m, max(__float_as_uint(x[i].x) & 0x7FFFFFFFu, __float_as_uint(x[i].y) & 0x7FFFFFFFu));
      }
      if (m >= 0x7F800000u) {  // an infinity or NaN: the group's outputs are NaN
#pragma unroll
        for (int o = 0; o < 4; ++o) psi[x0 + off[o]] = make_float2(__int_as_float(0x7FC00000), __int_as_float(0x7FC00000));
        continue;
      }
      const int se = fx_scale_exp(m);
      const float sc = pow2f(se);
      int xr[4], xi[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) xr[i] = __float2int_rn(x[i].x * sc), xi[i] = __float2int_rn(x[i].y * sc);
      const int k = -se - g.s;
#pragma unroll
      for (int o = 0; o < 4; ++o) {
        long long re, im;
        fx_row(g, o, xr, xi, re, im);
        psi[x0 + off[o]] = make_float2(fx_to_float(re, k), fx_to_float(im, k));
      }
    }
    __syncthreads();
  }
}

// Two disjoint gates per task (as pair_kernel) in exact fixed point: gate b on each
// quadruple of fixed ia, requantised to 32 bits, then gate a on each quadruple of fixed ib.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 512 / THREADS) fx_pair_kernel(const PairTask* __restrict__ tasks,
                                                          const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                                                          uint64_t total, const FxGate* __restrict__ gates,
                                                          uint64_t chunk_groups) {
  __shared__ __align__(16) FxGate g[2];
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const PairTask t = tasks[s_task];
    if (threadIdx.x < 72) {
      const int k = threadIdx.x / 36, j = threadIdx.x % 36;
      reinterpret_cast<int*>(&g[k])[j] = reinterpret_cast<const int*>(gates + (k ? t.gb : t.ga))[j];
    }
    __syncthreads();
    float2* psi = static_cast<float2*>(t.psi);
    const uint64_t ngroups = 1ull << (t.n - 4);
    const uint64_t g0 = (w - cbeg[s_task]) * chunk_groups;
    const uint64_t g1 = min(g0 + chunk_groups, ngroups);
    uint32_t pos[4] = {t.a0, t.a1, t.b0, t.b1};
#pragma unroll
    for (int i = 1; i < 4; ++i)
#pragma unroll
      for (int j = 3; j >= i; --j)
        if (pos[j - 1] > pos[j]) {
          const uint32_t tmp = pos[j - 1];
          pos[j - 1] = pos[j];
          pos[j] = tmp;
        }
    uint64_t offa[4], offb[4];
    offa[0] = 0, offa[1] = 1ull << t.a1, offa[2] = 1ull << t.a0, offa[3] = offa[1] + offa[2];
    offb[0] = 0, offb[1] = 1ull << t.b1, offb[2] = 1ull << t.b0, offb[3] = offb[1] + offb[2];
    const int sa = g[0].s, sb = g[1].s, shb = g[1].shift;
    for (uint64_t grp = g0 + threadIdx.x; grp < g1; grp += THREADS) {
      uint64_t x0 = grp;
#pragma unroll
      for (int i = 0; i < 4; ++i) x0 = insert_zero(x0, pos[i]);
      int xr[16], xi[16];
      int k;  // output scale: value = sum * 2^k
      {
        float2 x[16];
        uint32_t m = 0;
#pragma unroll
        for (int ia = 0; ia < 4; ++ia)
#pragma unroll
          for (int ib = 0; ib < 4; ++ib) {
            const float2 v = psi[x0 + offa[ia] + offb[ib]];
            x[ia * 4 + ib] = v;
            m = max(m, max(__float_as_uint(v.x) & 0x7FFFFFFFu, __float_as_uint(v.y) & 0x7FFFFFFFu));
          }
        if (m >= 0x7F800000u) {  // an infinity or NaN: the group's outputs are NaN
#pragma unroll
          for (int ia = 0; ia < 4; ++ia)
#pragma unroll
            for (int ib = 0; ib < 4; ++ib) psi[x0 + offa[ia] + offb[ib]] = make_float2(__int_as_float(0x7FC00000), __int_as_float(0x7FC00000));
          continue;
        }
        const int se = fx_scale_exp(m);
        const float sc = pow2f(se);
#pragma unroll
        for (int i = 0; i < 16; ++i) xr[i] = __float2int_rn(x[i].x * sc), xi[i] = __float2int_rn(x[i].y * sc);
        k = -se - sb + shb - sa;
      }
      {
        FxRegs u;
        // gate b on each quadruple of fixed ia (requantised in place)
        fx_load(g[1], u);
#pragma unroll
        for (int ia = 0; ia < 4; ++ia) {
          int vr[4], vi[4], yr[4], yi[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) vr[i] = xr[ia * 4 + i], vi[i] = xi[ia * 4 + i];
#pragma unroll
          for (int o = 0; o < 4; ++o) {
            long long re, im;
            fx_row_r(u, o, vr, vi, re, im);
            yr[o] = fx_requant(re, shb);
            yi[o] = fx_requant(im, shb);
          }
#pragma unroll
          for (int o = 0; o < 4; ++o) xr[ia * 4 + o] = yr[o], xi[ia * 4 + o] = yi[o];
        }
        // gate a on each quadruple of fixed ib, stored
        fx_load(g[0], u);
#pragma unroll
        for (int ib = 0; ib < 4; ++ib) {
          int vr[4], vi[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) vr[i] = xr[i * 4 + ib], vi[i] = xi[i * 4 + ib];
#pragma unroll
          for (int o = 0; o < 4; ++o) {
            long long re, im;
            fx_row_r(u, o, vr, vi, re, im);
            psi[x0 + offa[o] + offb[ib]] = make_float2(fx_to_float(re, k), fx_to_float(im, k));
          }
        }
      }
    }
    __syncthreads();
  }
}

// psi[x] *= lo[x & (2^split - 1)] * hi[x >> split] (tables of per-qubit phase products).
template <typename T>
__global__ void phase_kernel(const PhaseTask* __restrict__ tasks, const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                             uint64_t total, const T* __restrict__ tables, uint64_t chunk) {
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const PhaseTask t = tasks[s_task];
    T* psi = static_cast<T*>(t.psi);
    const uint64_t nel = 1ull << t.n;
    const uint64_t e0 = (w - cbeg[s_task]) * chunk, e1 = min(e0 + chunk, nel);
    const T* tlo = tables + t.table;
    const T* thi = tlo + (1ull << t.split);
    const uint64_t mask = (1ull << t.split) - 1;
    for (uint64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const T a = tlo[e & mask], b = thi[e >> t.split];
      const T f = Cx<T>::make(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
      const T x = psi[e];
      psi[e] = Cx<T>::make(f.x * x.x - f.y * x.y, f.x * x.y + f.y * x.x);
    }
    __syncthreads();
  }
}

// Exchange of two qubits (SwapTensor): amplitudes with bits (ba, bb) = (1, 0) and (0, 1).
template <typename T>
__global__ void swap_kernel(const SwapTask* __restrict__ tasks, const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                            uint64_t total, uint64_t chunk) {
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const SwapTask t = tasks[s_task];
    T* psi = static_cast<T*>(t.psi);
    const uint64_t npairs = 1ull << (t.n - 2);
    const uint64_t p0 = (w - cbeg[s_task]) * chunk, p1 = min(p0 + chunk, npairs);
    const uint32_t lo = min(t.ba, t.bb), hi = max(t.ba, t.bb);
    for (uint64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
      const uint64_t x = insert_zero(insert_zero(p, lo), hi);
      const uint64_t xa = x + (1ull << t.ba), xb = x + (1ull << t.bb);
      const T va = psi[xa], vb = psi[xb];
      psi[xa] = vb;
      psi[xb] = va;
    }
    __syncthreads();
  }
}

// Sum of |psi|^2 per task into norms[slot]: compensated sums per thread (TwoSum in the
// amplitude's precision), FP64 across threads and blocks.
template <typename T>
__global__ void norm_kernel(const NormTask* __restrict__ tasks, const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                            uint64_t total, uint64_t chunk, double* __restrict__ norms) {
  using R = typename Cx<T>::R;
  __shared__ uint32_t s_task;
  __shared__ double s_part[32];
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const NormTask t = tasks[s_task];
    const T* psi = static_cast<const T*>(t.psi);
    const uint64_t nel = 1ull << t.n;
    const uint64_t e0 = (w - cbeg[s_task]) * chunk, e1 = min(e0 + chunk, nel);
    R s = 0, c = 0;
    for (uint64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const T x = psi[e];
      const R v = fma(x.x, x.x, x.y * x.y);
      const R ns = s + v;
      const R bb = ns - s;
      c += (s - (ns - bb)) + (v - bb);
      s = ns;
    }
    double v = (double)s + (double)c;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) tot += s_part[i];
      atomicAdd(&norms[t.slot], tot);
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void scale_kernel(const NormTask* __restrict__ tasks, const uint64_t* __restrict__ cbeg, uint32_t ntasks,
                             uint64_t total, uint64_t chunk, const double* __restrict__ norms) {
  using R = typename Cx<T>::R;
  __shared__ uint32_t s_task;
  for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) s_task = find_task(cbeg, ntasks, w);
    __syncthreads();
    const NormTask t = tasks[s_task];
    T* psi = static_cast<T*>(t.psi);
    const double nrm = norms[t.slot];
    const R f = nrm > 0.0 ? (R)(1.0 / sqrt(nrm)) : (R)1;
    const uint64_t nel = 1ull << t.n;
    const uint64_t e0 = (w - cbeg[s_task]) * chunk, e1 = min(e0 + chunk, nel);
    for (uint64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const T x = psi[e];
      psi[e] = Cx<T>::make(x.x * f, x.y * f);
    }
    __syncthreads();
  }
}

// out[i] = psi[where[i]] as complex128.
template <typename T>
__global__ void gather_kernel(const T* __restrict__ psi, const uint64_t* __restrict__ where, uint64_t nq,
                              double2* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += (uint64_t)gridDim.x * blockDim.x) {
    const T x = psi[where[i]];
    out[i] = make_double2((double)x.x, (double)x.y);
  }
}

}  // namespace grp
}  // namespace qtnh_impl
