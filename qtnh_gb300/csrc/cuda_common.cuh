// CUDA-side helpers shared by the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "internal.h"

namespace qtnh_impl {

void check_cuda(cudaError_t e, const char* what);
int sm_count();

// complex<double> as two doubles: 16 bytes, one 128-bit load/store.
using c128 = double2;

__device__ __forceinline__ c128 cmul(c128 a, c128 b) {
  // (a.x + i a.y)(b.x + i b.y) with the same operation order as std::complex<double>'s
  // finite-value product: real = a.x*b.x - a.y*b.y, imag = a.x*b.y + a.y*b.x.
  return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                      __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

// a*b in four FP64 instructions (two multiplies, two fused multiply-adds).
__device__ __forceinline__ c128 cmul_fused(c128 a, c128 b) {
  return make_double2(fma(a.x, b.x, -(a.y * b.y)), fma(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ c128 cfma(c128 a, c128 b, c128 acc) {
  // acc + a*b with fused multiply-adds (one rounding per FMA).
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}

// Mixed-radix axis description used by kernels that decode a linear index.
// Powers of two decode with shift/mask; other extents with 64-bit division.
struct Axis {
  uint64_t dim;
  uint32_t log2;  // 0xFFFFFFFF when dim is not a power of two
  uint64_t s_in, s_out;
};

inline uint32_t log2_or_none(uint64_t d) {
  if (d && !(d & (d - 1))) {
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    return l;
  }
  return 0xFFFFFFFFu;
}

constexpr int KMAX = 40;  // axes after dropping size-1 axes (2^40 elements is far beyond HBM)

// A set of axes enumerated row-major (slowest first) with their strides in two layouts.
struct RestDesc {
  int n = 0;
  uint64_t total = 1;
  Axis ax[KMAX];
};

__device__ __forceinline__ void decode(uint64_t idx, const RestDesc& r, uint64_t& oin, uint64_t& oout) {
  oin = 0;
  oout = 0;
  for (int k = r.n - 1; k >= 0; --k) {
    const Axis& a = r.ax[k];
    uint64_t d;
    if (a.log2 != 0xFFFFFFFFu) {
      d = idx & (a.dim - 1);
      idx >>= a.log2;
    } else {
      d = idx % a.dim;
      idx /= a.dim;
    }
    oin += d * a.s_in;
    oout += d * a.s_out;
  }
}

inline void fill_axis(Axis& a, uint64_t dim, uint64_t s_in, uint64_t s_out) {
  a.dim = dim;
  a.log2 = log2_or_none(dim);
  a.s_in = s_in;
  a.s_out = s_out;
}

// Asynchronous 16-byte copies global -> shared (bypassing L1), in commit groups.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

inline int grid_for(uint64_t work_items, int per_sm) {
  uint64_t cap = (uint64_t)sm_count() * per_sm;
  return (int)(work_items < 1 ? 1 : (work_items < cap ? work_items : cap));
}

}  // namespace qtnh_impl
