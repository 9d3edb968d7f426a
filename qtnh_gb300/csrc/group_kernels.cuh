// Grouped kernels over many independent states: one launch applies an operation to a
// list of tasks (state, operands), each split into chunks; a persistent grid walks the
// (task, chunk) work items and finds a work item's task by binary search over the tasks'
// first chunk indices. Templated on the amplitude type: complex64 (float2, FP32 math; a
// gate is held as U_hi + U_lo in complex64) or complex128 (double2, FP64 math).
// Used by the batched executor (batch.cu) and the grouped layer step of the serving loop
// (group.cu).
#pragma once

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
