// Symmetric-gate and diagonal contractions applied in place.
//
// When the second operand of Tensor::contract is a SymmTensor whose inputs are all wired
// (src/tensor/contract.cpp:250-289), the result keeps the state's index order and each
// gate output replaces the state index wired to the matching input. The reference still
// runs the generic permute -> triple loop -> permute path (contract.cpp:12-201) through
// per-element iterator objects. Here, for D = prod(target dims) <= 4, it is a
// register-blocked kernel: each thread owns one group of D amplitudes (all other indices
// fixed), loads them with 128-bit loads, applies the D x D gate from shared memory and
// stores them back. Consecutive threads own consecutive groups, so loads and stores are
// coalesced unless a target is the innermost index, in which case every thread touches D
// contiguous elements. For D = 8, 9 and 16 the threads of a block share the groups
// through shared memory, one thread per (output, group) (gate_coop_kernel); any other D
// runs a general FP64 kernel out of a copy of the state (gate_kernel_any).
//
// DiagTensor contraction (the reference stubs DiagTensor: src/tensor/diag.cpp:65-117)
// is defined as contraction with D[in, out] = d[in] * delta(in, out); with the in-place
// rule that is an elementwise multiply psi[x] *= d[x restricted to the targets], a
// streaming kernel. A layer of single-index diagonals (one per qubit) is folded into two
// phase tables (trailing indices, leading indices) so the whole layer is one pass.

#include <algorithm>
#include <memory>
#include <numeric>

#include "cuda_common.cuh"
#include "df32.cuh"

namespace qtnh_impl {

namespace {

constexpr int GATE_MAX_D = 16;

struct GateParams {
  RestDesc other;              // indices that are not gate targets, merged, with state strides in s_in
  int64_t off[GATE_MAX_D];     // offsets of the D amplitudes of a group (row-major over targets)
  // When every dimension is a power of two, the group base is the group index with
  // zero bits inserted at the targets' bit positions (ascending): nins insertions of
  // ins_width[j] zero bits at bit ins_pos[j].
  int nins;
  uint32_t ins_pos[8], ins_width[8];
};

__device__ __forceinline__ uint64_t group_base(uint64_t grp, const GateParams& p) {
  if (p.nins >= 0) {
    uint64_t b = grp;
    for (int j = 0; j < p.nins; ++j) {
      const uint64_t low = b & ((1ull << p.ins_pos[j]) - 1);
      b = ((b >> p.ins_pos[j]) << (p.ins_pos[j] + p.ins_width[j])) | low;
    }
    return b;
  }
  uint64_t base, unused;
  decode(grp, p.other, base, unused);
  return base;
}

template <int D>
__global__ void __launch_bounds__(256) gate_kernel(c128* __restrict__ psi, const c128* __restrict__ gate,
                                                   const __grid_constant__ GateParams p) {
  __shared__ c128 g[D * D];
  for (int t = threadIdx.x; t < D * D; t += blockDim.x) g[t] = gate[t];
  __syncthreads();
  for (uint64_t grp = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; grp < p.other.total;
       grp += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t base = group_base(grp, p);
    c128 x[D];
#pragma unroll
    for (int i = 0; i < D; ++i) x[i] = psi[base + p.off[i]];
#pragma unroll
    for (int o = 0; o < D; ++o) {
      c128 acc = make_double2(0.0, 0.0);
#pragma unroll
      for (int i = 0; i < D; ++i) acc = cfma(g[i * D + o], x[i], acc);  // SymmTensor layout [in, out]
      psi[base + p.off[o]] = acc;
    }
  }
}

// Target decode of the general kernel: the D = prod(tdim) amplitudes of a group, row-major
// over the targets (the last target fastest), at state strides tstr.
struct GateAnyParams {
  uint64_t D;
  int k;
  uint64_t tdim[QTNH_MAX_RANK];
  int64_t tstr[QTNH_MAX_RANK];
};

// Any gate size: one thread per (group, output), reading the inputs from a copy of the
// state (`in`) and writing psi, in FP64 fused multiply-adds.
__global__ void __launch_bounds__(256) gate_kernel_any(c128* __restrict__ psi, const c128* __restrict__ in,
                                                       const c128* __restrict__ gate,
                                                       const __grid_constant__ GateParams p,
                                                       const __grid_constant__ GateAnyParams a) {
  const uint64_t total = p.other.total * a.D;
  for (uint64_t it = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; it < total;
       it += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t grp = it / a.D, o = it % a.D;
    const uint64_t base = group_base(grp, p);
    int64_t off_o = 0;
    uint64_t rem = o;
    for (int j = a.k - 1; j >= 0; --j) {
      off_o += (int64_t)(rem % a.tdim[j]) * a.tstr[j];
      rem /= a.tdim[j];
    }
    // inputs in row-major order: an odometer over the target digits
    uint64_t digit[QTNH_MAX_RANK];
    for (int j = 0; j < a.k; ++j) digit[j] = 0;
    int64_t off_i = 0;
    c128 acc = make_double2(0.0, 0.0);
    for (uint64_t i = 0; i < a.D; ++i) {
      acc = cfma(gate[i * a.D + o], in[base + off_i], acc);  // SymmTensor layout [in, out]
      for (int j = a.k - 1; j >= 0; --j) {
        if (++digit[j] < a.tdim[j]) {
          off_i += a.tstr[j];
          break;
        }
        digit[j] = 0;
        off_i -= (int64_t)(a.tdim[j] - 1) * a.tstr[j];
      }
    }
    psi[base + off_o] = acc;
  }
}

// FP64 fallback for one group (kept out of line so the float-float path is never
// predicated over it; it re-reads the group, which has not been written yet).
template <int D>
__device__ __noinline__ void gate_group_fp64(c128* __restrict__ psi, uint64_t base, const int64_t* off,
                                             const c128* __restrict__ g) {
  c128 x[D];
#pragma unroll
  for (int i = 0; i < D; ++i) x[i] = psi[base + off[i]];
#pragma unroll
  for (int o = 0; o < D; ++o) {
    c128 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int i = 0; i < D; ++i) acc = cfma(g[i * D + o], x[i], acc);
    psi[base + off[o]] = acc;
  }
}

// Float-float variant (see df32.cuh): the FP32 pipe does the arithmetic, complex128 in
// HBM. A warp whose groups have any element outside the split range takes the FP64
// path (a warp-uniform branch); so does every group when a gate element is out of range.
template <int D>
__global__ void __launch_bounds__(256, (D <= 4 ? 3 : 1)) gate_kernel_f32x2(c128* __restrict__ psi,
                                                                         const c128* __restrict__ gate,
                                                                         const __grid_constant__ GateParams p) {
  __shared__ c128 g[D * D];
  __shared__ df::cf2 gs[D * D];
  __shared__ int gate_ok;
  if (threadIdx.x == 0) gate_ok = 1;
  __syncthreads();
  for (int t = threadIdx.x; t < D * D; t += blockDim.x) {
    c128 v = gate[t];
    g[t] = v;
    bool ok = df::in_range_gate(v.x) && df::in_range_gate(v.y);
    if (!ok) gate_ok = 0;
    gs[t] = ok ? df::csplit(v.x, v.y) : df::cf2{{0.f, 0.f}, {0.f, 0.f}};
  }
  __syncthreads();
  const bool gok = gate_ok != 0;
  for (uint64_t grp = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; grp < p.other.total;
       grp += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t base = group_base(grp, p);
    c128 x[D];
    bool ok = gok;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      x[i] = psi[base + p.off[i]];
      ok = ok && df::in_range_state(x[i].x) && df::in_range_state(x[i].y);
    }
    if (__all_sync(__activemask(), ok)) {
      df::cf2 xs[D];
#pragma unroll
      for (int i = 0; i < D; ++i) xs[i] = df::csplit(x[i].x, x[i].y);
#pragma unroll
      for (int o = 0; o < D; ++o) {
        df::acc re, im;
        df::cmul_acc(gs[o], xs[0], re, im);
#pragma unroll
        for (int i = 1; i < D; ++i) {
          const df::cf2 gi = gs[i * D + o];
          df::acc_mac(re, gi.re, xs[i].re);
          df::acc_mac(re, df::neg(gi.im), xs[i].im);
          df::acc_mac(im, gi.re, xs[i].im);
          df::acc_mac(im, gi.im, xs[i].re);
        }
        psi[base + p.off[o]] = make_double2(df::to_double(re), df::to_double(im));
      }
    } else {
      gate_group_fp64<D>(psi, base, p.off, g);
    }
  }
}

// Gates of 8 or more amplitudes per group: the threads of a block share the groups'
// amplitudes through shared memory, one thread per (output, group) and GB = 256 / D
// groups per batch, instead of one thread holding a whole group in registers (which spills
// in FP64 and leaves one 8-warp block per SM in float-float). Thread t takes group t % GB
// and output t / GB, so loads and stores run over consecutive groups (coalesced), and the
// amplitudes are kept transposed in shared memory ([input][group]): a warp reads one
// input of consecutive groups (no bank conflict) while the gate element is broadcast.
// FF: float-float arithmetic with the amplitudes split once each; a batch holding an
// element outside the split range (or any gate element outside it) runs in FP64.
template <int D, bool FF>
__global__ void __launch_bounds__(256) gate_coop_kernel(c128* __restrict__ psi, const c128* __restrict__ gate,
                                                        const __grid_constant__ GateParams p) {
  constexpr int GB = 256 / D;
  __shared__ c128 g[D * D];
  __shared__ df::cf2 gs[FF ? D * D : 1];
  __shared__ c128 xs[D][GB];
  __shared__ df::cf2 xsp[FF ? D : 1][GB];
  __shared__ int gate_ok;
  if (threadIdx.x == 0) gate_ok = 1;
  __syncthreads();
  for (int t = threadIdx.x; t < D * D; t += blockDim.x) {
    const c128 v = gate[t];
    g[t] = v;
    if (FF) {
      const bool ok = df::in_range_gate(v.x) && df::in_range_gate(v.y);
      if (!ok) gate_ok = 0;
      gs[FF ? t : 0] = ok ? df::csplit(v.x, v.y) : df::cf2{{0.f, 0.f}, {0.f, 0.f}};
    }
  }
  __syncthreads();
  const bool gok = gate_ok != 0;
  const int gl = threadIdx.x % GB, o = threadIdx.x / GB;
  const bool active = o < D;  // D * GB <= 256 threads take part
  const uint64_t ngroups = p.other.total, stride = (uint64_t)gridDim.x * GB;
  // this thread's amplitude of the batch at g0 (loaded one batch ahead)
  auto fetch = [&](uint64_t g0, bool& live, uint64_t& addr, c128& x) {
    const uint64_t grp = g0 + gl;
    live = active && grp < ngroups;
    addr = live ? group_base(grp, p) + p.off[o] : 0;
    x = live ? psi[addr] : make_double2(0.0, 0.0);
  };
  bool live;
  uint64_t addr;
  c128 x;
  fetch(blockIdx.x * (uint64_t)GB, live, addr, x);
  for (uint64_t g0 = blockIdx.x * (uint64_t)GB; g0 < ngroups; g0 += stride) {
    bool ok = true;
    if (active) {
      xs[o][gl] = x;
      if (FF) {
        ok = gok && df::in_range_state(x.x) && df::in_range_state(x.y);
        xsp[FF ? o : 0][gl] = ok ? df::csplit(x.x, x.y) : df::cf2{{0.f, 0.f}, {0.f, 0.f}};
      }
    }
    const bool all_ok = __syncthreads_and(ok);  // the batch's amplitudes are in shared memory
    bool live_n;
    uint64_t addr_n;
    c128 x_n;
    fetch(g0 + stride, live_n, addr_n, x_n);  // other groups: in flight during the arithmetic
    if (live) {
      c128 y;
      if (FF && all_ok) {
        df::acc re, im;
        df::cmul_acc(gs[o], xsp[0][gl], re, im);
#pragma unroll
        for (int i = 1; i < D; ++i) {
          const df::cf2 gi = gs[FF ? i * D + o : 0];
          const df::cf2 xi = xsp[FF ? i : 0][gl];
          df::acc_mac(re, gi.re, xi.re);
          df::acc_mac(re, df::neg(gi.im), xi.im);
          df::acc_mac(im, gi.re, xi.im);
          df::acc_mac(im, gi.im, xi.re);
        }
        y = make_double2(df::to_double(re), df::to_double(im));
      } else {
        y = make_double2(0.0, 0.0);
#pragma unroll
        for (int i = 0; i < D; ++i) y = cfma(g[i * D + o], xs[i][gl], y);  // SymmTensor layout [in, out]
      }
      psi[addr] = y;
    }
    __syncthreads();  // shared copies free for the next batch
    live = live_n, addr = addr_n, x = x_n;
  }
}

struct DiagParams {
  uint64_t n;
  int k;
  uint64_t dim[8], stride[8], mult[8];
  uint32_t dim_log2[8], stride_log2[8];
};

// Streaming kernels move DU elements per thread per step, all loads issued before any
// arithmetic, so that enough bytes are in flight per SM to keep HBM busy. IT is the index
// type (32-bit when the state and the grid stride fit).
constexpr int DU = 4;
// Elements of a thread's DU per step that the default arithmetic mode multiplies in native
// FP64 beside the float-float ones (QTNH_ARITH_F32X2 keeps all DU in float-float).
constexpr int DIAG_FP64_SLOTS = 1;
constexpr int LAYER_FP64_SLOTS = 1;

template <typename IT>
__device__ __forceinline__ IT diag_index(IT e, const DiagParams& p) {
  IT idx = 0;
  for (int j = 0; j < p.k; ++j) {
    IT q;
    if (p.stride_log2[j] != 0xFFFFFFFFu) q = e >> p.stride_log2[j];
    else q = (IT)(e / (IT)p.stride[j]);
    const IT dg = (p.dim_log2[j] != 0xFFFFFFFFu) ? (q & (IT)(p.dim[j] - 1)) : (IT)(q % (IT)p.dim[j]);
    idx += dg * (IT)p.mult[j];
  }
  return idx;
}

__device__ __noinline__ c128 cmul_fp64_outofline(c128 a, c128 b) { return cmul(a, b); }

// psi[e] *= d[index of e over the targets] in FP64.
template <typename IT>
__global__ void __launch_bounds__(256) diag_kernel(c128* __restrict__ psi, const c128* __restrict__ d,
                                                   const __grid_constant__ DiagParams p) {
  const IT n = (IT)p.n, step = (IT)gridDim.x * blockDim.x * DU;
  for (IT base = (IT)blockIdx.x * blockDim.x * DU + threadIdx.x; base < n; base += step) {
    c128 x[DU], f[DU];
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e < n) x[u] = psi[e], f[u] = __ldg(d + diag_index<IT>(e, p));
    }
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e < n) psi[e] = cmul(x[u], f[u]);
    }
  }
}

// The same in float-float: the diagonal comes pre-split (ds, table_split_kernel; a NaN hi
// part flags an entry outside the float-float range), the amplitude is split per element.
// The first NF64 of a thread's DU elements per step are multiplied in native FP64 instead:
// the FP64 unit and the FP32 pipes then work side by side in one instruction stream (each
// alone caps the kernel below the HBM rate: FP64 by its throughput, float-float by issue).
template <typename IT, int NF64>
__global__ void __launch_bounds__(256) diag_kernel_f32x2(c128* __restrict__ psi, const c128* __restrict__ d,
                                                         const df::cf2* __restrict__ ds,
                                                         const __grid_constant__ DiagParams p) {
  static_assert(NF64 >= 0 && NF64 < DU, "at least one float-float element per step");
  const IT n = (IT)p.n, step = (IT)gridDim.x * blockDim.x * DU;
  for (IT base = (IT)blockIdx.x * blockDim.x * DU + threadIdx.x; base < n; base += step) {
    c128 x[DU], fd[NF64 > 0 ? NF64 : 1];
    df::cf2 f[DU];
    IT idx[DU];
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e < n) {
        idx[u] = diag_index<IT>(e, p), x[u] = psi[e];
        if (u < NF64) fd[u < NF64 ? u : 0] = __ldg(d + idx[u]);
        else f[u] = ds[idx[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e >= n) continue;
      if (u < NF64) {
        psi[e] = cmul_fused(x[u], fd[u < NF64 ? u : 0]);
        continue;
      }
      const bool ok = f[u].re.h == f[u].re.h && df::in_range_state(x[u].x) && df::in_range_state(x[u].y);
      if (__all_sync(__activemask(), ok)) {
        df::acc re, im;
        df::cmul_acc(df::csplit(x[u].x, x[u].y), f[u], re, im);
        psi[e] = make_double2(df::to_double(re), df::to_double(im));
      } else {
        psi[e] = cmul_fp64_outofline(x[u], __ldg(d + idx[u]));
      }
    }
  }
}

// ---- diagonal layer ----------------------------------------------------------------

constexpr int LAYER_MAX_FACTORS = 64;

struct LayerTableParams {
  uint64_t size;          // table entries
  uint64_t elem_stride;   // state elements per table step along the table's axes (unused by the kernel)
  int nf;                 // factors that fall into this table
  uint64_t f_stride[LAYER_MAX_FACTORS];  // stride of the factor's axis inside the table index
  uint64_t f_dim[LAYER_MAX_FACTORS];
  uint64_t f_off[LAYER_MAX_FACTORS];     // offset of the factor's entries in `factors`
};

__global__ void layer_table_kernel(const c128* __restrict__ factors, c128* __restrict__ table,
                                   const __grid_constant__ LayerTableParams p) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p.size; j += (uint64_t)gridDim.x * blockDim.x) {
    c128 v = make_double2(1.0, 0.0);
    for (int f = 0; f < p.nf; ++f) {
      uint64_t dgt = (j / p.f_stride[f]) % p.f_dim[f];
      v = cmul(v, factors[p.f_off[f] + dgt]);
    }
    table[j] = v;
  }
}

template <typename IT>
__device__ __forceinline__ void hi_lo(IT e, IT lo_size, uint32_t lo_log2, IT& h, IT& l) {
  if (lo_log2 != 0xFFFFFFFFu) h = e >> lo_log2, l = e & (lo_size - 1);
  else h = e / lo_size, l = e % lo_size;
}

// psi[e] *= hi[e / lo_size] * lo[e % lo_size]; lo_size is a power of two or general.
template <typename IT>
__global__ void __launch_bounds__(256) layer_apply_kernel(c128* __restrict__ psi, const c128* __restrict__ hi,
                                                          const c128* __restrict__ lo, uint64_t n64,
                                                          uint64_t lo_size64, uint32_t lo_log2) {
  const IT n = (IT)n64, lo_size = (IT)lo_size64, step = (IT)gridDim.x * blockDim.x * DU;
  for (IT base = (IT)blockIdx.x * blockDim.x * DU + threadIdx.x; base < n; base += step) {
    c128 x[DU], ph[DU];
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e < n) {
        IT h, l;
        hi_lo<IT>(e, lo_size, lo_log2, h, l);
        x[u] = psi[e];
        ph[u] = cmul(__ldg(hi + h), __ldg(lo + l));
      }
    }
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e < n) psi[e] = cmul(x[u], ph[u]);
    }
  }
}

// out[e] = gate[e] * diag[digit p of e's output index] (elements [in * D + o], the digit at
// stride `stride` and radix `dp`); one thread per element, in place allowed.
__global__ void diag_product_kernel(const c128* gate, const c128* __restrict__ diag, c128* out, uint64_t n, uint64_t D,
                                    uint64_t stride, uint64_t dp) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t o = e % D;
    out[e] = cmul(gate[e], diag[(o / stride) % dp]);
  }
}

// Split copy of a phase table (float pairs) plus a per-entry range flag in the sign of
// nothing: entries out of the gate range are kept as FP64 and flagged with NaN hi parts.
__global__ void table_split_kernel(const c128* __restrict__ t, df::cf2* __restrict__ ts, uint64_t n) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
    c128 v = t[j];
    if (df::in_range_gate(v.x) && df::in_range_gate(v.y)) ts[j] = df::csplit(v.x, v.y);
    else ts[j] = df::cf2{{__int_as_float(0x7FC00000), 0.f}, {0.f, 0.f}};
  }
}

// Float-float layer; the first NF64 of a thread's DU elements per step in native FP64
// (as diag_kernel_f32x2).
template <typename IT, int NF64>
__global__ void __launch_bounds__(256) layer_apply_kernel_f32x2(c128* __restrict__ psi, const c128* __restrict__ hi,
                                                                const c128* __restrict__ lo,
                                                                const df::cf2* __restrict__ his,
                                                                const df::cf2* __restrict__ los, uint64_t n64,
                                                                uint64_t lo_size64, uint32_t lo_log2) {
  static_assert(NF64 >= 0 && NF64 < DU, "at least one float-float element per step");
  const IT n = (IT)n64, lo_size = (IT)lo_size64, step = (IT)gridDim.x * blockDim.x * DU;
  for (IT base = (IT)blockIdx.x * blockDim.x * DU + threadIdx.x; base < n; base += step) {
    c128 x[DU], ad[NF64 > 0 ? NF64 : 1], bd[NF64 > 0 ? NF64 : 1];
    df::cf2 a[DU], b[DU];
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e < n) {
        IT h, l;
        hi_lo<IT>(e, lo_size, lo_log2, h, l);
        x[u] = psi[e];
        if (u < NF64) {
          ad[u < NF64 ? u : 0] = __ldg(hi + h);
          bd[u < NF64 ? u : 0] = __ldg(lo + l);
        } else {
          a[u] = his[h];
          b[u] = los[l];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < DU; ++u) {
      const IT e = base + (IT)(u * blockDim.x);
      if (e >= n) continue;
      if (u < NF64) {
        psi[e] = cmul_fused(x[u], cmul_fused(ad[u < NF64 ? u : 0], bd[u < NF64 ? u : 0]));
        continue;
      }
      const bool ok = a[u].re.h == a[u].re.h && b[u].re.h == b[u].re.h && df::in_range_state(x[u].x) &&
                      df::in_range_state(x[u].y);
      if (__all_sync(__activemask(), ok)) {
        df::acc pr, pi;
        df::cmul_acc(a[u], b[u], pr, pi);
        // the unnormalised pairs (sum, error) enter the next product as they are: its
        // TwoProduct multiplies out all four hi/lo terms, and the error part is a few
        // units in the last place of the sum
        const df::cf2 ph{{pr.s, pr.c}, {pi.s, pi.c}};
        df::acc re, im;
        df::cmul_acc(df::csplit(x[u].x, x[u].y), ph, re, im);
        psi[e] = make_double2(df::to_double(re), df::to_double(im));
      } else {
        IT h, l;
        hi_lo<IT>(e, lo_size, lo_log2, h, l);
        psi[e] = cmul_fp64_outofline(x[u], cmul_fp64_outofline(__ldg(hi + h), __ldg(lo + l)));
      }
    }
  }
}

// 32-bit indices when n plus one grid stride of DU elements per thread fits.
inline bool index32(uint64_t n, int grid) { return n + (uint64_t)grid * 256 * DU < (1ull << 32); }

// Merge the non-target axes into runs and describe them (state strides in s_in).
void other_axes(const dims_t& dims, const std::vector<uint16_t>& targets, RestDesc& out) {
  dims_t st = row_strides(dims);
  std::vector<char> is_t(dims.size(), 0);
  for (auto t : targets) is_t[t] = 1;
  dims_t md, ms;
  for (size_t i = 0; i < dims.size(); ++i) {
    if (is_t[i] || dims[i] == 1) continue;
    if (!md.empty() && i > 0 && !is_t[i - 1] && ms.back() == dims[i] * st[i]) {
      md.back() *= dims[i];
      ms.back() = st[i];
    } else {
      md.push_back(dims[i]);
      ms.push_back(st[i]);
    }
  }
  if ((int)md.size() > KMAX) throw Error(QTNH_ERR_UNSUPPORTED, "too many axes");
  out.n = (int)md.size();
  out.total = product(md);
  for (size_t i = 0; i < md.size(); ++i) fill_axis(out.ax[i], md[i], ms[i], 0);
}

void check_targets(const dims_t& dims, const std::vector<uint16_t>& targets) {
  std::vector<char> seen(dims.size(), 0);
  for (auto t : targets) {
    if (t >= dims.size()) throw Error(QTNH_ERR_OUT_OF_RANGE, "target index out of range");
    if (seen[t]++) throw Error(QTNH_ERR_INVALID_ARGUMENT, "target index repeated");
  }
}

}  // namespace

void apply_gate_device(void* state, const dims_t& dims, const std::vector<uint16_t>& targets, const void* gate,
                       void* stream) {
  check_targets(dims, targets);
  uint64_t D = 1;
  for (auto t : targets) D *= dims[t];
  if (product(dims) == 0) return;
  if (arithmetic_mode() == QTNH_ARITH_BF16X6 && apply_gate_tc_single(state, dims, targets, gate, stream)) return;
  GateParams p;
  other_axes(dims, targets, p.other);
  dims_t st = row_strides(dims);
  p.nins = -1;
  {
    bool pow2 = targets.size() <= 8;
    for (auto d : dims) pow2 = pow2 && log2_or_none(d) != 0xFFFFFFFFu;
    if (pow2) {
      std::vector<uint16_t> ts(targets);
      std::sort(ts.begin(), ts.end(), [&](uint16_t a, uint16_t b) { return st[a] < st[b]; });
      p.nins = (int)ts.size();
      for (size_t j = 0; j < ts.size(); ++j) {
        p.ins_pos[j] = log2_or_none(st[ts[j]]);
        p.ins_width[j] = log2_or_none(dims[ts[j]]);
      }
    }
  }
  for (uint64_t c = 0; c < D && D <= GATE_MAX_D; ++c) {
    uint64_t rem = c, off = 0;
    for (int j = (int)targets.size() - 1; j >= 0; --j) {
      uint64_t d = rem % dims[targets[j]];
      rem /= dims[targets[j]];
      off += d * st[targets[j]];
    }
    p.off[c] = (int64_t)off;
  }
  cudaStream_t s = (cudaStream_t)stream;
  c128* psi = static_cast<c128*>(state);
  const c128* g = static_cast<const c128*>(gate);
  int grid = grid_for((p.other.total + 255) / 256, 8);
  const bool ff = arithmetic_mode() != QTNH_ARITH_FP64;
#define QTNH_GATE_CASE(DD)                                                  \
  case DD:                                                                  \
    if (ff) gate_kernel_f32x2<DD><<<grid, 256, 0, s>>>(psi, g, p);          \
    else gate_kernel<DD><<<grid, 256, 0, s>>>(psi, g, p);                   \
    break;
#define QTNH_GATE_COOP_CASE(DD)                                                            \
  case DD: {                                                                               \
    const int cg = grid_for((p.other.total + 256 / DD - 1) / (256 / DD), 8);               \
    if (ff) gate_coop_kernel<DD, true><<<cg, 256, 0, s>>>(psi, g, p);                      \
    else gate_coop_kernel<DD, false><<<cg, 256, 0, s>>>(psi, g, p);                        \
    break;                                                                                 \
  }
  switch (D) {
    QTNH_GATE_CASE(1)
    QTNH_GATE_CASE(2)
    QTNH_GATE_CASE(3)
    QTNH_GATE_CASE(4)
    QTNH_GATE_COOP_CASE(8)
    QTNH_GATE_COOP_CASE(9)
    QTNH_GATE_COOP_CASE(16)
    default: {
      // other sizes: the general kernel out of a copy of the state
      GateAnyParams a;
      a.D = D;
      a.k = (int)targets.size();
      for (size_t j = 0; j < targets.size(); ++j) {
        a.tdim[j] = dims[targets[j]];
        a.tstr[j] = (int64_t)st[targets[j]];
      }
      const uint64_t n = product(dims);
      c128* copy = static_cast<c128*>(workspace_alloc(n * sizeof(c128), stream));
      cudaError_t e = cudaMemcpyAsync(copy, psi, n * sizeof(c128), cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess) {
        gate_kernel_any<<<grid_for((p.other.total * D + 255) / 256, 8), 256, 0, s>>>(psi, copy, g, p, a);
        e = cudaGetLastError();
      }
      workspace_free(copy, stream);
      check_cuda(e, "gate_kernel_any launch");
      break;
    }
  }
#undef QTNH_GATE_CASE
#undef QTNH_GATE_COOP_CASE
  count_launch();
  check_cuda(cudaGetLastError(), "gate_kernel launch");
}

void apply_diag_device(void* state, const dims_t& dims, const std::vector<uint16_t>& targets, const void* diag,
                       void* stream) {
  check_targets(dims, targets);
  if (targets.size() > 8) throw Error(QTNH_ERR_UNSUPPORTED, "diagonal over more than 8 indices");
  uint64_t n = product(dims);
  if (n == 0) return;
  DiagParams p;
  p.n = n;
  p.k = (int)targets.size();
  dims_t st = row_strides(dims);
  uint64_t m = 1;
  for (int j = p.k - 1; j >= 0; --j) {
    p.dim[j] = dims[targets[j]];
    p.stride[j] = st[targets[j]];
    p.dim_log2[j] = log2_or_none(p.dim[j]);
    p.stride_log2[j] = log2_or_none(p.stride[j]);
    p.mult[j] = m;
    m *= p.dim[j];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int grid = grid_for((n + 256 * DU - 1) / (256 * DU), 8);
  c128* st_ = static_cast<c128*>(state);
  const c128* d_ = static_cast<const c128*>(diag);
  const bool ff = arithmetic_mode() != QTNH_ARITH_FP64;
  if (ff) {
    // the diagonal's entries split once into float pairs
    df::cf2* ds = static_cast<df::cf2*>(workspace_alloc(m * sizeof(df::cf2), stream));
    table_split_kernel<<<grid_for((m + 255) / 256, 4), 256, 0, s>>>(d_, ds, m);
    const bool i32 = index32(n, grid);
    if (arithmetic_mode() == QTNH_ARITH_F32X2) {
      if (i32) diag_kernel_f32x2<uint32_t, 0><<<grid, 256, 0, s>>>(st_, d_, ds, p);
      else diag_kernel_f32x2<uint64_t, 0><<<grid, 256, 0, s>>>(st_, d_, ds, p);
    } else {
      if (i32) diag_kernel_f32x2<uint32_t, DIAG_FP64_SLOTS><<<grid, 256, 0, s>>>(st_, d_, ds, p);
      else diag_kernel_f32x2<uint64_t, DIAG_FP64_SLOTS><<<grid, 256, 0, s>>>(st_, d_, ds, p);
    }
    count_launch(2);
    const cudaError_t e = cudaGetLastError();
    workspace_free(ds, stream);
    check_cuda(e, "diag_kernel launch");
    return;
  }
  if (index32(n, grid)) diag_kernel<uint32_t><<<grid, 256, 0, s>>>(st_, d_, p);
  else diag_kernel<uint64_t><<<grid, 256, 0, s>>>(st_, d_, p);
  count_launch();
  check_cuda(cudaGetLastError(), "diag_kernel launch");
}

void apply_diag_layer_device(void* state, const dims_t& dims, const std::vector<uint16_t>& axes, const void* factors,
                             void* stream) {
  check_targets(dims, axes);
  if (axes.size() > (size_t)LAYER_MAX_FACTORS) throw Error(QTNH_ERR_UNSUPPORTED, "too many diagonal factors");
  const uint64_t n = product(dims);
  if (n == 0 || axes.empty()) return;
  // Split the indices: trailing ones whose extent product is at most 4096 form the
  // low table, the rest the high table.
  const int r = (int)dims.size();
  int split = r;
  uint64_t lo_size = 1;
  while (split > 0 && lo_size * dims[split - 1] <= 4096) lo_size *= dims[--split];
  const uint64_t hi_size = n / lo_size;
  dims_t st = row_strides(dims);
  std::vector<uint64_t> foff(axes.size());
  for (size_t f = 0, o = 0; f < axes.size(); ++f) foff[f] = o, o += dims[axes[f]];

  std::unique_ptr<LayerTableParams> lo(new LayerTableParams()), hi(new LayerTableParams());
  lo->size = lo_size;
  hi->size = hi_size;
  for (size_t f = 0; f < axes.size(); ++f) {
    int a = axes[f];
    LayerTableParams& t = (a >= split) ? *lo : *hi;
    // Stride of axis a inside the table index: the state stride divided by lo_size for
    // the high table (the high index is e / lo_size).
    t.f_stride[t.nf] = (a >= split) ? st[a] : st[a] / lo_size;
    t.f_dim[t.nf] = dims[a];
    t.f_off[t.nf] = foff[f];
    ++t.nf;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const bool ff = arithmetic_mode() != QTNH_ARITH_FP64;
  const size_t tab = lo_size + hi_size;
  c128* tables = static_cast<c128*>(workspace_alloc(tab * sizeof(c128) * (ff ? 2 : 1), stream));
  const c128* fac = static_cast<const c128*>(factors);
  layer_table_kernel<<<grid_for((lo_size + 255) / 256, 4), 256, 0, s>>>(fac, tables, *lo);
  layer_table_kernel<<<grid_for((hi_size + 255) / 256, 4), 256, 0, s>>>(fac, tables + lo_size, *hi);
  const int grid = grid_for((n + 256 * DU - 1) / (256 * DU), 8);
  const bool i32 = index32(n, grid);
  c128* st_ = static_cast<c128*>(state);
  const uint32_t lo_log2 = log2_or_none(lo_size);
  if (ff) {
    df::cf2* split_tab = reinterpret_cast<df::cf2*>(tables + tab);
    table_split_kernel<<<grid_for((tab + 255) / 256, 4), 256, 0, s>>>(tables, split_tab, tab);
    const c128* hi_t = tables + lo_size;
    const df::cf2* his = split_tab + lo_size;
    if (arithmetic_mode() == QTNH_ARITH_F32X2) {
      if (i32)
        layer_apply_kernel_f32x2<uint32_t, 0><<<grid, 256, 0, s>>>(st_, hi_t, tables, his, split_tab, n, lo_size, lo_log2);
      else
        layer_apply_kernel_f32x2<uint64_t, 0><<<grid, 256, 0, s>>>(st_, hi_t, tables, his, split_tab, n, lo_size, lo_log2);
    } else {
      if (i32)
        layer_apply_kernel_f32x2<uint32_t, LAYER_FP64_SLOTS><<<grid, 256, 0, s>>>(st_, hi_t, tables, his, split_tab, n,
                                                                                lo_size, lo_log2);
      else
        layer_apply_kernel_f32x2<uint64_t, LAYER_FP64_SLOTS><<<grid, 256, 0, s>>>(st_, hi_t, tables, his, split_tab, n,
                                                                                lo_size, lo_log2);
    }
    count_launch(4);
  } else {
    if (i32)
      layer_apply_kernel<uint32_t><<<grid, 256, 0, s>>>(st_, tables + lo_size, tables, n, lo_size, lo_log2);
    else
      layer_apply_kernel<uint64_t><<<grid, 256, 0, s>>>(st_, tables + lo_size, tables, n, lo_size, lo_log2);
    count_launch(3);
  }
  cudaError_t e = cudaGetLastError();
  workspace_free(tables, stream);
  check_cuda(e, "diagonal layer launch");
}

}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" {

int qtnh_apply_gate(void* state, int32_t rank, const uint64_t* dims, int32_t k, const uint16_t* targets,
                    const void* gate, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank < 0 || rank > QTNH_MAX_RANK || k < 0 || k > rank) throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    apply_gate_device(state, dims_t(dims, dims + rank), std::vector<uint16_t>(targets, targets + k), gate, stream);
    return QTNH_OK;
  });
}

int qtnh_apply_gate_layer(void* state, int32_t rank, const uint64_t* dims, int32_t ngates, const int32_t* gate_k,
                          const uint16_t* targets, const void* const* gates, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank < 0 || rank > QTNH_MAX_RANK || ngates < 0) throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    dims_t d(dims, dims + rank);
    std::vector<std::vector<uint16_t>> tl((size_t)ngates);
    size_t o = 0;
    for (int32_t g = 0; g < ngates; ++g) {
      if (gate_k[g] < 0 || gate_k[g] > rank) throw Error(QTNH_ERR_INVALID_ARGUMENT, "gate arity out of range");
      tl[g].assign(targets + o, targets + o + gate_k[g]);
      o += (size_t)gate_k[g];
    }
    if (arithmetic_mode() == QTNH_ARITH_BF16X6) {
      apply_gate_layer_tc(state, d, tl, std::vector<const void*>(gates, gates + ngates), stream);
    } else {
      for (int32_t g = 0; g < ngates; ++g) apply_gate_device(state, d, tl[g], gates[g], stream);
    }
    return QTNH_OK;
  });
}

int qtnh_apply_gate_runs(void* state, void* scratch, int32_t rank, const uint64_t* dims, int32_t nruns,
                         const int32_t* run_ngates, const int32_t* gate_k, const uint16_t* targets,
                         const void* const* gates, const uint16_t* ptups, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank < 0 || rank > QTNH_MAX_RANK || nruns < 1) throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    if (nruns > 1 && (!scratch || scratch == state)) throw Error(QTNH_ERR_INVALID_ARGUMENT, "no separate scratch buffer");
    // everything is checked before the first launch
    dims_t d(dims, dims + rank);
    dims_t dr = d;  // the dims when run r starts
    std::vector<GateRun> runs((size_t)nruns);
    size_t o = 0, gi = 0;
    for (int32_t r = 0; r < nruns; ++r) {
      if (run_ngates[r] < 0) throw Error(QTNH_ERR_INVALID_ARGUMENT, "negative gate count");
      for (int32_t g = 0; g < run_ngates[r]; ++g, ++gi) {
        const int32_t k = gate_k[gi];
        if (k < 0 || k > rank) throw Error(QTNH_ERR_INVALID_ARGUMENT, "gate arity out of range");
        std::vector<uint16_t> t(targets + o, targets + o + k);
        check_targets(dr, t);
        runs[r].targets.push_back(std::move(t));
        runs[r].gates.push_back(gates[gi]);
        o += (size_t)k;
      }
      if (r + 1 < nruns) {
        const uint16_t* pt = ptups + (size_t)r * (size_t)rank;
        std::vector<uint8_t> seen((size_t)rank, 0);
        for (int32_t i = 0; i < rank; ++i) {
          if (pt[i] >= rank || seen[pt[i]]) throw Error(QTNH_ERR_INVALID_ARGUMENT, "permutation tuple is not a permutation");
          seen[pt[i]] = 1;
        }
        runs[r].ptup.assign(pt, pt + rank);
        dims_t nd(dr.size());
        for (size_t i = 0; i < dr.size(); ++i) nd[pt[i]] = dr[i];
        dr = nd;
      }
    }
    if (arithmetic_mode() == QTNH_ARITH_BF16X6) {
      apply_gate_runs_tc(state, scratch, d, runs, stream);
    } else {
      void* cur = state;
      void* oth = scratch;
      for (const GateRun& run : runs) {
        for (size_t g = 0; g < run.gates.size(); ++g) apply_gate_device(cur, d, run.targets[g], run.gates[g], stream);
        if (!run.ptup.empty()) {
          permute_device(cur, oth, d, run.ptup, stream);
          dims_t nd(d.size());
          for (size_t i = 0; i < d.size(); ++i) nd[run.ptup[i]] = d[i];
          d = nd;
          std::swap(cur, oth);
        }
      }
    }
    return QTNH_OK;
  });
}

int qtnh_gate_timing(int enable, double* ms, uint64_t* launches) {
  return QTNH_API([&]() -> int {
    double t = 0;
    uint64_t n = 0;
    take_pass_times(t, n);
    if (ms) *ms = t;
    if (launches) *launches = n;
    set_pass_timing(enable != 0);
    return QTNH_OK;
  });
}

int qtnh_apply_diag(void* state, int32_t rank, const uint64_t* dims, int32_t k, const uint16_t* targets,
                    const void* diag, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank < 0 || rank > QTNH_MAX_RANK || k < 0 || k > rank) throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    apply_diag_device(state, dims_t(dims, dims + rank), std::vector<uint16_t>(targets, targets + k), diag, stream);
    return QTNH_OK;
  });
}

int qtnh_symm_diag_product(const void* gate, int32_t k, const uint64_t* tdims, int32_t p, const void* diag,
                           void* out, void* stream) {
  return QTNH_API([&]() -> int {
    if (k < 1 || k > QTNH_MAX_RANK || p < 0 || p >= k) throw Error(QTNH_ERR_INVALID_ARGUMENT, "target out of range");
    if (!gate || !diag || !out || !tdims) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null pointer");
    uint64_t D = 1, stride = 1;
    for (int32_t j = 0; j < k; ++j) {
      if (tdims[j] == 0) throw Error(QTNH_ERR_INVALID_ARGUMENT, "zero dimension");
      D *= tdims[j];
      if (j > p) stride *= tdims[j];
    }
    const uint64_t n = D * D;
    diag_product_kernel<<<grid_for((n + 255) / 256, 1), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const c128*>(gate), static_cast<const c128*>(diag), static_cast<c128*>(out), n, D, stride, tdims[p]);
    count_launch();
    check_cuda(cudaGetLastError(), "diag product launch");
    return QTNH_OK;
  });
}

int qtnh_apply_diag_layer(void* state, int32_t rank, const uint64_t* dims, int32_t nfactors, const uint16_t* axes,
                          const void* factors, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank < 0 || rank > QTNH_MAX_RANK || nfactors < 0) throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    apply_diag_layer_device(state, dims_t(dims, dims + rank), std::vector<uint16_t>(axes, axes + nfactors), factors,
                            stream);
    return QTNH_OK;
  });
}

}  // extern "C"
