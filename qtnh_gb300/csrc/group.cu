// Grouped operations on many independent resident states, for a request loop that
// advances all admitted requests together: one call applies the next layer of every
// given state (its two-qubit SymmTensor gates slot by slot -- consecutive disjoint gates
// as one pass of the pair kernel --, its phase DiagTensor layer,
// its SwapTensor exchange) as a few grouped launches (group_kernels.cuh), in plain
// complex128 (FP64 arithmetic) or mixed complex64 (gates in exact fixed point, phases in
// FP32 with split tables);
// plus FP64 renormalisation, amplitude gathers, and the 4-qubit reduced density matrix
// as a contracted-index sum in FP64 (rho = sum over the other indices of psi psi^*, the
// contraction of the state with its conjugate, src/tensor/contract.cpp:12-201).

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <complex>
#include <vector>

#include "group_kernels.cuh"

namespace qtnh_impl {
namespace {

constexpr uint64_t G_GATE_CHUNK = 1024;  // groups per work item
constexpr uint64_t G_PAIR_CHUNK = 256;   // 16-amplitude groups per work item of the pair kernel
constexpr uint64_t G_CHUNK = 4096;       // amplitudes (pairs) per work item
constexpr uint16_t NO_SWAP = 0xFFFF;

// Host vectors packed into one stream-ordered device block.
struct Upload {
  std::vector<unsigned char> host;
  size_t add(const void* p, size_t bytes) {
    const size_t off = (host.size() + 255) / 256 * 256;
    host.resize(off + bytes);
    if (bytes) memcpy(host.data() + off, p, bytes);
    return off;
  }
  unsigned char* dev = nullptr;
  void send(cudaStream_t s) {
    if (host.empty()) return;
    dev = static_cast<unsigned char*>(workspace_alloc(host.size(), s));
    check_cuda(cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, s), "group upload");
  }
  void release(cudaStream_t s) { workspace_free(dev, s); }
};

int grid_items(uint64_t total, int threads) {
  const int per_sm = std::max(1, 2048 / threads);
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(total, (uint64_t)sm_count() * per_sm));
}

template <typename Task>
uint64_t chunk_offsets(const std::vector<Task>&, const std::vector<uint64_t>& units, uint64_t chunk,
                       std::vector<uint64_t>& cb) {
  cb.resize(units.size());
  uint64_t acc = 0;
  for (size_t i = 0; i < units.size(); ++i) {
    cb[i] = acc;
    acc += (units[i] + chunk - 1) / chunk;
  }
  return acc;
}

template <typename T>
T from_complex(std::complex<double> z);
template <>
float2 from_complex<float2>(std::complex<double> z) {
  return make_float2((float)z.real(), (float)z.imag());
}
template <>
double2 from_complex<double2>(std::complex<double> z) {
  return make_double2(z.real(), z.imag());
}

template <typename T>
void group_layer(int32_t ns, void* const* states, const int32_t* nq, const int32_t* ngates, const uint16_t* pairs,
                 const std::complex<double>* els, const uint8_t* has_ph, const double* phases, const uint16_t* swaps,
                 cudaStream_t s) {
  constexpr int GW = grp::Cx<T>::GATE_WORDS;
  // gate table, in state order then gate order
  std::vector<T> table;
  std::vector<size_t> first_gate(ns), first_pair(ns);
  size_t ng = 0;
  for (int32_t i = 0; i < ns; ++i) {
    if (ngates[i] < 0 || 2 * ngates[i] > nq[i]) throw Error(QTNH_ERR_INVALID_ARGUMENT, "gate count out of range");
    first_gate[i] = ng;
    ng += (size_t)ngates[i];
  }
  table.resize(ng * GW);
  for (size_t g = 0; g < ng; ++g)
    for (int o = 0; o < 4; ++o)
      for (int in = 0; in < 4; ++in) {
        const std::complex<double> u = els[g * 16 + in * 4 + o];  // els[in * 4 + out] = U[out][in]
        const T hi = from_complex<T>(u);
        table[g * GW + o * 4 + in] = hi;
        if (GW == 32) table[g * GW + 16 + o * 4 + in] = from_complex<T>(u - std::complex<double>(hi.x, hi.y));
      }
  Upload up;
  const size_t gate_off = up.add(table.data(), table.size() * sizeof(T));
  // complex64: the exact fixed-point gate form (group_kernels.cuh)
  constexpr bool fx = GW == 32;
  size_t fx_off = 0;
  if (fx) {
    std::vector<grp::FxGate> fxt(ng);
    for (size_t g = 0; g < ng; ++g) {
      std::complex<double> U[16];
      for (int o = 0; o < 4; ++o)
        for (int in = 0; in < 4; ++in) U[o * 4 + in] = els[g * 16 + in * 4 + o];
      fxt[g] = grp::make_fx_gate(U);
    }
    fx_off = up.add(fxt.data(), fxt.size() * sizeof(grp::FxGate));
  }
  // gate items per state: consecutive disjoint gates paired; slot k holds the k-th item
  // of every state that has one (pairs and single gates in two launches)
  struct RoundRef {
    int kind;
    size_t tasks, cbeg;
    uint32_t ntasks;
    uint64_t total;
  };
  std::vector<RoundRef> rounds;
  std::vector<std::vector<std::pair<int, int>>> items(ns);  // (gate, second gate or -1)
  size_t nslots = 0;
  for (int32_t i = 0; i < ns; ++i) {
    for (int k = 0; k < ngates[i]; ++k) {
      const uint16_t qa = pairs[2 * (first_gate[i] + k)], qb = pairs[2 * (first_gate[i] + k) + 1];
      if (qa >= (uint32_t)nq[i] || qb >= (uint32_t)nq[i] || qa == qb)
        throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid gate qubits");
    }
    for (int k = 0; k < ngates[i];) {
      const uint16_t* x = pairs + 2 * (first_gate[i] + k);
      if (k + 1 < ngates[i]) {
        const uint16_t* y = x + 2;
        if (x[0] != y[0] && x[0] != y[1] && x[1] != y[0] && x[1] != y[1]) {
          items[i].emplace_back(k, k + 1);
          k += 2;
          continue;
        }
      }
      items[i].emplace_back(k, -1);
      k += 1;
    }
    nslots = std::max(nslots, items[i].size());
  }
  for (size_t k = 0; k < nslots; ++k) {
    std::vector<grp::PairTask> tp;
    std::vector<grp::GateTask> tg;
    std::vector<uint64_t> up_, ug, cbp, cbg;
    for (int32_t i = 0; i < ns; ++i) {
      if (k >= items[i].size()) continue;
      const int ga = items[i][k].first, gb = items[i][k].second;
      const uint32_t n = (uint32_t)nq[i];
      const uint16_t* x = pairs + 2 * (first_gate[i] + ga);
      if (gb >= 0) {
        const uint16_t* y = pairs + 2 * (first_gate[i] + gb);
        tp.push_back({states[i], n, n - 1 - x[0], n - 1 - x[1], n - 1 - y[0], n - 1 - y[1],
                      (uint32_t)(first_gate[i] + ga), (uint32_t)(first_gate[i] + gb)});
        up_.push_back(1ull << (n - 4));
      } else {
        tg.push_back({states[i], n, n - 1 - x[0], n - 1 - x[1], (uint32_t)(first_gate[i] + ga)});
        ug.push_back(1ull << (n - 2));
      }
    }
    if (!tp.empty()) {
      const uint64_t total = chunk_offsets(tp, up_, G_PAIR_CHUNK, cbp);
      rounds.push_back({grp::PAIR, up.add(tp.data(), tp.size() * sizeof(tp[0])), up.add(cbp.data(), cbp.size() * 8),
                        (uint32_t)tp.size(), total});
    }
    if (!tg.empty()) {
      const uint64_t total = chunk_offsets(tg, ug, G_GATE_CHUNK, cbg);
      rounds.push_back({grp::GATE, up.add(tg.data(), tg.size() * sizeof(tg[0])), up.add(cbg.data(), cbg.size() * 8),
                        (uint32_t)tg.size(), total});
    }
  }
  // phase round
  size_t tab_off = 0;
  {
    std::vector<T> tabs;
    std::vector<grp::PhaseTask> t;
    std::vector<uint64_t> u, cb;
    size_t ph = 0;
    for (int32_t i = 0; i < ns; ++i) {
      if (!has_ph || !has_ph[i]) continue;
      const uint32_t n = (uint32_t)nq[i], split = std::min<uint32_t>(n, 11);
      t.push_back({states[i], (uint64_t)tabs.size(), n, split});
      for (int part = 0; part < 2; ++part) {
        const uint32_t nbits = part ? n - split : split, shift = part ? split : 0;
        for (uint64_t v = 0; v < (1ull << nbits); ++v) {
          double a = 0;
          for (uint32_t j = 0; j < nbits; ++j)
            if ((v >> j) & 1) a += phases[ph + (n - 1 - (j + shift))];
          tabs.push_back(from_complex<T>(std::polar(1.0, a)));
        }
      }
      ph += n;
      u.push_back(1ull << n);
    }
    if (!t.empty()) {
      tab_off = up.add(tabs.data(), tabs.size() * sizeof(T));
      const uint64_t total = chunk_offsets(t, u, G_CHUNK, cb);
      rounds.push_back({grp::PHASE, up.add(t.data(), t.size() * sizeof(t[0])), up.add(cb.data(), cb.size() * 8),
                        (uint32_t)t.size(), total});
    }
  }
  // swap round
  {
    std::vector<grp::SwapTask> t;
    std::vector<uint64_t> u, cb;
    for (int32_t i = 0; i < ns; ++i) {
      if (!swaps || swaps[2 * i] == NO_SWAP) continue;
      const uint16_t qa = swaps[2 * i], qb = swaps[2 * i + 1];
      if (qa >= (uint32_t)nq[i] || qb >= (uint32_t)nq[i] || qa == qb) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid swap");
      t.push_back({states[i], (uint32_t)nq[i], (uint32_t)(nq[i] - 1 - qa), (uint32_t)(nq[i] - 1 - qb)});
      u.push_back(1ull << (nq[i] - 2));
    }
    if (!t.empty()) {
      const uint64_t total = chunk_offsets(t, u, G_CHUNK, cb);
      rounds.push_back({grp::SWAP, up.add(t.data(), t.size() * sizeof(t[0])), up.add(cb.data(), cb.size() * 8),
                        (uint32_t)t.size(), total});
    }
  }
  up.send(s);
  // complex128 with QTNH_BATCH_GATES=f32x2: gates in float-float (the plain method's values
  // at FP32 speed)
  const char* genv = std::getenv("QTNH_BATCH_GATES");
  const bool ff = !fx && genv && std::strcmp(genv, "f32x2") == 0;
  try {
    for (auto& r : rounds) {
      const uint64_t* cb = reinterpret_cast<const uint64_t*>(up.dev + r.cbeg);
      const grp::FxGate* fxg = reinterpret_cast<const grp::FxGate*>(up.dev + fx_off);
      if (ff && r.kind == grp::PAIR)
        grp::ff_pair_kernel<256><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::PairTask*>(up.dev + r.tasks), cb, r.ntasks, r.total,
            reinterpret_cast<const double2*>(up.dev + gate_off), G_PAIR_CHUNK);
      else if (ff && r.kind == grp::GATE)
        grp::ff_gate_kernel<256><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::GateTask*>(up.dev + r.tasks), cb, r.ntasks, r.total,
            reinterpret_cast<const double2*>(up.dev + gate_off), G_GATE_CHUNK);
      else if (fx && r.kind == grp::PAIR)
        grp::fx_pair_kernel<256><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::PairTask*>(up.dev + r.tasks), cb, r.ntasks, r.total, fxg, G_PAIR_CHUNK);
      else if (fx && r.kind == grp::GATE)
        grp::fx_gate_kernel<256><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::GateTask*>(up.dev + r.tasks), cb, r.ntasks, r.total, fxg, G_GATE_CHUNK);
      else if (r.kind == grp::PAIR)
        grp::pair_kernel<T, 256><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::PairTask*>(up.dev + r.tasks), cb, r.ntasks, r.total,
            reinterpret_cast<const T*>(up.dev + gate_off), G_PAIR_CHUNK);
      else if (r.kind == grp::GATE)
        grp::gate_kernel<T, 256><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::GateTask*>(up.dev + r.tasks), cb, r.ntasks, r.total,
            reinterpret_cast<const T*>(up.dev + gate_off), G_GATE_CHUNK);
      else if (r.kind == grp::PHASE)
        grp::phase_kernel<T><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::PhaseTask*>(up.dev + r.tasks), cb, r.ntasks, r.total,
            reinterpret_cast<const T*>(up.dev + tab_off), G_CHUNK);
      else
        grp::swap_kernel<T><<<grid_items(r.total, 256), 256, 0, s>>>(
            reinterpret_cast<const grp::SwapTask*>(up.dev + r.tasks), cb, r.ntasks, r.total, G_CHUNK);
      count_launch();
    }
    check_cuda(cudaGetLastError(), "grouped layer launch");
  } catch (...) {
    up.release(s);
    throw;
  }
  up.release(s);
}

template <typename T>
void group_renorm(int32_t ns, void* const* states, const int32_t* nq, cudaStream_t s) {
  std::vector<grp::NormTask> t;
  std::vector<uint64_t> u, cb;
  for (int32_t i = 0; i < ns; ++i) {
    t.push_back({states[i], (uint32_t)nq[i], (uint32_t)i});
    u.push_back(1ull << nq[i]);
  }
  const uint64_t total = chunk_offsets(t, u, G_CHUNK, cb);
  Upload up;
  const size_t to = up.add(t.data(), t.size() * sizeof(t[0])), co = up.add(cb.data(), cb.size() * 8);
  std::vector<double> zeros(ns, 0.0);
  const size_t no = up.add(zeros.data(), zeros.size() * sizeof(double));
  up.send(s);
  double* norms = reinterpret_cast<double*>(up.dev + no);
  const auto* tasks = reinterpret_cast<const grp::NormTask*>(up.dev + to);
  const auto* cbeg = reinterpret_cast<const uint64_t*>(up.dev + co);
  grp::norm_kernel<T><<<grid_items(total, 256), 256, 0, s>>>(tasks, cbeg, (uint32_t)ns, total, G_CHUNK, norms);
  grp::scale_kernel<T><<<grid_items(total, 256), 256, 0, s>>>(tasks, cbeg, (uint32_t)ns, total, G_CHUNK, norms);
  count_launch(2);
  const cudaError_t e = cudaGetLastError();
  up.release(s);
  check_cuda(e, "grouped renormalisation");
}

// rho[a][b] = sum_r psi[a, r] psi[b, r]^* over the indices r of the other qubits, in
// FP64; a, b = values of qubits (q0 q1 q2 q3), q0 most significant. Each block stages
// 16 x RCH amplitudes in shared memory, thread (a, b) accumulates its entry, and the
// blocks' partial sums are added atomically.
constexpr int RDM_RCH = 64;

template <typename T>
__global__ void __launch_bounds__(256) rdm4_kernel(const T* __restrict__ psi, uint64_t R, uint4 qbits, uint4 sorted,
                                                   double* __restrict__ rho) {
  __shared__ double2 M[16][RDM_RCH + 1];
  const int tid = threadIdx.x, a = tid >> 4, b = tid & 15;
  const uint32_t qb[4] = {qbits.x, qbits.y, qbits.z, qbits.w};
  const uint32_t sb[4] = {sorted.x, sorted.y, sorted.z, sorted.w};
  double re = 0, im = 0;
  const uint64_t nchunks = (R + RDM_RCH - 1) / RDM_RCH;
  for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    for (int e = tid; e < 16 * RDM_RCH; e += 256) {
      const int row = e / RDM_RCH, rr = e % RDM_RCH;
      const uint64_t r = c * RDM_RCH + rr;
      double2 v = make_double2(0.0, 0.0);
      if (r < R) {
        uint64_t x = r;
#pragma unroll
        for (int k = 0; k < 4; ++k) x = grp::insert_zero(x, sb[k]);
#pragma unroll
        for (int k = 0; k < 4; ++k) x |= (uint64_t)((row >> (3 - k)) & 1) << qb[k];
        const T p = psi[x];
        v = make_double2((double)p.x, (double)p.y);
      }
      M[row][rr] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int rr = 0; rr < RDM_RCH; ++rr) {
      const double2 x = M[a][rr], y = M[b][rr];
      re = fma(x.x, y.x, re);
      re = fma(x.y, y.y, re);
      im = fma(x.y, y.x, im);
      im = fma(-x.x, y.y, im);
    }
    __syncthreads();
  }
  atomicAdd(&rho[2 * tid], re);
  atomicAdd(&rho[2 * tid + 1], im);
}

template <typename T>
__global__ void convert_kernel(const void* __restrict__ in, void* __restrict__ out, uint64_t n, int to_c64) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    if (to_c64) {
      const double2 v = static_cast<const double2*>(in)[i];
      static_cast<float2*>(out)[i] = make_float2((float)v.x, (float)v.y);
    } else {
      const float2 v = static_cast<const float2*>(in)[i];
      static_cast<double2*>(out)[i] = make_double2((double)v.x, (double)v.y);
    }
  }
}

void check_precision(int32_t p) {
  if (p != QTNH_STATE_C128 && p != QTNH_STATE_C64) throw Error(QTNH_ERR_INVALID_ARGUMENT, "unknown state precision");
}

}  // namespace
}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" {

int qtnh_group_layer(int32_t precision, int32_t nstates, void* const* states, const int32_t* nqubits,
                     const int32_t* ngates, const uint16_t* pairs, const void* gates_c128, const uint8_t* has_phases,
                     const double* phases, const uint16_t* swaps, void* stream) {
  return QTNH_API([&]() -> int {
    check_precision(precision);
    if (nstates < 0 || (nstates && (!states || !nqubits || !ngates))) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid group");
    for (int32_t i = 0; i < nstates; ++i)
      if (nqubits[i] < 2 || nqubits[i] > 40) throw Error(QTNH_ERR_INVALID_ARGUMENT, "qubit count out of range");
    if (nstates == 0) return QTNH_OK;
    const auto* els = static_cast<const std::complex<double>*>(gates_c128);
    if (precision == QTNH_STATE_C64)
      group_layer<float2>(nstates, states, nqubits, ngates, pairs, els, has_phases, phases, swaps, (cudaStream_t)stream);
    else
      group_layer<double2>(nstates, states, nqubits, ngates, pairs, els, has_phases, phases, swaps,
                           (cudaStream_t)stream);
    return QTNH_OK;
  });
}

int qtnh_group_renorm(int32_t precision, int32_t nstates, void* const* states, const int32_t* nqubits, void* stream) {
  return QTNH_API([&]() -> int {
    check_precision(precision);
    if (nstates <= 0) return QTNH_OK;
    for (int32_t i = 0; i < nstates; ++i)
      if (nqubits[i] < 2 || nqubits[i] > 40) throw Error(QTNH_ERR_INVALID_ARGUMENT, "qubit count out of range");
    if (precision == QTNH_STATE_C64)
      group_renorm<float2>(nstates, states, nqubits, (cudaStream_t)stream);
    else
      group_renorm<double2>(nstates, states, nqubits, (cudaStream_t)stream);
    return QTNH_OK;
  });
}

int qtnh_gather(int32_t precision, const void* state, int32_t nqubits, int32_t nidx, const uint64_t* idx,
                void* out_c128, void* stream) {
  return QTNH_API([&]() -> int {
    check_precision(precision);
    if (nidx <= 0) return QTNH_OK;
    for (int32_t i = 0; i < nidx; ++i)
      if (idx[i] >= (1ull << nqubits)) throw Error(QTNH_ERR_OUT_OF_RANGE, "amplitude index out of range");
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t* w = static_cast<uint64_t*>(workspace_alloc(nidx * sizeof(uint64_t), s));
    check_cuda(cudaMemcpyAsync(w, idx, nidx * sizeof(uint64_t), cudaMemcpyHostToDevice, s), "gather upload");
    if (precision == QTNH_STATE_C64)
      grp::gather_kernel<float2><<<grid_for((nidx + 255) / 256, 2), 256, 0, s>>>(
          static_cast<const float2*>(state), w, (uint64_t)nidx, static_cast<double2*>(out_c128));
    else
      grp::gather_kernel<double2><<<grid_for((nidx + 255) / 256, 2), 256, 0, s>>>(
          static_cast<const double2*>(state), w, (uint64_t)nidx, static_cast<double2*>(out_c128));
    count_launch();
    const cudaError_t e = cudaGetLastError();
    workspace_free(w, s);
    check_cuda(e, "gather launch");
    return QTNH_OK;
  });
}

int qtnh_rdm4(int32_t precision, const void* state, int32_t nqubits, const uint16_t* qubits, void* out_c128,
              void* stream) {
  return QTNH_API([&]() -> int {
    check_precision(precision);
    if (nqubits < 4 || nqubits > 40 || !qubits) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid reduced density matrix");
    uint32_t qb[4], sb[4];
    for (int k = 0; k < 4; ++k) {
      if (qubits[k] >= nqubits) throw Error(QTNH_ERR_OUT_OF_RANGE, "qubit out of range");
      qb[k] = (uint32_t)(nqubits - 1 - qubits[k]);
      sb[k] = qb[k];
    }
    std::sort(sb, sb + 4);
    for (int k = 1; k < 4; ++k)
      if (sb[k] == sb[k - 1]) throw Error(QTNH_ERR_INVALID_ARGUMENT, "qubit repeated");
    cudaStream_t s = (cudaStream_t)stream;
    check_cuda(cudaMemsetAsync(out_c128, 0, 256 * sizeof(double2), s), "rdm reset");
    const uint64_t R = 1ull << (nqubits - 4);
    const int grid = grid_for((R + RDM_RCH - 1) / RDM_RCH, 4);
    const uint4 q4 = make_uint4(qb[0], qb[1], qb[2], qb[3]), s4 = make_uint4(sb[0], sb[1], sb[2], sb[3]);
    if (precision == QTNH_STATE_C64)
      rdm4_kernel<float2><<<grid, 256, 0, s>>>(static_cast<const float2*>(state), R, q4, s4,
                                              static_cast<double*>(out_c128));
    else
      rdm4_kernel<double2><<<grid, 256, 0, s>>>(static_cast<const double2*>(state), R, q4, s4,
                                               static_cast<double*>(out_c128));
    count_launch();
    check_cuda(cudaGetLastError(), "rdm launch");
    return QTNH_OK;
  });
}

int qtnh_state_convert(int32_t to_precision, const void* in, void* out, uint64_t n, void* stream) {
  return QTNH_API([&]() -> int {
    check_precision(to_precision);
    convert_kernel<float2><<<grid_for((n + 255) / 256, 4), 256, 0, (cudaStream_t)stream>>>(
        in, out, n, to_precision == QTNH_STATE_C64 ? 1 : 0);
    count_launch();
    check_cuda(cudaGetLastError(), "convert launch");
    return QTNH_OK;
  });
}

}  // extern "C"
