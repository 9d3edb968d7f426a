// Batched circuits: many independent circuits of uneven qubit counts and depths, states
// resident in HBM, run as layer-synchronous rounds of grouped persistent kernels under one
// captured CUDA graph. States are complex64 (mixed precision, the default) or complex128
// (the plain method: FP64 math throughout, the same schedule).
//
// Per circuit the operations are the reference's contractions with a layered circuit:
// two-qubit SymmTensor gates (include/tensor/symm.hpp:22-45 layout, applied in place as
// by the Symm rule of src/tensor/contract.cpp:250-289), a layer of single-qubit phase
// DiagTensors, and SwapTensor qubit exchanges; every `renorm` layers the state is
// renormalised with an FP64 norm, and the circuit ends in amplitude queries returned in
// complex128.
//
// Mixed-precision arithmetic: amplitudes complex64; gates in exact fixed point
// (group_kernels.cuh: each group of amplitudes scaled to 29-bit integers at its largest
// exponent, the gate to 30-bit integers, products summed exactly in 64-bit integers,
// one rounding per output when it is converted back to complex64; QTNH_BATCH_GATES=fp32
// selects FP32 accumulation with the gate held as complex64 U_hi + U_lo instead). Phase
// layers multiply by lo/hi tables of per-qubit phase products (built in FP64, stored
// complex64). Norms: per-thread compensated FP32 sums
// (TwoSum) reduced in FP64. Plain arithmetic: complex128 amplitudes, gates and phase
// tables, FP64 fused multiply-adds.
//
// Scheduling: `compile` groups the operations of all circuits into rounds (layer L: the
// gates of each circuit's layer in order, consecutive disjoint gates paired into one pass
// over the state; the s-th gate item of every circuit for each slot s, pairs and single
// gates in two launches; then the phase layers; then the swaps; then the
// renormalisation), so every round is one launch over a task table (circuit, operand) x
// chunks; a persistent grid walks the (task, chunk) work items, finding its task by
// binary search over the tasks' chunk offsets. An autotuner times the block size and
// chunk length of the pair kernel and of the single-gate kernel on their largest rounds.
// The whole
// schedule -- state reset from the initial states, norm reset, every round, the
// queries -- is captured once as a CUDA graph and replayed by `run`.

#include <algorithm>
#include <cmath>
#include <complex>
#include <memory>
#include <string>
#include <vector>

#include "group_kernels.cuh"

struct qtnh_batch;

namespace qtnh_impl {

namespace {

using c64 = float2;
using grp::GateTask;
using grp::NormTask;
using grp::PairTask;
using grp::PhaseTask;
using grp::SwapTask;

enum RoundKind {
  R_GATE = grp::GATE,
  R_PHASE = grp::PHASE,
  R_SWAP = grp::SWAP,
  R_NORM = grp::NORM,
  R_SCALE = grp::SCALE,
  R_PAIR = grp::PAIR
};

struct Round {
  int kind;
  uint32_t ntasks = 0;
  uint64_t total = 0;       // work items (chunks)
  void* tasks = nullptr;    // device task table
  uint64_t* cbeg = nullptr; // device chunk offsets (ntasks)
  uint64_t elems_per_chunk = 0;  // amplitudes, or groups (4 amplitudes a gate, 16 a pair)
  int threads = 256;
};

using c128 = double2;

__global__ void b_to_c64_kernel(const double2* __restrict__ in, c64* __restrict__ out, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

struct Op {
  int kind;  // R_GATE, R_PHASE, R_SWAP
  int layer;
  uint16_t qa = 0, qb = 0;
  uint32_t index = 0;  // gate table index / phase entry
};

}  // namespace

}  // namespace qtnh_impl

using namespace qtnh_impl;

struct qtnh_batch {
  int32_t precision = QTNH_STATE_C64;  // QTNH_STATE_C64 (mixed) or QTNH_STATE_C128 (plain)
  std::vector<uint32_t> nq;
  std::vector<uint64_t> base;
  uint64_t total_amps = 0;
  void* psi = nullptr;   // working states
  void* psi0 = nullptr;  // initial states
  std::vector<std::vector<Op>> ops;
  std::vector<std::complex<double>> gate_host;    // 16 per gate: U[out * 4 + in]
  std::vector<std::vector<double>> phase_host;    // per phase op: n phases
  std::vector<std::pair<uint64_t, uint64_t>> queries;  // (circuit, index)
  // compiled
  std::vector<Round> rounds;
  std::vector<void*> allocations;
  void* gates = nullptr;   // c64: U_hi[16], U_lo[16] per gate; c128: U[16]
  grp::FxGate* fx_gates = nullptr;  // c64: the exact fixed-point form (used unless fp32_gates)
  bool fp32_gates = false;          // c64: FP32 gate arithmetic (QTNH_BATCH_GATES=fp32)
  bool ff_gates = false;            // c128: float-float gate arithmetic (QTNH_BATCH_GATES=f32x2)
  void* tables = nullptr;  // phase tables in the state's type
  double* norms = nullptr;
  uint64_t nnorms = 0;
  uint64_t* query_where = nullptr;
  double2* query_out = nullptr;
  int gate_threads = 256;   // single-gate rounds (chunk in 4-amplitude groups)
  uint64_t gate_chunk = 1024;
  int pair_threads = 256;   // pair rounds (chunk in 16-amplitude groups)
  uint64_t pair_chunk = 256;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t launches_per_run = 0;
  int max_layer = -1;

  ~qtnh_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : allocations) cudaFree(p);
    if (psi) cudaFree(psi);
    if (psi0) cudaFree(psi0);
    if (stream) cudaStreamDestroy(stream);
  }

  template <typename T>
  T* upload(const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    void* p = nullptr;
    check_cuda(cudaMalloc(&p, v.size() * sizeof(T)), "batch allocation");
    allocations.push_back(p);
    check_cuda(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "batch upload");
    return static_cast<T*>(p);
  }

  uint32_t bit(uint32_t c, uint16_t q) const { return nq[c] - 1 - q; }
  size_t amp_bytes() const { return precision == QTNH_STATE_C128 ? sizeof(c128) : sizeof(c64); }
  void* state_of(uint64_t c) const { return static_cast<char*>(psi) + base[c] * amp_bytes(); }

  int grid(uint64_t total, int threads) const {
    const int per_sm = std::max(1, 2048 / threads);
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(total, (uint64_t)sm_count() * per_sm));
  }

  template <typename Task>
  Round make_round(int kind, const std::vector<Task>& tasks, const std::vector<uint64_t>& units, uint64_t chunk,
                   int threads = 256) {
    Round r;
    r.kind = kind;
    r.threads = threads;
    r.ntasks = (uint32_t)tasks.size();
    r.elems_per_chunk = chunk;
    std::vector<uint64_t> cb(tasks.size());
    uint64_t acc = 0;
    for (size_t i = 0; i < tasks.size(); ++i) {
      cb[i] = acc;
      acc += (units[i] + chunk - 1) / chunk;
    }
    r.total = acc;
    r.tasks = upload(tasks);
    r.cbeg = upload(cb);
    return r;
  }

  template <typename T>
  void launch_as(const Round& r, cudaStream_t s) {
    const T* g_tab = static_cast<const T*>(gates);
    const T* p_tab = static_cast<const T*>(tables);
    const uint64_t ch = r.elems_per_chunk;
    switch (r.kind) {
      case R_GATE: {
        const auto* t = static_cast<const GateTask*>(r.tasks);
        const int g = grid(r.total, r.threads);
        if (ff_gates) {
          const double2* gd = static_cast<const double2*>(gates);
          if (r.threads == 128)
            grp::ff_gate_kernel<128><<<g, 128, 0, s>>>(t, r.cbeg, r.ntasks, r.total, gd, ch);
          else if (r.threads == 512)
            grp::ff_gate_kernel<512><<<g, 512, 0, s>>>(t, r.cbeg, r.ntasks, r.total, gd, ch);
          else
            grp::ff_gate_kernel<256><<<g, 256, 0, s>>>(t, r.cbeg, r.ntasks, r.total, gd, ch);
          break;
        }
        if (fx_gates && !fp32_gates) {
          if (r.threads == 128)
            grp::fx_gate_kernel<128><<<g, 128, 0, s>>>(t, r.cbeg, r.ntasks, r.total, fx_gates, ch);
          else if (r.threads == 512)
            grp::fx_gate_kernel<512><<<g, 512, 0, s>>>(t, r.cbeg, r.ntasks, r.total, fx_gates, ch);
          else
            grp::fx_gate_kernel<256><<<g, 256, 0, s>>>(t, r.cbeg, r.ntasks, r.total, fx_gates, ch);
          break;
        }
        if (r.threads == 128)
          grp::gate_kernel<T, 128><<<g, 128, 0, s>>>(t, r.cbeg, r.ntasks, r.total, g_tab, ch);
        else if (r.threads == 512)
          grp::gate_kernel<T, 512><<<g, 512, 0, s>>>(t, r.cbeg, r.ntasks, r.total, g_tab, ch);
        else
          grp::gate_kernel<T, 256><<<g, 256, 0, s>>>(t, r.cbeg, r.ntasks, r.total, g_tab, ch);
        break;
      }
      case R_PAIR: {
        const auto* t = static_cast<const PairTask*>(r.tasks);
        const int g = grid(r.total, r.threads);
        if (ff_gates) {
          const double2* gd = static_cast<const double2*>(gates);
          if (r.threads == 128)
            grp::ff_pair_kernel<128><<<g, 128, 0, s>>>(t, r.cbeg, r.ntasks, r.total, gd, ch);
          else if (r.threads == 512)
            grp::ff_pair_kernel<512><<<g, 512, 0, s>>>(t, r.cbeg, r.ntasks, r.total, gd, ch);
          else
            grp::ff_pair_kernel<256><<<g, 256, 0, s>>>(t, r.cbeg, r.ntasks, r.total, gd, ch);
          break;
        }
        if (fx_gates && !fp32_gates) {
          if (r.threads == 128)
            grp::fx_pair_kernel<128><<<g, 128, 0, s>>>(t, r.cbeg, r.ntasks, r.total, fx_gates, ch);
          else if (r.threads == 512)
            grp::fx_pair_kernel<512><<<g, 512, 0, s>>>(t, r.cbeg, r.ntasks, r.total, fx_gates, ch);
          else
            grp::fx_pair_kernel<256><<<g, 256, 0, s>>>(t, r.cbeg, r.ntasks, r.total, fx_gates, ch);
          break;
        }
        if (r.threads == 128)
          grp::pair_kernel<T, 128><<<g, 128, 0, s>>>(t, r.cbeg, r.ntasks, r.total, g_tab, ch);
        else if (r.threads == 512)
          grp::pair_kernel<T, 512><<<g, 512, 0, s>>>(t, r.cbeg, r.ntasks, r.total, g_tab, ch);
        else
          grp::pair_kernel<T, 256><<<g, 256, 0, s>>>(t, r.cbeg, r.ntasks, r.total, g_tab, ch);
        break;
      }
      case R_PHASE:
        grp::phase_kernel<T><<<grid(r.total, 256), 256, 0, s>>>(static_cast<const PhaseTask*>(r.tasks), r.cbeg,
                                                                r.ntasks, r.total, p_tab, r.elems_per_chunk);
        break;
      case R_SWAP:
        grp::swap_kernel<T><<<grid(r.total, 256), 256, 0, s>>>(static_cast<const SwapTask*>(r.tasks), r.cbeg,
                                                               r.ntasks, r.total, r.elems_per_chunk);
        break;
      case R_NORM:
        grp::norm_kernel<T><<<grid(r.total, 256), 256, 0, s>>>(static_cast<const NormTask*>(r.tasks), r.cbeg,
                                                               r.ntasks, r.total, r.elems_per_chunk, norms);
        break;
      case R_SCALE:
        grp::scale_kernel<T><<<grid(r.total, 256), 256, 0, s>>>(static_cast<const NormTask*>(r.tasks), r.cbeg,
                                                                r.ntasks, r.total, r.elems_per_chunk, norms);
        break;
    }
    count_launch();
  }

  void launch(const Round& r, cudaStream_t s) {
    if (precision == QTNH_STATE_C128)
      launch_as<c128>(r, s);
    else
      launch_as<c64>(r, s);
  }

  // The same round with another block size and chunk length (chunk offsets rebuilt).
  Round rechunk(const Round& r, int threads, uint64_t chunk) {
    if (r.kind == R_PAIR) {
      std::vector<PairTask> t(r.ntasks);
      check_cuda(cudaMemcpy(t.data(), r.tasks, t.size() * sizeof(PairTask), cudaMemcpyDeviceToHost), "tune");
      std::vector<uint64_t> u;
      for (auto& x : t) u.push_back(1ull << (x.n - 4));
      return make_round(R_PAIR, t, u, chunk, threads);
    }
    std::vector<GateTask> t(r.ntasks);
    check_cuda(cudaMemcpy(t.data(), r.tasks, t.size() * sizeof(GateTask), cudaMemcpyDeviceToHost), "tune");
    std::vector<uint64_t> u;
    for (auto& x : t) u.push_back(1ull << (x.n - 2));
    return make_round(R_GATE, t, u, chunk, threads);
  }

  // out[i] = psi[where[i]] as complex128
  void gather(const uint64_t* where, uint64_t nq_, double2* out, cudaStream_t s) const {
    const int g = grid_for((nq_ + 255) / 256, 4);
    if (precision == QTNH_STATE_C128)
      grp::gather_kernel<c128><<<g, 256, 0, s>>>(static_cast<const c128*>(psi), where, nq_, out);
    else
      grp::gather_kernel<c64><<<g, 256, 0, s>>>(static_cast<const c64*>(psi), where, nq_, out);
    count_launch();
  }
};

namespace {
constexpr uint64_t B_CHUNK = 4096;  // amplitudes (or pairs) per work item of the streaming rounds

qtnh_batch* checked(qtnh_batch* b) {
  if (!b) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null batch");
  return b;
}
void check_circuit(qtnh_batch* b, int32_t c) {
  if (c < 0 || (size_t)c >= b->nq.size()) throw Error(QTNH_ERR_OUT_OF_RANGE, "circuit index out of range");
  if (b->exec) throw Error(QTNH_ERR_RUNTIME, "batch already compiled");
}
}  // namespace

extern "C" {

int qtnh_batch_create_typed(qtnh_batch** out, int32_t ncircuits, const int32_t* nqubits, int32_t precision) {
  return QTNH_API([&]() -> int {
    if (!out || ncircuits <= 0 || !nqubits) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid batch arguments");
    if (precision != QTNH_STATE_C64 && precision != QTNH_STATE_C128)
      throw Error(QTNH_ERR_INVALID_ARGUMENT, "unknown state precision");
    std::unique_ptr<qtnh_batch> b(new qtnh_batch());
    b->precision = precision;
    for (int32_t c = 0; c < ncircuits; ++c) {
      if (nqubits[c] < 2 || nqubits[c] > 34) throw Error(QTNH_ERR_INVALID_ARGUMENT, "qubit count outside 2..34");
      b->nq.push_back((uint32_t)nqubits[c]);
      b->base.push_back(b->total_amps);
      b->total_amps += 1ull << nqubits[c];
    }
    b->ops.resize(ncircuits);
    check_cuda(cudaMalloc(&b->psi, b->total_amps * b->amp_bytes()), "batch states");
    check_cuda(cudaMalloc(&b->psi0, b->total_amps * b->amp_bytes()), "batch initial states");
    check_cuda(cudaMemset(b->psi0, 0, b->total_amps * b->amp_bytes()), "batch initial states");
    check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "batch stream");
    *out = b.release();
    return QTNH_OK;
  });
}

int qtnh_batch_create(qtnh_batch** out, int32_t ncircuits, const int32_t* nqubits) {
  return qtnh_batch_create_typed(out, ncircuits, nqubits, QTNH_STATE_C64);
}

int qtnh_batch_destroy(qtnh_batch* b) {
  return QTNH_API([&]() -> int {
    delete b;
    return QTNH_OK;
  });
}

int qtnh_batch_set_state(qtnh_batch* b, int32_t c, const void* psi_c128, void* stream) {
  return QTNH_API([&]() -> int {
    checked(b);
    if (c < 0 || (size_t)c >= b->nq.size()) throw Error(QTNH_ERR_OUT_OF_RANGE, "circuit index out of range");
    const uint64_t n = 1ull << b->nq[c];
    if (!psi_c128) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null state");
    void* dst = static_cast<char*>(b->psi0) + b->base[c] * b->amp_bytes();
    if (b->precision == QTNH_STATE_C128) {
      check_cuda(cudaMemcpyAsync(dst, psi_c128, n * sizeof(c128), cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
                 "batch state");
    } else {
      b_to_c64_kernel<<<grid_for((n + 255) / 256, 4), 256, 0, (cudaStream_t)stream>>>(
          static_cast<const double2*>(psi_c128), static_cast<c64*>(dst), n);
      count_launch();
      check_cuda(cudaGetLastError(), "batch state conversion");
    }
    return QTNH_OK;
  });
}

int qtnh_batch_add_gate(qtnh_batch* b, int32_t c, int32_t layer, uint16_t qa, uint16_t qb, const void* els_c128) {
  return QTNH_API([&]() -> int {
    checked(b);
    check_circuit(b, c);
    if (layer < 0 || qa >= b->nq[c] || qb >= b->nq[c] || qa == qb || !els_c128)
      throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid gate");
    // SymmTensor elements els[in * 4 + out] = U[out][in]; kept as U[out * 4 + in]
    const std::complex<double>* e = static_cast<const std::complex<double>*>(els_c128);
    const size_t g0 = b->gate_host.size();
    b->gate_host.resize(g0 + 16);
    for (int o = 0; o < 4; ++o)
      for (int i = 0; i < 4; ++i) b->gate_host[g0 + o * 4 + i] = e[i * 4 + o];
    Op op;
    op.kind = R_GATE;
    op.layer = layer;
    op.qa = qa;
    op.qb = qb;
    op.index = (uint32_t)(g0 / 16);
    b->ops[c].push_back(op);
    b->max_layer = std::max(b->max_layer, (int)layer);
    return QTNH_OK;
  });
}

int qtnh_batch_add_phases(qtnh_batch* b, int32_t c, int32_t layer, const double* phases) {
  return QTNH_API([&]() -> int {
    checked(b);
    check_circuit(b, c);
    if (layer < 0 || !phases) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid phase layer");
    Op op;
    op.kind = R_PHASE;
    op.layer = layer;
    op.index = (uint32_t)b->phase_host.size();
    b->phase_host.emplace_back(phases, phases + b->nq[c]);
    b->ops[c].push_back(op);
    b->max_layer = std::max(b->max_layer, (int)layer);
    return QTNH_OK;
  });
}

int qtnh_batch_add_swap(qtnh_batch* b, int32_t c, int32_t layer, uint16_t qa, uint16_t qb) {
  return QTNH_API([&]() -> int {
    checked(b);
    check_circuit(b, c);
    if (layer < 0 || qa >= b->nq[c] || qb >= b->nq[c] || qa == qb) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid swap");
    Op op;
    op.kind = R_SWAP;
    op.layer = layer;
    op.qa = qa;
    op.qb = qb;
    b->ops[c].push_back(op);
    b->max_layer = std::max(b->max_layer, (int)layer);
    return QTNH_OK;
  });
}

int qtnh_batch_add_queries(qtnh_batch* b, int32_t c, int32_t nq, const uint64_t* idx) {
  return QTNH_API([&]() -> int {
    checked(b);
    check_circuit(b, c);
    if (nq < 0 || (nq && !idx)) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid queries");
    for (int32_t i = 0; i < nq; ++i) {
      if (idx[i] >= (1ull << b->nq[c])) throw Error(QTNH_ERR_OUT_OF_RANGE, "query index out of range");
      b->queries.emplace_back((uint64_t)c, idx[i]);
    }
    return QTNH_OK;
  });
}

int qtnh_batch_compile(qtnh_batch* b, int32_t renorm_every, int32_t autotune) {
  return QTNH_API([&]() -> int {
    checked(b);
    if (b->exec) throw Error(QTNH_ERR_RUNTIME, "batch already compiled");
    const size_t nc = b->nq.size();
    const bool plain = b->precision == QTNH_STATE_C128;
    // gate table: complex128 U, or complex64 U_hi followed by U_lo = U - U_hi
    if (plain) {
      std::vector<c128> g;
      for (auto& u : b->gate_host) g.push_back(make_double2(u.real(), u.imag()));
      b->gates = b->upload(g);
      const char* env = std::getenv("QTNH_BATCH_GATES");
      b->ff_gates = env && std::string(env) == "f32x2";
    } else {
      std::vector<c64> g;
      for (size_t g0 = 0; g0 < b->gate_host.size(); g0 += 16) {
        for (int k = 0; k < 16; ++k)
          g.push_back(make_float2((float)b->gate_host[g0 + k].real(), (float)b->gate_host[g0 + k].imag()));
        for (int k = 0; k < 16; ++k) {
          const std::complex<double> u = b->gate_host[g0 + k];
          g.push_back(make_float2((float)(u.real() - (double)(float)u.real()),
                                  (float)(u.imag() - (double)(float)u.imag())));
        }
      }
      b->gates = b->upload(g);
      std::vector<grp::FxGate> fx;
      for (size_t g0 = 0; g0 < b->gate_host.size(); g0 += 16) fx.push_back(grp::make_fx_gate(&b->gate_host[g0]));
      b->fx_gates = b->upload(fx);
      const char* env = std::getenv("QTNH_BATCH_GATES");
      b->fp32_gates = env && std::string(env) == "fp32";
    }
    // phase tables: per phase op, lo table over the low `split` bits and hi table over the rest
    std::vector<c128> tab;
    std::vector<uint64_t> tab_off(b->phase_host.size()), tab_split(b->phase_host.size());
    std::vector<int32_t> phase_circuit(b->phase_host.size(), -1);
    for (size_t c = 0; c < nc; ++c)
      for (auto& op : b->ops[c])
        if (op.kind == R_PHASE) phase_circuit[op.index] = (int32_t)c;
    for (size_t k = 0; k < b->phase_host.size(); ++k) {
      const uint32_t n = b->nq[phase_circuit[k]];
      const uint32_t split = std::min<uint32_t>(n, 11);
      tab_off[k] = tab.size();
      tab_split[k] = split;
      // bit j of the index is qubit n - 1 - j
      for (int part = 0; part < 2; ++part) {
        const uint32_t nbits = part ? n - split : split, shift = part ? split : 0;
        for (uint64_t v = 0; v < (1ull << nbits); ++v) {
          double ph = 0;
          for (uint32_t j = 0; j < nbits; ++j)
            if ((v >> j) & 1) ph += b->phase_host[k][n - 1 - (j + shift)];
          tab.push_back(make_double2(std::cos(ph), std::sin(ph)));
        }
      }
    }
    if (plain) {
      b->tables = b->upload(tab);
    } else {
      std::vector<c64> t32;
      for (auto& x : tab) t32.push_back(make_float2((float)x.x, (float)x.y));
      b->tables = b->upload(t32);
    }
    // rounds
    const int period = renorm_every > 0 ? renorm_every : 0;
    std::vector<uint64_t> norm_slot_base;
    for (int L = 0; L <= b->max_layer; ++L) {
      // gate items of each circuit's layer L: consecutive disjoint gates as pairs
      std::vector<std::vector<std::pair<const Op*, const Op*>>> items(nc);
      size_t nslots = 0;
      for (size_t c = 0; c < nc; ++c) {
        std::vector<const Op*> gl;
        for (auto& op : b->ops[c])
          if (op.kind == R_GATE && op.layer == L) gl.push_back(&op);
        for (size_t k = 0; k < gl.size();) {
          const Op* x = gl[k];
          const Op* y = k + 1 < gl.size() ? gl[k + 1] : nullptr;
          if (y && x->qa != y->qa && x->qa != y->qb && x->qb != y->qa && x->qb != y->qb) {
            items[c].emplace_back(x, y);
            k += 2;
          } else {
            items[c].emplace_back(x, nullptr);
            k += 1;
          }
        }
        nslots = std::max(nslots, items[c].size());
      }
      for (size_t slot = 0; slot < nslots; ++slot) {
        std::vector<PairTask> tp;
        std::vector<GateTask> tg;
        std::vector<uint64_t> up, ug;
        for (size_t c = 0; c < nc; ++c) {
          if (slot >= items[c].size()) continue;
          const Op* x = items[c][slot].first;
          const Op* y = items[c][slot].second;
          if (y) {
            tp.push_back({b->state_of(c), b->nq[c], b->bit(c, x->qa), b->bit(c, x->qb), b->bit(c, y->qa),
                          b->bit(c, y->qb), x->index, y->index});
            up.push_back(1ull << (b->nq[c] - 4));
          } else {
            tg.push_back({b->state_of(c), b->nq[c], b->bit(c, x->qa), b->bit(c, x->qb), x->index});
            ug.push_back(1ull << (b->nq[c] - 2));
          }
        }
        if (!tp.empty()) b->rounds.push_back(b->make_round(R_PAIR, tp, up, b->pair_chunk, b->pair_threads));
        if (!tg.empty()) b->rounds.push_back(b->make_round(R_GATE, tg, ug, b->gate_chunk, b->gate_threads));
      }
      {
        std::vector<PhaseTask> t;
        std::vector<uint64_t> u;
        for (size_t c = 0; c < nc; ++c)
          for (auto& op : b->ops[c])
            if (op.kind == R_PHASE && op.layer == L) {
              t.push_back({b->state_of(c), tab_off[op.index], b->nq[c], (uint32_t)tab_split[op.index]});
              u.push_back(1ull << b->nq[c]);
            }
        if (!t.empty()) b->rounds.push_back(b->make_round(R_PHASE, t, u, B_CHUNK));
      }
      for (int slot = 0;; ++slot) {
        std::vector<SwapTask> t;
        std::vector<uint64_t> u;
        for (size_t c = 0; c < nc; ++c) {
          int seen = 0;
          for (auto& op : b->ops[c])
            if (op.kind == R_SWAP && op.layer == L && seen++ == slot) {
              t.push_back({b->state_of(c), b->nq[c], b->bit(c, op.qa), b->bit(c, op.qb)});
              u.push_back(1ull << (b->nq[c] - 2));
            }
        }
        if (t.empty()) break;
        b->rounds.push_back(b->make_round(R_SWAP, t, u, B_CHUNK));
      }
      if (period && (L + 1) % period == 0) {
        std::vector<NormTask> t;
        std::vector<uint64_t> u;
        for (size_t c = 0; c < nc; ++c) {
          int last = -1;
          for (auto& op : b->ops[c]) last = std::max(last, op.layer);
          if (last < L) continue;  // the circuit has ended
          t.push_back({b->state_of(c), b->nq[c], (uint32_t)(b->nnorms++)});
          u.push_back(1ull << b->nq[c]);
        }
        if (!t.empty()) {
          b->rounds.push_back(b->make_round(R_NORM, t, u, B_CHUNK));
          b->rounds.push_back(b->make_round(R_SCALE, t, u, B_CHUNK));
        }
      }
    }
    if (b->nnorms) {
      void* p = nullptr;
      check_cuda(cudaMalloc(&p, b->nnorms * sizeof(double)), "batch norms");
      b->allocations.push_back(p);
      b->norms = static_cast<double*>(p);
    }
    std::vector<uint64_t> where;
    for (auto& qv : b->queries) where.push_back(b->base[qv.first] + qv.second);
    b->query_where = b->upload(where);
    if (!where.empty()) {
      void* p = nullptr;
      check_cuda(cudaMalloc(&p, where.size() * sizeof(double2)), "batch query results");
      b->allocations.push_back(p);
      b->query_out = static_cast<double2*>(p);
    }
    // autotune the pair and single-gate kernels on their largest rounds (block size x
    // chunk length); the probes run on the working states, which every run resets
    cudaStream_t s = b->stream;
    if (autotune) {
      cudaEvent_t e0, e1;
      check_cuda(cudaEventCreate(&e0), "event");
      check_cuda(cudaEventCreate(&e1), "event");
      for (int kind : {R_PAIR, R_GATE}) {
        const Round* big = nullptr;
        for (auto& r : b->rounds)
          if (r.kind == kind && (!big || r.ntasks > big->ntasks)) big = &r;
        if (!big) continue;
        float best = 1e30f;
        int best_th = 256;
        uint64_t best_ch = kind == R_PAIR ? 256 : 1024;
        const std::vector<uint64_t> chunks =
            kind == R_PAIR ? std::vector<uint64_t>{64, 256, 1024} : std::vector<uint64_t>{256, 1024, 4096};
        for (int th : {128, 256, 512})
          for (uint64_t ch : chunks) {
            Round probe = b->rechunk(*big, th, ch);
            b->launch(probe, s);  // warm-up
            check_cuda(cudaEventRecord(e0, s), "event");
            for (int rep = 0; rep < 3; ++rep) b->launch(probe, s);
            check_cuda(cudaEventRecord(e1, s), "event");
            check_cuda(cudaEventSynchronize(e1), "event");
            float ms = 0;
            check_cuda(cudaEventElapsedTime(&ms, e0, e1), "event");
            if (ms < best) best = ms, best_th = th, best_ch = ch;
          }
        if (kind == R_PAIR)
          b->pair_threads = best_th, b->pair_chunk = best_ch;
        else
          b->gate_threads = best_th, b->gate_chunk = best_ch;
        for (auto& r : b->rounds)
          if (r.kind == kind) r = b->rechunk(r, best_th, best_ch);
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
    }
    // capture the whole run as one graph
    check_cuda(cudaStreamSynchronize(s), "batch synchronize");
    check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    uint64_t n0 = g_launches.load();
    check_cuda(cudaMemcpyAsync(b->psi, b->psi0, b->total_amps * b->amp_bytes(), cudaMemcpyDeviceToDevice, s),
               "reset");
    if (b->nnorms) check_cuda(cudaMemsetAsync(b->norms, 0, b->nnorms * sizeof(double), s), "norm reset");
    for (auto& r : b->rounds) b->launch(r, s);
    if (!where.empty()) b->gather(b->query_where, where.size(), b->query_out, s);
    b->launches_per_run = g_launches.load() - n0;
    g_launches.fetch_sub(b->launches_per_run);  // counted when the graph runs
    check_cuda(cudaStreamEndCapture(s, &b->graph), "end capture");
    check_cuda(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    return QTNH_OK;
  });
}

int qtnh_batch_run(qtnh_batch* b, void* stream) {
  return QTNH_API([&]() -> int {
    checked(b);
    if (!b->exec) throw Error(QTNH_ERR_RUNTIME, "batch not compiled");
    // order against the caller's stream: caller -> batch stream -> caller
    cudaEvent_t e;
    check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    check_cuda(cudaEventRecord(e, (cudaStream_t)stream), "event record");
    check_cuda(cudaStreamWaitEvent(b->stream, e, 0), "stream wait");
    check_cuda(cudaGraphLaunch(b->exec, b->stream), "graph launch");
    check_cuda(cudaEventRecord(e, b->stream), "event record");
    check_cuda(cudaStreamWaitEvent((cudaStream_t)stream, e, 0), "stream wait");
    check_cuda(cudaEventDestroy(e), "event");
    count_launch(b->launches_per_run);
    return QTNH_OK;
  });
}

int qtnh_batch_results(qtnh_batch* b, void* out_c128, uint64_t capacity, void* stream) {
  return QTNH_API([&]() -> int {
    checked(b);
    if (capacity < b->queries.size()) throw Error(QTNH_ERR_CAPACITY, "result buffer too small");
    if (!b->queries.empty())
      check_cuda(cudaMemcpyAsync(out_c128, b->query_out, b->queries.size() * sizeof(double2), cudaMemcpyDeviceToDevice,
                                 (cudaStream_t)stream),
                 "batch results");
    return QTNH_OK;
  });
}

int qtnh_batch_info(qtnh_batch* b, uint64_t* amplitudes, uint64_t* rounds, uint64_t* launches_per_run,
                    int32_t* gate_threads, uint64_t* gate_chunk) {
  return QTNH_API([&]() -> int {
    checked(b);
    if (amplitudes) *amplitudes = b->total_amps;
    if (rounds) *rounds = b->rounds.size();
    if (launches_per_run) *launches_per_run = b->launches_per_run;
    bool pairs = false;
    for (auto& r : b->rounds) pairs = pairs || r.kind == R_PAIR;
    if (gate_threads) *gate_threads = pairs ? b->pair_threads : b->gate_threads;
    if (gate_chunk) *gate_chunk = pairs ? b->pair_chunk : b->gate_chunk;
    return QTNH_OK;
  });
}

int qtnh_batch_state(qtnh_batch* b, int32_t c, void* out_c128, void* stream) {
  return QTNH_API([&]() -> int {
    checked(b);
    if (c < 0 || (size_t)c >= b->nq.size()) throw Error(QTNH_ERR_OUT_OF_RANGE, "circuit index out of range");
    const uint64_t n = 1ull << b->nq[c];
    // to complex128 through the query kernel over consecutive positions
    std::vector<uint64_t> where(n);
    for (uint64_t i = 0; i < n; ++i) where[i] = b->base[c] + i;
    uint64_t* w = nullptr;
    check_cuda(cudaMallocAsync((void**)&w, n * sizeof(uint64_t), (cudaStream_t)stream), "batch state");
    check_cuda(cudaMemcpyAsync(w, where.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice, (cudaStream_t)stream),
               "batch state");
    b->gather(w, n, static_cast<double2*>(out_c128), (cudaStream_t)stream);
    check_cuda(cudaFreeAsync(w, (cudaStream_t)stream), "batch state");
    check_cuda(cudaStreamSynchronize((cudaStream_t)stream), "batch state");
    return QTNH_OK;
  });
}

}  // extern "C"
