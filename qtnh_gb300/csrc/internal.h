// Shared declarations of the engine's translation units (not installed).
#pragma once

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "qtnh_cuda.h"

namespace qtnh_impl {

using dims_t = std::vector<uint64_t>;

// Error carrying a QTNH_ERR_* code; entry points translate it into a return value.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);
int status_from_current_exception();

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (...) {
    return status_from_current_exception();
  }
}

// An NVTX range named after a C ABI entry point for the length of the call, so that a
// profiler shows every API operation around its kernels; without a profiler attached
// the push and pop do nothing.
struct ApiRange {
  explicit ApiRange(const char* name) { nvtxRangePushA(name); }
  ~ApiRange() { nvtxRangePop(); }
  ApiRange(const ApiRange&) = delete;
  ApiRange& operator=(const ApiRange&) = delete;
};

template <class F>
int guarded_api(const char* name, F&& f) {
  ApiRange range(name);
  return guarded(std::forward<F>(f));
}

// Body of a C ABI entry point: exceptions become status codes, the call an NVTX range.
#define QTNH_API(...) ::qtnh_impl::guarded_api(__func__, __VA_ARGS__)

extern std::atomic<uint64_t> g_launches;
int arithmetic_mode();  // QTNH_ARITH_*
int gemm_mode();        // QTNH_GEMM_*
int gemm_slice_steps(); // K-steps per split-K slice of the QTNH_GEMM_BF16X3 GEMM
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

inline uint64_t product(const dims_t& d) {
  uint64_t p = 1;
  for (auto x : d) p *= x;
  return p;
}

inline dims_t row_strides(const dims_t& dims) {
  dims_t s(dims.size(), 1);
  for (int i = (int)dims.size() - 2; i >= 0; --i) s[i] = s[i + 1] * dims[i + 1];
  return s;
}

// ---- host planning (plan.cpp; no CUDA) ---------------------------------------------

struct Wire {
  uint16_t first, second;
};

struct TensorMeta {
  int32_t kind = QTNH_KIND_DENSE;
  dims_t dis, loc;
  int32_t n_dis_in = 0;
  dims_t tot() const {
    dims_t t = dis;
    t.insert(t.end(), loc.begin(), loc.end());
    return t;
  }
  uint64_t n_loc_in() const;  // include/tensor/symm.hpp:26-28 (throws when the range underflows)
};

TensorMeta meta_from_desc(const qtnh_tensor_desc* d);

struct ContractPlan {
  std::vector<Wire> wires;       // as given (validated)
  std::vector<uint16_t> repls1;  // output position of t1 axes (QTNH_X when wired)
  std::vector<uint16_t> repls2;
  dims_t out_dims;
  int32_t out_ndis = 0;
  uint64_t out_str = 1;
  bool inplace_rule = false;  // the symmetric in-place rule fired (contract.cpp:262)
};

// Tensor::contract metadata (contract.cpp:204-289) plus the result layout of
// _contract_dense (contract.cpp:86-111, 180-200).
ContractPlan plan_contract(const TensorMeta& t1, const TensorMeta& t2, const std::vector<Wire>& wires,
                           bool use_default, const std::vector<uint16_t>& repls1_in,
                           const std::vector<uint16_t>& repls2_in);

// ---- device-side entry points shared across translation units -----------------------

void permute_device(const void* in, void* out, const dims_t& dims, const std::vector<uint16_t>& ptup, void* stream);
void apply_gate_device(void* state, const dims_t& dims, const std::vector<uint16_t>& targets, const void* gate,
                       void* stream);
void apply_diag_device(void* state, const dims_t& dims, const std::vector<uint16_t>& targets, const void* diag,
                       void* stream);
// A lone gate on 2, 3 or 4 size-2 indices of a power-of-two state applied on the tensor
// cores as one 16x16 operator (gate (x) I4, gate (x) I2, or the gate itself; the identity
// on free size-2 indices); false (nothing launched) where that does not apply.
bool apply_gate_tc_single(void* state, const dims_t& dims, const std::vector<uint16_t>& targets, const void* gate,
                          void* stream);
// Gate list in order; consecutive disjoint two-qubit pairs fused onto the tensor cores.
void apply_gate_layer_tc(void* state, const dims_t& dims, const std::vector<std::vector<uint16_t>>& targets,
                         const std::vector<const void*>& gates, void* stream);
// One run of gates of apply_gate_runs_tc, followed by the permutation ptup (none if empty).
struct GateRun {
  std::vector<std::vector<uint16_t>> targets;
  std::vector<const void*> gates;
  std::vector<uint16_t> ptup;
};
// Runs of gates with permutations between them (out of place, state <-> scratch); the
// fixed-point chain of fused pairs continues across the permutations. Returns whether
// the result is in scratch.
bool apply_gate_runs_tc(void* state, void* scratch, dims_t dims, const std::vector<GateRun>& runs, void* stream);
// CUDA-event timing of the fused gate-pair passes (qtnh_gate_timing).
void set_pass_timing(bool on);
void take_pass_times(double& ms, uint64_t& launches);
// C (M x N) = A (M x K) B (K x N), complex128 row-major, BF16x3 pieces on tcgen05.
void gemm_bf16x3(const void* A, const void* B, void* C, uint64_t M, uint64_t N, uint64_t K, void* stream);
// The same with the operand permutes fused into the piece splits (gemm_umma.cu).
void gemm_bf16x3_perm(const void* A, const dims_t& dims_a, const std::vector<uint16_t>& pA, int nrow_a,
                      const void* B, const dims_t& dims_b, const std::vector<uint16_t>& pB,
                      const std::vector<uint16_t>& pBt, int ncol_b, void* C, uint64_t M, uint64_t N, uint64_t K,
                      void* stream);
// Permute `in` to [rows | K] and write its bf16 pieces into GEMM operand planes (permute.cu).
void permute_split_device(const void* in, const dims_t& dims, const std::vector<uint16_t>& ptup, int nrow_axes,
                          uint64_t rows, uint64_t rows_pad, uint64_t K, uint64_t kcs, uint8_t* planes,
                          uint64_t plane_bytes, uint32_t tile_rows, uint32_t KS, bool two_rows, void* stream);
uint32_t take_gemm_error();
// C (M x N) = A'' (M x K) B''^T, A'' and B'' (N x K) complex128 row-major, FP64-accurate
// through exact digit products on tcgen05 (gemm_oz.cu).
void gemm_oz6(const void* A, const void* Bt, void* C, uint64_t M, uint64_t N, uint64_t K, void* stream);
uint32_t take_ozg_error();
// gemm: the GEMM precision (QTNH_GEMM_*), -1 for the process-wide mode.
void contract_dense_device(const void* a, const dims_t& dims_a, const void* b, const dims_t& dims_b,
                           const std::vector<Wire>& wires, const std::vector<uint16_t>& pos_a,
                           const std::vector<uint16_t>& pos_b, void* c, void* stream, int gemm = -1);
// Dense materialisation of an implicit kind (swap/iden/diag) into `out` (prod(dims) elements).
void materialise_device(const TensorMeta& t, const void* data, void* out, void* stream);

// Stream-ordered workspace (cudaMallocAsync pool).
void* workspace_alloc(size_t bytes, void* stream);
void workspace_free(void* p, void* stream);

}  // namespace qtnh_impl
