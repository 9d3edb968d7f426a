// Tensor::contract at the C boundary: plan (host) + kernel dispatch (device).
//
// Dispatch, in order of preference:
//   1. Symmetric gate / diagonal applied with the in-place rule (contract.cpp:250-289)
//      and every wire on an input -> register-blocked gate kernel or streaming diagonal
//      multiply, in place on the output buffer.
//   2. SwapTensor / IdenTensor where every delta pair has exactly one wired member ->
//      the contraction only relabels indices: one transpose, bit-exact.
//   3. Anything else -> materialise implicit operands and run the permute-fused GEMM.

#include <algorithm>
#include <memory>
#include <numeric>

#include "cuda_common.cuh"

namespace qtnh_impl {
void apply_diag_layer_device(void* state, const dims_t& dims, const std::vector<uint16_t>& axes, const void* factors,
                             void* stream);
}

using namespace qtnh_impl;

namespace {

std::vector<Wire> read_wires(int32_t nwires, const uint16_t* wires) {
  if (nwires < 0 || nwires > QTNH_MAX_RANK) throw Error(QTNH_ERR_INVALID_ARGUMENT, "wire count out of range");
  std::vector<Wire> ws(nwires);
  for (int32_t i = 0; i < nwires; ++i) ws[i] = {wires[2 * i], wires[2 * i + 1]};
  return ws;
}

ContractPlan run_plan(const qtnh_tensor_desc* t1d, const qtnh_tensor_desc* t2d, int32_t nwires, const uint16_t* wires,
                      int32_t use_default, uint16_t* repls1, uint16_t* repls2, int32_t* out_ndis, int32_t* out_nloc,
                      uint64_t* out_dims, uint64_t* out_str, TensorMeta& t1, TensorMeta& t2) {
  t1 = meta_from_desc(t1d);
  t2 = meta_from_desc(t2d);
  std::vector<uint16_t> r1, r2;
  if (!use_default) {
    r1.assign(repls1, repls1 + t1.tot().size());
    r2.assign(repls2, repls2 + t2.tot().size());
  }
  ContractPlan p = plan_contract(t1, t2, read_wires(nwires, wires), use_default != 0, r1, r2);
  std::copy(p.repls1.begin(), p.repls1.end(), repls1);
  std::copy(p.repls2.begin(), p.repls2.end(), repls2);
  *out_ndis = p.out_ndis;
  *out_nloc = (int32_t)p.out_dims.size() - p.out_ndis;
  std::copy(p.out_dims.begin(), p.out_dims.end(), out_dims);
  *out_str = p.out_str;
  return p;
}

// Case 1: gate targets (t1 axis wired to each input of t2, inputs in order) when the
// contraction is an in-place application, else empty.
bool inplace_targets(const ContractPlan& p, const TensorMeta& t1, const TensorMeta& t2, std::vector<uint16_t>& targets) {
  if (!p.inplace_rule || !t2.dis.empty()) return false;
  const size_t nli = t2.n_loc_in();
  if (p.wires.size() != nli || t2.loc.size() != 2 * nli) return false;
  std::vector<Wire> ws = p.wires;
  std::sort(ws.begin(), ws.end(), [](const Wire& a, const Wire& b) { return a.second < b.second; });
  for (size_t j = 0; j < ws.size(); ++j)
    if (ws[j].second != j) return false;  // exactly the inputs are wired
  targets.resize(nli);
  for (size_t j = 0; j < nli; ++j) {
    targets[j] = ws[j].first;
    if (p.repls2[nli + j] != ws[j].first) return false;  // output j replaces input j's index
    if (t1.loc[targets[j]] != t2.loc[nli + j]) return false;
  }
  return true;
}

// Case 1 in full: the kinds, the in-place rule and the sizes the in-place kernels take.
bool inplace_dispatch(const ContractPlan& p, const TensorMeta& t1, const TensorMeta& t2, std::vector<uint16_t>& targets) {
  if (!((t2.kind == QTNH_KIND_SYMM || t2.kind == QTNH_KIND_DIAG) &&
        (t1.kind == QTNH_KIND_DENSE || t1.kind == QTNH_KIND_SYMM) && inplace_targets(p, t1, t2, targets)))
    return false;
  const dims_t d1 = t1.tot();
  uint64_t D = 1;
  for (auto t : targets) D *= d1[t];
  return (t2.kind == QTNH_KIND_DIAG) ? targets.size() <= 8
                                      : (D == 1 || D == 2 || D == 3 || D == 4 || D == 8 || D == 9 || D == 16);
}

// Case 2: delta tensors. Partner of index i: Swap (0<->3, 1<->2); Iden (i <-> i +- m).
bool relabel_ptup(const ContractPlan& p, const TensorMeta& t1, const TensorMeta& t2, std::vector<uint16_t>& ptup) {
  if (t2.kind != QTNH_KIND_SWAP && t2.kind != QTNH_KIND_IDEN) return false;
  const size_t r2 = t2.tot().size(), r1 = t1.tot().size();
  if (t2.kind == QTNH_KIND_IDEN && (r2 % 2)) return false;
  auto partner = [&](size_t i) -> size_t {
    if (t2.kind == QTNH_KIND_SWAP) return 3 - i;
    size_t m = r2 / 2;
    return i < m ? i + m : i - m;
  };
  std::vector<int> wired_to(r2, -1);
  for (auto& w : p.wires) wired_to[w.second] = w.first;
  ptup.assign(r1, 0);
  for (size_t i = 0; i < r1; ++i) ptup[i] = p.repls1[i];
  for (size_t i = 0; i < r2; ++i) {
    size_t q = partner(i);
    if (t2.tot()[i] != t2.tot()[q]) return false;  // rectangular delta: not a relabelling
    bool wi = wired_to[i] >= 0, wq = wired_to[q] >= 0;
    if (wi == wq) return false;  // trace or free delta: not a relabelling
    if (wi) ptup[wired_to[i]] = p.repls2[q];
  }
  return true;
}

}  // namespace

extern "C" {

int qtnh_contract_plan(const qtnh_tensor_desc* t1, const qtnh_tensor_desc* t2, int32_t nwires, const uint16_t* wires,
                       int32_t use_default, uint16_t* repls1, uint16_t* repls2, int32_t* out_ndis, int32_t* out_nloc,
                       uint64_t* out_dims, uint64_t* out_str) {
  return QTNH_API([&]() -> int {
    TensorMeta m1, m2;
    run_plan(t1, t2, nwires, wires, use_default, repls1, repls2, out_ndis, out_nloc, out_dims, out_str, m1, m2);
    return QTNH_OK;
  });
}

int qtnh_contract_inplace(const qtnh_tensor_desc* t1, const qtnh_tensor_desc* t2, int32_t nwires, const uint16_t* wires,
                          int32_t use_default, uint16_t* repls1, uint16_t* repls2, int32_t* out_ndis, int32_t* out_nloc,
                          uint64_t* out_dims, uint64_t* out_str, int32_t* inplace, int32_t* ntargets, uint16_t* targets) {
  return QTNH_API([&]() -> int {
    if (!inplace || !ntargets || !targets) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null output pointer");
    TensorMeta m1, m2;
    ContractPlan p = run_plan(t1, t2, nwires, wires, use_default, repls1, repls2, out_ndis, out_nloc, out_dims, out_str,
                              m1, m2);
    std::vector<uint16_t> tg;
    const bool yes = inplace_dispatch(p, m1, m2, tg);
    *inplace = yes ? 1 : 0;
    *ntargets = yes ? (int32_t)tg.size() : 0;
    if (yes) std::copy(tg.begin(), tg.end(), targets);
    return QTNH_OK;
  });
}

int qtnh_contract(const qtnh_tensor_desc* t1d, const qtnh_tensor_desc* t2d, int32_t nwires, const uint16_t* wires,
                  int32_t use_default, uint16_t* repls1, uint16_t* repls2, int32_t* out_ndis, int32_t* out_nloc,
                  uint64_t* out_dims, uint64_t* out_str, void* out, uint64_t out_capacity, void* stream) {
  return QTNH_API([&]() -> int {
    TensorMeta t1, t2;
    ContractPlan p = run_plan(t1d, t2d, nwires, wires, use_default, repls1, repls2, out_ndis, out_nloc, out_dims,
                              out_str, t1, t2);
    const uint64_t nout = product(p.out_dims);
    if (!out || out_capacity < nout) {
      set_last_error("output buffer too small");
      return (int)QTNH_ERR_CAPACITY;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const dims_t d1 = t1.tot(), d2 = t2.tot();
    const uint64_t n1 = product(d1);

    // 1. in-place gate / diagonal
    std::vector<uint16_t> targets;
    if (inplace_dispatch(p, t1, t2, targets)) {
      if (out != t1d->data) check_cuda(cudaMemcpyAsync(out, t1d->data, n1 * sizeof(c128), cudaMemcpyDeviceToDevice, s), "copy");
      if (t2.kind == QTNH_KIND_SYMM) apply_gate_device(out, d1, targets, t2d->data, stream);
      else apply_diag_device(out, d1, targets, t2d->data, stream);
      return QTNH_OK;
    }

    // 2. delta tensors relabel indices
    std::vector<uint16_t> ptup;
    if ((t1.kind == QTNH_KIND_DENSE || t1.kind == QTNH_KIND_SYMM) && relabel_ptup(p, t1, t2, ptup)) {
      if (out == t1d->data) {
        bool ident = true;
        for (size_t i = 0; i < ptup.size(); ++i) ident = ident && ptup[i] == i;
        if (ident) return QTNH_OK;
        void* tmp = workspace_alloc(n1 * sizeof(c128), stream);
        try {
          permute_device(t1d->data, tmp, d1, ptup, stream);
          check_cuda(cudaMemcpyAsync(out, tmp, n1 * sizeof(c128), cudaMemcpyDeviceToDevice, s), "copy");
        } catch (...) {
          workspace_free(tmp, stream);
          throw;
        }
        workspace_free(tmp, stream);
      } else {
        permute_device(t1d->data, out, d1, ptup, stream);
      }
      return QTNH_OK;
    }

    // 3. general dense contraction
    const void* a = t1d->data;
    const void* b = t2d->data;
    void* a_tmp = nullptr;
    void* b_tmp = nullptr;
    void* c_tmp = nullptr;
    try {
      if (t1.kind != QTNH_KIND_DENSE && t1.kind != QTNH_KIND_SYMM) {
        a_tmp = workspace_alloc(n1 * sizeof(c128), stream);
        materialise_device(t1, t1d->data, a_tmp, stream);
        a = a_tmp;
      }
      if (t2.kind != QTNH_KIND_DENSE && t2.kind != QTNH_KIND_SYMM) {
        b_tmp = workspace_alloc(product(d2) * sizeof(c128), stream);
        materialise_device(t2, t2d->data, b_tmp, stream);
        b = b_tmp;
      }
      void* c = out;
      if (out == t1d->data || out == t2d->data) c = c_tmp = workspace_alloc(nout * sizeof(c128), stream);
      // a SwapTensor or IdenTensor operand holds only 0/1 weights with one nonzero term per
      // output: the FP64 FMA GEMM reproduces such relabellings bit-exactly, whatever the mode
      const bool delta = t1.kind == QTNH_KIND_SWAP || t1.kind == QTNH_KIND_IDEN || t2.kind == QTNH_KIND_SWAP ||
                         t2.kind == QTNH_KIND_IDEN;
      contract_dense_device(a, d1, b, d2, p.wires, p.repls1, p.repls2, c, stream, delta ? QTNH_GEMM_FP64 : -1);
      if (c_tmp) check_cuda(cudaMemcpyAsync(out, c_tmp, nout * sizeof(c128), cudaMemcpyDeviceToDevice, s), "copy");
    } catch (...) {
      workspace_free(a_tmp, stream);
      workspace_free(b_tmp, stream);
      workspace_free(c_tmp, stream);
      throw;
    }
    workspace_free(a_tmp, stream);
    workspace_free(b_tmp, stream);
    workspace_free(c_tmp, stream);
    return QTNH_OK;
  });
}

}  // extern "C"
