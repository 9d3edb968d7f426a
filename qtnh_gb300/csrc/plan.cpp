// Host-side contraction planning: the metadata half of Tensor::contract.
//
// Restates src/tensor/contract.cpp:204-289 (validation, default dimension
// replacements, the in-place rule for symmetric second operands) and the result
// layout that _contract_dense produces (contract.cpp:86-111 for the local part,
// 180-200 for the distributed part and the stretch factor). Pure C++: no GPU needed.

#include <algorithm>
#include <numeric>

#include "internal.h"

namespace qtnh_impl {

uint64_t TensorMeta::n_loc_in() const {
  // include/tensor/symm.hpp:26-28: loc[0 : loc.size()/2 - n_dis_in]. The reference builds
  // that range unchecked; a negative length is refused here.
  uint64_t half = loc.size() / 2;
  if (half < (uint64_t)n_dis_in) throw Error(QTNH_ERR_OUT_OF_RANGE, "symmetric tensor: local input range underflows");
  return half - (uint64_t)n_dis_in;
}

TensorMeta meta_from_desc(const qtnh_tensor_desc* d) {
  if (!d) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null tensor descriptor");
  if (d->ndis < 0 || d->nloc < 0 || d->ndis + d->nloc > QTNH_MAX_RANK)
    throw Error(QTNH_ERR_INVALID_ARGUMENT, "tensor rank out of range");
  if (d->kind < QTNH_KIND_DENSE || d->kind > QTNH_KIND_DIAG) throw Error(QTNH_ERR_INVALID_ARGUMENT, "unknown tensor kind");
  TensorMeta t;
  t.kind = d->kind;
  t.dis.assign(d->dims, d->dims + d->ndis);
  t.loc.assign(d->dims + d->ndis, d->dims + d->ndis + d->nloc);
  t.n_dis_in = d->n_dis_in;
  for (auto x : t.tot())
    if (x == 0) throw Error(QTNH_ERR_INVALID_ARGUMENT, "zero dimension");
  if (t.kind == QTNH_KIND_SWAP && t.tot().size() != 4) throw Error(QTNH_ERR_INVALID_ARGUMENT, "swap tensor must have rank 4");
  return t;
}

static bool by_first(const Wire& a, const Wire& b) { return a.first < b.first; }
static bool by_second(const Wire& a, const Wire& b) { return a.second < b.second; }

ContractPlan plan_contract(const TensorMeta& t1, const TensorMeta& t2, const std::vector<Wire>& wires_in,
                           bool use_default, const std::vector<uint16_t>& repls1_in,
                           const std::vector<uint16_t>& repls2_in) {
  ContractPlan p;
  dims_t tot1 = t1.tot(), tot2 = t2.tot();
  const size_t nd1 = t1.dis.size(), nd2 = t2.dis.size();
  std::vector<Wire> ws = wires_in;

  // contract.cpp:207-217
  size_t n_dis_ws = 0;
  for (auto& w : ws) {
    if (w.first >= tot1.size() || w.second >= tot2.size()) throw Error(QTNH_ERR_OUT_OF_RANGE, "wire index out of range");
    if (tot1[w.first] != tot2[w.second]) throw Error(QTNH_ERR_INVALID_ARGUMENT, "Incompatible contraction dimensions.");
    if ((w.first < nd1) != (w.second < nd2))
      throw Error(QTNH_ERR_INVALID_ARGUMENT, "Attempted to contract distributed and local dimensions.");
    if (w.first < nd1) ++n_dis_ws;
  }
  {
    // Self-contractions are unsupported in the reference (README.md:168) and undefined
    // there; refuse an index wired twice.
    std::vector<char> u1(tot1.size(), 0), u2(tot2.size(), 0);
    for (auto& w : ws)
      if (u1[w.first]++ || u2[w.second]++) throw Error(QTNH_ERR_INVALID_ARGUMENT, "An index is wired more than once.");
  }

  std::vector<uint16_t> r1, r2;
  if (use_default) {
    // contract.cpp:220-248
    r1.assign(tot1.size(), (uint16_t)QTNH_X);
    std::sort(ws.begin(), ws.end(), by_first);
    for (size_t i = 0, j = 0; i < tot1.size(); ++i) {
      if (j < ws.size() && i == ws[j].first) {
        ++j;
      } else {
        r1[i] = (uint16_t)(i - j);
        if (i >= nd1) r1[i] = (uint16_t)(r1[i] + (nd2 - n_dis_ws));
      }
    }
    r2.assign(tot2.size(), (uint16_t)QTNH_X);
    std::sort(ws.begin(), ws.end(), by_second);
    for (size_t i = 0, j = 0; i < tot2.size(); ++i) {
      if (j < ws.size() && i == ws[j].second) {
        ++j;
      } else {
        r2[i] = (uint16_t)(nd1 - n_dis_ws + i - j);
        if (i >= nd2) r2[i] = (uint16_t)(tot1.size() - ws.size() + i - j);
      }
    }
  } else {
    if (repls1_in.size() != tot1.size() || repls2_in.size() != tot2.size())
      throw Error(QTNH_ERR_OUT_OF_RANGE, "dimension replacement tuple has the wrong size");
    r1 = repls1_in;
    r2 = repls2_in;
  }

  // contract.cpp:250-289 — symmetric second operand (SymmTensor, SwapTensor, DiagTensor,
  // IdenTensor all derive from SymmTensorBase).
  if (t2.kind != QTNH_KIND_DENSE) {
    const size_t ndi = (size_t)t2.n_dis_in;
    const size_t nli = t2.n_loc_in();
    size_t input_count = 0;
    for (auto& w : ws)
      if (w.second < ndi || (w.second >= nd2 && w.second < nd2 + nli)) ++input_count;
    const int dis_imbal = (int)ndi - (int)(nd2 - ndi);
    if (dis_imbal == 0 && input_count == ndi + nli) {
      p.inplace_rule = true;
      r1.assign(tot1.size(), (uint16_t)QTNH_X);
      std::sort(ws.begin(), ws.end(), by_first);
      for (size_t i = 0, j = 0; i < tot1.size(); ++i) {
        if (j < ws.size() && i == ws[j].first) ++j;
        else r1[i] = (uint16_t)i;
      }
      r2.assign(tot2.size(), (uint16_t)QTNH_X);
      std::sort(ws.begin(), ws.end(), by_second);
      std::vector<uint16_t> from_dims(ws.size());
      for (size_t i = 0; i < ws.size(); ++i) from_dims[i] = ws[i].first;
      for (size_t i = 0, j = 0, k = 0; i < tot2.size(); ++i) {
        if (j < ws.size() && i == ws[j].second) ++j;
        else if (k < ws.size()) r2[i] = from_dims[k++];
      }
    }
  }

  // Result layout (global form of _contract_dense). Open indices land at their
  // replacement positions; the distributed ones must fill [0, n_open_dis) and the local
  // ones the rest (ptup3 at contract.cpp:181-194 only permutes the distributed block,
  // ptup_loc at 86-111 only the local block).
  std::vector<int> wired1(tot1.size(), 0), wired2(tot2.size(), 0);
  for (auto& w : ws) wired1[w.first] = wired2[w.second] = 1;
  const size_t n_open_dis = (nd1 - n_dis_ws) + (nd2 - n_dis_ws);
  const size_t n_out = tot1.size() + tot2.size() - 2 * ws.size();
  p.out_dims.assign(n_out, 0);
  std::vector<char> filled(n_out, 0);
  auto place = [&](uint16_t pos, uint64_t dim, bool is_dis) {
    if (pos >= n_out) throw Error(QTNH_ERR_OUT_OF_RANGE, "dimension replacement out of range");
    if (is_dis != (pos < n_open_dis))
      throw Error(QTNH_ERR_INVALID_ARGUMENT, "dimension replacement crosses the distributed/local border");
    if (filled[pos]++) throw Error(QTNH_ERR_INVALID_ARGUMENT, "dimension replacement repeats a position");
    p.out_dims[pos] = dim;
  };
  // Wired entries are ignored ("Closed indices are ignored", README.md:151) and left as given.
  for (size_t i = 0; i < tot1.size(); ++i)
    if (!wired1[i]) place(r1[i], tot1[i], i < nd1);
  for (size_t i = 0; i < tot2.size(); ++i)
    if (!wired2[i]) place(r2[i], tot2[i], i < nd2);
  p.out_ndis = (int32_t)n_open_dis;
  p.out_str = 1;
  for (auto& w : ws)
    if (w.first < nd1) p.out_str *= tot1[w.first];  // contract.cpp:196-198
  p.wires = ws;
  p.repls1 = std::move(r1);
  p.repls2 = std::move(r2);
  return p;
}

}  // namespace qtnh_impl
