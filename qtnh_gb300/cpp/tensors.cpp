// Tensor classes of the qtnh API on the GB300 engine.
//
// Metadata operations follow the reference (src/tensor/tensor.cpp, dense.cpp, symm.cpp,
// diag.cpp); element operations call the C ABI (include/qtnh_cuda.h) on the
// environment's stream.
#include <algorithm>
#include <iomanip>
#include <numeric>
#include <stdexcept>

#include "facade_internal.hpp"
#include "qtnh.hpp"
#include "qtnh_cuda.h"

namespace qtnh {

using detail::check;
using detail::DeviceArray;

namespace {

std::size_t tot_index(const tidx_tup& tot_idxs, const tidx_tup& dims) {
  if (tot_idxs.size() != dims.size()) throw std::out_of_range("index tuple has the wrong length");
  for (std::size_t i = 0; i < dims.size(); ++i)
    if (tot_idxs[i] >= dims[i]) throw std::out_of_range("index out of range");
  return utils::idxs_to_i(tot_idxs, dims);
}

std::vector<uint64_t> u64(const tidx_tup& d) { return std::vector<uint64_t>(d.begin(), d.end()); }

}  // namespace

// ---- Tensor -----------------------------------------------------------------------

Tensor::Broadcaster::Broadcaster(const QTNHEnv& env, qtnh::uint base, BcParams params)
    : env(env), base(base), str(params.str), cyc(params.cyc), off(params.off) {}

Tensor::Broadcaster& Tensor::Broadcaster::operator=(Broadcaster&& b) noexcept {
  base = b.base;
  str = b.str;
  cyc = b.cyc;
  off = b.off;
  active = b.active;
  group_id = b.group_id;
  return *this;
}

Tensor::Tensor(const QTNHEnv& env) : Tensor(env, tidx_tup(), tidx_tup()) {}
Tensor::Tensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims) : Tensor(env, dis_dims, loc_dims, BcParams{1, 1, 0}) {}
Tensor::Tensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, BcParams params)
    : dis_dims_(dis_dims), loc_dims_(loc_dims), bc_(env, (qtnh::uint)utils::dims_to_size(dis_dims), params) {}

template <> bool Tensor::canConvert<DenseTensor>() { return isDense(); }
template <> bool Tensor::canConvert<SymmTensor>() { return isSymm(); }
template <> bool Tensor::canConvert<DiagTensor>() { return isDiag(); }

template <> std::unique_ptr<DenseTensor> Tensor::convert<DenseTensor>(tptr tp) {
  Tensor* raw = tp.get();
  DenseTensor* d = raw->toDense();
  return utils::one_unique(std::move(tp), d);
}
template <> std::unique_ptr<SymmTensor> Tensor::convert<SymmTensor>(tptr tp) {
  Tensor* raw = tp.get();
  SymmTensor* s = raw->toSymm();
  return utils::one_unique(std::move(tp), s);
}
template <> std::unique_ptr<DiagTensor> Tensor::convert<DiagTensor>(tptr tp) {
  Tensor* raw = tp.get();
  DiagTensor* d = raw->toDiag();
  return utils::one_unique(std::move(tp), d);
}

bool Tensor::has(tidx_tup tot_idxs) const {
  if (!bc_.active) return false;
  tot_index(tot_idxs, totDims());
  return true;
}

tel Tensor::fetch(tidx_tup tot_idxs) const { return at(tot_idxs); }

std::vector<tel> Tensor::hostElements() const {
  const tidx_tup dims = totDims();
  const std::size_t n = utils::dims_to_size(dims);
  std::vector<tel> out(n);
  for (std::size_t i = 0; i < n; ++i) out[i] = at(utils::i_to_idxs(i, dims));
  return out;
}

// The transforms evaluate tp->X(...) before handing ownership over (the reference relies
// on argument evaluation order for this, include/tensor/tensor.hpp:169-192).
tptr Tensor::swap(tptr tp, tidx_tup_st idx1, tidx_tup_st idx2) {
  Tensor* raw = tp.get();
  Tensor* r = raw->swap(idx1, idx2);
  return utils::one_unique(std::move(tp), r);
}
tptr Tensor::rebcast(tptr tp, BcParams params) {
  Tensor* raw = tp.get();
  Tensor* r = raw->rebcast(params);
  return utils::one_unique(std::move(tp), r);
}
tptr Tensor::rescatter(tptr tp, int offset) {
  Tensor* raw = tp.get();
  Tensor* r = raw->rescatter(offset);
  return utils::one_unique(std::move(tp), r);
}
tptr Tensor::permute(tptr tp, std::vector<tidx_tup_st> ptup) {
  Tensor* raw = tp.get();
  Tensor* r = raw->permute(ptup);
  return utils::one_unique(std::move(tp), r);
}

tptr contract_on_device(tptr tp1, tptr tp2, ConParams& params);

tptr Tensor::contract(tptr tp1, tptr tp2, ConParams& params) { return contract_on_device(std::move(tp1), std::move(tp2), params); }

// ---- DenseTensorBase ----------------------------------------------------------------

DenseTensorBase::DenseTensorBase(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims) : Tensor(env, dis_dims, loc_dims) {}
DenseTensorBase::DenseTensorBase(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, BcParams params)
    : Tensor(env, dis_dims, loc_dims, params) {}

// src/tensor/dense.cpp:19-37: every element through the accessors, into a DenseTensor.
DenseTensor* DenseTensorBase::toDense() noexcept {
  return new DenseTensor(bc_.env, dis_dims_, loc_dims_, hostElements(), BcParams{bc_.str, bc_.cyc, bc_.off});
}

Tensor* DenseTensorBase::swap(tidx_tup_st idx1, tidx_tup_st idx2) { return toDense()->swap(idx1, idx2); }
Tensor* DenseTensorBase::rebcast(BcParams params) { return toDense()->rebcast(params); }
Tensor* DenseTensorBase::rescatter(int offset) { return toDense()->rescatter(offset); }
Tensor* DenseTensorBase::permute(std::vector<tidx_tup_st> ptup) { return toDense()->permute(ptup); }

// ---- DenseTensor --------------------------------------------------------------------

static std::vector<tel>&& checked_els(std::vector<tel>&& els, const tidx_tup& dis, const tidx_tup& loc) {
  const std::size_t n = utils::dims_to_size(dis) * utils::dims_to_size(loc);
  if (els.size() != n)
    throw std::invalid_argument("element count " + std::to_string(els.size()) + " differs from the tensor size " +
                                std::to_string(n) + " (all slabs, in rank order)");
  return std::move(els);
}

DenseTensor::DenseTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, std::vector<tel>&& els)
    : DenseTensorBase(env, dis_dims, loc_dims), els_(env, checked_els(std::move(els), dis_dims, loc_dims)) {}

DenseTensor::DenseTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, std::vector<tel>&& els, BcParams params)
    : DenseTensorBase(env, dis_dims, loc_dims, params), els_(env, checked_els(std::move(els), dis_dims, loc_dims)) {}

DenseTensor::DenseTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, DeviceArray&& els, BcParams params)
    : DenseTensorBase(env, dis_dims, loc_dims, params), els_(std::move(els)) {}

tptr DenseTensor::copy() const noexcept {
  return tptr(new DenseTensor(bc_.env, dis_dims_, loc_dims_, els_.clone(), BcParams{bc_.str, bc_.cyc, bc_.off}));
}

int DenseTensor::engineKind() const noexcept { return QTNH_KIND_DENSE; }

std::size_t DenseTensor::check_i(std::size_t i) const {
  if (i >= els_.size()) throw std::out_of_range("element index out of range");
  return i;
}

tel DenseTensor::operator[](tidx_tup loc_idxs) const { return els_.host_at(tot_index(loc_idxs, loc_dims_)); }
tel& DenseTensor::operator[](tidx_tup loc_idxs) { return els_.host_ref(tot_index(loc_idxs, loc_dims_)); }
tel DenseTensor::at(tidx_tup tot_idxs) const { return els_.host_at(tot_index(tot_idxs, totDims())); }
tel& DenseTensor::at(tidx_tup tot_idxs) { return els_.host_ref(tot_index(tot_idxs, totDims())); }
void DenseTensor::put(tidx_tup tot_idxs, tel el) { els_.host_ref(tot_index(tot_idxs, totDims())) = el; }

// src/tensor/dense.cpp:171-274: one on-device transpose for every case.
DenseTensor* DenseTensor::swap(tidx_tup_st idx1, tidx_tup_st idx2) {
  const tidx_tup dims = totDims();
  if (idx1 >= dims.size() || idx2 >= dims.size()) throw std::out_of_range("swap index out of range");
  if (dims[idx1] != dims[idx2]) throw std::runtime_error("Asymmetric swaps are currently not allowed");
  if (idx1 == idx2) return this;
  DeviceArray out(bc_.env, els_.size());
  auto d = u64(dims);
  check(qtnh_swap(els_.read(), out.write(), (int32_t)d.size(), d.data(), idx1, idx2, bc_.env.stream));
  els_ = std::move(out);
  return this;
}

DenseTensor* DenseTensor::rebcast(BcParams params) {
  bc_ = Broadcaster(bc_.env, bc_.base, params);
  return this;
}

// src/tensor/dense.cpp:123-150: the border moves, global order is unchanged.
DenseTensor* DenseTensor::rescatter(int offset) {
  if (offset < 0) {
    if ((std::size_t)(-offset) > dis_dims_.size()) throw std::out_of_range("rescatter offset beyond the distributed dims");
    tidx_tup moved(dis_dims_.end() + offset, dis_dims_.end());
    const qtnh::uint shift = (qtnh::uint)utils::dims_to_size(moved);
    loc_dims_.insert(loc_dims_.begin(), moved.begin(), moved.end());
    dis_dims_.erase(dis_dims_.end() + offset, dis_dims_.end());
    bc_ = Broadcaster(bc_.env, (qtnh::uint)disSize(), BcParams{bc_.str * shift, bc_.cyc, bc_.off});
  } else if (offset > 0) {
    if ((std::size_t)offset > loc_dims_.size()) throw std::out_of_range("rescatter offset beyond the local dims");
    tidx_tup moved(loc_dims_.begin(), loc_dims_.begin() + offset);
    const std::size_t shift = utils::dims_to_size(moved);
    BcParams params((qtnh::uint)std::max<std::size_t>(1, bc_.str / shift), bc_.cyc, bc_.off);
    loc_dims_.erase(loc_dims_.begin(), loc_dims_.begin() + offset);
    dis_dims_.insert(dis_dims_.end(), moved.begin(), moved.end());
    bc_ = Broadcaster(bc_.env, (qtnh::uint)disSize(), params);
  }
  return this;
}

// src/tensor/dense.cpp:152-169, 354-488.
DenseTensor* DenseTensor::permute(std::vector<tidx_tup_st> ptup) {
  const tidx_tup dims = totDims();
  if (ptup.size() != dims.size()) throw std::out_of_range("permutation tuple has the wrong length");
  tidx_tup nd(dims.size());
  for (std::size_t i = 0; i < dims.size(); ++i) nd.at(ptup[i]) = dims[i];
  // queued behind any in-place contractions on the elements, so that gate runs on both
  // sides of it are applied in one call (qtnh_apply_gate_runs)
  els_.defer_permute(ptup, u64(dims));
  auto parts = utils::split_dims(nd, (tidx_tup_st)dis_dims_.size());
  dis_dims_ = parts.first;
  loc_dims_ = parts.second;
  bc_ = Broadcaster(bc_.env, (qtnh::uint)disSize(), BcParams{bc_.str, bc_.cyc, bc_.off});
  return this;
}

// ---- SymmTensorBase -----------------------------------------------------------------

SymmTensorBase::SymmTensorBase(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims)
    : DenseTensorBase(env, dis_dims, loc_dims), n_dis_in_dims_(n_dis_in_dims) {}
SymmTensorBase::SymmTensorBase(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims,
                               BcParams params)
    : DenseTensorBase(env, dis_dims, loc_dims, params), n_dis_in_dims_(n_dis_in_dims) {}

// include/tensor/symm.hpp:22-45 (the local input count is loc.size()/2 - n_dis_in; a
// negative count is refused).
static std::size_t loc_in_count(const tidx_tup& loc, tidx_tup_st n_dis_in) {
  if (loc.size() / 2 < n_dis_in) throw std::out_of_range("symmetric tensor: local input range underflows");
  return loc.size() / 2 - n_dis_in;
}
tidx_tup SymmTensorBase::disInDims() const {
  if (n_dis_in_dims_ > dis_dims_.size()) throw std::out_of_range("symmetric tensor: distributed input count");
  return tidx_tup(dis_dims_.begin(), dis_dims_.begin() + n_dis_in_dims_);
}
tidx_tup SymmTensorBase::locInDims() const {
  return tidx_tup(loc_dims_.begin(), loc_dims_.begin() + loc_in_count(loc_dims_, n_dis_in_dims_));
}
tidx_tup SymmTensorBase::disOutDims() const {
  if (n_dis_in_dims_ > dis_dims_.size()) throw std::out_of_range("symmetric tensor: distributed input count");
  return tidx_tup(dis_dims_.begin() + n_dis_in_dims_, dis_dims_.end());
}
tidx_tup SymmTensorBase::locOutDims() const {
  return tidx_tup(loc_dims_.begin() + loc_in_count(loc_dims_, n_dis_in_dims_), loc_dims_.end());
}

SymmTensor* SymmTensorBase::toSymm() noexcept {
  return new SymmTensor(bc_.env, dis_dims_, loc_dims_, n_dis_in_dims_, hostElements(), BcParams{bc_.str, bc_.cyc, bc_.off});
}

// ---- SymmTensor ---------------------------------------------------------------------

SymmTensor::SymmTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, std::vector<tel>&& els)
    : SymmTensorBase(env, dis_dims, loc_dims, n_dis_in_dims), els_(env, checked_els(std::move(els), dis_dims, loc_dims)) {}
SymmTensor::SymmTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, std::vector<tel>&& els,
                       BcParams params)
    : SymmTensorBase(env, dis_dims, loc_dims, n_dis_in_dims, params),
      els_(env, checked_els(std::move(els), dis_dims, loc_dims)) {}
SymmTensor::SymmTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, DeviceArray&& els,
                       BcParams params)
    : SymmTensorBase(env, dis_dims, loc_dims, n_dis_in_dims, params), els_(std::move(els)) {}

std::unique_ptr<Tensor> SymmTensor::copy() const noexcept {
  return tptr(new SymmTensor(bc_.env, dis_dims_, loc_dims_, n_dis_in_dims_, els_.clone(), BcParams{bc_.str, bc_.cyc, bc_.off}));
}

int SymmTensor::engineKind() const noexcept { return QTNH_KIND_SYMM; }

tel SymmTensor::operator[](tidx_tup loc_idxs) const { return els_.host_at(tot_index(loc_idxs, loc_dims_)); }
tel& SymmTensor::operator[](tidx_tup loc_idxs) { return els_.host_ref(tot_index(loc_idxs, loc_dims_)); }
tel SymmTensor::at(tidx_tup tot_idxs) const { return els_.host_at(tot_index(tot_idxs, totDims())); }
tel& SymmTensor::at(tidx_tup tot_idxs) { return els_.host_ref(tot_index(tot_idxs, totDims())); }
void SymmTensor::put(tidx_tup tot_idxs, tel el) { els_.host_ref(tot_index(tot_idxs, totDims())) = el; }

SymmTensor* SymmTensor::rebcast(BcParams params) {
  bc_ = Broadcaster(bc_.env, bc_.base, params);
  return this;
}

// ---- SwapTensor (src/tensor/symm.cpp:234-291) ----------------------------------------

SwapTensor::SwapTensor(const QTNHEnv& env, std::size_t n, std::size_t d)
    : SymmTensorBase(env, tidx_tup(2 * d, n), tidx_tup(4 - 2 * std::min<std::size_t>(d, 2), n), (tidx_tup_st)d) {
  if (d > 2) throw std::invalid_argument("swap tensor: at most 2 distributed inputs");
}
SwapTensor::SwapTensor(const QTNHEnv& env, std::size_t n, std::size_t d, BcParams params)
    : SymmTensorBase(env, tidx_tup(2 * d, n), tidx_tup(4 - 2 * std::min<std::size_t>(d, 2), n), (tidx_tup_st)d, params) {
  if (d > 2) throw std::invalid_argument("swap tensor: at most 2 distributed inputs");
}

std::unique_ptr<Tensor> SwapTensor::copy() const noexcept {
  const std::size_t n = dis_dims_.empty() ? loc_dims_.at(0) : dis_dims_.at(0);
  return tptr(new SwapTensor(bc_.env, n, n_dis_in_dims_, BcParams{bc_.str, bc_.cyc, bc_.off}));
}

int SwapTensor::engineKind() const noexcept { return QTNH_KIND_SWAP; }

static tel swap_element(const tidx_tup& t) { return (t.at(0) == t.at(3) && t.at(1) == t.at(2)) ? 1.0 : 0.0; }

tel SwapTensor::operator[](tidx_tup loc_idxs) const {
  return swap_element(utils::concat_dims(utils::i_to_idxs(0, dis_dims_), loc_idxs));
}
tel SwapTensor::operator[](std::size_t i) const {
  if (i >= totSize()) throw std::out_of_range("element index out of range");
  return swap_element(utils::i_to_idxs(i, totDims()));
}
tel SwapTensor::at(tidx_tup tot_idxs) const {
  tot_index(tot_idxs, totDims());
  return swap_element(tot_idxs);
}

SwapTensor* SwapTensor::rebcast(BcParams params) {
  bc_ = Broadcaster(bc_.env, bc_.base, params);
  return this;
}

// ---- DiagTensorBase / DiagTensor / IdenTensor ---------------------------------------

DiagTensorBase::DiagTensorBase(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, bool truncated)
    : SymmTensorBase(env, dis_dims, loc_dims, n_dis_in_dims), truncated_(truncated) {}
DiagTensorBase::DiagTensorBase(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, bool truncated,
                               BcParams params)
    : SymmTensorBase(env, dis_dims, loc_dims, n_dis_in_dims, params), truncated_(truncated) {}

DiagTensor* DiagTensorBase::toDiag() noexcept {
  const tidx_tup in = totInDims();
  const std::size_t n = utils::dims_to_size(in);
  std::vector<tel> d(n);
  const std::size_t ndi = n_dis_in_dims_, nd = dis_dims_.size(), nli = locInDims().size();
  for (std::size_t i = 0; i < n; ++i) {
    tidx_tup v = utils::i_to_idxs(i, in);
    tidx_tup tot(totDims().size());
    for (std::size_t j = 0; j < ndi; ++j) tot[j] = v[j];
    for (std::size_t j = 0; j < nli; ++j) tot[nd + j] = v[ndi + j];
    // outputs copy the inputs in order
    std::size_t k = 0;
    for (std::size_t j = ndi; j < nd; ++j) tot[j] = v[k++];
    for (std::size_t j = nd + nli; j < tot.size(); ++j) tot[j] = v[k++];
    d[i] = at(tot);
  }
  return new DiagTensor(bc_.env, dis_dims_, loc_dims_, n_dis_in_dims_, truncated_, std::move(d),
                        BcParams{bc_.str, bc_.cyc, bc_.off});
}

static std::size_t diag_size(const tidx_tup& dis, const tidx_tup& loc, tidx_tup_st ndi) {
  if (ndi > dis.size()) throw std::invalid_argument("diagonal tensor: distributed input count");
  const std::size_t nli = loc_in_count(loc, ndi);
  if (dis.size() - ndi + (loc.size() - nli) != ndi + nli)
    throw std::invalid_argument("diagonal tensor: input and output counts differ");
  std::size_t n = 1;
  for (std::size_t i = 0; i < ndi; ++i) n *= dis[i];
  for (std::size_t i = 0; i < nli; ++i) n *= loc[i];
  return n;
}

static std::vector<tel>&& checked_diag(std::vector<tel>&& d, const tidx_tup& dis, const tidx_tup& loc, tidx_tup_st ndi) {
  const std::size_t n = diag_size(dis, loc, ndi);
  if (d.size() != n)
    throw std::invalid_argument("diagonal element count " + std::to_string(d.size()) + " differs from " + std::to_string(n));
  return std::move(d);
}

DiagTensor::DiagTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, bool truncated,
                       std::vector<tel>&& diag_els)
    : DiagTensorBase(env, dis_dims, loc_dims, n_dis_in_dims, truncated),
      diag_(env, checked_diag(std::move(diag_els), dis_dims, loc_dims, n_dis_in_dims)) {}
DiagTensor::DiagTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, bool truncated,
                       std::vector<tel>&& diag_els, BcParams params)
    : DiagTensorBase(env, dis_dims, loc_dims, n_dis_in_dims, truncated, params),
      diag_(env, checked_diag(std::move(diag_els), dis_dims, loc_dims, n_dis_in_dims)) {}

std::unique_ptr<Tensor> DiagTensor::copy() const noexcept {
  auto d = diag_.to_host();
  return tptr(new DiagTensor(bc_.env, dis_dims_, loc_dims_, n_dis_in_dims_, truncated_, std::move(d),
                             BcParams{bc_.str, bc_.cyc, bc_.off}));
}

int DiagTensor::engineKind() const noexcept { return QTNH_KIND_DIAG; }

// Input and output index tuples of the symmetric split; true and the diagonal position
// when they are equal.
bool DiagTensor::diag_index(const tidx_tup& t, std::size_t& i) const {
  const tidx_tup dims = totDims();
  tot_index(t, dims);
  const std::size_t ndi = n_dis_in_dims_, nd = dis_dims_.size(), nli = locInDims().size();
  tidx_tup in, out, in_dims;
  for (std::size_t j = 0; j < ndi; ++j) in.push_back(t[j]), in_dims.push_back(dims[j]);
  for (std::size_t j = ndi; j < nd; ++j) out.push_back(t[j]);
  for (std::size_t j = 0; j < nli; ++j) in.push_back(t[nd + j]), in_dims.push_back(dims[nd + j]);
  for (std::size_t j = nd + nli; j < dims.size(); ++j) out.push_back(t[j]);
  if (in != out) return false;
  i = utils::idxs_to_i(in, in_dims);
  return true;
}

tel DiagTensor::at(tidx_tup tot_idxs) const {
  std::size_t i;
  return diag_index(tot_idxs, i) ? diag_.host_at(i) : tel(0.0);
}
tel DiagTensor::operator[](tidx_tup loc_idxs) const {
  return at(utils::concat_dims(utils::i_to_idxs(0, dis_dims_), loc_idxs));
}
tel& DiagTensor::at(tidx_tup tot_idxs) {
  std::size_t i;
  if (!diag_index(tot_idxs, i)) throw std::invalid_argument("element is off the diagonal");
  return diag_.host_ref(i);
}
void DiagTensor::put(tidx_tup tot_idxs, tel el) { at(tot_idxs) = el; }

DiagTensor* DiagTensor::rebcast(BcParams params) {
  bc_ = Broadcaster(bc_.env, bc_.base, params);
  return this;
}

IdenTensor::IdenTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, bool truncated)
    : DiagTensorBase(env, dis_dims, loc_dims, n_dis_in_dims, truncated) {}
IdenTensor::IdenTensor(const QTNHEnv& env, tidx_tup dis_dims, tidx_tup loc_dims, tidx_tup_st n_dis_in_dims, bool truncated,
                       BcParams params)
    : DiagTensorBase(env, dis_dims, loc_dims, n_dis_in_dims, truncated, params) {}

std::unique_ptr<Tensor> IdenTensor::copy() const noexcept {
  return tptr(new IdenTensor(bc_.env, dis_dims_, loc_dims_, n_dis_in_dims_, truncated_, BcParams{bc_.str, bc_.cyc, bc_.off}));
}

int IdenTensor::engineKind() const noexcept { return QTNH_KIND_IDEN; }

// src/tensor/diag.cpp:143-151.
tel IdenTensor::at(tidx_tup tot_idxs) const {
  tot_index(tot_idxs, totDims());
  const std::size_t h = tot_idxs.size() / 2;
  for (std::size_t i = 0; i < h; ++i)
    if (tot_idxs[i] != tot_idxs[h + i]) return 0.0;
  return 1.0;
}
tel IdenTensor::operator[](tidx_tup loc_idxs) const { return at(utils::concat_dims(utils::i_to_idxs(0, dis_dims_), loc_idxs)); }

IdenTensor* IdenTensor::rebcast(BcParams params) {
  bc_ = Broadcaster(bc_.env, bc_.base, params);
  return this;
}

// ---- contraction --------------------------------------------------------------------

// Tensor::contract (src/tensor/contract.cpp:204-313) through the C ABI. The result is a
// DenseTensor like the reference's (contract.cpp:200) with broadcast
// {product of contracted distributed dims, 1, min(off)}. When the result has the size of
// the first tensor its device buffer is reused (the first tensor is consumed).
//
// A SymmTensor gate or DiagTensor applied in place to a DenseTensor (qtnh_contract_inplace)
// is not run at once: it is queued on the state's device array (DeviceArray::defer), which
// applies queued runs as fused layers before the elements are next used. The metadata
// (dimension replacements, result dims, broadcaster) is the same either way.
tptr contract_on_device(tptr tp1, tptr tp2, ConParams& params) {
  const QTNHEnv& env = tp1->bc().env;
  const tidx_tup d1 = tp1->totDims(), d2 = tp2->totDims();
  auto u1 = u64(d1), u2 = u64(d2);
  // metadata first (host only): the element pointers are taken only when the work runs now
  qtnh_tensor_desc a{tp1->engineKind(), (int32_t)tp1->disDims().size(), (int32_t)tp1->locDims().size(),
                     tp1->engineDisIn(), u1.data(), nullptr};
  qtnh_tensor_desc b{tp2->engineKind(), (int32_t)tp2->disDims().size(), (int32_t)tp2->locDims().size(),
                     tp2->engineDisIn(), u2.data(), nullptr};
  std::vector<uint16_t> w;
  for (auto& x : params.wires) w.push_back(x.first), w.push_back(x.second);
  std::vector<uint16_t> r1(d1.size(), X), r2(d2.size(), X);
  if (!params.useDefRepls) {
    if (params.dimRepls1.size() != d1.size() || params.dimRepls2.size() != d2.size())
      throw std::out_of_range("dimension replacement tuple has the wrong size");
    std::copy(params.dimRepls1.begin(), params.dimRepls1.end(), r1.begin());
    std::copy(params.dimRepls2.begin(), params.dimRepls2.end(), r2.begin());
  }
  int32_t ndis = 0, nloc = 0, inplace = 0, ntg = 0;
  uint64_t str = 1;
  std::vector<uint64_t> od(d1.size() + d2.size() + 1);
  std::vector<uint16_t> targets(QTNH_MAX_RANK);
  check(qtnh_contract_inplace(&a, &b, (int32_t)params.wires.size(), w.data(), params.useDefRepls ? 1 : 0, r1.data(),
                              r2.data(), &ndis, &nloc, od.data(), &str, &inplace, &ntg, targets.data()));
  std::size_t nout = 1;
  for (int32_t i = 0; i < ndis + nloc; ++i) nout *= od[i];
  BcParams bp((qtnh::uint)str, 1, std::min(tp1->bc().off, tp2->bc().off));
  tidx_tup dis(od.begin(), od.begin() + ndis), loc(od.begin() + ndis, od.begin() + ndis + nloc);

  if (inplace && a.kind == QTNH_KIND_DENSE && nout == tp1->totSize()) {
    DeviceArray st = tp1->releaseStorage();
    DeviceArray op = tp2->releaseStorage();
    if (!st.empty() && !op.empty()) {
      st.defer(b.kind, std::vector<uint16_t>(targets.begin(), targets.begin() + ntg), u1, std::move(op));
      params.dimRepls1.assign(r1.begin(), r1.end());
      params.dimRepls2.assign(r2.begin(), r2.end());
      return tptr(new DenseTensor(env, dis, loc, std::move(st), bp));
    }
    throw std::logic_error("in-place contraction without element storage");
  }
  a.data = tp1->engineData();
  b.data = tp2->engineData();

  DeviceArray out;
  if (nout == tp1->totSize() && (a.kind == QTNH_KIND_DENSE || a.kind == QTNH_KIND_SYMM)) out = tp1->releaseStorage();
  if (out.empty()) out = DeviceArray(env, nout);
  check(qtnh_contract(&a, &b, (int32_t)params.wires.size(), w.data(), 0, r1.data(), r2.data(), &ndis, &nloc, od.data(), &str,
                      out.write(), nout, env.stream));
  params.dimRepls1.assign(r1.begin(), r1.end());
  params.dimRepls2.assign(r2.begin(), r2.end());
  return tptr(new DenseTensor(env, dis, loc, std::move(out), bp));
}

namespace ops {
std::ostream& operator<<(std::ostream& out, const Tensor& o) {
  if (!o.bc().active) return out << "Inactive";
  out << std::setprecision(2);
  const auto els = o.hostElements();
  const std::size_t slab = std::max<std::size_t>(o.locSize(), 1);
  for (std::size_t i = 0; i < els.size(); ++i) {
    out << els[i];
    if (i + 1 < els.size()) out << (((i + 1) % slab) ? ", " : " | ");
  }
  return out;
}
}  // namespace ops

}  // namespace qtnh
