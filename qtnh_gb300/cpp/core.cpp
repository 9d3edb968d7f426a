// QTNHEnv, utils, TIndexing and the device array behind every stored tensor.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <string>
#include <unordered_map>

#include "qtnh.hpp"
#include "qtnh_cuda.h"
#include "facade_internal.hpp"

namespace qtnh {

namespace detail {

void check(int rc) {
  if (rc == QTNH_OK) return;
  std::string msg = qtnh_last_error();
  switch (rc) {
    case QTNH_ERR_INVALID_ARGUMENT: throw std::invalid_argument(msg);
    case QTNH_ERR_OUT_OF_RANGE: throw std::out_of_range(msg);
    case QTNH_ERR_NO_MEMORY: throw std::bad_alloc();
    default: throw std::runtime_error(msg);
  }
}

// Host mirrors above this size are dropped after upload (re-read on demand).
static const std::size_t kKeepMirrorElems = (std::size_t)16 << 20;

// ---- in-place contractions queued on a tensor's elements ----------------------------
//
// Tensor::contract(state, gate, wires) with a SymmTensor gate or DiagTensor applied in
// place (the in-place rule, src/tensor/contract.cpp:250-289) is queued on the state's
// device array instead of running at once, and so is Tensor::permute of a DenseTensor
// (src/tensor/dense.cpp:152-169). The queue is applied when the elements are next needed:
// runs of gates and permutations through qtnh_apply_gate_runs (consecutive disjoint
// two-qubit gates share one pass over the state, and the fixed-point chain of the fused
// passes continues across the permutations, which move the elements between the array
// and a scratch buffer), runs of one-index diagonals through qtnh_apply_diag_layer (one
// pass), other diagonals one by one. The queue is keyed by the device pointer, which
// moves with the array; applying it may leave the elements in the scratch buffer, which
// the array then owns. QTNH_LAZY=0 turns queuing off.

// Kind of a queued permutation: targets hold the permutation tuple, no operand.
constexpr int kDeferPermute = -1;

struct DeferredOp {
  int kind;
  std::vector<uint16_t> targets;  // the wired indices, or the permutation tuple
  std::vector<uint64_t> dims;     // the elements' dims when the operation applies
  DeviceArray op;
};

struct DeferredQueue {
  const QTNHEnv* env = nullptr;
  std::vector<uint64_t> dims;  // the dims after every queued operation
  std::vector<DeferredOp> ops;
};

static std::mutex g_deferred_mu;
static std::unordered_map<const void*, DeferredQueue>& deferred_queues() {
  static std::unordered_map<const void*, DeferredQueue> q;
  return q;
}
static const std::size_t kMaxDeferred = 1024;  // applied once this many are queued

static void drop_queue(const void* dev) {
  if (!dev) return;
  DeferredQueue dead;
  {
    std::lock_guard<std::mutex> lk(g_deferred_mu);
    auto it = deferred_queues().find(dev);
    if (it == deferred_queues().end()) return;
    dead = std::move(it->second);
    deferred_queues().erase(it);
  }
}

// A one-index diagonal whose index was last touched, in queue order, by a gate is folded
// into that gate (qtnh_symm_diag_product, in place on the queued gate, which the
// contraction consumed): the diagonal commutes with everything between them, and the
// gate runs on both sides of it join into one fused run. A queued permutation between
// them maps the index back to its position before the permutation. Diagonals on an index
// whose last toucher is not a gate, or that no earlier queued operation touches, stay.
static void fold_diagonals(DeferredQueue& q) {
  void* st = q.env->stream;
  std::vector<char> gone(q.ops.size(), 0);
  for (std::size_t i = 0; i < q.ops.size(); ++i) {
    if (q.ops[i].kind != QTNH_KIND_DIAG || q.ops[i].targets.size() != 1) continue;
    uint16_t x = q.ops[i].targets[0];
    for (std::size_t j = i; j-- > 0;) {
      if (gone[j]) continue;
      const auto& tg = q.ops[j].targets;
      if (q.ops[j].kind == kDeferPermute) {  // old index k moved to tg[k]
        x = (uint16_t)(std::find(tg.begin(), tg.end(), x) - tg.begin());
        continue;
      }
      const auto it = std::find(tg.begin(), tg.end(), x);
      if (it == tg.end()) continue;
      if (q.ops[j].kind == QTNH_KIND_SYMM) {
        std::vector<uint64_t> td;
        for (uint16_t t : tg) td.push_back(q.ops[j].dims[t]);
        check(qtnh_symm_diag_product(q.ops[j].op.read(), (int32_t)tg.size(), td.data(), (int32_t)(it - tg.begin()),
                                     q.ops[i].op.read(), q.ops[j].op.write(), st));
        gone[i] = 1;
      }
      break;
    }
  }
  std::size_t k = 0;
  for (std::size_t i = 0; i < q.ops.size(); ++i)
    if (!gone[i]) {
      if (k != i) q.ops[k] = std::move(q.ops[i]);
      ++k;
    }
  q.ops.resize(k);
}

// Applies the queue to the elements at `cur`; permutations move them between cur and
// scratch (allocated on the first one), so cur ends where the result is.
static void apply_queue(void*& cur, void*& scratch, std::size_t n, DeferredQueue& q) {
  fold_diagonals(q);
  void* st = q.env->stream;
  std::size_t i = 0;
  while (i < q.ops.size()) {
    std::size_t j = i;
    const std::vector<uint64_t>& dims = q.ops[i].dims;
    const int32_t rank = (int32_t)dims.size();
    if (q.ops[i].kind == QTNH_KIND_SYMM || q.ops[i].kind == kDeferPermute) {
      // gates in runs separated by permutations, one call
      std::vector<int32_t> per_run(1, 0), ks;
      std::vector<uint16_t> tg, ptups;
      std::vector<const void*> ptrs;
      for (; j < q.ops.size() && (q.ops[j].kind == QTNH_KIND_SYMM || q.ops[j].kind == kDeferPermute); ++j) {
        const DeferredOp& o = q.ops[j];
        if (o.kind == kDeferPermute) {
          ptups.insert(ptups.end(), o.targets.begin(), o.targets.end());
          per_run.push_back(0);
          continue;
        }
        ++per_run.back();
        ks.push_back((int32_t)o.targets.size());
        tg.insert(tg.end(), o.targets.begin(), o.targets.end());
        ptrs.push_back(o.op.read());
      }
      const int32_t nruns = (int32_t)per_run.size();
      if (nruns == 1) {
        check(qtnh_apply_gate_layer(cur, rank, dims.data(), (int32_t)ks.size(), ks.data(), tg.data(), ptrs.data(), st));
      } else {
        if (!scratch) check(qtnh_malloc_async(&scratch, std::max<std::size_t>(n, 1) * sizeof(tel), st));
        check(qtnh_apply_gate_runs(cur, scratch, rank, dims.data(), nruns, per_run.data(), ks.data(), tg.data(),
                                   ptrs.data(), ptups.data(), st));
        if ((nruns - 1) % 2) std::swap(cur, scratch);
      }
    } else if (q.ops[i].targets.size() == 1) {
      while (j < q.ops.size() && q.ops[j].kind == QTNH_KIND_DIAG && q.ops[j].targets.size() == 1) ++j;
      if (j - i == 1) {
        check(qtnh_apply_diag(cur, rank, dims.data(), 1, q.ops[i].targets.data(), q.ops[i].op.read(), st));
      } else {
        // the one-index diagonals of the run, concatenated for one streaming pass
        std::vector<uint16_t> axes;
        std::size_t total = 0;
        for (std::size_t g = i; g < j; ++g) axes.push_back(q.ops[g].targets[0]), total += dims[q.ops[g].targets[0]];
        DeviceArray factors(*q.env, total);
        char* f = static_cast<char*>(factors.write());
        std::size_t off = 0;
        for (std::size_t g = i; g < j; ++g) {
          const std::size_t len = dims[q.ops[g].targets[0]];
          check(qtnh_memcpy_d2d(f + off * sizeof(tel), q.ops[g].op.read(), len * sizeof(tel), st));
          off += len;
        }
        check(qtnh_apply_diag_layer(cur, rank, dims.data(), (int32_t)axes.size(), axes.data(), factors.read(), st));
      }
    } else {
      ++j;
      check(qtnh_apply_diag(cur, rank, dims.data(), (int32_t)q.ops[i].targets.size(), q.ops[i].targets.data(),
                            q.ops[i].op.read(), st));
    }
    i = j;
  }
}

void DeviceArray::settle() const {
  if (!dev_) return;
  DeferredQueue q;
  {
    std::lock_guard<std::mutex> lk(g_deferred_mu);
    auto it = deferred_queues().find(dev_);
    if (it == deferred_queues().end()) return;
    q = std::move(it->second);
    deferred_queues().erase(it);
  }
  // the operands are freed (stream-ordered) after their kernels
  void* cur = dev_;
  void* scratch = nullptr;
  try {
    apply_queue(cur, scratch, n_, q);
  } catch (...) {
    if (scratch && scratch != dev_) qtnh_free_async(scratch, env_->stream);
    if (cur != dev_) qtnh_free_async(cur, env_->stream);  // (not reached: cur moves only after a call succeeded)
    throw;
  }
  if (cur != dev_) dev_ = cur;  // the elements ended in the scratch buffer: scratch is the old array
  if (scratch) qtnh_free_async(scratch, env_->stream);
}

static bool lazy_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("QTNH_LAZY");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  return on;
}

// Appends an operation on elements of dims `dims` (the tensor's current dims) that leaves
// them with dims `after`; returns the queue length.
static std::size_t enqueue(const void* dev, const QTNHEnv* env, DeferredOp&& op, const std::vector<uint64_t>& after) {
  std::lock_guard<std::mutex> lk(g_deferred_mu);
  DeferredQueue& q = deferred_queues()[dev];
  if (q.ops.empty()) {
    q.env = env;
  } else if (q.dims != op.dims) {
    throw std::logic_error("queued contractions on differently shaped elements");
  }
  q.dims = after;
  q.ops.push_back(std::move(op));
  return q.ops.size();
}

void DeviceArray::defer(int kind, const std::vector<uint16_t>& targets, const std::vector<uint64_t>& dims,
                        DeviceArray&& op) {
  if (!dev_) throw std::runtime_error("tensor has no storage");
  flush();  // host edits made so far come first
  host_valid_ = false;
  host_.clear();
  host_.shrink_to_fit();
  op.flush();
  const std::size_t queued = enqueue(dev_, env_, DeferredOp{kind, targets, dims, std::move(op)}, dims);
  if (queued >= kMaxDeferred || !lazy_enabled()) settle();
}

void DeviceArray::defer_permute(const std::vector<uint16_t>& ptup, const std::vector<uint64_t>& dims) {
  if (!dev_) throw std::runtime_error("tensor has no storage");
  std::vector<uint64_t> after(dims.size());
  std::vector<char> seen(dims.size(), 0);
  if (ptup.size() != dims.size()) throw std::invalid_argument("permutation tuple size differs from tensor rank");
  for (std::size_t i = 0; i < ptup.size(); ++i) {
    if (ptup[i] >= dims.size() || seen[ptup[i]]++) throw std::invalid_argument("permutation tuple is not a permutation");
    after[ptup[i]] = dims[i];
  }
  flush();
  host_valid_ = false;
  host_.clear();
  host_.shrink_to_fit();
  const std::size_t queued = enqueue(dev_, env_, DeferredOp{kDeferPermute, ptup, dims, DeviceArray()}, after);
  if (queued >= kMaxDeferred || !lazy_enabled()) settle();
}

DeviceArray::DeviceArray(const QTNHEnv& env, std::vector<tel>&& host) : env_(&env), n_(host.size()) {
  check(qtnh_malloc_async(&dev_, std::max<std::size_t>(n_, 1) * sizeof(tel), env.stream));
  if (n_) check(qtnh_memcpy_h2d(dev_, host.data(), n_ * sizeof(tel), env.stream));
  if (n_ <= kKeepMirrorElems) {
    host_ = std::move(host);
    host_valid_ = true;
  }
}

DeviceArray::DeviceArray(const QTNHEnv& env, std::size_t n) : env_(&env), n_(n) {
  check(qtnh_malloc_async(&dev_, std::max<std::size_t>(n_, 1) * sizeof(tel), env.stream));
}

DeviceArray::~DeviceArray() {
  drop_queue(dev_);
  if (dev_) qtnh_free_async(dev_, env_->stream);
}

DeviceArray::DeviceArray(DeviceArray&& o) noexcept
    : env_(o.env_), dev_(o.dev_), n_(o.n_), host_(std::move(o.host_)), host_valid_(o.host_valid_),
      host_dirty_(o.host_dirty_) {
  o.dev_ = nullptr;
  o.n_ = 0;
  o.host_valid_ = o.host_dirty_ = false;
}

DeviceArray& DeviceArray::operator=(DeviceArray&& o) noexcept {
  if (this != &o) {
    drop_queue(dev_);
    if (dev_) qtnh_free_async(dev_, env_->stream);
    env_ = o.env_;
    dev_ = o.dev_;
    n_ = o.n_;
    host_ = std::move(o.host_);
    host_valid_ = o.host_valid_;
    host_dirty_ = o.host_dirty_;
    o.dev_ = nullptr;
    o.n_ = 0;
    o.host_valid_ = o.host_dirty_ = false;
  }
  return *this;
}

void DeviceArray::flush() const {
  if (host_dirty_ && dev_) {
    check(qtnh_memcpy_h2d(dev_, host_.data(), n_ * sizeof(tel), env_->stream));
    check(qtnh_stream_synchronize(env_->stream));  // the mirror may change right after
    host_dirty_ = false;
  }
}

void DeviceArray::pull() const {
  settle();
  if (host_valid_) return;
  if (!dev_) throw std::runtime_error("tensor has no storage");
  host_.resize(n_);
  if (n_) check(qtnh_memcpy_d2h(host_.data(), dev_, n_ * sizeof(tel), env_->stream));
  check(qtnh_stream_synchronize(env_->stream));
  host_valid_ = true;
}

const void* DeviceArray::read() const {
  settle();
  flush();
  return dev_;
}

void* DeviceArray::write() {
  settle();
  flush();
  host_valid_ = false;
  host_.clear();
  host_.shrink_to_fit();
  return dev_;
}

const tel& DeviceArray::host_at(std::size_t i) const {
  pull();
  return host_.at(i);
}

tel& DeviceArray::host_ref(std::size_t i) {
  pull();
  tel& r = host_.at(i);
  host_dirty_ = true;
  return r;
}

std::vector<tel> DeviceArray::to_host() const {
  pull();
  return host_;
}

DeviceArray DeviceArray::clone() const {
  DeviceArray c(*env_, n_);
  settle();
  flush();
  if (n_) check(qtnh_memcpy_d2d(c.dev_, dev_, n_ * sizeof(tel), env_->stream));
  if (host_valid_ && !host_dirty_) {
    c.host_ = host_;
    c.host_valid_ = true;
  }
  return c;
}

}  // namespace detail

QTNHEnv::QTNHEnv() : proc_id(0), num_processes(1), device(0), stream(nullptr) {
  int n = 0;
  detail::check(qtnh_device_count(&n));
  if (n == 0) throw std::runtime_error("QTNHEnv: no CUDA device is visible");
  if (const char* d = std::getenv("QTNH_DEVICE")) device = std::atoi(d);
  detail::check(qtnh_set_device(device));
  detail::check(qtnh_stream_create(&stream));
}

QTNHEnv::~QTNHEnv() {
  if (stream) {
    qtnh_stream_synchronize(stream);
    qtnh_stream_destroy(stream);
  }
}

void QTNHEnv::synchronize() const { detail::check(qtnh_stream_synchronize(stream)); }

void QTNHEnv::print() const {
  std::cout << "Process ID: " << proc_id << std::endl;
  std::cout << "Process count: " << num_processes << std::endl;
  std::cout << "Device: " << device << std::endl;
}

namespace utils {

void throw_unimplemented() { throw std::runtime_error("Unimplemented function!"); }

bool is_root() { return true; }

void barrier() { detail::check(qtnh_device_synchronize()); }

std::size_t dims_to_size(qtnh::tidx_tup dims) {
  std::size_t s = 1;
  for (auto d : dims) s *= d;
  return s;
}

std::size_t idxs_to_i(qtnh::tidx_tup idxs, qtnh::tidx_tup dims) {
  std::size_t i = 0, base = 1;
  for (int j = (int)idxs.size() - 1; j >= 0; --j) {
    i += idxs.at(j) * base;
    base *= dims.at(j);
  }
  return i;
}

qtnh::tidx_tup i_to_idxs(std::size_t i, qtnh::tidx_tup dims) {
  qtnh::tidx_tup idxs(dims.size());
  for (int j = (int)dims.size() - 1; j >= 0; --j) {
    idxs.at(j) = i % dims.at(j);
    i /= dims.at(j);
  }
  return idxs;
}

qtnh::tidx_tup concat_dims(qtnh::tidx_tup dims1, qtnh::tidx_tup dims2) {
  dims1.insert(dims1.end(), dims2.begin(), dims2.end());
  return dims1;
}

std::pair<qtnh::tidx_tup, qtnh::tidx_tup> split_dims(qtnh::tidx_tup dims, qtnh::tidx_tup_st n) {
  if (n > dims.size()) throw std::out_of_range("split_dims: position beyond the tuple");
  return {qtnh::tidx_tup(dims.begin(), dims.begin() + n), qtnh::tidx_tup(dims.begin() + n, dims.end())};
}

std::vector<qtnh::wire> invert_wires(std::vector<qtnh::wire> ws) {
  for (auto& w : ws) std::swap(w.first, w.second);
  return ws;
}

bool equal(qtnh::tel a, qtnh::tel b, double tol) {
  const double dr = a.real() - b.real(), di = a.imag() - b.imag();
  return std::sqrt(dr * dr + di * di) < tol;
}

}  // namespace utils

// ---- TIndexing ---------------------------------------------------------------------

namespace ops {
std::ostream& operator<<(std::ostream& out, const qtnh::tidx_tup& o) {
  out << "(";
  for (std::size_t i = 0; i < o.size(); ++i) out << o[i] << (i + 1 < o.size() ? ", " : "");
  return out << ")";
}
std::ostream& operator<<(std::ostream& out, const TIFlag& o) { return out << "(" << o.tag << ", " << o.label << ")"; }
}  // namespace ops

// Fastest-first order: descending tag; among equal tags the last index first.
static std::vector<std::size_t> order_of(const std::vector<TIFlag>& ifls) {
  std::vector<std::size_t> m(ifls.size());
  std::iota(m.begin(), m.end(), 0);
  std::stable_sort(m.begin(), m.end(), [&](std::size_t a, std::size_t b) { return ifls[a].tag < ifls[b].tag; });
  std::reverse(m.begin(), m.end());
  return m;
}

TIndexing::TIndexing(qtnh::tidx_tup dims) : TIndexing(dims, std::vector<TIFlag>(dims.size(), {"default", 0})) {}
TIndexing::TIndexing(qtnh::tidx_tup dims, std::vector<TIFlag> ifls) : dims_(dims), ifls_(ifls), maps_(order_of(ifls_)) {}

bool TIndexing::isValid(qtnh::tidx_tup idxs) const {
  if (idxs.size() != dims_.size()) return false;
  for (std::size_t i = 0; i < idxs.size(); ++i)
    if (idxs[i] >= dims_[i]) return false;
  return true;
}

bool TIndexing::isEqual(qtnh::tidx_tup a, qtnh::tidx_tup b, std::string label) const {
  for (std::size_t i = 0; i < a.size(); ++i)
    if (ifls_.at(i).label == label && a[i] != b.at(i)) return false;
  return true;
}

bool TIndexing::isLast(qtnh::tidx_tup idxs, std::string label) const {
  for (std::size_t i = 0; i < idxs.size(); ++i)
    if (ifls_.at(i).label == label && idxs[i] != dims_.at(i) - 1) return false;
  return true;
}

qtnh::tidx_tup TIndexing::next(qtnh::tidx_tup idxs, std::string label) const {
  for (std::size_t i = 0; i < idxs.size(); ++i) {
    std::size_t k = maps_.at(i);
    if (ifls_.at(k).label != label) continue;
    if (idxs.at(k) < dims_.at(k) - 1) {
      ++idxs[k];
      return idxs;
    }
    if (idxs[k] == dims_[k] - 1) {
      idxs[k] = 0;
      continue;
    }
    break;
  }
  throw std::out_of_range("Tuple is outside of indexing.");
}

qtnh::tidx_tup TIndexing::prev(qtnh::tidx_tup idxs, std::string label) const {
  for (std::size_t i = 0; i < idxs.size(); ++i) {
    std::size_t k = maps_.at(i);
    if (ifls_.at(k).label != label) continue;
    if (idxs.at(k) == 0) {
      idxs[k] = dims_.at(k) - 1;
      continue;
    }
    if (idxs[k] < dims_.at(k)) {
      --idxs[k];
      return idxs;
    }
    break;
  }
  throw std::out_of_range("Tuple is outside of indexing.");
}

qtnh::tidx_tup TIndexing::reset(qtnh::tidx_tup idxs, std::string label) const {
  for (std::size_t i = 0; i < idxs.size(); ++i)
    if (ifls_.at(i).label == label) idxs[i] = 0;
  return idxs;
}

TIndexing TIndexing::cut(std::string label) const {
  qtnh::tidx_tup d;
  std::vector<TIFlag> f;
  for (std::size_t i = 0; i < dims_.size(); ++i)
    if (ifls_[i].label != label) d.push_back(dims_[i]), f.push_back(ifls_[i]);
  return TIndexing(d, f);
}

TIndexing TIndexing::keep(std::string label) const {
  qtnh::tidx_tup d;
  std::vector<TIFlag> f;
  for (std::size_t i = 0; i < dims_.size(); ++i)
    if (ifls_[i].label == label) d.push_back(dims_[i]), f.push_back(ifls_[i]);
  return TIndexing(d, f);
}

TIndexing::TupIterator::TupIterator(qtnh::tidx_tup dims, std::vector<std::size_t> order, qtnh::tidx_tup start, bool is_end)
    : dims_(dims), order_(order), current_(start), is_end_(is_end) {}

TIndexing::TupIterator TIndexing::TupIterator::begin() {
  auto s = current_;
  for (auto k : order_) s.at(k) = 0;
  return TupIterator(dims_, order_, s, false);
}

TIndexing::TupIterator TIndexing::TupIterator::end() { return TupIterator(dims_, order_, current_, true); }

TIndexing::TupIterator& TIndexing::TupIterator::operator++() {
  for (auto k : order_) {
    if (current_.at(k) < dims_.at(k) - 1) {
      ++current_[k];
      return *this;
    }
    if (current_[k] == dims_[k] - 1) current_[k] = 0;
  }
  is_end_ = true;
  return *this;
}

TIndexing::TupIterator TIndexing::TupIterator::operator++(int) {
  auto old = *this;
  ++*this;
  return old;
}

TIndexing::NumIterator::NumIterator(qtnh::tidx_tup dims, std::vector<std::size_t> incrs, std::size_t zero,
                                    qtnh::tidx_tup current_idxs, bool is_end)
    : dims_(dims), incrs_(incrs), zero_(zero), current_idxs_(current_idxs), is_end_(is_end) {}

TIndexing::NumIterator TIndexing::NumIterator::begin() {
  return NumIterator(dims_, incrs_, zero_, qtnh::tidx_tup(current_idxs_.size(), 0), false);
}

TIndexing::NumIterator TIndexing::NumIterator::end() { return NumIterator(dims_, incrs_, zero_, current_idxs_, true); }

TIndexing::NumIterator& TIndexing::NumIterator::operator++() {
  for (std::size_t i = 0; i < current_idxs_.size(); ++i) {
    if (current_idxs_[i] < dims_.at(i) - 1) {
      ++current_idxs_[i];
      return *this;
    }
    if (current_idxs_[i] == dims_[i] - 1) current_idxs_[i] = 0;
  }
  is_end_ = true;
  return *this;
}

TIndexing::NumIterator TIndexing::NumIterator::operator++(int) {
  auto old = *this;
  ++*this;
  return old;
}

std::size_t TIndexing::NumIterator::operator*() const {
  std::size_t r = zero_;
  for (std::size_t i = 0; i < current_idxs_.size(); ++i) r += current_idxs_[i] * incrs_.at(i);
  return r;
}

TIndexing::TupIterator TIndexing::tup(std::string label) const { return tup(label, qtnh::tidx_tup(dims_.size(), 0)); }

TIndexing::TupIterator TIndexing::tup(std::string label, qtnh::tidx_tup start) const {
  std::vector<std::size_t> order;
  for (auto k : maps_)
    if (ifls_.at(k).label == label) order.push_back(k);
  return TupIterator(dims_, order, start, false);
}

TIndexing::NumIterator TIndexing::num(std::string label) const { return num(label, qtnh::tidx_tup(dims_.size(), 0)); }

TIndexing::NumIterator TIndexing::num(std::string label, qtnh::tidx_tup start) const {
  const std::size_t n = dims_.size();
  std::vector<std::size_t> all(n);
  std::size_t zero = 0, base = 1;
  for (std::size_t i = 0; i < n; ++i) {
    std::size_t k = n - i - 1;
    all[k] = base;
    if (ifls_.at(k).label != label) zero += start.at(k) * base;
    base *= dims_[k];
  }
  qtnh::tidx_tup d, cur;
  std::vector<std::size_t> inc;
  for (auto k : maps_)
    if (ifls_.at(k).label == label) d.push_back(dims_[k]), inc.push_back(all[k]), cur.push_back(start.at(k));
  return NumIterator(d, inc, zero, cur, false);
}

TIndexing TIndexing::_app(const TIndexing& a, const TIndexing& b) {
  auto d = a.dims_;
  auto f = a.ifls_;
  d.insert(d.end(), b.dims_.begin(), b.dims_.end());
  f.insert(f.end(), b.ifls_.begin(), b.ifls_.end());
  return TIndexing(d, f);
}

}  // namespace qtnh
