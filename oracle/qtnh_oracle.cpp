// ORACLE — test infrastructure only.
//
// A CPU restatement of qtnh's tensor-contraction engine at world size 1 with every
// slab of a tensor resident in one host array: global row-major order over
// dis_dims ++ loc_dims (the distributed prefix is the slowest-varying block index,
// exactly the concatenation of the ranks' local vectors in rank order when
// str = cyc = 1, off = 0).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library, and only as the checker or as the timed CPU baseline ("port"). Nothing
// in the product (qtnh_gb300/, include/) links, loads or calls it.
//
// Each function cites the reference file:line it restates (paths relative to the
// reference project root). Arithmetic is plain scalar std::complex<double>, the same
// element type and product the reference uses (src/tensor/contract.cpp:149).
//
// Parity pinning: tests/test_oracle_golden.py checks this oracle against every
// golden vector of the reference's own test-suite (tests/gen/random-tensors.hpp and
// tests/gen/random-tn.hpp, extracted by tests/golden/make_golden.py).

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace orc {

using cplx = std::complex<double>;
using dims_t = std::vector<uint64_t>;

enum Kind : int32_t { DENSE = 0, SYMM = 1, SWAP = 2, IDEN = 3, DIAG = 4 };

enum Err : int32_t {
  OK = 0,
  ERR_INVALID_ARGUMENT = 1,  // std::invalid_argument in the reference
  ERR_RUNTIME = 2,           // std::runtime_error in the reference
  ERR_OUT_OF_RANGE = 3,      // std::out_of_range in the reference
  ERR_CAPACITY = 4,          // output buffer too small (query protocol)
  ERR_INTERNAL = 5,
};

static thread_local std::string g_last_error;

struct Tensor {
  int32_t kind = DENSE;
  dims_t dis, loc;
  int32_t n_dis_in = 0;
  std::vector<cplx> els;  // dense/symm: all elements; diag: diagonal over totInDims; swap/iden: empty
  uint32_t str = 1, cyc = 1, off = 0;

  dims_t tot() const {
    dims_t t = dis;
    t.insert(t.end(), loc.begin(), loc.end());
    return t;
  }
};

// src/core/utils.cpp:23-25
static uint64_t dims_to_size(const dims_t& d) {
  uint64_t s = 1;
  for (auto x : d) s *= x;
  return s;
}

// src/core/utils.cpp:27-36 (row-major, last index fastest)
static uint64_t idxs_to_i(const dims_t& idxs, const dims_t& dims) {
  uint64_t i = 0, base = 1;
  for (int j = (int)idxs.size() - 1; j >= 0; --j) {
    i += idxs.at(j) * base;
    base *= dims.at(j);
  }
  return i;
}

// src/core/utils.cpp:38-46
static dims_t i_to_idxs(uint64_t i, const dims_t& dims) {
  dims_t idxs(dims.size());
  for (int j = (int)dims.size() - 1; j >= 0; --j) {
    idxs.at(j) = i % dims.at(j);
    i /= dims.at(j);
  }
  return idxs;
}

static dims_t row_strides(const dims_t& dims) {
  dims_t s(dims.size(), 1);
  for (int i = (int)dims.size() - 2; i >= 0; --i) s[i] = s[i + 1] * dims[i + 1];
  return s;
}

// include/tensor/symm.hpp:22-45: in/out split of a symmetric tensor.
// locInDims takes loc[0 : loc.size()/2 - n_dis_in]; the reference forms the range
// without a check (it underflows when loc.size()/2 < n_dis_in), here that throws.
static uint64_t n_loc_in(const Tensor& t) {
  uint64_t half = t.loc.size() / 2;
  if (half < (uint64_t)t.n_dis_in) throw std::out_of_range("symmetric tensor: local input range underflows");
  return half - t.n_dis_in;
}

// Element of an implicit / compressed tensor at total indices.
//   SwapTensor: src/tensor/symm.cpp:584-591   (t0 == t3 && t1 == t2)
//   IdenTensor: src/tensor/diag.cpp:143-151   (first half of tot == second half)
//   DiagTensor: the reference stubs it (src/tensor/diag.cpp:65-117 throw). The element
//               is defined by its documentation (include/tensor/diag.hpp:11-14,
//               README.md:52): D[in, out] = d[in] if in == out else 0, with the in/out
//               split of the symmetric family (include/tensor/symm.hpp:22-45).
static cplx implicit_at(const Tensor& t, const dims_t& tot) {
  switch (t.kind) {
    case SWAP:
      return (tot.at(0) == tot.at(3) && tot.at(1) == tot.at(2)) ? cplx(1.0) : cplx(0.0);
    case IDEN: {
      size_t h = tot.size() / 2;
      for (size_t i = 0; i < h; ++i)
        if (tot[i] != tot[h + i]) return 0.0;
      return 1.0;
    }
    case DIAG: {
      uint64_t nli = n_loc_in(t);
      size_t ndi = t.n_dis_in, nd = t.dis.size();
      dims_t in_idx, out_idx, in_dims;
      for (size_t i = 0; i < ndi; ++i) in_idx.push_back(tot[i]), in_dims.push_back(t.dis[i]);
      for (size_t i = ndi; i < nd; ++i) out_idx.push_back(tot[i]);
      for (size_t i = 0; i < nli; ++i) in_idx.push_back(tot[nd + i]), in_dims.push_back(t.loc[i]);
      for (size_t i = nli; i < t.loc.size(); ++i) out_idx.push_back(tot[nd + i]);
      if (in_idx != out_idx) return 0.0;
      return t.els.at(idxs_to_i(in_idx, in_dims));
    }
    default:
      return t.els.at(idxs_to_i(tot, t.tot()));
  }
}

// Dense form of any tensor kind (the reference converts every operand through
// DenseTensorBase::toDense before the local loop: src/tensor/dense.cpp:19-37,
// reached from Tensor::permute in _contract_dense STEP 1, contract.cpp:46-47).
static std::vector<cplx> dense_elements(const Tensor& t) {
  if (t.kind == DENSE || t.kind == SYMM) return t.els;
  dims_t dims = t.tot();
  uint64_t n = dims_to_size(dims);
  std::vector<cplx> out(n);
  dims_t idx(dims.size(), 0);
  for (uint64_t i = 0; i < n; ++i) {
    out[i] = implicit_at(t, idx);
    for (int k = (int)dims.size() - 1; k >= 0; --k) {
      if (++idx[k] < dims[k]) break;
      idx[k] = 0;
    }
  }
  return out;
}

// Axis permutation, src/tensor/dense.cpp:354-488 and 152-169: old axis i moves to new
// position ptup[i]; new_dims[ptup[i]] = old_dims[i] (dense.cpp:367-369) and the element
// at old index tuple o lands at new tuple n with n[ptup[i]] = o[i] (the send/recv
// datatypes of dense.cpp:383-394 walk the same axis in both layouts).
static void permute(const cplx* in, cplx* out, const dims_t& dims, const std::vector<uint16_t>& ptup) {
  size_t r = dims.size();
  if (ptup.size() != r) throw std::invalid_argument("permutation tuple size differs from tensor rank");
  std::vector<bool> seen(r, false);
  for (auto p : ptup) {
    if (p >= r || seen[p]) throw std::invalid_argument("permutation tuple is not a permutation");
    seen[p] = true;
  }
  dims_t new_dims(r);
  for (size_t i = 0; i < r; ++i) new_dims[ptup[i]] = dims[i];
  dims_t ns = row_strides(new_dims);
  dims_t ostride_new(r);  // stride in the new array of old axis i
  for (size_t i = 0; i < r; ++i) ostride_new[i] = ns[ptup[i]];
  uint64_t n = dims_to_size(dims);
  dims_t idx(r, 0);
  uint64_t off = 0;
  for (uint64_t i = 0; i < n; ++i) {
    out[off] = in[i];
    for (int k = (int)r - 1; k >= 0; --k) {
      if (++idx[k] < dims[k]) {
        off += ostride_new[k];
        break;
      }
      off -= (dims[k] - 1) * ostride_new[k];
      idx[k] = 0;
    }
  }
}

// TIndexing iteration order, src/tensor/indexing.cpp:27-35 (_generate_maps): indices are
// stable-sorted by tag ascending and the order is reversed, so the first entry (the
// fastest-varying index) has the largest tag, and among equal tags the last index.
static std::vector<size_t> iteration_order(const std::vector<int>& tags) {
  std::vector<size_t> maps(tags.size());
  std::iota(maps.begin(), maps.end(), 0);
  std::stable_sort(maps.begin(), maps.end(), [&](size_t i, size_t j) { return tags[i] < tags[j]; });
  std::reverse(maps.begin(), maps.end());
  return maps;
}

struct ConParams {
  std::vector<std::pair<uint16_t, uint16_t>> wires;
  bool use_def = true;
  std::vector<uint16_t> repls1, repls2;
};

static bool wire_first(const std::pair<uint16_t, uint16_t>& a, const std::pair<uint16_t, uint16_t>& b) { return a.first < b.first; }
static bool wire_second(const std::pair<uint16_t, uint16_t>& a, const std::pair<uint16_t, uint16_t>& b) { return a.second < b.second; }

static constexpr uint16_t X = UINT16_MAX;  // include/core/typedefs.hpp:55

// Tensor::contract, src/tensor/contract.cpp:204-313, followed by the global form of
// _contract_dense (contract.cpp:12-201).
static Tensor contract(const Tensor& t1, const Tensor& t2, ConParams& params) {
  dims_t tot1 = t1.tot(), tot2 = t2.tot();
  size_t nd1 = t1.dis.size(), nd2 = t2.dis.size();
  size_t n_dis_ws = 0;

  // contract.cpp:207-217 — validation.
  for (auto& w : params.wires) {
    if (tot1.at(w.first) != tot2.at(w.second)) throw std::invalid_argument("Incompatible contraction dimensions.");
    if ((w.first < nd1) != (w.second < nd2)) throw std::invalid_argument("Attempted to contract distributed and local dimensions.");
    if (w.first < nd1) ++n_dis_ws;
  }
  {  // A self-contraction (one index wired twice) is undefined in the reference; refuse it.
    std::vector<int> u1(tot1.size(), 0), u2(tot2.size(), 0);
    for (auto& w : params.wires)
      if (u1[w.first]++ || u2[w.second]++) throw std::invalid_argument("An index is wired more than once.");
  }

  // contract.cpp:220-248 — default dimension replacements.
  if (params.use_def) {
    params.repls1.assign(tot1.size(), X);
    std::sort(params.wires.begin(), params.wires.end(), wire_first);
    for (size_t i = 0, j = 0; i < tot1.size(); ++i) {
      if (j < params.wires.size() && i == params.wires[j].first) {
        ++j;
      } else {
        params.repls1[i] = (uint16_t)(i - j);
        if (i >= nd1) params.repls1[i] += (uint16_t)(nd2 - n_dis_ws);
      }
    }
    params.repls2.assign(tot2.size(), X);
    std::sort(params.wires.begin(), params.wires.end(), wire_second);
    for (size_t i = 0, j = 0; i < tot2.size(); ++i) {
      if (j < params.wires.size() && i == params.wires[j].second) {
        ++j;
      } else {
        params.repls2[i] = (uint16_t)(nd1 - n_dis_ws + i - j);
        if (i >= nd2) params.repls2[i] = (uint16_t)(tot1.size() - params.wires.size() + i - j);
      }
    }
  }

  // contract.cpp:250-289 — in-place rule for symmetric second operands.
  if (t2.kind != DENSE) {
    size_t ndi = t2.n_dis_in, nli = n_loc_in(t2);
    size_t input_count = 0;
    for (auto& w : params.wires)
      if (w.second < ndi || (w.second >= nd2 && w.second < nd2 + nli)) ++input_count;
    int dis_imbal = (int)ndi - (int)(nd2 - ndi);
    if (dis_imbal == 0 && input_count == ndi + nli) {
      params.repls1.assign(tot1.size(), X);
      std::sort(params.wires.begin(), params.wires.end(), wire_first);
      for (size_t i = 0, j = 0; i < tot1.size(); ++i) {
        if (j < params.wires.size() && i == params.wires[j].first) ++j;
        else params.repls1[i] = (uint16_t)i;
      }
      params.repls2.assign(tot2.size(), X);
      std::sort(params.wires.begin(), params.wires.end(), wire_second);
      std::vector<uint16_t> from_dims(params.wires.size());
      for (size_t i = 0; i < params.wires.size(); ++i) from_dims[i] = params.wires[i].first;
      for (size_t i = 0, j = 0, k = 0; i < tot2.size(); ++i) {
        if (j < params.wires.size() && i == params.wires[j].second) ++j;
        else if (k < params.wires.size()) params.repls2[i] = from_dims[k++];
      }
    }
  }

  // _contract_dense (contract.cpp:12-201), global form.
  auto ws = params.wires;
  std::sort(ws.begin(), ws.end(), wire_second);  // contract.cpp:26
  if (params.repls1.size() != tot1.size() || params.repls2.size() != tot2.size())
    throw std::out_of_range("dimension replacement tuple has the wrong size");

  std::vector<int> role1(tot1.size(), -1), role2(tot2.size(), -1);  // wire number (sorted by second) or -1
  for (size_t i = 0; i < ws.size(); ++i) role1[ws[i].first] = (int)i, role2[ws[i].second] = (int)i;

  size_t n_open_dis = (nd1 - n_dis_ws) + (nd2 - n_dis_ws);
  size_t n_out = tot1.size() + tot2.size() - 2 * ws.size();
  dims_t out_dims(n_out, 0);
  std::vector<int> filled(n_out, 0);
  // Output position of every open index is its dimension replacement: the dis part goes
  // through ptup3 (contract.cpp:181-194), the local part through ptup_loc
  // (contract.cpp:86-111). A replacement that crosses the dis/loc border or repeats is
  // undefined in the reference; refuse it.
  auto place = [&](uint16_t pos, uint64_t dim, bool is_dis) {
    if (pos >= n_out) throw std::out_of_range("dimension replacement out of range");
    if (is_dis != (pos < n_open_dis)) throw std::invalid_argument("dimension replacement crosses the distributed/local border");
    if (filled[pos]++) throw std::invalid_argument("dimension replacement repeats a position");
    out_dims[pos] = dim;
  };
  for (size_t i = 0; i < tot1.size(); ++i)
    if (role1[i] < 0) place(params.repls1[i], tot1[i], i < nd1);
  for (size_t i = 0; i < tot2.size(); ++i)
    if (role2[i] < 0) place(params.repls2[i], tot2[i], i < nd2);

  std::vector<cplx> a = dense_elements(t1), b = dense_elements(t2);
  dims_t s1 = row_strides(tot1), s2 = row_strides(tot2), s3 = row_strides(out_dims);

  // Open index lists (original order) with their output strides.
  struct Open { uint64_t dim, in_stride, out_stride; };
  std::vector<Open> open1, open2;
  for (size_t i = 0; i < tot1.size(); ++i)
    if (role1[i] < 0) open1.push_back({tot1[i], s1[i], s3[params.repls1[i]]});
  for (size_t i = 0; i < tot2.size(); ++i)
    if (role2[i] < 0) open2.push_back({tot2[i], s2[i], s3[params.repls2[i]]});

  // Summed indices. Local wires ("closed", contract.cpp:76-77) iterate in TIndexing
  // order with tag = wire number (largest tag fastest, indexing.cpp:27-35). Distributed
  // wires ("reduced", contract.cpp:73-74) are summed by MPI_Allreduce over ranks
  // (contract.cpp:176); here their partial sums are added in rank (row-major) order.
  struct Sum { uint64_t dim, st1, st2; };
  std::vector<Sum> closed, reduced;
  {
    std::vector<int> tags;
    std::vector<size_t> loc_w;
    for (size_t i = 0; i < ws.size(); ++i)
      if (ws[i].first >= nd1) loc_w.push_back(i), tags.push_back((int)i);
    auto order = iteration_order(tags);
    for (auto k : order) {
      auto& w = ws[loc_w[k]];
      closed.push_back({tot1[w.first], s1[w.first], s2[w.second]});
    }
    for (size_t i = 0; i < ws.size(); ++i)
      if (ws[i].first < nd1) reduced.push_back({tot1[ws[i].first], s1[ws[i].first], s2[ws[i].second]});
  }

  uint64_t n3 = dims_to_size(out_dims);
  std::vector<cplx> c(n3, cplx(0.0));
  uint64_t n_open1 = 1, n_open2 = 1, n_closed = 1, n_red = 1;
  for (auto& o : open1) n_open1 *= o.dim;
  for (auto& o : open2) n_open2 *= o.dim;
  for (auto& s : closed) n_closed *= s.dim;
  for (auto& s : reduced) n_red *= s.dim;

  auto decode = [](uint64_t i, const auto& v, auto get_dim, auto on_digit) {
    for (int k = (int)v.size() - 1; k >= 0; --k) {
      uint64_t d = get_dim(v[k]);
      on_digit(k, i % d);
      i /= d;
    }
  };
  // Loop order: t1 open indices outer, t2 open indices inner (contract.cpp:133-134).
  for (uint64_t p1 = 0; p1 < n_open1; ++p1) {
    uint64_t off_a = 0, off_c1 = 0;
    decode(p1, open1, [](const Open& o) { return o.dim; }, [&](int k, uint64_t v) { off_a += v * open1[k].in_stride; off_c1 += v * open1[k].out_stride; });
    for (uint64_t p2 = 0; p2 < n_open2; ++p2) {
      uint64_t off_b = 0, off_c = off_c1;
      decode(p2, open2, [](const Open& o) { return o.dim; }, [&](int k, uint64_t v) { off_b += v * open2[k].in_stride; off_c += v * open2[k].out_stride; });
      cplx total = 0.0;
      for (uint64_t r = 0; r < n_red; ++r) {
        uint64_t ra = off_a, rb = off_b;
        decode(r, reduced, [](const Sum& s) { return s.dim; }, [&](int k, uint64_t v) { ra += v * reduced[k].st1; rb += v * reduced[k].st2; });
        cplx el3 = 0.0;
        // closed[0] is the fastest-varying index.
        for (uint64_t q = 0; q < n_closed; ++q) {
          uint64_t qa = ra, qb = rb, rem = q;
          for (size_t k = 0; k < closed.size(); ++k) {
            uint64_t v = rem % closed[k].dim;
            rem /= closed[k].dim;
            qa += v * closed[k].st1;
            qb += v * closed[k].st2;
          }
          el3 += a[qa] * b[qb];
        }
        total = (r == 0) ? el3 : total + el3;
      }
      c[off_c] = total;
    }
  }

  Tensor t3;
  t3.kind = DENSE;
  t3.dis.assign(out_dims.begin(), out_dims.begin() + n_open_dis);
  t3.loc.assign(out_dims.begin() + n_open_dis, out_dims.end());
  t3.els = std::move(c);
  // contract.cpp:59-63 and 196-200: result broadcast {prod(virtual dims), 1, min(off)}.
  uint64_t virt = 1;
  for (auto& w : ws)
    if (w.first < nd1) virt *= tot1[w.first];
  t3.str = (uint32_t)virt;
  t3.cyc = 1;
  t3.off = std::min(t1.off, t2.off);
  return t3;
}

// TensorNetwork, src/tensor/network.cpp:1-170. IDs come from process-wide counters
// (include/tensor/network.hpp:97-98) and maps are std::unordered_map, so that
// contractAll() visits bonds in the same order as the reference built with the same
// standard library.
struct Bond {
  std::pair<uint32_t, uint32_t> tids;
  std::vector<std::pair<uint16_t, uint16_t>> wires;
};
static uint32_t g_tensor_counter = 0, g_bond_counter = 0;

struct Network {
  std::unordered_map<uint32_t, Tensor> tensors;
  std::unordered_map<uint32_t, Bond> bonds;

  uint32_t insert(Tensor t) {
    tensors.insert({++g_tensor_counter, std::move(t)});
    return g_tensor_counter;
  }
  uint32_t add_bond(uint32_t a, uint32_t b, std::vector<std::pair<uint16_t, uint16_t>> ws) {
    bonds.insert({++g_bond_counter, Bond{{a, b}, std::move(ws)}});
    return g_bond_counter;
  }
  // network.cpp:60-106
  uint32_t contract_bond(uint32_t bid) {
    auto& b = bonds.at(bid);
    auto [tid1, tid2] = b.tids;
    ConParams params;
    params.wires = b.wires;
    Tensor t3 = contract(tensors.at(tid1), tensors.at(tid2), params);
    bonds.erase(bid);
    tensors.erase(tid1);
    tensors.erase(tid2);
    uint32_t tid3 = insert(std::move(t3));
    for (auto& [id, bb] : bonds) {
      if (bb.tids.first == tid1) {
        bb.tids.first = tid3;
        for (auto& w : bb.wires) w.first = params.repls1.at(w.first);
      } else if (bb.tids.first == tid2) {
        bb.tids.first = tid3;
        for (auto& w : bb.wires) w.first = params.repls2.at(w.first);
      }
      if (bb.tids.second == tid1) {
        bb.tids.second = tid3;
        for (auto& w : bb.wires) w.second = params.repls1.at(w.second);
      } else if (bb.tids.second == tid2) {
        bb.tids.second = tid3;
        for (auto& w : bb.wires) w.second = params.repls2.at(w.second);
      }
    }
    return tid3;
  }
  // network.cpp:108-126
  uint32_t contract_all() {
    uint32_t tid = tensors.begin()->first;
    auto temp = bonds;
    for (auto& [bid, b] : temp) tid = contract_bond(bid);
    return tid;
  }
  // network.cpp:128-170
  uint32_t contract_all(const std::vector<uint32_t>& order) {
    uint32_t tid = tensors.begin()->first;
    for (size_t i = 0, j = 1; i < order.size(); i += j) {
      uint32_t bid1 = order.at(i);
      auto& b1 = bonds.at(bid1);
      for (j = 1; i + j < order.size(); ++j) {
        uint32_t bid2 = order.at(i + j);
        auto b2 = bonds.at(bid2);
        if (b1.tids.first == b2.tids.first && b1.tids.second == b2.tids.second) {
          b1.wires.insert(b1.wires.end(), b2.wires.begin(), b2.wires.end());
          bonds.erase(bid2);
        } else {
          break;
        }
      }
      tid = contract_bond(bid1);
      auto& t = tensors.at(tid);  // rebcast {1, 1, 0}: metadata only with all slabs resident
      t.str = 1, t.cyc = 1, t.off = 0;
    }
    return tid;
  }
};

static int32_t fail(int32_t code, const char* what) {
  g_last_error = what;
  return code;
}

template <class F>
static int32_t guarded(F&& f) {
  try {
    return f();
  } catch (const std::invalid_argument& e) {
    return fail(ERR_INVALID_ARGUMENT, e.what());
  } catch (const std::out_of_range& e) {
    return fail(ERR_OUT_OF_RANGE, e.what());
  } catch (const std::runtime_error& e) {
    return fail(ERR_RUNTIME, e.what());
  } catch (const std::exception& e) {
    return fail(ERR_INTERNAL, e.what());
  }
}

}  // namespace orc

using namespace orc;

extern "C" {

// Flat tensor descriptor for the C interface. els: interleaved (re, im) doubles.
typedef struct {
  int32_t kind, ndis, nloc, n_dis_in;
  const uint64_t* dims;
  const double* els;  // dense/symm: totSize; diag: prod(totInDims); swap/iden: NULL
  uint32_t str, cyc, off;
} orc_tensor;

static Tensor from_desc(const orc_tensor* d) {
  Tensor t;
  t.kind = d->kind;
  t.dis.assign(d->dims, d->dims + d->ndis);
  t.loc.assign(d->dims + d->ndis, d->dims + d->ndis + d->nloc);
  t.n_dis_in = d->n_dis_in;
  t.str = d->str ? d->str : 1;
  t.cyc = d->cyc ? d->cyc : 1;
  t.off = d->off;
  uint64_t n = 0;
  if (t.kind == DENSE || t.kind == SYMM) {
    n = dims_to_size(t.tot());
  } else if (t.kind == DIAG) {
    n = 1;
    for (int32_t i = 0; i < t.n_dis_in; ++i) n *= t.dis.at(i);
    uint64_t nli = n_loc_in(t);
    for (uint64_t i = 0; i < nli; ++i) n *= t.loc.at(i);
  }
  if (t.kind == SWAP && t.tot().size() != 4) throw std::invalid_argument("swap tensor must have rank 4");
  t.els.resize(n);
  if (n) std::memcpy((void*)t.els.data(), d->els, n * sizeof(cplx));
  return t;
}

const char* orc_last_error(void) { return g_last_error.c_str(); }

int32_t orc_permute(const double* in, double* out, int32_t rank, const uint64_t* dims, const uint16_t* ptup) {
  return guarded([&] {
    permute(reinterpret_cast<const cplx*>(in), reinterpret_cast<cplx*>(out), dims_t(dims, dims + rank),
            std::vector<uint16_t>(ptup, ptup + rank));
    return (int32_t)OK;
  });
}

// Tensor::swap -> TIDense::_swap_internal, src/tensor/dense.cpp:171-274. All three cases
// (local, mixed, distributed) exchange the two axes of the global array; unequal axis
// dimensions throw std::runtime_error (dense.cpp:178-180).
int32_t orc_swap(const double* in, double* out, int32_t rank, const uint64_t* dims, int32_t i1, int32_t i2) {
  return guarded([&] {
    dims_t d(dims, dims + rank);
    if (i1 > i2) std::swap(i1, i2);
    if (d.at(i1) != d.at(i2)) throw std::runtime_error("Asymmetric swaps are currently not allowed");
    std::vector<uint16_t> ptup(rank);
    std::iota(ptup.begin(), ptup.end(), 0);
    std::swap(ptup[i1], ptup[i2]);
    permute(reinterpret_cast<const cplx*>(in), reinterpret_cast<cplx*>(out), d, ptup);
    return (int32_t)OK;
  });
}

// Tensor::contract (src/tensor/contract.cpp:204-313). repls1/repls2: in (when
// use_default == 0) and out (the replacements chosen, as the reference writes back into
// ConParams). out_dims must hold rank1 + rank2 entries. Returns ERR_CAPACITY (after
// filling the metadata) when out_els is NULL or out_cap is smaller than the result.
int32_t orc_contract(const orc_tensor* t1d, const orc_tensor* t2d, int32_t nwires, const uint16_t* wires,
                     int32_t use_default, uint16_t* repls1, uint16_t* repls2, int32_t* out_ndis, int32_t* out_nloc,
                     uint64_t* out_dims, uint32_t* out_bc, double* out_els, uint64_t out_cap) {
  return guarded([&] {
    Tensor t1 = from_desc(t1d), t2 = from_desc(t2d);
    ConParams p;
    for (int32_t i = 0; i < nwires; ++i) p.wires.push_back({wires[2 * i], wires[2 * i + 1]});
    p.use_def = use_default != 0;
    if (!p.use_def) {
      p.repls1.assign(repls1, repls1 + t1.tot().size());
      p.repls2.assign(repls2, repls2 + t2.tot().size());
    }
    Tensor t3 = contract(t1, t2, p);
    std::copy(p.repls1.begin(), p.repls1.end(), repls1);
    std::copy(p.repls2.begin(), p.repls2.end(), repls2);
    *out_ndis = (int32_t)t3.dis.size();
    *out_nloc = (int32_t)t3.loc.size();
    dims_t tot = t3.tot();
    std::copy(tot.begin(), tot.end(), out_dims);
    out_bc[0] = t3.str, out_bc[1] = t3.cyc, out_bc[2] = t3.off;
    if (!out_els || out_cap < t3.els.size()) return (int32_t)ERR_CAPACITY;
    std::memcpy(out_els, t3.els.data(), t3.els.size() * sizeof(cplx));
    return (int32_t)OK;
  });
}

// Dense elements of an implicit tensor kind (swap/iden/diag), as the reference's
// DenseTensorBase::toDense would produce them (src/tensor/dense.cpp:19-37).
int32_t orc_dense_of(const orc_tensor* td, double* out_els, uint64_t out_cap) {
  return guarded([&] {
    Tensor t = from_desc(td);
    auto e = dense_elements(t);
    if (out_cap < e.size()) return (int32_t)ERR_CAPACITY;
    std::memcpy(out_els, e.data(), e.size() * sizeof(cplx));
    return (int32_t)OK;
  });
}

// ---- TensorNetwork (src/tensor/network.cpp) -------------------------------------------

void* orc_tn_new(void) { return new Network(); }
void orc_tn_free(void* tn) { delete static_cast<Network*>(tn); }

int32_t orc_tn_insert(void* tn, const orc_tensor* td, uint32_t* tid) {
  return guarded([&] {
    *tid = static_cast<Network*>(tn)->insert(from_desc(td));
    return (int32_t)OK;
  });
}

int32_t orc_tn_add_bond(void* tn, uint32_t t1, uint32_t t2, int32_t nwires, const uint16_t* wires, uint32_t* bid) {
  return guarded([&] {
    std::vector<std::pair<uint16_t, uint16_t>> ws;
    for (int32_t i = 0; i < nwires; ++i) ws.push_back({wires[2 * i], wires[2 * i + 1]});
    *bid = static_cast<Network*>(tn)->add_bond(t1, t2, std::move(ws));
    return (int32_t)OK;
  });
}

int32_t orc_tn_contract_bond(void* tn, uint32_t bid, uint32_t* tid) {
  return guarded([&] {
    *tid = static_cast<Network*>(tn)->contract_bond(bid);
    return (int32_t)OK;
  });
}

// norder < 0: contractAll() without an order (network.cpp:108-126).
int32_t orc_tn_contract_all(void* tn, int32_t norder, const uint32_t* order, uint32_t* tid) {
  return guarded([&] {
    auto* n = static_cast<Network*>(tn);
    *tid = norder < 0 ? n->contract_all() : n->contract_all(std::vector<uint32_t>(order, order + norder));
    return (int32_t)OK;
  });
}

int32_t orc_tn_get(void* tn, uint32_t tid, int32_t* ndis, int32_t* nloc, uint64_t* dims, uint32_t* bc, double* els,
                   uint64_t cap) {
  return guarded([&] {
    auto& t = static_cast<Network*>(tn)->tensors.at(tid);
    *ndis = (int32_t)t.dis.size();
    *nloc = (int32_t)t.loc.size();
    dims_t tot = t.tot();
    std::copy(tot.begin(), tot.end(), dims);
    bc[0] = t.str, bc[1] = t.cyc, bc[2] = t.off;
    auto e = dense_elements(t);
    if (!els || cap < e.size()) return (int32_t)ERR_CAPACITY;
    std::memcpy(els, e.data(), e.size() * sizeof(cplx));
    return (int32_t)OK;
  });
}

}  // extern "C"
