// Tests of the qtnh C++ API on the GB300 engine, mirroring the reference's test-suite:
// tests/c2-indexing.cpp (indexing), tests/c2-tensor.cpp (construction, accessors,
// golden contractions), tests/c2-mpi.cpp (rescattered tensors and QFT with distributed
// qubits; here all slabs are resident, so the whole result is compared),
// tests/c2-network.cpp (networks, QFT amplitude). Golden data: tests/golden/*.txt.
//
// Usage: api_test <cpu|gpu> <golden dir>. "cpu" runs the host-only cases.
#include <cmath>
#include <complex>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "qtnh.hpp"

using namespace qtnh;
using namespace std::complex_literals;

static int g_fail = 0, g_checks = 0;
static std::string g_case;

#define REQUIRE(c)                                                                            \
  do {                                                                                        \
    ++g_checks;                                                                               \
    if (!(c)) {                                                                               \
      ++g_fail;                                                                               \
      std::cerr << "FAIL [" << g_case << "] " << __FILE__ << ":" << __LINE__ << ": " #c "\n"; \
    }                                                                                         \
  } while (0)
#define REQUIRE_THROWS(e)                                                                             \
  do {                                                                                                \
    bool thrown = false;                                                                              \
    try {                                                                                             \
      e;                                                                                              \
    } catch (...) {                                                                                   \
      thrown = true;                                                                                  \
    }                                                                                                 \
    ++g_checks;                                                                                       \
    if (!thrown) {                                                                                    \
      ++g_fail;                                                                                       \
      std::cerr << "FAIL [" << g_case << "] " << __FILE__ << ":" << __LINE__ << ": no throw: " #e "\n"; \
    }                                                                                                 \
  } while (0)
#define REQUIRE_THROWS_AS(e, T)                                                                       \
  do {                                                                                                \
    bool ok = false;                                                                                  \
    try {                                                                                             \
      e;                                                                                              \
    } catch (const T&) {                                                                              \
      ok = true;                                                                                      \
    } catch (...) {                                                                                   \
    }                                                                                                 \
    ++g_checks;                                                                                       \
    if (!ok) {                                                                                        \
      ++g_fail;                                                                                       \
      std::cerr << "FAIL [" << g_case << "] " << __FILE__ << ":" << __LINE__ << ": expected " #T "\n"; \
    }                                                                                                 \
  } while (0)

struct TensorInfo {
  tidx_tup dims;
  std::vector<tel> els;
};
struct Contraction {
  TensorInfo t1, t2, t3;
  std::vector<wire> wires;
};
struct BondInfo {
  std::size_t t1, t2;
  std::vector<wire> wires;
};
struct NetCase {
  std::vector<TensorInfo> tensors;
  std::vector<BondInfo> bonds;
  TensorInfo result;
};

static TensorInfo read_tensor(std::istream& in) {
  TensorInfo t;
  std::size_t r, n;
  in >> r;
  t.dims.resize(r);
  for (auto& d : t.dims) in >> d;
  in >> n;
  t.els.resize(n);
  for (auto& e : t.els) {
    double a, b;
    in >> a >> b;
    e = tel(a, b);
  }
  return t;
}

static std::vector<wire> read_wires(std::istream& in) {
  std::size_t n;
  in >> n;
  std::vector<wire> ws(n);
  for (auto& w : ws) in >> w.first >> w.second;
  return ws;
}

static std::map<std::string, std::vector<Contraction>> load_contractions(const std::string& path) {
  std::map<std::string, std::vector<Contraction>> g;
  std::ifstream f(path);
  std::string tag, name;
  std::size_t n;
  while (f >> tag >> name >> n) {
    for (std::size_t i = 0; i < n; ++i) {
      Contraction c;
      c.t1 = read_tensor(f);
      c.t2 = read_tensor(f);
      c.t3 = read_tensor(f);
      c.wires = read_wires(f);
      g[name].push_back(c);
    }
  }
  return g;
}

static std::map<std::string, std::vector<NetCase>> load_networks(const std::string& path) {
  std::map<std::string, std::vector<NetCase>> g;
  std::ifstream f(path);
  std::string tag, name;
  std::size_t n;
  while (f >> tag >> name >> n) {
    for (std::size_t i = 0; i < n; ++i) {
      NetCase c;
      std::size_t nt, nb;
      f >> nt;
      for (std::size_t k = 0; k < nt; ++k) c.tensors.push_back(read_tensor(f));
      f >> nb;
      for (std::size_t k = 0; k < nb; ++k) {
        BondInfo b;
        f >> b.t1 >> b.t2;
        b.wires = read_wires(f);
        c.bonds.push_back(b);
      }
      c.result = read_tensor(f);
      g[name].push_back(c);
    }
  }
  return g;
}

static bool all_close(Tensor& t, const TensorInfo& ref, double tol) {
  if (t.totDims() != ref.dims) return false;
  TIndexing ti(ref.dims);
  for (auto idxs : ti.tup())
    if (!utils::equal(t.at(idxs), ref.els.at(utils::idxs_to_i(idxs, ref.dims)), tol)) return false;
  return true;
}

// ---- host-only cases (tests/c2-indexing.cpp) --------------------------------------------

static void test_indexing() {
  tidx_tup dims = {2, 3, 4, 5};
  std::vector<TIFlag> ifls(4, {"open", 0});
  ifls.at(1) = {"closed", 0};
  TIndexing ti1(dims), ti2(dims, ifls);
  REQUIRE(ti1.dims() == dims);
  REQUIRE(ti1.ifls() == std::vector<TIFlag>(4, {"default", 0}));
  REQUIRE(ti2.ifls() == ifls);

  TIndexing ti({2, 2, 2, 2}, {{"default", 0}, {"default", 0}, {"other", 0}, {"default", 0}});
  REQUIRE((ti.next({0, 0, 0, 0}) == tidx_tup{0, 0, 0, 1}));
  REQUIRE((ti.next({0, 0, 0, 1}) == tidx_tup{0, 1, 0, 0}));
  REQUIRE((ti.next({0, 0, 0, 0}, "other") == tidx_tup{0, 0, 1, 0}));
  REQUIRE_THROWS(ti.next({1, 1, 1, 1}));
  REQUIRE_THROWS(ti.prev({0, 0, 0, 0}));
  REQUIRE((ti.prev({0, 0, 0, 1}) == tidx_tup{0, 0, 0, 0}));
  REQUIRE((ti.prev({0, 1, 0, 0}) == tidx_tup{0, 0, 0, 1}));
  REQUIRE((ti.prev({0, 0, 1, 0}, "other") == tidx_tup{0, 0, 0, 0}));
  tidx_tup idxs2 = {0, 0, 0, 0};
  for (auto idxs1 : ti.tup()) {
    REQUIRE(idxs1 == idxs2);
    if (!ti.isLast(idxs2)) idxs2 = ti.next(idxs2);
  }

  TIndexing t3({2, 3, 4, 5}, {{"default", 0}, {"default", 0}, {"other", 0}, {"default", 0}});
  REQUIRE((t3.cut().dims() == tidx_tup{4}));
  REQUIRE((t3.cut("other").dims() == tidx_tup{2, 3, 5}));
  REQUIRE((TIndexing::app(t3, TIndexing({6, 7, 8})).dims() == tidx_tup{2, 3, 4, 5, 6, 7, 8}));

  // README.md:217-233 iteration-order examples
  TIndexing tr({2, 3, 2}, {{"default", 1}, {"other", 0}, {"default", 0}});
  std::vector<tidx_tup> seq;
  for (auto idx : tr.tup()) seq.push_back(idx);
  REQUIRE((seq == std::vector<tidx_tup>{{0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1}}));
  std::vector<std::size_t> nums;
  for (auto i : tr.num()) nums.push_back(i);
  REQUIRE((nums == std::vector<std::size_t>{0, 6, 1, 7}));
}

static void test_utils() {
  tidx_tup d = {2, 3, 4};
  for (std::size_t i = 0; i < 24; ++i) REQUIRE(utils::idxs_to_i(utils::i_to_idxs(i, d), d) == i);
  REQUIRE(utils::dims_to_size(d) == 24);
  REQUIRE(utils::equal(1.0 + 1i, 1.0 + 1i + 1e-7));
  REQUIRE(!utils::equal(1.0, 1.1));
  REQUIRE((utils::permute_vec(std::vector<int>{10, 20, 30}, {2, 0, 1}) == std::vector<int>{20, 30, 10}));
  REQUIRE((utils::invert_wires({{1, 2}}) == std::vector<wire>{{2, 1}}));
}

// ---- device cases -------------------------------------------------------------------------

static void test_construction(QTNHEnv& env) {
  tptr t;
  t = DenseTensor::make(env, {}, {2, 2}, {1.0i, 2.0i, 3.0i, 4.0i});
  t = DenseTensor::make(env, {}, {2, 2}, {1.0i, 2.0i, 3.0i, 4.0i}, {1, 1, 0});
  t = SymmTensor::make(env, {}, {2, 2}, 0, {1.0i, 2.0i, 3.0i, 4.0i});
  t = SymmTensor::make(env, {}, {2, 2}, 0, {1.0i, 2.0i, 3.0i, 4.0i}, {1, 1, 0});
  t = SwapTensor::make(env, 2, 0);
  t = SwapTensor::make(env, 2, 0, {1, 1, 0});
  t = IdenTensor::make(env, {}, {2, 2}, 0, 0);
  t = IdenTensor::make(env, {}, {2, 2}, 0, 0, {1, 1, 0});
  t = DiagTensor::make(env, {}, {2, 2}, 0, false, {1.0i, 2.0i});
  REQUIRE(t->totSize() == 4);
  REQUIRE_THROWS_AS(DenseTensor::make(env, {}, {2, 2}, {1.0, 2.0, 3.0}), std::invalid_argument);
  REQUIRE_THROWS_AS(DiagTensor::make(env, {}, {2, 2}, 0, false, {1.0}), std::invalid_argument);
}

static void test_accessors(QTNHEnv& env) {
  auto tp_dense = DenseTensor::make(env, {}, {2, 2}, {1.0i, 2.0i, 3.0i, 4.0i});
  auto tp_symm = SymmTensor::make(env, {}, {2, 2}, 0, {1.0i, 2.0i, 3.0i, 4.0i});
  auto tp_swap = SwapTensor::make(env, 2, 0);
  auto tp_iden = IdenTensor::make(env, {}, {2, 2}, 0, 0);

  REQUIRE((tp_dense->totDims() == tidx_tup{2, 2}));
  REQUIRE((tp_swap->totDims() == tidx_tup{2, 2, 2, 2}));
  REQUIRE((tp_iden->locDims() == tidx_tup{2, 2}));
  REQUIRE((tp_swap->disDims() == tidx_tup{}));
  REQUIRE(tp_swap->totSize() == 16 && tp_swap->locSize() == 16 && tp_swap->disSize() == 1);

  std::vector<tel> els_swap = {1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, 1};
  std::vector<tel> els_iden = {1, 0, 0, 1};
  TIndexing ti_swap(tp_swap->totDims());
  for (auto idxs : ti_swap.tup()) REQUIRE(tp_swap->at(idxs) == els_swap.at(utils::idxs_to_i(idxs, tp_swap->totDims())));
  TIndexing ti_iden(tp_iden->totDims());
  for (auto idxs : ti_iden.tup()) REQUIRE(tp_iden->at(idxs) == els_iden.at(utils::idxs_to_i(idxs, tp_iden->totDims())));
  TIndexing ti_dense(tp_dense->totDims());
  for (auto idxs : ti_dense.tup()) REQUIRE(tp_dense->at(idxs) == tel(0, 1.0 + utils::idxs_to_i(idxs, {2, 2})));

  tp_dense->at({0, 0}) = 0.1i;
  REQUIRE(tp_dense->at({0, 0}) == 0.1i);
  tp_symm->at({0, 0}) = 0.1i;
  REQUIRE(tp_symm->at({0, 0}) == 0.1i);
  // an edited element reaches the device before the next operation
  tptr moved = Tensor::permute(std::move(tp_dense), {1, 0});
  REQUIRE(moved->at({0, 0}) == 0.1i && moved->at({1, 0}) == 2.0i);
  REQUIRE(tp_symm->has({1, 1}));
  REQUIRE(tp_symm->fetch({1, 1}) == 4.0i);
}

static void test_golden_contractions(QTNHEnv& env, std::map<std::string, std::vector<Contraction>>& rt) {
  g_case = "dense-dense";
  for (auto& cv : rt["dense_vals"]) {
    tptr tp1 = DenseTensor::make(env, {}, cv.t1.dims, std::vector<tel>(cv.t1.els));
    tptr tp2 = DenseTensor::make(env, {}, cv.t2.dims, std::vector<tel>(cv.t2.els));
    tptr tp3 = Tensor::contract(std::move(tp1), std::move(tp2), cv.wires);
    REQUIRE(all_close(*tp3, cv.t3, 1e-5));
  }
  {
    tptr tp1 = DenseTensor::make(env, {}, {2, 2}, {1.0, 2.0, 3.0, 4.0});
    tptr tp2 = DenseTensor::make(env, {}, {3}, {1.0, 2.0, 3.0});
    REQUIRE_THROWS_AS(Tensor::contract(std::move(tp1), std::move(tp2), {{0, 0}}), std::invalid_argument);
  }
  g_case = "dense-swap";
  for (auto& cv : rt["swap_vals"]) {
    tptr tp1 = DenseTensor::make(env, {}, cv.t1.dims, std::vector<tel>(cv.t1.els));
    tptr tp2 = SwapTensor::make(env, cv.t2.dims.at(0), 0);
    tptr tp3 = Tensor::contract(std::move(tp1), std::move(tp2), cv.wires);
    REQUIRE(all_close(*tp3, cv.t3, 1e-5));
  }
  for (auto& cv : rt["invalid_swaps"]) {
    tptr tp1 = DenseTensor::make(env, {}, cv.t1.dims, std::vector<tel>(cv.t1.els));
    tptr tp2 = SwapTensor::make(env, cv.t2.dims.at(0), 0);
    REQUIRE_THROWS(Tensor::contract(std::move(tp1), std::move(tp2), cv.wires));
  }
  g_case = "dense-identity";
  for (auto& cv : rt["id_vals"]) {
    tptr tp1 = DenseTensor::make(env, {}, cv.t1.dims, std::vector<tel>(cv.t1.els));
    tptr tp2 = IdenTensor::make(env, {}, cv.t2.dims, 0, 0);
    tptr tp3 = Tensor::contract(std::move(tp1), std::move(tp2), cv.wires);
    REQUIRE(all_close(*tp3, cv.t3, 1e-5));
  }
  // tests/c2-mpi.cpp:80-214, every slab resident
  const std::vector<std::tuple<std::string, int, int>> mpi = {
      {"mpi2r_vals", 1, 0}, {"mpi3r_vals", 1, 0}, {"mpi4r_vals", 1, 1}, {"mpi6r_vals", 1, 1}, {"mpi8r_vals", 2, 1}};
  for (auto& [group, s1, s2] : mpi) {
    g_case = group;
    for (auto& cv : rt[group]) {
      tptr tp1 = DenseTensor::make(env, {}, cv.t1.dims, std::vector<tel>(cv.t1.els));
      tptr tp2 = DenseTensor::make(env, {}, cv.t2.dims, std::vector<tel>(cv.t2.els));
      tp1 = Tensor::rescatter(std::move(tp1), s1);
      if (s2) tp2 = Tensor::rescatter(std::move(tp2), s2);
      tptr tp3 = Tensor::contract(std::move(tp1), std::move(tp2), cv.wires);
      REQUIRE(tp3->disDims().size() == (std::size_t)(s1 + s2));
      REQUIRE(all_close(*tp3, cv.t3, 1e-5));
    }
  }
}

static void test_scatter(QTNHEnv& env) {
  g_case = "scatter";
  // tests/c2-mpi.cpp:49-78 and 216-238
  std::vector<tel> els = {1.0 + 1.0i, 2.0 + 2.0i, 3.0 + 3.0i, 4.0 + 4.0i, 5.0 + 5.0i, 6.0 + 6.0i, 7.0 + 7.0i, 8.0 + 8.0i};
  tptr tp = DenseTensor::make(env, {}, {2, 2, 2}, std::vector<tel>(els));
  tp = Tensor::rescatter(std::move(tp), 1);
  REQUIRE((tp->disDims() == tidx_tup{2}) && (tp->locDims() == tidx_tup{2, 2}));
  REQUIRE(tp->at({0, 0, 0}) == 1.0 + 1.0i && tp->at({1, 0, 0}) == 5.0 + 5.0i);
  tp = Tensor::rescatter(std::move(tp), 1);
  REQUIRE(tp->at({0, 1, 0}) == 3.0 + 3.0i && tp->at({1, 1, 0}) == 7.0 + 7.0i);
  REQUIRE(tp->bc().base == 4);
  tp = Tensor::rescatter(std::move(tp), -2);
  REQUIRE(tp->disDims().empty() && tp->bc().str == 4);
  tp = Tensor::rebcast(std::move(tp), {1, 1, 0});
  REQUIRE(tp->bc().str == 1 && tp->bc().cyc == 1);
  REQUIRE_THROWS_AS(Tensor::rescatter(std::move(tp), 4), std::out_of_range);

  tptr a = DenseTensor::make(env, {}, {2, 2, 2}, std::vector<tel>(els));
  tptr b = DenseTensor::make(env, {}, {4, 2}, {5.0 + 5.0i, 6.0 + 6.0i, 7.0 + 7.0i, 8.0 + 8.0i, 1.0 + 1.0i, 2.0 + 2.0i,
                                              3.0 + 3.0i, 4.0 + 4.0i});
  a = Tensor::rescatter(std::move(a), 1);
  tptr c = Tensor::contract(std::move(b), std::move(a), {{1, 1}});
  REQUIRE((c->disDims() == tidx_tup{2}));
}

static void test_transforms(QTNHEnv& env) {
  g_case = "transforms";
  std::vector<tel> els(24);
  for (std::size_t i = 0; i < 24; ++i) els[i] = tel((double)i, -(double)i);
  tptr t = DenseTensor::make(env, {2}, {3, 4}, std::vector<tel>(els));
  t = Tensor::permute(std::move(t), {2, 0, 1});  // old 0 -> 2, old 1 -> 0, old 2 -> 1
  REQUIRE((t->totDims() == tidx_tup{3, 4, 2}) && (t->disDims() == tidx_tup{3}));
  bool ok = true;
  for (std::size_t a = 0; a < 2; ++a)
    for (std::size_t b = 0; b < 3; ++b)
      for (std::size_t c = 0; c < 4; ++c) ok = ok && t->at({b, c, a}) == els[a * 12 + b * 4 + c];
  REQUIRE(ok);
  tptr s = DenseTensor::make(env, {3}, {2, 3}, std::vector<tel>(18, 1.0));
  REQUIRE_THROWS_AS(Tensor::swap(std::move(s), 0, 1), std::runtime_error);
  tptr u = DenseTensor::make(env, {3}, {2, 3}, std::vector<tel>(els.begin(), els.begin() + 18));
  u = Tensor::swap(std::move(u), 0, 2);  // mixed distributed/local swap
  ok = true;
  for (std::size_t a = 0; a < 3; ++a)
    for (std::size_t b = 0; b < 2; ++b)
      for (std::size_t c = 0; c < 3; ++c) ok = ok && u->at({c, b, a}) == els[a * 6 + b * 3 + c];
  REQUIRE(ok);
  // transforms of a SymmTensor yield a DenseTensor (as the reference's DenseTensorBase does)
  tptr g = SymmTensor::make(env, {}, {2, 2}, 0, {1.0, 2.0, 3.0, 4.0});
  g = Tensor::permute(std::move(g), {1, 0});
  REQUIRE(g->type() == TT::denseTensor && g->at({0, 1}) == 3.0);
  tptr cp = g->copy();
  g->cast<DenseTensor>()->at({0, 0}) = 9.0;
  REQUIRE(cp->at({0, 0}) == 1.0 && g->at({0, 0}) == 9.0);
}

static void test_gates(QTNHEnv& env) {
  g_case = "gates";
  // in-place rule: a 2-qubit gate on a state with a distributed prefix keeps its layout
  const double s = std::pow(2, -.5);
  std::vector<tel> psi(16);
  for (std::size_t i = 0; i < 16; ++i) psi[i] = tel(std::cos(0.3 * i), std::sin(0.7 * i));
  tptr st = DenseTensor::make(env, {2}, {2, 2, 2}, std::vector<tel>(psi));
  tptr h = SymmTensor::make(env, {}, {2, 2}, 0, {s, s, s, -s});
  ConParams p({{2, 0}});
  st = Tensor::contract(std::move(st), std::move(h), p);
  REQUIRE((st->disDims() == tidx_tup{2}) && (st->locDims() == tidx_tup{2, 2, 2}));
  REQUIRE((p.dimRepls1 == std::vector<tidx_tup_st>{0, 1, X, 3}) && (p.dimRepls2 == std::vector<tidx_tup_st>{X, 2}));
  bool ok = true;
  for (std::size_t i = 0; i < 16; ++i) {
    auto idx = utils::i_to_idxs(i, {2, 2, 2, 2});
    auto i0 = idx, i1 = idx;
    i0[2] = 0, i1[2] = 1;
    tel ref = (idx[2] == 0 ? s : s) * psi[utils::idxs_to_i(i0, {2, 2, 2, 2})] +
              (idx[2] == 0 ? s : -s) * psi[utils::idxs_to_i(i1, {2, 2, 2, 2})];
    ok = ok && utils::equal(st->at(idx), ref, 1e-12);
  }
  REQUIRE(ok);
  // a diagonal tensor equals the symmetric tensor of its expanded form
  std::vector<tel> d = {1.0, std::exp(0.4i), std::exp(1.1i), std::exp(2.3i)};
  tptr a = DenseTensor::make(env, {}, {2, 2, 2}, std::vector<tel>(psi.begin(), psi.begin() + 8));
  tptr b = DenseTensor::make(env, {}, {2, 2, 2}, std::vector<tel>(psi.begin(), psi.begin() + 8));
  std::vector<tel> full(16, 0.0);
  for (int i = 0; i < 4; ++i) full[i * 4 + i] = d[i];
  a = Tensor::contract(std::move(a), DiagTensor::make(env, {}, {2, 2, 2, 2}, 0, false, std::vector<tel>(d)), {{2, 0}, {0, 1}});
  b = Tensor::contract(std::move(b), SymmTensor::make(env, {}, {2, 2, 2, 2}, 0, std::move(full)), {{2, 0}, {0, 1}});
  ok = a->totDims() == b->totDims();
  TIndexing ti(a->totDims());
  for (auto idx : ti.tup()) ok = ok && utils::equal(a->at(idx), b->at(idx), 1e-14);
  REQUIRE(ok);
  // README.md:153-165: custom replacements
  tptr phi = DenseTensor::make(env, {}, {2, 2, 2}, std::vector<tel>(psi.begin(), psi.begin() + 8));
  tptr had = DenseTensor::make(env, {}, {2, 2}, {s, s, s, -s});
  ConParams cp({{1, 0}}, {0, X, 2}, {X, 1});
  phi = Tensor::contract(std::move(phi), std::move(had), cp);
  REQUIRE((phi->totDims() == tidx_tup{2, 2, 2}));
  REQUIRE(utils::equal(phi->at({0, 1, 0}), s * psi[0] - s * psi[2], 1e-12));
}

// Plain-loop application of a k-qubit SymmTensor gate (els[in, out]) to a state of n
// qubits (index q = axis q, row-major): the definition of the in-place rule.
static std::vector<tel> apply_plain(const std::vector<tel>& psi, int n, const std::vector<int>& qs,
                                    const std::vector<tel>& els) {
  const int k = (int)qs.size(), D = 1 << k;
  std::vector<tel> out(psi.size(), 0.0);
  for (std::size_t x = 0; x < psi.size(); ++x) {
    int o = 0;
    for (int m = 0; m < k; ++m) o = o * 2 + (int)((x >> (n - 1 - qs[m])) & 1);
    for (int i = 0; i < D; ++i) {
      std::size_t y = x;
      for (int m = 0; m < k; ++m) {
        const int bit = (i >> (k - 1 - m)) & 1;
        const std::size_t mask = (std::size_t)1 << (n - 1 - qs[m]);
        y = bit ? (y | mask) : (y & ~mask);
      }
      out[x] += els[(std::size_t)i * D + o] * psi[y];
    }
  }
  return out;
}

// Gates and diagonals contracted in place are queued on the state (DeviceArray::defer) and
// applied, fused, when the elements are next used: every kind of use must see them all, in
// order, and host edits made in between must stay in sequence with them.
static void test_queued_contractions(QTNHEnv& env) {
  g_case = "queued";
  const int n = 8;
  const std::size_t N = (std::size_t)1 << n;
  std::vector<tel> psi(N);
  for (std::size_t i = 0; i < N; ++i) psi[i] = tel(std::cos(0.37 * i + 0.1), std::sin(1.3 * i));
  auto gate = [](int seed) {
    std::vector<tel> g(16);
    for (int i = 0; i < 16; ++i) g[i] = tel(std::sin(0.9 * i + seed), std::cos(0.4 * i * seed + 1.0));
    return g;
  };
  // elementwise within 1e-12 of the largest magnitude (the gates are not unitary, so the
  // values grow along the sequence)
  auto close = [&](Tensor& t, const std::vector<tel>& ref) {
    double big = 0;
    for (auto& r : ref) big = std::max(big, std::abs(r));
    bool ok = true;
    for (std::size_t i = 0; i < N; ++i)
      ok = ok && std::abs(t.at(utils::i_to_idxs(i, t.totDims())) - ref[i]) <= 1e-12 * big;
    return ok;
  };
  // four two-qubit gates (two disjoint pairs, then overlapping), a one-index diagonal run
  // (the diagonals on 1, 6 and 3 are folded into the queued gates on them, as their second,
  // second and first target; the one on 4 follows no gate and stays) and a two-index
  // diagonal, read back through at()
  const std::vector<std::vector<int>> qs = {{0, 5}, {2, 3}, {5, 1}, {7, 6}, {3, 0}};
  tptr st = DenseTensor::make(env, {}, tidx_tup(n, 2), std::vector<tel>(psi));
  std::vector<tel> ref = psi;
  for (std::size_t g = 0; g < qs.size(); ++g) {
    st = Tensor::contract(std::move(st), SymmTensor::make(env, {}, {2, 2, 2, 2}, 0, gate((int)g)),
                          {{(tidx_tup_st)qs[g][0], 0}, {(tidx_tup_st)qs[g][1], 1}});
    ref = apply_plain(ref, n, qs[g], gate((int)g));
  }
  for (int q : {1, 4, 6, 3}) {
    const std::vector<tel> d = {std::exp(0.3i * (double)q), std::exp(-1.1i * (double)q)};
    st = Tensor::contract(std::move(st), DiagTensor::make(env, {}, {2, 2}, 0, false, std::vector<tel>(d)),
                          {{(tidx_tup_st)q, 0}});
    ref = apply_plain(ref, n, {q}, {d[0], 0.0, 0.0, d[1]});
  }
  const std::vector<tel> d2 = {1.0, std::exp(0.7i), std::exp(-0.2i), -1.0};
  st = Tensor::contract(std::move(st), DiagTensor::make(env, {}, {2, 2, 2, 2}, 0, false, std::vector<tel>(d2)),
                        {{2, 0}, {7, 1}});
  std::vector<tel> e2(16, 0.0);
  for (int i = 0; i < 4; ++i) e2[i * 4 + i] = d2[i];
  ref = apply_plain(ref, n, {2, 7}, e2);
  REQUIRE(close(*st, ref));
  // a host edit between queued gates, then copy() of a tensor with queued gates
  static_cast<DenseTensor*>(st.get())->put(utils::i_to_idxs(5, st->totDims()), tel(0.25, -0.5));
  ref[5] = tel(0.25, -0.5);
  st = Tensor::contract(std::move(st), SymmTensor::make(env, {}, {2, 2, 2, 2}, 0, gate(9)), {{4, 0}, {1, 1}});
  ref = apply_plain(ref, n, {4, 1}, gate(9));
  auto cp = st->copy();
  REQUIRE(close(*cp, ref));
  REQUIRE(close(*st, ref));
  // a transform (swap) after queued gates sees them
  st = Tensor::contract(std::move(st), SymmTensor::make(env, {}, {2, 2, 2, 2}, 0, gate(4)), {{6, 0}, {2, 1}});
  ref = apply_plain(ref, n, {6, 2}, gate(4));
  st = Tensor::swap(std::move(st), 0, 3);
  std::vector<tel> sw(N);
  for (std::size_t x = 0; x < N; ++x) {
    auto idx = utils::i_to_idxs(x, tidx_tup(n, 2));
    std::swap(idx[0], idx[3]);
    sw[x] = ref[utils::idxs_to_i(idx, tidx_tup(n, 2))];
  }
  REQUIRE(close(*st, sw));
  // a permutation queued between gates (DeviceArray::defer_permute): the gate runs on both
  // sides of it are applied in one call (at 12 qubits one fixed-point chain on the tensor
  // cores), a one-index diagonal after it folds into a gate before it (on the index it
  // came from), two permutations in a row, and a permutation with nothing else queued
  {
    const int m = 12;
    const std::size_t M = (std::size_t)1 << m;
    const tidx_tup dm(m, 2);
    std::vector<tel> phi(M);
    for (std::size_t i = 0; i < M; ++i) phi[i] = tel(std::cos(0.11 * i + 0.3), std::sin(0.7 * i));
    auto permute_host = [&](const std::vector<tel>& v, const std::vector<tidx_tup_st>& pt) {
      std::vector<tel> out(M);
      for (std::size_t x = 0; x < M; ++x) {
        const auto idx = utils::i_to_idxs(x, dm);
        tidx_tup nidx(m);
        for (int i = 0; i < m; ++i) nidx[pt[i]] = idx[i];
        out[utils::idxs_to_i(nidx, dm)] = v[x];
      }
      return out;
    };
    auto close_m = [&](Tensor& t, const std::vector<tel>& r) {
      double big = 0;
      for (auto& v : r) big = std::max(big, std::abs(v));
      bool ok = t.totDims() == dm;
      for (std::size_t i = 0; ok && i < M; ++i) ok = std::abs(t.at(utils::i_to_idxs(i, dm)) - r[i]) <= 1e-12 * big;
      return ok;
    };
    auto apply_gate = [&](tptr t, std::vector<tel>& r, int a, int b, int seed) {
      r = apply_plain(r, m, {a, b}, gate(seed));
      return Tensor::contract(std::move(t), SymmTensor::make(env, {}, {2, 2, 2, 2}, 0, gate(seed)),
                              {{(tidx_tup_st)a, 0}, {(tidx_tup_st)b, 1}});
    };
    auto permute = [&](tptr t, std::vector<tel>& r, const std::vector<tidx_tup_st>& pt) {
      r = permute_host(r, pt);
      return Tensor::permute(std::move(t), pt);
    };
    std::vector<tidx_tup_st> rot(m), rev(m), sw05(m);
    for (int i = 0; i < m; ++i) rot[i] = (tidx_tup_st)((i + 3) % m), rev[i] = (tidx_tup_st)(m - 1 - i), sw05[i] = i;
    std::swap(sw05[0], sw05[5]);
    tptr pt = DenseTensor::make(env, {}, dm, std::vector<tel>(phi));
    std::vector<tel> pref = phi;
    pt = apply_gate(std::move(pt), pref, 0, 5, 11);
    pt = apply_gate(std::move(pt), pref, 2, 3, 12);
    pt = apply_gate(std::move(pt), pref, 7, 9, 13);
    pt = apply_gate(std::move(pt), pref, 10, 11, 14);
    pt = permute(std::move(pt), pref, rot);  // old index i -> (i + 3) % 12
    pt = apply_gate(std::move(pt), pref, 1, 4, 15);
    pt = apply_gate(std::move(pt), pref, 6, 8, 16);
    pt = apply_gate(std::move(pt), pref, 2, 11, 17);
    pt = apply_gate(std::move(pt), pref, 0, 3, 18);
    // index 10 came from index 7, last touched by the gate on (7, 9): folded into it
    const std::vector<tel> d = {std::exp(0.45i), std::exp(-0.8i)};
    pt = Tensor::contract(std::move(pt), DiagTensor::make(env, {}, {2, 2}, 0, false, std::vector<tel>(d)), {{10, 0}});
    pref = apply_plain(pref, m, {10}, {d[0], 0.0, 0.0, d[1]});
    pt = permute(std::move(pt), pref, rev);
    pt = permute(std::move(pt), pref, sw05);
    pt = apply_gate(std::move(pt), pref, 3, 7, 19);
    REQUIRE(close_m(*pt, pref));
    pt = permute(std::move(pt), pref, rot);
    REQUIRE(close_m(*pt, pref));
    std::vector<tidx_tup_st> bad(m, 0);
    bool threw = false;
    try {
      pt = Tensor::permute(std::move(pt), bad);
    } catch (const std::invalid_argument&) {
      threw = true;
    }
    REQUIRE(threw);
  }
  // a state dropped with gates still queued, then a fresh one: nothing leaks into it
  {
    tptr tmp = DenseTensor::make(env, {}, tidx_tup(n, 2), std::vector<tel>(psi));
    tmp = Tensor::contract(std::move(tmp), SymmTensor::make(env, {}, {2, 2, 2, 2}, 0, gate(2)), {{0, 0}, {1, 1}});
  }
  tptr fresh = DenseTensor::make(env, {}, tidx_tup(n, 2), std::vector<tel>(psi));
  REQUIRE(close(*fresh, psi));
  // more than the queue's bound (1024) of gates in a row
  tptr longrun = DenseTensor::make(env, {}, tidx_tup(n, 2), std::vector<tel>(psi));
  std::vector<tel> lref = psi;
  for (int g = 0; g < 1100; ++g) {
    const int a = g % n, b = (g * 3 + 1) % n == a ? (a + 1) % n : (g * 3 + 1) % n;
    std::vector<tel> u(16, 0.0);  // a phase-and-permutation unitary keeps the norm
    for (int i = 0; i < 4; ++i) u[i * 4 + ((i + g) % 4)] = std::exp(1i * (0.01 * g + i));
    longrun = Tensor::contract(std::move(longrun), SymmTensor::make(env, {}, {2, 2, 2, 2}, 0, std::vector<tel>(u)),
                               {{(tidx_tup_st)a, 0}, {(tidx_tup_st)b, 1}});
    lref = apply_plain(lref, n, {a, b}, u);
  }
  REQUIRE(close(*longrun, lref));
}

static void test_networks(QTNHEnv& env, std::map<std::string, std::vector<NetCase>>& tn) {
  auto run = [&](const NetCase& c, bool ordered) {
    TensorNetwork net;
    std::vector<qtnh::uint> ids, bids;
    for (auto& t : c.tensors) ids.push_back(net.make<DenseTensor>(env, tidx_tup{}, t.dims, std::vector<tel>(t.els)));
    for (auto& b : c.bonds) bids.push_back(net.addBond(ids.at(b.t1), ids.at(b.t2), b.wires));
    auto id = ordered ? net.contractAll(bids) : net.contractAll();
    return net.extract(id);
  };
  g_case = "tn2";
  for (auto& c : tn["tn2_vals"]) {
    auto tp = run(c, false);
    REQUIRE(all_close(*tp, c.result, 1e-5));
  }
  for (auto name : {"tn3_vals", "tn4_vals", "tn4c_vals"}) {
    g_case = name;
    for (auto& c : tn[name]) {
      auto tp = run(c, true);
      REQUIRE(all_close(*tp, c.result, 1e-2));
    }
  }
}

// QFT network of tests/gen/qft.hpp:49-142 (|+...+> -> |0...0>), dq distributed qubits.
static std::vector<qtnh::uint> qft(QTNHEnv& env, TensorNetwork& tn, qtnh::uint nq, qtnh::uint dq) {
  const double s = std::pow(2, -.5);
  std::vector<qtnh::uint> order, qid(nq);
  std::vector<tidx_tup_st> qidx(nq, 0);
  auto dist = [&](bool in) { return tn.make<IdenTensor>(env, tidx_tup{2}, tidx_tup{2}, (tidx_tup_st)in, false); };
  for (qtnh::uint i = 0; i < nq; ++i) {
    qid[i] = tn.make<DenseTensor>(env, tidx_tup{}, tidx_tup{2}, std::vector<tel>{s, s});
    if (i < dq) {
      auto t = dist(0);
      order.push_back(tn.addBond(qid[i], t, {{0, 1}}));
      qid[i] = t;
      qidx[i] = 0;
    }
    if (i > 0) order.push_back(tn.addBond(qid[i - 1], qid[i], {}));
  }
  for (qtnh::uint i = 0; i < nq; ++i) {
    auto h = tn.make<SymmTensor>(env, tidx_tup{}, tidx_tup{2, 2}, 0, std::vector<tel>{s, s, s, -s});
    auto t_in = h, t_out = h;
    tidx_tup_st out_idx = 1;
    if (i < dq) {
      t_in = dist(1);
      order.push_back(tn.addBond(t_in, h, {{1, 0}}));
      t_out = dist(0);
      order.push_back(tn.addBond(h, t_out, {{1, 1}}));
      out_idx = 0;
    }
    order.push_back(tn.addBond(qid[i], t_in, {{qidx[i], 0}}));
    qid[i] = t_out;
    qidx[i] = out_idx;
    for (qtnh::uint j = i + 1; j < nq; ++j) {
      std::vector<tel> cp(16, 0.0);
      cp[0] = cp[5] = cp[10] = 1.0;
      cp[15] = std::exp(1i * (M_PI / std::pow(2, j - i)));
      auto c = tn.make<SymmTensor>(env, tidx_tup{}, tidx_tup{2, 2, 2, 2}, 0, std::move(cp));
      auto a_in = c, b_in = c, a_out = c, b_out = c;
      tidx_tup_st ia_in = 0, ib_in = 1, ia_out = 2, ib_out = 3;
      if (i < dq) {
        a_in = dist(1);
        order.push_back(tn.addBond(a_in, c, {{1, 0}}));
        ia_in = 0;
        a_out = dist(0);
        order.push_back(tn.addBond(c, a_out, {{2, 1}}));
        ia_out = 0;
      }
      if (j < dq) {
        b_in = dist(1);
        order.push_back(tn.addBond(b_in, c, {{1, 1}}));
        ib_in = 0;
        b_out = dist(0);
        order.push_back(tn.addBond(c, b_out, {{3, 1}}));
        ib_out = 0;
      }
      order.push_back(tn.addBond(qid[i], a_in, {{qidx[i], ia_in}}));
      order.push_back(tn.addBond(qid[j], b_in, {{qidx[j], ib_in}}));
      qid[i] = a_out, qidx[i] = ia_out;
      qid[j] = b_out, qidx[j] = ib_out;
    }
  }
  return order;
}

static void test_qft(QTNHEnv& env) {
  // up to the 16-qubit QFT of the reference's example, on 1 and 2 (dq = 1) "ranks"
  const std::vector<std::pair<int, int>> cases = {{2, 0}, {3, 0}, {4, 0}, {5, 0}, {5, 2}, {6, 2},
                                                  {7, 3}, {8, 3}, {16, 0}, {16, 1}};
  for (auto [nq, dq] : cases) {
    g_case = "qft-" + std::to_string(nq) + "-" + std::to_string(dq);
    TensorNetwork tn;
    auto order = qft(env, tn, nq, dq);
    auto tp = tn.extract(tn.contractAll(order));
    REQUIRE(tp->totDims().size() == (std::size_t)nq);
    REQUIRE(utils::equal(tp->at(utils::i_to_idxs(0, tp->totDims())), 1.0, 1E-4));
    REQUIRE(std::abs(tp->at(utils::i_to_idxs(0, tp->totDims())) - 1.0) < 1e-12);
    double rest = 0;
    for (std::size_t i = 1; i < tp->totSize(); ++i) rest += std::norm(tp->at(utils::i_to_idxs(i, tp->totDims())));
    REQUIRE(rest < 1e-20);
  }
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cerr << "usage: api_test <cpu|gpu> <golden dir>\n";
    return 2;
  }
  const std::string mode = argv[1], dir = argv[2];
  g_case = "indexing";
  test_indexing();
  g_case = "utils";
  test_utils();
  if (mode == "gpu") {
    auto rt = load_contractions(dir + "/random_tensors.txt");
    auto tn = load_networks(dir + "/random_tn.txt");
    if (rt["dense_vals"].size() != 20 || tn["tn4c_vals"].size() != 5) {
      std::cerr << "golden fixtures not found in " << dir << "\n";
      return 2;
    }
    QTNHEnv env;
    g_case = "construction";
    test_construction(env);
    g_case = "accessors";
    test_accessors(env);
    test_golden_contractions(env, rt);
    test_scatter(env);
    test_transforms(env);
    test_gates(env);
    test_queued_contractions(env);
    test_networks(env, tn);
    test_qft(env);
  }
  std::cout << (g_fail ? "FAILED " : "ok ") << g_checks - g_fail << "/" << g_checks << " checks\n";
  return g_fail ? 1 : 0;
}
