// TEST INFRASTRUCTURE — C entry points over the reference's own C++ sources (src/core,
// src/tensor of the reference checkout, compiled with the single-process MPI subset in
// oracle/mpi_shim), so the tests can check the oracle restatement against the real code at
// world size 1 (one process: no distributed indices). Built by oracle/ref_build.py into
// oracle/_ref/libqtnh_ref.so; never linked by the product.
//
// Element arrays are interleaved (re, im) doubles in row-major order over the local dims.
#include <complex>
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "qtnh.hpp"

using namespace qtnh;

namespace {

std::string g_err;

QTNHEnv& env() {
  static QTNHEnv* e = new QTNHEnv();  // MPI_Init of the shim; never finalised
  return *e;
}

std::vector<tel> els_of(const double* els, std::size_t n) {
  std::vector<tel> v(n);
  if (els) std::memcpy(v.data(), els, n * sizeof(tel));
  return v;
}

// kinds as the engine's C ABI numbers them: dense, symm, swap, iden
tptr make(int kind, int nloc, int nin, const uint64_t* dims, const double* els) {
  tidx_tup loc(dims, dims + nloc);
  const std::size_t n = utils::dims_to_size(loc);
  switch (kind) {
    case 0: return DenseTensor::make(env(), {}, loc, els_of(els, n));
    case 1: return SymmTensor::make(env(), {}, loc, (tidx_tup_st)nin, els_of(els, n));
    case 2: return SwapTensor::make(env(), loc.at(0), 0);
    case 3: return IdenTensor::make(env(), {}, loc, (tidx_tup_st)nin, false);
    default: throw std::invalid_argument("kind not constructible in the reference at world size 1");
  }
}

int status(const std::exception& e) {
  g_err = e.what();
  if (dynamic_cast<const std::invalid_argument*>(&e)) return 1;
  if (dynamic_cast<const std::out_of_range*>(&e)) return 3;
  return 2;
}

void read_out(const Tensor& t, uint64_t* out_dims, double* out_els, uint64_t cap) {
  const auto d = t.totDims();
  for (std::size_t i = 0; i < d.size(); ++i) out_dims[i] = d[i];
  const std::size_t n = t.totSize();
  if (n > cap) throw std::out_of_range("output capacity too small");
  for (std::size_t i = 0; i < n; ++i) {
    const tel v = t[i];
    out_els[2 * i] = v.real();
    out_els[2 * i + 1] = v.imag();
  }
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Tensor::contract (src/tensor/contract.cpp:204-313): out_dims / out_els receive the
// result, repls1 / repls2 the dimension replacements (in/out when use_default == 0).
int ref_contract(int32_t kind1, int32_t nloc1, int32_t nin1, const uint64_t* dims1, const double* els1, int32_t kind2,
                 int32_t nloc2, int32_t nin2, const uint64_t* dims2, const double* els2, int32_t nwires,
                 const uint16_t* wires, int32_t use_default, uint16_t* repls1, uint16_t* repls2, int32_t* out_rank,
                 uint64_t* out_dims, double* out_els, uint64_t out_cap) {
  try {
    tptr t1 = make(kind1, nloc1, nin1, dims1, els1);
    tptr t2 = make(kind2, nloc2, nin2, dims2, els2);
    std::vector<wire> ws;
    for (int i = 0; i < nwires; ++i) ws.push_back({wires[2 * i], wires[2 * i + 1]});
    ConParams p = use_default ? ConParams(ws)
                              : ConParams(ws, std::vector<tidx_tup_st>(repls1, repls1 + nloc1),
                                          std::vector<tidx_tup_st>(repls2, repls2 + nloc2));
    tptr t3 = Tensor::contract(std::move(t1), std::move(t2), p);
    for (int i = 0; i < nloc1; ++i) repls1[i] = p.dimRepls1.at(i);
    for (int i = 0; i < nloc2; ++i) repls2[i] = p.dimRepls2.at(i);
    *out_rank = (int32_t)t3->totDims().size();
    read_out(*t3, out_dims, out_els, out_cap);
    return 0;
  } catch (const std::exception& e) {
    return status(e);
  }
}

// Tensor::permute (src/tensor/dense.cpp:152-169, 354-488): axis i moves to ptup[i].
int ref_permute(int32_t rank, const uint64_t* dims, const double* els, const uint16_t* ptup, uint64_t* out_dims,
                double* out_els) {
  try {
    tptr t = make(0, rank, 0, dims, els);
    t = Tensor::permute(std::move(t), std::vector<tidx_tup_st>(ptup, ptup + rank));
    read_out(*t, out_dims, out_els, t->totSize());
    return 0;
  } catch (const std::exception& e) {
    return status(e);
  }
}

// Tensor::swap (src/tensor/dense.cpp:171-274).
int ref_swap(int32_t rank, const uint64_t* dims, const double* els, int32_t i1, int32_t i2, uint64_t* out_dims,
             double* out_els) {
  try {
    tptr t = make(0, rank, 0, dims, els);
    t = Tensor::swap(std::move(t), (tidx_tup_st)i1, (tidx_tup_st)i2);
    read_out(*t, out_dims, out_els, t->totSize());
    return 0;
  } catch (const std::exception& e) {
    return status(e);
  }
}

// A layered circuit in the reference: one Tensor::contract per two-qubit SymmTensor gate
// (gates: 16 complex per gate; pairs: (qa, qb) per gate), for `layers` layers of `per`
// gates; the state (2^n, in and out) is replaced by the result. Used to time the
// reference's own CPU path.
int ref_gate_layers(int32_t n, double* state, int32_t ngates, const uint16_t* pairs, const double* gates) {
  try {
    tptr st = DenseTensor::make(env(), {}, tidx_tup(n, 2), els_of(state, (std::size_t)1 << n));
    for (int g = 0; g < ngates; ++g) {
      tptr u = SymmTensor::make(env(), {}, {2, 2, 2, 2}, 0, els_of(gates + 32 * g, 16));
      st = Tensor::contract(std::move(st), std::move(u), {{pairs[2 * g], 0}, {pairs[2 * g + 1], 1}});
    }
    for (std::size_t i = 0; i < ((std::size_t)1 << n); ++i) {
      const tel v = (*st)[i];
      state[2 * i] = v.real();
      state[2 * i + 1] = v.imag();
    }
    return 0;
  } catch (const std::exception& e) {
    return status(e);
  }
}

}  // extern "C"
