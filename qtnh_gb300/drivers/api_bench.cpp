// Workloads through the qtnh C++ API (include/qtnh.hpp), as a qtnh user writes them: the
// drop-in path's own throughput, timed on the host around the environment's stream.
//
//   api_bench circuit <in.bin> <out.bin> <warmup> <reps>
//       Random layered circuit, one Tensor::contract per gate (a SymmTensor with the
//       in-place rule, src/tensor/contract.cpp:250-289), one per qubit for a phase layer
//       (rank-2 DiagTensors), rescatter / permute / rescatter for a redistribution
//       (src/tensor/dense.cpp:123-169). The state is made once; every timed run applies
//       the whole circuit to it and ends with Tensor::copy (which waits for the queued
//       contractions, like any use of the elements). in.bin: int32 n, int32 layers,
//       int32 has_state, then complex128 state[2^n] (has_state = 1) or a uint64 seed of
//       an i.i.d. complex Gaussian state normalised to unit L2 (has_state = 0), then
//       per layer int32 gates, per gate uint16 qa, qb and
//       complex128 els[16] (SymmTensor layout), int32 has_phases [double phases[n]],
//       int32 has_perm [uint16 ptup[n]], int32 n_dis (rescatter offset around the
//       permutation).
//   api_bench qft <n> <dq> <in.bin> <out.bin> <warmup> <reps>
//       QFT on a random state as a TensorNetwork (examples/qft.cpp:53-149 of the
//       reference with its gate kinds: Hadamard SymmTensors, controlled-phase DiagTensors
//       of phase pi / 2^(j - i), SwapTensor reversals; gates on the dq distributed qubits
//       wrapped in "DIST" IdenTensors as tests/gen/qft.hpp:64-129) contracted with
//       TensorNetwork::contractAll(order). Every timed run builds the network from the
//       host state (DenseTensor::make copies it to the device), contracts it and copies
//       the result back. in.bin: complex128 state[2^n].
//
// Prints one JSON line: {"mode", "runs", "ms_per_run", "contractions_per_run"} and
// writes the last run's final state (complex128, the result's own index order) to
// out.bin.
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "qtnh.hpp"
#include "qtnh_cuda.h"

using namespace qtnh;
using namespace std::complex_literals;

namespace {

template <class T>
T get(std::ifstream& f) {
  T v;
  if (!f.read(reinterpret_cast<char*>(&v), sizeof(T))) throw std::runtime_error("input file too short");
  return v;
}

std::vector<tel> get_els(std::ifstream& f, std::size_t n) {
  std::vector<tel> v(n);
  if (!f.read(reinterpret_cast<char*>(v.data()), n * sizeof(tel))) throw std::runtime_error("input file too short");
  return v;
}

void write_state(const std::string& path, const Tensor& t) {
  const std::size_t n = t.totSize();
  std::vector<tel> h(n);
  if (qtnh_memcpy_d2h(h.data(), t.engineData(), n * sizeof(tel), t.bc().env.stream) != QTNH_OK ||
      qtnh_stream_synchronize(t.bc().env.stream) != QTNH_OK)
    throw std::runtime_error(qtnh_last_error());
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(h.data()), n * sizeof(tel));
}

struct Gate {
  uint16_t qa, qb;
  std::vector<tel> els;
};
struct Layer {
  std::vector<Gate> gates;
  std::vector<double> phases;
  std::vector<tidx_tup_st> ptup;
  int n_dis = 0;
};

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void sync(const QTNHEnv& env) {
  if (qtnh_stream_synchronize(env.stream) != QTNH_OK) throw std::runtime_error(qtnh_last_error());
}

int run_circuit(const std::string& in, const std::string& out, int warmup, int reps) {
  std::ifstream f(in, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + in);
  const int n = get<int32_t>(f), nl = get<int32_t>(f);
  std::vector<tel> psi;
  if (get<int32_t>(f)) {
    psi = get_els(f, (std::size_t)1 << n);
  } else {
    std::mt19937_64 rng(get<uint64_t>(f));
    std::normal_distribution<double> nd(0.0, 1.0);
    psi.resize((std::size_t)1 << n);
    double s = 0;
    for (auto& x : psi) x = tel(nd(rng), nd(rng)), s += std::norm(x);
    for (auto& x : psi) x /= std::sqrt(s);
  }
  std::vector<Layer> layers(nl);
  std::size_t contractions = 0;
  for (auto& L : layers) {
    const int ng = get<int32_t>(f);
    for (int g = 0; g < ng; ++g) {
      Gate G;
      G.qa = get<uint16_t>(f);
      G.qb = get<uint16_t>(f);
      G.els = get_els(f, 16);
      L.gates.push_back(std::move(G));
    }
    contractions += ng;
    if (get<int32_t>(f)) {
      L.phases.resize(n);
      for (auto& p : L.phases) p = get<double>(f);
      contractions += n;
    }
    if (get<int32_t>(f)) {
      L.ptup.resize(n);
      for (auto& p : L.ptup) p = get<uint16_t>(f);
    }
    L.n_dis = get<int32_t>(f);
  }

  QTNHEnv env;
  tptr state = DenseTensor::make(env, tidx_tup{}, tidx_tup(n, 2), std::move(psi));
  auto pass = [&]() {
    for (auto& L : layers) {
      for (auto& G : L.gates) {
        std::vector<tel> els = G.els;
        tptr g = SymmTensor::make(env, tidx_tup{}, tidx_tup{2, 2, 2, 2}, 0, std::move(els));
        state = Tensor::contract(std::move(state), std::move(g), {{G.qa, 0}, {G.qb, 1}});
      }
      if (!L.phases.empty()) {
        for (int q = 0; q < n; ++q) {
          tptr d = DiagTensor::make(env, tidx_tup{}, tidx_tup{2, 2}, 0, false,
                                    std::vector<tel>{1.0, std::exp(1i * L.phases[q])});
          state = Tensor::contract(std::move(state), std::move(d), {{(tidx_tup_st)q, 0}});
        }
      }
      if (!L.ptup.empty()) {
        state = Tensor::rescatter(std::move(state), L.n_dis);
        state = Tensor::permute(std::move(state), L.ptup);
        state = Tensor::rescatter(std::move(state), -L.n_dis);
      }
    }
  };
  // the timed runs apply the circuit repeatedly to the evolving state (unitary: the norm
  // stays 1); the result written is the state after warmup + reps passes
  for (int r = 0; r < warmup; ++r) {
    pass();
    auto c = state->copy();
  }
  sync(env);
  const double t0 = now_ms();
  for (int r = 0; r < reps; ++r) {
    pass();
    auto c = state->copy();  // waits on the queued contractions' results (D2D copy)
  }
  sync(env);
  const double ms = (now_ms() - t0) / reps;
  write_state(out, *state);
  std::printf("{\"mode\": \"circuit\", \"runs\": %d, \"ms_per_run\": %.6f, \"contractions_per_run\": %zu, "
              "\"layers\": %d}\n",
              reps, ms, contractions, nl);
  return 0;
}

// The QFT network; returns the bond order and the state tensor's ID.
std::vector<qtnh::uint> qft_network(const QTNHEnv& env, TensorNetwork& tn, int n, int dq, std::vector<tel>&& psi,
                                    std::size_t& contractions) {
  std::vector<qtnh::uint> order;
  const qtnh::uint st = tn.make<DenseTensor>(env, tidx_tup(dq, 2), tidx_tup(n - dq, 2), std::move(psi));
  std::vector<qtnh::uint> qid(n, st);  // tensor holding qubit q, and its index there
  std::vector<tidx_tup_st> qidx(n);
  for (int q = 0; q < n; ++q) qidx[q] = (tidx_tup_st)q;
  auto dist = [&](int in) { return tn.make<IdenTensor>(env, tidx_tup{2}, tidx_tup{2}, (tidx_tup_st)in, false); };
  const double s = std::pow(2, -.5);
  // one gate (tensor g with inputs 0..k-1 and outputs k..2k-1) on qubits qs
  auto apply = [&](qtnh::uint g, const std::vector<int>& qs) {
    const int k = (int)qs.size();
    std::vector<qtnh::uint> tin(k, g), tout(k, g);
    std::vector<tidx_tup_st> iin(k), iout(k);
    for (int m = 0; m < k; ++m) {
      iin[m] = (tidx_tup_st)m;
      iout[m] = (tidx_tup_st)(k + m);
      if (qs[m] < dq) {
        tin[m] = dist(1);
        order.push_back(tn.addBond(tin[m], g, {{1, (tidx_tup_st)m}}));
        iin[m] = 0;
        tout[m] = dist(0);
        order.push_back(tn.addBond(g, tout[m], {{(tidx_tup_st)(k + m), 1}}));
        iout[m] = 0;
        contractions += 2;
      }
    }
    for (int m = 0; m < k; ++m) order.push_back(tn.addBond(qid[qs[m]], tin[m], {{qidx[qs[m]], iin[m]}}));
    for (int m = 0; m < k; ++m) qid[qs[m]] = tout[m], qidx[qs[m]] = iout[m];
    contractions += 1;
  };
  for (int i = 0; i < n; ++i) {
    apply(tn.make<SymmTensor>(env, tidx_tup{}, tidx_tup{2, 2}, 0, std::vector<tel>{s, s, s, -s}), {i});
    for (int j = i + 1; j < n; ++j) {
      const tel ph = std::exp(1i * (M_PI / std::pow(2, j - i)));
      apply(tn.make<DiagTensor>(env, tidx_tup{}, tidx_tup{2, 2, 2, 2}, 0, false, std::vector<tel>{1.0, 1.0, 1.0, ph}),
            {i, j});
    }
  }
  for (int k = 0; k < n / 2; ++k) apply(tn.make<SwapTensor>(env, 2, 0), {k, n - 1 - k});
  return order;
}

int run_qft(int n, int dq, const std::string& in, const std::string& out, int warmup, int reps) {
  std::ifstream f(in, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + in);
  const std::vector<tel> psi = get_els(f, (std::size_t)1 << n);
  QTNHEnv env;
  std::size_t contractions = 0;
  tptr result;
  std::vector<tel> host((std::size_t)1 << n);
  auto one = [&]() {
    TensorNetwork tn;
    contractions = 0;
    auto order = qft_network(env, tn, n, dq, std::vector<tel>(psi), contractions);
    result = tn.extract(tn.contractAll(order));
    // the amplitudes back on the host (the result's own index order)
    if (qtnh_memcpy_d2h(host.data(), result->engineData(), host.size() * sizeof(tel), env.stream) != QTNH_OK)
      throw std::runtime_error(qtnh_last_error());
    sync(env);
  };
  for (int r = 0; r < warmup; ++r) one();
  const double t0 = now_ms();
  for (int r = 0; r < reps; ++r) one();
  const double ms = (now_ms() - t0) / reps;
  write_state(out, *result);
  std::printf("{\"mode\": \"qft\", \"runs\": %d, \"ms_per_run\": %.6f, \"contractions_per_run\": %zu, "
              "\"qubits\": %d, \"dq\": %d, \"dims\": [",
              reps, ms, contractions, n, dq);
  const auto d = result->totDims();
  for (std::size_t i = 0; i < d.size(); ++i) std::printf("%s%zu", i ? ", " : "", (std::size_t)d[i]);
  std::printf("], \"ndis\": %zu}\n", result->disDims().size());
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    const std::string mode = argc > 1 ? argv[1] : "";
    if (mode == "circuit" && argc == 6) return run_circuit(argv[2], argv[3], std::atoi(argv[4]), std::atoi(argv[5]));
    if (mode == "qft" && argc == 8)
      return run_qft(std::atoi(argv[2]), std::atoi(argv[3]), argv[4], argv[5], std::atoi(argv[6]), std::atoi(argv[7]));
    std::cerr << "usage: api_bench circuit <in.bin> <out.bin> <warmup> <reps>\n"
                 "       api_bench qft <n> <dq> <in.bin> <out.bin> <warmup> <reps>\n";
    return 2;
  } catch (const std::exception& e) {
    std::cerr << "api_bench: " << e.what() << "\n";
    return 1;
  }
}
