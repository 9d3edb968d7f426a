// qtnh_contract_dense without device allocation.
//
// For callers that may not allocate device memory while they run (a host framework that
// owns all device memory, a fixed memory budget, or a latency-critical loop): the
// permuted copies of the operands and of the result, which the regular path takes from
// the stream-ordered pool, come from one scratch array defined here at file scope.
// The array is process-wide and shared by every call; its contents from an earlier call
// are overwritten before use (the permutes and the GEMM write every element they later
// read), so nothing has to be cleared. Calls that overlap on the GPU race on it.

#include <mutex>
#include <numeric>
#include <vector>

#include "cuda_common.cuh"

namespace qtnh_impl {

static __device__ __align__(256) double2 g_noalloc_scratch[QTNH_NOALLOC_SCRATCH_ELEMS];

namespace {

// Device address of the scratch array for the current device, looked up once per device
// with that device current (the host-side symbol is only a stand-in, not an address).
// A cudaDeviceReset unloads the module, so the address cached here is stale afterwards:
// the entry point is not for use after a cudaDeviceReset in the same process.
c128* scratch_for_current_device() {
  static std::mutex mu;
  static std::vector<void*> ptrs;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lock(mu);
  if ((int)ptrs.size() <= dev) ptrs.resize(dev + 1, nullptr);
  if (!ptrs[dev]) {
    void* p = nullptr;
    check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
    ptrs[dev] = p;
  }
  return static_cast<c128*>(ptrs[dev]);
}

bool identity(const std::vector<uint16_t>& p) {
  for (size_t i = 0; i < p.size(); ++i)
    if (p[i] != i) return false;
  return true;
}

}  // namespace

// Defined in contract.cu; reused here.
void zgemm_launch(const c128* A, const c128* B, c128* C, uint64_t M, uint64_t N, uint64_t K, cudaStream_t s);
void zgemm_check_shape(uint64_t M, uint64_t N);

void contract_dense_noalloc_device(const void* a, const dims_t& dims_a, const void* b, const dims_t& dims_b,
                                   const std::vector<Wire>& wires, const std::vector<uint16_t>& pos_a,
                                   const std::vector<uint16_t>& pos_b, void* c, void* stream) {
  const size_t ra = dims_a.size(), rb = dims_b.size();
  std::vector<char> wa(ra, 0), wb(rb, 0);
  for (auto& w : wires) {
    if (w.first >= ra || w.second >= rb) throw Error(QTNH_ERR_OUT_OF_RANGE, "wire index out of range");
    if (dims_a[w.first] != dims_b[w.second]) throw Error(QTNH_ERR_INVALID_ARGUMENT, "Incompatible contraction dimensions.");
    if (wa[w.first]++ || wb[w.second]++) throw Error(QTNH_ERR_INVALID_ARGUMENT, "An index is wired more than once.");
  }
  std::vector<int> openA, openB;
  for (size_t i = 0; i < ra; ++i)
    if (!wa[i]) openA.push_back((int)i);
  for (size_t i = 0; i < rb; ++i)
    if (!wb[i]) openB.push_back((int)i);
  const size_t nout = openA.size() + openB.size();
  std::vector<char> used(nout, 0);
  for (int i : openA)
    if (pos_a.at(i) >= nout || used[pos_a[i]]++) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid output position");
  for (int i : openB)
    if (pos_b.at(i) >= nout || used[pos_b[i]]++) throw Error(QTNH_ERR_INVALID_ARGUMENT, "invalid output position");

  uint64_t M = 1, N = 1, K = 1;
  for (int i : openA) M *= dims_a[i];
  for (int i : openB) N *= dims_b[i];
  for (auto& w : wires) K *= dims_a[w.first];

  std::vector<uint16_t> pA(ra), pB(rb), pC(nout);
  for (size_t x = 0; x < openA.size(); ++x) pA[openA[x]] = (uint16_t)x;
  for (size_t j = 0; j < wires.size(); ++j) pA[wires[j].first] = (uint16_t)(openA.size() + j);
  for (size_t j = 0; j < wires.size(); ++j) pB[wires[j].second] = (uint16_t)j;
  for (size_t y = 0; y < openB.size(); ++y) pB[openB[y]] = (uint16_t)(wires.size() + y);
  dims_t dC;
  for (int i : openA) dC.push_back(dims_a[i]);
  for (int i : openB) dC.push_back(dims_b[i]);
  for (size_t x = 0; x < openA.size(); ++x) pC[x] = pos_a[openA[x]];
  for (size_t y = 0; y < openB.size(); ++y) pC[openA.size() + y] = pos_b[openB[y]];

  zgemm_check_shape(M, N);  // refused before any work is queued
  const bool permA = !identity(pA), permB = !identity(pB), permC = !identity(pC);
  const uint64_t need = (permA ? M * K : 0) + (permB ? K * N : 0) + (permC ? M * N : 0);
  if (need > QTNH_NOALLOC_SCRATCH_ELEMS)
    throw Error(QTNH_ERR_UNSUPPORTED, "contraction needs " + std::to_string(need) +
                                          " scratch elements; the allocation-free path holds " +
                                          std::to_string((unsigned long long)QTNH_NOALLOC_SCRATCH_ELEMS));
  cudaStream_t s = (cudaStream_t)stream;
  c128* scratch = need ? scratch_for_current_device() : nullptr;
  c128* Ap = permA ? scratch : nullptr;
  c128* Bp = permB ? scratch + (permA ? M * K : 0) : nullptr;
  c128* Cp = permC ? scratch + (permA ? M * K : 0) + (permB ? K * N : 0) : nullptr;
  if (permA) permute_device(a, Ap, dims_a, pA, stream);
  if (permB) permute_device(b, Bp, dims_b, pB, stream);
  zgemm_launch(permA ? Ap : static_cast<const c128*>(a), permB ? Bp : static_cast<const c128*>(b),
               permC ? Cp : static_cast<c128*>(c), M, N, K, s);
  if (permC) permute_device(Cp, c, dC, pC, stream);
}

}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" int qtnh_contract_dense_noalloc(const void* a, int32_t rank_a, const uint64_t* dims_a, const void* b,
                                           int32_t rank_b, const uint64_t* dims_b, int32_t nwires, const uint16_t* wires,
                                           const uint16_t* out_pos_a, const uint16_t* out_pos_b, void* c, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank_a < 0 || rank_b < 0 || rank_a > QTNH_MAX_RANK || rank_b > QTNH_MAX_RANK || nwires < 0)
      throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    std::vector<Wire> ws(nwires);
    for (int32_t i = 0; i < nwires; ++i) ws[i] = {wires[2 * i], wires[2 * i + 1]};
    contract_dense_noalloc_device(a, dims_t(dims_a, dims_a + rank_a), b, dims_t(dims_b, dims_b + rank_b), ws,
                                  std::vector<uint16_t>(out_pos_a, out_pos_a + rank_a),
                                  std::vector<uint16_t>(out_pos_b, out_pos_b + rank_b), c, stream);
    return QTNH_OK;
  });
}
