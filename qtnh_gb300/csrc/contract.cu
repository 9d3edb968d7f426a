// Dense contraction: the global form of _contract_dense (src/tensor/contract.cpp:12-201).
//
// The reference permutes the contracted distributed indices, re-broadcasts both
// operands, runs a triple loop over (t1 open local) x (t2 open local) x (closed) with
// per-element iterator objects, all-reduces the contracted distributed indices over MPI
// and permutes the result. With all slabs resident, distributed and local wires are the
// same summation, so the contraction is
//     A' = permute(A) to [open A | wired]      (M x K, row-major)
//     B' = permute(B) to [wired | open B]      (K x N, row-major)
//     C' = A' B'                               (complex FP64 GEMM)
//     C  = permute(C') to the replacement order (contract.cpp:86-111, 180-200)
// where each permute is skipped when it is the identity. The complex GEMM runs on the
// FP64 FMA pipe: on GB300 it is faster than FP64 DMMA (measured 1.20 vs 1.05 TFLOP/s),
// and both are far below the BF16/TF32 tensor rate, which the split-precision path uses.

#include <algorithm>
#include <numeric>

#include "cuda_common.cuh"

namespace qtnh_impl {

namespace {

constexpr int BM = 64, BN = 64, BK = 8, GEMM_THREADS = 256;

// C[M x N] = A[M x K] * B[K x N], all row-major, complex<double>.
// 256 threads, 64 x 64 tile, each thread 4 x 4 outputs at rows ty + 16 i, cols tx + 16 j.
__global__ void __launch_bounds__(GEMM_THREADS) zgemm_kernel(const c128* __restrict__ A, const c128* __restrict__ B,
                                                             c128* __restrict__ C, uint64_t M, uint64_t N, uint64_t K) {
  __shared__ c128 As[BK][BM];
  __shared__ c128 Bs[BK][BN];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const uint64_t m0 = (uint64_t)blockIdx.y * BM, n0 = (uint64_t)blockIdx.x * BN;
  c128 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);

  for (uint64_t k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      int idx = tid + r * GEMM_THREADS;
      int am = idx >> 3, ak = idx & 7;
      uint64_t gm = m0 + am, gk = k0 + ak;
      As[ak][am] = (gm < M && gk < K) ? __ldg(A + gm * K + gk) : make_double2(0.0, 0.0);
      int bk = idx >> 6, bn = idx & 63;
      uint64_t gk2 = k0 + bk, gn = n0 + bn;
      Bs[bk][bn] = (gk2 < K && gn < N) ? __ldg(B + gk2 * N + gn) : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      c128 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cfma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint64_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uint64_t gn = n0 + tx + 16 * j;
      if (gn < N) C[gm * N + gn] = acc[i][j];
    }
  }
}

}  // namespace

// The FP64 GEMM's grid has one block row per 64 rows of C (grid y is at most 65535).
void zgemm_check_shape(uint64_t M, uint64_t N) {
  (void)N;
  if ((M + BM - 1) / BM > 65535) throw Error(QTNH_ERR_UNSUPPORTED, "GEMM M dimension too large");
}

namespace {

void zgemm(const c128* A, const c128* B, c128* C, uint64_t M, uint64_t N, uint64_t K, cudaStream_t s) {
  if (M == 0 || N == 0) return;
  zgemm_check_shape(M, N);
  uint64_t gx = (N + BN - 1) / BN, gy = (M + BM - 1) / BM;
  zgemm_kernel<<<dim3((unsigned)gx, (unsigned)gy), GEMM_THREADS, 0, s>>>(A, B, C, M, N, K);
  count_launch();
  check_cuda(cudaGetLastError(), "zgemm_kernel launch");
}

// Dense elements of an implicit tensor (SwapTensor symm.cpp:584-591, IdenTensor
// diag.cpp:143-151, DiagTensor d[in] * delta(in, out)).
struct MaterialiseParams {
  int kind, rank, n_dis_in, ndis, nli;
  uint64_t dims[KMAX];
  uint64_t total;
};

__global__ void materialise_kernel(const c128* __restrict__ diag, c128* __restrict__ out,
                                   const __grid_constant__ MaterialiseParams p) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < p.total; e += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t idx[KMAX];
    uint64_t rem = e;
    for (int k = p.rank - 1; k >= 0; --k) idx[k] = rem % p.dims[k], rem /= p.dims[k];
    c128 v = make_double2(0.0, 0.0);
    if (p.kind == QTNH_KIND_SWAP) {
      if (idx[0] == idx[3] && idx[1] == idx[2]) v.x = 1.0;
    } else if (p.kind == QTNH_KIND_IDEN) {
      int h = p.rank / 2;
      bool eq = true;
      for (int i = 0; i < h; ++i) eq = eq && (idx[i] == idx[h + i]);
      if (eq) v.x = 1.0;
    } else {  // DIAG: inputs = dis[0:ndi] ++ loc[0:nli], outputs = the rest, in order
      const int ndi = p.n_dis_in, nd = p.ndis, nli = p.nli;
      const int nlo = p.rank - nd - nli;
      bool eq = (nd - ndi) + nlo == ndi + nli;
      uint64_t din = 0;
      for (int j = 0, io = 0; eq && j < ndi + nli; ++j) {
        int ii = (j < ndi) ? j : nd + (j - ndi);
        int oo = (io < nd - ndi) ? ndi + io : nd + nli + (io - (nd - ndi));
        ++io;
        eq = idx[ii] == idx[oo];
        din = din * p.dims[ii] + idx[ii];
      }
      if (eq) v = __ldg(diag + din);
    }
    out[e] = v;
  }
}

bool is_identity(const std::vector<uint16_t>& p) {
  for (size_t i = 0; i < p.size(); ++i)
    if (p[i] != i) return false;
  return true;
}

}  // namespace

// Whether the default plain GEMM runs on the tensor cores (gemm_oz.cu): from 2^18 complex
// multiply-adds and a contracted size of 16 on. Below that the digit preparation costs
// more than FP64 FMAs, and the FMA GEMM keeps the small-K contractions of relabelling
// tensors (0/1 entries, one term per output, e.g. a SwapTensor wrapped in identity tensors)
// bit-exact.
bool oz6_applies(uint64_t M, uint64_t N, uint64_t K) {
  const double work = (double)M * (double)N * (double)K;
  return work >= 262144.0 && K >= 16;
}

// GEMM launcher shared with the allocation-free contraction (noalloc.cu).
void zgemm_launch(const c128* A, const c128* B, c128* C, uint64_t M, uint64_t N, uint64_t K, cudaStream_t s) {
  zgemm(A, B, C, M, N, K, s);
}

void materialise_device(const TensorMeta& t, const void* data, void* out, void* stream) {
  MaterialiseParams p;
  dims_t tot = t.tot();
  if ((int)tot.size() > KMAX) throw Error(QTNH_ERR_UNSUPPORTED, "rank too large");
  p.kind = t.kind;
  p.rank = (int)tot.size();
  p.n_dis_in = t.n_dis_in;
  p.ndis = (int)t.dis.size();
  p.nli = (t.kind == QTNH_KIND_DIAG) ? (int)t.n_loc_in() : 0;
  for (int i = 0; i < p.rank; ++i) p.dims[i] = tot[i];
  p.total = product(tot);
  cudaStream_t s = (cudaStream_t)stream;
  if (t.kind == QTNH_KIND_DENSE || t.kind == QTNH_KIND_SYMM) {
    check_cuda(cudaMemcpyAsync(out, data, p.total * sizeof(c128), cudaMemcpyDeviceToDevice, s), "copy");
    return;
  }
  materialise_kernel<<<grid_for((p.total + 255) / 256, 4), 256, 0, s>>>(static_cast<const c128*>(data),
                                                                         static_cast<c128*>(out), p);
  count_launch();
  check_cuda(cudaGetLastError(), "materialise_kernel launch");
}

void contract_dense_device(const void* a, const dims_t& dims_a, const void* b, const dims_t& dims_b,
                           const std::vector<Wire>& wires, const std::vector<uint16_t>& pos_a,
                           const std::vector<uint16_t>& pos_b, void* c, void* stream, int gemm) {
  if (gemm < 0) gemm = gemm_mode();
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
  cudaStream_t s = (cudaStream_t)stream;
  const c128* A = static_cast<const c128*>(a);
  const c128* B = static_cast<const c128*>(b);

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

  c128* Ap = nullptr;
  c128* Bp = nullptr;
  c128* Cp = nullptr;
  if (gemm == QTNH_GEMM_OZ6 && oz6_applies(M, N, K)) {
    // FP64-accurate digit products on the tensor cores: A permuted to [open A | wired]
    // (M x K), B to [open B | wired] (N x K), the contracted index innermost in both
    std::vector<uint16_t> pBt(rb);
    for (size_t y = 0; y < openB.size(); ++y) pBt[openB[y]] = (uint16_t)y;
    for (size_t j = 0; j < wires.size(); ++j) pBt[wires[j].second] = (uint16_t)(openB.size() + j);
    const bool direct = is_identity(pC);
    try {
      if (!is_identity(pA)) {
        Ap = static_cast<c128*>(workspace_alloc(M * K * sizeof(c128), stream));
        permute_device(A, Ap, dims_a, pA, stream);
      }
      if (!is_identity(pBt)) {
        Bp = static_cast<c128*>(workspace_alloc(K * N * sizeof(c128), stream));
        permute_device(B, Bp, dims_b, pBt, stream);
      }
      if (!direct) Cp = static_cast<c128*>(workspace_alloc(M * N * sizeof(c128), stream));
      gemm_oz6(Ap ? Ap : A, Bp ? Bp : B, direct ? static_cast<c128*>(c) : Cp, M, N, K, stream);
      if (!direct) permute_device(Cp, c, dC, pC, stream);
    } catch (...) {
      workspace_free(Ap, stream);
      workspace_free(Bp, stream);
      workspace_free(Cp, stream);
      throw;
    }
    workspace_free(Ap, stream);
    workspace_free(Bp, stream);
    workspace_free(Cp, stream);
    return;
  }
  if (gemm == QTNH_GEMM_BF16X3) {
    // split precision: the operand permutes are fused into the piece splits
    std::vector<uint16_t> pBt(rb);
    for (size_t y = 0; y < openB.size(); ++y) pBt[openB[y]] = (uint16_t)y;
    for (size_t j = 0; j < wires.size(); ++j) pBt[wires[j].second] = (uint16_t)(openB.size() + j);
    const bool direct = is_identity(pC);
    try {
      if (!direct) Cp = static_cast<c128*>(workspace_alloc(M * N * sizeof(c128), stream));
      gemm_bf16x3_perm(A, dims_a, pA, (int)openA.size(), B, dims_b, pB, pBt, (int)openB.size(),
                       direct ? static_cast<c128*>(c) : Cp, M, N, K, stream);
      if (!direct) permute_device(Cp, c, dC, pC, stream);
    } catch (...) {
      workspace_free(Cp, stream);
      throw;
    }
    workspace_free(Cp, stream);
    return;
  }
  try {
    if (!is_identity(pA)) {
      Ap = static_cast<c128*>(workspace_alloc(M * K * sizeof(c128), stream));
      permute_device(A, Ap, dims_a, pA, stream);
    }
    if (!is_identity(pB)) {
      Bp = static_cast<c128*>(workspace_alloc(K * N * sizeof(c128), stream));
      permute_device(B, Bp, dims_b, pB, stream);
    }
    const bool direct = is_identity(pC);
    if (!direct) Cp = static_cast<c128*>(workspace_alloc(M * N * sizeof(c128), stream));
    zgemm(Ap ? Ap : A, Bp ? Bp : B, direct ? static_cast<c128*>(c) : Cp, M, N, K, s);
    if (!direct) permute_device(Cp, c, dC, pC, stream);
  } catch (...) {
    workspace_free(Ap, stream);
    workspace_free(Bp, stream);
    workspace_free(Cp, stream);
    throw;
  }
  workspace_free(Ap, stream);
  workspace_free(Bp, stream);
  workspace_free(Cp, stream);
}

}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" {

int qtnh_contract_dense(const void* a, int32_t rank_a, const uint64_t* dims_a, const void* b, int32_t rank_b,
                        const uint64_t* dims_b, int32_t nwires, const uint16_t* wires, const uint16_t* out_pos_a,
                        const uint16_t* out_pos_b, void* c, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank_a < 0 || rank_b < 0 || rank_a > QTNH_MAX_RANK || rank_b > QTNH_MAX_RANK || nwires < 0)
      throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    std::vector<Wire> ws(nwires);
    for (int32_t i = 0; i < nwires; ++i) ws[i] = {wires[2 * i], wires[2 * i + 1]};
    contract_dense_device(a, dims_t(dims_a, dims_a + rank_a), b, dims_t(dims_b, dims_b + rank_b), ws,
                          std::vector<uint16_t>(out_pos_a, out_pos_a + rank_a),
                          std::vector<uint16_t>(out_pos_b, out_pos_b + rank_b), c, stream);
    return QTNH_OK;
  });
}

}  // extern "C"
