// Two disjoint two-qubit gates fused into one 16x16 unitary, applied in place on the
// tensor cores with error-free bf16 digits (ozaki.cuh) -- the mma.sync kernel, used for
// states below 2048 amplitudes (gate_umma.cu holds the tcgen05 kernel for the rest; the
// two run at the same speed on large states and give identical results).
//
// A gate layer holds disjoint gates, which commute, so consecutive pairs of a
// qtnh_apply_gate_layer call fuse into U = U_a (x) U_b acting on the 16 amplitudes of a
// group (the four target bits varying). In real form the group update is y = R x with
// R = [[Re U, -Im U], [Im U, Re U]] (32 x 32) and x the 32 reals of the group. Per warp,
// eight groups form the N = 8 columns of mma.sync.m16n8k16 tiles:
//   * each lane fetches four complex amplitudes (2t, 2t+1, 2t+8, 2t+9 of group g =
//     lane / 4, t = lane % 4) -- exactly the B-fragment rows it owns for both k-tiles
//     (real parts k-tile 0, imaginary parts k-tile 1) -- two tiles ahead with cp.async,
//     takes the group's largest exponent with two shuffles and cuts its 8 reals into 6
//     balanced bf16 digits each;
//   * R's six digits (per-row exponents) are laid out once per CTA in shared memory as
//     per-lane A fragments;
//   * 21 digit pairs (i + j <= 5) x 2 m-tiles x 2 k-tiles = 84 MMAs accumulate six exact
//     FP32 level sums per output;
//   * every output real is recombined (compensated adds) and written back.
// A warp whose groups hold an infinity/NaN or a largest magnitude outside 2^-200..2^201
// takes an FP64 path for its eight groups (warp-uniform branch). Subnormal amplitudes
// (below 2^-1022) contribute zero digits: their weight against the group scale is below
// 2^-822.

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "gate_pair.cuh"

namespace qtnh_impl {

namespace {

constexpr int TC_THREADS = 256;
constexpr int TC_WARPS = TC_THREADS / 32;
constexpr int TC_STAGES = 2;

// Shared memory of one CTA (dynamic, 16-byte aligned).
struct TcSmem {
  uint4 afrag[oz::NS][2][2][32];              // digit, m-tile, k-tile, lane
  double2 U16[256];                           // fused unitary, U16[o * 16 + i]
  double2 stage[TC_STAGES][TC_WARPS][4][32];  // prefetched amplitudes: stage, warp, q, lane
  int32_t erow[16];                           // max exponent of row o of R (= of row 16 + o)
  int gate_ok;
};

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint4& a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

// FP64 path for one warp's eight groups (all loads before the first store); gbase is
// the lane's group base.
template <typename IT>
__device__ __noinline__ void pair_tile_fp64(double2* __restrict__ psi, IT gbase, const PairParams& p,
                                            const double2* U16) {
  const int lane = threadIdx.x & 31;
  double2 x[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) x[i] = psi[gbase + (IT)p.off[i]];
  __syncwarp();
  const int o0 = (lane & 3) * 4;
#pragma unroll
  for (int oo = 0; oo < 4; ++oo) {
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int i = 0; i < 16; ++i) acc = cfma(U16[(o0 + oo) * 16 + i], x[i], acc);
    psi[gbase + (IT)p.off[o0 + oo]] = acc;
  }
}

// Two CTAs per SM: up to 128 registers a thread, none spilled (three CTAs spill and run
// slower).
template <typename IT, uint32_t MODE>
__global__ void __launch_bounds__(TC_THREADS, 2) gate_pair_tc_kernel(double2* __restrict__ psi,
                                                                     const double2* __restrict__ ga,
                                                                     const double2* __restrict__ gb,
                                                                     const __grid_constant__ PairParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
  const int tid = threadIdx.x;

  // ---- the fused gate: U16, row exponents, A fragments of its six digits ----
  if (tid == 0) sm.gate_ok = 1;
  for (int t = tid; t < 256; t += TC_THREADS) sm.U16[t] = fused_entry<MODE>(ga, gb, t);
  __syncthreads();
  if (tid < 16) {
    bool ok;
    sm.erow[tid] = (int32_t)row_exponent(sm.U16, tid, ok);
    if (!ok) sm.gate_ok = 0;
  }
  __syncthreads();
  // entries (r, k), (r, k + 1) of digit i form half 0 / 1 of register
  // (r % 16) / 8 + 2 ((k % 16) / 8) of lane (r % 8) * 4 + (k % 8) / 2 in afrag[i][r / 16][k / 16]
  for (int t = tid; t < 512; t += TC_THREADS) {
    const int r = t >> 4, k = (t & 15) * 2;
    const uint32_t E = oz::digit_scale((uint32_t)sm.erow[r & 15]);
    float d0[oz::NS], d1[oz::NS];
    oz::digits(df::words(real_form(sm.U16, r, k)), E, d0);
    oz::digits(df::words(real_form(sm.U16, r, k + 1)), E, d1);
    const int rr = r & 15, kk = k & 15;
    const int lane = (rr & 7) * 4 + ((kk & 7) >> 1);
    const int reg = (rr >> 3) + 2 * (kk >> 3);
#pragma unroll
    for (int i = 0; i < oz::NS; ++i)
      reinterpret_cast<uint32_t*>(&sm.afrag[i][r >> 4][k >> 4][lane])[reg] = oz::pack(d0[i], d1[i]);
  }
  __syncthreads();
  const bool gok = sm.gate_ok != 0;

  // ---- per-lane constants ----
  const int lane = tid & 31, warp = tid >> 5, g = lane >> 2, t = lane & 3;
  IT ld_off[4];  // the lane's four amplitudes relative to the tile base
  {
    const IT gb0 = pair_base<IT>((IT)g, p);
    const int am[4] = {2 * t, 2 * t + 1, 2 * t + 8, 2 * t + 9};
#pragma unroll
    for (int q = 0; q < 4; ++q) ld_off[q] = gb0 + (IT)p.off[am[q]];
  }
  IT st_off[4];  // outputs c: row g + 8 (c / 2) of group 2t + (c % 2)
  {
    const IT c0 = pair_base<IT>((IT)(2 * t), p), c1 = pair_base<IT>((IT)(2 * t + 1), p);
#pragma unroll
    for (int c = 0; c < 4; ++c) st_off[c] = ((c & 1) ? c1 : c0) + (IT)p.off[g + ((c >> 1) << 3)];
  }
  const IT my_group = pair_base<IT>((IT)g, p);
  uint32_t krow[2];  // scale bits of the lane's rows without the group exponent
  krow[0] = oz::scale_bits(sm.erow[g]);
  krow[1] = oz::scale_bits(sm.erow[g + 8]);

  const uint64_t nwarps = (uint64_t)gridDim.x * TC_WARPS;
  const uint64_t first = (uint64_t)blockIdx.x * TC_WARPS + warp;
  const uint64_t ntiles = p.ngroups / 8;

  // tile base of a tile (its first group's first amplitude), computed when it is fetched
  auto prefetch = [&](uint64_t tile, int s) -> IT {
    IT tb = 0;
    if (tile < ntiles) {
      tb = pair_base<IT>((IT)(tile * 8), p);
#pragma unroll
      for (int q = 0; q < 4; ++q) cp_async16(&sm.stage[s][warp][q][lane], psi + (tb + ld_off[q]));
    }
    cp_async_commit();
    return tb;
  };

  IT tb_next = prefetch(first, 0);
  IT tb_next2 = prefetch(first + nwarps, 1);
  int s = 0;
  for (uint64_t tile = first; tile < ntiles; tile += nwarps, s ^= 1) {
    cp_async_wait_one();
    double2 x[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) x[q] = sm.stage[s][warp][q][lane];
    uint32_t key = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      key = max(key, max(oz::group_key(df::words(x[q].x)), oz::group_key(df::words(x[q].y))));
    key = max(key, __shfl_xor_sync(0xffffffffu, key, 1));
    key = max(key, __shfl_xor_sync(0xffffffffu, key, 2));
    const uint32_t emax = oz::key_exponent(key), escale = oz::digit_scale(emax);
    // the stage's values are in registers (used above): refill it two tiles ahead
    const IT tb = tb_next;
    tb_next = tb_next2;
    tb_next2 = prefetch(tile + 2 * nwarps, s);
    if (!__all_sync(0xffffffffu, gok && tc_scale_ok(emax))) {
      pair_tile_fp64<IT>(psi, tb + my_group, p, sm.U16);
      continue;
    }
    // B fragments: bf[j][kt][0] = {x_kt[2t], x_kt[2t+1]}, bf[j][kt][1] = {x_kt[2t+8], x_kt[2t+9]}
    uint32_t bf[oz::NS][2][2];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float d0[oz::NS], d1[oz::NS];
        oz::digits(df::words(kt ? x[2 * h].y : x[2 * h].x), escale, d0);
        oz::digits(df::words(kt ? x[2 * h + 1].y : x[2 * h + 1].x), escale, d1);
#pragma unroll
        for (int j = 0; j < oz::NS; ++j) bf[j][kt][h] = oz::pack(d0[j], d1[j]);
      }
    }
    // outputs: rows g, g+8 (amplitude), columns 2t, 2t+1 (group); m-tile 0 gives the
    // real parts, m-tile 1 the imaginary parts (one m-tile at a time: fewer live registers)
    const uint32_t ecol[2] = {__shfl_sync(0xffffffffu, emax, (2 * t) * 4) << 20,
                              __shfl_sync(0xffffffffu, emax, (2 * t + 1) * 4) << 20};
    // real parts written after m-tile 0, imaginary parts after m-tile 1
    double* out = reinterpret_cast<double*>(psi);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      float acc[oz::NL][4];
#pragma unroll
      for (int l = 0; l < oz::NL; ++l)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[l][c] = 0.0f;
#pragma unroll
      for (int i = 0; i < oz::NS; ++i) {
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
          const uint4 a = sm.afrag[i][mt][kt][lane];
#pragma unroll
          for (int j = 0; j < oz::NS; ++j)
            if (i + j < oz::NL) mma_bf16(acc[i + j], a, bf[j][kt][0], bf[j][kt][1]);
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float lv[oz::NL];
#pragma unroll
        for (int l = 0; l < oz::NL; ++l) lv[l] = acc[l][c];
        out[2 * (size_t)(tb + st_off[c]) + mt] = oz::combine(lv, ecol[c & 1] + krow[c >> 1]);
      }
    }
  }
  cp_async_wait_all();
}

template <typename IT, uint32_t MODE>
void launch_pair(double2* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s) {
  const size_t smem = sizeof(TcSmem);
  check_cuda(cudaFuncSetAttribute(gate_pair_tc_kernel<IT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
             "gate_pair_tc_kernel shared memory");
  const int grid = grid_for(((p.ngroups / 8) + TC_WARPS - 1) / TC_WARPS, 2);
  gate_pair_tc_kernel<IT, MODE><<<grid, TC_THREADS, smem, s>>>(psi, ga, gb, p);
}

}  // namespace

PairParams make_pair_params(const dims_t& dims, const uint16_t all[4]) {
  const dims_t st = row_strides(dims);
  PairParams p;
  p.ngroups = product(dims) / 16;
  uint16_t srt[4] = {all[0], all[1], all[2], all[3]};
  std::sort(srt, srt + 4, [&](uint16_t x, uint16_t y) { return st[x] < st[y]; });
  for (int j = 0; j < 4; ++j) p.ins_pos[j] = log2_or_none(st[srt[j]]);
  for (int c = 0; c < 16; ++c)
    p.off[c] = (int64_t)(((c >> 3) & 1) * st[all[0]] + ((c >> 2) & 1) * st[all[1]] + ((c >> 1) & 1) * st[all[2]] +
                         (c & 1) * st[all[3]]);
  return p;
}

namespace {

// The 4x4 identity in SymmTensor layout: the second gate of a lone gate's pair.
__device__ const double2 g_identity4[16] = {{1.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0},
                                            {0.0, 0.0}, {1.0, 0.0}, {0.0, 0.0}, {0.0, 0.0},
                                            {0.0, 0.0}, {0.0, 0.0}, {1.0, 0.0}, {0.0, 0.0},
                                            {0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}, {1.0, 0.0}};

// tcgen05 kernel from one 128-group tile up, mma.sync kernel below.
void launch_fused_pair(double2* psi, const double2* a, const double2* b, const PairParams& p, uint64_t n,
                       cudaStream_t s, uint32_t mode = PAIR_KRON) {
  if (!launch_pair_umma(psi, a, b, p, s, mode)) {
    if (mode == PAIR_KRON) {
      if (n <= (1ull << 32))
        launch_pair<uint32_t, PAIR_KRON>(psi, a, b, p, s);
      else
        launch_pair<uint64_t, PAIR_KRON>(psi, a, b, p, s);
    } else if (mode == PAIR_FULL) {
      launch_pair<uint32_t, PAIR_FULL>(psi, a, b, p, s);
    } else {
      launch_pair<uint32_t, PAIR_KRON_I2>(psi, a, b, p, s);
    }
  }
  count_launch();
  check_cuda(cudaGetLastError(), "gate pair kernel launch");
}

}  // namespace

bool apply_gate_tc_single(void* state, const dims_t& dims, const std::vector<uint16_t>& targets, const void* gate,
                          void* stream) {
  const size_t k = targets.size();
  if (k < 2 || k > 4) return false;
  for (auto d : dims)
    if (log2_or_none(d) == 0xFFFFFFFFu) return false;
  for (auto t : targets)
    if (dims[t] != 2) return false;
  const uint64_t n = product(dims);
  if (n < 128 || (k > 2 && n > (1ull << 32))) return false;
  // the identity factor takes the free size-2 axes of largest stride: the groups' varying
  // bits then stay above the low bits that consecutive groups run over
  uint16_t tg[4];
  for (size_t j = 0; j < k; ++j) tg[j] = targets[j];
  size_t found = k;
  for (size_t a = 0; a < dims.size() && found < 4; ++a)
    if (dims[a] == 2 && std::find(targets.begin(), targets.end(), (uint16_t)a) == targets.end()) tg[found++] = (uint16_t)a;
  if (found < 4) return false;
  const double2* g = static_cast<const double2*>(gate);
  const double2* second = nullptr;
  uint32_t mode = PAIR_FULL;
  if (k == 2) {
    void* ident = nullptr;
    check_cuda(cudaGetSymbolAddress(&ident, g_identity4), "identity gate address");
    second = static_cast<const double2*>(ident);
    mode = PAIR_KRON;
  } else if (k == 3) {
    mode = PAIR_KRON_I2;
  }
  launch_fused_pair(static_cast<double2*>(state), g, second, make_pair_params(dims, tg), n, (cudaStream_t)stream, mode);
  return true;
}

namespace {

// QTNH_GATE_CHAIN=0 keeps every pass of a layer in doubles (no fixed-point chain).
bool chain_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("QTNH_GATE_CHAIN");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  return on;
}

struct LayerStep {
  size_t g;        // first gate
  bool pair;       // gates g and g + 1 fused, else gate g alone
  PairParams p;    // pair parameters
  int perm;        // >= 0: not a gate but the permutation after run `perm`
  dims_t dims;     // the state's dims at this step (before the permutation)
};

// QTNH_FUSE_PERMUTE=0 keeps a permutation after a chain pass as a pass of its own.
bool fuse_permutes() {
  static const bool on = [] {
    const char* e = std::getenv("QTNH_FUSE_PERMUTE");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  return on;
}

// Optional CUDA-event timing of the tensor-core gate-pass launches (qtnh_gate_timing).
std::mutex g_pass_mu;
bool g_pass_timing = false;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_pass_events;

template <typename F>
void timed_pass(cudaStream_t s, F&& launch) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_pass_mu);
    if (g_pass_timing) {
      check_cuda(cudaEventCreate(&e0), "event");
      check_cuda(cudaEventCreate(&e1), "event");
    }
  }
  if (e0) check_cuda(cudaEventRecord(e0, s), "event record");
  launch();
  if (e1) {
    check_cuda(cudaEventRecord(e1, s), "event record");
    std::lock_guard<std::mutex> lk(g_pass_mu);
    g_pass_events.emplace_back(e0, e1);
  }
}

}  // namespace

// Pairs of consecutive, disjoint two-qubit gates on a power-of-two state are fused and
// applied on the tensor cores; everything else goes through apply_gate_device (where a
// lone gate on two, three or four qubits runs on the tensor cores too). A run of two or
// more fused pairs on the tcgen05 tile shape is a chain: the first pass reads and writes
// doubles and records their largest exponent, the next ones cut the state at that one
// scale and pass it on as 64-bit fixed point, the last writes doubles (ozaki.cuh,
// gate_umma.cu). A permutation between two runs of gates (runs[r].ptup) moves the
// elements from one buffer to the other; inside a chain it moves the fixed-point form
// (16-byte elements, values unchanged, so the chain's record still holds). Returns whether
// the result is in `scratch` (an odd number of permutations); all launches are issued.
bool apply_gate_runs_tc(void* state, void* scratch, dims_t dims, const std::vector<GateRun>& runs, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<LayerStep> steps;
  std::vector<const void*> gates;
  std::vector<std::vector<uint16_t>> targets;
  for (size_t r = 0; r < runs.size(); ++r) {
    const size_t rk = dims.size();
    bool pow2 = true;
    for (auto d : dims) pow2 = pow2 && log2_or_none(d) != 0xFFFFFFFFu;
    const uint64_t n = product(dims);
    const size_t base = gates.size();
    gates.insert(gates.end(), runs[r].gates.begin(), runs[r].gates.end());
    targets.insert(targets.end(), runs[r].targets.begin(), runs[r].targets.end());
    size_t g = base;
    while (g < gates.size()) {
      bool fused = false;
      if (pow2 && n >= 128 && g + 1 < gates.size() && targets[g].size() == 2 && targets[g + 1].size() == 2) {
        const auto& ta = targets[g];
        const auto& tb = targets[g + 1];
        std::vector<uint16_t> all = {ta[0], ta[1], tb[0], tb[1]};
        bool ok = true;
        for (auto a : all) ok = ok && a < rk && dims[a] == 2;
        std::vector<uint16_t> srt(all);
        std::sort(srt.begin(), srt.end());
        ok = ok && std::adjacent_find(srt.begin(), srt.end()) == srt.end();
        if (ok) {
          const uint16_t tg[4] = {ta[0], ta[1], tb[0], tb[1]};
          steps.push_back({g, true, make_pair_params(dims, tg), -1, dims});
          g += 2;
          fused = true;
        }
      }
      if (!fused) {
        steps.push_back({g, false, PairParams{}, -1, dims});
        g += 1;
      }
    }
    if (!runs[r].ptup.empty()) {
      steps.push_back({0, false, PairParams{}, (int)r, dims});
      dims_t nd(dims.size());
      for (size_t i = 0; i < dims.size(); ++i) nd[runs[r].ptup[i]] = dims[i];
      dims = nd;
    }
  }
  void* cur = state;
  void* oth = scratch;
  auto gate_ptr = [&](size_t i) { return static_cast<const double2*>(gates[i]); };
  auto permute = [&](const LayerStep& st) {
    permute_device(cur, oth, st.dims, runs[(size_t)st.perm].ptup, stream);
    std::swap(cur, oth);
  };
  size_t i = 0;
  while (i < steps.size()) {
    if (steps[i].perm >= 0) {
      permute(steps[i]);
      ++i;
      continue;
    }
    // a chain: fused pairs on the tile shape, with permutations between them
    size_t j = i, last = i, R = 0;
    while (j < steps.size() && (steps[j].perm >= 0 || (steps[j].pair && chain_applies(steps[j].p)))) {
      if (steps[j].perm < 0) ++R, last = j;
      ++j;
    }
    if (R >= 2 && chain_enabled()) {
      ChainRec* recs = static_cast<ChainRec*>(workspace_alloc(R * sizeof(ChainRec), stream));
      try {
        check_cuda(cudaMemsetAsync(recs, 0, R * sizeof(ChainRec), s), "clear chain records");
        size_t k = 0, t = i;
        for (; t <= last; ++t) {
          const LayerStep& sk = steps[t];
          if (sk.perm >= 0) {
            permute(sk);
            continue;
          }
          double2* psi = static_cast<double2*>(cur);
          // a chain pass followed by a permutation writes its outputs permuted, out of place
          BitPerm bp;
          const bool fuse = k > 0 && t + 1 < steps.size() && steps[t + 1].perm >= 0 && fuse_permutes() &&
                            make_bit_perm(steps[t + 1].dims, runs[(size_t)steps[t + 1].perm].ptup, sk.p, bp);
          if (k == 0)
            timed_pass(s, [&] { launch_pair_umma(psi, gate_ptr(sk.g), gate_ptr(sk.g + 1), sk.p, s, PAIR_KRON, &recs[0]); });
          else
            timed_pass(s, [&] {
              launch_pair_chain(psi, gate_ptr(sk.g), gate_ptr(sk.g + 1), sk.p, s, &recs[k - 1], &recs[k], k + 1 < R,
                                fuse ? oth : nullptr, fuse ? &bp : nullptr);
            });
          count_launch();
          ++k;
          if (fuse) {
            std::swap(cur, oth);
            ++t;  // the permutation is done
          }
        }
        check_cuda(cudaGetLastError(), "gate chain launch");
        i = t;
      } catch (...) {
        workspace_free(recs, stream);
        throw;
      }
      workspace_free(recs, stream);
      continue;
    }
    const LayerStep& st = steps[i];
    if (st.pair)
      timed_pass(s, [&] { launch_fused_pair(static_cast<double2*>(cur), gate_ptr(st.g), gate_ptr(st.g + 1), st.p,
                                            product(st.dims), s); });
    else
      apply_gate_device(cur, st.dims, targets[st.g], gates[st.g], stream);
    ++i;
  }
  return cur != state;
}

void apply_gate_layer_tc(void* state, const dims_t& dims, const std::vector<std::vector<uint16_t>>& targets,
                         const std::vector<const void*>& gates, void* stream) {
  std::vector<GateRun> runs(1);
  runs[0].targets = targets;
  runs[0].gates = gates;
  apply_gate_runs_tc(state, nullptr, dims, runs, stream);
}

void take_pass_times(double& ms, uint64_t& launches) {
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  {
    std::lock_guard<std::mutex> lk(g_pass_mu);
    ev.swap(g_pass_events);
  }
  ms = 0;
  launches = ev.size();
  for (auto& e : ev) {
    float t = 0;
    check_cuda(cudaEventSynchronize(e.second), "event synchronize");
    check_cuda(cudaEventElapsedTime(&t, e.first, e.second), "event elapsed");
    ms += t;
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
}

void set_pass_timing(bool on) {
  std::lock_guard<std::mutex> lk(g_pass_mu);
  g_pass_timing = on;
}

}  // namespace qtnh_impl
