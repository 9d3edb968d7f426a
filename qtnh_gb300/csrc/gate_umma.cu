// Fused gate pairs on the 5th-generation tensor cores (tcgen05): the same error-free bf16
// digit scheme as gate_tc.cu, with the MMA issued by one thread into tensor memory.
//
// A tile is 128 groups (16 amplitudes each). Per tile, D_l[g][o] = sum over digit pairs
// (i, j), i + j = l, of X_j[g][k] * R_i[o][k] (M = 128 groups, N = 32 output reals, K = 32
// input reals) -- 21 digit pairs x 2 K-steps = 42 tcgen05.mma (kind::f16, bf16 operands,
// FP32 accumulators) into six level column blocks of TMEM.
//
// CTA = 16 converting warps + one MMA warp, one CTA per SM (persistent), software-pipelined
// over the CTA's tiles with two buffers (fetched amplitudes, digits, TMEM level sums):
//   * group r of a tile belongs to four threads (warps r / 32 + 4 v, v = 0..3), each
//     owning amplitudes 4 v .. 4 v + 3: it fetches them two tiles ahead with cp.async,
//     the four exchange their largest exponents through shared memory (an mbarrier),
//     and each writes its 6 x 8 digits into shared memory in the UMMA K-major
//     core-matrix layout (8 rows x 16 bytes) and arrives on full[b];
//   * the MMA warp waits on full[b], issues the tile's 42 MMAs into TMEM buffer b and
//     commits them to done[b];
//   * meanwhile the converting warps recombine the previous tile: wait on its done,
//     read the level sums of their 4 amplitudes from their TMEM lane with tcgen05.ld,
//     recombine and store them; then the stage of the tile just converted is refilled.
// So the MMAs of tile m run while the warps finish tile m - 1, and every converting warp
// has work in every phase. Every wait is bounded by a clock limit; on expiry the CTA
// records an error flag, stops, lets its MMAs in flight finish and frees its tensor
// memory.
//
// Groups with an infinity/NaN or a largest magnitude outside 2^-200..2^201, and all
// groups when the gate has such entries, are computed in FP64 by their four threads.

#include <algorithm>

#include "gate_pair.cuh"

namespace qtnh_impl {

// bit 0: a wait for digits expired, bit 1: a wait for MMA completion expired, bit 2: a
// wait for the partner half's exponent expired
__device__ unsigned int g_umma_error;

namespace {

constexpr int UM_BUF = 2;                // pipeline buffers (tiles in flight)
constexpr int UM_WARPS = 16;             // converting warps (four threads per group)
constexpr int UM_THREADS = UM_WARPS * 32 + 32;
constexpr int UM_CONV = UM_WARPS * 32;   // converting threads
constexpr int UM_M = 128;                // groups per tile (MMA M)
constexpr int UM_N = 32;                 // output reals per group (MMA N)
constexpr int UM_COLS = 256;             // TMEM column stride of a buffer (its level sums use 32 * NL)
constexpr uint32_t UM_TMEM_COLS = 512;   // allocation (power of two >= UM_BUF * UM_COLS)
static_assert(oz::NL * UM_N <= UM_COLS, "level sums exceed a buffer's TMEM columns");
constexpr long long UM_WAIT_CYCLES = 1ll << 31;  // ~1 s at 2 GHz

// Shared memory of one CTA (dynamic). Operand layout (K-major, no swizzle): an 8-row x
// 16-byte core matrix is 128 contiguous bytes (row at 16 * row); for one K-step of 16,
// core (row group rg, K half kh) sits at rg * 256 + kh * 128: LBO = 128, SBO = 256.
struct UmSmem {
  uint8_t adig[UM_BUF][oz::NS][2][UM_M * 32];  // state digits: buffer, digit, K-step (4 KB each)
  uint8_t bdig[oz::NS][2][UM_N * 32];          // gate digits: digit, K-step (1 KB each)
  double2 stage[UM_BUF][16][UM_M];             // fetched amplitudes: buffer, amplitude, group
  uint32_t key[UM_BUF][4][UM_M];               // largest exponent key of each quarter group
  double2 U16[256];                            // fused unitary, U16[o * 16 + i]
  int32_t erow[16];                            // largest exponent of row o of U16
  uint32_t krow[16];                           // oz::scale_bits(erow[o])
  uint64_t keyx[UM_BUF];                       // all quarters' keys (and fetched amplitudes) are visible
  uint64_t full[UM_BUF];                       // digits of the buffer's tile are ready
  uint64_t done[UM_BUF];                       // MMAs of the buffer's tile are complete
  uint32_t tmem_base;
  int gate_ok;
  int abort;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Warp-uniform bounded wait for the phase of parity `parity`; false on expiry or abort.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const long long t0 = clock64();
  while (true) {
    const bool ok = mbar_try_wait(bar, parity);
    if (__all_sync(0xffffffffu, ok)) return true;
    if (__any_sync(0xffffffffu, *abort != 0 || clock64() - t0 > UM_WAIT_CYCLES)) return false;
  }
}

// Bounded wait that ignores the abort flag (draining MMAs in flight before teardown).
__device__ __forceinline__ bool mbar_wait_drain(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    const bool ok = mbar_try_wait(bar, parity);
    if (__all_sync(0xffffffffu, ok)) return true;
    if (__any_sync(0xffffffffu, clock64() - t0 > UM_WAIT_CYCLES)) return false;
  }
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, no swizzle, LBO 128 B (K direction), SBO
// 256 B (8-row groups), descriptor version 1 (bits 46-47).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(256u >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor, kind::f16: D F32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12
// = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t UM_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(UM_N >> 3) << 17) |
                              ((uint32_t)(UM_M >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(UM_IDESC), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 2 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, uint32_t (&v)[2]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=r"(v[0]), "=r"(v[1]) : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// FP64 outputs 4 v .. 4 v + 3 of one group whose 16 amplitudes are in the stage (stride
// UM_M); the four quarters' inputs are all read before any thread of the group writes.
template <typename IT>
__device__ __noinline__ void quarter_group_fp64(double2* __restrict__ psi, IT gbase, const PairParams& p,
                                                const double2* U16, const double2* stage_r, int v) {
  double2 x[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) x[c] = stage_r[c * UM_M];
#pragma unroll 1
  for (int o = 4 * v; o < 4 * v + 4; ++o) psi[gbase + (IT)p.off[o]] = group_output_fp64(U16, x, o);
}

template <typename IT>
__global__ void __launch_bounds__(UM_THREADS, 1) gate_pair_umma_kernel(double2* __restrict__ psi,
                                                                       const double2* __restrict__ ga,
                                                                       const double2* __restrict__ gb,
                                                                       const __grid_constant__ PairParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  UmSmem& sm = *reinterpret_cast<UmSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t ntiles = p.ngroups / UM_M;

  // ---- setup: barriers, tensor memory, the fused gate and its digits ----
  if (tid == 0) {
    sm.gate_ok = 1;
    sm.abort = 0;
    for (int b = 0; b < UM_BUF; ++b) {
      mbar_init(&sm.keyx[b], UM_CONV);
      mbar_init(&sm.full[b], UM_CONV);
      mbar_init(&sm.done[b], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == UM_WARPS) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(UM_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int t = tid; t < 256; t += UM_THREADS) sm.U16[t] = fused_entry(ga, gb, t);
  __syncthreads();
  if (tid < 16) {
    bool ok;
    const uint32_t e = row_exponent(sm.U16, tid, ok);
    sm.erow[tid] = (int32_t)e;
    sm.krow[tid] = oz::scale_bits((int32_t)e);
    if (!ok) sm.gate_ok = 0;
  }
  __syncthreads();
  if (tid < 128) {  // gate digits: output row o, K core kc (input reals 8 kc .. 8 kc + 7)
    const int o = tid >> 2, kc = tid & 3;
    const uint32_t E = oz::digit_scale((uint32_t)sm.erow[o & 15]);
    float d[8][oz::NS];
#pragma unroll
    for (int e = 0; e < 8; ++e) oz::digits(df::words(real_form(sm.U16, o, kc * 8 + e)), E, d[e]);
#pragma unroll
    for (int j = 0; j < oz::NS; ++j) {
      const uint4 v = make_uint4(oz::pack(d[0][j], d[1][j]), oz::pack(d[2][j], d[3][j]), oz::pack(d[4][j], d[5][j]),
                                 oz::pack(d[6][j], d[7][j]));
      *reinterpret_cast<uint4*>(&sm.bdig[j][kc >> 1][(o >> 3) * 256 + (kc & 1) * 128 + (o & 7) * 16]) = v;
    }
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  const bool gok = sm.gate_ok != 0;
  auto tile_of = [&](uint64_t m) -> uint64_t { return (uint64_t)blockIdx.x + m * gridDim.x; };

  if (warp < UM_WARPS) {
    // ---- converting warps: digits of tile m, recombination of tile m - 1 ----
    const int q = warp & 3, v = warp >> 2;
    const int r = q * 32 + lane;  // group row of the tile (TMEM lane; warp w reads lanes 32 (w % 4) ..)
    // this thread's 8-byte slot of a digit row: K core (v >> 1) of the real (K-step 0) or
    // imaginary (K-step 1) parts, elements 4 (v & 1) .. 4 (v & 1) + 3
    const uint32_t dig_off = (uint32_t)((r >> 3) * 256 + (v >> 1) * 128 + (r & 7) * 16 + (v & 1) * 8);
    IT off[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) off[a] = (IT)p.off[4 * v + a];
    auto fetch = [&](uint64_t m) {
      const uint64_t T = tile_of(m);
      if (T < ntiles) {
        const IT gbase = pair_base<IT>((IT)(T * UM_M + r), p);
        const int b = (int)(m & 1);
#pragma unroll
        for (int a = 0; a < 4; ++a) cp_async16(&sm.stage[b][4 * v + a][r], psi + (gbase + off[a]));
      }
      cp_async_commit();
    };
    // level sums of tile m from TMEM buffer m & 1 -> FP64 outputs (skipped for groups that
    // took the FP64 path)
    auto finish = [&](uint64_t m, IT gbase, uint32_t emax, bool ok) -> bool {
      const int b = (int)(m & 1);
      if (!mbar_wait_warp(&sm.done[b], (uint32_t)(m >> 1) & 1u, &sm.abort)) {
        atomicOr(&g_umma_error, 2u);
        sm.abort = 1;
        return false;
      }
      tc_fence_after();
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * UM_COLS) + (uint32_t)(4 * v);
#pragma unroll
      for (int a0 = 0; a0 < 4; a0 += 2) {  // two amplitudes at a time (24 registers of level sums)
        uint32_t re[oz::NL][2], im[oz::NL][2];
#pragma unroll
        for (int l = 0; l < oz::NL; ++l) {
          tmem_ld2(tbase + (uint32_t)(32 * l + a0), re[l]);
          tmem_ld2(tbase + (uint32_t)(32 * l + 16 + a0), im[l]);
        }
        tmem_wait_ld();
        if (ok) {
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            const uint32_t K20 = (emax << 20) + sm.krow[4 * v + a0 + a];
            float lr[oz::NL], li[oz::NL];
#pragma unroll
            for (int l = 0; l < oz::NL; ++l) lr[l] = __uint_as_float(re[l][a]), li[l] = __uint_as_float(im[l][a]);
            psi[gbase + off[a0 + a]] = make_double2(oz::combine(lr, K20), oz::combine(li, K20));
          }
        }
      }
      tc_fence_before();  // the buffer may be overwritten after this thread's next arrival on full
      return true;
    };
    fetch(0);
    fetch(1);
    IT pgbase = 0;  // tile m - 1: group base, exponent, digit path
    uint32_t pemax = 0;
    bool pok = false, alive = true;
    uint64_t m = 0;
    for (; tile_of(m) < ntiles; ++m) {
      const int b = (int)(m & 1);
      const uint32_t ph = (uint32_t)(m >> 1) & 1u;
      const IT gbase = pair_base<IT>((IT)(tile_of(m) * UM_M + r), p);
      cp_async_wait_one();  // tile m landed (tile m + 1 may still be in flight)
      double2 x[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) x[a] = sm.stage[b][4 * v + a][r];
      uint32_t key = 0;
#pragma unroll
      for (int a = 0; a < 4; ++a)
        key = max(key, max(oz::group_key(df::words(x[a].x)), oz::group_key(df::words(x[a].y))));
      sm.key[b][v][r] = key;
      mbar_arrive(&sm.keyx[b]);  // all quarters' keys and fetched amplitudes become visible
      if (!mbar_wait_warp(&sm.keyx[b], ph, &sm.abort)) {
        atomicOr(&g_umma_error, 4u);
        sm.abort = 1;
        alive = false;
        break;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) key = max(key, sm.key[b][u][r]);
      const uint32_t emax = oz::key_exponent(key), escale = oz::digit_scale(emax);
      const bool ok = gok && tc_scale_ok(emax);
      uint8_t* dig = &sm.adig[b][0][0][0] + dig_off;
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        float d[4][oz::NS];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          if (ok) {
            oz::digits(df::words(part ? x[a].y : x[a].x), escale, d[a]);
          } else {
#pragma unroll
            for (int j = 0; j < oz::NS; ++j) d[a][j] = 0.0f;
          }
        }
#pragma unroll
        for (int j = 0; j < oz::NS; ++j)
          *reinterpret_cast<uint2*>(dig + (j * 2 + part) * (UM_M * 32)) =
              make_uint2(oz::pack(d[0][j], d[1][j]), oz::pack(d[2][j], d[3][j]));
      }
      if (!ok) quarter_group_fp64<IT>(psi, gbase, p, sm.U16, &sm.stage[b][0][r], v);
      fence_proxy_async();
      mbar_arrive(&sm.full[b]);
      if (m > 0 && !finish(m - 1, pgbase, pemax, pok)) {
        alive = false;
        break;
      }
      // every converting thread has passed the digits (and FP64 path) of tile m: its
      // stage buffer is free for tile m + 2
      if (!mbar_wait_warp(&sm.full[b], ph, &sm.abort)) {
        atomicOr(&g_umma_error, 1u);
        sm.abort = 1;
        alive = false;
        break;
      }
      fetch(m + 2);
      pgbase = gbase;
      pemax = emax;
      pok = ok;
    }
    if (alive && m > 0) finish(m - 1, pgbase, pemax, pok);
    cp_async_wait_all();
  } else {
    // ---- MMA warp: one elected thread issues each tile's 42 MMAs ----
    const uint32_t bbase = smem_u32(&sm.bdig[0][0][0]);
    uint64_t issued = 0;
    for (uint64_t m = 0; tile_of(m) < ntiles; ++m) {
      const int b = (int)(m & 1);
      if (!mbar_wait_warp(&sm.full[b], (uint32_t)(m >> 1) & 1u, &sm.abort)) {
        atomicOr(&g_umma_error, 1u);
        sm.abort = 1;
        break;
      }
      tc_fence_after();
      if (lane == 0) {
        const uint32_t abase = smem_u32(&sm.adig[b][0][0][0]);
        const uint32_t dcol = tmem + (uint32_t)(b * UM_COLS);
#pragma unroll
        for (int l = 0; l < oz::NL; ++l) {
          uint32_t acc = 0;
#pragma unroll
          for (int i = 0; i < oz::NS; ++i) {
            const int j = l - i;
            if (j < 0 || j >= oz::NS) continue;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
              const uint64_t ad = smem_desc(abase + (uint32_t)((j * 2 + ks) * UM_M * 32));
              const uint64_t bd = smem_desc(bbase + (uint32_t)((i * 2 + ks) * UM_N * 32));
              umma_bf16(dcol + (uint32_t)(l * UM_N), ad, bd, acc);
              acc = 1;
            }
          }
        }
        umma_commit(&sm.done[b]);
      }
      __syncwarp();
      ++issued;
    }
    // after an abort, the last tile's MMAs may still be running: let them finish (their
    // commit arrives on done) before the tensor memory is freed
    if (issued && !mbar_wait_drain(&sm.done[(issued - 1) & 1], (uint32_t)((issued - 1) >> 1) & 1u))
      atomicOr(&g_umma_error, 2u);
  }

  // ---- teardown: all tensor-memory reads are done; free it ----
  tc_fence_before();
  __syncthreads();
  if (warp == UM_WARPS) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UM_TMEM_COLS) : "memory");
  }
}

template <typename IT>
void launch_umma(double2* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s) {
  const size_t smem = sizeof(UmSmem);
  check_cuda(cudaFuncSetAttribute(gate_pair_umma_kernel<IT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
             "gate_pair_umma_kernel shared memory");
  const uint64_t ntiles = p.ngroups / UM_M;
  const int grid = (int)std::min<uint64_t>(ntiles, (uint64_t)sm_count());
  gate_pair_umma_kernel<IT><<<grid, UM_THREADS, smem, s>>>(psi, ga, gb, p);
}

}  // namespace

bool launch_pair_umma(double2* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s) {
  if (p.ngroups < (uint64_t)UM_M || p.ngroups % UM_M) return false;
  if (p.ngroups * 16 <= (1ull << 32))
    launch_umma<uint32_t>(psi, ga, gb, p, s);
  else
    launch_umma<uint64_t>(psi, ga, gb, p, s);
  return true;
}

uint32_t take_umma_error() {
  uint32_t v = 0;
  check_cuda(cudaMemcpyFromSymbol(&v, g_umma_error, sizeof(v)), "read device error flags");
  const uint32_t zero = 0;
  check_cuda(cudaMemcpyToSymbol(g_umma_error, &zero, sizeof(zero)), "clear device error flags");
  return v;
}

}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" int qtnh_take_device_errors(uint32_t* flags) {
  return guarded([&]() -> int {
    if (!flags) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null flags pointer");
    check_cuda(cudaDeviceSynchronize(), "device synchronize");
    *flags = take_umma_error() | (take_gemm_error() << 8);
    return QTNH_OK;
  });
}
