// Fused gate pairs on the 5th-generation tensor cores (tcgen05): the same error-free bf16
// digit scheme as gate_tc.cu, with the MMA issued by one thread into tensor memory.
//
// A tile is 128 groups (16 amplitudes each). Per tile, D_l[g][o] = sum over digit pairs
// (i, j), i + j = l, of X_j[g][k] * R_i[o][k] (M = 128 groups, N = 32 output reals, K = 32
// input reals), the 21 digit pairs i + j <= 5, into six level column blocks of TMEM. The
// gate digits of one K-step lie stacked along N (digit i at rows 32 i ..), so state digit
// j meets gate digits 0 .. 5 - j in one tcgen05.mma (kind::f16, bf16 operands, FP32
// accumulators) of N = 32 (6 - j) into columns 32 j ..: 6 digits x 2 K-steps = 12 MMAs.
//
// First pass (gate_pair_umma_kernel, below; a later pass of a fixed-point chain has its
// own pipelined kernel, gate_pair_chain_kernel, further down).
// CTA = a team of eight warps + one MMA warp; two CTAs per SM (persistent; each holds half
// of the SM's tensor memory and ~97 KB of shared memory):
//   * the team handles every tile of its CTA; group r of a tile belongs to two threads
//     (warp quarter q = r / 32 of the team's first and second four warps), each
//     owning 8 of the group's 16 amplitudes: it fetches them one tile ahead with
//     cp.async, the two exchange their largest exponents through shared memory (an
//     mbarrier of the two warps of quarter q), and each writes its 6 x 16 digits into shared memory in the UMMA
//     K-major core-matrix layout (8 rows x 16 bytes) and arrives on full;
//   * the MMA warp waits on full, issues the 12 MMAs into the CTA's TMEM columns and
//     commits them to done;
//   * the team waits on done, and each thread reads the level sums of its 8 amplitudes
//     from its TMEM lane with tcgen05.ld, recombines and stores them.
// While one CTA's team waits for its MMAs, the other CTA on the SM converts (one CTA
// with two teams, or 16 warps issuing their own MMAs, measured slower). Every wait is
// bounded by a clock limit; on expiry the CTA records an error flag, stops and frees its
// tensor memory.
//
// Groups with an infinity/NaN or a largest magnitude outside 2^-200..2^201, and all
// groups when the gate has such entries, are computed in FP64 by their two threads.

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include <cuda_fp16.h>

#include "gate_pair.cuh"

namespace qtnh_impl {

// bit 0: a wait for digits expired, bit 1: a wait for MMA completion expired, bit 2: a
// wait for the partner half's exponent expired
__device__ unsigned int g_umma_error;
// Test hook (qtnh_debug_expire_exchange_wait): nonzero makes the pair kernel's first
// exponent exchange wait on a barrier that nothing completes, with a short limit.
__device__ int g_umma_test_expire;

namespace {

constexpr int UM_WG = 1;                 // teams per CTA, one tile in flight each
constexpr int UM_TEAM = 256;             // threads of a team (two per group)
constexpr int UM_THREADS = UM_WG * UM_TEAM + 32;
constexpr int UM_M = 128;                // groups per tile (MMA M)
constexpr int UM_N = 32;                 // output reals per group (MMA N)
constexpr int UM_COLS = 256;             // TMEM column stride of a team (its level sums use 32 * NL)
constexpr uint32_t UM_TMEM_COLS = 256;   // allocation (power of two >= UM_WG * UM_COLS): half of an SM's TMEM
static_assert(oz::NL * UM_N <= UM_COLS, "level sums exceed a team's TMEM columns");
constexpr long long UM_WAIT_CYCLES = 1ll << 31;  // ~1 s at 2 GHz
constexpr long long UM_TEST_WAIT_CYCLES = 1ll << 20;  // the test hook's wait: ~0.5 ms

// Shared memory of one CTA (dynamic). Operand layout (K-major, no swizzle): an 8-row x
// 16-byte core matrix is 128 contiguous bytes (row at 16 * row); for one K-step of 16,
// core (row group rg, K half kh) sits at rg * 256 + kh * 128: LBO = 128, SBO = 256.
struct UmSmem {
  uint8_t adig[UM_WG][oz::NS][2][UM_M * 32];  // state digits: team, digit, K-step (4 KB each)
  uint8_t bdig[2][oz::NS][UM_N * 32];         // gate digits: K-step, digit (1 KB each; digits stack along N)
  double2 stage[UM_WG][16][UM_M];             // fetched amplitudes: team, amplitude, group
  uint32_t key[UM_WG][2][UM_M];               // largest exponent key of each half group
  double2 U16[256];                           // fused unitary, U16[o * 16 + i]
  int32_t erow[16];                           // largest exponent of row o of U16
  uint32_t krow[16];                          // oz::scale_bits(erow[o])
  uint64_t keyx[UM_WG][4];                    // per row quarter: both halves' keys (and amplitudes) are visible
  uint64_t never;                             // test hook: a barrier no thread arrives on
  int test_expire;
  uint64_t full[UM_WG];                       // digits of team t's tile are ready
  uint64_t done[UM_WG];                       // MMAs of team t's tile are complete
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
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, volatile int* abort,
                                               long long limit = UM_WAIT_CYCLES) {
  const long long t0 = clock64();
  while (true) {
    const bool ok = mbar_try_wait(bar, parity);
    if (__all_sync(0xffffffffu, ok)) return true;
    if (__any_sync(0xffffffffu, *abort != 0 || clock64() - t0 > limit)) return false;
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
__host__ __device__ constexpr uint32_t um_idesc(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((uint32_t)(UM_M >> 4) << 24);
}
static_assert(oz::NS == oz::NL, "state digit j meets gate digits 0 .. NL - 1 - j");
static_assert(UM_N * oz::NL <= 256, "an MMA's N is at most 256");

__device__ __forceinline__ void umma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 4 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&v)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
               : "r"(taddr));
}
// 8 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Largest group key (oz::group_key) of an amplitude's two parts.
__device__ __forceinline__ uint32_t amp_key(double2 v) {
  return max(oz::group_key(df::words(v.x)), oz::group_key(df::words(v.y)));
}

// FP64 outputs 8 h .. 8 h + 7 of one group whose 16 amplitudes are in the stage
// (stride UM_M); the two halves' inputs are all read before either thread writes. Returns
// the largest key of the outputs.
template <typename IT>
__device__ __noinline__ uint32_t half_group_fp64(double2* __restrict__ psi, IT gbase, const PairParams& p,
                                                 const double2* U16, const double2* stage_r, int h) {
  double2 x[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) x[c] = stage_r[c * UM_M];
  uint32_t key = 0;
#pragma unroll 1
  for (int o = 8 * h; o < 8 * h + 8; ++o) {
    const double2 v = group_output_fp64(U16, x, o);
    key = max(key, amp_key(v));
    psi[gbase + (IT)p.off[o]] = v;
  }
  return key;
}

// RECORD: rec receives the largest group key of the outputs and the smallest exponent of a
// nonzero half group's largest output (atomicMax), for the next pass of a fixed-point chain.
template <typename IT, uint32_t MODE, bool RECORD>
__global__ void __launch_bounds__(UM_THREADS, 2) gate_pair_umma_kernel(double2* __restrict__ psi,
                                                                       const double2* __restrict__ ga,
                                                                       const double2* __restrict__ gb,
                                                                       const __grid_constant__ PairParams p,
                                                                       ChainRec* __restrict__ rec) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  UmSmem& sm = *reinterpret_cast<UmSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t ntiles = p.ngroups / UM_M;

  // ---- setup: barriers, tensor memory, the fused gate and its digits ----
  if (tid == 0) {
    sm.gate_ok = 1;
    sm.abort = 0;
    sm.test_expire = *(volatile int*)&g_umma_test_expire;
    for (int w = 0; w < UM_WG; ++w) {
      for (int qq = 0; qq < 4; ++qq) mbar_init(&sm.keyx[w][qq], 64);  // the quarter's two warps
      mbar_init(&sm.full[w], UM_TEAM);
      mbar_init(&sm.done[w], 1);
    }
    mbar_init(&sm.never, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == UM_WG * 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(UM_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int t = tid; t < 256; t += UM_THREADS) sm.U16[t] = fused_entry<MODE>(ga, gb, t);
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
      *reinterpret_cast<uint4*>(&sm.bdig[kc >> 1][j][(o >> 3) * 256 + (kc & 1) * 128 + (o & 7) * 16]) = v;
    }
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  const bool gok = sm.gate_ok != 0;
  auto tile_of = [&](uint64_t m) -> uint64_t { return (uint64_t)blockIdx.x + m * gridDim.x; };

  if (warp < UM_WG * 8) {
    // ---- team: fetch, digits, (MMA), recombination, store ----
    const int t = warp >> 3, v = warp & 7, q = v & 3, h = v >> 2;
    const int r = q * 32 + lane;  // group row of the tile (TMEM lane)
    const uint32_t row_off = (uint32_t)((r >> 3) * 256 + (r & 7) * 16);
    auto fetch = [&](uint64_t T) {
      if (T < ntiles) {
        const IT gbase = pair_base<IT>((IT)(T * UM_M + r), p);
#pragma unroll
        for (int c = 8 * h; c < 8 * h + 8; ++c) cp_async16(&sm.stage[t][c][r], psi + (gbase + (IT)p.off[c]));
      }
      cp_async_commit();
    };
    fetch(tile_of(t));
    uint32_t it = 0, okey = 0, ominc = 0;
    for (uint64_t m = t; tile_of(m) < ntiles; m += UM_WG, ++it) {
      const IT gbase = pair_base<IT>((IT)(tile_of(m) * UM_M + r), p);
      cp_async_wait_all();
      double2 x[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) x[c] = sm.stage[t][8 * h + c][r];
      uint32_t key = 0;
#pragma unroll
      for (int c = 0; c < 8; ++c) key = max(key, max(oz::group_key(df::words(x[c].x)), oz::group_key(df::words(x[c].y))));
      sm.key[t][h][r] = key;
      mbar_arrive(&sm.keyx[t][q]);  // both halves' keys and fetched amplitudes become visible
      // (test hook: the first exchange waits on a barrier nothing completes; no MMA, tensor
      // memory load or bulk copy of this CTA is in flight yet)
      const bool expire = sm.test_expire != 0 && it == 0;
      if (!mbar_wait_warp(expire ? &sm.never : &sm.keyx[t][q], expire ? 0u : (it & 1u), &sm.abort,
                          expire ? UM_TEST_WAIT_CYCLES : UM_WAIT_CYCLES)) {
        atomicOr(&g_umma_error, 4u);
        sm.abort = 1;
        break;
      }
      key = max(key, sm.key[t][h ^ 1][r]);
      const uint32_t emax = oz::key_exponent(key), escale = oz::digit_scale(emax);
      const bool ok = gok && tc_scale_ok(emax);
      // this thread's stage slots are read again only by the other half of its row, and
      // only when that row takes the FP64 path: a warp whose rows all take the tensor path
      // refills its slots with the next tile now, the others after the whole team arrived
      const bool early = __all_sync(0xffffffffu, ok);
      if (early) fetch(tile_of(m + UM_WG));
      // digits of this thread's 16 reals: K core h (real parts of amplitudes 8h..8h+7)
      // and K core 2 + h (their imaginary parts)
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        const int kc = 2 * part + h;
        float d[8][oz::NS];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          if (ok) {
            oz::digits(df::words(part ? x[e].y : x[e].x), escale, d[e]);
          } else {
#pragma unroll
            for (int j = 0; j < oz::NS; ++j) d[e][j] = 0.0f;
          }
        }
#pragma unroll
        for (int j = 0; j < oz::NS; ++j) {
          const uint4 vv = make_uint4(oz::pack(d[0][j], d[1][j]), oz::pack(d[2][j], d[3][j]),
                                      oz::pack(d[4][j], d[5][j]), oz::pack(d[6][j], d[7][j]));
          *reinterpret_cast<uint4*>(&sm.adig[t][j][kc >> 1][row_off + (kc & 1) * 128]) = vv;
        }
      }
      if (!ok) {
        const uint32_t k = half_group_fp64<IT>(psi, gbase, p, sm.U16, &sm.stage[t][0][r], h);
        if (RECORD) {
          okey = max(okey, k);
          if (k) ominc = max(ominc, 2047u - oz::key_exponent(k));
        }
      }
      fence_proxy_async();
      mbar_arrive(&sm.full[t]);
      if (!early) {
        // every thread of the team has arrived: the FP64 path of the rows is done with the stage
        if (!mbar_wait_warp(&sm.full[t], it & 1u, &sm.abort)) {
          atomicOr(&g_umma_error, 2u);
          sm.abort = 1;
          break;
        }
        fetch(tile_of(m + UM_WG));
      }
      if (!mbar_wait_warp(&sm.done[t], it & 1u, &sm.abort)) {
        atomicOr(&g_umma_error, 2u);
        sm.abort = 1;
        break;
      }
      tc_fence_after();
      // level sums: TMEM lane r, columns t * UM_COLS + 32 l + o (o < 16: real part of
      // amplitude o, o >= 16: imaginary part of amplitude o - 16)
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(t * UM_COLS);
      uint32_t hkey = 0;  // largest key of this half group's outputs
#pragma unroll
      for (int c4 = 0; c4 < 2; ++c4) {
        const int a0 = 8 * h + 4 * c4;
        uint32_t re[oz::NL][4], im[oz::NL][4];
#pragma unroll
        for (int l = 0; l < oz::NL; ++l) {
          tmem_ld4(tbase + (uint32_t)(32 * l + a0), re[l]);
          tmem_ld4(tbase + (uint32_t)(32 * l + 16 + a0), im[l]);
        }
        tmem_wait_ld();
        if (ok) {
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const uint32_t K20 = (emax << 20) + sm.krow[a0 + a];
            float lr[oz::NL], li[oz::NL];
#pragma unroll
            for (int l = 0; l < oz::NL; ++l) lr[l] = __uint_as_float(re[l][a]), li[l] = __uint_as_float(im[l][a]);
            const double2 v = make_double2(oz::combine(lr, K20), oz::combine(li, K20));
            if (RECORD) hkey = max(hkey, amp_key(v));
            psi[gbase + (IT)p.off[a0 + a]] = v;
          }
        }
      }
      if (RECORD && ok) {
        okey = max(okey, hkey);
        if (hkey) ominc = max(ominc, 2047u - oz::key_exponent(hkey));
      }
      tc_fence_before();
    }
    cp_async_wait_all();
    if (RECORD) {
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        okey = max(okey, __shfl_xor_sync(0xffffffffu, okey, o));
        ominc = max(ominc, __shfl_xor_sync(0xffffffffu, ominc, o));
      }
      if (lane == 0) {
        if (okey) atomicMax(&rec->maxkey, okey);
        if (ominc) atomicMax(&rec->minc, ominc);
      }
    }
  } else {
    // ---- MMA warp: one elected thread issues each tile's 12 MMAs ----
    const uint32_t bbase = smem_u32(&sm.bdig[0][0][0]);
    for (uint64_t m = 0; tile_of(m) < ntiles; ++m) {
      const int w = (int)(m % UM_WG);
      const uint32_t it = (uint32_t)(m / UM_WG);
      if (!mbar_wait_warp(&sm.full[w], it & 1u, &sm.abort)) {
        atomicOr(&g_umma_error, 1u);
        sm.abort = 1;
        break;
      }
      tc_fence_after();
      if (lane == 0) {
        const uint32_t abase = smem_u32(&sm.adig[w][0][0][0]);
        const uint32_t dcol = tmem + (uint32_t)(w * UM_COLS);
        // state digit j x gate digits 0 .. NL-1-j (stacked along N) -> levels j .. NL-1;
        // the first MMA (j = 0, all six levels) overwrites, the rest accumulate
#pragma unroll
        for (int j = 0; j < oz::NS; ++j) {
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const uint64_t ad = smem_desc(abase + (uint32_t)((j * 2 + ks) * UM_M * 32));
            const uint64_t bd = smem_desc(bbase + (uint32_t)(ks * oz::NS * UM_N * 32));
            umma_f16(dcol + (uint32_t)(j * UM_N), ad, bd, um_idesc((uint32_t)(UM_N * (oz::NL - j))),
                      (j | ks) != 0 ? 1u : 0u);
          }
        }
        umma_commit(&sm.done[w]);
      }
      __syncwarp();
    }
  }

  // ---- teardown: all tensor-memory reads are done; free it ----
  tc_fence_before();
  __syncthreads();
  if (warp == UM_WG * 8) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UM_TMEM_COLS) : "memory");
  }
}

// ---- a later pass of a gate layer's chain --------------------------------------------

// State digits of the chain passes: six (48 bits of the state's largest magnitude; seven
// measured 14 % slower per pass). Levels kept: 7 (level 6 = the five digit pairs i + j = 6
// of the six-by-six product, about 2.5x less error on long chains) or 6
// (QTNH_CHAIN_LEVELS=6).
constexpr int CH_ND = oz::NS;
constexpr int CH_NLMAX = 7;
constexpr int CH_WARPS = 16;                // team warps: four per TMEM lane quarter
constexpr int CH_TEAM = CH_WARPS * 32;      // two tiles in flight: digits of one, MMAs of the other
constexpr int CH_THREADS = CH_TEAM + 32;    // + the MMA warp
constexpr uint32_t CH_ACC = 256;            // TMEM columns of one accumulator set
constexpr uint32_t CH_TMEM_COLS = 512;      // two accumulator sets: all of an SM's TMEM

// The chain's digits are fp16 (both operands, kind::f16; balanced digits, |d| <= 128, are
// exact in fp16 as in bf16, and fp16 lets byte permutes build them): instruction
// descriptor with A and B formats F16.
__host__ __device__ constexpr uint32_t ch_idesc(uint32_t n) {
  return (1u << 4) | ((n >> 3) << 17) | ((uint32_t)(UM_M >> 4) << 24);
}
// Two floats (exact small integers) as an fp16x2 word: lo in the low half.
__device__ __forceinline__ uint32_t pack_h(float lo, float hi) {
  const __half2 v = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}
// Both halves minus 1152: the fp16 words of oz::digit_words_fixed -> balanced digits (exact).
__device__ __forceinline__ uint32_t unbias_h(uint32_t w) {
  const uint32_t c = 0x64806480u;
  const __half2 v = __hsub2(*reinterpret_cast<const __half2*>(&w), *reinterpret_cast<const __half2*>(&c));
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Shared memory of a chain CTA (one per SM): two buffers of state digits (K-major core
// layout as UmSmem), the six gate digits and, for seven levels, a zero seventh block
// stacked along N (it makes the first MMA write every level block), the stage, the
// fused gate.
struct ChSmem {
  uint8_t adig[2][CH_ND][2][UM_M * 32];  // state digits: buffer, digit, K-step (4 KB each)
  uint8_t bdig[2][CH_NLMAX][UM_N * 32];  // gate digits: K-step, digit (1 KB each)
  double2 stage[2][16][UM_M];           // fetched amplitudes (or fixed-point pairs), two tiles ahead
  double2 U16[256];
  int32_t erow[16];
  uint64_t full[2];                     // digits of the tiles using buffer b are ready
  uint64_t done[2];                     // MMAs into accumulator set b are complete
  uint32_t tmem_base;
  int gate_ok;
  int abort;
  int no_abort;                         // stays 0: the final wait for in-flight MMAs
  uint32_t ptab[4][256];                // PO: the permutation's bit tables (BitPerm)
  uint32_t poff[16];                    // PO: the permuted amplitude offsets
};
static_assert(CH_NLMAX * UM_N <= (int)CH_ACC, "chain level sums exceed an accumulator set");
static_assert(2 * CH_ACC <= CH_TMEM_COLS, "two accumulator sets");
static_assert(sizeof(ChSmem) + 1024 <= 227 * 1024, "chain shared memory");
//
// The input is what the previous pass wrote (rin): doubles with the largest group key of
// all of them, or 64-bit fixed point at scale rin->F with the largest |hi word|. Both are
// cut into digits at one scale for the whole state -- no per-group exponent exchange, and
// for fixed point no per-element exponent alignment (oz::digits_fixed). The output is
// fixed point at scale F = 2100 - E - max erow (want_fixed) or doubles; rout records it.
// When the input is doubles whose largest magnitude lies outside 2^-200..2^201 or the gate
// has entries the digits cannot carry (then gate_ok is 0), every group is computed in FP64
// (from the converted fixed-point input where that is the input) and doubles are written.
//
// Pipeline (persistent, one CTA per SM): group r of a tile belongs to four threads (warps
// q, q + 4, q + 8, q + 12 of the lane quarter q = r / 32), each owning 4 of its 16
// amplitudes. In iteration m the team writes the digits of tile m into digit buffer m % 2
// and arrives on full[m % 2]; then it waits for the MMAs of tile m - 1 (accumulator set
// (m - 1) % 2) and recombines and stores that tile. The MMA warp issues tile m's MMAs into
// accumulator set m % 2 as soon as its digits are complete, so the tensor cores work on
// tile m while the team recombines tile m - 1: the team never waits for its own MMAs
// unless they take longer than a digit phase. Buffer reuse: digits of tile m overwrite
// buffer m % 2 after the team waited (in iteration m - 1) for the MMAs of tile m - 2 that
// read it; the MMAs of tile m overwrite set m % 2 after every thread arrived on full for
// tile m, i.e. after its reads of tile m - 2's sums (tcgen05.fence before the arrive).
//
// PO (permuted output, IT = uint32_t): the outputs go out of place to outv, element x to
// index P(x) of the permutation `perm` (bit tables in shared memory; P(tile part | row
// part | offset) is the OR of the three parts' images, the row part's and the offsets'
// computed once), so the pass and the permutation after it take one pass over the state.
template <typename IT, uint32_t MODE, int NL, bool PO>
__global__ void __launch_bounds__(CH_THREADS, 1) gate_pair_chain_kernel(void* __restrict__ psiv,
                                                                        const double2* __restrict__ ga,
                                                                        const double2* __restrict__ gb,
                                                                        const __grid_constant__ PairParams p,
                                                                        const ChainRec* __restrict__ rin,
                                                                        ChainRec* __restrict__ rout, int want_fixed,
                                                                        void* __restrict__ outv,
                                                                        const BitPerm* __restrict__ perm) {
  static_assert(!PO || sizeof(IT) == 4, "permuted output for states of at most 2^32 elements");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  ChSmem& sm = *reinterpret_cast<ChSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t ntiles = p.ngroups / UM_M;
  const double2* psi = static_cast<const double2*>(psiv);
  const int64_t* psy = static_cast<const int64_t*>(psiv);
  double2* pso = static_cast<double2*>(PO ? outv : psiv);  // where the outputs go
  int64_t* pyo = static_cast<int64_t*>(PO ? outv : psiv);
  if (PO) {
    for (int t = tid; t < 4 * 256; t += CH_THREADS) (&sm.ptab[0][0])[t] = (&perm->tab[0][0])[t];
    if (tid < 16) sm.poff[tid] = perm->poff[tid];
  }
  // the image of a (tile or row) part of an element index under the permutation
  auto pimg = [&](uint32_t x) -> uint32_t {
    return sm.ptab[0][x & 255u] | sm.ptab[1][(x >> 8) & 255u] | sm.ptab[2][(x >> 16) & 255u] | sm.ptab[3][x >> 24];
  };

  // ---- setup as the pair kernel: barriers, tensor memory, the fused gate and its digits ----
  if (tid == 0) {
    sm.gate_ok = 1;
    sm.abort = 0;
    sm.no_abort = 0;
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.full[b], CH_TEAM);
      mbar_init(&sm.done[b], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == CH_WARPS) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(CH_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int t = tid; t < 256; t += CH_THREADS) sm.U16[t] = fused_entry<MODE>(ga, gb, t);
  __syncthreads();
  if (tid < 16) {
    bool ok;
    const uint32_t e = row_exponent(sm.U16, tid, ok);
    sm.erow[tid] = (int32_t)e;
    if (!ok) sm.gate_ok = 0;
  }
  __syncthreads();
  int max_erow = 0, min_erow = 0x7FFFFFFF;
#pragma unroll
  for (int o = 0; o < 16; ++o) max_erow = max(max_erow, sm.erow[o]), min_erow = min(min_erow, sm.erow[o]);
  const bool common = max_erow - min_erow <= oz::CHAIN_COMMON_SPAN;  // one digit scale for all rows
  if (tid < 128) {
    // B row n = output real (amplitude n / 2, real or imaginary part n % 2), K column k = input
    // real (amplitude k / 2, part k % 2): real and imaginary parts interleaved, so that the
    // 8 reals of 4 amplitudes are one core-matrix row (state digits) and 8 adjacent columns
    // (level sums)
    const int o = tid >> 2, kc = tid & 3;
    const int ro = (o & 1) * 16 + (o >> 1);  // the row of the real form R
    const uint32_t E = oz::digit_scale((uint32_t)(common ? max_erow : sm.erow[o >> 1]));
    float d[8][oz::NS];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = kc * 8 + e;
      oz::digits(df::words(real_form(sm.U16, ro, (k & 1) * 16 + (k >> 1))), E, d[e]);
    }
#pragma unroll
    for (int j = 0; j < oz::NS; ++j) {
      const uint4 v = make_uint4(pack_h(d[0][j], d[1][j]), pack_h(d[2][j], d[3][j]), pack_h(d[4][j], d[5][j]),
                                 pack_h(d[6][j], d[7][j]));
      *reinterpret_cast<uint4*>(&sm.bdig[kc >> 1][j][(o >> 3) * 256 + (kc & 1) * 128 + (o & 7) * 16]) = v;
    }
    if (NL > oz::NS)  // the seventh gate digit: zero (the first MMA then writes level 6 too)
      *reinterpret_cast<uint4*>(&sm.bdig[kc >> 1][NL - 1][(o >> 3) * 256 + (kc & 1) * 128 + (o & 7) * 16]) =
          make_uint4(0u, 0u, 0u, 0u);
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;

  // ---- the scales (the same in every CTA) ----
  const ChainRec ri = *rin;
  const bool in_fixed = ri.fmt == 1;
  int32_t sh = 0;
  int Ein;
  bool in_ok = true;
  if (in_fixed) {
    sh = oz::fixed_shift(ri.maxhi);
    Ein = oz::fixed_exponent(sh, ri.F);
  } else {
    // doubles: one scale for the whole state, if its largest magnitude is in the digit range
    // and (when recorded) no nonzero half group lies more than 2^CHAIN_RANGE below it
    const uint32_t E = oz::key_exponent(ri.maxkey);
    in_ok = tc_scale_ok(E) && (ri.minc == 0 || (int)E - (2047 - (int)ri.minc) <= CHAIN_RANGE);
    Ein = (int)oz::digit_scale(E);
  }
  if (in_fixed && sh > 15) in_ok = false;  // (not reached: outputs stay below 2^62, sh <= 15)
  const bool uni = in_ok && sm.gate_ok != 0;
  const bool out_fixed = uni && want_fixed != 0;
  const int F_out = 2100 - Ein - max_erow;
  if (blockIdx.x == 0 && tid == 0) {
    rout->fmt = out_fixed ? 1 : 0;
    rout->F = F_out;
  }
  auto tile_of = [&](uint64_t m) -> uint64_t { return (uint64_t)blockIdx.x + m * gridDim.x; };

  if (!uni) {
    // ---- every group in FP64 (no tensor cores): thread per group, doubles out; the output
    // range is recorded like the first pass's, so a later pass starts no chain on it ----
    uint32_t okey = 0, ominc = 0;
    for (uint64_t g = (uint64_t)blockIdx.x * CH_THREADS + tid; g < p.ngroups; g += (uint64_t)gridDim.x * CH_THREADS) {
      const IT gbase = pair_base<IT>((IT)g, p);
      double2 x[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const IT ix = gbase + (IT)p.off[c];
        x[c] = in_fixed ? make_double2(oz::fixed_to_double(psy[2 * (uint64_t)ix], 40 - ri.F),
                                       oz::fixed_to_double(psy[2 * (uint64_t)ix + 1], 40 - ri.F))
                        : psi[ix];
      }
      uint32_t gkey = 0;
      const uint32_t pbase = PO ? pimg((uint32_t)gbase) : 0u;
#pragma unroll 1
      for (int o = 0; o < 16; ++o) {
        const double2 v = group_output_fp64(sm.U16, x, o);
        gkey = max(gkey, amp_key(v));
        if (PO)
          pso[pbase | sm.poff[o]] = v;
        else
          pso[gbase + (IT)p.off[o]] = v;
      }
      okey = max(okey, gkey);
      if (gkey) ominc = max(ominc, 2047u - oz::key_exponent(gkey));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      okey = max(okey, __shfl_xor_sync(0xffffffffu, okey, o));
      ominc = max(ominc, __shfl_xor_sync(0xffffffffu, ominc, o));
    }
    if (lane == 0) {
      if (okey) atomicMax(&rout->maxkey, okey);
      if (ominc) atomicMax(&rout->minc, ominc);
    }
  } else if (warp < CH_WARPS) {
    // ---- team: fetch, digits at the common scale; recombination and store one tile behind ----
    const int q = warp & 3, h = warp >> 2;  // lane quarter; this thread's amplitudes 4h .. 4h + 3
    const int r = q * 32 + lane;            // group row of the tile (TMEM lane)
    // this thread's 8 reals (amplitudes 4h .. 4h + 3, real and imaginary parts interleaved)
    // are row r of K core h: K-step h / 2, core h % 2
    const uint32_t row_off = (uint32_t)((r >> 3) * 256 + (r & 7) * 16 + (h & 1) * 128);
    const uint64_t cadd = oz::fixed_addend(sh);
    // group base of row r of tile T = pair_base(T * 128) | pair_base(r): zero bits are inserted
    // into the tile's bits and the row's bits of the group index independently
    const IT rbase = pair_base<IT>((IT)r, p);
    const uint32_t prbase = PO ? pimg((uint32_t)rbase) : 0u;  // the row part's image
    auto tile_part = [&](uint64_t T) -> IT { return pair_base<IT>((IT)(T * UM_M), p); };
    // per output 4h + a: the row shift to the common output scale (fixed point), 8 bits
    // each, and the row's scale exponent (0 and max_erow when all rows share one scale)
    uint32_t kk = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) kk |= (common ? 0u : (uint32_t)min(62, max_erow - sm.erow[4 * h + a])) << (8 * a);
    // tile T into stage slot `slot` (its iteration % 2; one commit group per tile, empty past the end)
    auto fetch = [&](uint64_t T, IT tb, uint32_t slot) {
      if (T < ntiles) {
        const IT gbase = tb | rbase;
#pragma unroll
        for (int c = 4 * h; c < 4 * h + 4; ++c) cp_async16(&sm.stage[slot][c][r], psi + (gbase + (IT)p.off[c]));
      }
      cp_async_commit();
    };
    uint32_t okey = 0, ohi = 0;
    // level sums from accumulator set b -> the outputs 4h .. 4h + 3 of group r of the tile
    // whose tile part is tb
    auto recombine = [&](IT tb, uint32_t b) {
      const IT gbase = tb | rbase;
      const uint32_t obase = PO ? (pimg((uint32_t)tb) | prbase) : 0u;
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + b * CH_ACC + (uint32_t)(8 * h);
      uint32_t v[NL][8];  // level l, output real 8h + 2a + part
#pragma unroll
      for (int l = 0; l < NL; ++l) tmem_ld8(tbase + (uint32_t)(32 * l), v[l]);
      tmem_wait_ld();
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        float cr[NL], ci[NL];
#pragma unroll
        for (int l = 0; l < NL; ++l) cr[l] = __uint_as_float(v[l][2 * a]), ci[l] = __uint_as_float(v[l][2 * a + 1]);
        int64_t Tr, Ti;
        if constexpr (NL == 7) {
          Tr = oz::fixed_levels_merged(cr), Ti = oz::fixed_levels_merged(ci);
        } else {
          Tr = oz::fixed_levels<NL>(cr), Ti = oz::fixed_levels<NL>(ci);
        }
        const IT ix = PO ? (IT)(obase | sm.poff[4 * h + a]) : gbase + (IT)p.off[4 * h + a];
        if (out_fixed) {
          int64_t Yr = Tr, Yi = Ti;
          if (!common) {
            const uint32_t k = (kk >> (8 * a)) & 0xFFu;
            const int64_t rh = ((int64_t)1 << k) >> 1;  // rounding half (0 for no shift)
            Yr = (Tr + rh) >> k, Yi = (Ti + rh) >> k;
          }
          ohi |= oz::fixed_hi_mag(Yr) | oz::fixed_hi_mag(Yi);  // its bit length is the largest's
          *reinterpret_cast<longlong2*>(pyo + 2 * (uint64_t)ix) = make_longlong2(Yr, Yi);
        } else {
          const int e = (common ? max_erow : sm.erow[4 * h + a]) + Ein - 2060;
          const double2 vv = make_double2(oz::fixed_to_double(Tr, e), oz::fixed_to_double(Ti, e));
          okey = max(okey, amp_key(vv));
          pso[ix] = vv;
        }
      }
    };
    // tile parts of tiles m - 1 .. m + 2; the loads run two tiles ahead
    IT tb_prev = 0, tb_cur = tile_part(tile_of(0)), tb_next = tile_part(tile_of(1));
    fetch(tile_of(0), tb_cur, 0);
    fetch(tile_of(1), tb_next, 1);
    uint64_t m = 0;
    bool ok = true;
    for (; tile_of(m) < ntiles; ++m) {
      const uint32_t b = (uint32_t)(m & 1);
      cp_async_wait_one();  // tile m has landed (tile m + 1 may still be in flight)
      double2 x[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) x[c] = sm.stage[b][4 * h + c][r];
      const IT tb_next2 = tile_part(tile_of(m + 2));
      fetch(tile_of(m + 2), tb_next2, b);  // only this thread reads its stage slots
      // digits of this thread's 8 reals: digit j of amplitude 4h + a as one fp16x2 word (real,
      // imaginary); the four words of digit j fill the thread's core-matrix row
      uint32_t w[4][CH_ND];
      if (in_fixed) {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          oz::digit_words_biased(oz::fixed_biased((int64_t)df::d2u(x[a].x), sh, cadd),
                                 oz::fixed_biased((int64_t)df::d2u(x[a].y), sh, cadd), w[a]);
#pragma unroll
          for (int j = 0; j < CH_ND; ++j) w[a][j] = unbias_h(w[a][j]);
        }
      } else {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          float dr[CH_ND], di[CH_ND];
          oz::digits(df::words(x[a].x), (uint32_t)Ein, dr);
          oz::digits(df::words(x[a].y), (uint32_t)Ein, di);
#pragma unroll
          for (int j = 0; j < CH_ND; ++j) w[a][j] = pack_h(dr[j], di[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < CH_ND; ++j)
        *reinterpret_cast<uint4*>(&sm.adig[b][j][h >> 1][row_off]) = make_uint4(w[0][j], w[1][j], w[2][j], w[3][j]);
      fence_proxy_async();
      tc_fence_before();  // this thread's reads of set b (tile m - 2) precede the MMAs of tile m
      mbar_arrive(&sm.full[b]);
      if (m >= 1) {
        if (!mbar_wait_warp(&sm.done[b ^ 1u], (uint32_t)(((m - 1) >> 1) & 1), &sm.abort)) {
          atomicOr(&g_umma_error, 2u);
          sm.abort = 1;
          ok = false;
          break;
        }
        tc_fence_after();
        recombine(tb_prev, b ^ 1u);
      }
      tb_prev = tb_cur;
      tb_cur = tb_next;
      tb_next = tb_next2;
    }
    if (ok && m >= 1) {  // the last tile
      const uint32_t b = (uint32_t)((m - 1) & 1);
      if (mbar_wait_warp(&sm.done[b], (uint32_t)(((m - 1) >> 1) & 1), &sm.abort)) {
        tc_fence_after();
        recombine(tb_prev, b);
      } else {
        atomicOr(&g_umma_error, 2u);
        sm.abort = 1;
      }
    }
    cp_async_wait_all();
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      okey = max(okey, __shfl_xor_sync(0xffffffffu, okey, o));
      ohi = max(ohi, __shfl_xor_sync(0xffffffffu, ohi, o));
    }
    if (lane == 0) {
      if (okey) atomicMax(&rout->maxkey, okey);
      if (ohi) atomicMax(&rout->maxhi, ohi);
    }
  } else {
    // ---- MMA warp: one elected thread issues each tile's 12 MMAs into set m % 2 ----
    const uint32_t bbase = smem_u32(&sm.bdig[0][0][0]);
    uint64_t issued = 0;
    for (uint64_t m = 0; tile_of(m) < ntiles; ++m) {
      const uint32_t b = (uint32_t)(m & 1);
      if (!mbar_wait_warp(&sm.full[b], (uint32_t)((m >> 1) & 1), &sm.abort)) {
        atomicOr(&g_umma_error, 1u);
        sm.abort = 1;
        break;
      }
      tc_fence_after();
      if (lane == 0) {
        const uint32_t abase = smem_u32(&sm.adig[b][0][0][0]);
        // state digit j x gate digits 0 .. NL - 1 - j (stacked along N) -> levels j .. NL - 1;
        // the first MMA (j = 0, all levels) overwrites, the rest accumulate
#pragma unroll
        for (int j = 0; j < CH_ND; ++j) {
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const uint64_t ad = smem_desc(abase + (uint32_t)((j * 2 + ks) * UM_M * 32));
            const uint64_t bd = smem_desc(bbase + (uint32_t)(ks * CH_NLMAX * UM_N * 32));
            umma_f16(tmem + b * CH_ACC + (uint32_t)(j * UM_N), ad, bd, ch_idesc((uint32_t)(UM_N * (NL - j))),
                      (j | ks) != 0 ? 1u : 0u);
          }
        }
        umma_commit(&sm.done[b]);
      }
      __syncwarp();
      issued = m + 1;
    }
    // the team may have stopped early: let the last issued MMAs finish before tensor memory
    // is freed (no commit on that barrier follows, so its phase parity is stable)
    if (issued) mbar_wait_warp(&sm.done[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1), &sm.no_abort);
  }

  // ---- teardown: all tensor-memory reads are done; free it ----
  tc_fence_before();
  __syncthreads();
  if (warp == CH_WARPS) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(CH_TMEM_COLS) : "memory");
  }
}

template <typename IT, uint32_t MODE>
void launch_umma(double2* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s,
                 ChainRec* rec = nullptr) {
  const size_t smem = sizeof(UmSmem);
  const uint64_t ntiles = p.ngroups / UM_M;
  const int grid = (int)std::min<uint64_t>(ntiles, 2 * (uint64_t)sm_count());  // two CTAs per SM
  if (rec) {
    check_cuda(cudaFuncSetAttribute(gate_pair_umma_kernel<IT, MODE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem),
               "gate_pair_umma_kernel shared memory");
    gate_pair_umma_kernel<IT, MODE, true><<<grid, UM_THREADS, smem, s>>>(psi, ga, gb, p, rec);
  } else {
    check_cuda(cudaFuncSetAttribute(gate_pair_umma_kernel<IT, MODE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem),
               "gate_pair_umma_kernel shared memory");
    gate_pair_umma_kernel<IT, MODE, false><<<grid, UM_THREADS, smem, s>>>(psi, ga, gb, p, nullptr);
  }
}

template <typename IT, int NL, bool PO>
void launch_chain(void* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s,
                  const ChainRec* rin, ChainRec* rout, bool want_fixed, void* out, const BitPerm* perm) {
  const size_t smem = sizeof(ChSmem);
  check_cuda(cudaFuncSetAttribute(gate_pair_chain_kernel<IT, PAIR_KRON, NL, PO>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
             "gate_pair_chain_kernel shared memory");
  const uint64_t ntiles = p.ngroups / UM_M;
  const int grid = (int)std::min<uint64_t>(ntiles, (uint64_t)sm_count());  // one CTA per SM (all its TMEM)
  gate_pair_chain_kernel<IT, PAIR_KRON, NL, PO>
      <<<grid, CH_THREADS, smem, s>>>(psi, ga, gb, p, rin, rout, want_fixed ? 1 : 0, out, perm);
}

int chain_levels() {
  static const int nl = [] {
    const char* e = std::getenv("QTNH_CHAIN_LEVELS");
    return (e && std::strcmp(e, "6") == 0) ? 6 : 7;
  }();
  return nl;
}

}  // namespace

bool chain_applies(const PairParams& p) { return p.ngroups >= (uint64_t)UM_M && p.ngroups % UM_M == 0; }

void launch_pair_chain(void* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s,
                       const ChainRec* rin, ChainRec* rout, bool want_fixed, void* out, const BitPerm* perm) {
  const bool i32 = p.ngroups * 16 <= (1ull << 32);
  if (perm) {
    if (!i32 || !out || out == psi) throw Error(QTNH_ERR_UNSUPPORTED, "permuted chain output");
    // the tables travel in stream-ordered workspace, freed after the launch
    BitPerm* dperm = static_cast<BitPerm*>(workspace_alloc(sizeof(BitPerm), s));
    cudaError_t e = cudaMemcpyAsync(dperm, perm, sizeof(BitPerm), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      if (chain_levels() == 6)
        launch_chain<uint32_t, 6, true>(psi, ga, gb, p, s, rin, rout, want_fixed, out, dperm);
      else
        launch_chain<uint32_t, 7, true>(psi, ga, gb, p, s, rin, rout, want_fixed, out, dperm);
      e = cudaGetLastError();
    }
    workspace_free(dperm, s);
    check_cuda(e, "permuted chain launch");
    return;
  }
  if (chain_levels() == 6) {
    if (i32)
      launch_chain<uint32_t, 6, false>(psi, ga, gb, p, s, rin, rout, want_fixed, nullptr, nullptr);
    else
      launch_chain<uint64_t, 6, false>(psi, ga, gb, p, s, rin, rout, want_fixed, nullptr, nullptr);
  } else {
    if (i32)
      launch_chain<uint32_t, 7, false>(psi, ga, gb, p, s, rin, rout, want_fixed, nullptr, nullptr);
    else
      launch_chain<uint64_t, 7, false>(psi, ga, gb, p, s, rin, rout, want_fixed, nullptr, nullptr);
  }
}

bool make_bit_perm(const dims_t& dims, const std::vector<uint16_t>& ptup, const PairParams& p, BitPerm& bp) {
  const size_t r = dims.size();
  if (ptup.size() != r) return false;
  uint32_t total = 0;
  std::vector<uint32_t> w(r);
  for (size_t i = 0; i < r; ++i) {
    const uint32_t l = log2_or_none(dims[i]);
    if (l == 0xFFFFFFFFu) return false;
    w[i] = l;
    total += l;
  }
  if (total > 32) return false;
  dims_t nd(r);
  for (size_t i = 0; i < r; ++i) nd[ptup[i]] = dims[i];
  // bit position of the lowest bit of axis i in the input, and of position j in the output
  std::vector<uint32_t> in_lo(r), out_lo(r);
  uint32_t acc = 0;
  for (size_t i = r; i-- > 0;) in_lo[i] = acc, acc += w[i];
  acc = 0;
  for (size_t j = r; j-- > 0;) out_lo[j] = acc, acc += log2_or_none(nd[j]);
  uint32_t dst[32];
  for (int b = 0; b < 32; ++b) dst[b] = 32;  // bits above the state: never set
  for (size_t i = 0; i < r; ++i)
    for (uint32_t k = 0; k < w[i]; ++k) dst[in_lo[i] + k] = out_lo[ptup[i]] + k;
  for (int t = 0; t < 4; ++t)
    for (int v = 0; v < 256; ++v) {
      uint32_t x = 0;
      for (int k = 0; k < 8; ++k)
        if (((v >> k) & 1) && dst[8 * t + k] < 32) x |= 1u << dst[8 * t + k];
      bp.tab[t][v] = x;
    }
  for (int c = 0; c < 16; ++c) {
    const uint32_t o = (uint32_t)p.off[c];
    bp.poff[c] = bp.tab[0][o & 255u] | bp.tab[1][(o >> 8) & 255u] | bp.tab[2][(o >> 16) & 255u] | bp.tab[3][o >> 24];
  }
  return true;
}

bool launch_pair_umma(double2* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s,
                      uint32_t mode, ChainRec* rec) {
  if (p.ngroups < (uint64_t)UM_M || p.ngroups % UM_M) return false;
  const bool i32 = p.ngroups * 16 <= (1ull << 32);
  if (mode == PAIR_KRON) {
    if (i32)
      launch_umma<uint32_t, PAIR_KRON>(psi, ga, gb, p, s, rec);
    else
      launch_umma<uint64_t, PAIR_KRON>(psi, ga, gb, p, s, rec);
    return true;
  }
  if (!i32) return false;  // single three- and four-qubit gates: states up to 2^32 amplitudes
  if (mode == PAIR_FULL)
    launch_umma<uint32_t, PAIR_FULL>(psi, ga, gb, p, s);
  else
    launch_umma<uint32_t, PAIR_KRON_I2>(psi, ga, gb, p, s);
  return true;
}

void set_umma_test_expire(int on) {
  check_cuda(cudaMemcpyToSymbol(g_umma_test_expire, &on, sizeof(on)), "set test hook");
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

extern "C" int qtnh_debug_expire_exchange_wait(int on) {
  return QTNH_API([&]() -> int {
    set_umma_test_expire(on ? 1 : 0);
    return QTNH_OK;
  });
}

extern "C" int qtnh_take_device_errors(uint32_t* flags) {
  return QTNH_API([&]() -> int {
    if (!flags) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null flags pointer");
    check_cuda(cudaDeviceSynchronize(), "device synchronize");
    *flags = take_umma_error() | (take_gemm_error() << 8) | (take_ozg_error() << 16);
    return QTNH_OK;
  });
}
