// FP64-accurate complex GEMM on the 5th-generation tensor cores (tcgen05): the plain
// form of the dense contraction's GEMM (_contract_dense, src/tensor/contract.cpp:133-162
// of the reference sums complex<double> products over the closed indices).
//
// C (M x N) = A (M x K) B (K x N), complex128; here A is given as A'' (M x K row-major)
// and B as B'' (N x K row-major, the contracted index innermost in both).
//
// Real form: C^ (2M x N) = A^ (2M x 2K) B^^T with, for complex row m and column k,
//     A^[2m][2k] = Re a, A^[2m][2k+1] = -Im a, A^[2m+1][2k] = Im a, A^[2m+1][2k+1] = Re a,
//     B^[n][2k] = Re b, B^[n][2k+1] = Im b,
// so rows 2m / 2m+1 of C^ are Re / Im of C[m].
//
// Digits (the Ozaki scheme, ozaki.cuh): every real of complex row m of A is cut into six
// balanced base-256 digits at the row's largest exponent ea[m] (x ~= sum_i d_i 2^(-8i)
// 2^(ea - 1030), 48 significant bits relative to the row's largest element), every real
// of column n of B at eb[n]. Each digit is an integer of at most 8 significant bits:
// exact in bf16, and the product of two digits is exact in FP32. Then
//     C^[r][n] = 2^(ea + eb - 2060) sum_l 2^(-8l) S_l,  S_l = sum_{i+j=l} sum_k dA_i dB_j,
// levels l = 0..5 (the 21 digit pairs i + j <= 5; the dropped levels lie below 2^-48).
// Exactness: over a chunk of 128 reals of K (8 K-steps of 16) every level sum stays
// within 2^24 in magnitude (level 5: 128 * (2 * 256 * 128 + 4 * 128 * 128) = 2^24), so
// the tensor core's FP32 accumulators hold each chunk's level sums exactly. After each
// chunk the epilogue drains them from tensor memory and accumulates
//     T += S_0 2^24 + S_1 2^16 + S_2 2^8 + S_3   (exact, 64-bit integer),
//     F += S_4 + 2^-8 S_5                           (FP32; it lies below 2^-32 of T's scale),
// and at the end C^ = 2^(ea + eb - 2084) (T + 2^-8 F), rounded once to a double.
// The result is therefore accurate to ~2^-48 of the largest product magnitudes of its
// row and column, independent of K: FP64-level for the 1e-12 relative-L2 bar.
//
// Tile: 128 rows of C^ (64 complex rows) x 64 columns, as two halves of 32 columns. Per
// K-step the stage holds the six A digits (128 rows x 16 bf16 each, 24 KB) and, per half,
// the six B digits stacked along N (32 rows each, 6 KB), all in the UMMA K-major
// core-matrix layout (8 rows x 16 bytes; LBO 128 B, SBO 256 B). A digit i meets B digits
// 0 .. 5 - i of a half in one tcgen05.mma (kind::f16, bf16 in, FP32 out) of N = 32 (6 - i)
// into the half's level columns i ..: 6 MMAs per half and K-step, 12 per stage, the A
// digits read once per stage for both halves. Tensor memory: per half 6 levels x 32
// columns (192), both halves 384 of the SM's 512 columns.
// CTA (persistent, one per SM): warp 0 streams each K-step's 36 KB stage with bulk copies
// into a 5-stage ring, warp 1's elected thread issues the MMAs and commits, warps 2-9 (two
// per TMEM lane quarter, one per half) drain the level sums after each chunk and write
// the result (or, with split K, the exact partials T and F that a reduction kernel sums).
// Every wait is bounded by a clock limit; on expiry the CTA records an error flag
// (qtnh_take_device_errors, bits 16-18), stops and frees its tensor memory.
//
// Rows or columns holding an infinity or NaN (largest exponent 0x7FF) are recomputed in
// FP64 by a fix-up kernel after the GEMM; results outside the double range are scaled
// with scalbn (overflow to infinity, gradual underflow), as FP64 arithmetic would give.

#include <algorithm>

#include "cuda_common.cuh"
#include "ozaki.cuh"

namespace qtnh_impl {

// bit 0: producer wait expired, bit 1: MMA wait expired, bit 2: epilogue wait expired
__device__ unsigned int g_ozg_error;

namespace {

constexpr int OG_M = 128;                  // rows of C^ per tile (64 complex rows)
constexpr int OG_HN = 32;                  // columns of one half tile
constexpr int OG_H = 2;                    // halves per tile
constexpr int OG_N = OG_HN * OG_H;         // columns of C per tile
constexpr int OG_D = oz::NS;               // digits per real
constexpr int OG_L = oz::NL;               // levels kept
constexpr int OG_KSTEP = 16;               // bf16 K per MMA
constexpr uint32_t OG_CHUNK = 8;           // K-steps whose level sums are exact in FP32
constexpr int OG_A_DIGIT = OG_M * OG_KSTEP * 2;   // 4096 bytes
constexpr int OG_A_BLOCK = OG_D * OG_A_DIGIT;     // 24576 bytes: six A digits of one K-step
constexpr int OG_B_DIGIT = OG_HN * OG_KSTEP * 2;  // 1024 bytes
constexpr int OG_B_HALF = OG_D * OG_B_DIGIT;      // 6144 bytes: six B digits of a half
constexpr int OG_B_BLOCK = OG_H * OG_B_HALF;      // 12288 bytes
constexpr int OG_STAGE = OG_A_BLOCK + OG_B_BLOCK;  // 36864 bytes
constexpr int OG_STAGES = 5;
constexpr int OG_THREADS = 320;  // warp 0 producer, warp 1 MMA, warps 2-9 epilogue
constexpr uint32_t OG_EPI_THREADS = 256;
constexpr uint32_t OG_TMEM_COLS = 512;
constexpr uint32_t OG_HCOLS = OG_L * OG_HN;  // 192 columns per half
constexpr long long OG_WAIT_CYCLES = 1ll << 32;  // ~2 s at 2 GHz
constexpr uint32_t OG_SPECIAL = 0x7FFu;          // largest exponent of a row with an inf/NaN
static_assert(OG_H * OG_HCOLS <= OG_TMEM_COLS, "level sums exceed tensor memory");
static_assert(OG_HN * OG_L <= 256, "an MMA's N is at most 256");

struct OzParams {
  const uint8_t* a_planes;  // MT x KS blocks of OG_A_BLOCK bytes
  const uint8_t* b_planes;  // NT x KS blocks of OG_B_BLOCK bytes
  const uint32_t* ea;       // largest biased exponent of each complex row of A (0: all zero)
  const uint32_t* eb;       // largest biased exponent of each column of B
  double2* C;               // M x N row-major (one slice)
  long long* tpart;         // S x (MT * OG_M) x (NT * OG_N) exact partials T (several slices)
  float* fpart;             // the same shape: partials F
  uint64_t M, N;
  uint32_t MT, NT, KS;      // row tiles of C^, column tiles, K-steps
  uint32_t S, SK;           // K-slices, K-steps per slice (a multiple of OG_CHUNK)
};

struct OgSmem {
  uint8_t stage[OG_STAGES][OG_STAGE];
  uint64_t full[OG_STAGES];
  uint64_t empty[OG_STAGES];
  uint64_t tfull;   // a chunk's level sums are complete
  uint64_t tempty;  // the epilogue has drained them
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
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
__device__ __forceinline__ bool mbar_wait_thread(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort != 0 || clock64() - t0 > OG_WAIT_CYCLES) return false;
  }
  return true;
}
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const long long t0 = clock64();
  while (true) {
    const bool ok = mbar_try_wait(bar, parity);
    if (__all_sync(0xffffffffu, ok)) return true;
    if (__any_sync(0xffffffffu, *abort != 0 || clock64() - t0 > OG_WAIT_CYCLES)) return false;
  }
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major, no swizzle, LBO 128 B, SBO 256 B, descriptor version 1 (bits 46-47).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(256u >> 4) << 32) |
         (1ull << 46);
}

// kind::f16, D F32 (bits 4-5), A and B BF16 (bits 7-9, 10-12), K-major, N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__device__ __forceinline__ uint32_t og_idesc(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((uint32_t)(OG_M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
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

// 8 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__global__ void __launch_bounds__(OG_THREADS, 1) gemm_oz6_umma_kernel(const __grid_constant__ OzParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  OgSmem& sm = *reinterpret_cast<OgSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t ntiles = (uint64_t)p.MT * p.NT * p.S;
  // tile -> (column tile fastest, row tile, K-slice): neighbouring CTAs share the A rows
  auto tile_coords = [&](uint64_t tile, uint64_t& mt, uint64_t& nt, uint32_t& k0, uint32_t& k1) {
    nt = tile % p.NT;
    const uint64_t rest = tile / p.NT;
    mt = rest % p.MT;
    const uint32_t sl = (uint32_t)(rest / p.MT);
    k0 = sl * p.SK;
    k1 = min(p.KS, k0 + p.SK);
  };

  if (tid == 0) {
    sm.abort = 0;
    for (int s = 0; s < OG_STAGES; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    mbar_init(&sm.tfull, 1);
    mbar_init(&sm.tempty, OG_EPI_THREADS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(OG_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;

  if (warp == 0) {
    // ---- producer: one elected thread streams each K-step's digits ----
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        uint64_t mt, nt;
        uint32_t k0, k1;
        tile_coords(tile, mt, nt, k0, k1);
        for (uint32_t ks = k0; ks < k1; ++ks, ++it) {
          const uint32_t s = it % OG_STAGES, ph = (it / OG_STAGES) & 1u;
          if (!mbar_wait_thread(&sm.empty[s], ph ^ 1u, &sm.abort)) {
            atomicOr(&g_ozg_error, 1u);
            sm.abort = 1;
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&sm.full[s], (uint32_t)OG_STAGE);
          bulk_g2s(&sm.stage[s][0], p.a_planes + (mt * p.KS + ks) * (uint64_t)OG_A_BLOCK, OG_A_BLOCK, &sm.full[s]);
          bulk_g2s(&sm.stage[s][OG_A_BLOCK], p.b_planes + (nt * p.KS + ks) * (uint64_t)OG_B_BLOCK, OG_B_BLOCK,
                   &sm.full[s]);
        }
      }
    }
  } else if (warp == 1) {
    // ---- MMA: one elected thread; a chunk of up to OG_CHUNK K-steps per accumulation ----
    if (lane == 0) {
      uint32_t it = 0, ch = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        uint64_t mt, nt;
        uint32_t k0, k1;
        tile_coords(tile, mt, nt, k0, k1);
        for (uint32_t c0 = k0; ok && c0 < k1; c0 += OG_CHUNK, ++ch) {
          const uint32_t c1 = min(k1, c0 + OG_CHUNK);
          if (!mbar_wait_thread(&sm.tempty, (ch & 1u) ^ 1u, &sm.abort)) {
            atomicOr(&g_ozg_error, 2u);
            sm.abort = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          for (uint32_t ks = c0; ks < c1; ++ks, ++it) {
            const uint32_t s = it % OG_STAGES, ph = (it / OG_STAGES) & 1u;
            if (!mbar_wait_thread(&sm.full[s], ph, &sm.abort)) {
              atomicOr(&g_ozg_error, 2u);
              sm.abort = 1;
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t abase = smem_u32(&sm.stage[s][0]);
#pragma unroll
            for (int h = 0; h < OG_H; ++h) {
              const uint64_t bd = smem_desc(abase + (uint32_t)(OG_A_BLOCK + h * OG_B_HALF));
#pragma unroll
              for (int i = 0; i < OG_D; ++i) {
                // A digit i x B digits 0 .. 5 - i (stacked) -> levels i .. 5 of half h; the first
                // MMA of a chunk (i = 0, all six levels) overwrites, the rest accumulate
                const uint64_t ad = smem_desc(abase + (uint32_t)(i * OG_A_DIGIT));
                umma_bf16(tmem + (uint32_t)(h * OG_HCOLS + i * OG_HN), ad, bd, og_idesc((uint32_t)(OG_HN * (OG_L - i))),
                          (ks > c0 || i > 0) ? 1u : 0u);
              }
            }
            umma_commit(&sm.empty[s]);  // the stage is free once these MMAs have read it
          }
          if (ok) umma_commit(&sm.tfull);
        }
      }
    }
  } else {
    // ---- epilogue: warp w drains TMEM lanes 32 (w % 4) .. +31 of half (w - 2) / 4 ----
    const int q = warp & 3, h = (warp - 2) >> 2, r = q * 32 + lane;
    const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * OG_HCOLS);
    uint32_t ch = 0;
    bool ok = true;
    for (uint64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
      uint64_t mt, nt;
      uint32_t k0, k1;
      tile_coords(tile, mt, nt, k0, k1);
      long long T[OG_HN];
      float F[OG_HN];
#pragma unroll
      for (int c = 0; c < OG_HN; ++c) T[c] = 0, F[c] = 0.0f;
      for (uint32_t c0 = k0; c0 < k1; c0 += OG_CHUNK, ++ch) {
        if (!mbar_wait_warp(&sm.tfull, ch & 1u, &sm.abort)) {
          atomicOr(&g_ozg_error, 4u);
          sm.abort = 1;
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int g = 0; g < OG_HN / 8; ++g) {
          uint32_t v[OG_L][8];
#pragma unroll
          for (int l = 0; l < OG_L; ++l) tmem_ld8(tbase + (uint32_t)(l * OG_HN + 8 * g), v[l]);
          tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            // the level sums are exact integers of at most 2^24 in magnitude
            float lv[OG_L];
#pragma unroll
            for (int l = 0; l < OG_L; ++l) lv[l] = __uint_as_float(v[l][c]);
            oz::gemm_accumulate(lv, T[8 * g + c], F[8 * g + c]);
          }
        }
        tc_fence_before();
        mbar_arrive(&sm.tempty);
      }
      if (!ok) break;
      const uint64_t R = mt * OG_M + (uint64_t)r;  // row of C^: complex row R / 2, part R % 2
      const uint64_t n0 = nt * OG_N + (uint64_t)(h * OG_HN);
      if (p.S > 1) {
        const uint64_t ld = (uint64_t)p.NT * OG_N;
        const uint64_t base = ((uint64_t)(k0 / p.SK) * p.MT * OG_M + R) * ld + n0;
#pragma unroll
        for (int c = 0; c < OG_HN; c += 2) {
          *reinterpret_cast<longlong2*>(p.tpart + base + c) = make_longlong2(T[c], T[c + 1]);
        }
#pragma unroll
        for (int c = 0; c < OG_HN; c += 4) {
          *reinterpret_cast<float4*>(p.fpart + base + c) = make_float4(F[c], F[c + 1], F[c + 2], F[c + 3]);
        }
        continue;
      }
      // one slice: the even lane (Re row) writes columns 0..15 of the half, the odd lane
      // (Im row) columns 16..31; each receives the other part from its partner
      const uint64_t m = R >> 1;
      const bool odd = (lane & 1) != 0;
      const uint32_t ea = m < p.M ? p.ea[m] : 0u;
#pragma unroll
      for (int x = 0; x < OG_HN / 2; ++x) {
        // columns x (kept by the even lane) and 16 + x (kept by the odd lane)
        const uint64_t nlo = n0 + (uint64_t)x, nhi = nlo + OG_HN / 2;
        const uint32_t eblo = nlo < p.N ? p.eb[nlo] : 0u, ebhi = nhi < p.N ? p.eb[nhi] : 0u;
        const double vlo = oz::gemm_finish(T[x], F[x], oz::gemm_scale(ea, eblo));
        const double vhi = oz::gemm_finish(T[OG_HN / 2 + x], F[OG_HN / 2 + x], oz::gemm_scale(ea, ebhi));
        const double keep = odd ? vhi : vlo;
        const double recv = __shfl_xor_sync(0xffffffffu, odd ? vlo : vhi, 1);
        const uint64_t nk = odd ? nhi : nlo;
        if (m < p.M && nk < p.N) p.C[m * p.N + nk] = odd ? make_double2(recv, keep) : make_double2(keep, recv);
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OG_TMEM_COLS) : "memory");
  }
}

// Largest biased exponent of each of `rows` rows of X (rows x K complex128, row-major):
// one warp per row; 0 for an all-zero row, 0x7FF when the row holds an infinity or NaN.
__global__ void row_exponent_kernel(const double2* __restrict__ X, uint64_t rows, uint64_t K,
                                    uint32_t* __restrict__ e) {
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  for (uint64_t row = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < rows; row += warps) {
    const double2* x = X + row * K;
    uint32_t key = 0;
    for (uint64_t k = lane; k < K; k += 32) {
      const double2 v = x[k];
      key = max(key, max(oz::group_key(df::words(v.x)), oz::group_key(df::words(v.y))));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) key = max(key, __shfl_xor_sync(0xffffffffu, key, o));
    if (lane == 0) e[row] = oz::key_exponent(key);
  }
}

// Byte offset of the 16-byte core row (row rr of the tile, K-core kc) in digit `i` of
// the A block of (row tile, K-step).
__device__ __forceinline__ uint64_t og_a_offset(uint64_t row, uint64_t kc, int i, uint32_t KS) {
  const uint64_t mt = row >> 7, rr = row & 127;
  return ((mt * KS + (kc >> 1)) * OG_D + (uint64_t)i) * OG_A_DIGIT + ((rr >> 3) << 8) + ((kc & 1) << 7) + ((rr & 7) << 4);
}
// The same for B: column n (tile n / 64, half (n % 64) / 32, row n % 32 of the half).
__device__ __forceinline__ uint64_t og_b_offset(uint64_t n, uint64_t kc, int j, uint32_t KS) {
  const uint64_t nt = n >> 6, h = (n >> 5) & 1, rr = n & 31;
  return (((nt * KS + (kc >> 1)) * OG_H + h) * OG_D + (uint64_t)j) * OG_B_DIGIT + ((rr >> 3) << 8) + ((kc & 1) << 7) +
         ((rr & 7) << 4);
}

__device__ __forceinline__ uint32_t bf16_pair(float lo, float hi) { return oz::pack(lo, hi); }

// A^ digits: thread per (complex row m, K-core kc = complex columns 4 kc .. 4 kc + 3),
// consecutive threads on consecutive rows (their 16-byte core rows are contiguous).
// Rows 2m (Re a, -Im a) and 2m + 1 (Im a, Re a). Padding rows and columns are zero.
__global__ void oz_digits_a_kernel(const double2* __restrict__ A, const uint32_t* __restrict__ ea, uint64_t M,
                                   uint64_t K, uint64_t Mc, uint32_t KS, uint8_t* __restrict__ planes) {
  const uint64_t kcs = (uint64_t)KS * 2;
  const uint64_t total = Mc * kcs;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t m = t % Mc, kc = t / Mc;
    const uint32_t e = m < M ? ea[m] : 0u;
    const uint32_t es = oz::digit_scale(e);
    float re[4][OG_D], im[4][OG_D];
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      const uint64_t k = kc * 4 + x;
      const double2 a = (m < M && k < K && e != OG_SPECIAL) ? A[m * K + k] : make_double2(0.0, 0.0);
      oz::digits(df::words(a.x), es, re[x]);
      oz::digits(df::words(a.y), es, im[x]);
    }
#pragma unroll
    for (int i = 0; i < OG_D; ++i) {
      // row 2m: (Re, -Im) per complex column; row 2m + 1: (Im, Re)
      const uint4 r0 = make_uint4(bf16_pair(re[0][i], -im[0][i]), bf16_pair(re[1][i], -im[1][i]),
                                  bf16_pair(re[2][i], -im[2][i]), bf16_pair(re[3][i], -im[3][i]));
      const uint4 r1 = make_uint4(bf16_pair(im[0][i], re[0][i]), bf16_pair(im[1][i], re[1][i]),
                                  bf16_pair(im[2][i], re[2][i]), bf16_pair(im[3][i], re[3][i]));
      *reinterpret_cast<uint4*>(planes + og_a_offset(2 * m, kc, i, KS)) = r0;
      *reinterpret_cast<uint4*>(planes + og_a_offset(2 * m + 1, kc, i, KS)) = r1;
    }
  }
}

// B^ digits: thread per (column n, K-core kc = complex rows 4 kc .. 4 kc + 3) of B''
// (N x K row-major): B^[n][2k] = Re b, B^[n][2k+1] = Im b.
__global__ void oz_digits_b_kernel(const double2* __restrict__ Bt, const uint32_t* __restrict__ eb, uint64_t N,
                                   uint64_t K, uint64_t Nc, uint32_t KS, uint8_t* __restrict__ planes) {
  const uint64_t kcs = (uint64_t)KS * 2;
  const uint64_t total = Nc * kcs;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t n = t % Nc, kc = t / Nc;
    const uint32_t e = n < N ? eb[n] : 0u;
    const uint32_t es = oz::digit_scale(e);
    float re[4][OG_D], im[4][OG_D];
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      const uint64_t k = kc * 4 + x;
      const double2 b = (n < N && k < K && e != OG_SPECIAL) ? Bt[n * K + k] : make_double2(0.0, 0.0);
      oz::digits(df::words(b.x), es, re[x]);
      oz::digits(df::words(b.y), es, im[x]);
    }
#pragma unroll
    for (int j = 0; j < OG_D; ++j) {
      const uint4 v = make_uint4(bf16_pair(re[0][j], im[0][j]), bf16_pair(re[1][j], im[1][j]),
                                 bf16_pair(re[2][j], im[2][j]), bf16_pair(re[3][j], im[3][j]));
      *reinterpret_cast<uint4*>(planes + og_b_offset(n, kc, j, KS)) = v;
    }
  }
}

// C[m][n] from the S slices' exact partials of rows 2m (Re) and 2m + 1 (Im) of C^.
__global__ void oz_reduce_kernel(const long long* __restrict__ Tp, const float* __restrict__ Fp, uint32_t S,
                                 uint64_t rows, uint64_t ld, const uint32_t* __restrict__ ea,
                                 const uint32_t* __restrict__ eb, double2* __restrict__ C, uint64_t M, uint64_t N) {
  const uint64_t total = M * N;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t m = i / N, n = i % N;
    long long tr = 0, ti = 0;
    float fr = 0.0f, fi = 0.0f;
    for (uint32_t s = 0; s < S; ++s) {
      const uint64_t b = (uint64_t)s * rows * ld + (2 * m) * ld + n;
      tr += Tp[b];
      fr += Fp[b];
      ti += Tp[b + ld];
      fi += Fp[b + ld];
    }
    const int e = oz::gemm_scale(ea[m], eb[n]);
    C[i] = make_double2(oz::gemm_finish(tr, fr, e), oz::gemm_finish(ti, fi, e));
  }
}

// Outputs of rows of A or columns of B that hold an infinity or NaN, in FP64 (the
// digits cannot carry them); the kernel returns at once unless `flag` is set.
__global__ void oz_special_kernel(const double2* __restrict__ A, const double2* __restrict__ Bt,
                                  const uint32_t* __restrict__ ea, const uint32_t* __restrict__ eb,
                                  const uint32_t* __restrict__ flag, double2* __restrict__ C, uint64_t M, uint64_t N,
                                  uint64_t K) {
  if (*flag == 0u) return;
  const uint64_t total = M * N;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t m = i / N, n = i % N;
    if (ea[m] != OG_SPECIAL && eb[n] != OG_SPECIAL) continue;
    double2 acc = make_double2(0.0, 0.0);
    for (uint64_t k = 0; k < K; ++k) acc = cfma(A[m * K + k], Bt[n * K + k], acc);
    C[i] = acc;
  }
}

// Flags whether any row exponent is 0x7FF.
__global__ void oz_any_special_kernel(const uint32_t* __restrict__ e, uint64_t n, uint32_t* __restrict__ flag) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (e[i] == OG_SPECIAL) atomicOr(flag, 1u);
}

}  // namespace

// C (M x N) = A'' (M x K) B''^T, with A'' and B'' (N x K) complex128 row-major, on the
// tensor cores through exact digit products (see the file header).
void gemm_oz6(const void* Av, const void* Btv, void* Cv, uint64_t M, uint64_t N, uint64_t K, void* stream) {
  if (M == 0 || N == 0) return;
  const c128* A = static_cast<const c128*>(Av);
  const c128* Bt = static_cast<const c128*>(Btv);
  c128* C = static_cast<c128*>(Cv);
  cudaStream_t s = (cudaStream_t)stream;
  if (K == 0) {
    check_cuda(cudaMemsetAsync(C, 0, M * N * sizeof(c128), s), "zero C");
    return;
  }
  const uint64_t Kp = (K + 7) / 8 * 8;  // complex K padded: 2 Kp reals = KS K-steps
  const uint32_t KS = (uint32_t)(2 * Kp / OG_KSTEP);
  OzParams p{};
  p.MT = (uint32_t)((2 * M + OG_M - 1) / OG_M);
  p.NT = (uint32_t)((N + OG_N - 1) / OG_N);
  p.KS = KS;
  p.M = M;
  p.N = N;
  p.C = C;
  const uint64_t a_bytes = (uint64_t)p.MT * KS * OG_A_BLOCK;
  const uint64_t b_bytes = (uint64_t)p.NT * KS * OG_B_BLOCK;
  // split K over chunk-aligned slices when the tiles alone would leave SMs idle
  const uint64_t tiles = (uint64_t)p.MT * p.NT;
  const uint32_t chunks = (KS + OG_CHUNK - 1) / OG_CHUNK;
  uint32_t S = 1;
  if (tiles < (uint64_t)sm_count()) S = (uint32_t)std::min<uint64_t>(chunks, ((uint64_t)sm_count() + tiles - 1) / tiles);
  p.SK = ((chunks + S - 1) / S) * OG_CHUNK;
  p.S = (KS + p.SK - 1) / p.SK;
  const uint64_t rows = (uint64_t)p.MT * OG_M, ld = (uint64_t)p.NT * OG_N;
  const uint64_t part = p.S > 1 ? (uint64_t)p.S * rows * ld : 0;
  const uint64_t e_bytes = ((M + N + 64) * sizeof(uint32_t) + 255) / 256 * 256;
  const uint64_t bytes = a_bytes + b_bytes + e_bytes + part * (sizeof(long long) + sizeof(float));
  uint8_t* ws = static_cast<uint8_t*>(workspace_alloc(bytes, stream));
  try {
    uint8_t* apl = ws;
    uint8_t* bpl = ws + a_bytes;
    uint32_t* ea = reinterpret_cast<uint32_t*>(ws + a_bytes + b_bytes);
    uint32_t* eb = ea + M;
    uint32_t* flag = eb + N;
    p.a_planes = apl;
    p.b_planes = bpl;
    p.ea = ea;
    p.eb = eb;
    p.tpart = p.S > 1 ? reinterpret_cast<long long*>(ws + a_bytes + b_bytes + e_bytes) : nullptr;
    p.fpart = p.S > 1 ? reinterpret_cast<float*>(ws + a_bytes + b_bytes + e_bytes + part * sizeof(long long)) : nullptr;
    row_exponent_kernel<<<grid_for((M + 7) / 8, 8), 256, 0, s>>>(A, M, K, ea);
    row_exponent_kernel<<<grid_for((N + 7) / 8, 8), 256, 0, s>>>(Bt, N, K, eb);
    count_launch(2);
    const uint64_t Mc = (uint64_t)p.MT * (OG_M / 2), Nc = (uint64_t)p.NT * OG_N;
    oz_digits_a_kernel<<<grid_for((Mc * 2 * KS + 255) / 256, 8), 256, 0, s>>>(A, ea, M, K, Mc, KS, apl);
    oz_digits_b_kernel<<<grid_for((Nc * 2 * KS + 255) / 256, 8), 256, 0, s>>>(Bt, eb, N, K, Nc, KS, bpl);
    count_launch(2);
    const size_t smem = sizeof(OgSmem);
    check_cuda(cudaFuncSetAttribute(gemm_oz6_umma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "gemm_oz6_umma_kernel shared memory");
    const int grid = (int)std::min<uint64_t>((uint64_t)p.MT * p.NT * p.S, (uint64_t)sm_count());
    gemm_oz6_umma_kernel<<<grid, OG_THREADS, smem, s>>>(p);
    count_launch();
    if (p.S > 1) {
      oz_reduce_kernel<<<grid_for((M * N + 255) / 256, 8), 256, 0, s>>>(p.tpart, p.fpart, p.S, rows, ld, ea, eb, C, M,
                                                                          N);
      count_launch();
    }
    // rows / columns with an infinity or NaN: recomputed in FP64 on the device (in the
    // common case the second kernel reads the cleared flag and returns)
    check_cuda(cudaMemsetAsync(flag, 0, sizeof(uint32_t), s), "clear flag");
    oz_any_special_kernel<<<grid_for((M + N + 255) / 256, 2), 256, 0, s>>>(ea, M + N, flag);
    oz_special_kernel<<<grid_for((M * N + 255) / 256, 4), 256, 0, s>>>(A, Bt, ea, eb, flag, C, M, N, K);
    count_launch(2);
    check_cuda(cudaGetLastError(), "digit GEMM launch");
  } catch (...) {
    workspace_free(ws, stream);
    throw;
  }
  workspace_free(ws, stream);
}

uint32_t take_ozg_error() {
  uint32_t v = 0;
  check_cuda(cudaMemcpyFromSymbol(&v, g_ozg_error, sizeof(v)), "read device error flags");
  const uint32_t zero = 0;
  check_cuda(cudaMemcpyToSymbol(g_ozg_error, &zero, sizeof(zero)), "clear device error flags");
  return v;
}

}  // namespace qtnh_impl
