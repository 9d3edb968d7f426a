// Split-precision complex GEMM on the 5th-generation tensor cores (tcgen05), the
// QTNH_GEMM_BF16X3 form of the dense contraction (_contract_dense, contract.cpp:12-201 of
// the reference): C = A B with A (M x K), B (K x N) complex128, row-major.
//
// Real form: C_re = A_re B_re - A_im B_im, C_im = A_im B_re + A_re B_im is one real GEMM
// C^ (2M x N) = A^ (2M x 2K) B^ (2K x N) with, for complex row m and column k,
//     A^[2m][2k] = Re a, A^[2m][2k+1] = -Im a, A^[2m+1][2k] = Im a, A^[2m+1][2k+1] = Re a,
//     B^[2k][n] = Re b, B^[2k+1][n] = Im b,
// so rows 2m / 2m+1 of C^ are Re / Im of C[m]. Every real is split into three bf16
// pieces x = h + m + l (24 significant bits; the split runs through the float-float
// split of df32.cuh), and C^ = sum over the six piece pairs (i, j), i + j <= 2, of
// A^_i B^_j, accumulated in FP32 in tensor memory. The pieces hold 24 bits of every
// real; the tensor core's FP32 accumulation loses up to an ulp per accumulation step in
// one direction, so (1) the dominant pair h*h accumulates in its own TMEM accumulator
// and the five smaller pairs (<= 2^-8 of it) in a second one, and (2) K is split into
// slices of at most qtnh_get_gemm_slice() K-steps (default 32 = 512 reals), each
// accumulated on its own and written as FP32 partials, which a reduction kernel sums with
// compensated FP32 additions (split-K; it also spreads small GEMMs over all SMs). The
// error grows in proportion to the slice length (relative L2 2.3e-7, 4.7e-7, 1.0e-6,
// 2.1e-6 at 16, 32, 64, 128 K-steps), the partials' traffic in inverse proportion.
//
// Kernels: split_a / split_b write the pieces as bf16 planes in the UMMA K-major
// core-matrix layout (8 rows x 16 bytes; per tile and K-step of 16 a contiguous block,
// LBO 128 B, SBO 256 B). The GEMM is persistent, one CTA per SM, tiles of 128 rows of C^
// x 256 columns x one K-slice: warp 0 streams each K-step's six blocks (36 KB) into a 5-stage
// shared-memory ring with bulk copies (cp.async.bulk, mbarrier transaction counts),
// warp 1's elected thread issues six tcgen05.mma (M 128, N 256, K 16) per K-step into
// the two TMEM accumulators and commits the stage back to the producer, and warps 2-5
// read the finished accumulator (tcgen05.ld) and either pair the Re/Im rows with a
// shuffle and store complex128 (one slice) or store the FP32 partials. Every wait is
// bounded by a clock limit (device error flags).

#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "bf16x3.cuh"
#include "cuda_common.cuh"
#include "df32.cuh"

namespace qtnh_impl {

// bit 0: producer wait expired, bit 1: MMA wait expired, bit 2: epilogue wait expired
__device__ unsigned int g_gemm_error;

namespace {

constexpr int GM_M = 128;  // MMA M: rows of the real-form tile
constexpr int GM_N = 256;  // MMA N: columns of C per tile
constexpr int GM_K = bx3::K_STEP;  // bf16 K per MMA
constexpr int GM_P = bx3::PIECES;  // bf16 pieces per real
constexpr int GM_STAGES = 5;
constexpr int GM_A_BLOCK = GM_M * GM_K * 2;  // 4096 bytes: one plane, one tile, one K-step
constexpr int GM_B_BLOCK = GM_N * GM_K * 2;  // 8192 bytes
constexpr int GM_STAGE_BYTES = GM_P * (GM_A_BLOCK + GM_B_BLOCK);
constexpr int GM_THREADS = 192;            // warp 0 producer, warp 1 MMA, warps 2-5 epilogue
constexpr uint32_t GM_TMEM_COLS = 512;     // accumulators D1 (h*h) and D2 (other pairs), GM_N columns each
constexpr long long GM_WAIT_CYCLES = 1ll << 32;  // ~2 s at 2 GHz

// piece pairs (A piece, B piece) with i + j <= 2
__constant__ uint8_t c_pairs[6][2] = {{0, 0}, {0, 1}, {1, 0}, {0, 2}, {1, 1}, {2, 0}};

struct GemmParams {
  const uint8_t* a_planes;  // GM_P planes of MT x KS blocks of GM_A_BLOCK bytes
  const uint8_t* b_planes;  // GM_P planes of NT x KS blocks of GM_B_BLOCK bytes
  double2* C;               // M x N row-major (one slice)
  float* partial;           // S x (MT * GM_M) x (NT * GM_N) FP32 partials of C^ (several slices)
  uint64_t a_plane_bytes, b_plane_bytes;
  uint64_t M, N;            // complex rows / columns of C
  uint32_t MT, NT, KS;      // row tiles of C^, column tiles, K-steps
  uint32_t S, SK;           // K-slices, K-steps per slice
};

struct GmSmem {
  uint8_t stage[GM_STAGES][GM_STAGE_BYTES];  // A planes 0..2, then B planes 0..2
  uint64_t full[GM_STAGES];                  // stage loaded (transaction count)
  uint64_t empty[GM_STAGES];                 // stage consumed by the MMAs
  uint64_t tfull;                            // accumulators complete
  uint64_t tempty;                           // accumulators read by the epilogue
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
// One thread's bounded wait; false on expiry or abort.
__device__ __forceinline__ bool mbar_wait_thread(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort != 0 || clock64() - t0 > GM_WAIT_CYCLES) return false;
  }
  return true;
}
// Warp-uniform bounded wait.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const long long t0 = clock64();
  while (true) {
    const bool ok = mbar_try_wait(bar, parity);
    if (__all_sync(0xffffffffu, ok)) return true;
    if (__any_sync(0xffffffffu, *abort != 0 || clock64() - t0 > GM_WAIT_CYCLES)) return false;
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

// kind::f16, D F32, A and B BF16, K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t GM_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(GM_N >> 3) << 17) |
                              ((uint32_t)(GM_M >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(GM_IDESC), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__global__ void __launch_bounds__(GM_THREADS, 1) gemm_bf16x3_umma_kernel(const __grid_constant__ GemmParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  GmSmem& sm = *reinterpret_cast<GmSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t ntiles = (uint64_t)p.MT * p.NT * p.S;
  // tile -> (row tile, column tile, K-slice), row tiles fastest (neighbours share B)
  auto tile_coords = [&](uint64_t tile, uint64_t& mt, uint64_t& nt, uint32_t& k0, uint32_t& k1) {
    mt = tile % p.MT;
    const uint64_t rest = tile / p.MT;
    nt = rest % p.NT;
    const uint32_t sl = (uint32_t)(rest / p.NT);
    k0 = sl * p.SK;
    k1 = min(p.KS, k0 + p.SK);
  };

  if (tid == 0) {
    sm.abort = 0;
    for (int s = 0; s < GM_STAGES; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    mbar_init(&sm.tfull, 1);
    mbar_init(&sm.tempty, 128);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(GM_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;

  if (warp == 0) {
    // ---- producer: one elected thread streams the operand blocks ----
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        uint64_t mt, nt;
        uint32_t k0, k1;
        tile_coords(tile, mt, nt, k0, k1);
        for (uint32_t ks = k0; ks < k1; ++ks, ++it) {
          const uint32_t s = it % GM_STAGES, ph = (it / GM_STAGES) & 1u;
          if (!mbar_wait_thread(&sm.empty[s], ph ^ 1u, &sm.abort)) {
            atomicOr(&g_gemm_error, 1u);
            sm.abort = 1;
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&sm.full[s], (uint32_t)GM_STAGE_BYTES);
          const uint64_t ablk = (mt * p.KS + ks) * (uint64_t)GM_A_BLOCK;
          const uint64_t bblk = (nt * p.KS + ks) * (uint64_t)GM_B_BLOCK;
#pragma unroll
          for (int pl = 0; pl < GM_P; ++pl)
            bulk_g2s(&sm.stage[s][pl * GM_A_BLOCK], p.a_planes + pl * p.a_plane_bytes + ablk, GM_A_BLOCK, &sm.full[s]);
#pragma unroll
          for (int pl = 0; pl < GM_P; ++pl)
            bulk_g2s(&sm.stage[s][GM_P * GM_A_BLOCK + pl * GM_B_BLOCK], p.b_planes + pl * p.b_plane_bytes + bblk,
                     GM_B_BLOCK, &sm.full[s]);
        }
      }
    }
  } else if (warp == 1) {
    // ---- MMA: one elected thread ----
    if (lane == 0) {
      uint32_t it = 0, lt = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, ++lt) {
        if (!mbar_wait_thread(&sm.tempty, (lt & 1u) ^ 1u, &sm.abort)) {
          atomicOr(&g_gemm_error, 2u);
          sm.abort = 1;
          break;
        }
        tc_fence_after();
        const uint32_t d1 = tmem, d2 = tmem + (uint32_t)GM_N;
        uint64_t mt, nt;
        uint32_t k0, k1;
        tile_coords(tile, mt, nt, k0, k1);
        for (uint32_t ks = k0; ks < k1; ++ks, ++it) {
          const uint32_t s = it % GM_STAGES, ph = (it / GM_STAGES) & 1u;
          if (!mbar_wait_thread(&sm.full[s], ph, &sm.abort)) {
            atomicOr(&g_gemm_error, 2u);
            sm.abort = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t abase = smem_u32(&sm.stage[s][0]);
          const uint32_t bbase = abase + (uint32_t)(GM_P * GM_A_BLOCK);
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            const uint64_t ad = smem_desc(abase + (uint32_t)(c_pairs[q][0] * GM_A_BLOCK));
            const uint64_t bd = smem_desc(bbase + (uint32_t)(c_pairs[q][1] * GM_B_BLOCK));
            if (q == 0)
              umma_bf16(d1, ad, bd, ks > k0 ? 1u : 0u);
            else
              umma_bf16(d2, ad, bd, (ks > k0 || q > 1) ? 1u : 0u);
          }
          umma_commit(&sm.empty[s]);  // the stage is free once these MMAs have read it
        }
        if (ok) umma_commit(&sm.tfull);
      }
    }
  } else {
    // ---- epilogue: warps 2-5 read TMEM lanes 32 (warp % 4) .. +31 ----
    const int q = warp & 3, r = q * 32 + lane;
    uint32_t lt = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++lt) {
      if (!mbar_wait_warp(&sm.tfull, lt & 1u, &sm.abort)) {
        atomicOr(&g_gemm_error, 4u);
        sm.abort = 1;
        break;
      }
      tc_fence_after();
      uint64_t mt, nt;
      uint32_t k0, k1;
      tile_coords(tile, mt, nt, k0, k1);
      const uint64_t R = mt * GM_M + (uint64_t)r;  // row of C^: complex row R / 2, part R % 2
      const uint64_t m = R >> 1;
      const bool odd = (lane & 1) != 0;
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16);
      // 32 columns of D1 + D2 (one rounding to nearest)
      auto load_sum = [&](int ch, uint32_t (&v)[32]) {
        uint32_t w[32];
        tmem_ld32(tbase + (uint32_t)(ch * 32), v);
        tmem_ld32(tbase + (uint32_t)(GM_N + ch * 32), w);
        tmem_wait_ld();
#pragma unroll
        for (int x = 0; x < 32; ++x) v[x] = __float_as_uint(__fadd_rn(__uint_as_float(v[x]), __uint_as_float(w[x])));
      };
      if (p.S > 1) {
        // FP32 partials of this slice: row R of C^, 256 columns
        float* dst = p.partial + ((uint64_t)(k0 / p.SK) * p.MT * GM_M + R) * ((uint64_t)p.NT * GM_N) + nt * GM_N;
#pragma unroll 1
        for (int ch = 0; ch < GM_N / 32; ++ch) {
          uint32_t v[32];
          load_sum(ch, v);
#pragma unroll
          for (int x = 0; x < 32; x += 4)
            *reinterpret_cast<uint4*>(dst + ch * 32 + x) = make_uint4(v[x], v[x + 1], v[x + 2], v[x + 3]);
        }
        tc_fence_before();
        mbar_arrive(&sm.tempty);
        continue;
      }
#pragma unroll 1
      for (int ch = 0; ch < GM_N / 32; ++ch) {
        uint32_t v[32];
        load_sum(ch, v);
        // the even lane (Re row) writes columns 0..15 of the chunk, the odd lane (Im row)
        // columns 16..31; each receives the other part from its partner
        const uint64_t n0 = nt * GM_N + (uint64_t)ch * 32 + (odd ? 16 : 0);
#pragma unroll
        for (int x = 0; x < 16; ++x) {
          const uint32_t send = odd ? v[x] : v[16 + x];
          const uint32_t recv = __shfl_xor_sync(0xffffffffu, send, 1);
          const float re = __uint_as_float(odd ? recv : v[x]);
          const float im = __uint_as_float(odd ? v[16 + x] : recv);
          const uint64_t n = n0 + (uint64_t)x;
          if (m < p.M && n < p.N) p.C[m * p.N + n] = make_double2((double)re, (double)im);
        }
      }
      tc_fence_before();
      mbar_arrive(&sm.tempty);
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(GM_TMEM_COLS) : "memory");
  }
}

using bx3::pieces;
using bx3::plane_offset;

// A^ pieces: thread per (complex row m, K-core kc = complex columns 4 kc .. 4 kc + 3);
// rows 2m and 2m + 1 of A^. Out-of-range elements (padding) are zero.
__global__ void split_a_kernel(const double2* __restrict__ A, uint64_t M, uint64_t K, uint8_t* __restrict__ planes,
                               uint64_t plane_bytes, uint64_t Mpad, uint32_t KS) {
  const uint64_t kcs = (uint64_t)KS * 2;
  const uint64_t total = Mpad * kcs;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t m = i / kcs, kc = i % kcs;
    uint16_t re[4][GM_P], im[4][GM_P];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const uint64_t k = kc * 4 + e;
      const double2 a = (m < M && k < K) ? A[m * K + k] : make_double2(0.0, 0.0);
      pieces(a.x, re[e]);
      pieces(a.y, im[e]);
    }
#pragma unroll
    for (int pl = 0; pl < GM_P; ++pl) {
      uint32_t r0[4], r1[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        // row 2m: (Re a, -Im a); row 2m+1: (Im a, Re a)
        r0[e] = (uint32_t)re[e][pl] | ((uint32_t)(im[e][pl] ^ 0x8000u) << 16);
        r1[e] = (uint32_t)im[e][pl] | ((uint32_t)re[e][pl] << 16);
      }
      uint8_t* base = planes + pl * plane_bytes;
      *reinterpret_cast<uint4*>(base + plane_offset(2 * m, kc, GM_M, KS)) = make_uint4(r0[0], r0[1], r0[2], r0[3]);
      *reinterpret_cast<uint4*>(base + plane_offset(2 * m + 1, kc, GM_M, KS)) = make_uint4(r1[0], r1[1], r1[2], r1[3]);
    }
  }
}

// B^ pieces (stored N x 2K, K-major): thread per (column n, K-core kc = complex rows
// 4 kc .. 4 kc + 3): B^[2k][n] = Re b, B^[2k+1][n] = Im b.
__global__ void split_b_kernel(const double2* __restrict__ B, uint64_t K, uint64_t N, uint8_t* __restrict__ planes,
                               uint64_t plane_bytes, uint64_t Npad, uint32_t KS) {
  const uint64_t kcs = (uint64_t)KS * 2;
  const uint64_t total = Npad * kcs;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t n = i % Npad, kc = i / Npad;  // consecutive threads: consecutive columns
    uint16_t re[4][GM_P], im[4][GM_P];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const uint64_t k = kc * 4 + e;
      const double2 b = (n < N && k < K) ? B[k * N + n] : make_double2(0.0, 0.0);
      pieces(b.x, re[e]);
      pieces(b.y, im[e]);
    }
#pragma unroll
    for (int pl = 0; pl < GM_P; ++pl) {
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) w[e] = (uint32_t)re[e][pl] | ((uint32_t)im[e][pl] << 16);
      *reinterpret_cast<uint4*>(planes + pl * plane_bytes + plane_offset(n, kc, GM_N, KS)) =
          make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// C[m][n] = sum over the S slices of the partials of rows 2m (Re) and 2m + 1 (Im) of
// C^, with compensated FP32 additions (TwoSum), rounded once to double. Thread per (row m,
// four consecutive columns): 16-byte loads of both rows from every slice (the partial rows
// are padded to a multiple of 256 columns), rows over blockIdx.y (no index division).
__global__ void __launch_bounds__(256) reduce_partials_kernel(const float* __restrict__ P, uint32_t S, uint64_t rows,
                                                              uint64_t ldp, double2* __restrict__ C, uint64_t M,
                                                              uint64_t N) {
  const uint64_t nq = (N + 3) / 4;
  for (uint64_t m = blockIdx.y; m < M; m += gridDim.y) {
    for (uint64_t qd = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; qd < nq; qd += (uint64_t)gridDim.x * blockDim.x) {
      float sr[4] = {0.f, 0.f, 0.f, 0.f}, er[4] = {0.f, 0.f, 0.f, 0.f};
      float si[4] = {0.f, 0.f, 0.f, 0.f}, ei[4] = {0.f, 0.f, 0.f, 0.f};
      const float* pr = P + (2 * m) * ldp + 4 * qd;
#pragma unroll 2
      for (uint32_t sl = 0; sl < S; ++sl, pr += rows * ldp) {
        const float4 a = *reinterpret_cast<const float4*>(pr);
        const float4 b = *reinterpret_cast<const float4*>(pr + ldp);
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int x = 0; x < 4; ++x) {
          float t, e;
          df::two_sum(sr[x], av[x], t, e);
          sr[x] = t;
          er[x] = __fadd_rn(er[x], e);
          df::two_sum(si[x], bv[x], t, e);
          si[x] = t;
          ei[x] = __fadd_rn(ei[x], e);
        }
      }
#pragma unroll
      for (int x = 0; x < 4; ++x) {
        const uint64_t n = 4 * qd + (uint64_t)x;
        if (n < N) C[m * N + n] = make_double2((double)sr[x] + (double)er[x], (double)si[x] + (double)ei[x]);
      }
    }
  }
}

}  // namespace

// Optional CUDA-event timing of the GEMM kernel launches (qtnh_gemm_timing).
static std::mutex g_timing_mu;
static bool g_timing = false;
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_timing_events;

// Operand preparation: fills the GM_P planes of one operand (pieces in the UMMA layout).
struct Prep {
  // A^ (two real rows per complex row) or B^ (one row per column)
  bool is_a;
  const c128* data;                 // the operand
  const dims_t* dims = nullptr;     // non-null: permute (fused) with ptup to [rows | K]
  const std::vector<uint16_t>* ptup = nullptr;
  int nrow_axes = 0;
};

// C (M x N) = A (M x K) B (K x N), complex128 row-major, through BF16x3 pieces on tcgen05.
static void gemm_core(const Prep& pa, const Prep& pb, void* Cv, uint64_t M, uint64_t N, uint64_t K, void* stream) {
  if (M == 0 || N == 0) return;
  c128* C = static_cast<c128*>(Cv);
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t Kp = std::max<uint64_t>(8, (K + 7) / 8 * 8);  // complex K padded: 2 Kp reals = KS K-steps
  const uint32_t KS = (uint32_t)(2 * Kp / GM_K);
  const uint64_t Mpad = (M + GM_M / 2 - 1) / (GM_M / 2) * (GM_M / 2);  // complex rows: 2 Mpad reals per plane
  const uint64_t Npad = (N + GM_N - 1) / GM_N * GM_N;
  GemmParams p;
  p.MT = (uint32_t)(2 * Mpad / GM_M);
  p.NT = (uint32_t)(Npad / GM_N);
  p.KS = KS;
  p.M = M;
  p.N = N;
  p.C = C;
  p.a_plane_bytes = (uint64_t)p.MT * KS * GM_A_BLOCK;
  p.b_plane_bytes = (uint64_t)p.NT * KS * GM_B_BLOCK;
  p.SK = (uint32_t)gemm_slice_steps();
  p.S = (KS + p.SK - 1) / p.SK;
  const uint64_t planes = GM_P * (p.a_plane_bytes + p.b_plane_bytes);
  const uint64_t part = p.S > 1 ? (uint64_t)p.S * p.MT * GM_M * p.NT * GM_N * sizeof(float) : 0;
  uint8_t* ws = static_cast<uint8_t*>(workspace_alloc(planes + part, stream));
  p.a_planes = ws;
  p.b_planes = ws + GM_P * p.a_plane_bytes;
  p.partial = p.S > 1 ? reinterpret_cast<float*>(ws + planes) : nullptr;
  try {
    if (pa.dims) {
      permute_split_device(pa.data, *pa.dims, *pa.ptup, pa.nrow_axes, M, Mpad, K, 2 * (uint64_t)KS, ws,
                           p.a_plane_bytes, GM_M, KS, true, stream);
    } else {
      const uint64_t na = Mpad * KS * 2;
      split_a_kernel<<<grid_for((na + 255) / 256, 8), 256, 0, s>>>(pa.data, M, K, ws, p.a_plane_bytes, Mpad, KS);
      count_launch();
    }
    uint8_t* bpl = ws + GM_P * p.a_plane_bytes;
    if (pb.dims) {
      permute_split_device(pb.data, *pb.dims, *pb.ptup, pb.nrow_axes, N, Npad, K, 2 * (uint64_t)KS, bpl,
                           p.b_plane_bytes, GM_N, KS, false, stream);
    } else {
      const uint64_t nb = Npad * KS * 2;
      split_b_kernel<<<grid_for((nb + 255) / 256, 8), 256, 0, s>>>(pb.data, K, N, bpl, p.b_plane_bytes, Npad, KS);
      count_launch();
    }
    const size_t smem = sizeof(GmSmem);
    check_cuda(cudaFuncSetAttribute(gemm_bf16x3_umma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "gemm_bf16x3_umma_kernel shared memory");
    const int grid = (int)std::min<uint64_t>((uint64_t)p.MT * p.NT * p.S, (uint64_t)sm_count());
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    {
      std::lock_guard<std::mutex> lk(g_timing_mu);
      if (g_timing) {
        check_cuda(cudaEventCreate(&e0), "event");
        check_cuda(cudaEventCreate(&e1), "event");
        check_cuda(cudaEventRecord(e0, s), "event record");
      }
    }
    gemm_bf16x3_umma_kernel<<<grid, GM_THREADS, smem, s>>>(p);
    if (e0) {
      check_cuda(cudaEventRecord(e1, s), "event record");
      std::lock_guard<std::mutex> lk(g_timing_mu);
      g_timing_events.emplace_back(e0, e1);
    }
    count_launch();
    if (p.S > 1) {
      // about 8 blocks of 256 threads per SM: column blocks along x, rows along y
      const uint64_t gx = std::min<uint64_t>(((N + 3) / 4 + 255) / 256, 64);
      const dim3 rgrid((unsigned)gx, (unsigned)std::min<uint64_t>(M, std::max<uint64_t>(1, 8ull * sm_count() / gx)));
      reduce_partials_kernel<<<rgrid, 256, 0, s>>>(p.partial, p.S, (uint64_t)p.MT * GM_M, (uint64_t)p.NT * GM_N, C, M,
                                                   N);
      count_launch();
    }
    check_cuda(cudaGetLastError(), "split GEMM launch");
  } catch (...) {
    workspace_free(ws, stream);
    throw;
  }
  workspace_free(ws, stream);
}

void gemm_bf16x3(const void* Av, const void* Bv, void* Cv, uint64_t M, uint64_t N, uint64_t K, void* stream) {
  Prep pa{true, static_cast<const c128*>(Av)}, pb{false, static_cast<const c128*>(Bv)};
  gemm_core(pa, pb, Cv, M, N, K, stream);
}

// The contraction's GEMM with the operand permutes fused into the piece splits: A' = A
// permuted by pA to [rows | K] (nrow_a row axes; identity: A is read directly), B' = B
// permuted by pB to [K | columns] (identity: read directly), else B is permuted by pBt to
// [columns | K] (ncol_b column axes) and written straight into the B^ planes.
void gemm_bf16x3_perm(const void* A, const dims_t& dims_a, const std::vector<uint16_t>& pA, int nrow_a,
                      const void* B, const dims_t& dims_b, const std::vector<uint16_t>& pB,
                      const std::vector<uint16_t>& pBt, int ncol_b, void* C, uint64_t M, uint64_t N, uint64_t K,
                      void* stream) {
  auto identity = [](const std::vector<uint16_t>& p) {
    for (size_t i = 0; i < p.size(); ++i)
      if (p[i] != i) return false;
    return true;
  };
  Prep pa{true, static_cast<const c128*>(A)}, pb{false, static_cast<const c128*>(B)};
  if (!identity(pA)) pa.dims = &dims_a, pa.ptup = &pA, pa.nrow_axes = nrow_a;
  if (!identity(pB)) pb.dims = &dims_b, pb.ptup = &pBt, pb.nrow_axes = ncol_b;
  gemm_core(pa, pb, C, M, N, K, stream);
}

// Sum of the recorded GEMM kernel durations (synchronizes on each event pair).
static void take_gemm_times(double& ms, uint64_t& launches) {
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    ev.swap(g_timing_events);
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

uint32_t take_gemm_error() {
  uint32_t v = 0;
  check_cuda(cudaMemcpyFromSymbol(&v, g_gemm_error, sizeof(v)), "read device error flags");
  const uint32_t zero = 0;
  check_cuda(cudaMemcpyToSymbol(g_gemm_error, &zero, sizeof(zero)), "clear device error flags");
  return v;
}

}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" int qtnh_gemm_timing(int enable, double* ms, uint64_t* launches) {
  return QTNH_API([&]() -> int {
    double t = 0;
    uint64_t n = 0;
    take_gemm_times(t, n);
    if (ms) *ms = t;
    if (launches) *launches = n;
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timing = enable != 0;
    return QTNH_OK;
  });
}
