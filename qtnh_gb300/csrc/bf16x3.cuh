// The three-piece bf16 form of complex128 operands for the split-precision GEMM
// (gemm_umma.cu): every real x = h + m + l in bf16 (24 significant bits), written into
// planes in the UMMA K-major core-matrix layout (8 rows x 16 bytes; per tile of `tile`
// rows and K-step of 16 bf16 a contiguous block, LBO 128 B, SBO 256 B). Shared by the
// split kernels of the GEMM and the fused permute-and-split kernels of permute.cu.
#pragma once

#include <cuda_bf16.h>

#include "cuda_common.cuh"
#include "df32.cuh"

namespace qtnh_impl {
namespace bx3 {

constexpr int K_STEP = 16;  // bf16 K per MMA
constexpr int PIECES = 3;   // bf16 pieces per real

// x = h + m + l in bf16 (24 significant bits), through the float-float split where x is
// in its range, else through FP64 arithmetic.
__device__ __forceinline__ void pieces(double x, uint16_t (&out)[PIECES]) {
  const df::dwords w = df::words(x);
  float hi, lo;
  if (df::in_range_state(w)) {
    const df::f2 f = df::split(w);
    hi = f.h;
    lo = f.l;
  } else {
    hi = (float)x;
    lo = (float)(x - (double)hi);
  }
  const __nv_bfloat16 h = __float2bfloat16_rn(hi);
  const float r = __fadd_rn(__fsub_rn(hi, __bfloat162float(h)), lo);
  const __nv_bfloat16 m = __float2bfloat16_rn(r);
  const __nv_bfloat16 l = __float2bfloat16_rn(__fsub_rn(r, __bfloat162float(m)));
  out[0] = __bfloat16_as_ushort(h);
  out[1] = __bfloat16_as_ushort(m);
  out[2] = __bfloat16_as_ushort(l);
}

// Byte offset of row `row`, K-core kc (8 reals) in a plane of tiles of `tile` rows and
// KS K-steps per tile.
__device__ __forceinline__ uint64_t plane_offset(uint64_t row, uint64_t kc, uint32_t tile, uint32_t KS) {
  const uint64_t t = row / tile, rr = row % tile;
  return (t * KS + kc / 2) * (uint64_t)(tile * K_STEP * 2) + (rr / 8) * 256 + (kc & 1) * 128 + (rr % 8) * 16;
}

// The same with the tile height as a power of two (shifts instead of divisions).
__device__ __forceinline__ uint64_t plane_offset_log2(uint64_t row, uint64_t kc, uint32_t tile_log2, uint32_t KS) {
  const uint64_t t = row >> tile_log2, rr = row & ((1ull << tile_log2) - 1);
  return ((t * KS + (kc >> 1)) << (tile_log2 + 5)) + ((rr >> 3) << 8) + ((kc & 1) << 7) + ((rr & 7) << 4);
}

// Where the pieces of an operand go.
struct Planes {
  uint8_t* base;         // PIECES planes, plane_bytes apart
  uint64_t plane_bytes;
  uint32_t tile_log2;    // rows per tile: 2^7 for A^, 2^8 for B^
  uint32_t KS;           // K-steps per tile
  int two_rows;          // 1: A^ (complex row m -> real rows 2m, 2m+1), 0: B^ (one row per column n)
};

// The pieces of complex element v at (row, complex column k): A^ rows 2m = (Re, -Im),
// 2m + 1 = (Im, Re) at reals 2k, 2k + 1; B^ row n = (Re, Im). One 4-byte store per piece
// and row.
__device__ __forceinline__ void write_pieces(const Planes& o, uint64_t row, uint64_t k, double2 v) {
  uint16_t re[PIECES], im[PIECES];
  pieces(v.x, re);
  pieces(v.y, im);
  const uint64_t kc = k >> 2, sub = (k & 3) * 4;
  if (o.two_rows) {
    const uint64_t off0 = plane_offset_log2(2 * row, kc, o.tile_log2, o.KS) + sub;
    const uint64_t off1 = plane_offset_log2(2 * row + 1, kc, o.tile_log2, o.KS) + sub;
#pragma unroll
    for (int p = 0; p < PIECES; ++p) {
      uint8_t* pl = o.base + p * o.plane_bytes;
      *reinterpret_cast<uint32_t*>(pl + off0) = (uint32_t)re[p] | ((uint32_t)(im[p] ^ 0x8000u) << 16);
      *reinterpret_cast<uint32_t*>(pl + off1) = (uint32_t)im[p] | ((uint32_t)re[p] << 16);
    }
  } else {
    const uint64_t off = plane_offset_log2(row, kc, o.tile_log2, o.KS) + sub;
#pragma unroll
    for (int p = 0; p < PIECES; ++p)
      *reinterpret_cast<uint32_t*>(o.base + p * o.plane_bytes + off) = (uint32_t)re[p] | ((uint32_t)im[p] << 16);
  }
}

// Four consecutive complex columns k .. k + 3 (k % 4 == 0) of one row: whole 16-byte
// chunks, one store per piece and row.
__device__ __forceinline__ void write_pieces4(const Planes& o, uint64_t row, uint64_t k, const double2 (&v)[4]) {
  uint16_t re[4][PIECES], im[4][PIECES];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    pieces(v[e].x, re[e]);
    pieces(v[e].y, im[e]);
  }
  const uint64_t kc = k >> 2;
  if (o.two_rows) {
    const uint64_t off0 = plane_offset_log2(2 * row, kc, o.tile_log2, o.KS);
    const uint64_t off1 = plane_offset_log2(2 * row + 1, kc, o.tile_log2, o.KS);
#pragma unroll
    for (int p = 0; p < PIECES; ++p) {
      uint32_t r0[4], r1[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        r0[e] = (uint32_t)re[e][p] | ((uint32_t)(im[e][p] ^ 0x8000u) << 16);
        r1[e] = (uint32_t)im[e][p] | ((uint32_t)re[e][p] << 16);
      }
      uint8_t* pl = o.base + p * o.plane_bytes;
      *reinterpret_cast<uint4*>(pl + off0) = make_uint4(r0[0], r0[1], r0[2], r0[3]);
      *reinterpret_cast<uint4*>(pl + off1) = make_uint4(r1[0], r1[1], r1[2], r1[3]);
    }
  } else {
    const uint64_t off = plane_offset_log2(row, kc, o.tile_log2, o.KS);
#pragma unroll
    for (int p = 0; p < PIECES; ++p) {
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) w[e] = (uint32_t)re[e][p] | ((uint32_t)im[e][p] << 16);
      *reinterpret_cast<uint4*>(o.base + p * o.plane_bytes + off) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

}  // namespace bx3
}  // namespace qtnh_impl
