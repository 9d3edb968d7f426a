// Axis permutation of complex128 tensors: Tensor::permute / Tensor::swap on one GPU.
//
// The reference moves data with MPI datatypes and MPI_Alltoallv even for a purely local
// permutation (src/tensor/dense.cpp:354-488) and swaps with per-pair std::swap,
// MPI_Scatter or MPI_Sendrecv (dense.cpp:171-274). Here all slabs are resident, so every
// case is one out-of-place transpose of a row-major array in HBM, bound by HBM
// bandwidth (algorithmic traffic 32 bytes per element: one 16-byte read, one write).
//
// Planner: drop size-1 axes, merge input-adjacent axes that stay adjacent, then pick
//   * a straight copy when the merged permutation is the identity;
//   * a run copy when the innermost axis stays innermost with >= 32 elements
//     (each contiguous run of the input is one contiguous run of the output);
//   * otherwise a tiled transpose: the tile spans the input's trailing axes (>= 32
//     contiguous elements, coalesced 128-bit loads) and the output's trailing axes
//     (>= 32 contiguous elements, coalesced 128-bit stores); a merged axis too large
//     for the tile is split into (outer, inner) parts so the tile takes only the inner
//     part it needs (e.g. an exchange of the top and bottom 3 axes of a 28-axis state:
//     dims (8, 2^22, 8) become (8, 2^20, 4, 8) and the tile is 8 x 4 x 8). The tile is
//     staged in shared memory in XOR-swizzled rows (one padding slot per row where the
//     row length is not a multiple of 8); the per-element offsets of
//     the tile come as tables in the kernel parameters (copied to shared memory), and
//     small tiles are processed several per step so that enough loads are in flight;
//   * a gather (coalesced stores, indexed loads) when no tile fits.

#include <algorithm>
#include <cstring>
#include <memory>
#include <numeric>

#include "bf16x3.cuh"
#include "cuda_common.cuh"

namespace qtnh_impl {

namespace {

constexpr int TILE_MAX = 1024;   // elements per transpose tile
constexpr int TILE_THREADS = 256;
constexpr int STEP_ELEMS = 2048;  // elements of the tiles moved per step of a block (power-of-two tiles)
constexpr int TILE_PER_THREAD = STEP_ELEMS / TILE_THREADS;
static_assert(TILE_MAX <= STEP_ELEMS, "one step holds at least one tile");


struct TileParams {
  RestDesc rest;
  int T;           // elements per tile
  int G;           // tiles per step (T is a power of two when G > 1)
  uint32_t T_log2;
  int quad;        // fused split: write order runs in aligned quads of consecutive columns
  int tile_slots;
  int64_t rin[TILE_MAX];   // read order: input offset within the tile
  int64_t wout[TILE_MAX];  // write order: output offset within the tile
  int32_t rslot[TILE_MAX];
  int32_t wslot[TILE_MAX];
};

struct RunParams {
  RestDesc rest;  // all axes but the innermost
  uint64_t L;     // run length (innermost axis)
  uint32_t L_log2;
};

__global__ void __launch_bounds__(TILE_THREADS, 4) tiled_permute_kernel(const c128* __restrict__ in, c128* __restrict__ out,
                                                                     const __grid_constant__ TileParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = p.T, G = p.G, S = p.tile_slots;
  c128* tile = reinterpret_cast<c128*>(smem_raw);  // G tiles of S slots
  uint64_t* s_bin = reinterpret_cast<uint64_t*>(tile + (size_t)G * S);
  uint64_t* s_bout = s_bin + G;
  int64_t* s_rin = reinterpret_cast<int64_t*>(s_bout + G);
  int64_t* s_wout = s_rin + T;
  int32_t* s_rslot = reinterpret_cast<int32_t*>(s_wout + T);
  int32_t* s_wslot = s_rslot + T;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    s_rin[t] = p.rin[t];
    s_wout[t] = p.wout[t];
    s_rslot[t] = p.rslot[t];
    s_wslot[t] = p.wslot[t];
  }
  const uint64_t total = p.rest.total;
  for (uint64_t r0 = (uint64_t)blockIdx.x * G; r0 < total; r0 += (uint64_t)gridDim.x * G) {
    for (int g = threadIdx.x; g < G && r0 + g < total; g += blockDim.x) {
      uint64_t bin, bout;
      decode(r0 + g, p.rest, bin, bout);
      s_bin[g] = bin;
      s_bout[g] = bout;
    }
    __syncthreads();
    const uint64_t left = total - r0;
    const int n = (left < (uint64_t)G ? (int)left : G) * T;  // <= STEP_ELEMS
    // all of this thread's loads are issued before any is stored to shared memory
    c128 v[TILE_PER_THREAD];
    int slot[TILE_PER_THREAD];
#pragma unroll
    for (int k = 0; k < TILE_PER_THREAD; ++k) {
      const int e = threadIdx.x + k * TILE_THREADS;
      if (e < n) {
        const int g = G > 1 ? e >> p.T_log2 : 0, t = G > 1 ? e & (T - 1) : e;
        slot[k] = g * S + s_rslot[t];
        v[k] = __ldg(in + s_bin[g] + s_rin[t]);
      }
    }
#pragma unroll
    for (int k = 0; k < TILE_PER_THREAD; ++k)
      if (threadIdx.x + k * TILE_THREADS < n) tile[slot[k]] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TILE_PER_THREAD; ++k) {
      const int e = threadIdx.x + k * TILE_THREADS;
      if (e < n) {
        const int g = G > 1 ? e >> p.T_log2 : 0, t = G > 1 ? e & (T - 1) : e;
        out[s_bout[g] + s_wout[t]] = tile[g * S + s_wslot[t]];
      }
    }
    __syncthreads();
  }
}

// Innermost axis fixed: copy runs of L elements. When L is a multiple of 128 every warp
// copies 128 contiguous elements (4 per lane) of a single run per step.
__global__ void __launch_bounds__(256) run_copy_kernel(const c128* __restrict__ in, c128* __restrict__ out,
                                                       const __grid_constant__ RunParams p) {
  const uint64_t N = p.rest.total * p.L;
  const int lane = threadIdx.x & 31;
  if ((p.L & 127) == 0) {
    const uint64_t nchunks = N >> 7;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t c = warp; c < nchunks; c += nwarps) {
      const uint64_t e0 = c << 7;
      uint64_t run, t0;
      if (p.L_log2 != 0xFFFFFFFFu) run = e0 >> p.L_log2, t0 = e0 & (p.L - 1);
      else run = e0 / p.L, t0 = e0 % p.L;
      uint64_t bin, bout;
      decode(run, p.rest, bin, bout);
      const c128* src = in + bin + t0;
      c128* dst = out + bout + t0;
      c128 v0 = __ldg(src + lane), v1 = __ldg(src + lane + 32), v2 = __ldg(src + lane + 64), v3 = __ldg(src + lane + 96);
      dst[lane] = v0;
      dst[lane + 32] = v1;
      dst[lane + 64] = v2;
      dst[lane + 96] = v3;
    }
  } else {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < N; e += (uint64_t)gridDim.x * blockDim.x) {
      uint64_t run, t;
      if (p.L_log2 != 0xFFFFFFFFu) run = e >> p.L_log2, t = e & (p.L - 1);
      else run = e / p.L, t = e % p.L;
      uint64_t bin, bout;
      decode(run, p.rest, bin, bout);
      out[bout + t] = __ldg(in + bin + t);
    }
  }
}

// Fallback: one thread per output element; axes in output order with input strides.
__global__ void __launch_bounds__(256) gather_permute_kernel(const c128* __restrict__ in, c128* __restrict__ out,
                                                             const __grid_constant__ RestDesc p) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < p.total; e += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t src, unused;
    decode(e, p, src, unused);
    out[e] = __ldg(in + src);
  }
}

// Fused permute and split (the split-precision GEMM's operands): the same transpose, but
// each element is written as its bf16 pieces into the GEMM's operand planes at (row, k).
// Software-pipelined over two tile buffers: the elements of step j + 1 travel global ->
// shared by cp.async while the block converts and writes step j, so the loads stay in
// flight through the piece arithmetic and the scattered plane stores. The bases of the
// tiles of a step are decoded two steps ahead into one of three slots. A thread handles
// the same positions of the step's tiles at every step, so it keeps their table entries
// (slots and offsets) in registers. QUAD: write order in aligned quads of consecutive
// columns (whole 16-byte chunks per piece and row).
template <bool QUAD>
__global__ void __launch_bounds__(TILE_THREADS, 2) tiled_split_kernel(const c128* __restrict__ in,
                                                                      const __grid_constant__ TileParams p,
                                                                      const bx3::Planes o) {
  constexpr int WPT = QUAD ? STEP_ELEMS / (4 * TILE_THREADS) : TILE_PER_THREAD;  // writes per thread and step
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = p.T, G = p.G, S = p.tile_slots, GS = G * S;
  c128* tile = reinterpret_cast<c128*>(smem_raw);  // two buffers of G tiles of S slots
  uint64_t* s_bin = reinterpret_cast<uint64_t*>(tile + 2 * (size_t)GS);  // [3][G]
  uint64_t* s_bout = s_bin + 3 * G;                                      // [3][G]
  int64_t* s_rin = reinterpret_cast<int64_t*>(s_bout + 3 * G);
  int64_t* s_wout = s_rin + T;
  int32_t* s_rslot = reinterpret_cast<int32_t*>(s_wout + T);
  int32_t* s_wslot = s_rslot + T;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    s_rin[t] = p.rin[t];
    s_wout[t] = p.wout[t];
    s_rslot[t] = p.rslot[t];
    s_wslot[t] = p.wslot[t];
  }
  const uint64_t total = p.rest.total;
  const uint64_t first = (uint64_t)blockIdx.x * G, stride = (uint64_t)gridDim.x * G;
  auto elems = [&](uint64_t r0) {  // elements of the step starting at tile r0 (<= STEP_ELEMS)
    const uint64_t left = total - r0;
    return (left < (uint64_t)G ? (int)left : G) * T;
  };
  auto tile_of = [&](int e) { return G > 1 ? e >> p.T_log2 : 0; };
  auto pos_of = [&](int e) { return G > 1 ? (e & (T - 1)) : e; };
  auto decode_step = [&](uint64_t r0, int q) {
    for (int g = threadIdx.x; g < G && r0 + g < total; g += blockDim.x) {
      uint64_t bin, bout;
      decode(r0 + g, p.rest, bin, bout);
      s_bin[q * G + g] = bin;
      s_bout[q * G + g] = bout;
    }
  };
  decode_step(first, 0);
  decode_step(first + stride, 1);
  __syncthreads();  // tables and the bases of the first two steps
  // this thread's table entries (positions past a full step are never used)
  const int full = G * T;
  int32_t rslot[TILE_PER_THREAD];
  int64_t rin[TILE_PER_THREAD];
#pragma unroll
  for (int k = 0; k < TILE_PER_THREAD; ++k) {
    const int e = threadIdx.x + k * TILE_THREADS;
    const int t = pos_of(e < full ? e : 0);
    rslot[k] = tile_of(e) * S + s_rslot[t];
    rin[k] = s_rin[t];
  }
  int32_t wslot[WPT][QUAD ? 4 : 1];
  int64_t wout[WPT];
#pragma unroll
  for (int i = 0; i < WPT; ++i) {
    const int e = QUAD ? 4 * threadIdx.x + i * 4 * TILE_THREADS : threadIdx.x + i * TILE_THREADS;
    const int t = pos_of(e < full ? e : 0);
#pragma unroll
    for (int x = 0; x < (QUAD ? 4 : 1); ++x) wslot[i][x] = tile_of(e) * S + s_wslot[t + x];
    wout[i] = s_wout[t];
  }
  auto issue = [&](uint64_t r0, int q, c128* buf) {
    if (r0 < total) {
      const int n = elems(r0);
#pragma unroll
      for (int k = 0; k < TILE_PER_THREAD; ++k) {
        const int e = threadIdx.x + k * TILE_THREADS;
        if (e < n) cp_async16(&buf[rslot[k]], in + s_bin[q * G + tile_of(e)] + rin[k]);
      }
    }
    cp_async_commit();  // one group per step (empty past the end), so wait_group 1 is exact
  };
  issue(first, 0, tile);
  int j = 0;
  for (uint64_t r0 = first; r0 < total; r0 += stride, ++j) {
    const c128* cur = tile + (size_t)(j & 1) * GS;
    const uint64_t* bout = s_bout + (j % 3) * G;
    issue(r0 + stride, (j + 1) % 3, tile + (size_t)((j + 1) & 1) * GS);
    cp_async_wait_one();  // this thread's copies of step j have landed
    __syncthreads();      // and everyone's
    decode_step(r0 + 2 * stride, (j + 2) % 3);
    const int n = elems(r0);
#pragma unroll
    for (int i = 0; i < WPT; ++i) {
      const int e = QUAD ? 4 * threadIdx.x + i * 4 * TILE_THREADS : threadIdx.x + i * TILE_THREADS;
      if (e < n) {
        const uint64_t rk = bout[tile_of(e)] + (uint64_t)wout[i];  // (row << 32) + k
        if (QUAD) {
          double2 v[4];
#pragma unroll
          for (int x = 0; x < 4; ++x) v[x] = cur[wslot[i][QUAD ? x : 0]];
          bx3::write_pieces4(o, rk >> 32, rk & 0xFFFFFFFFull, v);
        } else {
          bx3::write_pieces(o, rk >> 32, rk & 0xFFFFFFFFull, cur[wslot[i][0]]);
        }
      }
    }
    __syncthreads();  // buffer j & 1 and base slot j % 3 are free again
  }
  cp_async_wait_all();
}

// Fused fallback: one thread per element in output order.
__global__ void __launch_bounds__(256) gather_split_kernel(const c128* __restrict__ in, const __grid_constant__ RestDesc p,
                                                           const bx3::Planes o) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < p.total; e += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t src, rk;
    decode(e, p, src, rk);
    bx3::write_pieces(o, rk >> 32, rk & 0xFFFFFFFFull, __ldg(in + src));
  }
}

// Zeros of the padding of an operand's planes: rows in [rows, rows_pad) and complex
// columns in [K, Kp) (K-core granularity 4 columns, one 4-byte slot per column).
__global__ void __launch_bounds__(256) pad_planes_kernel(bx3::Planes o, uint64_t rows, uint64_t rows_pad, uint64_t K,
                                                         uint64_t kcs) {
  // items: (row < rows, kc in [K / 4, kcs)) then (row in [rows, rows_pad), every kc)
  const uint64_t kc0 = K / 4, n1 = rows * (kcs - kc0), n2 = (rows_pad - rows) * kcs;
  const int prow = o.two_rows ? 2 : 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n1 + n2; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t row, kc;
    if (i < n1) row = i / (kcs - kc0), kc = kc0 + i % (kcs - kc0);
    else row = rows + (i - n1) / kcs, kc = (i - n1) % kcs;
    for (int sub = 0; sub < 4; ++sub) {
      const uint64_t k = kc * 4 + sub;
      if (row < rows && k < K) continue;
      for (int rr = 0; rr < prow; ++rr) {
        const uint64_t off = bx3::plane_offset_log2(prow * row + rr, kc, o.tile_log2, o.KS) + 4 * sub;
        for (int pc = 0; pc < bx3::PIECES; ++pc) *reinterpret_cast<uint32_t*>(o.base + pc * o.plane_bytes + off) = 0u;
      }
    }
  }
}

struct Canon {
  dims_t dims;            // merged input dims
  std::vector<int> ptup;  // merged axis -> new position
  std::vector<char> row;  // fused split: the axis is one of the output's row axes
};

// Drops size-1 axes and merges input-adjacent axes that stay adjacent in the output;
// with boundary >= 0 (fused split), output positions below it are row axes and no merge
// crosses from a row axis to a column axis.
Canon canonicalise(const dims_t& dims, const std::vector<uint16_t>& ptup, int boundary) {
  std::vector<int> keep;
  for (size_t i = 0; i < dims.size(); ++i)
    if (dims[i] > 1) keep.push_back((int)i);
  std::vector<int> order(keep.size());
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int x, int y) { return ptup[keep[x]] < ptup[keep[y]]; });
  std::vector<int> kp(keep.size());
  for (size_t j = 0; j < order.size(); ++j) kp[order[j]] = (int)j;
  auto is_row = [&](size_t x) { return boundary >= 0 && (int)ptup[keep[x]] < boundary; };
  dims_t gd;
  std::vector<int> gp;
  std::vector<char> gr;
  for (size_t x = 0; x < keep.size(); ++x) {
    if (x > 0 && kp[x] == kp[x - 1] + 1 && is_row(x) == is_row(x - 1)) {
      gd.back() *= dims[keep[x]];
    } else {
      gd.push_back(dims[keep[x]]);
      gp.push_back(kp[x]);
      gr.push_back(is_row(x) ? 1 : 0);
    }
  }
  std::vector<int> go(gd.size());
  std::iota(go.begin(), go.end(), 0);
  std::sort(go.begin(), go.end(), [&](int x, int y) { return gp[x] < gp[y]; });
  Canon c;
  c.dims = gd;
  c.row = gr;
  c.ptup.assign(gd.size(), 0);
  for (size_t j = 0; j < go.size(); ++j) c.ptup[go[j]] = (int)j;
  return c;
}

// Splits merged axis i into (dims[i] / lo, lo); the two parts stay adjacent, in this
// order, in the input and in the output.
void split_axis(Canon& c, int i, uint64_t lo) {
  const int P = c.ptup[i];
  for (auto& x : c.ptup)
    if (x > P) ++x;
  c.dims[i] /= lo;
  c.dims.insert(c.dims.begin() + i + 1, lo);
  c.ptup.insert(c.ptup.begin() + i + 1, P + 1);
  c.row.insert(c.row.begin() + i + 1, c.row[i]);
}

// Smallest divisor f of d with want <= f <= TILE_MAX and f < d, or 0.
uint64_t inner_factor(uint64_t d, uint64_t want) {
  for (uint64_t f = std::max<uint64_t>(want, 2); f <= (uint64_t)TILE_MAX && f < d; ++f)
    if (d % f == 0) return f;
  return 0;
}

struct Plan {
  enum Kind { COPY, RUN, TILED, GATHER } kind = COPY;
  std::unique_ptr<TileParams> tile;  // ~25 KB, passed by value to the launch
  size_t smem = 0;
  int grid = 0;
  RunParams run;
  RestDesc gather;
};

// The launch plan of a permutation. boundary < 0: plain permute (output offsets are
// element offsets; copy and run-copy shortcuts). boundary >= 0: fused split (output
// "offsets" are (row << 32) + k with rows over the output positions below the boundary
// and k over the rest, each row-major; only the tiled and gather forms).
Plan plan_permute(const dims_t& dims, const std::vector<uint16_t>& ptup, int boundary) {
  const uint64_t N = product(dims);
  Canon c = canonicalise(dims, ptup, boundary);
  if ((int)c.dims.size() > KMAX) throw Error(QTNH_ERR_UNSUPPORTED, "too many non-trivial axes");
  Plan plan;
  if (boundary < 0 && c.dims.size() <= 1) {
    plan.kind = Plan::COPY;
    return plan;
  }
  if (c.dims.empty()) {  // a single element (fused): one gather step
    c.dims.push_back(1);
    c.ptup.push_back(0);
    c.row.push_back(boundary > 0 ? 1 : 0);
  }
  // output strides: plain, or packed (row << 32) + k
  auto out_strides = [&](int r) {
    dims_t nd(r), os(r);
    for (int i = 0; i < r; ++i) nd[c.ptup[i]] = c.dims[i];
    if (boundary < 0) {
      dims_t ns = row_strides(nd);
      for (int i = 0; i < r; ++i) os[i] = ns[c.ptup[i]];
      return os;
    }
    std::vector<char> prow(r);
    for (int i = 0; i < r; ++i) prow[c.ptup[i]] = c.row[i];
    dims_t ns(r);
    uint64_t rs = 1, ks = 1;
    for (int j = r - 1; j >= 0; --j) {
      if (prow[j]) ns[j] = rs << 32, rs *= nd[j];
      else ns[j] = ks, ks *= nd[j];
    }
    for (int i = 0; i < r; ++i) os[i] = ns[c.ptup[i]];
    return os;
  };
  // Run copy.
  if (boundary < 0 && c.ptup.back() == (int)c.dims.size() - 1 && c.dims.back() >= 32) {
    const int r = (int)c.dims.size();
    dims_t in_stride = row_strides(c.dims), os = out_strides(r);
    plan.kind = Plan::RUN;
    plan.run.L = c.dims[r - 1];
    plan.run.L_log2 = log2_or_none(plan.run.L);
    plan.run.rest.n = r - 1;
    plan.run.rest.total = N / plan.run.L;
    for (int i = 0; i < r - 1; ++i) fill_axis(plan.run.rest.ax[i], c.dims[i], in_stride[i], os[i]);
    plan.grid = grid_for((N + 1023) / 1024, 16);
    return plan;
  }

  // Tiled transpose: A = the input's trailing axes (>= 32 contiguous input elements), B =
  // further axes completing the output's trailing run (>= 32 contiguous output elements).
  // A merged axis that would overflow the tile is split and the plan restarts.
  int r = 0;
  dims_t in_stride, new_dims, out_stride;
  std::vector<int> inv, A, B;
  std::vector<char> inA, inB;
  uint64_t PA = 1, PB = 1;
  bool tiled = false;
  for (int attempt = 0; attempt <= KMAX; ++attempt) {
    r = (int)c.dims.size();
    in_stride = row_strides(c.dims);
    new_dims.assign(r, 0);
    for (int i = 0; i < r; ++i) new_dims[c.ptup[i]] = c.dims[i];
    out_stride = out_strides(r);
    inv.assign(r, 0);
    for (int i = 0; i < r; ++i) inv[c.ptup[i]] = i;
    A.clear();
    B.clear();
    inA.assign(r, 0);
    inB.assign(r, 0);
    PA = 1;
    PB = 1;
    const bool may_split = r < KMAX;
    bool restart = false;
    for (int i = r - 1; i >= 0 && PA < 32; --i) {
      if (PA * c.dims[i] > 64 && may_split) {
        const uint64_t f = inner_factor(c.dims[i], (32 + PA - 1) / PA);
        if (f) {
          split_axis(c, i, f);
          restart = true;
          break;
        }
      }
      A.push_back(i), PA *= c.dims[i], inA[i] = 1;
    }
    if (restart) continue;
    tiled = PA <= (uint64_t)TILE_MAX;
    if (!tiled) break;
    uint64_t run = 1;
    for (int j = r - 1; j >= 0 && run < 32; --j) {
      const int i = inv[j];
      if (inA[i]) {
        run *= c.dims[i];
        continue;
      }
      if (PA * PB * c.dims[i] > (uint64_t)TILE_MAX) {
        const uint64_t f = may_split ? inner_factor(c.dims[i], (32 + run - 1) / run) : 0;
        if (f && PA * PB * f <= (uint64_t)TILE_MAX) {
          split_axis(c, i, f);
          restart = true;
        }
        break;
      }
      B.push_back(i), PB *= c.dims[i], inB[i] = 1, run *= c.dims[i];
    }
    if (!restart) break;
  }
  if (tiled) {
    std::sort(A.begin(), A.end());
    std::sort(B.begin(), B.end());
    plan.kind = Plan::TILED;
    plan.tile.reset(new TileParams());
    TileParams& p = *plan.tile;
    const int T = (int)(PA * PB);
    p.T = T;
    // Shared-memory slot of tile element (a, b), a over the input-contiguous axes. With PA
    // a multiple of 8, rows are unpadded and the 16-byte slot within each aligned group of
    // 8 is XOR-swizzled by b ^ (b >> 2): consecutive a (the loads), consecutive b (the
    // single-element writes) and b = 4j + x over j (the quad writes: lane j reads column
    // x of its quad) each hit the 8 bank groups once per 8 lanes. Else one padding slot
    // per row.
    const bool swz = PA % 8 == 0;
    auto slot_of = [&](uint64_t a, uint64_t b) {
      return swz ? (int32_t)(b * PA + (a ^ ((b ^ (b >> 2)) & 7))) : (int32_t)(b * (PA + 1) + a);
    };
    p.tile_slots = (int)(swz ? PB * PA : PB * (PA + 1));
    const uint32_t tl = log2_or_none((uint64_t)T);
    p.G = (tl != 0xFFFFFFFFu && T < STEP_ELEMS) ? std::min(STEP_ELEMS / T, 256) : 1;
    p.T_log2 = tl == 0xFFFFFFFFu ? 0 : tl;
    // fused split: the tile's trailing output positions that are column axes form a run
    // of consecutive columns (stride 1 innermost); if its length is a multiple of 4,
    // write order goes in aligned quads (every other axis strides by multiples of it)
    p.quad = 0;
    if (boundary >= 0) {
      uint64_t run = 1;
      for (int j = r - 1; j >= 0; --j) {
        const int i = inv[j];
        if (!(inA[i] || inB[i]) || c.row[i]) break;
        run *= c.dims[i];
      }
      p.quad = (run % 4 == 0) ? 1 : 0;
    }
    // Row-major multipliers over A and B (input order).
    auto mults = [&](const std::vector<int>& axes) {
      std::vector<uint64_t> m(axes.size(), 1);
      for (int k = (int)axes.size() - 2; k >= 0; --k) m[k] = m[k + 1] * c.dims[axes[k + 1]];
      return m;
    };
    auto mA = mults(A), mB = mults(B);
    // Read order: t = b * PA + a.
    for (uint64_t b = 0; b < PB; ++b) {
      uint64_t offb = 0, rem = b;
      for (int k = (int)B.size() - 1; k >= 0; --k) {
        uint64_t d = rem % c.dims[B[k]];
        rem /= c.dims[B[k]];
        offb += d * in_stride[B[k]];
      }
      for (uint64_t a = 0; a < PA; ++a) {
        uint64_t offa = 0, ra = a;
        for (int k = (int)A.size() - 1; k >= 0; --k) {
          uint64_t d = ra % c.dims[A[k]];
          ra /= c.dims[A[k]];
          offa += d * in_stride[A[k]];
        }
        int t = (int)(b * PA + a);
        p.rin[t] = (int64_t)(offa + offb);
        p.rslot[t] = slot_of(a, b);
      }
    }
    // Write order: tile axes by output position, row-major.
    std::vector<int> tax(A);
    tax.insert(tax.end(), B.begin(), B.end());
    std::sort(tax.begin(), tax.end(), [&](int x, int y) { return c.ptup[x] < c.ptup[y]; });
    for (int w = 0; w < T; ++w) {
      uint64_t rem = (uint64_t)w, off = 0, a = 0, b = 0;
      for (int k = (int)tax.size() - 1; k >= 0; --k) {
        int i = tax[k];
        uint64_t d = rem % c.dims[i];
        rem /= c.dims[i];
        off += d * out_stride[i];
        if (inA[i]) a += d * mA[std::find(A.begin(), A.end(), i) - A.begin()];
        else b += d * mB[std::find(B.begin(), B.end(), i) - B.begin()];
      }
      p.wout[w] = (int64_t)off;
      p.wslot[w] = slot_of(a, b);
    }
    int nr = 0;
    for (int i = 0; i < r; ++i)
      if (!inA[i] && !inB[i]) fill_axis(p.rest.ax[nr++], c.dims[i], in_stride[i], out_stride[i]);
    p.rest.n = nr;
    p.rest.total = N / (uint64_t)T;
    // the fused split double-buffers its tiles and keeps three slots of tile bases
    const size_t nbuf = boundary >= 0 ? 2 : 1, nbase = boundary >= 0 ? 3 : 1;
    plan.smem = nbuf * (size_t)p.G * p.tile_slots * sizeof(c128) + 2 * nbase * (size_t)p.G * sizeof(uint64_t) +
                (size_t)T * (2 * sizeof(int64_t) + 2 * sizeof(int32_t));
    // as many blocks per SM as shared memory and registers allow (at most 4)
    const int per_sm = (int)std::max<size_t>(1, std::min<size_t>(4, (220 * 1024) / (plan.smem + 1024)));
    plan.grid = grid_for((p.rest.total + p.G - 1) / p.G, per_sm);
    return plan;
  }

  // Gather fallback: axes in output order, input strides (and output strides).
  plan.kind = Plan::GATHER;
  plan.gather.n = r;
  plan.gather.total = N;
  for (int j = 0; j < r; ++j) fill_axis(plan.gather.ax[j], new_dims[j], in_stride[inv[j]], out_stride[inv[j]]);
  plan.grid = grid_for((N + 255) / 256, 16);
  return plan;
}

void check_permutation(const dims_t& dims, const std::vector<uint16_t>& ptup) {
  const size_t r0 = dims.size();
  if (ptup.size() != r0) throw Error(QTNH_ERR_INVALID_ARGUMENT, "permutation tuple size differs from tensor rank");
  std::vector<char> seen(r0, 0);
  for (auto p : ptup) {
    if (p >= r0 || seen[p]) throw Error(QTNH_ERR_INVALID_ARGUMENT, "permutation tuple is not a permutation");
    seen[p] = 1;
  }
}

}  // namespace

void permute_device(const void* in_v, void* out_v, const dims_t& dims, const std::vector<uint16_t>& ptup, void* stream) {
  check_permutation(dims, ptup);
  const uint64_t N = product(dims);
  if (N == 0) return;
  cudaStream_t s = (cudaStream_t)stream;
  const c128* in = static_cast<const c128*>(in_v);
  c128* out = static_cast<c128*>(out_v);
  Plan plan = plan_permute(dims, ptup, -1);
  switch (plan.kind) {
    case Plan::COPY:
      check_cuda(cudaMemcpyAsync(out, in, N * sizeof(c128), cudaMemcpyDeviceToDevice, s), "permute copy");
      return;
    case Plan::RUN:
      run_copy_kernel<<<plan.grid, 256, 0, s>>>(in, out, plan.run);
      count_launch();
      check_cuda(cudaGetLastError(), "run_copy_kernel launch");
      return;
    case Plan::TILED:
      if (plan.smem > 48 * 1024)
        check_cuda(cudaFuncSetAttribute(tiled_permute_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)plan.smem),
                   "tiled_permute_kernel shared memory");
      tiled_permute_kernel<<<plan.grid, TILE_THREADS, plan.smem, s>>>(in, out, *plan.tile);
      count_launch();
      check_cuda(cudaGetLastError(), "tiled_permute_kernel launch");
      return;
    case Plan::GATHER:
      gather_permute_kernel<<<plan.grid, 256, 0, s>>>(in, out, plan.gather);
      count_launch();
      check_cuda(cudaGetLastError(), "gather_permute_kernel launch");
      return;
  }
}

void permute_split_device(const void* in_v, const dims_t& dims, const std::vector<uint16_t>& ptup, int nrow_axes,
                          uint64_t rows, uint64_t rows_pad, uint64_t K, uint64_t kcs, uint8_t* planes,
                          uint64_t plane_bytes, uint32_t tile_rows, uint32_t KS, bool two_rows, void* stream) {
  check_permutation(dims, ptup);
  cudaStream_t s = (cudaStream_t)stream;
  const c128* in = static_cast<const c128*>(in_v);
  if (tile_rows != 128 && tile_rows != 256) throw Error(QTNH_ERR_UNSUPPORTED, "operand tile height");
  bx3::Planes o{planes, plane_bytes, tile_rows == 128 ? 7u : 8u, KS, two_rows ? 1 : 0};
  if (rows_pad > rows || kcs * 4 > K) {
    const uint64_t items = rows * (kcs - K / 4) + (rows_pad - rows) * kcs;
    pad_planes_kernel<<<grid_for((items + 255) / 256, 8), 256, 0, s>>>(o, rows, rows_pad, K, kcs);
    count_launch();
  }
  if (product(dims) == 0) return;
  Plan plan = plan_permute(dims, ptup, nrow_axes);
  if (plan.kind == Plan::TILED) {
    if (plan.smem > 48 * 1024) {
      check_cuda(cudaFuncSetAttribute(tiled_split_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)plan.smem),
                 "tiled_split_kernel shared memory");
      check_cuda(cudaFuncSetAttribute(tiled_split_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)plan.smem),
                 "tiled_split_kernel shared memory");
    }
    if (plan.tile->quad)
      tiled_split_kernel<true><<<plan.grid, TILE_THREADS, plan.smem, s>>>(in, *plan.tile, o);
    else
      tiled_split_kernel<false><<<plan.grid, TILE_THREADS, plan.smem, s>>>(in, *plan.tile, o);
  } else {
    gather_split_kernel<<<plan.grid, 256, 0, s>>>(in, plan.gather, o);
  }
  count_launch();
  check_cuda(cudaGetLastError(), "permute-split launch");
}

}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" {

int qtnh_permute(const void* in, void* out, int32_t rank, const uint64_t* dims, const uint16_t* ptup, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank < 0 || rank > QTNH_MAX_RANK) throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    permute_device(in, out, dims_t(dims, dims + rank), std::vector<uint16_t>(ptup, ptup + rank), stream);
    return QTNH_OK;
  });
}

int qtnh_swap(const void* in, void* out, int32_t rank, const uint64_t* dims, int32_t idx1, int32_t idx2, void* stream) {
  return QTNH_API([&]() -> int {
    if (rank < 0 || rank > QTNH_MAX_RANK) throw Error(QTNH_ERR_INVALID_ARGUMENT, "rank out of range");
    if (idx1 < 0 || idx2 < 0 || idx1 >= rank || idx2 >= rank) throw Error(QTNH_ERR_OUT_OF_RANGE, "swap index out of range");
    if (dims[idx1] != dims[idx2]) throw Error(QTNH_ERR_RUNTIME, "Asymmetric swaps are currently not allowed");
    std::vector<uint16_t> ptup(rank);
    std::iota(ptup.begin(), ptup.end(), 0);
    std::swap(ptup[idx1], ptup[idx2]);
    permute_device(in, out, dims_t(dims, dims + rank), ptup, stream);
    return QTNH_OK;
  });
}

}  // extern "C"
