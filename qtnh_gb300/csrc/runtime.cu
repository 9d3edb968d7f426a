// Library runtime: error reporting, device memory, copies, stream helpers, FP64 norm.
//
// Replaces the reference's QTNHEnv/MPI plumbing (src/core/env.cpp:9-29): one process
// drives one GPU, tensors live in HBM, and every former MPI exchange is a device
// operation on a caller-supplied stream.

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "cuda_common.cuh"
#include "df32.cuh"

namespace qtnh_impl {

static thread_local std::string g_last_error = "";
std::atomic<uint64_t> g_launches{0};

void set_last_error(const std::string& msg) { g_last_error = msg; }

static std::atomic<int> g_arith{-1};

int arithmetic_mode() {
  int m = g_arith.load(std::memory_order_relaxed);
  if (m < 0) {
    const char* e = std::getenv("QTNH_ARITH");
    m = QTNH_ARITH_BF16X6;
    if (e && std::strcmp(e, "fp64") == 0) m = QTNH_ARITH_FP64;
    if (e && std::strcmp(e, "f32x2") == 0) m = QTNH_ARITH_F32X2;
    g_arith.store(m);
  }
  return m;
}

static std::atomic<int> g_gemm{-1};

int gemm_mode() {
  int m = g_gemm.load(std::memory_order_relaxed);
  if (m < 0) {
    const char* e = std::getenv("QTNH_GEMM");
    m = QTNH_GEMM_OZ6;
    if (e && std::strcmp(e, "bf16x3") == 0) m = QTNH_GEMM_BF16X3;
    if (e && std::strcmp(e, "fp64") == 0) m = QTNH_GEMM_FP64;
    g_gemm.store(m);
  }
  return m;
}

static std::atomic<int> g_gemm_slice{0};

int gemm_slice_steps() {
  int k = g_gemm_slice.load(std::memory_order_relaxed);
  if (k <= 0) {
    const char* e = std::getenv("QTNH_GEMM_SLICE");
    k = e ? std::atoi(e) : 0;
    if (k < 1 || k > QTNH_GEMM_SLICE_MAX) k = QTNH_GEMM_SLICE_DEFAULT;
    g_gemm_slice.store(k);
  }
  return k;
}

int status_from_current_exception() {
  try {
    throw;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc& e) {
    set_last_error("host allocation failed");
    return QTNH_ERR_NO_MEMORY;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return QTNH_ERR_RUNTIME;
  } catch (...) {
    set_last_error("unknown error");
    return QTNH_ERR_RUNTIME;
  }
}

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    if (e == cudaErrorMemoryAllocation) throw Error(QTNH_ERR_NO_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    throw Error(QTNH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

static std::atomic<uint64_t> g_workspace_allocs{0};

// The workspace comes from the device's default stream-ordered pool. By default the pool
// returns freed memory to the device at every synchronization, so the next large
// workspace maps physical memory again (milliseconds per GB); the engine lets the pool
// keep up to an eighth of the device memory (at most 32 GiB) cached instead, set once per
// device on its first workspace.
static void keep_pool_memory() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 0 || dev >= 64 || done[dev]) return;
  done[dev] = true;
  size_t free_b = 0, total_b = 0;
  check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  cudaMemPool_t pool;
  check_cuda(cudaDeviceGetDefaultMemPool(&pool, dev), "cudaDeviceGetDefaultMemPool");
  unsigned long long keep = std::min<unsigned long long>(total_b / 8, 32ull << 30);
  check_cuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
}

void* workspace_alloc(size_t bytes, void* stream) {
  if (bytes == 0) return nullptr;
  keep_pool_memory();
  g_workspace_allocs.fetch_add(1, std::memory_order_relaxed);
  void* p = nullptr;
  check_cuda(cudaMallocAsync(&p, bytes, (cudaStream_t)stream), "cudaMallocAsync");
  return p;
}

void workspace_free(void* p, void* stream) {
  if (p) check_cuda(cudaFreeAsync(p, (cudaStream_t)stream), "cudaFreeAsync");
}

// A square added to a float-float accumulator (fs, fc): x = h + l split exactly, x^2 =
// h^2 (product and its exact FMA error) + 2 h l (the l^2 term, below 2^-48 of x^2, is left
// out).
__device__ __forceinline__ void ff_square_add(df::dwords w, float& fs, float& fc) {
  const df::f2 a = df::split(w);
  const float p = df::mul(a.h, a.h);
  float e = df::fma(a.h, a.h, -p);
  e = df::fma(df::add(a.h, a.h), a.l, e);
  float t, err;
  df::two_sum(fs, p, t, err);
  fs = t;
  fc = df::add(fc, df::add(err, e));
}

// Sum of |x|^2 to FP64 accuracy: grid-stride partial sums, one atomic per block. Of a
// thread's four elements per step, two are squared with FP64 FMAs and two as exact
// float-float squares (a warp with an element outside the float-float range takes FP64
// for them), so that the FP64 unit does half of the work and the FP32 pipes the rest:
// FP64 alone caps this read-only stream at about half of the HBM rate on GB300.
__global__ void norm2_kernel(const double2* __restrict__ x, uint64_t n, double* __restrict__ acc) {
  // four elements per thread per step, loads first, independent accumulators
  double s = 0.0, s2 = 0.0;
  float fs = 0.0f, fc = 0.0f;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x * 4;
  for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x * 4 + threadIdx.x; b < n; b += step) {
    double2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint64_t i = b + (uint64_t)u * blockDim.x;
      v[u] = i < n ? x[i] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      s = fma(v[u].x, v[u].x, s);
      s2 = fma(v[u].y, v[u].y, s2);
    }
#pragma unroll
    for (int u = 2; u < 4; ++u) {
      const df::dwords wx = df::words(v[u].x), wy = df::words(v[u].y);
      if (__all_sync(__activemask(), df::in_range_state(wx) && df::in_range_state(wy))) {
        ff_square_add(wx, fs, fc);
        ff_square_add(wy, fs, fc);
      } else {
        s = fma(v[u].x, v[u].x, s);
        s2 = fma(v[u].y, v[u].y, s2);
      }
    }
  }
  s += s2 + ((double)fs + (double)fc);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ double ws[32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) ws[warp] = s;
  __syncthreads();
  if (warp == 0) {
    s = (lane < (int)(blockDim.x >> 5)) ? ws[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) atomicAdd(acc, s);
  }
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  }
  return n;
}

}  // namespace qtnh_impl

using namespace qtnh_impl;

extern "C" {

const char* qtnh_last_error(void) { return g_last_error.c_str(); }
int qtnh_abi_version(void) { return QTNH_ABI_VERSION; }
uint64_t qtnh_kernel_launch_count(void) { return g_launches.load(); }

int qtnh_set_arithmetic(int mode) {
  return QTNH_API([&]() -> int {
    if (mode != QTNH_ARITH_FP64 && mode != QTNH_ARITH_F32X2 && mode != QTNH_ARITH_BF16X6) throw Error(QTNH_ERR_INVALID_ARGUMENT, "unknown arithmetic mode");
    g_arith.store(mode);
    return QTNH_OK;
  });
}

int qtnh_get_arithmetic(void) { return arithmetic_mode(); }

int qtnh_set_gemm_precision(int mode) {
  return QTNH_API([&]() -> int {
    if (mode != QTNH_GEMM_FP64 && mode != QTNH_GEMM_BF16X3 && mode != QTNH_GEMM_OZ6)
      throw Error(QTNH_ERR_INVALID_ARGUMENT, "unknown GEMM precision");
    g_gemm.store(mode);
    return QTNH_OK;
  });
}

int qtnh_get_gemm_precision(void) { return gemm_mode(); }

int qtnh_set_gemm_slice(int k_steps) {
  return QTNH_API([&]() -> int {
    if (k_steps < 1 || k_steps > QTNH_GEMM_SLICE_MAX) throw Error(QTNH_ERR_INVALID_ARGUMENT, "slice length out of range");
    g_gemm_slice.store(k_steps);
    return QTNH_OK;
  });
}

int qtnh_get_gemm_slice(void) { return gemm_slice_steps(); }

int qtnh_device_count(int* count) {
  return QTNH_API([&]() -> int {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) n = 0, cudaGetLastError();
    *count = n;
    return QTNH_OK;
  });
}

int qtnh_set_device(int device) {
  return QTNH_API([&]() -> int {
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    return QTNH_OK;
  });
}

int qtnh_malloc(void** ptr, size_t bytes) {
  return QTNH_API([&]() -> int {
    *ptr = nullptr;
    if (bytes == 0) bytes = 16;
    check_cuda(cudaMalloc(ptr, bytes), "cudaMalloc");
    return QTNH_OK;
  });
}

int qtnh_free(void* ptr) {
  return QTNH_API([&]() -> int {
    if (ptr) check_cuda(cudaFree(ptr), "cudaFree");
    return QTNH_OK;
  });
}

int qtnh_memcpy_h2d(void* dst, const void* src_host, size_t bytes, void* stream) {
  return QTNH_API([&]() -> int {
    if (bytes) check_cuda(cudaMemcpyAsync(dst, src_host, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream), "h2d copy");
    return QTNH_OK;
  });
}

int qtnh_memcpy_d2h(void* dst_host, const void* src, size_t bytes, void* stream) {
  return QTNH_API([&]() -> int {
    if (bytes) check_cuda(cudaMemcpyAsync(dst_host, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream), "d2h copy");
    return QTNH_OK;
  });
}

int qtnh_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream) {
  return QTNH_API([&]() -> int {
    if (bytes) check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream), "d2d copy");
    return QTNH_OK;
  });
}

int qtnh_memset(void* dst, int value, size_t bytes, void* stream) {
  return QTNH_API([&]() -> int {
    if (bytes) check_cuda(cudaMemsetAsync(dst, value, bytes, (cudaStream_t)stream), "memset");
    return QTNH_OK;
  });
}

int qtnh_stream_synchronize(void* stream) {
  return QTNH_API([&]() -> int {
    check_cuda(cudaStreamSynchronize((cudaStream_t)stream), "stream synchronize");
    return QTNH_OK;
  });
}

int qtnh_device_synchronize(void) {
  return QTNH_API([&]() -> int {
    check_cuda(cudaDeviceSynchronize(), "device synchronize");
    return QTNH_OK;
  });
}

int qtnh_stream_create(void** stream) {
  return QTNH_API([&]() -> int {
    cudaStream_t s = nullptr;
    check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    *stream = (void*)s;
    return QTNH_OK;
  });
}

int qtnh_stream_destroy(void* stream) {
  return QTNH_API([&]() -> int {
    if (stream) check_cuda(cudaStreamDestroy((cudaStream_t)stream), "cudaStreamDestroy");
    return QTNH_OK;
  });
}

int qtnh_workspace_stats(uint64_t* allocations, uint64_t* pool_used_bytes) {
  return QTNH_API([&]() -> int {
    if (!allocations || !pool_used_bytes) throw Error(QTNH_ERR_INVALID_ARGUMENT, "null output pointer");
    *allocations = g_workspace_allocs.load(std::memory_order_relaxed);
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    cudaMemPool_t pool;
    check_cuda(cudaDeviceGetDefaultMemPool(&pool, dev), "cudaDeviceGetDefaultMemPool");
    unsigned long long used = 0;  // the attribute is a 64-bit unsigned value
    check_cuda(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used), "cudaMemPoolGetAttribute");
    *pool_used_bytes = (uint64_t)used;
    return QTNH_OK;
  });
}

int qtnh_malloc_async(void** ptr, size_t bytes, void* stream) {
  return QTNH_API([&]() -> int {
    *ptr = nullptr;
    if (bytes == 0) bytes = 16;
    check_cuda(cudaMallocAsync(ptr, bytes, (cudaStream_t)stream), "cudaMallocAsync");
    return QTNH_OK;
  });
}

int qtnh_free_async(void* ptr, void* stream) {
  return QTNH_API([&]() -> int {
    if (ptr) check_cuda(cudaFreeAsync(ptr, (cudaStream_t)stream), "cudaFreeAsync");
    return QTNH_OK;
  });
}

int qtnh_norm2(const void* x, uint64_t n, double* result_host, void* stream) {
  return QTNH_API([&]() -> int {
    cudaStream_t s = (cudaStream_t)stream;
    double* acc = (double*)workspace_alloc(sizeof(double), stream);
    check_cuda(cudaMemsetAsync(acc, 0, sizeof(double), s), "memset");
    if (n) {
      int grid = sm_count() * 4;
      norm2_kernel<<<grid, 512, 0, s>>>((const double2*)x, n, acc);
      count_launch();
      check_cuda(cudaGetLastError(), "norm2 launch");
    }
    check_cuda(cudaMemcpyAsync(result_host, acc, sizeof(double), cudaMemcpyDeviceToHost, s), "d2h copy");
    workspace_free(acc, stream);
    check_cuda(cudaStreamSynchronize(s), "stream synchronize");
    return QTNH_OK;
  });
}

}  // extern "C"
