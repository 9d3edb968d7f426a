/*
 * qtnh_cuda.h — C ABI of the GB300 (sm_103a) tensor-contraction engine.
 *
 * This is the boundary between host code written against qtnh's C++ API and the
 * CUDA kernels. Every entry point takes plain pointers and sizes, returns an
 * int status (QTNH_OK == 0) and records a message readable with qtnh_last_error().
 *
 * Element type: complex<double> (the reference's `tel`, include/core/typedefs.hpp:21),
 * stored as interleaved (re, im) doubles, 16 bytes per element. Tensors are dense
 * row-major arrays over dis_dims ++ loc_dims (last index fastest,
 * src/core/utils.cpp:27-46). The reference spreads the leading dis_dims over MPI
 * ranks; here all slabs are resident in one HBM array in rank order, which is the
 * same global row-major order, so rescatter and rebcast are metadata-only and
 * distributed swaps/permutes are on-device transposes.
 *
 * Data pointers are device pointers unless named *_host. `stream` is a cudaStream_t
 * passed as void* (NULL = the legacy default stream). Calls are asynchronous with
 * respect to the host unless stated otherwise.
 *
 * Axis indices are uint16_t like the reference's tidx_tup_st
 * (include/core/typedefs.hpp:16); QTNH_X (0xFFFF) is the reference's wildcard X
 * (include/core/typedefs.hpp:55).
 */
#ifndef QTNH_CUDA_H
#define QTNH_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QTNH_ABI_VERSION 1
#define QTNH_X 0xFFFFu
#define QTNH_MAX_RANK 64

/* Status codes. The C++ facade maps them back to the reference's exception types. */
enum {
  QTNH_OK = 0,
  QTNH_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument (contract.cpp:210,213; dense.cpp:80,89) */
  QTNH_ERR_RUNTIME = 2,          /* std::runtime_error (dense.cpp:179; utils.cpp:10)            */
  QTNH_ERR_OUT_OF_RANGE = 3,     /* std::out_of_range (indexing.cpp:96,118; .at())               */
  QTNH_ERR_CUDA = 4,             /* CUDA runtime error                                           */
  QTNH_ERR_NO_MEMORY = 5,        /* device allocation failed                                     */
  QTNH_ERR_UNSUPPORTED = 6,      /* shape outside what a specialised kernel handles              */
  QTNH_ERR_CAPACITY = 7          /* output buffer too small (query protocol)                     */
};

/* Tensor kinds (include/core/typedefs.hpp:36-46, restricted to constructible classes). */
enum {
  QTNH_KIND_DENSE = 0, /* DenseTensor  (include/tensor/dense.hpp:75)               */
  QTNH_KIND_SYMM = 1,  /* SymmTensor   (include/tensor/symm.hpp:93)                */
  QTNH_KIND_SWAP = 2,  /* SwapTensor   (include/tensor/symm.hpp:230), implicit      */
  QTNH_KIND_IDEN = 3,  /* IdenTensor   (include/tensor/diag.hpp:204), implicit      */
  QTNH_KIND_DIAG = 4   /* DiagTensor   (include/tensor/diag.hpp:65), diagonal only  */
};

/* A tensor as the engine sees it. `data` is a device pointer:
 *   DENSE/SYMM: all prod(dims) elements;
 *   DIAG:       prod(input dims) diagonal elements, row-major over the input indices
 *               (dis inputs then local inputs, include/tensor/symm.hpp:22-45);
 *   SWAP/IDEN:  NULL (elements are implicit). */
typedef struct qtnh_tensor_desc {
  int32_t kind;
  int32_t ndis;
  int32_t nloc;
  int32_t n_dis_in;      /* symmetric family: number of distributed input indices */
  const uint64_t* dims;  /* ndis + nloc entries, host memory                     */
  const void* data;
} qtnh_tensor_desc;

/* ---- library, device and memory --------------------------------------------------- */

/* Message of the last failed call on this host thread (never NULL). */
const char* qtnh_last_error(void);
int qtnh_abi_version(void);
int qtnh_device_count(int* count);
int qtnh_set_device(int device);
int qtnh_malloc(void** ptr, size_t bytes);                    /* stream-ordered pool */
int qtnh_free(void* ptr);
int qtnh_memcpy_h2d(void* dst, const void* src_host, size_t bytes, void* stream);
int qtnh_memcpy_d2h(void* dst_host, const void* src, size_t bytes, void* stream);
int qtnh_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream);
int qtnh_memset(void* dst, int value, size_t bytes, void* stream);
int qtnh_stream_synchronize(void* stream);
int qtnh_device_synchronize(void);
int qtnh_stream_create(void** stream);  /* non-blocking stream */
int qtnh_stream_destroy(void* stream);
/* Stream-ordered allocation from the device's memory pool (cudaMallocAsync): cheap
 * for the many small tensors of a network, reused without device synchronisation. */
int qtnh_malloc_async(void** ptr, size_t bytes, void* stream);
int qtnh_free_async(void* ptr, void* stream);
/* Number of kernels this library has launched since load (all entry points). */
uint64_t qtnh_kernel_launch_count(void);
/* Allocation diagnostics (no counterpart in the reference): `allocations` = how many
 * temporary device buffers (scratch) the entry points have taken from the stream-ordered
 * pool since load; `pool_used_bytes` = the bytes in use in the current device's default
 * memory pool now. */
int qtnh_workspace_stats(uint64_t* allocations, uint64_t* pool_used_bytes);

/* Device-side error flags of the kernels whose waits are bounded (the tcgen05 gate-pair
 * kernel: bit 0 = a wait for converted digits expired, bit 1 = a wait for MMA completion
 * expired, bit 2 = a wait for the other half of a group expired; the tcgen05 GEMMs:
 * bits 8-10 (split precision) and 16-18 (QTNH_GEMM_OZ6) = a producer / MMA / epilogue
 * wait expired; the kernel then stops early and its output is incomplete). Synchronizes the device, returns the flags raised since the
 * previous call and clears them. */
int qtnh_take_device_errors(uint32_t* flags);

/* Test hook of the bounded waits (no counterpart in the reference; off by default): while
 * on != 0, every launch of the tcgen05 gate-pair kernel makes its first exponent exchange
 * wait on a shared-memory barrier that nothing completes, with a limit of ~2^20 cycles.
 * The wait expires before any tensor-core work of the CTA is issued; the CTA raises error
 * bit 2, frees its tensor memory and returns without writing, so the state is left as it
 * was and the next launch (hook off) runs normally. Synchronous with the host; process-wide. */
int qtnh_debug_expire_exchange_wait(int on);

/* Arithmetic of the complex128 gate and diagonal kernels (storage is always complex128).
 * QTNH_ARITH_BF16X6 (default): qtnh_apply_gate_layer fuses consecutive disjoint pairs of
 *   two-qubit gates (all dims 2) into 16x16 unitaries applied on the bf16 tensor cores:
 *   each operand is cut into six error-free balanced 8-bit digits, every digit-product
 *   level is summed exactly in FP32 (Ozaki scheme), and the levels are recombined to ~48
 *   bits; relative error ~1e-14 per fused pair. Groups whose largest magnitude lies
 *   outside 2^-200..2^200 (or holds an infinity/NaN) take FP64; subnormal amplitudes
 *   count as zero there. A lone gate on 2, 3 or 4 size-2 indices (qtnh_apply_gate, or
 *   the odd one of a layer) of a power-of-two state runs the same way as one 16x16
 *   operator: gate (x) I4, gate (x) I2 (free size-2 indices), or the four-qubit gate
 *   itself. Every other gate runs as QTNH_ARITH_F32X2; diagonals (single
 *   DiagTensors and per-index layers) multiply one element in four in native FP64 (two
 *   fused multiply-adds per component) and the other three as QTNH_ARITH_F32X2, so the
 *   FP64 unit works beside the FP32 pipes.
 * QTNH_ARITH_F32X2: products and sums as compensated FP32 pairs (error-free
 *   transformations) on the FP32 pipe; ~48-bit significands, per-contraction relative
 *   error ~1e-14; groups with elements outside 2^-90..2^90 fall back to FP64.
 * QTNH_ARITH_FP64: native FP64 fused multiply-adds.
 * The environment variable QTNH_ARITH=fp64|f32x2|bf16x6 sets the initial mode.
 * Process-wide. */
enum { QTNH_ARITH_FP64 = 0, QTNH_ARITH_F32X2 = 1, QTNH_ARITH_BF16X6 = 2 };
int qtnh_set_arithmetic(int mode);
int qtnh_get_arithmetic(void);

/* Precision of the complex GEMM inside dense contractions (_contract_dense,
 * src/tensor/contract.cpp:12-201).
 * QTNH_GEMM_OZ6 (default): the plain method on the tcgen05 tensor cores. Every real of a
 *   row of A (column of B) is cut into six error-free balanced 8-bit digits at the row's
 *   (column's) largest exponent, the 21 digit-pair products of levels 0..5 are summed
 *   exactly in FP32 over chunks of 128 reals of K, and the chunks are accumulated exactly
 *   in 64-bit integers (levels 0-3) and FP32 (levels 4-5, below 2^-32): each result is
 *   accurate to ~2^-48 of its row's and column's largest products, whatever K (reproduces
 *   the reference within 1e-12 relative L2). Rows or columns holding an infinity or NaN
 *   are recomputed in FP64. GEMMs below 2^18 complex multiply-adds or with a contracted
 *   size below 16, and contractions with a SwapTensor or IdenTensor operand, run as
 *   QTNH_GEMM_FP64 (which keeps relabellings by 0/1 tensors bit-exact).
 * QTNH_GEMM_FP64: complex128 FP64 fused multiply-adds on the FP64 pipe.
 * QTNH_GEMM_BF16X3: split precision on the tcgen05 tensor cores: every real split into
 *   three bf16 pieces (24 bits), the six piece products with i + j <= 2 accumulated in
 *   FP32 on the tensor cores; FP32-level error (~1e-6 relative L2 at K ~ 100, growing
 *   with K; report it against QTNH_GEMM_FP64).
 * The environment variable QTNH_GEMM=oz6|fp64|bf16x3 sets the initial mode. Process-wide. */
enum { QTNH_GEMM_FP64 = 0, QTNH_GEMM_BF16X3 = 1, QTNH_GEMM_OZ6 = 2 };
int qtnh_set_gemm_precision(int mode);
int qtnh_get_gemm_precision(void);

/* K-steps (16 bf16 reals each) accumulated on their own in one split-K slice of the
 * QTNH_GEMM_BF16X3 GEMM, 1..QTNH_GEMM_SLICE_MAX (default 32; the environment variable
 * QTNH_GEMM_SLICE sets the initial value). The tensor core's FP32 accumulation loses up to
 * an ulp per K-step, so the error grows in proportion to the slice length while the FP32
 * partials written per slice (8 bytes per output element) shrink in inverse proportion:
 * on the 64-pair precision study, relative L2 vs FP64 2.3e-7 / 4.7e-7 / 1.0e-6 / 2.1e-6
 * at 16 / 32 / 64 / 128 K-steps, for 134 / 178 / 205 / 215 complex TFLOP/s.
 * Process-wide. */
#define QTNH_GEMM_SLICE_DEFAULT 32
#define QTNH_GEMM_SLICE_MAX 4096
int qtnh_set_gemm_slice(int k_steps);
int qtnh_get_gemm_slice(void);

/* CUDA-event timing of the tcgen05 GEMM kernel launches (measurement support): returns
 * the summed duration (ms) and count of the launches recorded since the previous call
 * (synchronizing on them), then enables (enable != 0) or disables recording. */
int qtnh_gemm_timing(int enable, double* ms, uint64_t* launches);

/* ---- data movement: TIDense kernels ------------------------------------------------ */

/* Tensor::permute / TIDense::_permute_internal (src/tensor/dense.cpp:152-169, 354-488):
 * old axis i moves to new position ptup[i]; out has dims new[ptup[i]] = dims[i].
 * Bit-exact. `in` and `out` must not overlap. */
int qtnh_permute(const void* in, void* out, int32_t rank, const uint64_t* dims, const uint16_t* ptup,
                 void* stream);

/* Tensor::swap / TIDense::_swap_internal (src/tensor/dense.cpp:171-274): exchange two
 * axes of equal dimension (local, mixed and distributed cases alike). Unequal
 * dimensions fail with QTNH_ERR_RUNTIME like dense.cpp:178-180. Bit-exact. */
int qtnh_swap(const void* in, void* out, int32_t rank, const uint64_t* dims, int32_t idx1, int32_t idx2,
              void* stream);

/* ---- contraction metadata: Tensor::contract (src/tensor/contract.cpp:204-289) ------ */

/* Validates the wires and chooses the dimension replacements exactly as the reference:
 * default order [t1 open dis, t2 open dis, t1 open loc, t2 open loc] (contract.cpp:220-248)
 * or, for a symmetric second operand with all inputs wired, the in-place rule
 * (contract.cpp:250-289). With use_default == 0 the caller's repls are kept.
 * repls1/repls2 are in/out (rank1 / rank2 entries, QTNH_X for closed indices).
 * out_dims must hold rank1 + rank2 entries; out_str receives the stretch factor of the
 * result's broadcaster (product of contracted distributed dimensions, contract.cpp:196-200).
 * Host-only: needs no GPU. */
int qtnh_contract_plan(const qtnh_tensor_desc* t1, const qtnh_tensor_desc* t2, int32_t nwires,
                       const uint16_t* wires, int32_t use_default, uint16_t* repls1, uint16_t* repls2,
                       int32_t* out_ndis, int32_t* out_nloc, uint64_t* out_dims, uint64_t* out_str);

/* Host-only companion of qtnh_contract: plans as qtnh_contract_plan (same outputs) and
 * reports whether qtnh_contract would apply t2 in place to t1 -- a SymmTensor gate or a
 * DiagTensor whose inputs are exactly the wired indices, with the in-place rule of
 * contract.cpp:250-289 -- and, if so (*inplace = 1), t1's indices wired to t2's inputs in
 * input order (*ntargets entries of `targets`, which must hold QTNH_MAX_RANK). The C++
 * API uses it to queue such contractions and apply runs of them as fused layers. */
int qtnh_contract_inplace(const qtnh_tensor_desc* t1, const qtnh_tensor_desc* t2, int32_t nwires,
                          const uint16_t* wires, int32_t use_default, uint16_t* repls1, uint16_t* repls2,
                          int32_t* out_ndis, int32_t* out_nloc, uint64_t* out_dims, uint64_t* out_str,
                          int32_t* inplace, int32_t* ntargets, uint16_t* targets);

/* ---- contraction ------------------------------------------------------------------- */

/* Tensor::contract (contract.cpp:204-313 with _contract_dense, 12-201): plans as
 * qtnh_contract_plan, then computes C[out] = sum over wired index pairs of t1 * t2 with
 * the result index order given by the replacements. Dispatches to specialised kernels:
 * symmetric gates applied in place (register-blocked group kernel), diagonal tensors
 * (streaming phase multiply), swap/identity tensors (transpose, bit-exact), and
 * everything else to the permute-fused complex GEMM. `out` receives prod(out_dims)
 * elements (out_capacity is in elements); with out == NULL only the metadata is filled
 * and QTNH_ERR_CAPACITY is returned. `out` may alias t1->data when the result has the
 * same size as t1 (the caller gives up t1, as Tensor::contract consumes tp1). */
int qtnh_contract(const qtnh_tensor_desc* t1, const qtnh_tensor_desc* t2, int32_t nwires, const uint16_t* wires,
                  int32_t use_default, uint16_t* repls1, uint16_t* repls2, int32_t* out_ndis, int32_t* out_nloc,
                  uint64_t* out_dims, uint64_t* out_str, void* out, uint64_t out_capacity, void* stream);

/* General dense contraction with explicit output positions (the global form of
 * _contract_dense): C[...] = sum_wired A * B, where open axis i of A goes to output
 * position out_pos_a[i] and open axis j of B to out_pos_b[j] (QTNH_X for wired axes).
 * Permute-fused FP64 complex GEMM. `c` must not overlap `a` or `b`. */
int qtnh_contract_dense(const void* a, int32_t rank_a, const uint64_t* dims_a, const void* b, int32_t rank_b,
                        const uint64_t* dims_b, int32_t nwires, const uint16_t* wires, const uint16_t* out_pos_a,
                        const uint16_t* out_pos_b, void* c, void* stream);

/* The contraction of qtnh_contract_dense, for callers that cannot allocate device
 * memory while they run: hosts whose device memory is owned by their own allocator or
 * fixed budget, and latency-critical loops where a cudaMalloc would stall or fragment.
 * It has no counterpart in the reference (which contracts on host memory over MPI).
 * The permuted copies of A, B and C live in one scratch array that the library defines
 * at file scope in device memory (QTNH_NOALLOC_SCRATCH_ELEMS complex128 elements,
 * 16 MiB, held by every GPU that loads the library until the process exits). The call
 * allocates nothing; contractions whose permuted copies need more elements than that
 * fail with QTNH_ERR_UNSUPPORTED before any work is issued. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress, with that device current);
 * make that first call before any stream capture. A cudaDeviceReset invalidates the
 * address looked up then, so the entry point is not for use after a cudaDeviceReset in
 * the same process. The GEMM is always the plain FP64 one (the QTNH_GEMM_FP64 numerics),
 * whatever qtnh_set_gemm_precision selects: the split-precision and digit GEMMs need
 * operand planes that this path has no room for. Every call shares the one array and
 * it keeps the previous call's contents (nothing in it needs to start at zero): calls
 * that can overlap on the GPU, on different streams or threads, race on it and must be
 * serialised by the caller. */
#define QTNH_NOALLOC_SCRATCH_ELEMS (1u << 20)
int qtnh_contract_dense_noalloc(const void* a, int32_t rank_a, const uint64_t* dims_a, const void* b, int32_t rank_b,
                                const uint64_t* dims_b, int32_t nwires, const uint16_t* wires,
                                const uint16_t* out_pos_a, const uint16_t* out_pos_b, void* c, void* stream);

/* ---- symmetric gates and diagonals (the in-place rule, contract.cpp:250-289) -------- */

/* psi'[.., o_j at targets[j], ..] = sum_in G[in, o] psi[.., in_j at targets[j], ..] where
 * G = gate elements in SymmTensor layout [in_0..in_{k-1}, out_0..out_{k-1}] row-major
 * (include/tensor/symm.hpp:22-45). All target dims must be equal to the gate's.
 * In place (state is read and overwritten). Device pointer `gate`. Gate sizes D (product
 * of the target dims) of 1, 2, 3, 4, 8, 9 and 16 run register-blocked kernels; any other
 * size runs a general FP64 kernel that reads a copy of the state (workspace of the
 * state's size). */
int qtnh_apply_gate(void* state, int32_t rank, const uint64_t* dims, int32_t k, const uint16_t* targets,
                    const void* gate, void* stream);

/* Several gates applied in list order (each as qtnh_apply_gate), fused into as few
 * passes over the state as the target sets allow. gate_k[g] targets per gate,
 * targets: concatenated target lists, gates: device pointers (one per gate). */
int qtnh_apply_gate_layer(void* state, int32_t rank, const uint64_t* dims, int32_t ngates, const int32_t* gate_k,
                          const uint16_t* targets, const void* const* gates, void* stream);

/* Runs of in-place gate contractions with a permutation between consecutive runs: the
 * sequence qtnh_apply_gate_layer(run 0), Tensor::permute (src/tensor/dense.cpp:152-169,
 * ptups[0]), qtnh_apply_gate_layer(run 1), ... as one call. Run r holds run_ngates[r]
 * gates (gate_k, targets and gates concatenated over the runs, targets naming the axes
 * of the state as it is when the run starts); ptups holds nruns - 1 permutation tuples
 * of rank entries each (the qtnh_permute convention). Permutations go out of place
 * between state and scratch (same size, no overlap; unused when nruns == 1), so the
 * result is in scratch when nruns - 1 is odd and in state otherwise; the other buffer's
 * contents are undefined afterwards. With QTNH_ARITH_BF16X6 the fused gate-pair passes
 * of all runs form one fixed-point chain (the permutations move the fixed-point
 * elements), so a permutation does not end the chain. All arguments are checked before
 * the first launch. Device pointers state, scratch and gates. */
int qtnh_apply_gate_runs(void* state, void* scratch, int32_t rank, const uint64_t* dims, int32_t nruns,
                         const int32_t* run_ngates, const int32_t* gate_k, const uint16_t* targets,
                         const void* const* gates, const uint16_t* ptups, void* stream);

/* CUDA-event timing of the fused gate-pair passes (QTNH_ARITH_BF16X6; measurement
 * support): returns the summed duration (ms) and count of the passes recorded since the
 * previous call (synchronizing on them), then enables (enable != 0) or disables
 * recording. */
int qtnh_gate_timing(int enable, double* ms, uint64_t* launches);

/* DiagTensor contraction in place: psi[x] *= d[x restricted to targets] with d the
 * diagonal (row-major over the target dims). Device pointer `diag`. */
int qtnh_apply_diag(void* state, int32_t rank, const uint64_t* dims, int32_t k, const uint16_t* targets,
                    const void* diag, void* stream);

/* The product of a gate and a diagonal on one of its outputs, for queues of in-place
 * contractions: out[in, o] = gate[in, o] * diag[o_p] (SymmTensor layout, k targets of dims
 * tdims, o_p the output's digit at target position p; diag tdims[p] long). Applying the
 * gate and then the diagonal on its p-th target (two in-place contractions,
 * src/tensor/contract.cpp:250-289) equals applying this product once. out may be gate
 * (in place). Device pointers gate, diag, out. */
int qtnh_symm_diag_product(const void* gate, int32_t k, const uint64_t* tdims, int32_t p, const void* diag,
                           void* out, void* stream);

/* A layer of single-index diagonals in one streaming pass:
 * psi[x] *= prod_f d_f[x_{axes[f]}], d_f = factors + offset_f (each dims[axes[f]] long,
 * concatenated in f order). Device pointer `factors`. */
int qtnh_apply_diag_layer(void* state, int32_t rank, const uint64_t* dims, int32_t nfactors, const uint16_t* axes,
                          const void* factors, void* stream);

/* ---- reductions (FP64) ------------------------------------------------------------- */

/* sum |x|^2 over n elements to FP64 accuracy on the device (half of the squares as FP64
 * FMAs, half as exact float-float products, partial sums combined in FP64); result to
 * host. Synchronous. */
int qtnh_norm2(const void* x, uint64_t n, double* result_host, void* stream);

/* ---- grouped operations on many resident states (request loops) ---------------------- */

/* State precision: plain complex128 (FP64 arithmetic) or mixed complex64 (FP32
 * arithmetic, gates held as complex64 hi + lo; FP64 norms and sums). */
enum { QTNH_STATE_C128 = 0, QTNH_STATE_C64 = 1 };

/* The next layer of each of `nstates` device states (states[i], nqubits[i] qubits,
 * qubit q = bit n - 1 - q): ngates[i] two-qubit SymmTensor gates (pairs: concatenated
 * (qa, qb) per gate, input 0 on qa; gates_c128: host, 16 complex128 per gate in
 * SymmTensor layout, include/tensor/symm.hpp:22-45), then if has_phases[i] a phase
 * DiagTensor on every qubit (phases: host, concatenated nqubits[i] per such state), then
 * if swaps[2i] != 0xFFFF the exchange of qubits swaps[2i], swaps[2i+1]. Gates of one
 * state must be disjoint. Grouped launches: one per gate slot, one for the phases, one
 * for the swaps. has_phases, phases and swaps may be null. */
int qtnh_group_layer(int32_t precision, int32_t nstates, void* const* states, const int32_t* nqubits,
                     const int32_t* ngates, const uint16_t* pairs, const void* gates_c128, const uint8_t* has_phases,
                     const double* phases, const uint16_t* swaps, void* stream);
/* Renormalise each state to unit L2 norm (FP64 norm). */
int qtnh_group_renorm(int32_t precision, int32_t nstates, void* const* states, const int32_t* nqubits, void* stream);
/* out_c128[i] = state[idx[i]] (idx: host; out: device complex128). */
int qtnh_gather(int32_t precision, const void* state, int32_t nqubits, int32_t nidx, const uint64_t* idx,
                void* out_c128, void* stream);
/* Reduced density matrix of qubits[0..3] (host): out_c128 (device, 16 x 16 complex128,
 * row-major, index bits q0 q1 q2 q3) = sum over the other qubits of psi psi^*, in FP64. */
int qtnh_rdm4(int32_t precision, const void* state, int32_t nqubits, const uint16_t* qubits, void* out_c128,
              void* stream);
/* n amplitudes complex128 -> complex64 (to_precision QTNH_STATE_C64) or back. */
int qtnh_state_convert(int32_t to_precision, const void* in, void* out, uint64_t n, void* stream);

/* ---- batched circuits ---------------------------------------------------------------- */

/* Many independent circuits of uneven qubit counts and depths, states resident in HBM:
 * complex64 (mixed precision; qtnh_batch_create: gates in exact 64-bit fixed-point sums
 * with one rounding per output, phases in FP32) or complex128 with FP64 math (the plain
 * method; qtnh_batch_create_typed with QTNH_STATE_C128). Operations per circuit follow the layered-circuit contractions: two-qubit
 * SymmTensor gates (els in SymmTensor layout, host pointer to 16 complex128; input 0 on
 * qubit qa, input 1 on qb; include/tensor/symm.hpp:22-45), a phase layer (n host
 * phases: DiagTensor (1, e^{i phase}) on every qubit) and SwapTensor qubit exchanges,
 * applied per layer in that order; every `renorm_every` layers each state is
 * renormalised with an FP64 norm; queries return amplitudes as complex128 (host index
 * lists). Qubit q is bit n - 1 - q of the amplitude index (row-major dims [2]*n).
 * qtnh_batch_compile groups the operations of all circuits into rounds of grouped
 * persistent kernels (consecutive disjoint gates of a layer applied as one pass),
 * optionally autotunes the gate kernels, and captures the whole run
 * (state reset from the initial states, every round, the queries) as one CUDA graph;
 * qtnh_batch_run replays it ordered after and before work on `stream`. */
typedef struct qtnh_batch qtnh_batch;
int qtnh_batch_create(qtnh_batch** out, int32_t ncircuits, const int32_t* nqubits);
/* precision: QTNH_STATE_C64 (as qtnh_batch_create) or QTNH_STATE_C128. */
int qtnh_batch_create_typed(qtnh_batch** out, int32_t ncircuits, const int32_t* nqubits, int32_t precision);
int qtnh_batch_destroy(qtnh_batch* b);
/* Initial state of circuit c from a device complex128 array (converted to complex64 in a
 * mixed-precision batch). */
int qtnh_batch_set_state(qtnh_batch* b, int32_t c, const void* psi_c128, void* stream);
int qtnh_batch_add_gate(qtnh_batch* b, int32_t c, int32_t layer, uint16_t qa, uint16_t qb, const void* els_c128);
int qtnh_batch_add_phases(qtnh_batch* b, int32_t c, int32_t layer, const double* phases);
int qtnh_batch_add_swap(qtnh_batch* b, int32_t c, int32_t layer, uint16_t qa, uint16_t qb);
int qtnh_batch_add_queries(qtnh_batch* b, int32_t c, int32_t nq, const uint64_t* idx);
int qtnh_batch_compile(qtnh_batch* b, int32_t renorm_every, int32_t autotune);
int qtnh_batch_run(qtnh_batch* b, void* stream);
/* All query results (registration order) into a device complex128 array. */
int qtnh_batch_results(qtnh_batch* b, void* out_c128, uint64_t capacity, void* stream);
/* Final state of circuit c as complex128 (device array of 2^n; synchronizes `stream`). */
int qtnh_batch_state(qtnh_batch* b, int32_t c, void* out_c128, void* stream);
/* gate_threads / gate_chunk: the autotuned block size and chunk length of the dominant
 * gate kernel -- the two-gate pair kernel (chunk in 16-amplitude groups) when the batch
 * has pair rounds, else the single-gate kernel (chunk in 4-amplitude groups). */
int qtnh_batch_info(qtnh_batch* b, uint64_t* amplitudes, uint64_t* rounds, uint64_t* launches_per_run,
                    int32_t* gate_threads, uint64_t* gate_chunk);

#ifdef __cplusplus
}
#endif

#endif /* QTNH_CUDA_H */
