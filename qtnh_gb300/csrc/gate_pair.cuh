// Shared pieces of the fused gate-pair kernels (gate_tc.cu: mma.sync, gate_umma.cu:
// tcgen05): two disjoint two-qubit gates of a layer act on a group of 16 amplitudes (the
// four target bits varying) as one 16x16 operator U16 = Ua (x) Ub, in real form
// R = [[Re U16, -Im U16], [Im U16, Re U16]] (32 x 32) on the group's 32 reals
// (real parts k = 0..15, imaginary parts k = 16..31), through bf16 digits (ozaki.cuh).
// A lone gate uses the same kernels with U16 = gate (x) I4, gate (x) I2 or a four-qubit
// gate itself (PairGate).
#pragma once

#include "cuda_common.cuh"
#include "ozaki.cuh"

namespace qtnh_impl {

// How the 16x16 operator of a group is formed from the gate pointers (ga, gb).
enum PairGate : uint32_t {
  PAIR_KRON = 0,   // two two-qubit gates: U16 = Ua (x) Ub
  PAIR_FULL = 1,   // one four-qubit gate: U16 = Ua (16 x 16; gb unused)
  PAIR_KRON_I2 = 2 // one three-qubit gate on the first three targets: U16 = Ua (8 x 8) (x) I2
};

struct PairParams {
  uint64_t ngroups;     // state size / 16
  uint32_t ins_pos[4];  // the four target bit positions, ascending
  int64_t off[16];      // offset of amplitude (a0 a1 b0 b1) of a group from its base
};

// Index of the first amplitude of group `grp`: zero bits inserted at the target positions.
template <typename IT>
__device__ __forceinline__ IT pair_base(IT grp, const PairParams& p) {
  IT b = grp;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const IT low = b & ((IT(1) << p.ins_pos[j]) - 1);
    b = ((b >> p.ins_pos[j]) << (p.ins_pos[j] + 1)) | low;
  }
  return b;
}

// A group's (or a gate row's) largest biased exponent must lie in [TC_EMIN, TC_EMAX]
// (magnitudes 2^-200 .. 2^201) unless it is 0 (zeros and subnormals only); infinities
// and NaNs (exponent 0x7FF) fail. Then the level sums, scaled by 2^(Esum - 2060) through
// the exponent field, stay normal doubles.
constexpr uint32_t TC_EMIN = 823, TC_EMAX = 1224;

// Gate entries: zero or a normal double (no subnormal, infinity or NaN).
__device__ __forceinline__ bool tc_element_ok(df::dwords w) {
  const uint32_t e = oz::exponent(w);
  return e == 0 ? (((w.hi << 1) | w.lo) == 0u) : (e != 0x7FFu);
}

__device__ __forceinline__ bool tc_scale_ok(uint32_t emax) { return emax == 0 || (emax >= TC_EMIN && emax <= TC_EMAX); }

// U16[o * 16 + i] from gates in SymmTensor layout G[in * D + out] = U[out][in]:
// PAIR_KRON: Ua[oa][ia] Ub[ob][ib] (o = oa * 4 + ob, i = ia * 4 + ib); PAIR_FULL: Ua[o][i];
// PAIR_KRON_I2: Ua[o >> 1][i >> 1] where the last bits of o and i agree, else 0.
// (MODE is a template parameter of the kernels, so the gate-pair path compiles as before.)
template <uint32_t MODE>
__device__ __forceinline__ double2 fused_entry(const double2* __restrict__ ga, const double2* __restrict__ gb, int t) {
  const int o = t >> 4, i = t & 15;
  if (MODE == PAIR_FULL) return ga[i * 16 + o];
  if (MODE == PAIR_KRON_I2) return ((o ^ i) & 1) ? make_double2(0.0, 0.0) : ga[(i >> 1) * 8 + (o >> 1)];
  return cmul(ga[(i >> 2) * 4 + (o >> 2)], gb[(i & 3) * 4 + (o & 3)]);
}

// Element (r, k) of the real form R of U16.
__device__ __forceinline__ double real_form(const double2* U16, int r, int k) {
  const double2 u = U16[(r & 15) * 16 + (k & 15)];
  if (r < 16) return k < 16 ? u.x : -u.y;
  return k < 16 ? u.y : u.x;
}

// Largest exponent of row o of U16 (shared by rows o and 16 + o of R) and whether the
// row is usable by the digit path.
__device__ __forceinline__ uint32_t row_exponent(const double2* U16, int o, bool& ok) {
  uint32_t e = 0;
  ok = true;
#pragma unroll 4
  for (int i = 0; i < 16; ++i) {
    const double2 u = U16[o * 16 + i];
    const df::dwords wr = df::words(u.x), wi = df::words(u.y);
    ok = ok && tc_element_ok(wr) && tc_element_ok(wi);
    e = max(e, max(oz::exponent(wr), oz::exponent(wi)));
  }
  ok = ok && tc_scale_ok(e);
  return e;
}

// The 16 outputs of one group in FP64 (U16 in shared memory).
__device__ __forceinline__ double2 group_output_fp64(const double2* U16, const double2 (&x)[16], int o) {
  double2 acc = make_double2(0.0, 0.0);
#pragma unroll
  for (int i = 0; i < 16; ++i) acc = cfma(U16[o * 16 + i], x[i], acc);
  return acc;
}

// Host side: the pair's parameters (targets of gate a, then gate b; all dims 2).
PairParams make_pair_params(const dims_t& dims, const uint16_t all[4]);

struct ChainRec;
// tcgen05 kernel for states of at least 2048 amplitudes; false if it does not apply.
// rec (may be null) receives the largest group key of the outputs and the smallest
// nonzero half group (ChainRec::maxkey, ::minc; atomicMax).
bool launch_pair_umma(double2* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s,
                      uint32_t mode = PAIR_KRON, ChainRec* rec = nullptr);

// What one pass of a gate layer's fixed-point chain wrote (device memory; the host zeroes
// the chain's records before its first pass).
struct ChainRec {
  uint32_t maxkey;  // doubles written: the largest oz::group_key of the outputs
  uint32_t maxhi;   // fixed point written: a value with the bit length of the largest |hi
                    // word| of the outputs (an OR of them)
  int32_t F;        // fixed point written: value = Y 2^-F
  int32_t fmt;      // 1: fixed point written, 0: doubles
  uint32_t minc;    // doubles written by the first pass: 2047 - the smallest exponent of a
                    // nonzero half group's largest output (0: none)
  uint32_t pad[3];
};

// A chain starts only when every nonzero half group the first pass wrote lies within
// 2^CHAIN_RANGE of the largest magnitude: fixed point carries ~46 bits of the largest
// magnitude, so every group keeps ~40 bits of its own.
constexpr int CHAIN_RANGE = 6;


// A permutation of a power-of-two state as a permutation of the bits of the element index
// (states of at most 2^32 elements): P(x) = the OR over the index's four bytes of
// tab[k][byte k], and poff[c] = P(off[c]) for the pair's 16 amplitude offsets. P is
// linear over disjoint bit sets, so P(base | off) = P(base) | P(off).
struct BitPerm {
  uint32_t tab[4][256];
  uint32_t poff[16];
};
// The bit tables of the permutation ptup (Tensor::permute convention) of a state of dims
// `dims` and the pair's permuted offsets; false if the dims are not all powers of two or the
// state has more than 2^32 elements.
bool make_bit_perm(const dims_t& dims, const std::vector<uint16_t>& ptup, const PairParams& p, BitPerm& bp);

// Whether the chain kernel takes a pair of this shape (the tcgen05 tile shape).
bool chain_applies(const PairParams& p);
// A later pass of a chain (two disjoint two-qubit gates): reads what rin describes, writes
// fixed point (want_fixed, when the scales allow) or doubles, and records it in rout. With
// `perm` (host memory) it writes out of place, to `out`, with every element at its index
// under the permutation (the pass and the permutation after it in one pass over the state).
void launch_pair_chain(void* psi, const double2* ga, const double2* gb, const PairParams& p, cudaStream_t s,
                       const ChainRec* rin, ChainRec* rout, bool want_fixed, void* out = nullptr,
                       const BitPerm* perm = nullptr);

// Reads and clears the tcgen05 kernel's device error flags (bounded waits that expired).
uint32_t take_umma_error();

}  // namespace qtnh_impl
