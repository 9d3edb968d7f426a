// Element, index and parameter types of the qtnh API (GB300 engine).
// Same names and meanings as the reference's include/core/typedefs.hpp:15-55.
#ifndef QTNH_CORE_TYPEDEFS_HPP
#define QTNH_CORE_TYPEDEFS_HPP

#include <complex>
#include <cstdint>
#include <functional>
#include <iostream>
#include <numeric>
#include <vector>

// Print from the root process. One process drives the GPU, so it is always the root.
#define ROOT_COUT std::cout

namespace qtnh {
  typedef std::size_t tidx;                ///< Tensor index dimension.
  typedef unsigned short int tidx_tup_st;  ///< Position of an index in a tuple.
  typedef unsigned int uint;               ///< Unsigned int for IDs.

  typedef std::vector<qtnh::tidx> tidx_tup;  ///< Tuple of tensor indices or dimensions.

  typedef std::complex<double> tel;  ///< Tensor element type (stored as complex128 in HBM).

  typedef std::pair<qtnh::tidx_tup_st, qtnh::tidx_tup_st> wire;  ///< A pair of contracted indices.

  /// Broadcast parameters. With every slab of a tensor resident on the one GPU they are
  /// bookkeeping only: stretch, cycles and offset are recorded and reported, no copies
  /// are made.
  struct BcParams {
    qtnh::uint str;  ///< Times each slab is repeated across contiguous ranks.
    qtnh::uint cyc;  ///< Times the whole tensor structure is repeated.
    qtnh::uint off;  ///< Empty ranks before the tensor begins.

    BcParams(qtnh::uint str, qtnh::uint cyc, qtnh::uint off) : str(str), cyc(cyc), off(off) {}
  };

  /// Tensor class labels.
  enum class TT {
    tensor,
    denseTensorBase,
    denseTensor,
    symmTensorBase,
    symmTensor,
    swapTensor,
    diagTensorBase,
    diagTensor,
    idenTensor
  };

  /// Input/output labels of symmetric tensor indices.
  enum class TIdxIO {
    in,   ///< Input indices: the first half of the distributed and of the local dimensions.
    out   ///< Output indices: the second half.
  };

  const qtnh::tidx_tup_st X = UINT16_MAX;  ///< Wildcard position (closed index).
}

#endif
