// qtnh API on one GB300 GPU: tensors in HBM, contractions as CUDA kernels behind the
// C ABI of include/qtnh_cuda.h. Same headers, classes and functions as the reference's
// include/qtnh.hpp:13-22.
#ifndef QTNH_HPP
#define QTNH_HPP

namespace qtnh {
  namespace ops {}
  namespace utils {}
}

#include "core/env.hpp"
#include "core/typedefs.hpp"
#include "core/utils.hpp"

#include "tensor/dense.hpp"
#include "tensor/diag.hpp"
#include "tensor/indexing.hpp"
#include "tensor/network.hpp"
#include "tensor/symm.hpp"
#include "tensor/tensor.hpp"

#endif
