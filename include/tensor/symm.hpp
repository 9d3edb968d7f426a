// Symmetric tensors: indices split into equal input and output halves (mirrors the
// reference's include/tensor/symm.hpp:13-305).
#ifndef QTNH_TENSOR_SYMM_HPP
#define QTNH_TENSOR_SYMM_HPP

#include "tensor/dense.hpp"

namespace qtnh {
  class SymmTensorBase;
  class SymmTensor;
  class SwapTensor;

  /// Symmetric tensor base. Distributed dimensions are [inputs | outputs], local
  /// dimensions likewise; the in/out helpers use the reference's formulas
  /// (include/tensor/symm.hpp:22-45).
  class SymmTensorBase : public DenseTensorBase {
    public:
      SymmTensorBase() = delete;
      SymmTensorBase(const SymmTensorBase&) = delete;
      virtual ~SymmTensorBase() = default;

      virtual TT type() const noexcept override { return TT::symmTensorBase; }

      qtnh::tidx_tup disInDims() const;
      qtnh::tidx_tup locInDims() const;
      qtnh::tidx_tup totInDims() const { return utils::concat_dims(disInDims(), locInDims()); }
      qtnh::tidx_tup disOutDims() const;
      qtnh::tidx_tup locOutDims() const;
      qtnh::tidx_tup totOutDims() const { return utils::concat_dims(disOutDims(), locOutDims()); }

      virtual int engineDisIn() const noexcept override { return n_dis_in_dims_; }

    protected:
      SymmTensorBase(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims);
      SymmTensorBase(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                     BcParams params);

      virtual bool isSymm() const noexcept override { return true; }
      virtual SymmTensor* toSymm() noexcept override;

      qtnh::tidx_tup_st n_dis_in_dims_;
  };

  /// Writable symmetric tensor (gates). Elements are ordered [inputs..., outputs...]:
  /// contracting all inputs applies the gate in place (the result keeps the first
  /// tensor's index order), computed by the engine's register-blocked gate kernel.
  class SymmTensor : public SymmTensorBase {
    public:
      friend class SymmTensorBase;

      SymmTensor() = delete;
      SymmTensor(const SymmTensor&) = delete;
      ~SymmTensor() = default;

      static std::unique_ptr<SymmTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                              qtnh::tidx_tup_st n_dis_in_dims, std::vector<qtnh::tel>&& els) {
        return std::unique_ptr<SymmTensor>(new SymmTensor(env, dis_dims, loc_dims, n_dis_in_dims, std::move(els)));
      }
      static std::unique_ptr<SymmTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                              qtnh::tidx_tup_st n_dis_in_dims, std::vector<qtnh::tel>&& els,
                                              BcParams params) {
        return std::unique_ptr<SymmTensor>(new SymmTensor(env, dis_dims, loc_dims, n_dis_in_dims, std::move(els), params));
      }

      virtual std::unique_ptr<Tensor> copy() const noexcept override;
      virtual TT type() const noexcept override { return TT::symmTensor; }

      virtual qtnh::tel operator[](qtnh::tidx_tup loc_idxs) const override;
      qtnh::tel& operator[](qtnh::tidx_tup loc_idxs);
      virtual qtnh::tel operator[](std::size_t i) const override { return els_.host_at(i); }
      virtual qtnh::tel at(qtnh::tidx_tup tot_idxs) const override;
      qtnh::tel& operator[](std::size_t i) { return els_.host_ref(i); }
      qtnh::tel& at(qtnh::tidx_tup tot_idxs);
      void put(qtnh::tidx_tup tot_idxs, qtnh::tel el);

      virtual int engineKind() const noexcept override;
      virtual const void* engineData() const override { return els_.read(); }
      virtual std::vector<qtnh::tel> hostElements() const override { return els_.to_host(); }

    protected:
      SymmTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                 std::vector<qtnh::tel>&& els);
      SymmTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                 std::vector<qtnh::tel>&& els, BcParams params);
      SymmTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                 detail::DeviceArray&& els, BcParams params);

      virtual SymmTensor* toSymm() noexcept override { return this; }
      virtual SymmTensor* rebcast(BcParams params) override;
      virtual detail::DeviceArray releaseStorage() override { return std::move(els_); }

      detail::DeviceArray els_;
  };

  /// Rank-4 swap tensor, element [a, b, c, d] = (a == d && b == c); implicit (no storage).
  class SwapTensor : public SymmTensorBase {
    public:
      SwapTensor() = delete;
      SwapTensor(const SymmTensor&) = delete;
      ~SwapTensor() = default;

      /// n: dimension of the swapped indices; d: distributed inputs/outputs (0, 1 or 2).
      static std::unique_ptr<SwapTensor> make(const QTNHEnv& env, std::size_t n, std::size_t d) {
        return std::unique_ptr<SwapTensor>(new SwapTensor(env, n, d));
      }
      static std::unique_ptr<SwapTensor> make(const QTNHEnv& env, std::size_t n, std::size_t d, BcParams params) {
        return std::unique_ptr<SwapTensor>(new SwapTensor(env, n, d, params));
      }

      virtual std::unique_ptr<Tensor> copy() const noexcept override;
      virtual TT type() const noexcept override { return TT::swapTensor; }

      virtual qtnh::tel operator[](qtnh::tidx_tup loc_idxs) const override;
      virtual qtnh::tel operator[](std::size_t i) const override;
      virtual qtnh::tel at(qtnh::tidx_tup tot_idxs) const override;

      virtual int engineKind() const noexcept override;

    protected:
      SwapTensor(const QTNHEnv& env, std::size_t n, std::size_t d);
      SwapTensor(const QTNHEnv& env, std::size_t n, std::size_t d, BcParams params);
      virtual SwapTensor* rebcast(BcParams params) override;
  };
}

#endif
