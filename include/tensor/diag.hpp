// Diagonal tensors (the reference declares them in include/tensor/diag.hpp:15-287 but
// leaves DiagTensor unimplemented, src/tensor/diag.cpp:65-117).
//
// Semantics implemented here, from the reference's documentation (diag.hpp:11-14,
// README.md:52): a diagonal tensor is a symmetric tensor whose only non-zero elements
// have equal total input and output indices, D[in, out] = d[in] * delta(in, out), where
// the inputs are the distributed inputs followed by the local inputs and d is stored
// row-major over them. Contracting all inputs multiplies the first tensor elementwise
// (a streaming kernel on the GPU).
#ifndef QTNH_TENSOR_DIAG_HPP
#define QTNH_TENSOR_DIAG_HPP

#include "tensor/symm.hpp"

namespace qtnh {
  class DiagTensorBase;
  class DiagTensor;
  class IdenTensor;

  class DiagTensorBase : public SymmTensorBase {
    public:
      DiagTensorBase() = delete;
      DiagTensorBase(const DiagTensorBase&) = delete;
      virtual ~DiagTensorBase() = default;

      virtual TT type() const noexcept override { return TT::diagTensorBase; }
      bool truncated() const noexcept { return truncated_; }

    protected:
      DiagTensorBase(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                     bool truncated);
      DiagTensorBase(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                     bool truncated, BcParams params);

      virtual bool isDiag() const noexcept override { return true; }
      virtual DiagTensor* toDiag() noexcept override;

      bool truncated_;  ///< Recorded; with all slabs resident it changes nothing.
  };

  /// Diagonal tensor with stored diagonal.
  class DiagTensor : public DiagTensorBase {
    public:
      friend class DiagTensorBase;

      DiagTensor() = delete;
      DiagTensor(const DiagTensor&) = delete;
      ~DiagTensor() = default;

      /// diag_els: prod(totInDims()) elements, row-major over the input indices
      /// (std::invalid_argument on a size mismatch).
      static std::unique_ptr<DiagTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                              qtnh::tidx_tup_st n_dis_in_dims, bool truncated,
                                              std::vector<qtnh::tel>&& diag_els) {
        return std::unique_ptr<DiagTensor>(
            new DiagTensor(env, dis_dims, loc_dims, n_dis_in_dims, truncated, std::move(diag_els)));
      }
      static std::unique_ptr<DiagTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                              qtnh::tidx_tup_st n_dis_in_dims, bool truncated,
                                              std::vector<qtnh::tel>&& diag_els, BcParams params) {
        return std::unique_ptr<DiagTensor>(
            new DiagTensor(env, dis_dims, loc_dims, n_dis_in_dims, truncated, std::move(diag_els), params));
      }

      virtual std::unique_ptr<Tensor> copy() const noexcept override;
      virtual TT type() const noexcept override { return TT::diagTensor; }

      virtual qtnh::tel operator[](qtnh::tidx_tup loc_idxs) const override;
      /// Diagonal element i (the stored array is the diagonal).
      virtual qtnh::tel operator[](std::size_t i) const override { return diag_.host_at(i); }
      virtual qtnh::tel at(qtnh::tidx_tup tot_idxs) const override;
      qtnh::tel& operator[](std::size_t i) { return diag_.host_ref(i); }
      /// Reference to the stored diagonal element addressed by tot_idxs (std::invalid_argument
      /// when the element is off the diagonal).
      qtnh::tel& at(qtnh::tidx_tup tot_idxs);
      void put(qtnh::tidx_tup tot_idxs, qtnh::tel el);

      virtual int engineKind() const noexcept override;
      virtual const void* engineData() const override { return diag_.read(); }

    protected:
      DiagTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                 bool truncated, std::vector<qtnh::tel>&& diag_els);
      DiagTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                 bool truncated, std::vector<qtnh::tel>&& diag_els, BcParams params);

      virtual DiagTensor* toDiag() noexcept override { return this; }
      virtual DiagTensor* rebcast(BcParams params) override;
      virtual detail::DeviceArray releaseStorage() override { return std::move(diag_); }
      bool diag_index(const qtnh::tidx_tup& tot_idxs, std::size_t& i) const;

      detail::DeviceArray diag_;
  };

  /// Identity: ones on the diagonal of [first half | second half] of the total indices
  /// (reference src/tensor/diag.cpp:143-151); implicit. Used to move indices between
  /// the distributed and the local part ("DIST" tensors).
  class IdenTensor : public DiagTensorBase {
    public:
      IdenTensor() = delete;
      IdenTensor(const IdenTensor&) = delete;
      ~IdenTensor() = default;

      static std::unique_ptr<IdenTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                              qtnh::tidx_tup_st n_dis_in_dims, bool truncated) {
        return std::unique_ptr<IdenTensor>(new IdenTensor(env, dis_dims, loc_dims, n_dis_in_dims, truncated));
      }
      static std::unique_ptr<IdenTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                              qtnh::tidx_tup_st n_dis_in_dims, bool truncated, BcParams params) {
        return std::unique_ptr<IdenTensor>(new IdenTensor(env, dis_dims, loc_dims, n_dis_in_dims, truncated, params));
      }

      virtual std::unique_ptr<Tensor> copy() const noexcept override;
      virtual TT type() const noexcept override { return TT::idenTensor; }

      virtual qtnh::tel operator[](qtnh::tidx_tup loc_idxs) const override;
      /// The reference returns 1 for every stored position (include/tensor/diag.hpp:258).
      virtual qtnh::tel operator[](std::size_t) const override { return 1; }
      virtual qtnh::tel at(qtnh::tidx_tup tot_idxs) const override;

      virtual int engineKind() const noexcept override;

    protected:
      IdenTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                 bool truncated);
      IdenTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, qtnh::tidx_tup_st n_dis_in_dims,
                 bool truncated, BcParams params);
      virtual IdenTensor* rebcast(BcParams params) override;
  };
}

#endif
