// Dense tensors (mirrors the reference's include/tensor/dense.hpp:10-203).
#ifndef QTNH_TENSOR_DENSE_HPP
#define QTNH_TENSOR_DENSE_HPP

#include "tensor/tensor.hpp"

namespace qtnh {
  class DenseTensorBase;
  class DenseTensor;

  /// Tensors whose elements can all be stored. Transforms of derived classes that do not
  /// override them convert to DenseTensor first, as the reference does.
  class DenseTensorBase : public Tensor {
    public:
      DenseTensorBase() = delete;
      DenseTensorBase(const DenseTensorBase&) = delete;
      virtual ~DenseTensorBase() = default;

      virtual TT type() const noexcept override { return TT::denseTensorBase; }

    protected:
      DenseTensorBase(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims);
      DenseTensorBase(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, BcParams params);

      virtual bool isDense() const noexcept override { return true; }
      virtual DenseTensor* toDense() noexcept override;

      virtual Tensor* swap(qtnh::tidx_tup_st idx1, qtnh::tidx_tup_st idx2) override;
      virtual Tensor* rebcast(BcParams params) override;
      virtual Tensor* rescatter(int offset) override;
      virtual Tensor* permute(std::vector<qtnh::tidx_tup_st> ptup) override;
  };

  /// Writable dense tensor.
  class DenseTensor : public DenseTensorBase {
    public:
      friend class DenseTensorBase;
      friend qtnh::tptr contract_on_device(qtnh::tptr tp1, qtnh::tptr tp2, ConParams& params);

      DenseTensor() = delete;
      DenseTensor(const DenseTensor&) = delete;
      ~DenseTensor() = default;

      /// els holds every element in global row-major order over dis_dims ++ loc_dims
      /// (the concatenation of all ranks' local vectors in rank order); its size must be
      /// the tensor's total size (std::invalid_argument otherwise). Uploaded to HBM.
      static std::unique_ptr<DenseTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                               std::vector<qtnh::tel>&& els) {
        return std::unique_ptr<DenseTensor>(new DenseTensor(env, dis_dims, loc_dims, std::move(els)));
      }
      static std::unique_ptr<DenseTensor> make(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims,
                                               std::vector<qtnh::tel>&& els, BcParams params) {
        return std::unique_ptr<DenseTensor>(new DenseTensor(env, dis_dims, loc_dims, std::move(els), params));
      }

      virtual qtnh::tptr copy() const noexcept override;
      virtual TT type() const noexcept override { return TT::denseTensor; }

      virtual qtnh::tel operator[](qtnh::tidx_tup loc_idxs) const override;
      qtnh::tel& operator[](qtnh::tidx_tup loc_idxs);
      virtual qtnh::tel operator[](std::size_t i) const override { return els_.host_at(check_i(i)); }
      virtual qtnh::tel at(qtnh::tidx_tup tot_idxs) const override;
      qtnh::tel& operator[](std::size_t i) { return els_.host_ref(check_i(i)); }
      qtnh::tel& at(qtnh::tidx_tup tot_idxs);
      void put(qtnh::tidx_tup tot_idxs, qtnh::tel el);

      virtual int engineKind() const noexcept override;
      virtual const void* engineData() const override { return els_.read(); }
      virtual std::vector<qtnh::tel> hostElements() const override { return els_.to_host(); }

    protected:
      DenseTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, std::vector<qtnh::tel>&& els);
      DenseTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, std::vector<qtnh::tel>&& els,
                  BcParams params);
      DenseTensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, detail::DeviceArray&& els,
                  BcParams params);

      virtual DenseTensor* toDense() noexcept override { return this; }
      virtual DenseTensor* swap(qtnh::tidx_tup_st idx1, qtnh::tidx_tup_st idx2) override;
      virtual DenseTensor* rebcast(BcParams params) override;
      virtual DenseTensor* rescatter(int offset) override;
      virtual DenseTensor* permute(std::vector<qtnh::tidx_tup_st> ptup) override;
      virtual detail::DeviceArray releaseStorage() override { return std::move(els_); }

      std::size_t check_i(std::size_t i) const;
      detail::DeviceArray els_;
  };
}

#endif
