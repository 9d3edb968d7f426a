// Tensor base class of the qtnh API on one GB300 (mirrors the reference's
// include/tensor/tensor.hpp:19-275).
//
// Storage model: a tensor with dis_dims D and loc_dims L is one row-major array over
// D ++ L in HBM. The reference gives rank r the slab r of that array; here every slab is
// resident, which is the same global order, so rescatter and rebcast change metadata
// only and all elements are addressable from this process. Element accessors read and
// write through a host mirror that is synchronised with the device lazily.
#ifndef QTNH_TENSOR_TENSOR_HPP
#define QTNH_TENSOR_TENSOR_HPP

#include <cstdint>
#include <memory>
#include <vector>

#include "core/env.hpp"
#include "core/typedefs.hpp"
#include "core/utils.hpp"

namespace qtnh {
  class Tensor;
  typedef std::unique_ptr<Tensor> tptr;

  class DenseTensor;
  class SymmTensor;
  class DiagTensor;

  namespace detail {
    /// Complex128 elements in HBM with a lazily synchronised host mirror.
    class DeviceArray {
      public:
        DeviceArray() = default;
        DeviceArray(const QTNHEnv& env, std::vector<qtnh::tel>&& host);  // uploads
        DeviceArray(const QTNHEnv& env, std::size_t n);                  // uninitialised
        ~DeviceArray();
        DeviceArray(DeviceArray&& o) noexcept;
        DeviceArray& operator=(DeviceArray&& o) noexcept;
        DeviceArray(const DeviceArray&) = delete;
        DeviceArray& operator=(const DeviceArray&) = delete;

        std::size_t size() const noexcept { return n_; }
        bool empty() const noexcept { return dev_ == nullptr; }
        /// Device pointer for reading (pending host edits are uploaded first).
        const void* read() const;
        /// Device pointer for writing (pending host edits uploaded, host mirror dropped).
        void* write();
        const qtnh::tel& host_at(std::size_t i) const;
        qtnh::tel& host_ref(std::size_t i);
        std::vector<qtnh::tel> to_host() const;
        DeviceArray clone() const;
        const QTNHEnv* env() const noexcept { return env_; }
        /// Queues an in-place application of `op` (a SymmTensor gate, kind QTNH_KIND_SYMM, or
        /// a DiagTensor diagonal, QTNH_KIND_DIAG) to these elements, with dims the tensor's
        /// total dims and targets its indices wired to op's inputs. Queued applications
        /// run, in order and fused into as few passes as their targets allow, before the
        /// elements are next read, written, copied or fetched.
        void defer(int kind, const std::vector<std::uint16_t>& targets, const std::vector<std::uint64_t>& dims,
                   DeviceArray&& op);
        /// Queues the permutation ptup of these elements (dims: their current dims; old index
        /// i moves to ptup[i]) behind the queued applications; it runs with them (moving the
        /// elements into a new buffer that the array then owns).
        void defer_permute(const std::vector<std::uint16_t>& ptup, const std::vector<std::uint64_t>& dims);
        /// Runs the queued applications now (on the environment's stream).
        void settle() const;

      private:
        void flush() const;
        void pull() const;
        const QTNHEnv* env_ = nullptr;
        mutable void* dev_ = nullptr;  // settle() may move the elements to a new buffer
        std::size_t n_ = 0;
        mutable std::vector<qtnh::tel> host_;
        mutable bool host_valid_ = false;
        mutable bool host_dirty_ = false;
    };
  }

  /// Contraction parameters (reference include/tensor/tensor.hpp:19-35).
  struct ConParams {
    public:
      ConParams() = delete;
      ConParams(std::vector<qtnh::wire> wires) : wires(wires), useDefRepls(true), dimRepls1(0), dimRepls2(0) {}
      ConParams(std::vector<qtnh::wire> wires, std::vector<qtnh::tidx_tup_st> dim_repls1,
                std::vector<qtnh::tidx_tup_st> dim_repls2)
          : wires(wires), useDefRepls(false), dimRepls1(dim_repls1), dimRepls2(dim_repls2) {}
      ~ConParams() = default;

      std::vector<qtnh::wire> wires;
      bool useDefRepls;
      std::vector<qtnh::tidx_tup_st> dimRepls1;  ///< Result position of each index of the first tensor.
      std::vector<qtnh::tidx_tup_st> dimRepls2;  ///< Result position of each index of the second tensor.
  };

  /// General tensor class.
  class Tensor {
    public:
      Tensor() = delete;
      Tensor(const Tensor&) = delete;
      virtual ~Tensor() = default;

      /// Distribution bookkeeping (reference tensor.hpp:45-70). All slabs are resident,
      /// so the tensor is active and every element is available on this process.
      struct Broadcaster {
        const QTNHEnv& env;
        qtnh::uint base;  ///< Number of slabs (product of distributed dimensions).
        qtnh::uint str;
        qtnh::uint cyc;
        qtnh::uint off;
        bool active = true;
        int group_id = 0;

        Broadcaster() = delete;
        Broadcaster(const QTNHEnv& env, qtnh::uint base, BcParams params);
        Broadcaster& operator=(Broadcaster&& b) noexcept;

        qtnh::uint span() const noexcept { return str * base * cyc; }
        std::pair<qtnh::uint, qtnh::uint> range() const noexcept { return {off, off + span()}; }
      };

      virtual TT type() const noexcept { return TT::tensor; }

      template <class T>
      T* cast() {
        return dynamic_cast<T*>(this);
      }
      template <class T>
      static std::unique_ptr<T> cast(qtnh::tptr tp) {
        return std::unique_ptr<T>(dynamic_cast<T*>(tp.release()));
      }

      template <class T>
      bool canConvert() {
        return false;
      }
      template <class T>
      static std::unique_ptr<T> convert(qtnh::tptr tp) {
        return std::unique_ptr<T>(nullptr);
      }

      /// Deep copy (device-to-device).
      virtual qtnh::tptr copy() const noexcept = 0;

      qtnh::tidx_tup locDims() const noexcept { return loc_dims_; }
      qtnh::tidx_tup disDims() const noexcept { return dis_dims_; }
      const Broadcaster& bc() const noexcept { return bc_; }

      qtnh::tidx_tup totDims() const { return utils::concat_dims(dis_dims_, loc_dims_); }
      std::size_t locSize() const { return utils::dims_to_size(loc_dims_); }
      std::size_t disSize() const { return utils::dims_to_size(dis_dims_); }
      std::size_t totSize() const { return utils::dims_to_size(totDims()); }

      /// Element i of the stored array. With every slab resident the array is the whole
      /// tensor in global row-major order, so i ranges over totSize() (the reference's
      /// rank-local array is slab 0 of it).
      virtual qtnh::tel operator[](std::size_t i) const = 0;
      /// Element at local indices of slab 0.
      virtual qtnh::tel operator[](qtnh::tidx_tup loc_idxs) const = 0;
      /// Element at total indices.
      virtual qtnh::tel at(qtnh::tidx_tup tot_idxs) const = 0;
      /// True: every element is resident.
      virtual bool has(qtnh::tidx_tup tot_idxs) const;
      /// Element at total indices (no communication needed).
      virtual qtnh::tel fetch(qtnh::tidx_tup tot_idxs) const;

      /// Exchanges two indices of equal dimension (std::runtime_error otherwise).
      static qtnh::tptr swap(qtnh::tptr tp, qtnh::tidx_tup_st idx1, qtnh::tidx_tup_st idx2);
      /// Sets the broadcast parameters (bookkeeping only).
      static qtnh::tptr rebcast(qtnh::tptr tp, BcParams params);
      /// Moves the distributed/local border by offset (positive scatters the first local
      /// indices, negative gathers the last distributed ones). Metadata only.
      static qtnh::tptr rescatter(qtnh::tptr tp, int offset);
      /// Old index i moves to position ptup[i] (on-device transpose).
      static qtnh::tptr permute(qtnh::tptr tp, std::vector<qtnh::tidx_tup_st> ptup);

      /// Contracts tp1 with tp2 (both consumed). params.dimRepls1/2 receive the
      /// replacements used when params.useDefRepls is set.
      static qtnh::tptr contract(qtnh::tptr tp1, qtnh::tptr tp2, ConParams& params);
      static qtnh::tptr contract(qtnh::tptr tp1, qtnh::tptr tp2, std::vector<qtnh::wire> wires) {
        ConParams params(wires);
        return contract(std::move(tp1), std::move(tp2), params);
      }

      // ---- engine interface (GB300 additions) ----
      /// Kind code of the C ABI (QTNH_KIND_*).
      virtual int engineKind() const noexcept = 0;
      /// Number of distributed input indices (symmetric family).
      virtual int engineDisIn() const noexcept { return 0; }
      /// Device elements in the engine's layout (null for implicit tensors).
      virtual const void* engineData() const { return nullptr; }
      /// All elements, global row-major (downloads them).
      virtual std::vector<qtnh::tel> hostElements() const;

    protected:
      Tensor(const QTNHEnv& env);
      Tensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims);
      Tensor(const QTNHEnv& env, qtnh::tidx_tup dis_dims, qtnh::tidx_tup loc_dims, BcParams params);

      qtnh::tidx_tup dis_dims_;
      qtnh::tidx_tup loc_dims_;
      Broadcaster bc_;

      virtual DenseTensor* toDense() noexcept { return nullptr; }
      virtual SymmTensor* toSymm() noexcept { return nullptr; }
      virtual DiagTensor* toDiag() noexcept { return nullptr; }

      virtual bool isDense() const noexcept { return false; }
      virtual bool isSymm() const noexcept { return false; }
      virtual bool isDiag() const noexcept { return false; }

      virtual Tensor* swap(qtnh::tidx_tup_st idx1, qtnh::tidx_tup_st idx2) = 0;
      virtual Tensor* rebcast(BcParams params) = 0;
      virtual Tensor* rescatter(int offset) = 0;
      virtual Tensor* permute(std::vector<qtnh::tidx_tup_st> ptup) = 0;

      /// Gives up the device buffer so a result can reuse it (returns an empty array
      /// when the tensor has none it can hand over).
      virtual detail::DeviceArray releaseStorage() { return detail::DeviceArray(); }

      friend qtnh::tptr contract_on_device(qtnh::tptr tp1, qtnh::tptr tp2, ConParams& params);
  };

  template <> bool Tensor::canConvert<DenseTensor>();
  template <> bool Tensor::canConvert<SymmTensor>();
  template <> bool Tensor::canConvert<DiagTensor>();

  template <> std::unique_ptr<DenseTensor> Tensor::convert<DenseTensor>(qtnh::tptr tp);
  template <> std::unique_ptr<SymmTensor> Tensor::convert<SymmTensor>(qtnh::tptr tp);
  template <> std::unique_ptr<DiagTensor> Tensor::convert<DiagTensor>(qtnh::tptr tp);

  namespace ops {
    /// Prints the elements (two significant digits), like the reference's printer.
    std::ostream& operator<<(std::ostream&, const Tensor&);
  }
}

#endif
